"""The watertight triangle test (pico_gpu_set_triangle_test, opt-in).

The reference's Moeller-Trumbore (Core/LowerLevelMeshBVH.cpp:165-207) can let a
ray through the crack between two triangles that share an edge or a vertex: each
triangle rounds its own barycentrics and both can reject a ray that passes exactly
between them.  The watertight test (Woop, Benthin and Wald, JCGT 2013) evaluates
the shared edge's function bit-identically, negated, in both triangles, so such a
ray always hits one of them; and the variant's box tests are conservative (a
vertex shared by a closed fan lies on the faces of the fan's sub-boxes, where the
reference's slab arithmetic can reject every one of them).  Checked here on rays
aimed at points of shared edges (quads split along a diagonal) and at shared
vertices (closed triangle fans around an interior vertex), in both traversal
orders; and away from edges the watertight variant finds the same triangles as
the reference's test, with distances equal up to rounding (1e-5 relative, or
4e-7 of the coordinates' magnitude: the world distance is taken between points
whose coordinates carry that much rounding).
"""
import numpy as np
import pytest

import pico_gb300
from pico_gb300 import scenes
from pico_gb300.types import DIFFUSE, RAY_DTYPE, Instance, Material, Mesh, SceneData

pytestmark = pytest.mark.gpu
MOLLER_TRUMBORE, WATERTIGHT = 0, 1


def frame(rng):
    a = rng.normal(size=3)
    a /= np.linalg.norm(a)
    b = np.cross(a, rng.normal(size=3))
    b /= np.linalg.norm(b)
    return a, b, np.cross(a, b)


def rays_at(targets, normals, rng, dist=5.0):
    """Rays from random directions (at least 25 degrees off the surface) ending at the targets."""
    n = len(targets)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    cos = np.abs(np.sum(d * normals, axis=1))
    d[cos < 0.42] = normals[cos < 0.42]
    o = (targets - dist * d).astype(np.float32)
    dd = (targets.astype(np.float32) - o).astype(np.float64)
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    r = np.zeros(n, RAY_DTYPE)
    r["org"][:, :3] = o
    r["org"][:, 3] = 1.0
    r["dir"][:, :3] = dd.astype(np.float32)
    r["dir"][:, 3] = 1e4
    return r


def shared_edge_scene(nquads, per, seed):
    """Quads in general position, each split along its diagonal v0-v2 (the shared edge), far
    apart; `per` rays per quad aimed at random points of the diagonal's interior."""
    rng = np.random.default_rng(seed)
    s = SceneData(materials=[Material(diffuse=(0.5, 0.5, 0.5))])
    targets, normals, owner = [], [], []
    for q in range(nquads):
        c = rng.uniform(-300.0, 300.0, 3)
        a, b, n = frame(rng)
        uv = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], float) * rng.uniform(0.5, 2.0, 2)
        uv += rng.uniform(-0.2, 0.2, (4, 2))
        p = (c + uv[:, :1] * a + uv[:, 1:] * b).astype(np.float32)
        s.meshes.append(scenes.quad_mesh(p, n))
        s.instances.append(Instance(q, scenes.glm_storage(np.eye(4)), DIFFUSE, 0))
        t = rng.uniform(0.02, 0.98, per)[:, None]
        targets.append(p[0] + t * (p[2].astype(np.float64) - p[0]))
        normals.append(np.tile(n, (per, 1)))
        owner.append(np.full(per, q))
    return s, rays_at(np.concatenate(targets), np.concatenate(normals), rng), np.concatenate(owner)


def shared_vertex_scene(nfans, per, seed, k=7):
    """Closed fans of k triangles around an interior vertex, in general position; `per` rays per
    fan aimed exactly at that vertex.  The ring's angles are even or jittered, every angular gap
    below pi: a gap above pi would fold its triangle over to the other side, and the fan would no
    longer cover the plane around the vertex (rays passing on the open side miss rightly)."""
    rng = np.random.default_rng(seed)
    s = SceneData(materials=[Material(diffuse=(0.5, 0.5, 0.5))])
    targets, normals, owner = [], [], []
    for f in range(nfans):
        c = rng.uniform(-300.0, 300.0, 3)
        a, b, n = frame(rng)
        jitter = rng.uniform(-0.45, 0.45, k) if f % 2 else np.zeros(k)
        ang = (np.arange(k) + jitter) * (2 * np.pi / k)
        assert np.diff(np.append(ang, ang[0] + 2 * np.pi)).max() < np.pi
        rad = rng.uniform(0.5, 2.0, k)
        ring = c + (rad * np.cos(ang))[:, None] * a + (rad * np.sin(ang))[:, None] * b
        p = np.vstack([c, ring]).astype(np.float32)
        idx = np.array([[0, 1 + i, 1 + (i + 1) % k] for i in range(k)], np.uint32)
        s.meshes.append(Mesh(p, np.tile(n, (k + 1, 1)), idx))
        s.instances.append(Instance(f, scenes.glm_storage(np.eye(4)), DIFFUSE, 0))
        targets.append(np.tile(p[0].astype(np.float64), (per, 1)))
        normals.append(np.tile(n, (per, 1)))
        owner.append(np.full(per, f))
    return s, rays_at(np.concatenate(targets), np.concatenate(normals), rng), np.concatenate(owner)


def trace(ctx, scene, rays, test, order):
    ctx.set_triangle_test(test)
    ctx.set_traversal_order(order)
    try:
        gs = ctx.upload(scene)
        hits = gs.trace_closest(rays)
        gs.free()
    finally:
        ctx.set_triangle_test(MOLLER_TRUMBORE)
        ctx.set_traversal_order(0)
    return hits


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("make", [shared_edge_scene, shared_vertex_scene])
def test_no_ray_passes_between_adjacent_triangles(ctx, order, make):
    scene, rays, owner = make(200, 100, 31)
    wt = trace(ctx, scene, rays, WATERTIGHT, order)
    mt = trace(ctx, scene, rays, MOLLER_TRUMBORE, order)
    wt_miss = int((wt["inst"] != owner).sum())
    mt_miss = int((mt["inst"] != owner).sum())
    print(f"{make.__name__}, order {order}: {len(rays)} rays, Moeller-Trumbore misses {mt_miss}, watertight {wt_miss}")
    assert wt_miss == 0, wt_miss
    # where both hit, the distances agree (the hit point is the same up to rounding)
    both = (mt["inst"] == owner)
    np.testing.assert_allclose(wt["t"][both], mt["t"][both], rtol=1e-5, atol=300 * 4e-7)   # |coordinates| < 302


def test_watertight_finds_the_reference_triangles_away_from_edges(ctx, oracle):
    scene = scenes.instance_field(n_instances=256, level=3, seed=31, extent=20.0)
    cam = scenes.field_camera(128)
    cam.position = (0.0, 0.0, -60.0)
    rays = np.concatenate([scenes.primary_rays(cam, seed=1), scenes.surface_rays(scene, 30000, seed=2)])
    want = oracle.scene(scene).trace(rays)
    for order in (0, 1):
        got = trace(ctx, scene, rays, WATERTIGHT, order)
        np.testing.assert_array_equal(got["inst"] != pico_gb300.MISS, want["inst"] != pico_gb300.MISS)
        same = (got["inst"] == want["inst"]) & (got["prim"] == want["prim"])
        assert same.mean() > 0.999, same.mean()
        hit = same & (want["inst"] != pico_gb300.MISS)
        np.testing.assert_allclose(got["t"][hit], want["t"][hit], rtol=1e-5, atol=60 * 4e-7)   # |coordinates| < 60
        # barycentrics lose digits as the ray grazes the triangle (both forms divide by a determinant
        # that goes to zero); the largest difference seen over 24,544 hits was 2.6e-4
        np.testing.assert_allclose(got["u"][hit], want["u"][hit], atol=1e-3)
        np.testing.assert_allclose(got["v"][hit], want["v"][hit], atol=1e-3)


def test_watertight_render_runs_and_the_setting_is_checked(ctx):
    gs = ctx.upload(scenes.cornell_box())
    ctx.set_triangle_test(WATERTIGHT)
    try:
        pix, cnt, _ = gs.render(scenes.cornell_camera(32, 32), 5, 4, seed=3, estimator=1)
        assert np.isfinite(pix).all() and (cnt == 4).all() and pix.mean() > 0
    finally:
        ctx.set_triangle_test(MOLLER_TRUMBORE)
        gs.free()
    with pytest.raises(pico_gb300.PicoError):
        ctx.set_triangle_test(2)
