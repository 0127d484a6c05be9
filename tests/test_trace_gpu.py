"""Closest-hit parity: the sm_103a traversal against the oracle, bit for bit.

UpperLevelBVH::get_closest_intersection (Core/UpperLevelBVH.cpp:12-20) returns,
for every ray, the instance and triangle hit first and the world distance.
Here the GPU result must equal the oracle's exactly: same instance, same
triangle, same float bits for t, u and v.  Ties (equal distances) must resolve
like the reference's depth-first first-found rule, which the tie scenes check.
"""
from pathlib import Path

import numpy as np
import pytest

import pico_gb300
from pico_gb300 import scenes
from pico_gb300.types import DIFFUSE, HIT_DTYPE, RAY_DTYPE, Instance, Material, Mesh, SceneData

pytestmark = pytest.mark.gpu


def assert_same_hits(got, want, label=""):
    for k in ("inst", "prim"):
        bad = np.nonzero(got[k] != want[k])[0]
        assert len(bad) == 0, f"{label}: {k} differs on {len(bad)} of {len(want)} rays (first {bad[:5]})"
    for k in ("t", "u", "v"):
        bad = np.nonzero(got[k].view(np.uint32) != want[k].view(np.uint32))[0]
        assert len(bad) == 0, f"{label}: {k} bits differ on {len(bad)} rays (first {bad[:5]})"


def random_rays(rng, n, lo, hi, normalize=True):
    """Unnormalized directions are scaled to length >= 1: the reference prunes
    TLAS nodes by comparing a parametric slab distance with a Euclidean hit
    distance, which is conservative only for |D| >= 1; below that its answer
    depends on its own visit order (every reference caller normalizes)."""
    r = np.zeros(n, RAY_DTYPE)
    r["org"][:, :3] = rng.uniform(lo, hi, size=(n, 3))
    r["org"][:, 3] = 1.0
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    if not normalize:
        d *= rng.uniform(1.0, 4.0, size=(n, 1))
    r["dir"][:, :3] = d
    r["dir"][:, 3] = 10000.0
    return r


def check(ctx, oracle, scene, rays, label):
    """Both traversal orders must reproduce the oracle exactly on these batches."""
    gs = ctx.upload(scene)
    want = oracle.scene(scene).trace(rays)
    try:
        for order in (1, 0):
            ctx.set_traversal_order(order)
            got = gs.trace_closest(rays)
            assert_same_hits(got, want, f"{label} (order {order})")
    finally:
        ctx.set_traversal_order(0)
    return got, want


def test_cornell_primary_and_bounce(ctx, oracle):
    scene = scenes.cornell_box()
    rays = np.concatenate([scenes.primary_rays(scenes.cornell_camera(128, 128), seed=3),
                           scenes.surface_rays(scene, 20000, seed=4)])
    got, want = check(ctx, oracle, scene, rays, "cornell")
    assert (want["inst"] != pico_gb300.MISS).mean() > 0.5


def test_instance_field(ctx, oracle):
    scene = scenes.instance_field(n_instances=512, level=3, seed=21, extent=30.0)
    cam = scenes.field_camera(256)
    cam.position = (0.0, 0.0, -80.0)
    rays = np.concatenate([scenes.primary_rays(cam, seed=5), scenes.surface_rays(scene, 60000, seed=6)])
    got, want = check(ctx, oracle, scene, rays, "field")
    assert (want["inst"] != pico_gb300.MISS).mean() > 0.3


def test_random_origins_inside_and_outside(ctx, oracle):
    scene = scenes.instance_field(n_instances=128, level=2, seed=8, extent=6.0)
    rng = np.random.default_rng(9)
    rays = np.concatenate([random_rays(rng, 30000, -8, 8), random_rays(rng, 5000, -8, 8, normalize=False)])
    check(ctx, oracle, scene, rays, "random")


def test_axis_aligned_rays_and_slab_planes(ctx, oracle):
    """Zero direction components give infinite inverse directions and, with an
    origin on a slab plane, NaN slab distances; the reference's selects decide."""
    scene = scenes.cornell_box()
    rng = np.random.default_rng(10)
    n = 6000
    r = np.zeros(n, RAY_DTYPE)
    grid = np.array([0.0, 0.25, 0.3, 0.375, 0.5, 0.625, 0.7, 1.0], np.float32)
    r["org"][:, :3] = rng.choice(grid, size=(n, 3))
    r["org"][:, 3] = 1.0
    axes = np.eye(3, dtype=np.float32)
    d = axes[rng.integers(0, 3, n)] * rng.choice(np.array([-1.0, 1.0], np.float32), size=(n, 1))
    r["dir"][:, :3] = d
    r["dir"][:, 3] = 10000.0
    check(ctx, oracle, scene, r, "axis")


def test_ties_between_instances(ctx, oracle):
    """Two instances with one transform: every hit is a tie at equal world t."""
    s = scenes.instance_field(n_instances=16, level=2, seed=2, extent=4.0)
    dup = list(s.instances)
    for inst in s.instances[:8]:
        dup.append(Instance(inst.mesh, inst.transform.copy(), DIFFUSE, 0))
    s.instances = dup
    rng = np.random.default_rng(12)
    rays = random_rays(rng, 20000, -6, 6)
    got, want = check(ctx, oracle, s, rays, "instance ties")
    assert np.isin(want["inst"], np.arange(8)).any()


def test_ties_within_mesh_and_large_leaves(ctx, oracle):
    """40 copies of one triangle share a centroid, so the SAH leaves them in one
    leaf (split into node chains on the GPU) and every hit is a 40-way tie."""
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    k = 40
    pos = np.tile(p, (k, 1))
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (3 * k, 1))
    idx = np.arange(3 * k, dtype=np.uint32).reshape(k, 3)
    s = SceneData(meshes=[Mesh(pos, nrm, idx), scenes.quad_mesh([[0, 0, 2], [1, 0, 2], [1, 1, 2], [0, 1, 2]], [0, 0, -1])],
                  materials=[Material()])
    eye = scenes.glm_storage(np.eye(4))
    s.instances = [Instance(0, eye), Instance(1, eye), Instance(0, scenes.glm_storage(scenes.translate([0, 0, 1])))]
    rng = np.random.default_rng(13)
    r = np.zeros(5000, RAY_DTYPE)
    r["org"][:, :3] = np.c_[rng.uniform(-0.2, 1.2, (5000, 2)), np.full(5000, -1.0)]
    r["org"][:, 3] = 1.0
    r["dir"][:, :3] = [0, 0, 1]
    r["dir"][:, 3] = 100.0
    got, want = check(ctx, oracle, s, r, "mesh ties")
    assert (want["prim"][want["inst"] == 0] == 0).all()   # the reference keeps the first-found copy


def test_single_instance_and_misses(ctx, oracle):
    s = SceneData(meshes=[scenes.quad_mesh([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], [0, 0, 1])],
                  instances=[Instance(0, scenes.glm_storage(np.eye(4)))], materials=[Material()])
    rng = np.random.default_rng(14)
    rays = random_rays(rng, 4000, -2, 2)
    got, want = check(ctx, oracle, s, rays, "single")
    miss = want["inst"] == pico_gb300.MISS
    assert miss.any() and (~miss).any()
    assert np.isinf(got["t"][miss]).all()


def test_full_size_instance_field(ctx, oracle):
    """The traversal workload at its full size: 4096 instances of a level-4 icosphere
    (5120 triangles each), 16,777,216 rays (half primary rays of a 4096x4096 pinhole,
    half cosine-distributed bounce rays from surface points), both orders bit-exact."""
    scene = scenes.instance_field(n_instances=4096, level=4, seed=12345)
    rays = scenes.field_rays(scene, n_total=1 << 24, resolution=4096, seed=7)
    got, want = check(ctx, oracle, scene, rays, "full-size field")
    hit = want["inst"] != pico_gb300.MISS
    assert 0.2 < hit.mean() < 1.0


def test_empty_batch(ctx):
    gs = ctx.upload(scenes.cornell_box())
    out = gs.trace_closest(np.zeros(0, RAY_DTYPE))
    assert out.shape == (0,)


def test_device_pointer_path_matches_host_path(ctx, oracle):
    torch = pytest.importorskip("torch")
    scene = scenes.instance_field(n_instances=256, level=3, seed=31, extent=20.0)
    rays = np.concatenate([scenes.primary_rays(scenes.field_camera(128), seed=1),
                           scenes.surface_rays(scene, 30000, seed=2)])
    gs = ctx.upload(scene)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.empty(len(rays) * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    gs.trace_closest_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), stream)
    gs.check(stream)
    got = d_hits.cpu().numpy().view(HIT_DTYPE)
    assert_same_hits(got, oracle.scene(scene).trace(rays), "device path")
    stats = gs.trace_stats(d_rays.data_ptr(), len(rays), stream)
    assert stats["nodes"] > 0 and stats["tris"] > 0 and stats["instances"] > 0


def test_pinned_host_buffers_match_oracle(ctx, oracle):
    """Page-locked, mapped host buffers are traversed in place (no staging copies); pinned
    rays with pageable hits take the chunked copies: both give the oracle's hits."""
    torch = pytest.importorskip("torch")
    scene = scenes.instance_field(n_instances=256, level=3, seed=33, extent=20.0)
    rays = np.concatenate([scenes.primary_rays(scenes.field_camera(256), seed=3),
                           scenes.surface_rays(scene, 40000, seed=4)])
    want = oracle.scene(scene).trace(rays)
    gs = ctx.upload(scene)
    h_rays = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
    h_hits = torch.zeros(len(rays) * HIT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
    gs.trace_closest_ptr(h_rays.data_ptr(), len(rays), h_hits.data_ptr())
    assert_same_hits(h_hits.numpy().view(HIT_DTYPE), want, "pinned")
    pageable = np.zeros(len(rays), HIT_DTYPE)
    gs.trace_closest_ptr(h_rays.data_ptr(), len(rays), pageable.ctypes.data)
    assert_same_hits(pageable, want, "pinned rays, pageable hits")


def test_scene_info(ctx):
    gs = ctx.upload(scenes.instance_field(n_instances=64, level=2, seed=1))
    info = gs.info()
    assert info["instances"] == 64 and info["triangles"] == 320 and info["tlas_nodes"] > 0


def test_unsupported_bsdf_is_rejected(ctx):
    s = scenes.cornell_box()
    s.instances[0].bsdf = 7   # past Specular_Delta_BRDF
    with pytest.raises(pico_gb300.PicoError) as e:
        ctx.upload(s)
    assert e.value.status == -8


def test_implicit_spheres_and_cubes(ctx, oracle):
    """LowerLevelSphereBVH / LowerLevelCube instances (scaled, rotated) among meshes:
    both orders reproduce the oracle (and so the reference's golden hits) exactly,
    including the object-space t an implicit hit reports in u."""
    z = np.load(Path(__file__).resolve().parent / "golden" / "shapes.npz")
    scene = scenes.cornell_shapes()
    got, want = check(ctx, oracle, scene, z["rays"], "shapes")
    np.testing.assert_array_equal(got["inst"], z["hit_inst"])
    np.testing.assert_array_equal(got["prim"], z["hit_prim"])
    hit = z["hit_inst"] != pico_gb300.MISS
    np.testing.assert_array_equal(got["t"][hit].view(np.uint32), z["hit_t"][hit].view(np.uint32))
    assert (got["prim"] == 0xFFFFFFFE).sum() > 1000


def test_implicit_cubes_in_near_first_order(ctx, oracle):
    """Cube instances alone keep the near-first walk: every cube hit lies inside its
    instance's box along the ray, so near-first reproduces the reference."""
    s = scenes.cornell_box()
    cube = len(s.meshes)
    s.meshes.append(scenes.implicit_mesh(pico_gb300.SHAPE_CUBE))
    for k, (t, sc, rot) in enumerate([((0.3, 0.3, 0.4), 0.2, 15.0), ((0.7, 0.25, 0.6), 0.3, -40.0),
                                      ((0.5, 0.75, 0.5), 0.15, 60.0)]):
        m = scenes.translate(t) @ scenes.rotate_y(rot) @ scenes.scale(sc)
        s.instances.append(Instance(cube, scenes.glm_storage(m), DIFFUSE, 0))
    rays = random_rays(np.random.default_rng(5), 20000, 0.02, 0.98)
    got, want = check(ctx, oracle, s, rays, "cubes")
    assert (want["prim"] == 0xFFFFFFFE).sum() > 1000


@pytest.mark.parametrize("n", [1, 7, 31, 32, 33, 63, 64, 65, 100, 1000, 4097, 50021])
def test_ragged_batches(ctx, oracle, n):
    """Warps claim rays in chunks of 64 (32 when a launch holds fewer than 1024 rays
    per warp) and refill idle lanes from them: every batch size, around the chunk and
    warp sizes and far below one ray per warp of the grid, gives the oracle's hits,
    device-resident and from host memory, with each ray's hit in its own slot."""
    torch = pytest.importorskip("torch")
    scene = scenes.instance_field(n_instances=128, level=2, seed=41, extent=15.0)
    rng = np.random.default_rng(n)
    rays = np.concatenate([scenes.surface_rays(scene, n // 2 + 1, seed=n),
                           random_rays(rng, n, -20.0, 20.0)])[:n]
    want = oracle.scene(scene).trace(rays)
    gs = ctx.upload(scene)
    assert_same_hits(gs.trace_closest(rays), want, f"host, {n} rays")
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.full((n * HIT_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    gs.trace_closest_device(d_rays.data_ptr(), n, d_hits.data_ptr(), stream)
    gs.check(stream)
    assert_same_hits(d_hits.cpu().numpy().view(HIT_DTYPE), want, f"device, {n} rays")
    gs.free()
