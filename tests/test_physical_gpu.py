"""The physical estimator on the GPU against its FP64 oracle.

The estimator has no counterpart in the reference; its oracle (oracle/po_physical.c,
pinned by the CPU tests in test_physical_oracle.py) restates the same published
methods in double precision.  The device BSDF must agree with it to 1e-5 relative
on f and pdf, device renders must agree with the oracle's converged pixels within
their statistical error, and the render loop must count every sample.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

from pico_gb300 import PicoError, scenes
from pico_gb300.types import BTDF, DIELECTRIC, DIFFUSE, ESTIMATOR_PHYSICAL, FRESNEL, LIGHT, SPECULAR, Material

sys.path.insert(0, str(Path(__file__).resolve().parent))
from calibration import assert_like_oracle, stats  # noqa: E402

pytestmark = pytest.mark.gpu

PICO_ERR_INVALID_ARG, PICO_ERR_UNSUPPORTED = -1, -8


def random_tuples(n, seed, rough_lo):
    rng = np.random.default_rng(seed)
    kinds = rng.choice([DIFFUSE, SPECULAR, DIELECTRIC], n)
    mats = [Material(diffuse=tuple(rng.uniform(0.05, 0.9, 3)), specular=tuple(rng.uniform(0.02, 0.95, 3)),
                     roughness=float(rng.uniform(rough_lo, 1.0))) for _ in range(n)]

    def unit(a):
        return a / np.linalg.norm(a, axis=1, keepdims=True)

    N = unit(rng.normal(size=(n, 3)))
    V = unit(rng.normal(size=(n, 3)))
    V = np.where((np.sum(V * N, 1) < 0)[:, None], -V, V)
    keep = np.sum(V * N, 1) > 0.05
    L = unit(rng.normal(size=(n, 3)))
    u = rng.random((n, 3))
    f32 = [a.astype(np.float32) for a in (V, N, L, u)]
    return kinds[keep], [m for m, k in zip(mats, keep) if k], *[a[keep] for a in f32]


@pytest.mark.parametrize("rough_lo,rtol", [(0.2, 1e-5), (0.05, 1e-4)])
def test_device_bsdf_matches_fp64_oracle(ctx, oracle, rough_lo, rtol):
    kinds, mats, V, N, L, u = random_tuples(3000, 41, rough_lo)
    f, pdf, sl, spdf, sw, ok = ctx.phys_bsdf_eval(kinds, mats, V, N, L, u)
    checked = 0
    for i in range(len(kinds)):
        v, n, l, uu = (a[i].astype(np.float64) for a in (V, N, L, u))
        fo, po = oracle.phys_bsdf_eval(int(kinds[i]), mats[i], v, n, l)
        np.testing.assert_allclose(f[i], fo, rtol=rtol, atol=1e-7)
        np.testing.assert_allclose(pdf[i], po, rtol=rtol, atol=1e-7)
        oko, lo, pso, wo = oracle.phys_bsdf_sample(int(kinds[i]), mats[i], v, n, uu)
        if abs(lo @ n) < 1e-4:
            continue   # leaves along the horizon: either side is right
        assert ok[i] == oko
        if oko:
            checked += 1
            np.testing.assert_allclose(sl[i], lo, atol=2e-5)
            np.testing.assert_allclose(spdf[i], pso, rtol=20 * rtol, atol=1e-6)
            np.testing.assert_allclose(sw[i], wo, rtol=20 * rtol, atol=1e-6)
    assert checked > len(kinds) // 2


def check_against_oracle(ctx, oracle, scene, cam, depth, spp, judge_spp, npix, seed):
    W, H = cam.resolution
    gs = ctx.upload(scene)
    pix, cnt, _ = gs.render(cam, depth, spp, seed=seed, estimator=ESTIMATOR_PHYSICAL)
    gs.free()
    assert (cnt == spp).all()
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(W * H, npix, replace=False)).astype(np.uint32)
    mean, var = oracle.scene(scene).phys_render_mean(cam, depth, judge_spp, idx,
                                                     rng.integers(1, 2**63, npix, dtype=np.uint64))
    got = pix.reshape(-1, 3)[idx].astype(np.float64)
    noisy = var > 0
    # the bars: what independent oracle renders of the same pixels at the same spp show
    # against the same judge (tests/calibration.py), not a fixed rate
    os_ = oracle.scene(scene)
    runs = []
    for k in range(3):
        ox, _ = os_.phys_render_mean(cam, depth, spp, idx, rng.integers(1, 2**63, npix, dtype=np.uint64))
        runs.append(stats(ox, mean, var, spp, judge_spp))
    assert_like_oracle(stats(got, mean, var, spp, judge_spp), runs, "physical render")
    # no bias overall: the mean difference is within its standard error
    se = np.sqrt(np.sum(var * (1.0 / spp + 1.0 / judge_spp))) / var.size
    assert abs(np.mean(got - mean)) < 4 * se
    # flat pixels (the sky seen directly) are exact up to float accumulation
    np.testing.assert_allclose(got[~noisy], mean[~noisy], rtol=1e-5, atol=1e-6)
    return got, mean, var


def test_cornell_physical_render_matches_oracle(ctx, oracle):
    check_against_oracle(ctx, oracle, scenes.cornell_box(), scenes.cornell_camera(64, 64), 5, 1024, 4096, 512, 11)


def test_glossy_field_physical_render_matches_oracle(ctx, oracle):
    """GGX metals and dielectrics, a mirror, three quad lights, a constant sky and the sun."""
    check_against_oracle(ctx, oracle, scenes.glossy_field(), scenes.glossy_field_camera(64, 48), 6, 1024, 4096,
                         512, 12)


def test_many_light_field_physical_render_matches_oracle(ctx, oracle):
    """300 quad lights over a small field: the power-proportional light pick bisects a
    301-slot table (the oracle scans it)."""
    from pico_gb300.types import Camera
    scene = scenes.lit_field(n_instances=48, level=2, seed=77, n_lights=300, extent=20.0)
    cam = Camera(position=(0.0, 8.0, -60.0), direction=(0.0, -0.15, 1.0), resolution=(48, 32), aspect=1.5)
    check_against_oracle(ctx, oracle, scene, cam, 5, 1024, 2048, 256, 13)


def test_physical_counts_every_sample(ctx):
    """No early exit and no dropped first sample: black pixels take every sample too."""
    gs = ctx.upload(scenes.cornell_box())
    cam = scenes.cornell_camera(32, 32)
    pix, cnt, var = gs.render(cam, 5, 7, seed=3, estimator=ESTIMATOR_PHYSICAL)
    assert (cnt == 7).all()
    assert ctx.render_stats()["samples"] == 32 * 32 * 7
    assert np.isfinite(pix).all() and np.isfinite(var).all()
    # a second call continues the plain mean of the same pixels; as in the reference's
    # loop, a pixel below max_samples takes max_samples more (Scene.cpp:164-198)
    pix2, cnt2, _ = gs.render(cam, 5, 9, seed=4, pixels=pix, sample_count=cnt, variance=var,
                              estimator=ESTIMATOR_PHYSICAL)
    assert (cnt2 == 16).all() and ctx.render_stats()["samples"] == 32 * 32 * 9
    gs.free()


def test_btdf_scenes_render_and_the_cache_estimator_rejects_them(ctx):
    """Transparent and Fresnel instances render through the physical estimator; the radiance
    cache estimator returns PICO_ERR_UNSUPPORTED for them, and without a cache attached it
    rejects the arguments."""
    scene = scenes.cornell_box()
    scene.instances[0].bsdf = BTDF
    gs = ctx.upload(scene)
    cam = scenes.cornell_camera(8, 8)
    pix, cnt, _ = gs.render(cam, 5, 4, estimator=ESTIMATOR_PHYSICAL)
    assert (cnt == 4).all() and np.isfinite(pix).all()
    with pytest.raises(PicoError) as e:
        gs.render(cam, 5, 1, estimator=2)
    assert e.value.status == PICO_ERR_UNSUPPORTED
    gs.free()
    gs = ctx.upload(scenes.cornell_box())
    with pytest.raises(PicoError) as e:
        gs.render(cam, 5, 1, estimator=2)
    assert e.value.status == PICO_ERR_INVALID_ARG
    gs.free()


def glass_field():
    """The glossy field with every third instance made of rough tinted glass (Transparent and
    Fresnel kinds alternating, roughness 0.05-0.5, index 1.3-1.8)."""
    s = scenes.glossy_field()
    rng = np.random.default_rng(3)
    for k, inst in enumerate(s.instances):
        if inst.bsdf != LIGHT and k % 3 == 0:
            s.materials.append(Material(diffuse=tuple(rng.uniform(0.5, 1.0, 3)), roughness=float(rng.uniform(0.05, 0.5)),
                                        ior=float(rng.uniform(1.3, 1.8))))
            inst.material = len(s.materials) - 1
            inst.bsdf = FRESNEL if (k // 3) % 2 else BTDF
    return s


def test_glass_field_physical_render_matches_oracle(ctx, oracle):
    """Rough dielectric interfaces (refraction, Fresnel reflection, total internal reflection,
    paths through glass) next to GGX metals, a mirror, three quad lights and the sun."""
    check_against_oracle(ctx, oracle, glass_field(), scenes.glossy_field_camera(64, 48), 8, 1024, 4096, 512, 14)


@pytest.mark.parametrize("kind_name", ["BTDF", "FRESNEL"])
def test_smooth_glass_slab_furnace(ctx, kind_name):
    """A smooth glass slab under a uniform sky of radiance 1 renders 1 (tests/analytic.py)."""
    import analytic
    from pico_gb300 import types
    gs = ctx.upload(analytic.glass_slab_scene(getattr(types, kind_name)))
    try:
        spp = 1024
        pix, cnt, var = gs.render(analytic.glass_slab_camera(16), 32, spp, seed=3, estimator=ESTIMATOR_PHYSICAL)
    finally:
        gs.free()
    se = np.sqrt(np.maximum(var.astype(np.float64), 0.0) / spp)
    assert np.mean(np.abs(pix - 1.0) < 4 * se + 1e-4) >= 0.98
    assert abs(np.mean(pix) - 1.0) < 4 * np.sqrt(np.sum(se ** 2)) / pix.size + 1e-5


def test_direct_light_matches_lamberts_closed_form(ctx):
    """The device's physical estimator against a closed form (tests/analytic.py): direct light
    from one quad emitter onto a Lambertian plane, every pixel within 4 standard errors of
    Lambert's contour integral (all but 1 %), and no bias over the image."""
    import analytic
    gs = ctx.upload(analytic.lit_plane_scene())
    try:
        spp = 2048
        pix, cnt, var = gs.render(analytic.lit_plane_camera(32), 2, spp, seed=5, estimator=ESTIMATOR_PHYSICAL)
    finally:
        gs.free()
    assert (cnt == spp).all()
    want = analytic.expected_pixels(32).reshape(32, 32, 3)
    se = np.sqrt(var.astype(np.float64) / spp)
    z = np.abs(pix - want) / se
    assert np.mean(z < 4) >= 0.99, np.sort(z.ravel())[-5:]
    assert abs(np.sum(pix - want)) < 4 * np.sqrt(np.sum(se ** 2))
