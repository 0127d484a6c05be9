"""Renders through the radiance cache (PICO_ESTIMATOR_RADIANCE_CACHE) on the GPU.

The cache form has no counterpart in the reference.  Its path logic is checked
against the FP64 oracle of the physical estimator (oracle/po_physical.c) with a
cache whose answer is known: zero (the image is then exactly the physical
estimator cut after one bounce, bit for bit, when every first vertex is rough)
and a constant (the oracle adds throughput * constant where the device ends
each path).  Training is checked end to end: on the Cornell box the trained
cache must recover most of the indirect light that the zero cache misses.
"""
import numpy as np
import pytest

from pico_gb300 import RadianceCache, scenes
from pico_gb300.types import ESTIMATOR_PHYSICAL, ESTIMATOR_RADIANCE_CACHE

pytestmark = pytest.mark.gpu


def constant_network(k):
    """Weights whose network output is the constant k whatever the input (bf16-exact values)."""
    mlp = np.zeros((6, 64, 64), np.float32)
    mlp[0, 0, 55] = 1.0          # the constant input
    for l in range(1, 5):
        mlp[l, 0, 0] = 1.0
    mlp[5, :3, 0] = k
    return mlp


def fixed_cache(ctx, k, scene_box=None):
    c = RadianceCache(ctx, log2_table_size=12, max_train_steps=0, train_paths=0, seed=5,
                      **({"aabb_min": scene_box[0], "aabb_max": scene_box[1]} if scene_box else {}))
    mlp = constant_network(k)
    c.set_params(mlp, np.zeros((16, c.table_size, 2), np.float32))
    c.attach()
    return c


def test_zero_cache_equals_physical_cut_after_one_bounce(ctx):
    scene = scenes.cornell_box()     # every material has roughness 1: paths end after one bounce
    cam = scenes.cornell_camera(48, 40)
    c = fixed_cache(ctx, (0.0, 0.0, 0.0))
    gs = ctx.upload(scene)
    a, ca, _ = gs.render(cam, 5, 6, seed=17, estimator=ESTIMATOR_RADIANCE_CACHE)
    b, cb, _ = gs.render(cam, 1, 6, seed=17, estimator=ESTIMATOR_PHYSICAL)
    assert (ca == 6).all() and (cb == 6).all()
    np.testing.assert_array_equal(a, b)
    st = c.stats()
    assert st["queries"] > 0 and st["train_steps"] == 0
    gs.free()
    c.free()


@pytest.mark.parametrize("scene_name", ["cornell", "glossy"])
def test_constant_cache_matches_oracle(ctx, oracle, scene_name):
    if scene_name == "cornell":
        scene, cam, depth = scenes.cornell_box(), scenes.cornell_camera(48, 48), 5
    else:
        scene, cam, depth = scenes.glossy_field(), scenes.glossy_field_camera(48, 36), 6
    k = np.array([0.5, 0.25, 1.5])
    c = fixed_cache(ctx, k)
    gs = ctx.upload(scene)
    spp, judge_spp, npix = 1024, 4096, 384
    pix, cnt, _ = gs.render(cam, depth, spp, seed=23, estimator=ESTIMATOR_RADIANCE_CACHE)
    assert (cnt == spp).all()
    W, H = cam.resolution
    rng = np.random.default_rng(24)
    idx = np.sort(rng.choice(W * H, npix, replace=False)).astype(np.uint32)
    mean, var = oracle.scene(scene).phys_render_mean_cached(cam, depth, judge_spp, idx,
                                                            rng.integers(1, 2**63, npix, dtype=np.uint64), k)
    got = pix.reshape(-1, 3)[idx].astype(np.float64)
    noisy = var > 0
    z = np.abs(got - mean)[noisy] / np.sqrt(var[noisy] * (1.0 / spp + 1.0 / judge_spp))
    assert np.mean(z < 4) >= 0.99, np.sort(z)[-8:]
    se = np.sqrt(np.sum(var * (1.0 / spp + 1.0 / judge_spp))) / var.size
    assert abs(np.mean(got - mean)) < 4 * se
    np.testing.assert_allclose(got[~noisy], mean[~noisy], rtol=1e-5, atol=1e-6)
    gs.free()
    c.free()


def test_trained_cache_recovers_indirect_light(ctx, oracle):
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(64, 64)
    W, H = cam.resolution
    rng = np.random.default_rng(31)
    idx = np.sort(rng.choice(W * H, 512, replace=False)).astype(np.uint32)
    judge, _ = oracle.scene(scene).phys_render_mean(cam, 8, 4096, idx, rng.integers(1, 2**63, 512, dtype=np.uint64))
    gs = ctx.upload(scene)

    def relmse(img):
        x = img.reshape(-1, 3)[idx].astype(np.float64)
        return float(np.mean((x - judge) ** 2 / (judge ** 2 + 0.01)))

    untrained = fixed_cache(ctx, (0.0, 0.0, 0.0))
    cut, _, _ = gs.render(cam, 8, 256, seed=41, estimator=ESTIMATOR_RADIANCE_CACHE)
    untrained.free()
    c = RadianceCache(ctx, log2_table_size=16, train_paths=16384, train_batch=16384, max_train_steps=2,
                      warmup_frames=32, seed=6)
    c.attach()
    img, cnt, _ = gs.render(cam, 8, 256, seed=42, estimator=ESTIMATOR_RADIANCE_CACHE)
    assert (cnt == 256).all()
    st = c.stats()
    assert st["train_paths"] == 16384 * (256 + 32) and st["train_steps"] > 256 and st["queries"] > 0
    assert c.info()["frames"] == 256
    e_cut, e_nrc = relmse(cut), relmse(img)
    assert e_nrc < 0.25 * e_cut, (e_nrc, e_cut)
    assert e_nrc < 0.02, e_nrc
    # an unattached context renders nothing through a freed cache
    c.free()
    gs.free()
