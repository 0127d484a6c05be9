"""Batched rendering: many renders in one CUDA graph launch (pico_gpu_render_many).

Each render of a batch runs the same kernels on the same random streams as a
pico_gpu_render call with the same arguments, so its buffers must come out bit
for bit identical, whatever the wavefront size, closest-hit grid or number of
graph branches; the autotuner must return one of the settings it timed.
"""
import numpy as np
import pytest

from pico_gb300 import PicoError, scenes
from pico_gb300.types import ESTIMATOR_PHYSICAL, ESTIMATOR_REFERENCE

pytestmark = pytest.mark.gpu

PICO_ERR_INVALID_ARG = -1


@pytest.fixture(scope="module")
def batch(ctx):
    specs = [(scenes.cornell_box(), scenes.cornell_camera(40, 32), 6, 5, ESTIMATOR_PHYSICAL),
             (scenes.glossy_field(), scenes.glossy_field_camera(64, 48), 5, 6, ESTIMATOR_PHYSICAL),
             (scenes.cornell_box(), scenes.cornell_camera(24, 24), 9, 4, ESTIMATOR_REFERENCE),
             (scenes.lit_field(n_instances=96, level=2, seed=5, extent=10.0), scenes.lit_field_camera(48, 27), 3, 8,
              ESTIMATOR_PHYSICAL),
             (scenes.glossy_field(seed=7), scenes.glossy_field_camera(16, 16), 4, 5, ESTIMATOR_REFERENCE)]
    gscenes = [ctx.upload(s) for s, *_ in specs]
    yield specs, gscenes
    for g in gscenes:
        g.free()


def renders_of(specs, gscenes):
    return [{"gpu_scene": g, "camera": cam, "max_samples": spp, "max_depth": depth, "estimator": est,
             "seed": 100 + k, "max_variance": 0.0}
            for k, ((_, cam, spp, depth, est), g) in enumerate(zip(specs, gscenes))]


def singles(specs, gscenes):
    out = []
    for k, ((_, cam, spp, depth, est), g) in enumerate(zip(specs, gscenes)):
        out.append(g.render(cam, depth, spp, seed=100 + k, estimator=est))
    return out


@pytest.mark.parametrize("wavefront,ctas,branches,piece_paths,threads",
                         [(0, 0, 0, 0, 0), (1 << 12, 2, 2, 0, 64), (1 << 14, 1, 1, 0, 256), (0, 0, 0, 3000, 128),
                          (1 << 12, 4, 3, 777, 64)])
def test_batch_equals_single_renders(ctx, batch, wavefront, ctas, branches, piece_paths, threads):
    """Also with renders split into pieces of disjoint pixel ranges on different branches."""
    specs, gscenes = batch
    want = singles(specs, gscenes)
    renders = renders_of(specs, gscenes)
    done_ms, rep = ctx.render_many(renders, wavefront=wavefront, extend_ctas_per_sm=ctas, branches=branches,
                                   piece_paths=piece_paths, extend_threads=threads)
    for r, (px, cnt, var) in zip(renders, want):
        np.testing.assert_array_equal(r["pixels"], px)
        np.testing.assert_array_equal(r["sample_count"], cnt)
        np.testing.assert_array_equal(r["variance"], var)
    assert rep["samples"] == sum(int(c.sum()) for _, c, _ in want)
    assert rep["rays"] > 0 and rep["graph_nodes"] > len(renders)
    assert np.all(done_ms > 0) and np.all(done_ms <= rep["run_ms"] + 1.0)


def test_batch_continues_progressive_buffers(ctx, batch):
    """A second batch call continues each render's running mean like a second pico_gpu_render."""
    specs, gscenes = batch
    renders = renders_of(specs, gscenes)[:2]
    ctx.render_many(renders, branches=2)
    for r in renders:
        r["max_samples"] += 3
    ctx.render_many(renders, branches=2)
    (_, cam0, spp0, d0, e0), g0 = specs[0], gscenes[0]
    px, cnt, var = g0.render(cam0, d0, spp0, seed=100, estimator=e0)
    px, cnt, var = g0.render(cam0, d0, spp0 + 3, seed=100, estimator=e0, pixels=px, sample_count=cnt, variance=var)
    np.testing.assert_array_equal(renders[0]["pixels"], px)
    # as in the reference's loop, a pixel below max_samples takes max_samples more (Scene.cpp:164-198)
    np.testing.assert_array_equal(renders[0]["sample_count"], cnt)
    assert (cnt == spp0 + spp0 + 3).all()


def test_autotune_picks_a_timed_setting(ctx, batch):
    specs, gscenes = batch
    renders = renders_of(specs, gscenes)
    best, trials = ctx.autotune_batch(renders, trial_samples=1)
    assert len(trials) == 15 and all(rate > 0 for _, rate in trials)
    assert best == max(trials, key=lambda t: t[1])[0]
    # the items' own buffers are untouched
    for r in renders:
        assert not r["sample_count"].any() and not r["pixels"].any()


def test_batch_rejects_denoise_and_cache_estimator(ctx, batch):
    specs, gscenes = batch
    renders = renders_of(specs, gscenes)[:1]
    renders[0]["estimator"] = 2
    with pytest.raises(PicoError) as e:
        ctx.render_many(renders)
    assert e.value.status == PICO_ERR_INVALID_ARG
    done, rep = ctx.render_many([])
    assert rep["samples"] == 0
