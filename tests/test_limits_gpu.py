"""The device-side bounds of the traversal, run out on purpose.

Every ray walk is bounded by an iteration count and by the entries of its
stack; a walk that needs more stops and latches an error that the call returns
(PICO_ERR_TIMEOUT, PICO_ERR_STACK_OVERFLOW).  These are plain loop bounds with
no asynchronous work in flight, so running them out only ends the walks early:
the tests shrink the bounds through pico_gpu_set_traversal_limits, check every
entry point reports the error, then restore the defaults and check the next
calls succeed with the oracle's answers (the latched status was cleared).
"""
import numpy as np
import pytest

import pico_gb300
from pico_gb300 import scenes
from pico_gb300.types import HIT_DTYPE

pytestmark = pytest.mark.gpu

STACK_OVERFLOW, TIMEOUT, INVALID_ARG = -4, -5, -1


@pytest.fixture(scope="module")
def field():
    scene = scenes.instance_field(n_instances=128, level=3, seed=41, extent=12.0)
    cam = scenes.field_camera(64)
    cam.position = (0.0, 0.0, -35.0)
    rays = np.concatenate([scenes.primary_rays(cam, seed=1), scenes.surface_rays(scene, 8192, seed=2)])
    return scene, cam, rays


def status_of(fn):
    with pytest.raises(pico_gb300.PicoError) as e:
        fn()
    return e.value.status


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("limits,status", [((0, 1), STACK_OVERFLOW), ((3, 0), TIMEOUT)])
def test_bounds_run_out_and_the_context_recovers(ctx, oracle, field, order, limits, status):
    torch = pytest.importorskip("torch")
    scene, cam, rays = field
    gs = ctx.upload(scene)
    ctx.set_traversal_order(order)
    try:
        ctx.set_traversal_limits(*limits)
        # host buffers, device buffers (latched, returned by the check), a render
        assert status_of(lambda: gs.trace_closest(rays)) == status
        d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
        d_hits = torch.empty(len(rays) * HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        gs.trace_closest_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), stream)
        assert status_of(lambda: gs.check(stream)) == status
        assert status_of(lambda: gs.render(cam, 3, 2, seed=5, estimator=1)) == status
        # defaults again: every call succeeds and the hits are the oracle's
        ctx.set_traversal_limits()
        got = gs.trace_closest(rays)
        want = oracle.scene(scene).trace(rays)
        np.testing.assert_array_equal(got["inst"], want["inst"])
        np.testing.assert_array_equal(got["prim"], want["prim"])
        np.testing.assert_array_equal(got["t"].view(np.uint32), want["t"].view(np.uint32))
        gs.trace_closest_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), stream)
        gs.check(stream)
        pix, cnt, _ = gs.render(cam, 3, 2, seed=5, estimator=1)
        assert np.isfinite(pix).all() and (cnt == 2).all()
    finally:
        ctx.set_traversal_limits()
        ctx.set_traversal_order(0)
        gs.free()


def test_limits_are_checked(ctx):
    assert status_of(lambda: ctx.set_traversal_limits(0, 97)) == INVALID_ARG
    ctx.set_traversal_limits(0, 96)
    ctx.set_traversal_limits()


def test_default_bounds_hold_deep_scenes(ctx, oracle):
    """A deep, degenerate scene (many instances stacked on one line, a long chain of nested
    boxes) stays within the default bounds: the walk needs far fewer than 96 entries."""
    scene = scenes.instance_field(n_instances=1024, level=1, seed=9, extent=0.5)
    rays = scenes.surface_rays(scene, 4096, seed=3)
    gs = ctx.upload(scene)
    got = gs.trace_closest(rays)
    want = oracle.scene(scene).trace(rays)
    np.testing.assert_array_equal(got["inst"], want["inst"])
    np.testing.assert_array_equal(got["t"].view(np.uint32), want["t"].view(np.uint32))
