"""pico_gpu_atrous_device_noalloc against pico_gpu_atrous_device, through the C ABI.

The no-allocation entry point runs the same a-trous kernels with its scratch in
a fixed device array shared by every call on the device, so two calls in a row
(different images, different sizes) must each match the allocating entry
point, within the a-trous tolerance of the other GPU tests (1e-4 relative,
1e-6 absolute, identical NaN pattern).  The file's name makes pytest collect
it last; it passes alone in a fresh process as well.
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
from scene_io import load_camera  # noqa: E402

GOLDEN = HERE / "golden"
PICO_ERR_INVALID_ARG = -1


def atrous_close(got, want, rtol=1e-4):
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    np.testing.assert_array_equal(nan_g, nan_w)
    ok = ~nan_w
    np.testing.assert_allclose(got[ok], want[ok], rtol=rtol, atol=1e-6)


def golden_inputs():
    z = np.load(GOLDEN / "atrous.npz")
    W, H = load_camera(z["cam"]).resolution
    return [np.ascontiguousarray(z[k]) for k in ("pixels", "normals", "positions", "diffuse")], int(W), int(H)


def random_inputs(W, H, seed):
    rng = np.random.default_rng(seed)
    return [rng.gamma(1.0, 1.0, (H, W, 3)).astype(np.float32),
            rng.normal(size=(H, W, 3)).astype(np.float32),
            (rng.normal(size=(H, W, 3)) * 3).astype(np.float32),
            rng.random((H, W, 3)).astype(np.float32)], W, H


@pytest.mark.gpu
def test_no_alloc_atrous_matches_allocating_entry_point(ctx):
    torch = pytest.importorskip("torch")
    stream = torch.cuda.current_stream().cuda_stream
    cases = [golden_inputs(), random_inputs(130, 70, 11)]
    dev = [[torch.from_numpy(a).cuda() for a in arrs] for arrs, _, _ in cases]
    outs = [torch.full_like(d[0], -7.0) for d in dev]

    # two calls in a row through the C ABI, sharing the fixed scratch; after the
    # first call's set-up, device free memory does not move
    free = []
    for d, out, (_, W, H) in zip(dev, outs, cases):
        st = ctx.lib.pico_gpu_atrous_device_noalloc(ctx.handle, *[t.data_ptr() for t in d], W, H,
                                                    out.data_ptr(), stream)
        assert st == 0, ctx.lib.pico_gpu_last_error(ctx.handle)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    assert free[1] == free[0]

    for d, out, (_, W, H) in zip(dev, outs, cases):
        want = torch.empty_like(d[0])
        st = ctx.lib.pico_gpu_atrous_device(ctx.handle, *[t.data_ptr() for t in d], W, H, want.data_ptr(), stream)
        assert st == 0, ctx.lib.pico_gpu_last_error(ctx.handle)
        torch.cuda.synchronize()
        atrous_close(out.cpu().numpy(), want.cpu().numpy())


@pytest.mark.gpu
def test_no_alloc_atrous_rejects_images_beyond_its_scratch(ctx):
    torch = pytest.importorskip("torch")
    d = [torch.zeros(12, device="cuda") for _ in range(5)]
    ptrs = [t.data_ptr() for t in d]
    for W, H in [(2049, 1024), (1, 65536), (1 << 21, 2)]:
        st = ctx.lib.pico_gpu_atrous_device_noalloc(ctx.handle, *ptrs[:4], W, H, ptrs[4], None)
        assert st == PICO_ERR_INVALID_ARG, (W, H, st)
        assert b"exceeds the fixed scratch" in ctx.lib.pico_gpu_last_error(ctx.handle)
    assert ctx.lib.pico_gpu_atrous_device_noalloc(ctx.handle, *ptrs[:4], 0, 0, ptrs[4], None) == 0
    # an image of exactly the maximum size is accepted and matches
    arrs, W, H = random_inputs(2048, 1024, 5)
    dv = [torch.from_numpy(a).cuda() for a in arrs]
    got, want = torch.empty_like(dv[0]), torch.empty_like(dv[0])
    assert ctx.lib.pico_gpu_atrous_device_noalloc(ctx.handle, *[t.data_ptr() for t in dv], W, H,
                                                  got.data_ptr(), None) == 0
    assert ctx.lib.pico_gpu_atrous_device(ctx.handle, *[t.data_ptr() for t in dv], W, H,
                                          want.data_ptr(), None) == 0
    torch.cuda.synchronize()
    atrous_close(got.cpu().numpy(), want.cpu().numpy())
