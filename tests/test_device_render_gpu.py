"""Device-buffer renders, measurement hooks and argument guards of the C ABI.

* pico_gpu_render_device gives the bytes pico_gpu_render gives (both estimators,
  denoise and tone map, fresh and continued progressive buffers), and its work
  through pico_gpu_render_stats.
* The render probe: the counting closest-hit variant leaves the image unchanged
  and counts work; the timer brackets every closest-hit launch.
* The L2 read probe reports a bandwidth.
* A cancel flag is seen within one batch of at most 16 samples per pixel.
* Host buffers are traversed in place only inside one pinned allocation.
* A-trous outputs that overlap an input are rejected.
"""
import ctypes as C
import os
import threading
import time

import numpy as np
import pytest

import pico_gb300
from pico_gb300 import scenes
from pico_gb300.types import HIT_DTYPE, RAY_DTYPE

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def device_render(ctx, gs, cam, depth, spp, seed, estimator=0, denoise=False, tonemap=False, start=None):
    W, H = cam.resolution
    if start is None:
        pix = torch.zeros((H, W, 3), dtype=torch.float32, device="cuda")
        var = torch.zeros((H, W, 3), dtype=torch.float32, device="cuda")
        cnt = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    else:
        pix, cnt, var = (torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in
                         (start[0], start[1].view(np.int32), start[2]))
    stream = torch.cuda.current_stream().cuda_stream
    gs.render_device(cam, depth, spp, pix.data_ptr(), cnt.data_ptr(), var.data_ptr(), stream, seed=seed,
                     denoise=denoise, tonemap=tonemap, estimator=estimator)
    gs.check(stream)
    return pix.cpu().numpy(), cnt.cpu().numpy().view(np.uint32), var.cpu().numpy()


@pytest.mark.parametrize("estimator", [0, 1])
def test_device_render_equals_host_render(ctx, estimator):
    gs = ctx.upload(scenes.cornell_box())
    cam = scenes.cornell_camera(48, 40)
    want = gs.render(cam, 5, 12, seed=31, estimator=estimator, denoise=True, tonemap=True)
    want_stats = ctx.render_stats()
    got = device_render(ctx, gs, cam, 5, 12, 31, estimator=estimator, denoise=True, tonemap=True)
    got_stats = ctx.render_stats()
    for g, w, name in zip(got, want, ("pixels", "sample counts", "variance")):
        np.testing.assert_array_equal(g, w, err_msg=name)
    assert got_stats == want_stats
    assert got_stats["samples"] == int(got[1].sum()) > 0


@pytest.mark.parametrize("estimator", [0, 1])
@pytest.mark.parametrize("limit", [100_000, 20_000, 3_000, 64])
def test_images_do_not_depend_on_the_path_limit(ctx, estimator, limit):
    """A path depends only on its pixel and sample index and every pixel takes its samples in
    order, so the batching cannot change an image: the Cornell box at 96 x 80 (7,680 pixels, 16 spp,
    some pixels resumed from a first render) is rendered bit for bit alike, through both entry
    points, with the default limit and with 100,000 paths (exit-aware rounds of 6, then 13 samples
    per pixel), 20,000 (the first round capped below its 6 samples: rounds of 2), 3,000 (fewer paths
    than pixels: the chunked schedule) and 64."""
    gs = ctx.upload(scenes.cornell_box())
    cam = scenes.cornell_camera(96, 80)
    try:
        start = gs.render(cam, 5, 3, seed=8)
        start[1][::7] = 0                       # some pixels start afresh, the others resume
        runs = []
        for lim in (0, limit):
            ctx.set_path_limit(lim)
            runs.append(gs.render(cam, 5, 16, seed=9, estimator=estimator, pixels=start[0].copy(),
                                  sample_count=start[1].copy(), variance=start[2].copy(), denoise=True))
            runs.append(device_render(ctx, gs, cam, 5, 16, 9, estimator=estimator, denoise=True,
                                      start=(start[0], start[1], start[2])))
    finally:
        ctx.set_path_limit(0)
        gs.free()
    for other in runs[1:]:
        for g, w, name in zip(other, runs[0], ("pixels", "sample counts", "variance")):
            np.testing.assert_array_equal(g, w, err_msg=name)
    with pytest.raises(pico_gb300.PicoError):
        ctx.set_path_limit(10)


def test_device_render_continues_progressive_buffers(ctx):
    gs = ctx.upload(scenes.cornell_box())
    cam = scenes.cornell_camera(32, 32)
    first = gs.render(cam, 5, 6, seed=3)
    want = gs.render(cam, 5, 14, seed=4, pixels=first[0].copy(), sample_count=first[1].copy(),
                     variance=first[2].copy())
    got = device_render(ctx, gs, cam, 5, 14, 4, start=first)
    for g, w in zip(got, want):
        np.testing.assert_array_equal(g, w)
    assert ctx.render_stats()["samples"] == int(got[1].sum()) - int(first[1].sum())


def test_device_render_rejects_the_cache_estimator(ctx):
    gs = ctx.upload(scenes.cornell_box())
    with pytest.raises(pico_gb300.PicoError):
        device_render(ctx, gs, scenes.cornell_camera(8, 8), 3, 2, 1, estimator=2)


def test_render_probe_counts_and_times_without_changing_the_image(ctx):
    gs = ctx.upload(scenes.instance_field(n_instances=64, level=2, seed=5, extent=10.0))
    cam = scenes.field_camera(64)
    cam.position = (0.0, 0.0, -30.0)
    depth, spp = 4, 8
    plain = gs.render(cam, depth, spp, seed=9, estimator=1)
    ctx.set_render_probe(count_work=True)
    counted = gs.render(cam, depth, spp, seed=9, estimator=1)
    work = ctx.render_probe_read()
    ctx.set_render_probe(time_extend=True)
    timed = gs.render(cam, depth, spp, seed=9, estimator=1)
    timing = ctx.render_probe_read()
    ctx.set_render_probe()
    for a, b, c in zip(plain, counted, timed):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(a, c)
    st = ctx.render_stats()
    rays = st["camera_paths"] + st["bounce_rays"] + st["shadow_rays"]
    assert rays > 0 and work["nodes"] > 0 and work["tris"] > 0 and work["instances"] > 0
    assert work["launches"] == 0 and timing["nodes"] == 0
    # one batch of 64^2 x 8 paths: depths 0..depth each one closest-hit launch
    assert timing["launches"] == depth + 1 and timing["extend_ms"] > 0.0


def test_l2_read_probe(ctx):
    gbs = ctx.l2_read_bandwidth(32 << 20, 50)
    assert gbs > 1000.0
    with pytest.raises(pico_gb300.PicoError):
        ctx.l2_read_bandwidth(1 << 10, 1)


def test_cancel_is_seen_within_one_batch(ctx):
    """With a cancel flag a batch holds at most 16 samples per pixel: a flag set while a long
    render runs stops it at a whole number of such batches, long before its end, with the
    buffers holding every sample taken."""
    gs = ctx.upload(scenes.cornell_box())
    cam = scenes.cornell_camera(256, 256)
    pix = np.zeros((256, 256, 3), np.float32)
    cnt = np.zeros((256, 256), np.uint32)
    var = np.zeros((256, 256, 3), np.float32)
    flag = C.c_int32(0)
    timer = threading.Timer(0.05, lambda: setattr(flag, "value", 1))
    timer.start()
    t0 = time.perf_counter()
    with pytest.raises(pico_gb300.PicoError) as e:
        gs.render(cam, 8, 4096, seed=2, pixels=pix, sample_count=cnt, variance=var, max_variance=-1.0,
                  should_quit=flag)
    secs = time.perf_counter() - t0
    timer.join()
    assert e.value.status == -6
    taken = np.unique(cnt)   # no early exit: every pixel took the same batches
    assert len(taken) == 1 and 0 < taken[0] < 4096 and taken[0] % 16 == 0, taken
    assert secs < 5.0


def page_aligned(nbytes, page):
    raw = np.zeros(nbytes + page, np.uint8)
    off = (-raw.ctypes.data) % page
    return raw, raw[off:off + nbytes]


def test_host_range_across_two_pinned_registrations_is_staged(ctx, oracle):
    """A host range whose ends lie in two separate pinned registrations, with pageable memory
    between them, is not traversed in place; one registration is.  Both give the oracle's hits."""
    cudart = torch.cuda.cudart()
    if not hasattr(cudart, "cudaHostRegister"):
        pytest.skip("torch exposes no cudaHostRegister")
    page = max(os.sysconf("SC_PAGE_SIZE"), 1 << 16)
    scene = scenes.instance_field(n_instances=64, level=2, seed=5, extent=10.0)
    n = 3 * page // RAY_DTYPE.itemsize
    rays = scenes.surface_rays(scene, n, seed=8)
    want = oracle.scene(scene).trace(rays)
    gs = ctx.upload(scene)
    keep, buf = page_aligned(3 * page, page)
    buf[:] = rays.view(np.uint8)
    base = buf.ctypes.data
    hits = np.zeros(n, HIT_DTYPE)
    assert int(cudart.cudaHostRegister(base, page, 0)) == 0
    try:
        assert int(cudart.cudaHostRegister(base + 2 * page, page, 0)) == 0
        try:
            assert ctx.host_buffer_in_place(base, page)
            assert not ctx.host_buffer_in_place(base, 3 * page)
            gs.trace_closest_ptr(base, n, hits.ctypes.data)
            np.testing.assert_array_equal(hits["inst"], want["inst"])
            np.testing.assert_array_equal(hits["prim"], want["prim"])
            np.testing.assert_array_equal(hits["t"].view(np.uint32), want["t"].view(np.uint32))
        finally:
            cudart.cudaHostUnregister(base + 2 * page)
    finally:
        cudart.cudaHostUnregister(base)
    del keep
    pinned = torch.zeros(4096, dtype=torch.uint8).pin_memory()
    assert ctx.host_buffer_in_place(pinned.data_ptr(), 4096)
    assert not ctx.host_buffer_in_place(np.zeros(4096, np.uint8).ctypes.data, 4096)


@pytest.mark.parametrize("alias", ["pixels", "normals", "positions", "diffuse", "shifted"])
def test_atrous_output_overlapping_an_input_is_rejected(ctx, alias):
    W, H = 32, 16
    n3 = W * H * 3
    bufs = {k: torch.rand(n3, device="cuda") for k in ("pixels", "normals", "positions", "diffuse")}
    big = torch.zeros(2 * n3, device="cuda")
    if alias == "shifted":
        bufs["normals"] = big[:n3]
        out = big[n3 // 2: n3 // 2 + n3]     # overlaps the second half of the normals
    else:
        out = bufs[alias]
    args = [bufs[k].data_ptr() for k in ("pixels", "normals", "positions", "diffuse")]
    stream = torch.cuda.current_stream().cuda_stream
    for call in (ctx.atrous_device, ctx.atrous_device_noalloc):
        with pytest.raises(pico_gb300.PicoError) as e:
            call(*args, W, H, out.data_ptr(), stream)
        assert e.value.status == -1
    # an adjacent, non-overlapping output is accepted
    ok = big[n3:] if alias == "shifted" else torch.empty(n3, device="cuda")
    ctx.atrous_device(*args, W, H, ok.data_ptr(), stream)
    torch.cuda.synchronize()
