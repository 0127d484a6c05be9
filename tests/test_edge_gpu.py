"""Edge cases of the image-side entry points and the render loop, on the GPU.

Sizes and values the reference meets at its borders: images one pixel wide or
tall, widths on both sides of the run-length threshold of stbi_write_hdr,
runs longer than one 127-byte packet, all-zero images whose Reinhard white
point is 0, a one-pixel render, a single sample per pixel and a call with no
samples left to take.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

from pico_gb300 import scenes  # noqa: E402

pytestmark = pytest.mark.gpu


def atrous_close(got, want, rtol=1e-4):
    np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
    ok = ~np.isnan(want)
    np.testing.assert_allclose(got[ok], want[ok], rtol=rtol, atol=1e-6)


@pytest.mark.parametrize("W,H", [(1, 1), (1, 7), (7, 1), (2, 3), (65, 1), (1, 130), (129, 2)])
def test_atrous_tiny_and_thin_images(ctx, oracle, W, H):
    """Every tap clamps at the border; partial 64 x 64 tiles on both axes."""
    rng = np.random.default_rng(W * 131 + H)
    pix = rng.gamma(1.0, 1.0, (H, W, 3)).astype(np.float32)
    nrm = rng.normal(size=(H, W, 3)).astype(np.float32)
    pos = (rng.normal(size=(H, W, 3)) * 3).astype(np.float32)
    dif = rng.random((H, W, 3)).astype(np.float32)
    atrous_close(ctx.atrous(pix, nrm, pos, dif, W, H), oracle.atrous(pix, nrm, pos, dif, W, H))


def test_tonemap_degenerate_images(ctx, oracle):
    """An all-zero image (white point 0, so 0 / 0 = NaN per channel), negative
    luminances (never the white point) and one very bright pixel, bit for bit."""
    cases = [np.zeros((4, 5, 3), np.float32),
             np.full((3, 3, 3), -0.5, np.float32),
             np.random.default_rng(3).random((6, 7, 3)).astype(np.float32)]
    cases[2][2, 3] = (1e30, 2e30, 5e29)
    for img in cases:
        H, W = img.shape[:2]
        got, want = ctx.tonemap(img, W, H), oracle.reinhard(img, W, H)
        np.testing.assert_array_equal(np.isnan(got), np.isnan(want))
        ok = ~np.isnan(want)
        np.testing.assert_array_equal(got[ok].view(np.uint32), want[ok].view(np.uint32))


@pytest.mark.parametrize("W", [1, 7, 8, 9, 127, 128, 129, 300])
def test_hdr_widths_runs_and_zeros(ctx, oracle, W):
    """Raw scanlines below 8 pixels, run-length coding from 8; constant rows give
    runs split into 127-byte packets; zeros, tiny and negative values code as 0."""
    rng = np.random.default_rng(W)
    H = 3
    img = rng.gamma(0.5, 2.0, (H, W, 3)).astype(np.float32)
    img[1] = 0.75                       # one constant row: long runs in every component
    img[2, : W // 2] = 1e-35            # below the 1e-32 cut-off
    if W > 2:
        img[2, -1] = (-1.0, 2.0, 0.5)   # a negative component
    flat = img.reshape(-1, 3)
    assert ctx.encode_hdr(flat[::-1].copy(), W, H) == oracle.hdr_file(img, W, H)


def test_render_one_pixel_and_one_sample(ctx):
    """A 1 x 1 image; one sample per pixel replaces the mean and leaves the
    variance 0 (Scene.cpp:185-191); a second call with max_samples reached
    takes no sample and leaves the buffers as they were."""
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(1, 1)
    gs = ctx.upload(scene)
    pix, cnt, var = gs.render(cam, 5, 1, seed=9)
    assert cnt[0, 0] == 1 and np.isfinite(pix).all() and (var == 0).all()
    cam2 = scenes.cornell_camera(16, 8)
    pix, cnt, var = gs.render(cam2, 5, 1, seed=10)
    assert (cnt == 1).all() and (var == 0).all()
    before = (pix.copy(), cnt.copy(), var.copy())
    gs.render(cam2, 5, 1, seed=11, pixels=pix, sample_count=cnt, variance=var)
    assert ctx.render_stats()["samples"] == 0
    for a, b in zip((pix, cnt, var), before):
        np.testing.assert_array_equal(a, b)
