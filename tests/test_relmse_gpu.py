"""relMSE of device renders against the converged judge of the reference's own samples.

The judge (FP64 mean and variance of 4096 reference samples per pixel on 4096
seeded pixels of the 256 x 256 Cornell box) gives the relMSE an unbiased
estimator averaging n samples must show: mean(var (1/n + 1/4096) / (mean^2 +
0.01)).  The device render loop keeps samples 2..n (Scene.cpp:185-191), so n
is max_samples - 1.  With the reference's default early exit (max_variance 0)
it must instead show the reference's own bias.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE / "golden")]

from judge import Judge  # noqa: E402
from pico_gb300 import scenes  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cornell(ctx):
    j = Judge("cornell")
    scene = scenes.cornell_box()
    j.check_scene(scene)
    gs = ctx.upload(scene)
    yield j, gs, scenes.cornell_camera(j.width, j.height)
    gs.free()


@pytest.mark.parametrize("spp", [16, 256])
def test_device_relmse_is_that_of_an_unbiased_estimator(cornell, spp):
    j, gs, cam = cornell
    pix, cnt, _ = gs.render(cam, j.depth, spp, seed=300 + spp, max_variance=-1.0)
    assert (cnt == spp).all()
    ratio = j.relmse(pix) / j.expected(spp - 1)
    assert 0.6 < ratio < 1.5, ratio


def test_device_early_exit_bias_matches_the_reference(cornell):
    j, gs, cam = cornell
    pix, cnt, _ = gs.render(cam, j.depth, 64, seed=377)
    exited = int((cnt.reshape(-1)[j.pixels] < 64).sum())
    assert abs(exited - j.ref64_exited) < 150, (exited, j.ref64_exited)
    ratio = j.relmse(pix) / j.ref64_relmse
    assert 0.6 < ratio < 1.6, ratio
