"""Converged-judge checks of the estimator, on the CPU.

The judge fixture holds FP64 means and variances of 4096 samples per pixel of
the reference's own integrator (Render/Integrators.cpp:130-154) on seeded
pixel subsets.  Against it, the oracle port's render loop must show the relMSE
of an unbiased estimator, and with the reference's default early exit
(Scene.cpp:185-191 with max_variance 0) the same bias as the reference's own
render loop: that exit stops a pixel whose first samples were all black.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE / "golden")]

from judge import Judge  # noqa: E402
from pico_gb300 import scenes  # noqa: E402
from pico_gb300.types import Material  # noqa: E402


@pytest.fixture(scope="module")
def cornell_judge():
    j = Judge("cornell")
    scene = scenes.cornell_box()
    j.check_scene(scene)
    return j, scene, scenes.cornell_camera(j.width, j.height)


def test_judge_fixtures_match_their_scenes():
    Judge("lit").check_scene(scenes.lit_field())
    Judge("cornell").check_scene(scenes.cornell_box())
    changed = scenes.cornell_box()
    changed.materials[0] = Material(diffuse=(0.5, 0.5, 0.5))
    with pytest.raises(ValueError):
        Judge("cornell").check_scene(changed)


def test_port_relmse_is_that_of_an_unbiased_estimator(oracle, cornell_judge):
    j, scene, cam = cornell_judge
    os_ = oracle.scene(scene)
    seeds = np.random.default_rng(71).integers(1, 2**63, len(j.pixels), dtype=np.uint64)
    pix, cnt, _ = os_.render_pixels(cam, j.depth, 16, j.pixels, seeds, max_variance=-1.0)
    assert (cnt.reshape(-1)[j.pixels] == 16).all()
    # the running mean keeps samples 2..n (Scene.cpp:185-191)
    ratio = j.relmse(pix) / j.expected(15)
    assert 0.6 < ratio < 1.5, ratio


def test_port_early_exit_bias_matches_the_reference(oracle, cornell_judge):
    j, scene, cam = cornell_judge
    os_ = oracle.scene(scene)
    seeds = np.random.default_rng(72).integers(1, 2**63, len(j.pixels), dtype=np.uint64)
    pix, cnt, _ = os_.render_pixels(cam, j.depth, 64, j.pixels, seeds)
    exited = int((cnt.reshape(-1)[j.pixels] < 64).sum())
    # two binomial counts over 4096 pixels (p ~ 0.12): 5 sigma of their difference ~ 150
    assert abs(exited - j.ref64_exited) < 150, (exited, j.ref64_exited)
    ratio = j.relmse(pix) / j.ref64_relmse
    assert 0.6 < ratio < 1.6, ratio
    assert j.ref64_relmse > 1.5 * j.expected(63)
