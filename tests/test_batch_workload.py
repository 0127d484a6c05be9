"""The batched-rendering workload generator (host only): each render draws its
resolution, instance count, samples per pixel and depth from the stated sets,
from its own seed, reproducibly."""
import numpy as np

from pico_gb300 import scenes


def test_batch_workload_draws_from_the_stated_sets():
    work = scenes.batch_workload(24, seed=11, level=1)
    assert len(work) == 24
    res = {tuple(int(v) for v in w["camera"].resolution) for w in work}
    assert res <= set(scenes.BATCH_RESOLUTIONS)
    assert {w["max_samples"] for w in work} <= set(scenes.BATCH_SPP)
    assert all(4 <= w["max_depth"] <= 8 for w in work)
    assert all(64 <= w["instances"] <= 4096 for w in work)
    assert all(len(w["scene"].instances) == w["instances"] + 1 + 8 for w in work)   # + ground + 8 lights
    assert len({w["seed"] for w in work}) == 24


def test_batch_workload_is_reproducible():
    a = scenes.batch_workload(6, seed=3, level=1)
    b = scenes.batch_workload(6, seed=3, level=1)
    for x, y in zip(a, b):
        assert x["max_samples"] == y["max_samples"] and x["max_depth"] == y["max_depth"]
        np.testing.assert_array_equal(x["scene"].instances[5].transform, y["scene"].instances[5].transform)
    c = scenes.batch_workload(6, seed=4, level=1)
    assert [w["instances"] for w in a] != [w["instances"] for w in c]
