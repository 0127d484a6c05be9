"""Statistical bars calibrated against the oracle itself.

A device render and a converged judge are compared per pixel channel through
z = (x - judge mean) / SE, SE from the judge's per-sample variance and both
sample counts.  Path-traced radiance is heavy-tailed (lamps of radiance up to 50
reached by rare paths), so even an exact estimator shows more |z| > 4 than a
normal law would, all of them above the judge, and a median z a little below 0.
Instead of fixed rates, every bar here is what the same statistic gives for
independent renders of the oracle (the CPU restatement of the same estimator,
same pixels, same sample count, same judge), plus a binomial margin:

  beyond     the fraction of noisy channels with |z| > 4;
  above      the fraction with z > 4 (a one-sided excess is what a small bias
             looks like, so it is bounded on its own);
  positive   the fraction with z > 0 (a sign test: a biased device render moves
             it away from the oracle's, whatever the tails do);
  zsum       sum(x - mean) / sqrt(sum(SE^2)) over the noisy channels, the
             standardised error of the image's total (checked against the spread
             of the oracle runs' values).

Margins count pixels, not channels (the three channels of a pixel share paths),
at four standard deviations of the difference of two proportions.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Stats:
    beyond: float
    above: float
    positive: float
    zsum: float
    channels: int

    def __str__(self):
        return (f"beyond 4 SE {self.beyond:.4f}, above +4 SE {self.above:.4f}, z > 0 {self.positive:.3f}, "
                f"total z {self.zsum:+.2f} over {self.channels} channels")


def stats(x, mean, var, n, judge_n) -> Stats:
    """The statistics of render x (n samples per pixel) against a judge of judge_n samples."""
    x = np.asarray(x, np.float64).reshape(np.shape(mean))
    se2 = np.asarray(var, np.float64) * (1.0 / n + 1.0 / judge_n)
    noisy = se2 > 0
    d = (x - mean)[noisy]
    z = d / np.sqrt(se2[noisy])
    return Stats(beyond=float(np.mean(np.abs(z) > 4.0)), above=float(np.mean(z > 4.0)),
                 positive=float(np.mean(z > 0.0)), zsum=float(d.sum() / np.sqrt(se2[noisy].sum())),
                 channels=int(noisy.sum()))


def _margin(p: float, n_a: float, n_b: float) -> float:
    p = min(max(p, 1.0 / n_b), 1.0 - 1.0 / n_b)
    return 4.0 * np.sqrt(p * (1.0 - p) * (1.0 / n_a + 1.0 / n_b))


def assert_like_oracle(device: Stats, oracle_runs: list[Stats], label: str = "") -> None:
    """The device statistics lie within the oracle runs' values plus binomial margins."""
    k = len(oracle_runs)
    n_dev = device.channels / 3.0
    n_or = k * np.mean([r.channels for r in oracle_runs]) / 3.0
    msg = f"{label}: device {device}; oracle " + "; ".join(str(r) for r in oracle_runs)
    beyond = float(np.mean([r.beyond for r in oracle_runs]))
    above = float(np.mean([r.above for r in oracle_runs]))
    positive = float(np.mean([r.positive for r in oracle_runs]))
    assert device.beyond <= beyond + _margin(beyond, n_dev, n_or), msg
    assert device.above <= above + _margin(above, n_dev, n_or), msg
    assert abs(device.positive - positive) <= _margin(positive, n_dev, n_or), msg
    zs = np.array([r.zsum for r in oracle_runs])
    spread = max(float(np.std(zs, ddof=1)) if k > 1 else 0.0, 1.0)
    assert abs(device.zsum - float(np.mean(zs))) <= 4.0 * spread, msg
