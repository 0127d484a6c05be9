"""Converged judge renders and the relative MSE measured against them.

A judge fixture holds, for a seeded subset of the pixels of one scene and
camera, the plain FP64 mean and sample variance of many samples of the
reference's own integrator (Render/Integrators.cpp:130-154), generated by
make_golden.py.  Scenes are rebuilt from their seeded generators at run time;
the fixture stores a digest of the scene so that a stale fixture is refused.
"""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np

from scene_io import scene_arrays

HERE = Path(__file__).resolve().parent
JUDGE_FILE = HERE / "judge.npz"
RELMSE_EPS = 0.01


def scene_digest(scene) -> str:
    h = hashlib.sha256()
    for k, v in sorted(scene_arrays(scene).items()):
        h.update(k.encode())
        h.update(np.ascontiguousarray(v).tobytes())
    return h.hexdigest()


def relmse(image: np.ndarray, judge_mean: np.ndarray, eps: float = RELMSE_EPS) -> float:
    """mean over pixels and channels of (x - r)^2 / (r^2 + eps)."""
    x = np.asarray(image, np.float64).reshape(judge_mean.shape)
    return float(np.mean((x - judge_mean) ** 2 / (judge_mean ** 2 + eps)))


def expected_relmse(judge_mean: np.ndarray, judge_var: np.ndarray, samples: float, judge_spp: int,
                    eps: float = RELMSE_EPS) -> float:
    """relMSE an unbiased estimator averaging `samples` samples per pixel should show against
    the judge: its variance plus the judge's own."""
    return float(np.mean(judge_var * (1.0 / samples + 1.0 / judge_spp) / (judge_mean ** 2 + eps)))


class Judge:
    def __init__(self, name: str, path: Path = JUDGE_FILE):
        z = np.load(path)
        self.pixels = z[f"{name}_idx"]
        self.mean = z[f"{name}_mean"]
        self.var = z[f"{name}_var"]
        self.spp = int(z[f"{name}_spp"])
        self.depth = int(z[f"{name}_depth"])
        self.width, self.height = (int(v) for v in z[f"{name}_res"])
        self.digest = str(z[f"{name}_digest"])
        self.ref64_exited = int(z[f"{name}_ref64_exited"])
        self.ref64_relmse = float(z[f"{name}_ref64_relmse"])

    def check_scene(self, scene) -> None:
        if scene_digest(scene) != self.digest:
            raise ValueError("the scene differs from the one the judge fixture was rendered from")

    def take(self, image: np.ndarray) -> np.ndarray:
        """The judged pixels of an (H, W, 3) image."""
        return np.asarray(image).reshape(-1, 3)[self.pixels]

    def relmse(self, image: np.ndarray) -> float:
        return relmse(self.take(image), self.mean)

    def relmse_finite(self, image: np.ndarray) -> tuple[float, int]:
        """relMSE over the judged pixels whose three channels are finite, and how many are not
        (the reference's a-trous pass leaves NaN where a tile's white point is 0)."""
        x = self.take(image).astype(np.float64)
        ok = np.isfinite(x).all(axis=1)
        return relmse(x[ok], self.mean[ok]), int((~ok).sum())

    def expected(self, samples: float) -> float:
        return expected_relmse(self.mean, self.var, samples, self.spp)
