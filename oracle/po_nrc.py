"""Oracle of the neural radiance cache: a numpy restatement (float64 arithmetic).

TEST INFRASTRUCTURE: only the tests, the smoke entry point and the benchmark's
CPU leg use this module, as the checker of the device kernels.

The radiance cache has no counterpart in the reference (glowing-chemist/Pico
renders without one), so this oracle cannot be pinned to reference outputs:
parity is unpinned against the reference.  It restates the published methods
the device code follows and is pinned by consistency instead (its hand-written
backward pass against torch autograd, tests/test_nrc_oracle.py):

  * multiresolution hash encoding: Mueller, Evans, Schied, Keller 2022,
    "Instant neural graphics primitives with a multiresolution hash encoding"
    (16 levels, 2 features, trilinear interpolation, the spatial hash
    x*1 ^ y*2654435761 ^ z*805459861 modulo the table size, dense indexing
    where a level's grid fits its table);
  * real spherical harmonics of degrees 0-3 of the direction, from their
    definition (normalised associated Legendre functions);
  * the network, loss and training of Mueller, Rousselle, Novak, Keller 2021,
    "Real-time neural radiance caching for path tracing": a 64-wide fully
    connected ReLU network without biases, relative L2 loss with the
    denominator held constant, Adam (Kingma and Ba 2015).

`rounding=True` reproduces where the device rounds to bf16: the network inputs,
the weights, every hidden activation and every back-propagated output gradient;
products accumulate without rounding (fp32 on the device, float64 here).
"""
from __future__ import annotations

import math

import numpy as np

LEVELS, WIDTH, LAYERS, HIDDEN, OUTPUTS = 16, 64, 6, 5, 3
PRIMES = (1, 2654435761, 805459861)
IN_HASH, IN_SH, IN_NORMAL, IN_ROUGH, IN_ALBEDO, IN_BIAS = 0, 32, 48, 51, 52, 55
QUERY_DTYPE = np.dtype([("position", "<f4", (3,)), ("direction", "<f4", (3,)), ("normal", "<f4", (3,)),
                        ("roughness", "<f4"), ("albedo", "<f4", (3,)), ("payload", "<u4"), ("pad", "<u4", (2,))])


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest bf16 (ties to even), returned as float64."""
    f = np.asarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


class Geometry:
    """Per-level scales and dense grid sizes, computed like the library does."""

    def __init__(self, log2_table: int = 19, base: float = 16.0, finest: float = 4096.0,
                 lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
        self.log2_table = log2_table
        self.T = 1 << log2_table
        b = math.exp((math.log(float(np.float32(finest))) - math.log(float(np.float32(base)))) / (LEVELS - 1))
        self.scale = np.array([np.float32(float(np.float32(base)) * math.pow(b, l)) for l in range(LEVELS)],
                              np.float32)
        self.res1 = []
        for s in self.scale:
            r1 = int(math.floor(float(s))) + 2
            self.res1.append(r1 if r1 ** 3 <= self.T else 0)
        self.lo = np.asarray(lo, np.float32)
        hi = np.asarray(hi, np.float32)
        ext = (hi - self.lo).astype(np.float32)
        self.inv_extent = np.where(ext > 0, np.float32(1.0) / np.where(ext > 0, ext, 1), 0).astype(np.float32)

    def unit(self, pos: np.ndarray) -> np.ndarray:
        """Positions normalised to the unit cube in float32 (the device's arithmetic)."""
        u = ((np.asarray(pos, np.float32) - self.lo) * self.inv_extent).astype(np.float32)
        u = np.where(np.isnan(u), np.float32(0.0), u)      # fmaxf(NaN, 0) = 0 on the device
        return np.clip(u, np.float32(0.0), np.float32(1.0))

    def corners(self, u: np.ndarray, level: int):
        """Table indices (n, 8) and trilinear weights (n, 8) of one level."""
        x = (u * self.scale[level]).astype(np.float32)
        c = np.floor(x)
        f = (x - c).astype(np.float64)
        c = c.astype(np.uint64)
        idx = np.empty((len(u), 8), np.int64)
        w = np.empty((len(u), 8), np.float64)
        r = self.res1[level]
        for k in range(8):
            d = np.array([k & 1, (k >> 1) & 1, k >> 2], np.uint64)
            cc = c + d
            if r:
                idx[:, k] = (cc[:, 0] + r * (cc[:, 1] + r * cc[:, 2])).astype(np.int64)
            else:
                h = (cc[:, 0] * PRIMES[0]) ^ ((cc[:, 1] * PRIMES[1]) & 0xFFFFFFFF) ^ ((cc[:, 2] * PRIMES[2]) & 0xFFFFFFFF)
                idx[:, k] = (h & (self.T - 1)).astype(np.int64)
            ww = np.ones(len(u))
            for a in range(3):
                ww = ww * (f[:, a] if d[a] else 1.0 - f[:, a])
            w[:, k] = ww
        return idx, w


def sh16(d: np.ndarray) -> np.ndarray:
    """Real spherical harmonics of degrees 0-3 of unit directions (n, 3) -> (n, 16), order
    (0,0), (1,-1), (1,0), (1,1), (2,-2), ..., (3,3), with Y_lm = K_lm P_l^|m|(z) times
    sqrt(2) cos(m phi) (m > 0) or sqrt(2) sin(|m| phi) (m < 0), Condon-Shortley phase included."""
    d = np.asarray(d, np.float64)
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    out = np.empty((len(d), 16))
    col = 0
    rho = np.sqrt(x * x + y * y)
    phi = np.arctan2(y, x)
    for l in range(4):
        for m in range(-l, l + 1):
            am = abs(m)
            K = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            # P_l^m(cos theta) = (-1)^m sin^m theta d^m/dz^m P_l(z); sin theta = rho
            P = _legendre_assoc(l, am, z, rho)
            if m == 0:
                out[:, col] = K * P
            elif m > 0:
                out[:, col] = math.sqrt(2) * K * P * np.cos(m * phi)
            else:
                out[:, col] = math.sqrt(2) * K * P * np.sin(am * phi)
            col += 1
    return out


def _legendre_assoc(l: int, m: int, z: np.ndarray, s: np.ndarray) -> np.ndarray:
    """Associated Legendre function P_l^m with the Condon-Shortley phase, s = sin(theta)."""
    coeffs = np.polynomial.legendre.leg2poly([0] * l + [1])          # P_l as a power series in z
    deriv = np.polynomial.polynomial.polyder(coeffs, m) if m else coeffs
    return ((-1) ** m) * (s ** m) * np.polynomial.polynomial.polyval(z, deriv)


def encode(geo: Geometry, table: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Network inputs (n, 64) of query records; table: (levels, T, 2) features (fp16 values)."""
    n = len(q)
    out = np.zeros((n, WIDTH))
    u = geo.unit(q["position"])
    for l in range(LEVELS):
        idx, w = geo.corners(u, l)
        feats = table[l].astype(np.float64)[idx]            # (n, 8, 2)
        out[:, IN_HASH + 2 * l:IN_HASH + 2 * l + 2] = np.einsum("nk,nkf->nf", w, feats)
    out[:, IN_SH:IN_SH + 16] = sh16(q["direction"])
    out[:, IN_NORMAL:IN_NORMAL + 3] = q["normal"]
    out[:, IN_ROUGH] = q["roughness"]
    out[:, IN_ALBEDO:IN_ALBEDO + 3] = q["albedo"]
    out[:, IN_BIAS] = 1.0
    return out


def forward(mlp: np.ndarray, x0: np.ndarray, rounding: bool = True):
    """Network outputs (n, 3) and the layer inputs X_0 .. X_5 (each (n, 64))."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W = [r(mlp[l]) for l in range(LAYERS)]
    xs = [r(x0)]
    for l in range(HIDDEN):
        xs.append(r(np.maximum(xs[-1] @ W[l].T, 0.0)))
    out = xs[-1] @ W[HIDDEN][:OUTPUTS].T
    return out, xs


def loss_and_grad(pred: np.ndarray, target: np.ndarray, n: int | None = None):
    """Relative L2 loss (mean over n records and 3 channels) and its gradient (denominator constant)."""
    n = len(pred) if n is None else n
    den = pred * pred + 0.01
    diff = pred - target
    loss = float(np.sum(diff * diff / den) / (3 * n))
    return loss, 2.0 * diff / den / (3 * n)


def backward(mlp: np.ndarray, xs, dpred: np.ndarray, rounding: bool = True):
    """Weight gradients (6, 64, 64) and the input gradient (n, 64)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W = [r(mlp[l]) for l in range(LAYERS)]
    gW = np.zeros((LAYERS, WIDTH, WIDTH))
    dy = np.zeros((len(dpred), WIDTH))
    dy[:, :OUTPUTS] = dpred
    dy = r(dy)
    for l in range(LAYERS - 1, -1, -1):
        rows = OUTPUTS if l == HIDDEN else WIDTH
        gW[l, :rows] = dy[:, :rows].T @ xs[l]
        dx = dy[:, :rows] @ W[l][:rows]
        if l > 0:
            dy = r(dx * (xs[l] > 0))
        else:
            return gW, dx
    raise AssertionError("unreachable")


def grid_gradient(geo: Geometry, q: np.ndarray, dx0: np.ndarray) -> np.ndarray:
    """Gradient (levels, T, 2) of the hash-grid features from the input gradient."""
    g = np.zeros((LEVELS, geo.T, 2))
    u = geo.unit(q["position"])
    for l in range(LEVELS):
        idx, w = geo.corners(u, l)
        for f in range(2):
            np.add.at(g[l, :, f], idx.reshape(-1), (w * dx0[:, IN_HASH + 2 * l + f][:, None]).reshape(-1))
    return g


def train_gradients(geo: Geometry, mlp: np.ndarray, table: np.ndarray, q: np.ndarray, target: np.ndarray,
                    rounding: bool = True):
    """Loss, network gradient and grid gradient of one batch (records with non-finite targets skipped)."""
    ok = np.isfinite(target).all(axis=1)
    x0 = encode(geo, table, q)
    x0[~ok] = 0.0
    pred, xs = forward(mlp, x0, rounding)
    tgt = np.where(ok[:, None], target, 0.0)
    loss, dpred = loss_and_grad(pred, tgt, len(q))
    dpred[~ok] = 0.0
    loss = float(np.sum(np.where(ok[:, None], (pred - tgt) ** 2 / (pred * pred + 0.01), 0.0)) / (3 * len(q)))
    gW, dx0 = backward(mlp, xs, dpred, rounding)
    dx0[~ok] = 0.0
    return loss, gW, grid_gradient(geo, q[ok], dx0[ok])


def adam(param, m, v, g, step, lr=1e-2, beta1=0.9, beta2=0.99, eps=1e-15):
    """One Adam step in float32, as the device computes it; returns (param, m, v)."""
    f = np.float32
    c1 = f(1.0 / (1.0 - beta1 ** step))
    c2 = f(1.0 / (1.0 - beta2 ** step))
    m = (f(beta1) * m + f(1.0 - beta1) * g).astype(f)
    v = (f(beta2) * v + f(1.0 - beta2) * g * g).astype(f)
    p = (param - f(lr) * (m * c1) / (np.sqrt(v * c2) + f(eps))).astype(f)
    return p, m, v


def make_queries(n: int, seed: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)) -> np.ndarray:
    """Seeded query records: positions in the box, unit directions and normals, roughness and albedo."""
    rng = np.random.default_rng(seed)
    q = np.zeros(n, QUERY_DTYPE)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    q["position"] = lo + (hi - lo) * rng.random((n, 3))
    d = rng.normal(size=(n, 3))
    q["direction"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3))
    q["normal"] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    q["roughness"] = rng.random(n)
    q["albedo"] = rng.random((n, 3))
    q["payload"] = np.arange(n, dtype=np.uint32)
    return q
