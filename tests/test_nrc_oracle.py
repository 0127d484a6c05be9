"""The radiance-cache oracle (oracle/po_nrc.py) pinned by consistency on the CPU.

The cache has no counterpart in the reference, so its oracle cannot be checked
against reference outputs; instead its hand-written backward pass, hash-grid
gradient and Adam step are checked against torch autograd / torch.optim in
float64, and its spherical harmonics against their orthonormality.
"""
import numpy as np
import pytest

import po_nrc

torch = pytest.importorskip("torch")


def small_setup(seed=0, n=96, log2=10):
    geo = po_nrc.Geometry(log2_table=log2, base=4.0, finest=64.0, lo=(-1, -2, -3), hi=(2, 1, 4))
    rng = np.random.default_rng(seed)
    table = rng.uniform(-1, 1, (po_nrc.LEVELS, geo.T, 2))
    mlp = np.zeros((6, 64, 64))
    for l in range(6):
        rows = 64 if l < 5 else 3
        mlp[l, :rows] = rng.uniform(-1, 1, (rows, 64)) * np.sqrt(6.0 / (64 + rows))
    q = po_nrc.make_queries(n, seed + 1, lo=(-1, -2, -3), hi=(2, 1, 4))
    target = rng.gamma(1.0, 1.0, (n, 3))
    return geo, table, mlp, q, target


def torch_loss(geo, table, mlp, q, target):
    """The same network and loss in torch float64 with autograd through the table and weights."""
    tt = torch.tensor(table, dtype=torch.float64, requires_grad=True)
    W = torch.tensor(mlp, dtype=torch.float64, requires_grad=True)
    n = len(q)
    u = geo.unit(q["position"])
    cols = []
    for l in range(po_nrc.LEVELS):
        idx, w = geo.corners(u, l)
        feats = tt[l][torch.tensor(idx)]                     # (n, 8, 2)
        cols.append(torch.einsum("nk,nkf->nf", torch.tensor(w), feats))
    rest = torch.tensor(po_nrc.encode(geo, np.zeros_like(table), q)[:, 32:])
    x = torch.cat(cols + [rest], dim=1)
    for l in range(5):
        x = torch.relu(x @ W[l].T)
    pred = x @ W[5][:3].T
    den = (pred * pred + 0.01).detach()
    t = torch.tensor(target)
    loss = ((pred - t) ** 2 / den).sum() / (3 * n)
    loss.backward()
    return float(loss.detach()), W.grad.numpy(), tt.grad.numpy()


def test_backward_matches_autograd():
    geo, table, mlp, q, target = small_setup()
    loss, gW, gG = po_nrc.train_gradients(geo, mlp, table, q, target, rounding=False)
    tl, tW, tG = torch_loss(geo, table, mlp, q, target)
    assert loss == pytest.approx(tl, rel=1e-12)
    np.testing.assert_allclose(gW, tW, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(gG, tG, rtol=1e-9, atol=1e-14)


def test_nonfinite_targets_are_skipped():
    geo, table, mlp, q, target = small_setup(seed=3)
    bad = target.copy()
    bad[::5] = np.nan
    loss, gW, gG = po_nrc.train_gradients(geo, mlp, table, q, bad, rounding=False)
    keep = np.ones(len(q), bool)
    keep[::5] = False
    # the loss is averaged over the whole batch size, so scale the kept-only reference
    tl, tW, tG = torch_loss(geo, table, mlp, q[keep], target[keep])
    s = keep.sum() / len(q)
    assert loss == pytest.approx(tl * s, rel=1e-12)
    np.testing.assert_allclose(gW, tW * s, rtol=1e-9, atol=1e-14)
    np.testing.assert_allclose(gG, tG * s, rtol=1e-9, atol=1e-14)


def test_adam_matches_torch():
    rng = np.random.default_rng(4)
    p0 = rng.normal(size=257).astype(np.float32)
    grads = [rng.normal(size=257).astype(np.float32) * 1e-3 for _ in range(5)]
    tp = torch.tensor(p0.astype(np.float64), requires_grad=True)
    opt = torch.optim.Adam([tp], lr=1e-2, betas=(0.9, 0.99), eps=1e-15)
    p, m, v = p0.copy(), np.zeros_like(p0), np.zeros_like(p0)
    for k, g in enumerate(grads, 1):
        p, m, v = po_nrc.adam(p, m, v, g, k)
        opt.zero_grad()
        tp.grad = torch.tensor(g.astype(np.float64))
        opt.step()
    np.testing.assert_allclose(p, tp.detach().numpy(), rtol=2e-5, atol=1e-6)


def test_sh_orthonormal():
    """Monte Carlo over the sphere: <Y_i, Y_j> = delta_ij."""
    rng = np.random.default_rng(5)
    d = rng.normal(size=(400000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    Y = po_nrc.sh16(d)
    gram = 4 * np.pi * (Y.T @ Y) / len(d)
    np.testing.assert_allclose(gram, np.eye(16), atol=0.02)


def test_hash_and_dense_levels():
    geo = po_nrc.Geometry()
    assert geo.res1[:5] == [18, 25, 35, 50, 72] and all(r == 0 for r in geo.res1[5:])
    u = np.array([[0.0, 0.0, 0.0], [1.0, 1.0, 1.0], [0.5, 0.25, 0.75]], np.float32)
    for l in range(16):
        idx, w = geo.corners(u, l)
        assert idx.min() >= 0 and idx.max() < geo.T
        np.testing.assert_allclose(w.sum(axis=1), 1.0, rtol=1e-12)


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0], np.float32)
    r = po_nrc.bf16(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa (1.0) wins
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] - -3.0e-3) < 2e-5 and r[4] == 65536.0
