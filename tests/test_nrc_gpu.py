"""The radiance cache's device kernels against its oracle and a torch fp32 reference.

Encoding: the 64 network inputs agree with the oracle to 1e-5 (fp32 arithmetic on
fp16 table values).  Network: the tcgen05 forward pass agrees with the oracle,
which rounds to bf16 where the device does, to 2e-2 of the output scale (a
different fp32 summation order can flip a bf16 rounding), and with a plain torch
fp32 network on the same bf16 weights to 5e-2.  Training: the weight and grid
gradients of one batch agree with the oracle's to 3e-2 of their norm, the Adam
step applied to the device's own gradient matches the oracle's Adam to 1e-5, and
a few hundred steps fit a smooth target.
"""
import numpy as np
import pytest

import po_nrc
from pico_gb300 import RadianceCache

pytestmark = pytest.mark.gpu

LO, HI = (-1.0, -2.0, -3.0), (2.0, 1.0, 4.0)


@pytest.fixture(scope="module")
def cache(ctx):
    c = RadianceCache(ctx, log2_table_size=14, aabb_min=LO, aabb_max=HI, seed=3)
    yield c
    c.free()


def geometry(cache):
    cfg = cache.config
    return po_nrc.Geometry(log2_table=cfg.log2_table_size, base=cfg.base_resolution, finest=cfg.max_resolution,
                           lo=LO, hi=HI)


def lively_params(cache, seed):
    """Parameters with O(1) activations: grid features in [-1, 1], Xavier weights."""
    rng = np.random.default_rng(seed)
    mlp = np.zeros((6, 64, 64), np.float32)
    for l in range(6):
        rows = 64 if l < 5 else 3
        mlp[l, :rows] = rng.uniform(-1, 1, (rows, 64)) * np.sqrt(6.0 / (64 + rows)) * 1.5
    grid = rng.uniform(-1, 1, (16, cache.table_size, 2)).astype(np.float32)
    grid = grid.astype(np.float16).astype(np.float32)    # representable in the fp16 table
    cache.set_params(mlp, grid)
    return mlp, grid


def test_encoding_matches_oracle(cache):
    mlp, grid = lively_params(cache, 1)
    q = po_nrc.make_queries(3000, 7, LO, HI)
    q["position"][:5] = [LO, HI, (-5, 0, 0), (0.5, 0.5, 10), (np.nan, 0, 0)]   # corners, outside the box, NaN
    got = cache.encode(q)
    want = po_nrc.encode(geometry(cache), grid, q)
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=2e-6)


@pytest.mark.parametrize("n", [1, 127, 128, 5000])
def test_inference_matches_oracle_and_torch(cache, n):
    torch = pytest.importorskip("torch")
    mlp, grid = lively_params(cache, 2)
    q = po_nrc.make_queries(n, 11 + n, LO, HI)
    got = cache.infer(q)
    geo = geometry(cache)
    x0 = po_nrc.encode(geo, grid, q)
    want, _ = po_nrc.forward(mlp, x0, rounding=True)
    scale = max(np.abs(want).max(), 1e-3)
    assert np.abs(got - want).max() <= 2e-2 * scale
    # plain fp32 network on the bf16 weights and the fp32 inputs
    x = torch.tensor(x0, dtype=torch.float32)
    W = torch.tensor(po_nrc.bf16(mlp), dtype=torch.float32)
    for l in range(5):
        x = torch.relu(x @ W[l].T)
    ref = (x @ W[5][:3].T).numpy()
    assert np.abs(got - ref).max() <= 5e-2 * scale


def test_inference_device_entry(cache, ctx):
    torch = pytest.importorskip("torch")
    lively_params(cache, 3)
    q = po_nrc.make_queries(4096, 5, LO, HI)
    host = cache.infer(q)
    d_q = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    d_out = torch.empty((len(q), 3), dtype=torch.float32, device="cuda")
    cache.infer_device(d_q.data_ptr(), len(q), d_out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(d_out.cpu().numpy(), host)


@pytest.mark.parametrize("n", [100, 128 * 160 + 37])
def test_gradients_match_oracle(cache, n):
    mlp, grid = lively_params(cache, 4)
    q = po_nrc.make_queries(n, 21, LO, HI)
    rng = np.random.default_rng(22)
    target = rng.gamma(1.0, 1.0, (n, 3)).astype(np.float32)
    target[::17] = np.nan                                   # skipped records
    loss = cache.train(q, target, apply=False)
    gW, gG = cache.gradients()
    geo = geometry(cache)
    wl, wW, wG = po_nrc.train_gradients(geo, mlp, grid, q, target.astype(np.float64), rounding=True)
    assert loss == pytest.approx(wl, rel=2e-2)
    for l in range(6):
        rows = 64 if l < 5 else 3
        a, b = gW[l, :rows], wW[l, :rows]
        assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b), f"layer {l}"
        assert np.all(gW[5, 3:] == 0)
    assert np.linalg.norm(gG - wG) <= 3e-2 * np.linalg.norm(wG)


def test_adam_step_matches_oracle(cache):
    mlp, grid = lively_params(cache, 5)                      # resets the optimiser state
    q = po_nrc.make_queries(2048, 31, LO, HI)
    target = np.random.default_rng(32).gamma(1.0, 1.0, (2048, 3)).astype(np.float32)
    cache.train(q, target, apply=True)
    gW, gG = cache.gradients()                               # the gradient that step applied
    pW, pG = cache.params()
    eW, _, _ = po_nrc.adam(mlp, np.zeros_like(mlp), np.zeros_like(mlp), gW, 1)
    eG, _, _ = po_nrc.adam(grid, np.zeros_like(grid), np.zeros_like(grid), gG, 1)
    np.testing.assert_allclose(pW[:5], eW[:5], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(pW[5, :3], eW[5, :3], rtol=1e-5, atol=1e-6)
    assert np.all(pW[5, 3:] == 0)
    np.testing.assert_allclose(pG, eG, rtol=1e-5, atol=1e-6)
    assert cache.info()["steps"] == 1


def test_invalid_configurations_and_arguments(ctx):
    from pico_gb300 import PicoError
    from pico_gb300.types import ESTIMATOR_RADIANCE_CACHE
    from pico_gb300 import scenes
    bad = [dict(log2_table_size=9), dict(log2_table_size=23), dict(base_resolution=0.5),
           dict(base_resolution=64.0, max_resolution=32.0), dict(learning_rate=0.0), dict(beta1=1.0),
           dict(train_batch=0), dict(train_batch=(1 << 20) + 1), dict(bounces=0), dict(infer_groups=3)]
    for cfg in bad:
        with pytest.raises(PicoError) as e:
            RadianceCache(ctx, **cfg)
        assert e.value.status == -1, cfg
    # a render through the cache without one attached is refused before any work
    gs = ctx.upload(scenes.cornell_box())
    ctx.lib.pico_gpu_set_radiance_cache(ctx.handle, None)
    with pytest.raises(PicoError) as e:
        gs.render(scenes.cornell_camera(8, 8), 5, 1, estimator=ESTIMATOR_RADIANCE_CACHE)
    assert e.value.status == -1
    gs.free()
    # a training batch over 2^20 records is refused
    c = RadianceCache(ctx, log2_table_size=12)
    big = np.zeros((1 << 20) + 1, po_nrc.QUERY_DTYPE)
    with pytest.raises(PicoError) as e:
        c.train(big, np.zeros((len(big), 3), np.float32))
    assert e.value.status == -1 and c.info()["steps"] == 0
    assert c.infer(big[:0]).shape == (0, 3)     # an empty query batch is fine
    c.free()


def test_training_fits_a_smooth_target(ctx):
    c = RadianceCache(ctx, log2_table_size=16, aabb_min=LO, aabb_max=HI, seed=9)
    try:
        rng = np.random.default_rng(40)

        def field(q):
            p = q["position"].astype(np.float64)
            d = q["direction"].astype(np.float64)
            base = 1.0 + 0.5 * np.sin(2.0 * p[:, 0]) * np.cos(1.5 * p[:, 1]) + 0.3 * p[:, 2] / 4
            return np.stack([base * (1.2 + 0.5 * d[:, 0]), base * (1.0 + 0.3 * d[:, 1]), base * 0.8 * q["albedo"][:, 2]
                             + 0.1], 1).astype(np.float32)

        test_q = po_nrc.make_queries(4096, 41, LO, HI)
        first = None
        for step in range(300):
            q = po_nrc.make_queries(8192, 100 + step, LO, HI)
            loss = c.train(q, field(q))
            first = loss if first is None else first
        pred = c.infer(test_q)
        t = field(test_q)
        rel = np.mean((pred - t) ** 2 / (t ** 2 + 0.01))
        assert loss < 0.05 * first
        assert rel < 0.01
        assert c.info()["steps"] == 300
    finally:
        c.free()


def test_a_wait_that_runs_out_reports_a_timeout_and_the_context_stays_usable(ctx):
    """The kernels' mbarrier waits are bounded: with the inference's weight-load barrier expecting
    bytes that never arrive (the copy itself completes), the wait gives up after its limit, the
    call returns PICO_ERR_TIMEOUT, and the same cache then infers as before."""
    import pico_gb300
    c = RadianceCache(ctx, log2_table_size=14, aabb_min=LO, aabb_max=HI, seed=3)
    try:
        lively_params(c, 2)
        q = po_nrc.make_queries(300, 8, LO, HI)
        want = c.infer(q)
        c.set_wait_limit(limit_ns=2_000_000, withheld_bytes=16)
        with pytest.raises(pico_gb300.PicoError) as err:
            c.infer(q)
        assert err.value.status == -5          # PICO_ERR_TIMEOUT
        c.set_wait_limit()                     # defaults: 1 s, nothing withheld
        np.testing.assert_array_equal(c.infer(q), want)
        with pytest.raises(pico_gb300.PicoError):
            c.set_wait_limit(limit_ns=0)
        with pytest.raises(pico_gb300.PicoError):
            c.set_wait_limit(withheld_bytes=8)
    finally:
        c.free()
