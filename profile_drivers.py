"""Small drivers that run one part of the library on synthetic inputs, for profiling
(the commands of the ncu summaries under profiles/; a bench helper, not part of the
package).

    python profile_drivers.py cache [--queries N] [--records N] [--reps K]
        radiance-cache inference over N queries and K training steps over N records
        (uniformly random positions over a 400 x 125 x 400 box, seeded)
    python profile_drivers.py cache-render [--passes K]
        a 1920x1080 render of the lit field through the radiance cache
    python profile_drivers.py render [--estimator E] [--passes K] [--width W --height H]
        a render of the lit field (1920x1080 by default), K samples per pixel, estimator E
        (0 the reference's, 1 the physical one)
    python profile_drivers.py cornell [--passes K]
        K renders of the Cornell box at 256x256, 16 spp, depth 5, denoised
        (after one warm-up render)
    python profile_drivers.py trace [--reps K] [--rays N]
        K closest-hit passes over the instance-field batch (4096 level-4 icospheres,
        N rays: half primary rays of a 4096^2 pinhole, half cosine bounce rays),
        device buffers, after one warm-up pass
    python profile_drivers.py atrous [--reps K]
        K a-trous calls on 1920x1080 device buffers (seeded values), a 512 MiB L2
        flush before each, after one warm-up call
    python profile_drivers.py batch [--renders N] [--scale S]
        N renders of the batched-rendering workload (resolutions times S) in one
        CUDA-graph launch, physical estimator, 2^22-path wavefront, 64-thread
        closest-hit CTAs, 8 branches
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))

import pico_gb300  # noqa: E402
from pico_gb300 import RadianceCache, scenes
from pico_gb300.types import NRC_QUERY_DTYPE

LO, HI = (-200.0, -60.0, -200.0), (200.0, 65.0, 200.0)


def random_queries(n: int, seed: int = 5) -> np.ndarray:
    rng = np.random.default_rng(seed)
    q = np.zeros(n, NRC_QUERY_DTYPE)
    q["position"] = np.asarray(LO) + (np.asarray(HI) - np.asarray(LO)) * rng.random((n, 3))
    for k in ("direction", "normal"):
        d = rng.normal(size=(n, 3))
        q[k] = d / np.linalg.norm(d, axis=1, keepdims=True)
    q["roughness"] = rng.random(n)
    q["albedo"] = rng.random((n, 3))
    return q


def cache(queries: int, records: int, reps: int) -> None:
    import torch
    ctx = pico_gb300.Context(0)
    c = RadianceCache(ctx, seed=3, aabb_min=LO, aabb_max=HI)
    q = random_queries(max(queries, records))
    dq = torch.from_numpy(q.view(np.uint8).copy()).cuda()
    out = torch.empty((queries, 3), dtype=torch.float32, device="cuda")
    tgt = torch.from_numpy(np.random.default_rng(1).gamma(1.0, 1.0, (records, 4)).astype(np.float32)).cuda()
    s = torch.cuda.current_stream().cuda_stream
    for _ in range(reps):
        c.infer_device(dq.data_ptr(), queries, out.data_ptr(), s)
    for _ in range(reps):
        c.train_device(dq.data_ptr(), tgt.data_ptr(), records, True, s)
    torch.cuda.synchronize()
    print(f"cache driver: {reps} inferences of {queries} queries, {reps} training steps of {records} records, "
          f"{c.info()['steps']} optimiser steps")
    c.free()
    ctx.close()


def cache_render(passes: int) -> None:
    ctx = pico_gb300.Context(0)
    scene = scenes.lit_field()
    cam = scenes.lit_field_camera(1920, 1080)
    gs = ctx.upload(scene)
    c = RadianceCache(ctx, seed=3)
    c.attach()
    gs.render(cam, 8, passes, seed=99, estimator=2)
    print("cache-render driver:", c.stats())
    c.free()
    gs.free()
    ctx.close()


def render(estimator: int, passes: int, width: int, height: int) -> None:
    ctx = pico_gb300.Context(0)
    gs = ctx.upload(scenes.lit_field())
    gs.render(scenes.lit_field_camera(width, height), 8, passes, seed=99, estimator=estimator, cancellable=False)
    print("render driver:", ctx.render_stats())
    gs.free()
    ctx.close()


def cornell(passes: int) -> None:
    ctx = pico_gb300.Context(0)
    gs = ctx.upload(scenes.cornell_box())
    cam = scenes.cornell_camera(256, 256)
    for k in range(passes + 1):
        gs.render(cam, 5, 16, seed=11 + k, denoise=True)
    print("cornell driver:", ctx.render_stats())
    gs.free()
    ctx.close()


def trace(reps: int, nrays: int) -> None:
    import torch
    ctx = pico_gb300.Context(0)
    scene = scenes.instance_field(n_instances=4096, level=4, seed=12345)
    rays = scenes.field_rays(scene, n_total=nrays, resolution=4096, seed=7)
    gs = ctx.upload(scene)
    d_rays = torch.from_numpy(rays.view(np.uint8)).cuda()
    d_hits = torch.empty(len(rays) * 20, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    for _ in range(reps + 1):
        gs.trace_closest_device(d_rays.data_ptr(), len(rays), d_hits.data_ptr(), s)
    gs.check(s)
    print(f"trace driver: {reps + 1} passes of {len(rays)} rays")
    gs.free()
    ctx.close()


def atrous(reps: int) -> None:
    import torch
    ctx = pico_gb300.Context(0)
    W, H = 1920, 1080
    rng = np.random.default_rng(5)
    bufs = [torch.from_numpy(a).cuda() for a in (
        rng.gamma(1.0, 1.0, (H, W, 3)).astype(np.float32), rng.normal(size=(H, W, 3)).astype(np.float32),
        (rng.normal(size=(H, W, 3)) * 3).astype(np.float32), rng.random((H, W, 3)).astype(np.float32))]
    out = torch.empty_like(bufs[0])
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    for _ in range(reps + 1):
        flush.fill_(1)
        ctx.atrous_device(*[b.data_ptr() for b in bufs], W, H, out.data_ptr(), s)
    torch.cuda.synchronize()
    print(f"atrous driver: {reps + 1} calls")
    ctx.close()


def batch(renders: int, scale: float) -> None:
    ctx = pico_gb300.Context(0)
    work = scenes.batch_workload(renders, size_scale=scale)
    gsc = [ctx.upload(w["scene"]) for w in work]
    items = [{"gpu_scene": g, "camera": w["camera"], "max_samples": w["max_samples"], "max_depth": w["max_depth"],
              "seed": w["seed"], "estimator": 1} for g, w in zip(gsc, work)]
    done, rep = ctx.render_many(items, wavefront=1 << 22, extend_threads=64, branches=8)
    print("batch driver:", rep, "completion p50 %.2f ms" % float(np.percentile(done, 50)))
    for g in gsc:
        g.free()
    ctx.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["cache", "cache-render", "render", "batch", "cornell", "trace", "atrous"])
    ap.add_argument("--rays", type=int, default=1 << 24)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--renders", type=int, default=16)
    ap.add_argument("--scale", type=float, default=0.5)
    ap.add_argument("--queries", type=int, default=1 << 21)
    ap.add_argument("--records", type=int, default=1 << 16)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--passes", type=int, default=3)
    ap.add_argument("--estimator", type=int, default=1)
    a = ap.parse_args()
    if a.what == "cache":
        cache(a.queries, a.records, a.reps)
    elif a.what == "cache-render":
        cache_render(a.passes)
    elif a.what == "render":
        render(a.estimator, a.passes, a.width, a.height)
    elif a.what == "cornell":
        cornell(a.passes)
    elif a.what == "trace":
        trace(a.reps, a.rays)
    elif a.what == "atrous":
        atrous(a.reps)
    else:
        batch(a.renders, a.scale)


if __name__ == "__main__":
    main()
