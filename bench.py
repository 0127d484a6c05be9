"""Benchmark: path-traced 1080p renders (Msamples/s, with Mrays/s beside it).

Headline workload (the metric's own configuration): the lit field -- 4096
instances of a level-4 icosphere (5120 triangles each) under random translation,
log-uniform scale and random rotation, metalness-roughness materials, a ground
quad and 8 quad area lights -- rendered at 1920 x 1080, 64 samples per pixel,
path depth 8, a-trous denoised, with the reference's estimator
(Monte_Carlo_Integrator, Render/Integrators.cpp:46-209, and the render loop of
Scene::render_scene_to_memory, Core/Scene.cpp:143-235, early exit included).
One step = one whole render of the image from cleared buffers.

  value   samples/s with the scene and the image buffers in HBM
          (pico_gpu_render_device), CUDA events on the launching stream.
  e2e     samples/s through pico_gpu_render with pinned host buffers: every step
          copies the progressive buffers in and the image, counts and variance out.
  roofline  the closest-hit (extend) kernel, 90 % of a render's GPU time: its
          algorithmic bytes (64 B per node visited, 48 B per triangle tested,
          144 B per instance entry, 52 B of ray and hit per ray; counted by the
          counting variant of the same launches on the same render) over its
          launches' durations (CUDA events around every launch of the timed
          renders), against the L2 read bandwidth measured in the same run (the
          scene data stays in L2), with the fraction of HBM beside it.
  cpu_baseline / --impl reference
          the reference's render loop on this machine's host cores, on a seeded
          subset of the same image's pixels: the reference's own code where its
          harness is built here (oracle/_ref), else the oracle port.

Secondary objects on the same line: the closest-hit microbench (16,777,216 rays on
the instance field), the physical estimator at 1080p, the radiance-cache series,
batched renders, the Cornell box, a-trous, tone map and .hdr output.

With --gpus N under torchrun each rank renders the whole image on its own GPU
(replicas: the path does not shard) and value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

from pico_gb300 import scenes  # noqa: E402
from pico_gb300.types import HIT_DTYPE, RAY_DTYPE  # noqa: E402

RAY_BYTES, HIT_BYTES = RAY_DTYPE.itemsize, HIT_DTYPE.itemsize
NODE_BYTES, TRI_BYTES, INST_BYTES = 64, 48, 144
SHADE_VERTEX_BYTES = 32 + 2 * 64 + 8   # material, path state read + written, queue entries (per shaded vertex)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--rays", type=int, default=1 << 24)
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--level", type=int, default=4)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-sample", type=int, default=1 << 22)
    ap.add_argument("--order", type=int, default=0, choices=[0, 1],
                    help="traversal order: 0 near-first (default), 1 the reference's child order")
    ap.add_argument("--no-render", action="store_true", help="skip the 1080p render and a-trous measurements")
    ap.add_argument("--render-spp", type=int, default=64)
    ap.add_argument("--render-depth", type=int, default=8)
    ap.add_argument("--render-cpu-pixels", type=int, default=32768,
                    help="seeded pixels of the 1080p image the CPU baseline renders")
    ap.add_argument("--headline", choices=["render", "trace"], default="render",
                    help="the line's headline: the 1080p render (default) or the closest-hit microbench")
    ap.add_argument("--nrc-passes", type=int, nargs="*", default=[16, 32, 64, 96, 128])
    ap.add_argument("--batch-renders", type=int, default=64, help="renders of the batched-rendering line (0: skip)")
    return ap.parse_args()


def workload(args):
    scene = scenes.instance_field(n_instances=args.instances, level=args.level, seed=12345)
    rays = scenes.field_rays(scene, n_total=args.rays, resolution=4096, seed=7)
    return scene, rays


def config_of(args, n_gpus):
    return {"workload": f"instance field: {args.instances} x level-{args.level} icosphere "
                        f"({20 * 4 ** args.level} tris each), {args.rays} rays (50% primary 4096^2 pinhole, "
                        f"50% cosine bounce from surface points)",
            "instances": args.instances, "triangles_per_mesh": 20 * 4 ** args.level, "rays": args.rays,
            "l2": (f"inputs larger than L2 (rays {args.rays * 32 >> 20} MiB + hits {args.rays * 20 >> 20} MiB "
                   f"per step)" if args.rays * 52 > 129 << 20 else
                   f"inputs smaller than L2 (rays + hits {args.rays * 52 >> 20} MiB)"),
            "parallelism": f"replicas x{n_gpus}"}


def cpu_sample(rays, k):
    step = max(1, len(rays) // k)
    return np.ascontiguousarray(rays[::step][:k])


def cpu_trace(scene, rays, nthreads=0):
    """Times the reference algorithm on host cores; returns (kind, seconds, threads)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pico_oracle
    cores = os.cpu_count() or 1
    try:
        ref = pico_oracle.Reference()
        rs = ref.scene(scene)
        _, secs = rs.trace_timed(rays, nthreads)
        return "reference", secs, nthreads or cores
    except (FileNotFoundError, OSError):
        pass
    o = pico_oracle.Oracle()
    os_ = o.scene(scene)
    t0 = time.perf_counter()
    os_.trace(rays, nthreads)
    return "port", time.perf_counter() - t0, nthreads or cores


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.reader.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() in ("active", "0x1") or val.startswith("Active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        busy = [s for s in sm if s > 0.5 * max(sm)]
        return {"sm_mhz": float(np.median(busy)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def max_over_ranks(x: float, dist, device) -> float:
    """The slowest rank's time (replicas: every rank traces the whole batch)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: int, world: int, seconds: float) -> float:
    """Whole-job throughput in millions of units per second: every rank processed its
    own units in at most `seconds` (the max over ranks)."""
    return world * units_per_rank / seconds / 1e6


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dram_traffic_per_ray():
    """DRAM bytes per ray measured by ncu for the closest-hit kernel (profiles/trace_kernel_dram.txt)."""
    p = ROOT / "profiles" / "trace_kernel_dram.txt"
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) == 2 and parts[0] == "dram_bytes_per_ray":
                return float(parts[1])
    return None


ATROUS_BYTES_PER_PIXEL_LEVEL = 60   # 4 x 12 B in (colour, normal, position, albedo) + 12 B out
L2_FLUSH_BYTES = 512 << 20


class PinnedImage:
    """Pinned host image buffers of one resolution, reused by every wall-clock render measurement
    (as the headline's end-to-end leg): pico_gpu_render from and into page-locked memory, without a
    cancel flag.  `render` returns its wall time; the image stays in .pix until the next render."""

    def __init__(self, torch, cam):
        W, H = cam.resolution
        self._keep = [torch.zeros((H, W, 3), dtype=torch.float32).pin_memory(),
                      torch.zeros((H, W, 3), dtype=torch.float32).pin_memory(),
                      torch.zeros((H, W), dtype=torch.int32).pin_memory()]
        self.pix, self.var = self._keep[0].numpy(), self._keep[1].numpy()
        self.cnt = self._keep[2].numpy().view(np.uint32)

    def render(self, gs, cam, depth, spp, seed, **kw):
        self.cnt.fill(0)
        t0 = time.perf_counter()
        gs.render(cam, depth, spp, seed=seed, pixels=self.pix, sample_count=self.cnt, variance=self.var,
                  cancellable=False, **kw)
        return time.perf_counter() - t0


def bench_render(ctx, args, torch, local, estimator=0, with_cpu=True):
    """1080p render of the lit field through pico_gpu_render (host buffers in and out, denoised):
    wall time per render, samples added and rays traced (camera, bounce, shadow, G-buffer).
    estimator 0 is the reference's estimator, 1 the physical one (NEE + BSDF sampling with MIS)."""
    scene = scenes.lit_field()
    cam = scenes.lit_field_camera(1920, 1080)
    gs = ctx.upload(scene)
    img = PinnedImage(torch, cam)
    img.render(gs, cam, args.render_depth, 2, 99, denoise=True, estimator=estimator)          # warm-up
    runs = []
    with ClockSampler(local) as clocks:
        for k in range(2):
            secs = img.render(gs, cam, args.render_depth, args.render_spp, 1 + k, denoise=True, estimator=estimator)
            runs.append((secs, ctx.render_stats()))
    secs = float(np.mean([r[0] for r in runs]))
    st = runs[-1][1]
    rays = st["camera_paths"] + st["bounce_rays"] + st["shadow_rays"] + st["gbuffer_rays"]
    name = "physical estimator (GGX, NEE + BSDF sampling with MIS, RR from depth 3)" if estimator else \
        "reference estimator"
    out = {"workload": f"lit field (4096 level-4 icospheres, ground quad, 8 quad lights), 1920x1080, "
                       f"{args.render_spp} spp, depth {args.render_depth}, a-trous denoise, {name}",
           "Msamples_per_s": st["samples"] / secs / 1e6, "Mrays_per_s": rays / secs / 1e6,
           "ms_per_render": secs * 1e3, "samples": st["samples"], "camera_paths": st["camera_paths"],
           "rays": {k: st[k] for k in ("camera_paths", "bounce_rays", "shadow_rays", "gbuffer_rays")},
           "timing": "wall clock around pico_gpu_render, pinned host buffers in and out",
           "clocks": clocks.summary()}
    conv = convergence(ctx, gs, scene, cam, args, img, estimator)
    if conv:
        out["relmse"] = conv
    if with_cpu and not args.no_cpu and args.render_cpu_pixels > 0 and estimator == 0:
        out["cpu_baseline"] = cpu_render(scene, cam, args)
    gs.free()
    return out


def convergence(ctx, gs, scene, cam, args, img, estimator=0):
    """relMSE against the converged judge of the lit field (FP64 mean of 4096 samples on 1024
    seeded pixels, of the reference's integrator or, for the physical estimator, of its FP64
    oracle): of the timed render, and of plain renders at 64 and 256 spp (the reference
    estimator without its early exit), noisy and after the a-trous pass, with their wall time.
    `img` holds the timed render (PinnedImage) and renders the plain ones."""
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from judge import Judge
    try:
        j = Judge("lit_phys" if estimator else "lit")
        j.check_scene(scene)
    except (OSError, KeyError, ValueError):
        return None
    if (j.width, j.height) != tuple(cam.resolution) or j.depth != args.render_depth:
        return None
    W, H = cam.resolution
    timed = j.relmse_finite(img.pix)
    nrm, pos, dif = gs.denoiser_inputs(cam)
    series = []
    for spp in (64, 256):
        secs = img.render(gs, cam, args.render_depth, spp, 500 + spp, max_variance=-1.0, estimator=estimator)
        pix = img.pix
        den, bad = j.relmse_finite(ctx.atrous(pix, nrm, pos, dif, W, H))
        series.append({"spp": spp, "seconds": secs, "relmse": j.relmse(pix), "relmse_denoised": den,
                       "denoised_nan_pixels": bad})
    source = "samples of the FP64 oracle of the physical estimator" if estimator else \
        "reference samples (Integrators.cpp:130-154)"
    return {"judge": f"FP64 mean of {j.spp} {source} on {len(j.pixels)} seeded pixels", "eps": 0.01,
            "timed_render": timed[0], "timed_render_nan_pixels": timed[1],
            "timed_render_note": ("denoised" if estimator else "denoised, reference early exit") +
                                 "; relMSE over the finite judged pixels",
            "plain_no_early_exit": series}


NRC_FLOPS_PER_QUERY = 2 * (5 * 64 * 64 + 64 * 3)   # five 64x64 layers and the 64 -> 3 output


def bench_radiance_cache(ctx, args, torch, local, plain_series):
    """The radiance-cache form on the lit field at 1920x1080, depth 8: wall time and relMSE
    (against the FP64 judge of the physical estimator) of renders of N passes from a fresh
    cache, next to the plain physical tracer's relMSE at 256 spp; plus the inference and
    training kernels timed alone with CUDA events (tensor roofline of the inference)."""
    from pico_gb300 import RadianceCache
    sys.path.insert(0, str(ROOT / "tests" / "golden"))
    from judge import Judge
    scene = scenes.lit_field()
    cam = scenes.lit_field_camera(1920, 1080)
    gs = ctx.upload(scene)
    try:
        j = Judge("lit_phys")
        j.check_scene(scene)
    except (OSError, KeyError, ValueError):
        j = None
    img = PinnedImage(torch, cam)
    cfg = dict(seed=3)
    warm = RadianceCache(ctx, **cfg)
    warm.attach()
    img.render(gs, cam, args.render_depth, 2, 98, estimator=2)
    warm.free()
    series = []
    with ClockSampler(local) as clocks:
        for n in args.nrc_passes:
            c = RadianceCache(ctx, **cfg)
            c.attach()
            secs = img.render(gs, cam, args.render_depth, n, 700 + n, estimator=2)
            pix = img.pix
            st, rs = c.stats(), ctx.render_stats()
            rays = rs["camera_paths"] + rs["bounce_rays"] + rs["shadow_rays"]
            series.append({"passes": n, "seconds": secs, "relmse": j.relmse(pix) if j else None,
                           "Msamples_per_s": rs["samples"] / secs / 1e6, "Mrays_per_s": rays / secs / 1e6,
                           "train_paths": st["train_paths"], "train_records": st["train_records"],
                           "train_steps": st["train_steps"], "cache_queries": st["queries"]})
            c.free()
    # the cache's error floor and pass cost without training: a cache trained over 256 passes,
    # copied into a cache that does not train (no training paths, no optimiser steps), renders N
    # passes; the time leaves out the training, so this bounds what any online schedule can reach
    frozen = []
    if j is not None:
        trained = RadianceCache(ctx, **cfg)
        trained.attach()
        img.render(gs, cam, args.render_depth, 256, 880, estimator=2)
        mlp, grid = trained.params()
        trained.free()
        fz = RadianceCache(ctx, **cfg, train_paths=0, max_train_steps=0)
        fz.set_params(mlp, grid)
        fz.attach()
        img.render(gs, cam, args.render_depth, 2, 881, estimator=2)   # warm-up
        for n in (16, 32, 64, 128):
            secs = img.render(gs, cam, args.render_depth, n, 900 + n, estimator=2)
            frozen.append({"passes": n, "seconds": secs, "relmse": j.relmse(img.pix)})
        fz.free()
    out = {"workload": f"lit field 1920x1080, depth {args.render_depth}, radiance cache (16-level hash grid 2^19, "
                       f"SH4, 5 x 64 ReLU, bf16 tcgen05), 65536 training paths and up to 4 Adam steps of 65536 "
                       f"records per pass, paths end after 1 bounce (2 behind roughness < 0.1)",
           "timing": "wall clock around pico_gpu_render (pinned host buffers in and out), fresh cache per render",
           "series": series, "clocks": clocks.summary(),
           "pretrained_frozen": {"series": frozen,
                                 "note": "a cache trained over a 256-pass render, copied into a cache that does not "
                                         "train, renders N passes: its relMSE approaches the trained cache's error "
                                         "floor, its time is the pass cost without training (training excluded)"}}
    if len(frozen) >= 2:
        # relMSE ~ a / N + floor, least squares over the series
        A = np.array([[1.0 / f["passes"], 1.0] for f in frozen])
        a, floor = np.linalg.lstsq(A, np.array([f["relmse"] for f in frozen]), rcond=None)[0]
        out["pretrained_frozen"]["fit"] = {"variance_term": float(a), "floor": float(floor),
                                           "ms_per_pass": float(np.mean([f["seconds"] / f["passes"] for f in frozen])
                                                                * 1e3)}
    plain = {p["spp"]: p for p in plain_series or []}
    if j is not None and 256 in plain:
        target, budget = plain[256]["relmse"], plain[256]["seconds"]
        reached = [s for s in series if s["relmse"] is not None and s["relmse"] <= target]
        out["target"] = {"plain_256spp_relmse": target, "plain_256spp_seconds": budget,
                         "cache_seconds_to_target": min((s["seconds"] for s in reached), default=None),
                         "best_cache_relmse": min(s["relmse"] for s in series),
                         "cache_relmse_within_a_third": min((s["relmse"] for s in series
                                                             if s["seconds"] <= budget / 3), default=None)}
        if 64 in plain:
            eq = [s for s in series if s["seconds"] <= plain[64]["seconds"] * 1.05]
            out["target"]["equal_time_vs_plain_64spp"] = {
                "plain_relmse": plain[64]["relmse"], "plain_seconds": plain[64]["seconds"],
                "cache_relmse": min((s["relmse"] for s in eq), default=None)}
    out["kernels"] = bench_cache_kernels(ctx, torch, local)
    gs.free()
    return out


class MeasuredL2:
    """The L2 read bandwidth measured at the start of the run (GB/s), for the secondary rooflines."""
    gbs = None


def bench_cache_kernels(ctx, torch, local):
    """Inference over 2^21 queries and one training step over 2^16 records, device buffers."""
    from pico_gb300 import RadianceCache
    from pico_gb300.types import NRC_QUERY_DTYPE
    lo, hi = (-200.0, -60.0, -200.0), (200.0, 65.0, 200.0)
    c = RadianceCache(ctx, seed=3, aabb_min=lo, aabb_max=hi)
    n = 1 << 21
    rng = np.random.default_rng(5)
    q = np.zeros(n, NRC_QUERY_DTYPE)
    q["position"] = np.asarray(lo) + (np.asarray(hi) - np.asarray(lo)) * rng.random((n, 3))
    for k in ("direction", "normal"):
        d = rng.normal(size=(n, 3))
        q[k] = d / np.linalg.norm(d, axis=1, keepdims=True)
    q["roughness"] = rng.random(n)
    q["albedo"] = rng.random((n, 3))
    dev = f"cuda:{local}"
    dq = torch.from_numpy(q.view(np.uint8).copy()).to(dev)
    dout = torch.empty((n, 3), dtype=torch.float32, device=dev)
    s = torch.cuda.current_stream()

    def timed(fn, reps=20):
        for _ in range(3):
            fn()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(reps):
            fn()
        b.record(s)
        b.synchronize()
        return a.elapsed_time(b) / reps

    ms_inf = timed(lambda: c.infer_device(dq.data_ptr(), n, dout.data_ptr(), s.cuda_stream))
    per_groups = {}
    for groups in (1, 2, 4):
        cg = RadianceCache(ctx, seed=3, aabb_min=lo, aabb_max=hi, infer_groups=groups)
        per_groups[str(groups)] = timed(lambda: cg.infer_device(dq.data_ptr(), n, dout.data_ptr(), s.cuda_stream))
        cg.free()
    nt = 1 << 16
    tt = torch.from_numpy(np.random.default_rng(1).gamma(1.0, 1.0, (nt, 4)).astype(np.float32)).to(dev)
    ms_train = timed(lambda: c.train_device(dq.data_ptr(), tt.data_ptr(), nt, True, s.cuda_stream))
    c.free()
    peak = measured_bf16_peak()
    ach = NRC_FLOPS_PER_QUERY * n / (ms_inf / 1e3) / 1e12
    # the hash-grid encoding against the L2 (the 32 MiB table stays in L2): 16 levels x 8 corners
    # of 4-byte features per query, each gather a 32-byte sector
    gather_bytes = n * 16 * 8 * 32 / (ms_inf / 1e3) / 1e9
    l2 = MeasuredL2.gbs
    gather = {"bound": "l2", "achieved": gather_bytes, "unit": "GB/s",
              "sector_bytes_per_query": 16 * 8 * 32, "algorithmic_bytes_per_query": 16 * 8 * 4,
              "note": "sector traffic of the corner gathers (an upper bound: neighbouring corners of the dense "
                      "levels can share a sector)"}
    if l2:
        gather.update({"peak": l2, "frac": gather_bytes / l2,
                       "peak_source": "measured in this run: L2 read bandwidth (pico_gpu_l2_read_bandwidth)"})
    return {"inference": {"queries": n, "ms": ms_inf, "Mqueries_per_s": n / ms_inf / 1e3,
                          "ms_by_warpgroups_per_cta": per_groups,
                          "queries_note": "uniformly random positions over the lit field's box: incoherent "
                                          "hash-grid gathers (render queries are coherent)",
                          "roofline": {"bound": "tensor", "achieved": ach, "peak": peak[0], "unit": "TFLOP/s",
                                       "frac": ach / peak[0], "peak_source": peak[1],
                                       "algorithmic_flops_per_query": NRC_FLOPS_PER_QUERY},
                          "gather_roofline": gather,
                          "encoding_bytes_per_query": 16 * 8 * 4},
            "training_step": {"records": nt, "ms": ms_train,
                              "note": "grid-gradient clear, fused forward+backward, weight-gradient reduction and "
                                      "Adam over the network and all 16 x 2^19 x 2 grid features"}}


def bench_batch(ctx, args, local):
    """Batched heterogeneous rendering: args.batch_renders renders (resolutions from 128^2 to 1024^2,
    lit fields of 64-4096 instances, 4/16/64 spp, depth 4-8, physical estimator) in one CUDA-graph
    launch with launch parameters chosen by the autotuner; aggregate Msamples/s over the graph's run
    and per-render completion times; the same renders as back-to-back pico_gpu_render calls beside it."""
    work = scenes.batch_workload(args.batch_renders)
    gsc = [ctx.upload(w["scene"]) for w in work]

    def items():
        return [{"gpu_scene": g, "camera": w["camera"], "max_samples": w["max_samples"], "max_depth": w["max_depth"],
                 "seed": w["seed"], "estimator": 1} for g, w in zip(gsc, work)]
    t0 = time.perf_counter()
    best, trials = ctx.autotune_batch(items(), trial_samples=8)
    tune_s = time.perf_counter() - t0
    its = items()
    with ClockSampler(local) as clocks:
        done, rep = ctx.render_many(its, **best)
    t0 = time.perf_counter()
    seq_samples = 0
    for g, w in zip(gsc, work):
        _, cnt, _ = g.render(w["camera"], w["max_depth"], w["max_samples"], seed=w["seed"], estimator=1)
        seq_samples += int(cnt.sum())
    seq_s = time.perf_counter() - t0
    for g in gsc:
        g.free()
    res = sorted({f"{w['camera'].resolution[0]}x{w['camera'].resolution[1]}" for w in work})
    return {"workload": f"{len(work)} renders in one CUDA graph: resolutions {', '.join(res)}, lit fields of "
                        f"{min(w['instances'] for w in work)}-{max(w['instances'] for w in work)} instances, "
                        f"spp 4/16/64, depth 4-8, physical estimator",
            "Msamples_per_s": rep["samples"] / rep["run_ms"] / 1e3, "Mrays_per_s": rep["rays"] / rep["run_ms"] / 1e3,
            "samples": rep["samples"], "run_ms": rep["run_ms"], "graph_build_ms": rep["build_ms"],
            "graph_nodes": rep["graph_nodes"],
            "completion_ms": {"p50": float(np.percentile(done, 50)), "p99": float(np.percentile(done, 99)),
                              "max": float(done.max())},
            "autotuner": {"chosen": best, "seconds": tune_s,
                          "trials": [{"params": t, "Msamples_per_s": r} for t, r in trials]},
            "sequential_calls": {"Msamples_per_s": seq_samples / seq_s / 1e6, "seconds": seq_s,
                                 "note": "the same renders as back-to-back pico_gpu_render calls (host buffers)"},
            "timing": "run_ms: host clock around the graph launch and its completion; completion times from "
                      "device timestamps at the graph start and at the end of each render",
            "clocks": clocks.summary()}


def measured_bf16_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def bench_cornell(ctx, args, torch, local):
    """The reference's CPU-runnable case: the Cornell box at 256x256, 16 spp, depth 5, reference
    estimator, a-trous denoise, through pico_gpu_render (pinned host buffers), next to the reference's
    render loop over the whole image on the host cores (its own code where its harness is built,
    else the port; no denoise on the CPU side)."""
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(256, 256)
    gs = ctx.upload(scene)
    img = PinnedImage(torch, cam)
    img.render(gs, cam, 5, 16, 7, denoise=True)   # warm-up
    times, samples = [], 0
    with ClockSampler(local) as clocks:   # ~0.5 s of renders, long enough for the clock samples
        for k in range(300):
            times.append(img.render(gs, cam, 5, 16, 11 + k, denoise=True))
            samples = ctx.render_stats()["samples"]
    gs.free()
    secs = float(np.median(times))
    out = {"workload": "Cornell box 256x256, 16 spp, depth 5, reference estimator (early exit at zero variance), "
                       "a-trous 5 levels", "ms_per_render": secs * 1e3, "Msamples_per_s": samples / secs / 1e6,
           "samples": samples, "timing": "median wall clock of 300 pico_gpu_render calls, pinned host buffers in and out",
           "clocks": clocks.summary()}
    if not args.no_cpu:
        sys.path.insert(0, str(ROOT / "oracle"))
        import pico_oracle
        W, H = cam.resolution
        idx = np.arange(W * H, dtype=np.uint32)
        seeds = np.random.default_rng(3).integers(1, 2**32 - 1, size=W * H, dtype=np.uint64)
        cores = os.cpu_count() or 1
        try:
            rs = pico_oracle.Reference().scene(scene)
            _, cnt, _, csecs = rs.render_pixels(cam, 5, 16, idx, seeds)
            kind = "reference"
        except (FileNotFoundError, OSError):
            os_ = pico_oracle.Oracle().scene(scene)
            t0 = time.perf_counter()
            _, cnt, _ = os_.render_pixels(cam, 5, 16, idx, seeds)
            csecs = time.perf_counter() - t0
            kind = "port"
        out["cpu_baseline"] = {"value": int(cnt.sum()) / csecs / 1e6, "unit": "Msamples/s", "cores": cores,
                               "kind": kind, "sample": "the whole 256x256 image, 16 spp, depth 5, no denoise",
                               "ms_per_render": csecs * 1e3}
    return out


def cpu_render(scene, cam, args):
    """The reference render loop on host cores over a seeded pixel subset (reference code, else the port)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pico_oracle
    W, H = cam.resolution
    rng = np.random.default_rng(3)
    idx = np.sort(rng.choice(W * H, size=min(args.render_cpu_pixels, W * H), replace=False)).astype(np.uint32)
    seeds = rng.integers(1, 2**32 - 1, size=len(idx), dtype=np.uint64)
    cores = os.cpu_count() or 1
    try:
        rs = pico_oracle.Reference().scene(scene)
        _, cnt, _, secs = rs.render_pixels(cam, args.render_depth, args.render_spp, idx, seeds)
        kind = "reference"
    except (FileNotFoundError, OSError):
        os_ = pico_oracle.Oracle().scene(scene)
        t0 = time.perf_counter()
        _, cnt, _ = os_.render_pixels(cam, args.render_depth, args.render_spp, idx, seeds)
        secs = time.perf_counter() - t0
        kind = "port"
    samples = int(cnt.reshape(-1)[idx].sum())
    return {"value": samples / secs / 1e6, "unit": "Msamples/s", "cores": cores, "kind": kind,
            "sample": f"{len(idx)} seeded pixels of the 1920x1080 image, {args.render_spp} spp, "
                      f"depth {args.render_depth}, reference estimator with its early exit, no denoise",
            "samples": samples, "seconds": secs}


def bench_atrous(ctx, args, torch, local):
    """pico_gpu_atrous_device on 1920x1080 device buffers, L2 flushed before every call."""
    W, H = 1920, 1080
    rng = np.random.default_rng(5)
    dev = f"cuda:{local}"
    bufs = [torch.from_numpy(a).to(dev) for a in (
        rng.gamma(1.0, 1.0, (H, W, 3)).astype(np.float32), rng.normal(size=(H, W, 3)).astype(np.float32),
        (rng.normal(size=(H, W, 3)) * 3).astype(np.float32), rng.random((H, W, 3)).astype(np.float32))]
    out = torch.empty_like(bufs[0])
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    ptrs = [b.data_ptr() for b in bufs]
    for _ in range(3):
        ctx.atrous_device(*ptrs, W, H, out.data_ptr(), stream.cuda_stream)
    times = []
    for _ in range(10):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.atrous_device(*ptrs, W, H, out.data_ptr(), stream.cuda_stream)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    ms = float(np.mean(times))
    algo = ATROUS_BYTES_PER_PIXEL_LEVEL * 5 * W * H
    peak, src = measured_peaks()
    return {"workload": "a-trous, 5 levels, 1920x1080, device buffers, L2 flushed before each call",
            "ms_per_call": ms, "Mpixels_per_s": W * H / (ms / 1e3) / 1e6, "gpu_launches_per_call": 10,
            "roofline": {"bound": "hbm", "achieved": algo / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": algo / (ms / 1e3) / 1e9 / peak, "peak_source": src,
                         "algorithmic_bytes_per_call": algo,
                         "traffic": atrous_traffic_per_call()}}


def bench_tonemap_and_hdr(ctx, args, torch, local):
    """Reinhard tone mapping on a 1920x1080 device image (L2 flushed before each call;
    algorithmic bytes: the white-point pass reads 12 B per pixel, the map reads and
    writes 12 B each) and the Radiance .hdr encoder on the same image from host memory."""
    W, H = 1920, 1080
    rng = np.random.default_rng(6)
    img = rng.gamma(1.0, 1.0, (H, W, 3)).astype(np.float32)
    dev = f"cuda:{local}"
    src = torch.from_numpy(img).to(dev)
    buf = torch.empty_like(src)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    for _ in range(3):
        buf.copy_(src)
        ctx.check(ctx.lib.pico_gpu_tonemap_device(ctx.handle, buf.data_ptr(), W, H, stream.cuda_stream), "tonemap")
    times = []
    for _ in range(10):
        buf.copy_(src)
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        ctx.check(ctx.lib.pico_gpu_tonemap_device(ctx.handle, buf.data_ptr(), W, H, stream.cuda_stream), "tonemap")
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    ms = float(np.mean(times))
    algo = 36 * W * H
    peak, src_ = measured_peaks()
    tonemap = {"workload": "Reinhard tone map, 1920x1080, device buffer, L2 flushed before each call",
               "ms_per_call": ms, "gpu_launches_per_call": 2,
               "roofline": {"bound": "hbm", "achieved": algo / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                            "frac": algo / (ms / 1e3) / 1e9 / peak, "peak_source": src_,
                            "algorithmic_bytes_per_call": algo}}
    ctx.encode_hdr(img, W, H)   # warm-up
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        data = ctx.encode_hdr(img, W, H)
    hdr = {"workload": "stbi_write_hdr-compatible RGBE + run-length encode of a 1920x1080 image, host buffers",
           "ms_per_image": (time.perf_counter() - t0) / reps * 1e3, "file_bytes": len(data)}
    return tonemap, hdr


def atrous_traffic_per_call():
    """DRAM bytes of one 1080p a-trous call measured by ncu (profiles/atrous_1080p.md), if recorded."""
    p = ROOT / "profiles" / "atrous_1080p.md"
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) == 2 and parts[0] == "dram_bytes_per_call":
                return float(parts[1])
    return None


RENDER_WORKLOAD = ("lit field: 4096 x level-4 icosphere (5120 tris each) with metalness-roughness materials, "
                   "ground quad, 8 quad lights; 1920x1080, {spp} spp, depth {depth}, a-trous 5 levels; reference "
                   "estimator (Integrators.cpp:46-209, Scene.cpp:143-235: zero-variance pixels stop at their sixth sample)")


def render_config(args, n_gpus):
    return {"workload": RENDER_WORKLOAD.format(spp=args.render_spp, depth=args.render_depth),
            "resolution": [1920, 1080], "spp": args.render_spp, "max_depth": args.render_depth,
            "instances": 4096, "triangles_per_mesh": 5120, "lights": 8, "denoise": "a-trous 5 levels",
            "seed": "fixed: every step renders the same seed from cleared buffers (identical work per step)",
            "l2": "path state (up to 2^26 paths x 208 B = 14 GB per round) and image buffers (57 MB) exceed L2; "
                  "the scene (1.5 MB) stays in L2 by design",
            "parallelism": f"replicas x{n_gpus}"}


def run_reference(args, rank, world):
    """The reference arm: the reference's CPU implementation on this machine's host cores (rank 0 only)."""
    if rank != 0:
        return
    if args.headline == "trace":
        scene, rays = workload(args)
        sample = cpu_sample(rays, args.cpu_sample)
        times = []
        kind = cores = None
        for i in range(args.warmup + args.steps):
            kind, secs, cores = cpu_trace(scene, sample)
            if i >= args.warmup:
                times.append(secs)
        t = float(np.mean(times))
        v = len(sample) / t / 1e6
        line = {"metric": "Mrays/s", "value": v, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "impl": "reference",
                "config": config_of(args, args.gpus),
                "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": cores, "kind": kind,
                                 "sample": f"{len(sample)} rays, every {len(rays) // len(sample)}th ray of the batch"},
                "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    scene = scenes.lit_field()
    cam = scenes.lit_field_camera(1920, 1080)
    runs = []
    for i in range(args.warmup + args.steps):
        r = cpu_render(scene, cam, args)
        if i >= args.warmup:
            runs.append(r)
    secs = float(np.mean([r["seconds"] for r in runs]))
    v = runs[-1]["samples"] / secs / 1e6
    base = dict(runs[-1])
    base.pop("seconds")
    base["value"] = v
    line = {"metric": "Msamples/s", "value": v, "unit": "Msamples/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "impl": "reference",
            "config": render_config(args, args.gpus), "cpu_baseline": base,
            "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def l2_peak(ctx):
    """L2 read bandwidth measured now (GB/s), the roof of the closest-hit kernels."""
    return ctx.l2_read_bandwidth(32 << 20, 200)


def extend_traffic_per_launch():
    """DRAM bytes per closest-hit launch of the 1080p render, from an ncu capture of the same
    render (profiles/extend_kernel_render_1080p.md), if recorded."""
    p = ROOT / "profiles" / "extend_kernel_render_1080p.md"
    if p.exists():
        for line in p.read_text().splitlines():
            parts = line.split()
            if len(parts) == 2 and parts[0] == "dram_bytes_per_launch":
                return float(parts[1])
    return None


def bench_render_headline(ctx, args, torch, local, dist, world, l2_gbs):
    """The headline: whole 1080p renders of the lit field (reference estimator, denoised) with the image
    buffers in HBM (pico_gpu_render_device, CUDA events), then through pico_gpu_render with pinned host
    buffers (e2e); the extend kernel's roofline from its counted work and its timed launches."""
    scene = scenes.lit_field()
    cam = scenes.lit_field_camera(1920, 1080)
    W, H = cam.resolution
    gs = ctx.upload(scene)
    dev = f"cuda:{local}"
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    d_pix = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
    d_var = torch.zeros((H, W, 3), dtype=torch.float32, device=dev)
    d_cnt = torch.zeros((H, W), dtype=torch.int32, device=dev)
    seed, depth, spp = 1, args.render_depth, args.render_spp

    # a fresh render needs cleared sample counts only: a pixel's mean and variance restart at
    # its first sample (Scene.cpp:185-191)
    def step():
        d_cnt.zero_()
        gs.render_device(cam, depth, spp, d_pix.data_ptr(), d_cnt.data_ptr(), d_var.data_ptr(), sh, seed=seed,
                         denoise=True)

    for _ in range(args.warmup):
        step()
    gs.check(sh)
    # work of one render, counted by the counting variant of the same closest-hit launches
    ctx.set_render_probe(count_work=True)
    step()
    gs.check(sh)
    work = ctx.render_probe_read()
    ctx.set_render_probe(time_extend=True)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        evs[0].record(stream)
        for k in range(args.steps):
            step()
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
    gs.check(sh)
    timing = ctx.render_probe_read()
    ctx.set_render_probe()
    st = ctx.render_stats()
    total_ms = max_over_ranks(evs[0].elapsed_time(evs[-1]), dist, dev)
    ms = total_ms / args.steps
    rays = st["camera_paths"] + st["bounce_rays"] + st["shadow_rays"] + st["gbuffer_rays"]
    value = replica_throughput(st["samples"], world, ms / 1e3)

    # end to end: pico_gpu_render with pinned host buffers in and out every step
    h_pix = torch.zeros((H, W, 3), dtype=torch.float32).pin_memory()
    h_var = torch.zeros((H, W, 3), dtype=torch.float32).pin_memory()
    h_cnt = torch.zeros((H, W), dtype=torch.int32).pin_memory()
    np_pix, np_var, np_cnt = h_pix.numpy(), h_var.numpy(), h_cnt.numpy().view(np.uint32)

    def e2e_step():
        np_cnt.fill(0)
        gs.render(cam, depth, spp, seed=seed, pixels=np_pix, sample_count=np_cnt, variance=np_var, denoise=True,
                  cancellable=False)

    for _ in range(max(1, min(args.warmup, 2))):
        e2e_step()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, dist, dev)
    e2e_samples = ctx.render_stats()["samples"]
    io_bytes = W * H * (12 + 12 + 4)
    e2e = {"value": replica_throughput(e2e_samples, world, e2e_s), "unit": "Msamples/s",
           "h2d_bytes_per_step": io_bytes, "d2h_bytes_per_step": io_bytes, "ms_per_step": e2e_s * 1e3,
           "Mrays_per_s": replica_throughput(rays, world, e2e_s),
           "transfer": "pico_gpu_render from pinned host buffers (mean, count, variance in; denoised image, "
                       "count, variance out), wall clock per call"}

    # roofline of the closest-hit kernel: counted bytes over the timed launches
    launches = timing["launches"] // args.steps
    traced = st["camera_paths"] + st["bounce_rays"] + st["shadow_rays"]
    algo_render = (work["nodes"] * NODE_BYTES + work["tris"] * TRI_BYTES + work["instances"] * INST_BYTES
                   + traced * (RAY_BYTES + HIT_BYTES))
    algo_launch = algo_render / max(launches, 1)
    launch_ms = timing["extend_ms"] / max(timing["launches"], 1)
    achieved = algo_launch / (launch_ms / 1e3) / 1e9
    hbm, hbm_src = measured_peaks()
    roofline = {"bound": "l2", "achieved": achieved, "peak": l2_gbs, "unit": "GB/s", "frac": achieved / l2_gbs,
                "peak_source": "measured in this run: L2 read bandwidth (pico_gpu_l2_read_bandwidth, 32 MiB "
                               "buffer, loads cached in L2 only)",
                "hbm_peak": hbm, "hbm_frac": achieved / hbm, "hbm_peak_source": hbm_src,
                "traffic": extend_traffic_per_launch(),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per extend launch of the same "
                                  "render (profiles/extend_kernel_render_1080p.md)",
                "kernel": "extend_kernel<near-first, 128 threads> (closest hit of path segments and shadow rays)",
                "launches_per_render": launches, "ms_per_launch": launch_ms,
                "extend_ms_per_render": timing["extend_ms"] / args.steps,
                "extend_share_of_step": timing["extend_ms"] / args.steps / ms,
                "algorithmic_bytes_per_launch": algo_launch,
                "work_per_render": {"nodes": work["nodes"], "triangle_tests": work["tris"],
                                    "instance_entries": work["instances"], "rays": traced},
                "bytes_model": "64 B per node visited, 48 B per triangle tested, 144 B per instance entry, "
                               "52 B of ray in / hit out per ray"}
    # the shade kernel against HBM: the per-vertex byte model over its timed launches
    shade_ms = timing["shade_ms"] / args.steps
    shaded = st["camera_paths"] + st["bounce_rays"]   # the path segments the shade launches take
    shade_bytes = shaded * SHADE_VERTEX_BYTES
    shade_rate = shade_bytes / (shade_ms / 1e3) / 1e9 if shade_ms > 0 else 0.0
    shade_roofline = {"bound": "hbm", "achieved": shade_rate, "peak": hbm, "unit": "GB/s",
                      "frac": shade_rate / hbm, "peak_source": hbm_src,
                      "kernel": "shade_kernel (reference estimator)",
                      "launches_per_render": timing["shade_launches"] // args.steps, "ms_per_render": shade_ms,
                      "share_of_step": shade_ms / ms, "vertices_per_render": shaded,
                      "algorithmic_bytes_per_render": shade_bytes,
                      "bytes_model": f"{SHADE_VERTEX_BYTES} B per shaded path vertex: 32 B of material, 2 x 64 B of "
                                     "path state read and written, 8 B of queue entries"}
    # kernels per render: extend and shade per depth; per round plan, raygen, accumulate and the
    # compaction (none after the last round); plan set-up, image preparation, G-buffer, a-trous
    rounds = launches // (depth + 1) if launches else 0
    kernels_per_render = 2 * launches + 4 * rounds - 1 + 2 + 1 + 12
    out = {"value": value, "ms_per_step": ms, "Mrays_per_s": replica_throughput(rays, world, ms / 1e3),
           "samples_per_render": st["samples"], "rays_per_render": {k: st[k] for k in (
               "camera_paths", "bounce_rays", "shadow_rays", "gbuffer_rays")},
           "e2e": e2e, "roofline": roofline, "shade_roofline": shade_roofline, "clocks": clocks.summary(),
           "gpu_launches": kernels_per_render * args.steps}
    gs.free()
    return out


def bench_trace(ctx, args, torch, local, dist, world, l2_gbs):
    """The closest-hit microbench on the instance field: 16,777,216 rays per step, device-resident and
    end to end through the host-buffer entry point; roofline against the measured L2 bandwidth."""
    scene, rays = workload(args)
    n = len(rays)
    ctx.set_traversal_order(args.order)
    gs = ctx.upload(scene)
    info = gs.info()
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    d_rays = torch.from_numpy(rays.view(np.uint8)).to(f"cuda:{local}")
    d_hits = torch.empty(n * HIT_BYTES, dtype=torch.uint8, device=f"cuda:{local}")

    def step():
        gs.trace_closest_device(d_rays.data_ptr(), n, d_hits.data_ptr(), sh)

    for _ in range(args.warmup):
        step()
    gs.check(sh)
    counts = gs.trace_stats(d_rays.data_ptr(), n, sh)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    with ClockSampler(local) as clocks:
        evs[0].record(stream)
        for k in range(args.steps):
            step()
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
    gs.check(sh)
    per_step = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    total_ms = max_over_ranks(evs[0].elapsed_time(evs[-1]), dist, f"cuda:{local}")
    ms = total_ms / args.steps
    value = replica_throughput(n, world, ms / 1e3)
    e2e = None
    if not args.no_e2e:
        h_rays = torch.from_numpy(rays.view(np.uint8)).pin_memory()
        h_hits = torch.empty(n * HIT_BYTES, dtype=torch.uint8).pin_memory()
        in_place = ctx.host_buffer_in_place(h_rays.data_ptr(), n * RAY_BYTES) and \
            ctx.host_buffer_in_place(h_hits.data_ptr(), n * HIT_BYTES)
        for _ in range(max(1, min(args.warmup, 2))):
            gs.trace_closest_ptr(h_rays.data_ptr(), n, h_hits.data_ptr())
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            gs.trace_closest_ptr(h_rays.data_ptr(), n, h_hits.data_ptr())
        e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps, dist, f"cuda:{local}")
        e2e = {"value": replica_throughput(n, world, e2e_s), "unit": "Mrays/s", "h2d_bytes_per_step": n * RAY_BYTES,
               "d2h_bytes_per_step": n * HIT_BYTES, "ms_per_step": e2e_s * 1e3,
               "transfer": ("pinned buffers read and written in place by the kernel over NVLink-C2C" if in_place
                            else "pinned buffers staged through device memory in overlapped 1M-ray chunks")}
    algo_bytes = (counts["nodes"] * NODE_BYTES + counts["tris"] * TRI_BYTES + counts["instances"] * INST_BYTES
                  + n * (RAY_BYTES + HIT_BYTES))
    launch_s = float(np.mean(per_step)) / 1e3
    achieved = algo_bytes / launch_s / 1e9
    hbm, hbm_src = measured_peaks()
    dpr = dram_traffic_per_ray()
    roofline = {"bound": "l2", "achieved": achieved, "peak": l2_gbs, "unit": "GB/s", "frac": achieved / l2_gbs,
                "peak_source": "measured in this run: L2 read bandwidth (pico_gpu_l2_read_bandwidth)",
                "hbm_peak": hbm, "hbm_frac": achieved / hbm, "hbm_peak_source": hbm_src,
                "traffic": dpr * n if dpr else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of trace_kernel on this "
                                  "16,777,216-ray batch (profiles/trace_kernel_dram.txt)",
                "kernel": f"trace_kernel<false, {'near-first' if args.order == 0 else 'reference order'}>",
                "algorithmic_bytes_per_launch": algo_bytes,
                "visits_per_ray": {k: v / n for k, v in counts.items()},
                "bytes_model": "64 B per node visited, 48 B per triangle tested, 144 B per instance entry, "
                               "32 B ray in + 20 B hit out per ray"}
    cpu = None
    if not args.no_cpu:
        sample = cpu_sample(rays, args.cpu_sample)
        kind, secs, cores = cpu_trace(scene, sample)
        cpu = {"value": len(sample) / secs / 1e6, "unit": "Mrays/s", "cores": cores, "kind": kind,
               "sample": f"{len(sample)} rays, every {n // len(sample)}th ray of the batch"}
    gs.free()
    ctx.set_traversal_order(0)
    return {"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "ms_per_step": ms,
            "config": config_of(args, world), "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
            "clocks": clocks.summary(), "scene": info, "gpu_launches": args.steps}


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    import pico_gb300
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    ctx = pico_gb300.Context(local)
    l2_gbs = l2_peak(ctx)
    MeasuredL2.gbs = l2_gbs
    trace = bench_trace(ctx, args, torch, local, dist, world, l2_gbs)
    render = None
    if args.headline == "render":
        render = bench_render_headline(ctx, args, torch, local, dist, world, l2_gbs)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    cpu_render_line = None
    extras = {}
    if not args.no_render:
        scene = scenes.lit_field()
        cam = scenes.lit_field_camera(1920, 1080)
        if not args.no_cpu and args.render_cpu_pixels > 0:
            r = cpu_render(scene, cam, args)
            r.pop("seconds")
            cpu_render_line = r
        extras["cornell_256"] = bench_cornell(ctx, args, torch, local)
        extras["render_1080p_physical"] = bench_render(ctx, args, torch, local, estimator=1)
        extras["render_1080p_relmse"] = bench_render(ctx, args, torch, local, estimator=0, with_cpu=False)
        if args.nrc_passes:
            plain = (extras["render_1080p_physical"].get("relmse") or {}).get("plain_no_early_exit")
            extras["render_1080p_radiance_cache"] = bench_radiance_cache(ctx, args, torch, local, plain)
        if args.batch_renders > 0:
            extras["batched_renders"] = bench_batch(ctx, args, local)
        extras["atrous_1080p"] = bench_atrous(ctx, args, torch, local)
        extras["tonemap_1080p"], extras["hdr_1080p"] = bench_tonemap_and_hdr(ctx, args, torch, local)

    common = {"n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
              "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)"}
    if render is not None:
        line = {"metric": "Msamples/s", "value": render["value"], "unit": "Msamples/s", **common,
                "ms_per_step": render["ms_per_step"], "Mrays_per_s": render["Mrays_per_s"],
                "config": render_config(args, world), "e2e": render["e2e"],
                "gpu_launches": render["gpu_launches"], "roofline": render["roofline"],
                "shade_roofline": render["shade_roofline"],
                "cpu_baseline": cpu_render_line, "clocks": render["clocks"],
                "samples_per_render": render["samples_per_render"], "rays_per_render": render["rays_per_render"],
                "l2_read_gbs": l2_gbs, "traversal_microbench": trace, **extras}
    else:
        line = {**common, **trace, "l2_read_gbs": l2_gbs, **extras}
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
