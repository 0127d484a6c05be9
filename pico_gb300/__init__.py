"""pico_gb300: the Pico path tracer's rendering hot path on one GB300.

The compute path is libpico_gpu.so (hand-written sm_103a kernels behind the C
ABI of include/pico_gpu.h).  This package loads it with ctypes and offers
thin Python handles mirroring the reference's entry points:

    Context.upload(scene)            Scene construction (BLAS/TLAS build + upload)
    GpuScene.trace_closest(rays)     UpperLevelBVH::get_closest_intersection
    GpuScene.render(camera, params)  Scene::render_scene_to_memory
    Context.atrous(...)              Util::atrous_denoise

and the additions without a reference counterpart:

    RadianceCache(ctx, ...)          neural radiance cache (encode / infer / train, attach
                                     for GpuScene.render(..., estimator=2))
    Context.render_many(renders)     many renders in one CUDA graph launch
    Context.autotune_batch(renders)  launch parameters for render_many

There is no CPU fallback: if the library is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .types import (SKY_CONSTANT, SKY_CUBE_RGBA8, SKY_EQUIRECT_RGBAF, Sky, SHAPE_TRIANGLES, SHAPE_SPHERE,  # noqa: F401
                    SHAPE_CUBE, BTDF, FRESNEL, DELTA,  # noqa: F401
                    CCamera, CNrcConfig, CRenderConfig, CSceneDesc, CRenderItem, CLaunchParams, CBatchReport, NRC_QUERY_DTYPE, ESTIMATOR_RADIANCE_CACHE, HIT_DTYPE, RAY_DTYPE, Camera, Instance,  # noqa: F401
                    MarshalledScene, Material, Mesh, SceneData, DIFFUSE, SPECULAR, DIELECTRIC, LIGHT, MISS)

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libpico_gpu.so"

PICO_OK = 0
STATUS_NAMES = {0: "PICO_OK", -1: "PICO_ERR_INVALID_ARG", -2: "PICO_ERR_CUDA", -3: "PICO_ERR_OUT_OF_MEMORY",
                -4: "PICO_ERR_STACK_OVERFLOW", -5: "PICO_ERR_TIMEOUT", -6: "PICO_ERR_CANCELLED",
                -7: "PICO_ERR_NO_DEVICE", -8: "PICO_ERR_UNSUPPORTED"}

# Every symbol include/pico_gpu.h declares, with its ctypes signature.
_vp, _u32, _u64, _i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int32
_fp = C.POINTER(C.c_float)
SIGNATURES = {
    "pico_gpu_init": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "pico_gpu_shutdown": (None, [_vp]),
    "pico_gpu_status_string": (C.c_char_p, [C.c_int]),
    "pico_gpu_last_error": (C.c_char_p, [_vp]),
    "pico_gpu_set_traversal_order": (C.c_int, [_vp, C.c_int]),
    "pico_gpu_set_traversal_limits": (C.c_int, [_vp, _u32, _u32]),
    "pico_gpu_set_triangle_test": (C.c_int, [_vp, C.c_int]),
    "pico_gpu_scene_upload": (C.c_int, [_vp, C.POINTER(CSceneDesc), C.POINTER(_vp)]),
    "pico_gpu_scene_free": (None, [_vp]),
    "pico_gpu_scene_info": (C.c_int, [_vp, C.POINTER(_u64)]),
    "pico_gpu_reference_bvh": (C.c_int, [C.POINTER(CSceneDesc), _i32, _vp, _vp, _vp, C.POINTER(_u32),
                                         C.POINTER(_u32)]),
    "pico_gpu_trace_closest": (C.c_int, [_vp, _vp, _vp, _u64, _vp]),
    "pico_gpu_trace_closest_device": (C.c_int, [_vp, _vp, _vp, _u64, _vp, _vp]),
    "pico_gpu_host_buffer_in_place": (C.c_int, [_vp, _vp, _u64, C.POINTER(_i32)]),
    "pico_gpu_check": (C.c_int, [_vp, _vp]),
    "pico_gpu_trace_stats": (C.c_int, [_vp, _vp, _vp, _u64, C.POINTER(_u64), _vp]),
    "pico_gpu_render": (C.c_int, [_vp, _vp, C.POINTER(CCamera), C.POINTER(CRenderConfig), _fp,
                                  C.POINTER(_u32), _fp, C.POINTER(_i32)]),
    "pico_gpu_render_stats": (C.c_int, [_vp, C.POINTER(_u64)]),
    "pico_gpu_render_device": (C.c_int, [_vp, _vp, C.POINTER(CCamera), C.POINTER(CRenderConfig), _vp, _vp, _vp,
                                         _vp]),
    "pico_gpu_set_render_probe": (C.c_int, [_vp, _i32, _i32]),
    "pico_gpu_set_path_limit": (C.c_int, [_vp, C.c_uint32]),
    "pico_gpu_render_probe_read": (C.c_int, [_vp, C.POINTER(_u64), C.POINTER(C.c_double)]),
    "pico_gpu_render_probe_read_shade": (C.c_int, [_vp, C.POINTER(_u64), C.POINTER(C.c_double)]),
    "pico_gpu_l2_read_bandwidth": (C.c_int, [_vp, _u64, _u32, C.POINTER(C.c_double)]),
    "pico_gpu_denoiser_inputs": (C.c_int, [_vp, _vp, C.POINTER(CCamera), _fp, _fp, _fp]),
    "pico_gpu_atrous": (C.c_int, [_vp, _fp, _fp, _fp, _fp, _u32, _u32, _fp]),
    "pico_gpu_atrous_device": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _u32, _u32, _vp, _vp]),
    "pico_gpu_atrous_device_noalloc": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _u32, _u32, _vp, _vp]),
    "pico_gpu_tonemap": (C.c_int, [_vp, _fp, _u32, _u32]),
    "pico_gpu_tonemap_device": (C.c_int, [_vp, _vp, _u32, _u32, _vp]),
    "pico_gpu_render_to_file": (C.c_int, [_vp, _vp, C.POINTER(CCamera), C.POINTER(CRenderConfig), _fp,
                                          C.POINTER(_u32), _fp, C.c_char_p]),
    "pico_gpu_hdr_bound": (C.c_size_t, [_u32, _u32]),
    "pico_gpu_encode_hdr": (C.c_int, [_vp, _fp, _u32, _u32, _vp, C.c_size_t, C.POINTER(C.c_size_t)]),
    "pico_gpu_bsdf_eval": (C.c_int, [_vp, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "pico_gpu_phys_bsdf_eval": (C.c_int, [_vp, _u64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                          _vp]),
    "pico_gpu_nrc_default_config": (C.c_int, [C.POINTER(CNrcConfig)]),
    "pico_gpu_nrc_create": (C.c_int, [_vp, C.POINTER(CNrcConfig), C.POINTER(_vp)]),
    "pico_gpu_nrc_free": (None, [_vp]),
    "pico_gpu_nrc_get_params": (C.c_int, [_vp, _vp, _vp]),
    "pico_gpu_nrc_set_params": (C.c_int, [_vp, _vp, _vp]),
    "pico_gpu_nrc_set_bounds": (C.c_int, [_vp, _fp, _fp]),
    "pico_gpu_nrc_info": (C.c_int, [_vp, C.POINTER(_u64)]),
    "pico_gpu_nrc_stats": (C.c_int, [_vp, C.POINTER(_u64)]),
    "pico_gpu_nrc_encode": (C.c_int, [_vp, _vp, _u64, _vp]),
    "pico_gpu_nrc_infer": (C.c_int, [_vp, _vp, _u64, _vp]),
    "pico_gpu_nrc_infer_device": (C.c_int, [_vp, _vp, _u64, _vp, _vp]),
    "pico_gpu_nrc_set_wait_limit": (C.c_int, [_vp, _u64, C.c_uint32]),
    "pico_gpu_nrc_train": (C.c_int, [_vp, _vp, _vp, _u64, C.c_int, _fp]),
    "pico_gpu_nrc_train_device": (C.c_int, [_vp, _vp, _vp, _u64, C.c_int, _vp]),
    "pico_gpu_nrc_gradients": (C.c_int, [_vp, _vp, _vp]),
    "pico_gpu_set_radiance_cache": (C.c_int, [_vp, _vp]),
    "pico_gpu_render_many": (C.c_int, [_vp, _u32, _vp, C.POINTER(CLaunchParams), C.POINTER(C.c_double),
                                       C.POINTER(CBatchReport)]),
    "pico_gpu_autotune_batch": (C.c_int, [_vp, _u32, _vp, _u32, C.POINTER(CLaunchParams), C.POINTER(CLaunchParams),
                                          C.POINTER(C.c_double), _u32, C.POINTER(_u32)]),
}

_lib = None


class PicoError(RuntimeError):
    def __init__(self, status: int, message: str = ""):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


def load_library(path: Path | str | None = None) -> C.CDLL:
    """Loads libpico_gpu.so and binds every declared entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -m pico_gb300.build`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def reference_bvh(scene: SceneData, which: int):
    """pico_gpu_reference_bvh (host only): the binary BVH the upload builds, in the reference's
    layout -- which = -1 the TLAS, else mesh `which`'s BLAS -- as (boxes (n, 6), links (n, 4), values)."""
    lib = load_library()
    m = MarshalledScene(scene)
    nn, nv = C.c_uint32(0), C.c_uint32(0)
    st = lib.pico_gpu_reference_bvh(C.byref(m.desc), which, None, None, None, C.byref(nn), C.byref(nv))
    if st != PICO_OK:
        raise PicoError(st, "reference_bvh")
    boxes = np.empty((nn.value, 6), np.float32)
    links = np.empty((nn.value, 4), np.uint32)
    values = np.empty(max(nv.value, 1), np.uint32)
    st = lib.pico_gpu_reference_bvh(C.byref(m.desc), which, boxes.ctypes.data, links.ctypes.data, values.ctypes.data,
                                    C.byref(nn), C.byref(nv))
    if st != PICO_OK:
        raise PicoError(st, "reference_bvh")
    return boxes, links, values[:nv.value]


def _f32(a: np.ndarray):
    return a.ctypes.data_as(_fp)


class Context:
    """pico_gpu_ctx: one device, its streams and scratch buffers."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = _vp()
        st = self.lib.pico_gpu_init(device, C.byref(h))
        if st != PICO_OK:
            raise PicoError(st, "pico_gpu_init")
        self.handle = h

    def check(self, status: int, what: str):
        if status != PICO_OK:
            msg = self.lib.pico_gpu_last_error(self.handle) or b""
            raise PicoError(status, f"{what}: {msg.decode()}")

    def close(self):
        if getattr(self, "handle", None):
            self.lib.pico_gpu_shutdown(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_traversal_order(self, order: int):
        """0: near-first (default), 1: the reference's child order (exact in near-tie cases)."""
        self.check(self.lib.pico_gpu_set_traversal_order(self.handle, order), "set_traversal_order")

    def set_traversal_limits(self, max_iterations: int = 0, stack_entries: int = 0):
        """Bounds of every ray walk of this context (0: the defaults, 2^24 steps and 96 stack entries)."""
        self.check(self.lib.pico_gpu_set_traversal_limits(self.handle, max_iterations, stack_entries),
                   "set_traversal_limits")

    def set_triangle_test(self, test: int):
        """0: the reference's Moeller-Trumbore (default), 1: the watertight test (Woop et al. 2013)."""
        self.check(self.lib.pico_gpu_set_triangle_test(self.handle, test), "set_triangle_test")

    def host_buffer_in_place(self, ptr: int, nbytes: int) -> bool:
        """Whether trace_closest reads / writes the host range [ptr, ptr + nbytes) in place (it lies in one
        page-locked, mapped allocation) rather than staging it through device memory."""
        out = C.c_int32(0)
        self.check(self.lib.pico_gpu_host_buffer_in_place(self.handle, ptr, nbytes, C.byref(out)),
                   "host_buffer_in_place")
        return bool(out.value)

    def set_path_limit(self, max_paths: int = 0):
        """pico_gpu_set_path_limit: the most paths a render batch holds (0: the default, 2^26)."""
        self.check(self.lib.pico_gpu_set_path_limit(self.handle, int(max_paths)), "set_path_limit")

    def set_render_probe(self, time_extend: bool = False, count_work: bool = False):
        """Measurement hooks on the closest-hit launches of renders (events / work counters); clears totals."""
        self.check(self.lib.pico_gpu_set_render_probe(self.handle, int(time_extend), int(count_work)),
                   "set_render_probe")

    def render_probe_read(self) -> dict:
        out = (C.c_uint64 * 4)()
        ms = C.c_double(0.0)
        self.check(self.lib.pico_gpu_render_probe_read(self.handle, out, C.byref(ms)), "render_probe_read")
        n_shade = C.c_uint64(0)
        shade_ms = C.c_double(0.0)
        self.check(self.lib.pico_gpu_render_probe_read_shade(self.handle, C.byref(n_shade), C.byref(shade_ms)),
                   "render_probe_read_shade")
        return {"launches": int(out[0]), "nodes": int(out[1]), "tris": int(out[2]), "instances": int(out[3]),
                "extend_ms": ms.value, "shade_launches": int(n_shade.value), "shade_ms": shade_ms.value}

    def l2_read_bandwidth(self, nbytes: int = 0, passes: int = 0) -> float:
        """Measured L2 read bandwidth in GB/s (pico_gpu_l2_read_bandwidth)."""
        g = C.c_double(0.0)
        self.check(self.lib.pico_gpu_l2_read_bandwidth(self.handle, nbytes, passes, C.byref(g)), "l2_read_bandwidth")
        return g.value

    def render_stats(self) -> dict:
        """Work of the last render: samples added, camera paths, bounce, shadow and G-buffer rays."""
        out = (C.c_uint64 * 5)()
        self.check(self.lib.pico_gpu_render_stats(self.handle, out), "render_stats")
        keys = ["samples", "camera_paths", "bounce_rays", "shadow_rays", "gbuffer_rays"]
        return dict(zip(keys, [int(x) for x in out]))

    def upload(self, scene: SceneData) -> "GpuScene":
        return GpuScene(self, scene)

    @staticmethod
    def _items(renders):
        """pico_render_item array for renders given as dicts: gpu_scene, camera, max_depth, max_samples, and
        optionally seed, estimator, max_variance, pixels, sample_count, variance (allocated when absent)."""
        arr = (CRenderItem * max(len(renders), 1))()
        for k, r in enumerate(renders):
            cam = r["camera"]
            W, H = int(cam.resolution[0]), int(cam.resolution[1])
            r.setdefault("pixels", np.zeros((H, W, 3), np.float32))
            r.setdefault("sample_count", np.zeros((H, W), np.uint32))
            r.setdefault("variance", np.zeros((H, W, 3), np.float32))
            it = arr[k]
            it.scene = r["gpu_scene"].handle
            it.camera = cam.to_c()
            it.config = CRenderConfig(r["max_depth"], r["max_samples"], r.get("max_variance", 0.0), H, W, 0, 0,
                                      r.get("estimator", 1), r.get("seed", 1))
            it.pixels_rgb = _f32(r["pixels"])
            it.sample_count = r["sample_count"].ctypes.data_as(C.POINTER(C.c_uint32))
            it.variance_rgb = _f32(r["variance"])
        return arr

    def render_many(self, renders, wavefront: int = 0, extend_ctas_per_sm: int = 0, branches: int = 0,
                    piece_paths: int = 0, extend_threads: int = 0):
        """pico_gpu_render_many: all renders in one CUDA graph launch; their buffers are updated in place.
        Returns (per-render completion times in ms, report dict)."""
        arr = self._items(renders)
        params = CLaunchParams(wavefront, extend_ctas_per_sm, branches, piece_paths, extend_threads, 0)
        done = (C.c_double * max(len(renders), 1))()
        rep = CBatchReport()
        self.check(self.lib.pico_gpu_render_many(self.handle, len(renders), arr, C.byref(params), done,
                                                 C.byref(rep)), "render_many")
        report = {k: getattr(rep, k) for k in ("build_ms", "run_ms", "graph_nodes", "samples", "rays")}
        return np.array(done[:len(renders)]), report

    def autotune_batch(self, renders, trial_samples: int = 1):
        """pico_gpu_autotune_batch: (best launch parameters, [(parameters, Msamples/s) per trial])."""
        arr = self._items(renders)
        best = CLaunchParams()
        trials = (CLaunchParams * 16)()
        rates = (C.c_double * 16)()
        nt = C.c_uint32(0)
        self.check(self.lib.pico_gpu_autotune_batch(self.handle, len(renders), arr, trial_samples, C.byref(best),
                                                    trials, rates, 16, C.byref(nt)), "autotune_batch")

        def as_dict(p):
            return {"wavefront": p.wavefront, "extend_ctas_per_sm": p.extend_ctas_per_sm, "branches": p.branches,
                    "piece_paths": p.piece_paths, "extend_threads": p.extend_threads}
        return as_dict(best), [(as_dict(trials[i]), rates[i]) for i in range(nt.value)]

    def atrous(self, pixels, normals, positions, diffuse, width: int, height: int) -> np.ndarray:
        arrs = [np.ascontiguousarray(a, dtype=np.float32).reshape(-1) for a in (pixels, normals, positions, diffuse)]
        out = np.empty(width * height * 3, np.float32)
        self.check(self.lib.pico_gpu_atrous(self.handle, *map(_f32, arrs), width, height, _f32(out)), "atrous")
        return out.reshape(height, width, 3)

    def tonemap(self, pixels, width: int, height: int) -> np.ndarray:
        """Util::reinhard_tone_mapping on a copy of `pixels`."""
        out = np.ascontiguousarray(pixels, dtype=np.float32).copy()
        self.check(self.lib.pico_gpu_tonemap(self.handle, _f32(out), width, height), "tonemap")
        return out

    def encode_hdr(self, pixels, width: int, height: int) -> bytes:
        """stbi_write_hdr's file image of `pixels` (no reversal)."""
        px = np.ascontiguousarray(pixels, dtype=np.float32)
        cap = self.lib.pico_gpu_hdr_bound(width, height)
        buf = np.empty(cap, np.uint8)
        n = C.c_size_t(0)
        self.check(self.lib.pico_gpu_encode_hdr(self.handle, _f32(px), width, height, buf.ctypes.data, cap,
                                                C.byref(n)), "encode_hdr")
        return buf[:n.value].tobytes()

    def phys_bsdf_eval(self, kinds, materials, V, N, L, u):
        """The physical estimator's device BSDF: (f, pdf, sample L, sample pdf, sample weight, sample ok)."""
        from .types import CMaterial
        n = len(kinds)
        k = np.ascontiguousarray(kinds, np.uint32)
        mats = (CMaterial * max(n, 1))()
        for i, m in enumerate(materials):
            mats[i].diffuse[:] = list(m.diffuse)
            mats[i].specular[:] = list(m.specular)
            mats[i].roughness = m.roughness
        arr = [np.ascontiguousarray(a, np.float32).reshape(n, 3) for a in (V, N, L, u)]
        f, sl, sw = (np.empty((n, 3), np.float32) for _ in range(3))
        pdf, spdf = np.empty(n, np.float32), np.empty(n, np.float32)
        ok = np.empty(n, np.uint32)
        self.check(self.lib.pico_gpu_phys_bsdf_eval(self.handle, n, k.ctypes.data, mats, *[a.ctypes.data for a in arr],
                                                    f.ctypes.data, pdf.ctypes.data, sl.ctypes.data, spdf.ctypes.data,
                                                    sw.ctypes.data, ok.ctypes.data), "phys_bsdf_eval")
        return f, pdf, sl, spdf, sw, ok.astype(bool)

    def bsdf_eval(self, kinds, materials, V, N, H, xi):
        """Device BSRDF routines on given inputs: (pdf, L, P, energy, direct_pdf)."""
        from .types import CMaterial
        n = len(kinds)
        k = np.ascontiguousarray(kinds, np.uint32)
        mats = (CMaterial * max(n, 1))()
        for i, m in enumerate(materials):
            mats[i].diffuse[:] = list(m.diffuse)
            mats[i].specular[:] = list(m.specular)
            mats[i].roughness = m.roughness
            mats[i].emissive[:] = list(m.emissive)
            mats[i].index_of_refraction = m.ior
        arr = [np.ascontiguousarray(a, np.float32) for a in (V, N, H, xi)]
        pdf, P, dl = (np.empty(n, np.float32) for _ in range(3))
        L, E = np.empty((n, 3), np.float32), np.empty((n, 3), np.float32)
        self.check(self.lib.pico_gpu_bsdf_eval(self.handle, n, k.ctypes.data, mats, *[a.ctypes.data for a in arr],
                                               pdf.ctypes.data, L.ctypes.data, P.ctypes.data, E.ctypes.data,
                                               dl.ctypes.data), "bsdf_eval")
        return pdf, L, P, E, dl

    def atrous_device(self, d_pixels: int, d_normals: int, d_positions: int, d_diffuse: int, width: int,
                      height: int, d_out: int, stream: int = 0):
        self.check(self.lib.pico_gpu_atrous_device(self.handle, d_pixels, d_normals, d_positions, d_diffuse,
                                                   width, height, d_out, stream or None), "atrous_device")

    def atrous_device_noalloc(self, d_pixels: int, d_normals: int, d_positions: int, d_diffuse: int, width: int,
                              height: int, d_out: int, stream: int = 0):
        """atrous_device without device allocation: fixed scratch of at most 2,097,152 pixels, shared by
        every call on the device (calls that overlap on the GPU race)."""
        self.check(self.lib.pico_gpu_atrous_device_noalloc(self.handle, d_pixels, d_normals, d_positions, d_diffuse,
                                                           width, height, d_out, stream or None),
                   "atrous_device_noalloc")


class GpuScene:
    """pico_gpu_scene: the flattened BVHs, instances, materials and lights in HBM."""

    def __init__(self, ctx: Context, scene: SceneData):
        self.ctx = ctx
        self.lib = ctx.lib
        m = MarshalledScene(scene)
        h = _vp()
        ctx.check(self.lib.pico_gpu_scene_upload(ctx.handle, C.byref(m.desc), C.byref(h)), "scene_upload")
        self.handle = h

    def info(self) -> dict:
        out = (C.c_uint64 * 6)()
        self.ctx.check(self.lib.pico_gpu_scene_info(self.handle, out), "scene_info")
        keys = ["tlas_nodes", "blas_nodes", "triangles", "instances", "device_bytes", "lights"]
        return dict(zip(keys, [int(x) for x in out]))

    def free(self):
        if getattr(self, "handle", None):
            self.lib.pico_gpu_scene_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def trace_closest(self, rays: np.ndarray) -> np.ndarray:
        """Host-buffer closest hit: rays (n,) RAY_DTYPE or (n, 8) float32 -> (n,) HIT_DTYPE."""
        r = np.ascontiguousarray(rays).view(np.float32).reshape(-1, 8)
        hits = np.empty(len(r), HIT_DTYPE)
        self.ctx.check(self.lib.pico_gpu_trace_closest(self.ctx.handle, self.handle, r.ctypes.data, len(r),
                                                       hits.ctypes.data), "trace_closest")
        return hits

    def trace_closest_ptr(self, rays_ptr: int, n: int, hits_ptr: int):
        """Host-buffer closest hit on raw host pointers (for pinned buffers)."""
        self.ctx.check(self.lib.pico_gpu_trace_closest(self.ctx.handle, self.handle, rays_ptr, n, hits_ptr),
                       "trace_closest")

    def trace_closest_device(self, d_rays: int, n: int, d_hits: int, stream: int = 0):
        self.ctx.check(self.lib.pico_gpu_trace_closest_device(self.ctx.handle, self.handle, d_rays, n, d_hits,
                                                              stream or None), "trace_closest_device")

    def check(self, stream: int = 0):
        self.ctx.check(self.lib.pico_gpu_check(self.ctx.handle, stream or None), "device status")

    def trace_stats(self, d_rays: int, n: int, stream: int = 0) -> dict:
        out = (C.c_uint64 * 3)()
        self.ctx.check(self.lib.pico_gpu_trace_stats(self.ctx.handle, self.handle, d_rays, n, out, stream or None),
                       "trace_stats")
        return {"nodes": int(out[0]), "tris": int(out[1]), "instances": int(out[2])}

    def render(self, camera: Camera, max_depth: int, max_samples: int, seed: int = 1, pixels=None,
               sample_count=None, variance=None, max_variance: float = 0.0, denoise: bool = False,
               tonemap: bool = False, should_quit=None, estimator: int = 0, cancellable: bool = True):
        """Scene::render_scene_to_memory into (H, W, 3) buffers that are updated in place;
        estimator 1 (ESTIMATOR_PHYSICAL) selects the physical estimator of pico_gpu.h.
        should_quit: a ctypes c_int32 the render polls (a zero flag of its own by default);
        cancellable=False passes no flag (batches are then not limited to 16 samples per pixel)."""
        W, H = int(camera.resolution[0]), int(camera.resolution[1])
        if pixels is None:
            pixels = np.zeros((H, W, 3), np.float32)
        if sample_count is None:
            sample_count = np.zeros((H, W), np.uint32)
        if variance is None:
            variance = np.zeros((H, W, 3), np.float32)
        cfg = CRenderConfig(max_depth, max_samples, max_variance, H, W, int(tonemap), int(denoise), int(estimator),
                            seed)
        cam = camera.to_c()
        quit_flag = should_quit if should_quit is not None else C.c_int32(0)
        self.ctx.check(self.lib.pico_gpu_render(self.ctx.handle, self.handle, C.byref(cam), C.byref(cfg),
                                                _f32(pixels), sample_count.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                _f32(variance), C.byref(quit_flag) if cancellable else None),
                       "render")
        return pixels, sample_count, variance

    def render_device(self, camera: Camera, max_depth: int, max_samples: int, d_pixels: int, d_count: int,
                      d_variance: int, stream: int = 0, seed: int = 1, max_variance: float = 0.0,
                      denoise: bool = False, tonemap: bool = False, estimator: int = 0):
        """pico_gpu_render_device: the render on caller device buffers (pointers as ints: W*H*3 floats,
        W*H uint32, W*H*3 floats), enqueued on `stream` without waiting for it."""
        W, H = int(camera.resolution[0]), int(camera.resolution[1])
        cfg = CRenderConfig(max_depth, max_samples, max_variance, H, W, int(tonemap), int(denoise), int(estimator),
                            seed)
        cam = camera.to_c()
        self.ctx.check(self.lib.pico_gpu_render_device(self.ctx.handle, self.handle, C.byref(cam), C.byref(cfg),
                                                       d_pixels, d_count, d_variance, stream or None),
                       "render_device")

    def render_to_file(self, camera: Camera, max_depth: int, max_samples: int, path, seed: int = 1,
                       pixels=None, sample_count=None, variance=None, denoise: bool = False, tonemap: bool = False):
        """Scene::render_scene_to_file: renders, reverses `pixels` in place and writes a Radiance .hdr."""
        W, H = int(camera.resolution[0]), int(camera.resolution[1])
        pixels = np.zeros((H, W, 3), np.float32) if pixels is None else pixels
        sample_count = np.zeros((H, W), np.uint32) if sample_count is None else sample_count
        variance = np.zeros((H, W, 3), np.float32) if variance is None else variance
        cfg = CRenderConfig(max_depth, max_samples, 0.0, H, W, int(tonemap), int(denoise), 0, seed)
        cam = camera.to_c()
        self.ctx.check(self.lib.pico_gpu_render_to_file(self.ctx.handle, self.handle, C.byref(cam), C.byref(cfg),
                                                        _f32(pixels), sample_count.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                        _f32(variance), str(path).encode()), "render_to_file")
        return pixels, sample_count, variance

    def denoiser_inputs(self, camera: Camera):
        W, H = int(camera.resolution[0]), int(camera.resolution[1])
        n, p, d = (np.empty((H, W, 3), np.float32) for _ in range(3))
        cam = camera.to_c()
        self.ctx.check(self.lib.pico_gpu_denoiser_inputs(self.ctx.handle, self.handle, C.byref(cam), _f32(n),
                                                         _f32(p), _f32(d)), "denoiser_inputs")
        return n, p, d


class RadianceCache:
    """pico_gpu_nrc: a neural radiance cache on the context's device (see pico_gpu.h)."""

    LEVELS, WIDTH, LAYERS = 16, 64, 6

    def __init__(self, ctx: Context, **overrides):
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = CNrcConfig()
        self.lib.pico_gpu_nrc_default_config(C.byref(cfg))
        for k, v in overrides.items():
            if k in ("aabb_min", "aabb_max"):
                getattr(cfg, k)[:] = [float(x) for x in v]
            else:
                setattr(cfg, k, v)
        self.config = cfg
        h = _vp()
        ctx.check(self.lib.pico_gpu_nrc_create(ctx.handle, C.byref(cfg), C.byref(h)), "nrc_create")
        self.handle = h
        self.table_size = 1 << cfg.log2_table_size

    def free(self):
        if getattr(self, "handle", None):
            self.lib.pico_gpu_nrc_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def params(self):
        """(network (6, 64, 64) float32, grid (16, T, 2) float32) master parameters."""
        mlp = np.empty((self.LAYERS, self.WIDTH, self.WIDTH), np.float32)
        grid = np.empty((self.LEVELS, self.table_size, 2), np.float32)
        self.ctx.check(self.lib.pico_gpu_nrc_get_params(self.handle, mlp.ctypes.data, grid.ctypes.data), "nrc_params")
        return mlp, grid

    def set_params(self, mlp, grid):
        m = np.ascontiguousarray(mlp, np.float32)
        g = np.ascontiguousarray(grid, np.float32)
        self.ctx.check(self.lib.pico_gpu_nrc_set_params(self.handle, m.ctypes.data, g.ctypes.data), "nrc_set_params")

    def set_bounds(self, lo, hi):
        a = np.ascontiguousarray(lo, np.float32)
        b = np.ascontiguousarray(hi, np.float32)
        self.ctx.check(self.lib.pico_gpu_nrc_set_bounds(self.handle, _f32(a), _f32(b)), "nrc_set_bounds")

    def info(self) -> dict:
        out = (C.c_uint64 * 4)()
        self.ctx.check(self.lib.pico_gpu_nrc_info(self.handle, out), "nrc_info")
        return dict(zip(["steps", "grid_entries", "mlp_params", "frames"], [int(x) for x in out]))

    def stats(self) -> dict:
        """Cumulative render work with this cache."""
        out = (C.c_uint64 * 4)()
        self.ctx.check(self.lib.pico_gpu_nrc_stats(self.handle, out), "nrc_stats")
        return dict(zip(["train_paths", "train_records", "train_steps", "queries"], [int(x) for x in out]))

    def encode(self, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, NRC_QUERY_DTYPE)
        out = np.empty((len(q), self.WIDTH), np.float32)
        self.ctx.check(self.lib.pico_gpu_nrc_encode(self.handle, q.ctypes.data, len(q), out.ctypes.data),
                       "nrc_encode")
        return out

    def infer(self, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, NRC_QUERY_DTYPE)
        out = np.empty((len(q), 3), np.float32)
        self.ctx.check(self.lib.pico_gpu_nrc_infer(self.handle, q.ctypes.data, len(q), out.ctypes.data), "nrc_infer")
        return out

    def set_wait_limit(self, limit_ns: int = 1_000_000_000, withheld_bytes: int = 0):
        """pico_gpu_nrc_set_wait_limit: how long the kernels' mbarrier waits last before they give up
        (PICO_ERR_TIMEOUT); withheld_bytes > 0 makes the inference's weight-load wait run out (tests)."""
        self.ctx.check(self.lib.pico_gpu_nrc_set_wait_limit(self.handle, int(limit_ns), int(withheld_bytes)),
                       "nrc_set_wait_limit")

    def infer_device(self, d_queries: int, n: int, d_rgb: int, stream: int = 0):
        self.ctx.check(self.lib.pico_gpu_nrc_infer_device(self.handle, d_queries, n, d_rgb, stream or None),
                       "nrc_infer_device")

    def train(self, queries: np.ndarray, targets: np.ndarray, apply: bool = True) -> float:
        """One optimiser step (or, with apply=False, only the gradients); returns the batch loss."""
        q = np.ascontiguousarray(queries, NRC_QUERY_DTYPE)
        t = np.ascontiguousarray(targets, np.float32).reshape(-1, 3)
        loss = C.c_float(0.0)
        self.ctx.check(self.lib.pico_gpu_nrc_train(self.handle, q.ctypes.data, t.ctypes.data, len(q), int(apply),
                                                   C.byref(loss)), "nrc_train")
        return float(loss.value)

    def train_device(self, d_queries: int, d_targets: int, n: int, apply: bool = True, stream: int = 0):
        self.ctx.check(self.lib.pico_gpu_nrc_train_device(self.handle, d_queries, d_targets, n, int(apply),
                                                          stream or None), "nrc_train_device")

    def gradients(self):
        """Gradients of the last train call: (network (6, 64, 64), grid (16, T, 2))."""
        mlp = np.empty((self.LAYERS, self.WIDTH, self.WIDTH), np.float32)
        grid = np.empty((self.LEVELS, self.table_size, 2), np.float32)
        self.ctx.check(self.lib.pico_gpu_nrc_gradients(self.handle, mlp.ctypes.data, grid.ctypes.data),
                       "nrc_gradients")
        return mlp, grid

    def attach(self):
        """Makes this the cache of the context's ESTIMATOR_RADIANCE_CACHE renders."""
        self.ctx.check(self.lib.pico_gpu_set_radiance_cache(self.ctx.handle, self.handle), "set_radiance_cache")
