"""ctypes bindings of the oracle (test infrastructure only).

Two libraries:
  * _build/libpico_oracle.so -- the C restatement of the reference hot path
    (po_*.c), buildable on any machine;
  * _ref/libpico_ref.so      -- the Pico reference's own sources plus
    ref/harness.cpp, buildable only where the Pico tree is present.

Only tests/, the smoke entry and the CPU-baseline leg of bench.py use this
module; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from pico_gb300.types import HIT_DTYPE, RAY_DTYPE, CCamera, CMaterial, MarshalledScene, Material, SceneData, Sky

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "libpico_oracle.so"
REF_LIB = HERE / "_ref" / "libpico_ref.so"
# The Pico source tree the harness was built from, recorded by build_reference.
REF_TREE_RECORD = HERE / "_ref" / "reference_tree.txt"

FRAG_DTYPE = np.dtype([("inst", "<u4"), ("prim", "<u4"), ("t", "<f4"), ("u", "<f4"), ("v", "<f4"),
                       ("position", "<f4", (4,)), ("normal", "<f4", (3,)), ("uv", "<f4", (2,))])

_vp, _u32, _u64, _i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
_fp, _up = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
_dp = C.POINTER(C.c_double)


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return ORACLE_LIB


def build_reference(tree: str | os.PathLike | None = None) -> Path | None:
    """Compiles the reference harness from the Pico source tree `tree` (default: the
    PICO_REFERENCE environment variable); returns None when no tree is given or present.
    The tree's path is recorded beside the library for the tests that compile against
    the reference's headers."""
    tree = tree or os.environ.get("PICO_REFERENCE")
    if not tree or not (Path(tree) / "Source" / "Core" / "BVH.cpp").exists():
        return None
    jobs = str(os.cpu_count() or 4)
    subprocess.run(["make", "-s", "-j", jobs, "-C", str(HERE), "ref", f"REF={tree}"], check=True)
    REF_TREE_RECORD.write_text(str(Path(tree).resolve()) + "\n")
    return REF_LIB


def reference_tree() -> Path | None:
    """The Pico source tree the reference harness was built from, if it is still there."""
    if REF_TREE_RECORD.exists():
        p = Path(REF_TREE_RECORD.read_text().strip())
        if (p / "Source" / "Core" / "Scene.hpp").exists():
            return p
    return None


def _mat(m: Material) -> CMaterial:
    c = CMaterial()
    c.diffuse[:] = list(m.diffuse)
    c.specular[:] = list(m.specular)
    c.roughness = m.roughness
    c.emissive[:] = list(m.emissive)
    c.index_of_refraction = m.ior
    return c


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(_fp)


class _SceneLib:
    prefix = ""

    def _scene(self, scene: SceneData):
        m = MarshalledScene(scene)
        h = getattr(self.lib, f"{self.prefix}scene_create")(m.meshes, len(scene.meshes), m.instances,
                                                            len(scene.instances), m.materials, len(scene.materials))
        rgb = (C.c_float * 3)(*[float(x) for x in scene.sky])
        getattr(self.lib, f"{self.prefix}scene_set_sky")(h, C.byref(m.sky) if m.sky is not None else None, rgb)
        return h, m

    def sky_sample(self, sky: Sky, dirs) -> np.ndarray:
        """ImageCube::sample4 (Core/Image.cpp:361-397): RGBA per direction."""
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        out = np.empty((len(d), 4), np.float32)
        c = sky.to_c()
        getattr(self.lib, f"{self.prefix}sky_sample")(C.byref(c), d.ctypes.data, len(d), out.ctypes.data)
        return out


class Oracle(_SceneLib):
    """The C restatement (po_*)."""
    prefix = "po_"

    def __init__(self, path: Path | None = None):
        p = path or ORACLE_LIB
        if not p.exists():
            build_oracle()
        lib = C.CDLL(str(p))
        sig = {
            "po_scene_create": (_vp, [_vp, _u32, _vp, _u32, _vp, _u32]),
            "po_scene_destroy": (None, [_vp]),
            "po_scene_set_sky": (None, [_vp, _vp, _vp]),
            "po_sky_sample": (None, [_vp, _vp, _u32, _vp]),
            "po_blas_node_count": (_u32, [_vp, _u32]),
            "po_tlas_node_count": (_u32, [_vp]),
            "po_blas_nodes": (None, [_vp, _u32, _fp, _up, _up]),
            "po_tlas_nodes": (None, [_vp, _fp, _up, _up]),
            "po_instance_matrices": (None, [_vp, _u32, _fp, _fp]),
            "po_mat4_inverse": (None, [_fp, _fp]),
            "po_trace": (None, [_vp, _vp, _u32, _vp, _i32]),
            "po_trace_fragments": (None, [_vp, _vp, _u32, _vp]),
            "po_trace_stats": (None, [_vp, _vp, _u32, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_u64)]),
            "po_generate_ray": (None, [C.POINTER(CCamera), C.c_float, C.c_float, _u32, _u32, _vp]),
            "po_xorshift_next": (_u32, [_up]),
            "po_xorshift_seed": (None, [_u32, _up]),
            "po_radical_inverse": (C.c_float, [_u32]),
            "po_hammersley_next": (None, [_up, _fp]),
            "po_uniform_sample_triangle": (None, [_fp, _fp]),
            "po_mt64_seed": (None, [C.POINTER(_u64), _u64]),
            "po_mt64_uniform": (C.c_float, [C.POINTER(_u64)]),
            "po_tangent_frame": (None, [_fp, _fp, _fp]),
            "po_cos_sample": (None, [_fp, _fp]),
            "po_cos_pdf": (C.c_float, [_fp]),
            "po_beckmann_sample": (None, [_fp, _fp, C.c_float, _fp]),
            "po_beckmann_pdf": (C.c_float, [_fp, C.c_float]),
            "po_bsdf_pdf": (C.c_float, [_i32, _fp, _fp, C.c_float, C.c_float]),
            "po_bsdf_sample": (None, [_i32, C.POINTER(CMaterial), _fp, _fp, _fp, _fp, _fp, _fp]),
            "po_direct_lighting_pdf": (C.c_float, [_i32, C.POINTER(CMaterial), _fp, _fp, _fp]),
            "po_alias_build": (None, [_fp, _u32, _fp, _up]),
            "po_triangle_weights": (None, [_vp, _fp]),
            "po_integrate_ray": (None, [_vp, C.POINTER(CCamera), _u32, _u32, _u32, _u64, _u32, _fp]),
            "po_render_pixels": (None, [_vp, C.POINTER(CCamera), _u32, _u32, C.c_float, _up, C.POINTER(_u64),
                                        _u32, _fp, _up, _fp, _i32]),
            "po_accumulate": (None, [_fp, _u32, _u32, C.c_float, _fp, _up, _fp]),
            "po_phys_bsdf_eval": (None, [_i32, C.POINTER(CMaterial), _dp, _dp, _dp, _dp, _dp]),
            "po_phys_bsdf_sample": (_i32, [_i32, C.POINTER(CMaterial), _dp, _dp, _dp, _dp, _dp, _dp]),
            "po_phys_render_mean": (None, [_vp, C.POINTER(CCamera), _u32, _u32, _up, C.POINTER(_u64), _u32, _i32,
                                           _dp, _dp, _i32]),
            "po_phys_render_mean_cached": (None, [_vp, C.POINTER(CCamera), _u32, _u32, _up, C.POINTER(_u64), _u32,
                                                  _dp, _dp, _dp, _i32]),
            "po_denoiser_inputs": (None, [_vp, C.POINTER(CCamera), _u32, _u32, _fp, _fp, _fp]),
            "po_view_matrix": (None, [C.POINTER(CCamera), _fp]),
            "po_atrous_denoise": (None, [_fp, _fp, _fp, _fp, _u32, _u32, _fp]),
            "po_reinhard": (None, [_fp, _u32, _u32]),
            "po_reverse_pixels": (None, [_fp, _u32]),
            "po_encode_hdr": (C.c_size_t, [_fp, _u32, _u32, C.c_void_p, C.c_size_t]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        self.lib = lib

    # ---- scenes
    def scene(self, scene: SceneData) -> "OracleScene":
        return OracleScene(self, scene)

    # ---- building blocks
    def mat4_inverse(self, m: np.ndarray) -> np.ndarray:
        out = np.empty(16, np.float32)
        self.lib.po_mat4_inverse(_f(np.asarray(m, np.float32).reshape(-1)), out.ctypes.data_as(_fp))
        return out.reshape(4, 4)

    def generate_ray(self, cam, xi, px, py) -> np.ndarray:
        out = np.zeros(1, RAY_DTYPE)
        c = cam.to_c()
        self.lib.po_generate_ray(C.byref(c), float(xi[0]), float(xi[1]), px, py, out.ctypes.data)
        return out[0]

    def xorshift(self, seed: int, n: int) -> np.ndarray:
        st = (C.c_uint32 * 4)()
        self.lib.po_xorshift_seed(seed, st)
        return np.array([self.lib.po_xorshift_next(st) for _ in range(n)], np.uint32)

    def hammersley(self, seed: int, n: int) -> np.ndarray:
        st = (C.c_uint32 * 4)()
        self.lib.po_xorshift_seed(seed, st)
        out = np.empty((n, 2), np.float32)
        for i in range(n):
            self.lib.po_hammersley_next(st, out[i].ctypes.data_as(_fp))
        return out

    def radical_inverse(self, bits: int) -> float:
        return self.lib.po_radical_inverse(bits)

    def uniform_sample_triangle(self, xi) -> np.ndarray:
        out = np.empty(2, np.float32)
        self.lib.po_uniform_sample_triangle(_f(xi), out.ctypes.data_as(_fp))
        return out

    def mt_uniform(self, seed: int, n: int) -> np.ndarray:
        st = (C.c_uint64 * 313)()
        self.lib.po_mt64_seed(st, seed)
        return np.array([self.lib.po_mt64_uniform(st) for _ in range(n)], np.float32)

    def tangent_frame(self, V, N) -> np.ndarray:
        out = np.empty(9, np.float32)
        self.lib.po_tangent_frame(_f(V), _f(N), out.ctypes.data_as(_fp))
        return out.reshape(3, 3)

    def cos_sample(self, xi) -> np.ndarray:
        out = np.empty(3, np.float32)
        self.lib.po_cos_sample(_f(xi), out.ctypes.data_as(_fp))
        return out

    def cos_pdf(self, H) -> float:
        return self.lib.po_cos_pdf(_f(H))

    def beckmann_sample(self, xi, V, R) -> np.ndarray:
        out = np.empty(3, np.float32)
        self.lib.po_beckmann_sample(_f(xi), _f(V), R, out.ctypes.data_as(_fp))
        return out

    def beckmann_pdf(self, H, R) -> float:
        return self.lib.po_beckmann_pdf(_f(H), R)

    def bsdf_pdf(self, kind, wo, H, roughness, reflectance) -> float:
        return self.lib.po_bsdf_pdf(kind, _f(wo), _f(H), roughness, reflectance)

    def bsdf_sample(self, kind, material: Material, V, N, xi):
        L, P, E = np.empty(3, np.float32), np.empty(1, np.float32), np.empty(3, np.float32)
        m = _mat(material)
        self.lib.po_bsdf_sample(kind, C.byref(m), _f(V), _f(N), _f(np.asarray(xi, np.float32).reshape(-1)),
                                L.ctypes.data_as(_fp), P.ctypes.data_as(_fp), E.ctypes.data_as(_fp))
        return L, float(P[0]), E

    def direct_lighting_pdf(self, kind, material: Material, N, wi, wo) -> float:
        m = _mat(material)
        return self.lib.po_direct_lighting_pdf(kind, C.byref(m), _f(N), _f(wi), _f(wo))

    def phys_bsdf_eval(self, kind, material: Material, V, N, L):
        """Physical estimator's BSDF (FP64): (f rgb, pdf) for unit V, N, L."""
        v, n, l = (np.ascontiguousarray(a, np.float64) for a in (V, N, L))
        f, pdf = np.empty(3), np.empty(1)
        m = _mat(material)
        self.lib.po_phys_bsdf_eval(kind, C.byref(m), v.ctypes.data_as(_dp), n.ctypes.data_as(_dp),
                                   l.ctypes.data_as(_dp), f.ctypes.data_as(_dp), pdf.ctypes.data_as(_dp))
        return f, float(pdf[0])

    def phys_bsdf_sample(self, kind, material: Material, V, N, u):
        """Physical estimator's BSDF sample (FP64) from three uniforms: (ok, L, pdf, weight rgb)."""
        v, n, uu = (np.ascontiguousarray(a, np.float64) for a in (V, N, u))
        L, pdf, w = np.empty(3), np.empty(1), np.empty(3)
        m = _mat(material)
        ok = self.lib.po_phys_bsdf_sample(kind, C.byref(m), v.ctypes.data_as(_dp), n.ctypes.data_as(_dp),
                                          uu.ctypes.data_as(_dp), L.ctypes.data_as(_dp), pdf.ctypes.data_as(_dp),
                                          w.ctypes.data_as(_dp))
        return bool(ok), L, float(pdf[0]), w

    def alias_build(self, weights) -> tuple[np.ndarray, np.ndarray]:
        w = np.ascontiguousarray(weights, np.float32)
        bw, ba = np.empty(len(w), np.float32), np.empty(len(w), np.uint32)
        self.lib.po_alias_build(w.ctypes.data_as(_fp), len(w), bw.ctypes.data_as(_fp), ba.ctypes.data_as(_up))
        return bw, ba

    def triangle_weights(self, scene: SceneData, mesh: int) -> np.ndarray:
        m = MarshalledScene(scene)
        out = np.empty(len(scene.meshes[mesh].indices), np.float32)
        self.lib.po_triangle_weights(C.byref(m.meshes[mesh]), out.ctypes.data_as(_fp))
        return out

    def view_matrix(self, cam) -> np.ndarray:
        out = np.empty(16, np.float32)
        c = cam.to_c()
        self.lib.po_view_matrix(C.byref(c), out.ctypes.data_as(_fp))
        return out.reshape(4, 4)

    def accumulate(self, samples, max_samples, max_variance=0.0, pixel=None, count=0, variance=None):
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 3)
        px = np.zeros(3, np.float32) if pixel is None else np.array(pixel, np.float32)
        var = np.zeros(3, np.float32) if variance is None else np.array(variance, np.float32)
        cnt = np.array([count], np.uint32)
        self.lib.po_accumulate(s.ctypes.data_as(_fp), len(s), max_samples, max_variance, px.ctypes.data_as(_fp),
                               cnt.ctypes.data_as(_up), var.ctypes.data_as(_fp))
        return px, int(cnt[0]), var

    def reinhard(self, pixels, W, H) -> np.ndarray:
        return _reinhard(self.lib.po_reinhard, pixels, W, H)

    def hdr_file(self, pixels, W, H) -> bytes:
        """render_scene_to_file's output: reversed pixels written as a Radiance .hdr."""
        px = np.ascontiguousarray(pixels, np.float32).reshape(-1).copy()
        self.lib.po_reverse_pixels(px.ctypes.data_as(_fp), W * H)
        n = self.lib.po_encode_hdr(px.ctypes.data_as(_fp), W, H, None, 0)
        out = (C.c_ubyte * n)()
        self.lib.po_encode_hdr(px.ctypes.data_as(_fp), W, H, out, n)
        return bytes(out)

    def atrous(self, pixels, normals, positions, diffuse, W, H) -> np.ndarray:
        out = np.empty(W * H * 3, np.float32)
        self.lib.po_atrous_denoise(_f(pixels), _f(normals), _f(positions), _f(diffuse), W, H,
                                   out.ctypes.data_as(_fp))
        return out.reshape(H, W, 3)


def _reinhard(fn, pixels, W, H):
    out = np.ascontiguousarray(pixels, np.float32).copy()
    fn(out.ctypes.data_as(_fp), W, H)
    return out


class OracleScene:
    def __init__(self, oracle: Oracle, scene: SceneData):
        self.o = oracle
        self.lib = oracle.lib
        self.handle, self._keep = oracle._scene(scene)

    def __del__(self):
        try:
            self.lib.po_scene_destroy(self.handle)
        except Exception:
            pass

    def trace(self, rays: np.ndarray, nthreads: int = 0) -> np.ndarray:
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.empty(len(r), HIT_DTYPE)
        self.lib.po_trace(self.handle, r.ctypes.data, len(r), hits.ctypes.data, nthreads)
        return hits

    def fragments(self, rays: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        out = np.empty(len(r), FRAG_DTYPE)
        self.lib.po_trace_fragments(self.handle, r.ctypes.data, len(r), out.ctypes.data)
        return out

    def stats(self, rays: np.ndarray) -> dict:
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self.lib.po_trace_stats(self.handle, r.ctypes.data, len(r), C.byref(a), C.byref(b), C.byref(c))
        return {"nodes": a.value, "tris": b.value, "instances": c.value}

    def blas_nodes(self, mesh: int):
        n = self.lib.po_blas_node_count(self.handle, mesh)
        boxes, links = np.empty((n, 6), np.float32), np.empty((n, 4), np.uint32)
        nv = int(links[:, 3].sum()) if n else 0
        self.lib.po_blas_nodes(self.handle, mesh, boxes.ctypes.data_as(_fp), links.ctypes.data_as(_up), None)
        nv = int(links[:, 3].sum())
        values = np.empty(max(nv, 1), np.uint32)
        self.lib.po_blas_nodes(self.handle, mesh, None, None, values.ctypes.data_as(_up))
        return boxes, links, values[:nv]

    def tlas_nodes(self):
        n = self.lib.po_tlas_node_count(self.handle)
        boxes, links = np.empty((n, 6), np.float32), np.empty((n, 4), np.uint32)
        self.lib.po_tlas_nodes(self.handle, boxes.ctypes.data_as(_fp), links.ctypes.data_as(_up), None)
        nv = int(links[:, 3].sum())
        values = np.empty(max(nv, 1), np.uint32)
        self.lib.po_tlas_nodes(self.handle, None, None, values.ctypes.data_as(_up))
        return boxes, links, values[:nv]

    def integrate(self, cam, px, py, max_depth, seed, nsamples) -> np.ndarray:
        out = np.empty((nsamples, 3), np.float32)
        c = cam.to_c()
        self.lib.po_integrate_ray(self.handle, C.byref(c), px, py, max_depth, seed, nsamples, out.ctypes.data_as(_fp))
        return out

    def render_pixels(self, cam, max_depth, max_samples, pixel_index, seeds, pixels=None, counts=None,
                      variance=None, max_variance=0.0, nthreads=0):
        W, H = int(cam.resolution[0]), int(cam.resolution[1])
        pixels = np.zeros((H, W, 3), np.float32) if pixels is None else pixels
        counts = np.zeros((H, W), np.uint32) if counts is None else counts
        variance = np.zeros((H, W, 3), np.float32) if variance is None else variance
        idx = np.ascontiguousarray(pixel_index, np.uint32)
        sd = np.ascontiguousarray(seeds, np.uint64)
        c = cam.to_c()
        self.lib.po_render_pixels(self.handle, C.byref(c), max_depth, max_samples, max_variance,
                                  idx.ctypes.data_as(_up), sd.ctypes.data_as(C.POINTER(_u64)), len(idx),
                                  pixels.ctypes.data_as(_fp), counts.ctypes.data_as(_up),
                                  variance.ctypes.data_as(_fp), nthreads)
        return pixels, counts, variance

    def phys_render_mean(self, cam, max_depth, spp, pixel_index, seeds, strategy=0, nthreads=0):
        """Physical estimator: FP64 mean and sample variance of `spp` paths per listed pixel;
        strategy 0 combines light and BSDF sampling, 1 samples lights alone, 2 the BSDF alone."""
        idx = np.ascontiguousarray(pixel_index, np.uint32)
        sd = np.ascontiguousarray(seeds, np.uint64)
        mean, var = np.empty((len(idx), 3)), np.empty((len(idx), 3))
        c = cam.to_c()
        self.lib.po_phys_render_mean(self.handle, C.byref(c), max_depth, spp, idx.ctypes.data_as(_up),
                                     sd.ctypes.data_as(C.POINTER(_u64)), len(idx), strategy,
                                     mean.ctypes.data_as(_dp), var.ctypes.data_as(_dp), nthreads)
        return mean, var

    def phys_render_mean_cached(self, cam, max_depth, spp, pixel_index, seeds, cache_rgb, nthreads=0):
        """The radiance-cache form of the physical estimator with a cache answering the constant
        cache_rgb (FP64 mean and sample variance of `spp` paths per listed pixel)."""
        idx = np.ascontiguousarray(pixel_index, np.uint32)
        sd = np.ascontiguousarray(seeds, np.uint64)
        k = np.ascontiguousarray(cache_rgb, np.float64)
        mean, var = np.empty((len(idx), 3)), np.empty((len(idx), 3))
        c = cam.to_c()
        self.lib.po_phys_render_mean_cached(self.handle, C.byref(c), max_depth, spp, idx.ctypes.data_as(_up),
                                            sd.ctypes.data_as(C.POINTER(_u64)), len(idx), k.ctypes.data_as(_dp),
                                            mean.ctypes.data_as(_dp), var.ctypes.data_as(_dp), nthreads)
        return mean, var

    def denoiser_inputs(self, cam):
        W, H = int(cam.resolution[0]), int(cam.resolution[1])
        n, p, d = (np.empty((H, W, 3), np.float32) for _ in range(3))
        c = cam.to_c()
        self.lib.po_denoiser_inputs(self.handle, C.byref(c), W, H, n.ctypes.data_as(_fp), p.ctypes.data_as(_fp),
                                    d.ctypes.data_as(_fp))
        return n, p, d


class Reference(_SceneLib):
    """The Pico reference's own code through ref/harness.cpp (ref_*)."""
    prefix = "ref_"

    def __init__(self, path: Path | None = None):
        p = path or REF_LIB
        if not p.exists():
            raise FileNotFoundError(f"{p} is not built (needs the Pico source tree)")
        lib = C.CDLL(str(p))
        sig = {
            "ref_scene_create": (_vp, [_vp, _u32, _vp, _u32, _vp, _u32]),
            "ref_scene_destroy": (None, [_vp]),
            "ref_scene_set_sky": (None, [_vp, _vp, _vp]),
            "ref_sky_sample": (None, [_vp, _vp, _u32, _vp]),
            "ref_trace": (None, [_vp, _vp, _u32, _vp]),
            "ref_trace_timed": (C.c_double, [_vp, _vp, _u32, _vp, _i32]),
            "ref_blas_node_count": (_u32, [_vp, _u32]),
            "ref_blas_root": (_u32, [_vp, _u32]),
            "ref_blas_nodes": (None, [_vp, _u32, _fp, _up, _up]),
            "ref_tlas_node_count": (_u32, [_vp]),
            "ref_tlas_root": (_u32, [_vp]),
            "ref_tlas_nodes": (None, [_vp, _fp, _up, _up]),
            "ref_instance_inverse": (None, [_vp, _u32, _fp]),
            "ref_light_table": (_u32, [_vp, _u32, _fp, _fp, _up]),
            "ref_mat4_inverse": (None, [_fp, _fp]),
            "ref_generate_ray": (None, [C.POINTER(CCamera), C.c_float, C.c_float, _u32, _u32, _vp]),
            "ref_view_matrix": (None, [C.POINTER(CCamera), _fp]),
            "ref_xorshift": (None, [_u32, _u32, _up]),
            "ref_hammersley": (None, [_u32, _u32, _fp]),
            "ref_radical_inverse": (C.c_float, [_u32]),
            "ref_uniform_sample_triangle": (None, [_fp, _fp]),
            "ref_mt_uniform": (None, [_u64, _u32, _fp]),
            "ref_tangent_frame": (None, [_fp, _fp, _fp]),
            "ref_cos_sample": (None, [_fp, _fp]),
            "ref_cos_pdf": (C.c_float, [_fp]),
            "ref_beckmann_sample": (None, [_fp, _fp, C.c_float, _fp]),
            "ref_beckmann_pdf": (C.c_float, [_fp, C.c_float]),
            "ref_bsdf_pdf": (C.c_float, [_i32, _fp, _fp, C.c_float, C.c_float]),
            "ref_bsdf_sample": (None, [_i32, C.POINTER(CMaterial), _fp, _fp, _u32, _fp, _fp, _fp]),
            "ref_direct_lighting_pdf": (C.c_float, [_i32, C.POINTER(CMaterial), _fp, _fp, _fp]),
            "ref_integrate": (None, [_vp, C.POINTER(CCamera), _u32, _u32, _u32, _u64, _u32, _fp]),
            "ref_render_pixels": (C.c_double, [_vp, C.POINTER(CCamera), _u32, _u32, C.c_float, _up,
                                               C.POINTER(_u64), _u32, _fp, _up, _fp, _i32]),
            "ref_render_mean64": (C.c_double, [_vp, C.POINTER(CCamera), _u32, _u32, _up, C.POINTER(_u64), _u32,
                                               C.POINTER(C.c_double), C.POINTER(C.c_double), _i32]),
            "ref_denoiser_inputs": (None, [_vp, C.POINTER(CCamera), _u32, _u32, _fp, _fp, _fp]),
            "ref_atrous": (C.c_double, [_fp, _fp, _fp, _fp, _u32, _u32, _fp, _i32]),
            "ref_reinhard": (None, [_fp, _u32, _u32]),
            "ref_write_hdr": (_i32, [_fp, _u32, _u32, C.c_char_p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(lib, name)
            fn.restype, fn.argtypes = res, args
        self.lib = lib

    def scene(self, scene: SceneData) -> "ReferenceScene":
        return ReferenceScene(self, scene)

    def reinhard(self, pixels, W, H) -> np.ndarray:
        return _reinhard(self.lib.ref_reinhard, pixels, W, H)

    def hdr_file(self, pixels, W, H, path) -> bytes:
        px = np.ascontiguousarray(pixels, np.float32)
        if not self.lib.ref_write_hdr(px.ctypes.data_as(_fp), W, H, str(path).encode()):
            raise RuntimeError("stbi_write_hdr failed")
        return Path(path).read_bytes()


class ReferenceScene:
    def __init__(self, ref: Reference, scene: SceneData):
        self.lib = ref.lib
        self.handle, self._keep = ref._scene(scene)

    def __del__(self):
        try:
            self.lib.ref_scene_destroy(self.handle)
        except Exception:
            pass

    def fragments(self, rays: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        out = np.empty(len(r), FRAG_DTYPE)
        self.lib.ref_trace(self.handle, r.ctypes.data, len(r), out.ctypes.data)
        return out

    def trace_timed(self, rays: np.ndarray, nthreads: int = 0):
        r = np.ascontiguousarray(rays, RAY_DTYPE)
        hits = np.empty(len(r), HIT_DTYPE)
        secs = self.lib.ref_trace_timed(self.handle, r.ctypes.data, len(r), hits.ctypes.data, nthreads)
        return hits, secs

    def _nodes(self, count, dump, *pre):
        n = count(self.handle, *pre)
        boxes, links = np.empty((n, 6), np.float32), np.empty((n, 4), np.uint32)
        dump(self.handle, *pre, boxes.ctypes.data_as(_fp), links.ctypes.data_as(_up), None)
        nv = int(links[:, 3].sum())
        values = np.empty(max(nv, 1), np.uint32)
        dump(self.handle, *pre, None, None, values.ctypes.data_as(_up))
        return boxes, links, values[:nv]

    def blas_nodes(self, mesh: int):
        return self._nodes(self.lib.ref_blas_node_count, self.lib.ref_blas_nodes, mesh)

    def tlas_nodes(self):
        return self._nodes(self.lib.ref_tlas_node_count, self.lib.ref_tlas_nodes)

    def integrate(self, cam, px, py, max_depth, seed, nsamples) -> np.ndarray:
        out = np.empty((nsamples, 3), np.float32)
        c = cam.to_c()
        self.lib.ref_integrate(self.handle, C.byref(c), px, py, max_depth, seed, nsamples, out.ctypes.data_as(_fp))
        return out

    def render_pixels(self, cam, max_depth, max_samples, pixel_index, seeds, max_variance=0.0, nthreads=0):
        W, H = int(cam.resolution[0]), int(cam.resolution[1])
        pixels = np.zeros((H, W, 3), np.float32)
        counts = np.zeros((H, W), np.uint32)
        variance = np.zeros((H, W, 3), np.float32)
        idx = np.ascontiguousarray(pixel_index, np.uint32)
        sd = np.ascontiguousarray(seeds, np.uint64)
        c = cam.to_c()
        secs = self.lib.ref_render_pixels(self.handle, C.byref(c), max_depth, max_samples, max_variance,
                                          idx.ctypes.data_as(_up), sd.ctypes.data_as(C.POINTER(_u64)), len(idx),
                                          pixels.ctypes.data_as(_fp), counts.ctypes.data_as(_up),
                                          variance.ctypes.data_as(_fp), nthreads)
        return pixels, counts, variance, secs

    def render_mean64(self, cam, max_depth, spp, pixel_index, seeds, nthreads=0):
        """Plain FP64 mean and sample variance of `spp` reference samples per listed pixel."""
        idx = np.ascontiguousarray(pixel_index, np.uint32)
        sd = np.ascontiguousarray(seeds, np.uint64)
        mean, var = np.empty((len(idx), 3)), np.empty((len(idx), 3))
        c = cam.to_c()
        secs = self.lib.ref_render_mean64(self.handle, C.byref(c), max_depth, spp, idx.ctypes.data_as(_up),
                                          sd.ctypes.data_as(C.POINTER(_u64)), len(idx),
                                          mean.ctypes.data_as(C.POINTER(C.c_double)),
                                          var.ctypes.data_as(C.POINTER(C.c_double)), nthreads)
        return mean, var, secs

    def denoiser_inputs(self, cam):
        W, H = int(cam.resolution[0]), int(cam.resolution[1])
        n, p, d = (np.empty((H, W, 3), np.float32) for _ in range(3))
        c = cam.to_c()
        self.lib.ref_denoiser_inputs(self.handle, C.byref(c), W, H, n.ctypes.data_as(_fp), p.ctypes.data_as(_fp),
                                     d.ctypes.data_as(_fp))
        return n, p, d

    def light_table(self, mesh: int, ntris: int):
        a, w, i = np.empty(ntris, np.float32), np.empty(ntris, np.float32), np.empty(ntris, np.uint32)
        n = self.lib.ref_light_table(self.handle, mesh, a.ctypes.data_as(_fp), w.ctypes.data_as(_fp),
                                     i.ctypes.data_as(_up))
        return a[:n], w[:n], i[:n]
