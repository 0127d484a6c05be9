"""Generates the golden vectors in this directory from the Pico reference itself.

Runs the reference's own code through oracle/_ref/libpico_ref.so (built from
the Pico source tree named by PICO_REFERENCE) on seeded inputs and stores
inputs and outputs as .npz files.  The reference has no tests or fixtures of
its own, so these files are the pins for the oracle restatement: the CPU test
suite checks the oracle against them bit for bit, and the GPU tests check the
kernels against the oracle.

    PICO_REFERENCE=<Pico source tree> python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "oracle"), str(HERE)]

import pico_oracle  # noqa: E402
from pico_gb300 import scenes  # noqa: E402
from pico_gb300.types import (DIELECTRIC, DIFFUSE, LIGHT, RAY_DTYPE, SKY_CUBE_RGBA8, SKY_EQUIRECT_RGBAF,  # noqa: E402
                              SPECULAR, Camera, CMaterial, Instance, Material, Sky)
from scene_io import camera_array, scene_arrays, sky_arrays  # noqa: E402

import ctypes as C  # noqa: E402


def frag_arrays(f, prefix):
    return {f"{prefix}_{k}": f[k] for k in f.dtype.names}


def axis_rays(rng, n):
    r = np.zeros(n, RAY_DTYPE)
    grid = np.array([0.0, 0.25, 0.3, 0.375, 0.5, 0.625, 0.7, 1.0], np.float32)
    r["org"][:, :3] = rng.choice(grid, size=(n, 3))
    r["org"][:, 3] = 1.0
    d = np.eye(3, dtype=np.float32)[rng.integers(0, 3, n)] * rng.choice(np.array([-1.0, 1.0], np.float32), (n, 1))
    r["dir"][:, :3] = d
    r["dir"][:, 3] = 10000.0
    return r


def trace_fixtures(ref):
    out = {}
    cornell = scenes.cornell_box()
    cam = scenes.cornell_camera(64, 64)
    rng = np.random.default_rng(101)
    rays = np.concatenate([scenes.primary_rays(cam, seed=102), scenes.surface_rays(cornell, 3000, seed=103),
                           axis_rays(rng, 1000)])
    rs = ref.scene(cornell)
    out.update(scene_arrays(cornell, "cornell"))
    out["cornell_rays"] = rays
    out.update(frag_arrays(rs.fragments(rays), "cornell_hit"))
    for mi in range(len(cornell.meshes)):
        b, l, v = rs.blas_nodes(mi)
        out[f"cornell_blas{mi}_boxes"], out[f"cornell_blas{mi}_links"], out[f"cornell_blas{mi}_values"] = b, l, v
    out["cornell_tlas_boxes"], out["cornell_tlas_links"], out["cornell_tlas_values"] = rs.tlas_nodes()

    field = scenes.instance_field(n_instances=256, level=3, seed=104, extent=25.0)
    fcam = scenes.field_camera(128)
    fcam.position = (0.0, 0.0, -70.0)
    frays = np.concatenate([scenes.primary_rays(fcam, seed=105), scenes.surface_rays(field, 8000, seed=106)])
    fs = ref.scene(field)
    out.update(scene_arrays(field, "field"))
    out["field_rays"] = frays
    out.update(frag_arrays(fs.fragments(frays), "field_hit"))
    b, l, v = fs.blas_nodes(0)
    out["field_blas0_boxes"], out["field_blas0_links"], out["field_blas0_values"] = b, l, v
    out["field_tlas_boxes"], out["field_tlas_links"], out["field_tlas_values"] = fs.tlas_nodes()
    inv = np.empty((len(field.instances), 16), np.float32)
    for i in range(len(field.instances)):
        ref.lib.ref_instance_inverse(fs.handle, i, inv[i].ctypes.data_as(C.POINTER(C.c_float)))
    out["field_inverse"] = inv
    np.savez_compressed(HERE / "trace.npz", **out)


def cmat(m: Material) -> CMaterial:
    c = CMaterial()
    c.diffuse[:] = list(m.diffuse)
    c.specular[:] = list(m.specular)
    c.roughness = m.roughness
    c.emissive[:] = list(m.emissive)
    return c


def sampling_fixtures(ref):
    lib = ref.lib
    fp = C.POINTER(C.c_float)
    rng = np.random.default_rng(201)
    out = {}
    seeds = np.array([0, 1, 7, 12345, 0xDEADBEEF, 0xFFFFFFFF], np.uint32)
    out["xs_seeds"] = seeds
    xs = np.empty((len(seeds), 64), np.uint32)
    ham = np.empty((len(seeds), 64, 2), np.float32)
    for i, s in enumerate(seeds):
        lib.ref_xorshift(int(s), 64, xs[i].ctypes.data_as(C.POINTER(C.c_uint32)))
        lib.ref_hammersley(int(s), 64, ham[i].ctypes.data_as(fp))
    out["xorshift"], out["hammersley"] = xs, ham
    bits = np.concatenate([np.array([0, 1, 0x80000000, 0xFFFFFFFF], np.uint32),
                           rng.integers(0, 2 ** 32, 256, dtype=np.uint64).astype(np.uint32)])
    out["ri_bits"] = bits
    out["ri_value"] = np.array([lib.ref_radical_inverse(int(b)) for b in bits], np.float32)
    tri_xi = rng.random((256, 2)).astype(np.float32)
    tri_out = np.empty((256, 2), np.float32)
    for i in range(256):
        lib.ref_uniform_sample_triangle(tri_xi[i].ctypes.data_as(fp), tri_out[i].ctypes.data_as(fp))
    out["tri_xi"], out["tri_out"] = tri_xi, tri_out
    mt_seeds = np.array([0, 1, 5489, 2 ** 32 - 1, 2 ** 40 + 3], np.uint64)
    mt = np.empty((len(mt_seeds), 700), np.float32)
    for i, s in enumerate(mt_seeds):
        lib.ref_mt_uniform(int(s), 700, mt[i].ctypes.data_as(fp))
    out["mt_seeds"], out["mt_uniform"] = mt_seeds, mt

    # tangent frames, lobes and pdfs on random directions (including near-parallel V/N)
    n = 512
    N = rng.normal(size=(n, 3)); N /= np.linalg.norm(N, axis=1, keepdims=True)
    V = rng.normal(size=(n, 3)); V /= np.linalg.norm(V, axis=1, keepdims=True)
    V[::8] = N[::8] * np.where(rng.random((n // 8, 1)) < 0.5, 1.0, -1.0) + 1e-3 * rng.normal(size=(n // 8, 3))
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    N[5::16] = [0.0, 0.0, 1.0]
    N, V = N.astype(np.float32), V.astype(np.float32)
    out["dir_N"], out["dir_V"] = N, V
    frames = np.empty((n, 9), np.float32)
    for i in range(n):
        lib.ref_tangent_frame(V[i].ctypes.data_as(fp), N[i].ctypes.data_as(fp), frames[i].ctypes.data_as(fp))
    out["frames"] = frames
    xi = rng.random((n, 2)).astype(np.float32)
    xi[:4] = [[0, 0], [0.99999994, 0.5], [0.5, 0.99999994], [1.0, 0.0]]
    R = rng.uniform(0.0, 1.0, n).astype(np.float32)
    R[:3] = [0.0, 1e-4, 1.0]
    out["lobe_xi"], out["lobe_R"] = xi, R
    cs, cp, bs, bp = (np.empty((n, 3), np.float32), np.empty(n, np.float32), np.empty((n, 3), np.float32),
                      np.empty(n, np.float32))
    for i in range(n):
        lib.ref_cos_sample(xi[i].ctypes.data_as(fp), cs[i].ctypes.data_as(fp))
        cp[i] = lib.ref_cos_pdf(cs[i].ctypes.data_as(fp))
        lib.ref_beckmann_sample(xi[i].ctypes.data_as(fp), V[i].ctypes.data_as(fp), float(R[i]), bs[i].ctypes.data_as(fp))
        bp[i] = lib.ref_beckmann_pdf(bs[i].ctypes.data_as(fp), float(R[i]))
    out["cos_sample"], out["cos_pdf"], out["beckmann_sample"], out["beckmann_pdf"] = cs, cp, bs, bp
    refl = rng.uniform(0.0, 1.0, n).astype(np.float32)
    out["pdf_refl"] = refl
    pdfs = np.empty((5, n), np.float32)
    for kind in (DIFFUSE, SPECULAR, DIELECTRIC, LIGHT):
        for i in range(n):
            pdfs[kind, i] = lib.ref_bsdf_pdf(kind, V[i].ctypes.data_as(fp), bs[i].ctypes.data_as(fp), float(R[i]),
                                             float(refl[i]))
    out["bsdf_pdf"] = pdfs

    mats = [Material(diffuse=(0.73, 0.73, 0.73)),
            Material(diffuse=(0.5, 0.2, 0.1), specular=(0.04, 0.04, 0.04), roughness=0.3),
            Material(diffuse=(0.05, 0.05, 0.05), specular=(0.9, 0.8, 0.7), roughness=0.05),
            Material(diffuse=(0.78, 0.78, 0.78), emissive=(17.0, 12.0, 4.0))]
    out["mats"] = np.array([[*m.diffuse, *m.specular, m.roughness, *m.emissive] for m in mats], np.float32)
    m_ids = rng.integers(0, len(mats), n).astype(np.uint32)
    kinds = rng.choice(np.array([DIFFUSE, SPECULAR, DIELECTRIC, LIGHT], np.uint32), n)
    sseeds = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    out["samp_mat"], out["samp_kind"], out["samp_seed"] = m_ids, kinds, sseeds
    L, P, E = np.empty((n, 3), np.float32), np.empty(n, np.float32), np.empty((n, 3), np.float32)
    dl = np.empty(n, np.float32)
    for i in range(n):
        cm = cmat(mats[m_ids[i]])
        p = np.empty(1, np.float32)
        lib.ref_bsdf_sample(int(kinds[i]), C.byref(cm), V[i].ctypes.data_as(fp), N[i].ctypes.data_as(fp),
                            int(sseeds[i]), L[i].ctypes.data_as(fp), p.ctypes.data_as(fp), E[i].ctypes.data_as(fp))
        P[i] = p[0]
        dl[i] = lib.ref_direct_lighting_pdf(int(kinds[i]), C.byref(cm), N[i].ctypes.data_as(fp),
                                            V[i].ctypes.data_as(fp), L[i].ctypes.data_as(fp))
    out["samp_L"], out["samp_P"], out["samp_E"], out["direct_pdf"] = L, P, E, dl

    # matrices, camera rays, view matrix
    M = np.empty((64, 16), np.float32)
    Minv = np.empty((64, 16), np.float32)
    field = scenes.instance_field(n_instances=64, level=0, seed=202)
    for i in range(64):
        M[i] = np.asarray(field.instances[i].transform, np.float32).reshape(-1)
        lib.ref_mat4_inverse(M[i].ctypes.data_as(fp), Minv[i].ctypes.data_as(fp))
    out["mat4"], out["mat4_inverse"] = M, Minv
    cams = [scenes.cornell_camera(64, 64), scenes.field_camera(4096),
            Camera(position=(1.5, -2.0, 3.25), direction=(-0.3, 0.2, -0.9), resolution=(1920, 1080),
                                aspect=1.0, up=(0.0, 1.0, 0.0), far_plane=10000.0)]
    out["cams"] = np.stack([camera_array(c) for c in cams])
    pix = rng.integers(0, 1080, (len(cams), 64, 2)).astype(np.uint32)
    cxi = rng.random((len(cams), 64, 2)).astype(np.float32)
    crays = np.zeros((len(cams), 64), RAY_DTYPE)
    views = np.empty((len(cams), 16), np.float32)
    for c, cam in enumerate(cams):
        cc = cam.to_c()
        for k in range(64):
            lib.ref_generate_ray(C.byref(cc), float(cxi[c, k, 0]), float(cxi[c, k, 1]), int(pix[c, k, 0]),
                                 int(pix[c, k, 1]), crays[c, k:k + 1].ctypes.data)
        lib.ref_view_matrix(C.byref(cc), views[c].ctypes.data_as(fp))
    out["cam_pix"], out["cam_xi"], out["cam_rays"], out["cam_view"] = pix, cxi, crays, views

    # light sampling tables of the Cornell lamp and of a 20-triangle light mesh
    s = scenes.cornell_box()
    s.meshes.append(scenes.icosphere(0))
    s.instances.append(Instance(len(s.meshes) - 1, scenes.glm_storage(scenes.translate([0.5, 0.5, 0.5])
                                                                                   @ scenes.scale(0.05)), LIGHT, 3))
    rs = ref.scene(s)
    out.update(scene_arrays(s, "lights"))
    for mi in (len(s.meshes) - 2, len(s.meshes) - 1):
        a, w, ix = rs.light_table(mi, len(s.meshes[mi].indices))
        out[f"light{mi}_area"], out[f"light{mi}_weight"], out[f"light{mi}_alias"] = a, w, ix
    np.savez_compressed(HERE / "sampling.npz", **out)


def integrator_fixtures(ref):
    out = {}
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(32, 32)
    out.update(scene_arrays(scene, "cornell"))
    out["cam"] = camera_array(cam)
    rs = ref.scene(scene)
    px = np.array([[16, 16], [3, 28], [30, 1], [10, 20], [25, 12], [0, 0]], np.uint32)
    seeds = np.array([1, 2, 99, 12345, 0xFFFFFFFF, 7], np.uint64)
    samples = np.empty((len(px), 48, 3), np.float32)
    for i in range(len(px)):
        samples[i] = rs.integrate(cam, int(px[i, 0]), int(px[i, 1]), 5, int(seeds[i]), 48)
    out["integ_px"], out["integ_seed"], out["integ_samples"] = px, seeds, samples
    idx = np.arange(32 * 32, dtype=np.uint32)
    pseeds = (np.arange(32 * 32, dtype=np.uint64) * np.uint64(2654435761)) % np.uint64(2 ** 32)
    pixels, counts, variance, _ = rs.render_pixels(cam, 5, 16, idx, pseeds, nthreads=1)
    out["render_seeds"], out["render_pixels"], out["render_counts"], out["render_variance"] = pseeds, pixels, counts, variance
    np.savez_compressed(HERE / "integrator.npz", **out)


def atrous_fixtures(ref):
    out = {}
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(96, 80)
    cam.aspect = 1.0
    rs = ref.scene(scene)
    n, p, d = rs.denoiser_inputs(cam)
    out.update(scene_arrays(scene, "cornell"))
    out["cam"] = camera_array(cam)
    out["normals"], out["positions"], out["diffuse"] = n, p, d
    W, H = 96, 80
    idx = np.arange(W * H, dtype=np.uint32)
    pseeds = (np.arange(W * H, dtype=np.uint64) * np.uint64(40503) + np.uint64(17)) % np.uint64(2 ** 32)
    pixels, _, _, _ = rs.render_pixels(cam, 5, 4, idx, pseeds, nthreads=0)
    out["pixels"] = pixels
    res = np.empty(W * H * 3, np.float32)
    fp = C.POINTER(C.c_float)
    args = [np.ascontiguousarray(a, np.float32) for a in (pixels, n, p, d)]
    ref.lib.ref_atrous(*[a.ctypes.data_as(fp) for a in args], W, H, res.ctypes.data_as(fp), 1)
    out["denoised"] = res.reshape(H, W, 3)
    out["tonemapped"] = ref.reinhard(out["denoised"], W, H)   # Util::reinhard_tone_mapping
    np.savez_compressed(HERE / "atrous.npz", **out)
    # render_scene_to_file's output step: std::reverse + stbi_write_hdr, on the
    # tone-mapped image and on a ragged 5 x 3 image (no run-length coding)
    hdr = {"image": out["tonemapped"]}
    small = np.random.default_rng(301).gamma(0.5, 2.0, (3, 5, 3)).astype(np.float32)
    hdr["small"] = small
    hdr["image_file"] = np.frombuffer(ref.hdr_file(out["tonemapped"], W, H, "/tmp/pico_golden.hdr"), np.uint8)
    hdr["small_file"] = np.frombuffer(ref.hdr_file(small, 5, 3, "/tmp/pico_golden_small.hdr"), np.uint8)
    np.savez_compressed(HERE / "hdr.npz", **hdr)


def sky_dirs(rng, n):
    """Random unit directions plus face diagonals, axes and signed zeros."""
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    e = np.array([[1, 1, 0], [1, 0, 1], [0, 1, 1], [1, 1, 1], [-1, 1, -1], [0, 0, 1], [1, 0, 0], [0, 1, 0],
                  [0.5, -0.5, 0.5], [-0.0, 1, 0], [0, -0.0, 1], [3, 4, 0]], np.float32)
    e /= np.linalg.norm(e, axis=1, keepdims=True)
    return np.concatenate([d, e, -e]).astype(np.float32)


def sky_scene(kind, seed):
    rng = np.random.default_rng(seed)
    if kind == SKY_CUBE_RGBA8:
        px = rng.integers(0, 256, (6, 8, 8, 4), dtype=np.uint8)
    else:
        px = (rng.gamma(1.0, 2.0, (16, 32, 4))).astype(np.float32)
    sun = np.array([0.3, -0.4, 0.9], np.float64)
    sun = tuple((sun / np.linalg.norm(sun)).astype(np.float32))
    return Sky(kind, px, True, sun, (4.0, 3.5, 3.0))


def sky_fixtures(ref):
    """ImageCube::sample4 on both sky kinds, and integrator samples / G-buffer of the
    Cornell box under a cube sky and a sun (Integrators.cpp:54-76, 152, 208)."""
    out = {}
    rng = np.random.default_rng(501)
    dirs = sky_dirs(rng, 4096)
    out["dirs"] = dirs
    for name, kind in (("cube", SKY_CUBE_RGBA8), ("equirect", SKY_EQUIRECT_RGBAF)):
        sky = sky_scene(kind, 502 if kind == SKY_CUBE_RGBA8 else 503)
        out.update(sky_arrays(sky, name))
        out[f"{name}_rgba"] = ref.sky_sample(sky, dirs)
    scene = scenes.cornell_box()
    scene.sky_image = sky_scene(SKY_CUBE_RGBA8, 502)
    cam = scenes.cornell_camera(64, 32)
    cam.aspect = 2.0
    out.update(scene_arrays(scene, "cornell"))
    out["cam"] = camera_array(cam)
    rs = ref.scene(scene)
    px = np.array([[32, 16], [2, 16], [62, 30], [20, 8], [45, 25], [0, 0], [40, 16]], np.uint32)
    seeds = np.array([3, 5, 77, 2024, 0xFFFFFFFE, 9, 31337], np.uint64)
    samples = np.empty((len(px), 48, 3), np.float32)
    for i in range(len(px)):
        samples[i] = rs.integrate(cam, int(px[i, 0]), int(px[i, 1]), 5, int(seeds[i]), 48)
    out["integ_px"], out["integ_seed"], out["integ_samples"] = px, seeds, samples
    n, p, d = rs.denoiser_inputs(cam)
    out["normals"], out["positions"], out["diffuse"] = n, p, d
    np.savez_compressed(HERE / "sky.npz", **out)


def shapes_fixtures(ref):
    """Implicit sphere / cube instances, the Transparent, Fresnel and Delta lobes with the
    ray's index-of-refraction stack, and implicit area lights (Cornell box)."""
    out = {}
    scene = scenes.cornell_shapes()
    out.update(scene_arrays(scene, "shapes"))
    rs = ref.scene(scene)
    rng = np.random.default_rng(601)
    n = 8192
    org = rng.uniform(0.05, 0.95, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, RAY_DTYPE)
    rays["org"][:, :3], rays["org"][:, 3] = org, 1.0
    rays["dir"][:, :3], rays["dir"][:, 3] = d, 10000.0
    out["rays"] = rays
    f = rs.fragments(rays)
    for k in ("inst", "prim", "t", "position", "normal"):
        out[f"hit_{k}"] = f[k]
    cam = scenes.cornell_camera(48, 48)
    out["cam"] = camera_array(cam)
    px = np.array([[24, 24], [14, 34], [34, 30], [16, 12], [33, 14], [24, 8], [8, 40], [40, 40]], np.uint32)
    seeds = np.array([11, 12, 13, 14, 15, 16, 17, 18], np.uint64)
    samples = np.empty((len(px), 64, 3), np.float32)
    for i in range(len(px)):
        samples[i] = rs.integrate(cam, int(px[i, 0]), int(px[i, 1]), 6, int(seeds[i]), 64)
    out["integ_px"], out["integ_seed"], out["integ_samples"] = px, seeds, samples
    n_, p_, d_ = rs.denoiser_inputs(cam)
    out["normals"], out["positions"], out["diffuse"] = n_, p_, d_
    np.savez_compressed(HERE / "shapes.npz", **out)


def judge_fixtures(ref, spp: int = 4096):
    """Converged judges: `spp` reference samples per pixel summed in FP64, on 4096 seeded
    pixels of the 256 x 256 Cornell box (depth 5) and 1024 of the 1920 x 1080 lit field
    (depth 8); and for the physical estimator, which the reference lacks, `spp` samples of
    the FP64 oracle on the same lit-field pixels."""
    from judge import relmse, scene_digest
    out = {}
    cases = [("cornell", scenes.cornell_box(), scenes.cornell_camera(256, 256), 5, 4096, 601),
             ("lit", scenes.lit_field(), scenes.lit_field_camera(1920, 1080), 8, 1024, 602)]
    for name, scene, cam, depth, npix, seed in cases:
        W, H = cam.resolution
        rng = np.random.default_rng(seed)
        idx = np.sort(rng.choice(W * H, npix, replace=False)).astype(np.uint32)
        seeds = rng.integers(1, 2**63, npix, dtype=np.uint64)
        rs = ref.scene(scene)
        mean, var, secs = rs.render_mean64(cam, depth, spp, idx, seeds)
        print(f"judge {name}: {npix} pixels x {spp} spp in {secs:.1f} s")
        # the reference's own render loop at 64 spp with its default early exit
        # (max_variance 0, Scene.cpp:185-191): pixels it stopped and its relMSE
        pix, cnt, _, _ = rs.render_pixels(cam, depth, 64, idx, rng.integers(1, 2**63, npix, dtype=np.uint64))
        out[f"{name}_ref64_exited"] = np.array(int((cnt.reshape(-1)[idx] < 64).sum()))
        out[f"{name}_ref64_relmse"] = np.array(relmse(pix.reshape(-1, 3)[idx], mean))
        out.update({f"{name}_idx": idx, f"{name}_mean": mean, f"{name}_var": var, f"{name}_spp": np.array(spp),
                    f"{name}_depth": np.array(depth), f"{name}_res": np.array([W, H]),
                    f"{name}_digest": np.array(scene_digest(scene))})
    # the physical estimator has no reference counterpart: its judge is the FP64 oracle
    oracle = pico_oracle.Oracle()
    scene, cam = scenes.lit_field(), scenes.lit_field_camera(1920, 1080)
    rng = np.random.default_rng(603)
    idx = out["lit_idx"]
    mean, var = oracle.scene(scene).phys_render_mean(cam, 8, spp, idx,
                                                     rng.integers(1, 2**63, len(idx), dtype=np.uint64))
    print(f"judge lit_phys: {len(idx)} pixels x {spp} spp (oracle)")
    out.update({"lit_phys_idx": idx, "lit_phys_mean": mean, "lit_phys_var": var, "lit_phys_spp": np.array(spp),
                "lit_phys_depth": np.array(8), "lit_phys_res": np.array([1920, 1080]),
                "lit_phys_digest": out["lit_digest"], "lit_phys_ref64_exited": np.array(0),
                "lit_phys_ref64_relmse": np.array(np.nan)})
    np.savez_compressed(HERE / "judge.npz", **out)


FIXTURES = {"trace": trace_fixtures, "sampling": sampling_fixtures, "integrator": integrator_fixtures,
            "atrous": atrous_fixtures, "sky": sky_fixtures, "shapes": shapes_fixtures, "judge": judge_fixtures}


def main():
    """python make_golden.py [fixture ...]: all fixtures, or the named ones."""
    pico_oracle.build_reference()
    ref = pico_oracle.Reference()
    for name in (sys.argv[1:] or list(FIXTURES)):
        FIXTURES[name](ref)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
