"""The oracle restatement against golden vectors produced by the Pico reference.

tests/golden/*.npz were written by tests/golden/make_golden.py, which runs the
reference's own sources (oracle/_ref).  Every comparison here is bit-exact:
the oracle restates the reference's float operation order, so any difference
is a restatement bug.
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
from scene_io import load_camera, load_scene, load_sky  # noqa: E402

from pico_gb300.types import Material  # noqa: E402

GOLDEN = HERE / "golden"


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def assert_bits(a, b, what):
    a, b = bits(a), bits(b)
    bad = np.nonzero(a.reshape(len(a), -1) != b.reshape(len(b), -1))[0] if a.ndim else []
    assert a.shape == b.shape and len(bad) == 0, f"{what}: {len(bad)} rows differ (first {list(bad[:5])})"


@pytest.fixture(scope="module")
def trace():
    return np.load(GOLDEN / "trace.npz")


@pytest.fixture(scope="module")
def sampling():
    return np.load(GOLDEN / "sampling.npz")


@pytest.mark.parametrize("prefix", ["cornell", "field"])
def test_closest_hits_match_reference(oracle, trace, prefix):
    scene = load_scene(trace, prefix)
    frags = oracle.scene(scene).fragments(trace[f"{prefix}_rays"])
    for k in ("inst", "prim"):
        np.testing.assert_array_equal(frags[k], trace[f"{prefix}_hit_{k}"], err_msg=k)
    hit = trace[f"{prefix}_hit_inst"] != 0xFFFFFFFF
    assert hit.mean() > 0.2
    for k in ("t", "position", "normal"):
        assert_bits(frags[k][hit], trace[f"{prefix}_hit_{k}"][hit], k)
    # The harness reads (u, v) back from interpolated UVs, (0,0)/(1,0)/(0,1) per
    # vertex: exact values, but a -0.0 barycentric comes back as +0.0.
    for k in ("u", "v"):
        np.testing.assert_array_equal(frags[k][hit], trace[f"{prefix}_hit_{k}"][hit], err_msg=k)


@pytest.mark.parametrize("prefix", ["cornell", "field"])
def test_bvh_topology_matches_reference(oracle, trace, prefix):
    scene = load_scene(trace, prefix)
    os_ = oracle.scene(scene)
    for mi in range(len(scene.meshes)):
        boxes, links, values = os_.blas_nodes(mi)
        assert_bits(boxes, trace[f"{prefix}_blas{mi}_boxes"], f"BLAS {mi} boxes")
        np.testing.assert_array_equal(links, trace[f"{prefix}_blas{mi}_links"])
        np.testing.assert_array_equal(values, trace[f"{prefix}_blas{mi}_values"])
    boxes, links, values = os_.tlas_nodes()
    assert_bits(boxes, trace[f"{prefix}_tlas_boxes"], "TLAS boxes")
    np.testing.assert_array_equal(links, trace[f"{prefix}_tlas_links"])
    np.testing.assert_array_equal(values, trace[f"{prefix}_tlas_values"])


def test_instance_inverse_matches_glm(oracle, trace):
    scene = load_scene(trace, "field")
    got = np.stack([oracle.mat4_inverse(np.asarray(i.transform).reshape(-1)).reshape(-1) for i in scene.instances])
    assert_bits(got, trace["field_inverse"], "inverse")


def test_random_streams(oracle, sampling):
    for i, s in enumerate(sampling["xs_seeds"]):
        np.testing.assert_array_equal(oracle.xorshift(int(s), 64), sampling["xorshift"][i])
        assert_bits(oracle.hammersley(int(s), 64), sampling["hammersley"][i], "hammersley")
    got = np.array([oracle.radical_inverse(int(b)) for b in sampling["ri_bits"]], np.float32)
    assert_bits(got, sampling["ri_value"], "radical inverse")
    got = np.stack([oracle.uniform_sample_triangle(x) for x in sampling["tri_xi"]])
    assert_bits(got, sampling["tri_out"], "uniform_sample_triangle")
    for i, s in enumerate(sampling["mt_seeds"]):
        assert_bits(oracle.mt_uniform(int(s), 700), sampling["mt_uniform"][i], "mt19937_64 uniform")


def test_tangent_frames_and_lobes(oracle, sampling):
    N, V, xi, R = sampling["dir_N"], sampling["dir_V"], sampling["lobe_xi"], sampling["lobe_R"]
    frames = np.stack([oracle.tangent_frame(V[i], N[i]).reshape(-1) for i in range(len(N))])
    assert_bits(frames, sampling["frames"], "tangent frame")
    cs = np.stack([oracle.cos_sample(x) for x in xi])
    assert_bits(cs, sampling["cos_sample"], "cosine sample")
    assert_bits(np.array([oracle.cos_pdf(h) for h in cs], np.float32), sampling["cos_pdf"], "cosine pdf")
    bs = np.stack([oracle.beckmann_sample(xi[i], V[i], float(R[i])) for i in range(len(xi))])
    assert_bits(bs, sampling["beckmann_sample"], "Beckmann sample")
    bp = np.array([oracle.beckmann_pdf(bs[i], float(R[i])) for i in range(len(xi))], np.float32)
    assert_bits(bp, sampling["beckmann_pdf"], "Beckmann pdf")
    refl = sampling["pdf_refl"]
    for kind in (0, 1, 2, 4):
        got = np.array([oracle.bsdf_pdf(kind, V[i], bs[i], float(R[i]), float(refl[i])) for i in range(len(V))],
                       np.float32)
        assert_bits(got, sampling["bsdf_pdf"][kind], f"BSRDF {kind} pdf")


def test_bsdf_samples_and_direct_lighting_pdf(oracle, sampling):
    mats = [Material(tuple(r[0:3]), tuple(r[3:6]), float(r[6]), tuple(r[7:10])) for r in sampling["mats"]]
    N, V = sampling["dir_N"], sampling["dir_V"]
    for i in range(len(N)):
        kind, seed = int(sampling["samp_kind"][i]), int(sampling["samp_seed"][i])
        mat = mats[int(sampling["samp_mat"][i])]
        xi = oracle.hammersley(seed, 2)
        L, P, E = oracle.bsdf_sample(kind, mat, V[i], N[i], xi)
        assert_bits(L, sampling["samp_L"][i], f"sample {i} L")
        assert_bits(np.float32(P), sampling["samp_P"][i], f"sample {i} P")
        assert_bits(E, sampling["samp_E"][i], f"sample {i} energy")
        d = oracle.direct_lighting_pdf(kind, mat, N[i], V[i], sampling["samp_L"][i])
        assert_bits(np.float32(d), sampling["direct_pdf"][i], f"sample {i} direct pdf")


def test_matrices_and_camera(oracle, sampling):
    got = np.stack([oracle.mat4_inverse(m) .reshape(-1) for m in sampling["mat4"]])
    assert_bits(got, sampling["mat4_inverse"], "mat4 inverse")
    for c, arr in enumerate(sampling["cams"]):
        cam = load_camera(arr)
        for k in range(sampling["cam_pix"].shape[1]):
            px, py = (int(v) for v in sampling["cam_pix"][c, k])
            r = oracle.generate_ray(cam, sampling["cam_xi"][c, k], px, py)
            want = sampling["cam_rays"][c, k]
            assert_bits(r["org"], want["org"], "ray origin")
            assert_bits(r["dir"], want["dir"], "ray direction")
        assert_bits(oracle.view_matrix(cam).reshape(-1), sampling["cam_view"][c], "view matrix")


def test_light_tables(oracle, sampling):
    scene = load_scene(sampling, "lights")
    for mi in (len(scene.meshes) - 2, len(scene.meshes) - 1):
        w = oracle.triangle_weights(scene, mi)
        assert_bits(w, sampling[f"light{mi}_area"], "triangle weights")
        bw, ba = oracle.alias_build(w)
        assert_bits(bw, sampling[f"light{mi}_weight"], "alias weights")
        np.testing.assert_array_equal(ba, sampling[f"light{mi}_alias"])


def test_integrator_samples_match_reference(oracle):
    z = np.load(GOLDEN / "integrator.npz")
    scene, cam = load_scene(z, "cornell"), load_camera(z["cam"])
    os_ = oracle.scene(scene)
    for i, (px, py) in enumerate(z["integ_px"]):
        got = os_.integrate(cam, int(px), int(py), 5, int(z["integ_seed"][i]), z["integ_samples"].shape[1])
        assert_bits(got, z["integ_samples"][i], f"pixel {i} samples")


def test_render_loop_matches_reference(oracle):
    z = np.load(GOLDEN / "integrator.npz")
    scene, cam = load_scene(z, "cornell"), load_camera(z["cam"])
    W, H = cam.resolution
    pixels, counts, variance = oracle.scene(scene).render_pixels(cam, 5, 16, np.arange(W * H), z["render_seeds"])
    assert_bits(pixels, z["render_pixels"], "mean")
    np.testing.assert_array_equal(counts, z["render_counts"])
    assert_bits(variance, z["render_variance"], "variance")


def test_denoiser_inputs_and_atrous_match_reference(oracle):
    z = np.load(GOLDEN / "atrous.npz")
    scene, cam = load_scene(z, "cornell"), load_camera(z["cam"])
    n, p, d = oracle.scene(scene).denoiser_inputs(cam)
    assert_bits(n, z["normals"], "normals")
    assert_bits(p, z["positions"], "positions")
    assert_bits(d, z["diffuse"], "albedo")
    W, H = cam.resolution
    out = oracle.atrous(z["pixels"], n, p, d, W, H)
    assert_bits(out, z["denoised"], "a-trous output")


def test_reinhard_matches_reference(oracle):
    z = np.load(GOLDEN / "atrous.npz")
    W, H = load_camera(z["cam"]).resolution
    assert_bits(oracle.reinhard(z["denoised"], W, H), z["tonemapped"], "tone mapped")


def test_hdr_file_matches_reference(oracle):
    """Reversal plus stbi_write_hdr, byte for byte (run-length coded and raw widths)."""
    z = np.load(GOLDEN / "hdr.npz")
    H, W = z["image"].shape[:2]
    assert oracle.hdr_file(z["image"], W, H) == z["image_file"].tobytes()
    assert oracle.hdr_file(z["small"], 5, 3) == z["small_file"].tobytes()


def test_sky_lookup_matches_reference(oracle):
    """ImageCube::sample4 on a 6-face RGBA8 cube and an RGBA float HDRI, including
    face diagonals, axes and signed zeros."""
    z = np.load(GOLDEN / "sky.npz")
    for name in ("cube", "equirect"):
        got = oracle.sky_sample(load_sky(z, name), z["dirs"])
        assert_bits(got, z[f"{name}_rgba"], f"{name} sky")


def test_integrator_with_sky_and_sun_matches_reference(oracle):
    """integrate_ray with sky radiance on misses and the sun in the light pick."""
    z = np.load(GOLDEN / "sky.npz")
    scene, cam = load_scene(z, "cornell"), load_camera(z["cam"])
    assert scene.sky_image is not None and scene.sky_image.use_sun
    os_ = oracle.scene(scene)
    for i, (px, py) in enumerate(z["integ_px"]):
        got = os_.integrate(cam, int(px), int(py), 5, int(z["integ_seed"][i]), z["integ_samples"].shape[1])
        assert_bits(got, z["integ_samples"][i], f"pixel {i} samples")
    n, p, d = os_.denoiser_inputs(cam)
    for got, key in ((n, "normals"), (p, "positions"), (d, "diffuse")):
        assert_bits(got, z[key], f"G-buffer {key}")


def test_implicit_shapes_match_reference(oracle):
    """LowerLevelSphereBVH / LowerLevelCube hits through scaled, rotated instances."""
    z = np.load(GOLDEN / "shapes.npz")
    f = oracle.scene(load_scene(z, "shapes")).fragments(z["rays"])
    for k in ("inst", "prim"):
        np.testing.assert_array_equal(f[k], z[f"hit_{k}"], err_msg=k)
    hit = z["hit_inst"] != 0xFFFFFFFF
    assert (z["hit_prim"] == 0xFFFFFFFE).sum() > 1000
    for k in ("t", "position", "normal"):
        assert_bits(f[k][hit], z[f"hit_{k}"][hit], k)


def test_integrator_with_btdfs_and_implicit_lights_matches_reference(oracle):
    """Transparent and Fresnel glass (index-of-refraction stack), a Delta mirror, and
    sphere / cube area lights, sample for sample."""
    z = np.load(GOLDEN / "shapes.npz")
    scene, cam = load_scene(z, "shapes"), load_camera(z["cam"])
    os_ = oracle.scene(scene)
    for i, (px, py) in enumerate(z["integ_px"]):
        got = os_.integrate(cam, int(px), int(py), 6, int(z["integ_seed"][i]), z["integ_samples"].shape[1])
        assert_bits(got, z["integ_samples"][i], f"pixel {i} samples")
    n, p, d = os_.denoiser_inputs(cam)
    for got, key in ((n, "normals"), (p, "positions"), (d, "diffuse")):
        assert_bits(got, z[key], f"G-buffer {key}")


def test_accumulate_drops_first_sample(oracle):
    """Scene.cpp:185-191: mean += (x - mean) / prev_count, so the first sample is replaced."""
    s = np.array([[10, 10, 10], [1, 1, 1], [3, 3, 3]], np.float32)
    px, count, var = oracle.accumulate(s, 16)
    assert count == 3 and np.allclose(px, 2.0)
