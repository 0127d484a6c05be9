"""Rendering, shading and denoising on the GPU against the oracle.

* BSRDF pdf / sample and the direct-lighting pdf on the reference's own golden
  inputs: within 1e-5 (the only differences come from CUDA's cosf/sinf/logf/expf
  against the host libm).
* Denoiser inputs (one primary ray per pixel): bit-exact.
* A-trous on identical G-buffers: within 1e-4 relative, NaN where the reference
  produces NaN.
* The Monte Carlo render: statistically, per pixel, against the oracle's
  restatement of the reference integrator run with the reference's own random
  streams (the GPU draws different random numbers, so the test compares means
  within a few standard errors).
* The progressive-buffer contract of Scene::render_scene_to_memory: counts,
  resume, early exit, cancellation.
"""
import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

import pico_gb300
from pico_gb300 import scenes
from pico_gb300.types import Material

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
from scene_io import load_camera, load_scene, load_sky  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = HERE / "golden"


def test_bsdf_routines_match_reference(ctx, oracle):
    z = np.load(GOLDEN / "sampling.npz")
    mats = [Material(tuple(r[0:3]), tuple(r[3:6]), float(r[6]), tuple(r[7:10])) for r in z["mats"]]
    n = len(z["samp_kind"])
    kinds = z["samp_kind"]
    mat_list = [mats[int(i)] for i in z["samp_mat"]]
    xi = np.stack([oracle.hammersley(int(s), 2).reshape(-1) for s in z["samp_seed"]])
    H = z["beckmann_sample"]
    pdf, L, P, E, dl = ctx.bsdf_eval(kinds, mat_list, z["dir_V"], z["dir_N"], H, xi)
    # BSRDF::pdf(wo = V, H) for each lobe kind, against the reference value
    refl = np.array([np.linalg.norm(m.specular) / (np.linalg.norm(m.specular) + np.linalg.norm(m.diffuse))
                     for m in mat_list], np.float32)
    want_pdf = np.array([oracle.bsdf_pdf(int(kinds[i]), z["dir_V"][i], H[i], mat_list[i].roughness, float(refl[i]))
                         for i in range(n)], np.float32)
    np.testing.assert_allclose(pdf, want_pdf, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(L, z["samp_L"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(P, z["samp_P"], rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(E, z["samp_E"])
    np.testing.assert_allclose(dl, z["direct_pdf"], rtol=1e-5, atol=1e-5)


def test_denoiser_inputs_bit_exact(ctx, oracle):
    """In the reference's traversal order the G-buffer is bit-exact; near-first
    differs only on pixels whose primary ray grazes the edge where two box-aligned
    walls meet, where the reference's own slab test decides between near-equal hits."""
    z = np.load(GOLDEN / "atrous.npz")
    scene, cam = load_scene(z, "cornell"), load_camera(z["cam"])
    gs = ctx.upload(scene)
    try:
        ctx.set_traversal_order(1)
        n, p, d = gs.denoiser_inputs(cam)
    finally:
        ctx.set_traversal_order(0)
    for got, key in ((n, "normals"), (p, "positions"), (d, "diffuse")):
        np.testing.assert_array_equal(got.view(np.uint32), z[key].view(np.uint32), err_msg=key)
    n2, p2, d2 = gs.denoiser_inputs(cam)
    differ = (p2 != z["positions"]).any(axis=2)
    assert differ.mean() < 1e-3
    # the near-first choice is an equally near hit: positions agree to float precision
    np.testing.assert_allclose(p2[differ], z["positions"][differ], rtol=1e-5, atol=1e-5)


def atrous_close(got, want, rtol=1e-4):
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    np.testing.assert_array_equal(nan_g, nan_w)
    ok = ~nan_w
    np.testing.assert_allclose(got[ok], want[ok], rtol=rtol, atol=1e-6)


def test_atrous_matches_reference(ctx):
    z = np.load(GOLDEN / "atrous.npz")
    W, H = load_camera(z["cam"]).resolution
    got = ctx.atrous(z["pixels"], z["normals"], z["positions"], z["diffuse"], W, H)
    atrous_close(got, z["denoised"])


@pytest.mark.parametrize("W,H", [(64, 64), (130, 70), (17, 200)])
def test_atrous_ragged_sizes(ctx, oracle, W, H):
    """Partial tiles at the right and bottom edges and tiles narrower than the tap span."""
    rng = np.random.default_rng(W * 1000 + H)
    pix = rng.gamma(1.0, 1.0, (H, W, 3)).astype(np.float32)
    nrm = rng.normal(size=(H, W, 3)).astype(np.float32)
    pos = rng.normal(size=(H, W, 3)).astype(np.float32) * 3
    dif = rng.random((H, W, 3)).astype(np.float32)
    got = ctx.atrous(pix, nrm, pos, dif, W, H)
    atrous_close(got, oracle.atrous(pix, nrm, pos, dif, W, H))


def test_tonemap_matches_reference(ctx):
    """Util::reinhard_tone_mapping: exact float operations, so bit-exact."""
    z = np.load(GOLDEN / "atrous.npz")
    W, H = load_camera(z["cam"]).resolution
    got = ctx.tonemap(z["denoised"], W, H)
    np.testing.assert_array_equal(np.isnan(got), np.isnan(z["tonemapped"]))
    ok = ~np.isnan(got)
    np.testing.assert_array_equal(got[ok].view(np.uint32), z["tonemapped"][ok].view(np.uint32))


def test_hdr_encoding_byte_identical(ctx):
    """The device RGBE + run-length encoder against stbi_write_hdr's bytes."""
    z = np.load(GOLDEN / "hdr.npz")
    H, W = z["image"].shape[:2]
    flipped = z["image"].reshape(-1, 3)[::-1].copy()    # render_scene_to_file reverses first
    assert ctx.encode_hdr(flipped, W, H) == z["image_file"].tobytes()
    assert ctx.encode_hdr(z["small"].reshape(-1, 3)[::-1].copy(), 5, 3) == z["small_file"].tobytes()


def test_render_to_file(ctx, oracle, tmp_path):
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(40, 24)
    cam.aspect = 1.0
    gs = ctx.upload(scene)
    path = tmp_path / "out.hdr"
    pix, cnt, var = gs.render_to_file(cam, 3, 4, path, seed=5)
    # the caller's buffer is left reversed, as std::reverse leaves it in the reference
    data = path.read_bytes()
    assert data == oracle.hdr_file(pix.reshape(-1, 3)[::-1].copy(), 40, 24)
    assert data.startswith(b"#?RADIANCE\n")


def test_render_denoise_and_tonemap_pipeline(ctx, oracle):
    """render -> a-trous -> Reinhard, the post-processing order of Scene.cpp:212-234."""
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(64, 64)
    gs = ctx.upload(scene)
    raw, _, _ = gs.render(cam, 5, 8, seed=21)
    final, _, _ = gs.render(cam, 5, 8, seed=21, denoise=True, tonemap=True)
    n, p, d = gs.denoiser_inputs(cam)
    want = oracle.reinhard(oracle.atrous(raw, n, p, d, 64, 64), 64, 64)
    atrous_close(final, want)


def test_atrous_device_path(ctx, oracle):
    torch = pytest.importorskip("torch")
    z = np.load(GOLDEN / "atrous.npz")
    W, H = load_camera(z["cam"]).resolution
    d = [torch.from_numpy(np.ascontiguousarray(z[k])).cuda() for k in ("pixels", "normals", "positions", "diffuse")]
    out = torch.empty_like(d[0])
    stream = torch.cuda.current_stream().cuda_stream
    ctx.atrous_device(*[t.data_ptr() for t in d], W, H, out.data_ptr(), stream)
    torch.cuda.synchronize()
    atrous_close(out.cpu().numpy(), z["denoised"])


def batch_means(render_batch, K):
    """K independent renders (fresh progressive buffers each): mean and standard
    error per pixel channel from the spread of the batch means.  The estimator has
    rare high-value paths, so one render's own variance buffer underestimates the
    error of some pixels; batch means do not."""
    imgs, counts = [], []
    for k in range(K):
        pix, cnt = render_batch(k)
        imgs.append(pix)
        counts.append(cnt)
    imgs = np.stack(imgs)
    return imgs.mean(0), imgs.std(0, ddof=1) / np.sqrt(K), np.stack(counts)


def test_render_statistically_matches_reference(ctx, oracle):
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(48, 48)
    W, H = cam.resolution
    K, spp, depth = 16, 32, 5
    gs = ctx.upload(scene)
    os_ = oracle.scene(scene)
    idx = np.arange(W * H, dtype=np.uint32)
    rng = np.random.default_rng(77)

    def gpu_batch(k):
        pix, cnt, _ = gs.render(cam, depth, spp, seed=1000 + k)
        return pix, cnt

    def ref_batch(k):
        pix, cnt, _ = os_.render_pixels(cam, depth, spp, idx, rng.integers(0, 2 ** 32, W * H, dtype=np.uint64))
        return pix, cnt

    g_mean, g_se, g_cnt = batch_means(gpu_batch, K)
    r_mean, r_se, r_cnt = batch_means(ref_batch, K)
    # a second, independent oracle batch set calibrates the bars: the same statistics of
    # oracle against oracle bound those of device against oracle (binomial margins over pixels)
    o_mean, o_se, _ = batch_means(ref_batch, K)

    def zs(m, se):
        return (m - r_mean) / np.maximum(np.sqrt(se ** 2 + r_se ** 2), 1e-6)

    z, zo = zs(g_mean, g_se), zs(o_mean, o_se)
    npx = W * H
    for label, a, b in (("beyond 4 SE", np.abs(z) > 4, np.abs(zo) > 4), ("above +4 SE", z > 4, zo > 4)):
        p = max(b.mean(), 1.0 / npx)
        assert a.mean() <= b.mean() + 4 * np.sqrt(2 * p * (1 - p) / npx), (label, a.mean(), b.mean())
    q = (zo > 0).mean()
    assert abs((z > 0).mean() - q) <= 4 * np.sqrt(2 * q * (1 - q) / npx), ((z > 0).mean(), q)
    assert np.abs(z).mean() < np.abs(zo).mean() + 0.15, (np.abs(z).mean(), np.abs(zo).mean())
    # pixels that only see the black sky stop after 6 samples in both
    # (variance exactly 0 after more than 4 samples, Scene.cpp:196-197)
    sky = sky_pixels(oracle, scene, cam)
    assert sky.any() and (g_cnt[:, sky] == 6).all() and (r_cnt[:, sky] == 6).all()
    assert abs(g_mean.mean() - r_mean.mean()) < 0.01 * r_mean.mean()


def sky_pixels(oracle, scene, cam):
    """Pixels whose primary rays miss everything for every jitter (xi in [0, 1)^2 -> [0, 0.5) px)."""
    W, H = cam.resolution
    os_ = oracle.scene(scene)
    miss = np.ones((H, W), bool)
    for xi in ((0.0, 0.0), (0.9999, 0.0), (0.0, 0.9999), (0.9999, 0.9999)):
        rays = np.stack([oracle.generate_ray(cam, xi, x, y) for y in range(H) for x in range(W)])
        miss &= (os_.trace(rays)["inst"] == pico_gb300.MISS).reshape(H, W)
    return miss


def test_render_counts_resume_and_cancel(ctx):
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(32, 32)
    gs = ctx.upload(scene)
    pix, cnt, var = gs.render(cam, 5, 8, seed=3)
    # a pixel with a non-zero mean has a positive variance, so it never stops early
    inside = (pix > 0).any(axis=2)
    assert inside.mean() > 0.5 and (cnt[inside] == 8).all()
    before = cnt.copy()
    # a second call runs max_samples more samples on every pixel below max_samples
    pix, cnt, var = gs.render(cam, 5, 16, seed=4, pixels=pix, sample_count=cnt, variance=var)
    assert (cnt[inside] == before[inside] + 16).all()
    # pixels at or above max_samples are skipped
    pix2, cnt2, var2 = gs.render(cam, 5, 8, seed=5, pixels=pix.copy(), sample_count=cnt.copy(), variance=var.copy())
    np.testing.assert_array_equal(cnt2[inside], cnt[inside])
    # cancellation before the first batch leaves the buffers untouched
    flag = C.c_int32(1)
    with pytest.raises(pico_gb300.PicoError) as e:
        gs.render(cam, 5, 64, seed=6, pixels=pix.copy(), sample_count=cnt.copy(), variance=var.copy(),
                  should_quit=flag)
    assert e.value.status == -6


def test_render_with_denoise_matches_atrous_of_render(ctx, oracle):
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(64, 64)
    gs = ctx.upload(scene)
    raw, cnt, var = gs.render(cam, 5, 8, seed=11)
    den, cnt2, var2 = gs.render(cam, 5, 8, seed=11, denoise=True)
    np.testing.assert_array_equal(cnt, cnt2)
    n, p, d = gs.denoiser_inputs(cam)   # the same traversal order the render used
    atrous_close(den, oracle.atrous(raw, n, p, d, 64, 64))


def test_render_instance_field_runs(ctx):
    """Many instances, a Lambert field lit by two quad lights; checks finite, non-trivial output."""
    s = scenes.instance_field(n_instances=128, level=2, seed=17, extent=8.0)
    s.materials.append(Material(diffuse=(0.8, 0.8, 0.8), emissive=(20.0, 20.0, 20.0)))
    for k, y in enumerate((12.0, -12.0)):
        s.meshes.append(scenes.quad_mesh([[-4, y, -4], [4, y, -4], [4, y, 4], [-4, y, 4]], [0, -np.sign(y), 0]))
        s.instances.append(pico_gb300.Instance(len(s.meshes) - 1, scenes.glm_storage(np.eye(4)), pico_gb300.LIGHT, 1))
    cam = scenes.field_camera(64)
    cam.position = (0.0, 0.0, -25.0)
    gs = ctx.upload(s)
    assert gs.info()["lights"] == 2
    pix, cnt, var = gs.render(cam, 5, 16, seed=2)
    assert np.isfinite(pix).all() and pix.mean() > 0.0


def test_render_stats_count_the_work(ctx):
    """pico_gpu_render_stats: samples added equal the growth of sample_count; rays are bounded by the paths."""
    scene = scenes.cornell_box()
    cam = scenes.cornell_camera(32, 24)
    gs = ctx.upload(scene)
    depth, spp = 5, 8
    pix, cnt, var = gs.render(cam, depth, spp, seed=3)
    st = ctx.render_stats()
    assert st["samples"] == int(cnt.sum()) > 0
    assert st["camera_paths"] >= st["samples"]
    assert st["camera_paths"] <= 32 * 24 * spp
    assert 0 < st["bounce_rays"] <= st["camera_paths"] * depth
    assert 0 < st["shadow_rays"] <= st["camera_paths"] + st["bounce_rays"]
    assert st["gbuffer_rays"] == 0
    # a second call continues the progressive buffers: only the new samples are counted
    gs.render(cam, depth, 2 * spp, seed=4, pixels=pix, sample_count=cnt, variance=var, denoise=True)
    st2 = ctx.render_stats()
    assert st2["samples"] == int(cnt.sum()) - st["samples"]
    assert st2["gbuffer_rays"] == 32 * 24


def test_denoiser_inputs_with_sky_bit_exact(ctx, oracle):
    """Misses take the sky texel as albedo (Scene.cpp:283-288): the cube sky bit-exact,
    the equirectangular one exact except where atan2 / asin land on a texel edge."""
    z = np.load(GOLDEN / "sky.npz")
    scene, cam = load_scene(z, "cornell"), load_camera(z["cam"])
    gs = ctx.upload(scene)
    try:
        ctx.set_traversal_order(1)
        n, p, d = gs.denoiser_inputs(cam)
    finally:
        ctx.set_traversal_order(0)
    for got, key in ((n, "normals"), (p, "positions"), (d, "diffuse")):
        np.testing.assert_array_equal(got.view(np.uint32), z[key].view(np.uint32), err_msg=key)
    miss = (np.abs(p).max(-1) > 100)
    assert miss.mean() > 0.2 and (d[miss] > 0).any()
    # an HDRI sky seen by a wide camera
    scene.sky_image = load_sky(z, "equirect")
    wide = load_camera(z["cam"])
    wide.position, wide.direction = (0.5, 0.5, -0.2), (0.3, 0.4, -1.0)
    gs2 = ctx.upload(scene)
    _, _, d2 = gs2.denoiser_inputs(wide)
    _, _, w2 = oracle.scene(scene).denoiser_inputs(wide)
    same = (d2.view(np.uint32) == w2.view(np.uint32)).all(-1)
    assert same.mean() > 0.999, f"{(~same).sum()} albedo texels differ"


def test_render_with_sky_and_sun_statistically_matches(ctx, oracle):
    """Camera misses see the sky, escaping bounces add throughput * sky, and the sun
    joins the light pick; per-pixel batch means agree with the oracle."""
    z = np.load(GOLDEN / "sky.npz")
    scene, cam = load_scene(z, "cornell"), load_camera(z["cam"])
    W, H = cam.resolution
    K, spp, depth = 16, 16, 5
    gs = ctx.upload(scene)
    os_ = oracle.scene(scene)
    idx = np.arange(W * H, dtype=np.uint32)
    rng = np.random.default_rng(78)

    def gpu_batch(k):
        pix, cnt, _ = gs.render(cam, depth, spp, seed=2000 + k, max_variance=-1.0)
        return pix, cnt

    def ref_batch(k):
        pix, cnt, _ = os_.render_pixels(cam, depth, spp, idx, rng.integers(0, 2 ** 32, W * H, dtype=np.uint64),
                                        max_variance=-1.0)
        return pix, cnt

    g_mean, g_se, _ = batch_means(gpu_batch, K)
    r_mean, r_se, _ = batch_means(ref_batch, K)
    z_ = np.abs(g_mean - r_mean) / np.maximum(np.sqrt(g_se ** 2 + r_se ** 2), 1e-6)
    frac = (z_ <= 4.0).mean()
    assert frac >= 0.995, f"only {frac:.4f} of pixel channels within 4 standard errors"
    assert z_.mean() < 1.0, f"mean |z| {z_.mean():.3f}"
    assert abs(g_mean.mean() - r_mean.mean()) < 0.01 * r_mean.mean()


def test_btdf_and_delta_lobes_match_oracle(ctx, oracle):
    """Transparent_BTDF, Fresnel_BTDF and Specular_Delta_BRDF samples on a fresh
    index-of-refraction stack {1.0}: directions and pdfs within 1e-5 (the device's
    cosf / sinf / logf / expf differ from libm by a few ulp), energies exact, and
    total internal reflection (a NaN direction) in the same cases."""
    rng = np.random.default_rng(91)
    n = 3000
    kinds = np.array([3, 5, 6] * (n // 3), np.uint32)
    N = rng.normal(size=(n, 3)).astype(np.float32)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    V = rng.normal(size=(n, 3)).astype(np.float32)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    mats = [Material(tuple(rng.uniform(0.1, 0.9, 3)), tuple(rng.uniform(0.02, 0.9, 3)), float(rng.uniform(0.05, 1.0)),
                     (0.0, 0.0, 0.0), float(rng.choice([1.33, 1.5, 2.4]))) for _ in range(n)]
    xi = rng.random((n, 4), dtype=np.float32)
    H = np.tile(np.array([0, 0, 1], np.float32), (n, 1))
    pdf, L, P, E, _ = ctx.bsdf_eval(kinds, mats, V, N, H, xi)
    for i in range(n):
        wl, wp, we = oracle.bsdf_sample(int(kinds[i]), mats[i], V[i], N[i], xi[i])
        assert np.isnan(L[i]).any() == np.isnan(wl).any(), i
        if not np.isnan(wl).any():
            np.testing.assert_allclose(L[i], wl, rtol=1e-4, atol=1e-5, err_msg=f"L {i} kind {kinds[i]}")
            np.testing.assert_allclose(P[i], wp, rtol=1e-4, atol=1e-6, err_msg=f"P {i} kind {kinds[i]}")
        np.testing.assert_array_equal(E[i], we)


def test_denoiser_inputs_with_shapes_bit_exact(ctx):
    """G-buffer over implicit shapes and glass, in the reference's traversal order."""
    z = np.load(GOLDEN / "shapes.npz")
    scene, cam = load_scene(z, "shapes"), load_camera(z["cam"])
    gs = ctx.upload(scene)
    try:
        ctx.set_traversal_order(1)
        n, p, d = gs.denoiser_inputs(cam)
    finally:
        ctx.set_traversal_order(0)
    for got, key in ((n, "normals"), (p, "positions"), (d, "diffuse")):
        np.testing.assert_array_equal(got.view(np.uint32), z[key].view(np.uint32), err_msg=key)


def test_render_with_btdfs_and_implicit_lights_statistically_matches(ctx, oracle):
    """Glass spheres (index-of-refraction stack), a mirror cube and sphere / cube
    lights: per-pixel batch means agree with the oracle."""
    scene = scenes.cornell_shapes()
    cam = scenes.cornell_camera(40, 40)
    W, H = cam.resolution
    K, spp, depth = 16, 32, 6
    gs = ctx.upload(scene)
    os_ = oracle.scene(scene)
    idx = np.arange(W * H, dtype=np.uint32)
    rng = np.random.default_rng(79)

    def gpu_batch(k):
        pix, cnt, _ = gs.render(cam, depth, spp, seed=3000 + k, max_variance=-1.0)
        return pix, cnt

    def ref_batch(k):
        pix, cnt, _ = os_.render_pixels(cam, depth, spp, idx, rng.integers(0, 2 ** 32, W * H, dtype=np.uint64),
                                        max_variance=-1.0)
        return pix, cnt

    g_mean, g_se, _ = batch_means(gpu_batch, K)
    r_mean, r_se, _ = batch_means(ref_batch, K)
    z_ = np.abs(g_mean - r_mean) / np.maximum(np.sqrt(g_se ** 2 + r_se ** 2), 1e-6)
    frac = (z_ <= 4.0).mean()
    assert frac >= 0.995, f"only {frac:.4f} of pixel channels within 4 standard errors"
    assert z_.mean() < 1.0, f"mean |z| {z_.mean():.3f}"
    assert abs(g_mean.mean() - r_mean.mean()) < 0.02 * r_mean.mean()


def stacked_lights_scene() -> "pico_gb300.types.SceneData":
    """Quad lights over a few icospheres and a ground, built so that shadow rays end at
    every distance from their lights: light B hangs just below light A (rays aimed at A
    end on B), a sphere sits just under light C and another right beside it, and a sun
    shines through the gaps."""
    from pico_gb300.types import DIFFUSE, DIELECTRIC, LIGHT, Instance, SceneData, Sky
    s = SceneData(materials=[Material(diffuse=(0.6, 0.6, 0.6))], sky=(0.0, 0.0, 0.0))
    s.sky_image = Sky(use_sun=True, sun_direction=(0.3, -1.0, 0.2), sun_colour=(2.0, 1.8, 1.5))
    s.meshes.append(scenes.quad_mesh([[-30, 0, -30], [-30, 0, 30], [30, 0, 30], [30, 0, -30]], [0, 1, 0]))
    s.instances.append(Instance(0, scenes.glm_storage(np.eye(4)), DIFFUSE, 0))
    s.meshes.append(scenes.icosphere(2))
    s.materials.append(scenes.metalness_roughness((0.7, 0.4, 0.3), 0.0, 0.6))
    for pos, r in (((0, 1.5, 0), 1.5), ((4, 1, 3), 1.0), ((-5, 2, -2), 2.0), ((8, 8.6, 0), 1.0),
                   ((9.4, 8.0, 1.5), 0.5), ((-3, 6, 4), 1.2)):
        T = scenes.translate(pos) @ scenes.scale(r)
        s.instances.append(Instance(1, scenes.glm_storage(T), DIELECTRIC, 1))
    for (cx, y, cz, h, le) in ((0, 10, 0, 3, 8.0), (0, 9.6, 0, 1.2, 20.0), (8, 10, 0, 2, 15.0),
                               (-8, 12, 6, 2.5, 5.0)):
        s.meshes.append(scenes.quad_mesh([[cx - h, y, cz - h], [cx + h, y, cz - h], [cx + h, y, cz + h],
                                          [cx - h, y, cz + h]], [0, -1, 0]))
        s.materials.append(Material(diffuse=(0.8, 0.8, 0.8), emissive=(le, le, le)))
        s.instances.append(Instance(len(s.meshes) - 1, scenes.glm_storage(np.eye(4)), LIGHT, len(s.materials) - 1))
    return s


@pytest.mark.parametrize("scene_name", ["stacked_lights", "lit_field"])
def test_shadow_early_exit_keeps_images(ctx, scene_name):
    """A closest-hit shadow ray of the near-first walk stops at a hit nearer than every
    light's box (a sun ray at its first hit), the reference order never stops early; both
    walks return the oracle's hits, so the renders must agree bit for bit."""
    if scene_name == "stacked_lights":
        scene = stacked_lights_scene()
        cam = pico_gb300.types.Camera(position=(0.0, 6.0, -22.0), direction=(0.0, -0.1, 1.0),
                                      resolution=(64, 48), aspect=64 / 48)
    else:
        scene = scenes.lit_field(n_instances=256, level=2, seed=77, n_lights=6, extent=20.0)
        cam = scenes.lit_field_camera(64, 48)
    gs = ctx.upload(scene)
    out = {}
    try:
        for order in (1, 0):
            ctx.set_traversal_order(order)
            out[order] = gs.render(cam, 5, 16, seed=9, max_variance=-1.0)
    finally:
        ctx.set_traversal_order(0)
        gs.free()
    for g, w, name in zip(out[0], out[1], ("pixels", "sample counts", "variance")):
        np.testing.assert_array_equal(g, w, err_msg=name)
    assert out[0][0].mean() > 0.0
