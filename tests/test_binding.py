"""The reference-side binding, compiled against the Pico tree's own headers.

pico_gb300/integration/pico_scene_binding.cpp is what Pico's Scene runs in place of
its tiled CPU integrator (Scene::render_scene_to_memory, Core/Scene.hpp:68).  This
test compiles it, with a small driver, against the reference's Core/Scene.hpp and
Core/Camera.hpp and include/pico_gpu.h, links both against libpico_gpu.so with
--no-undefined, and runs the driver's conversions of the reference's own Camera and
RenderParams (no device needed): a renamed field, a changed signature or struct
layout on either side fails here.  The Pico tree is the one the oracle's reference
harness was built from (its path is recorded beside the harness); without it the
test is skipped.
"""
import subprocess
from pathlib import Path

import pytest

from pico_gb300 import build

ROOT = Path(__file__).resolve().parent.parent
BINDING = ROOT / "pico_gb300" / "integration"

DRIVER = r'''
#include "pico_scene_binding.hpp"
#include <cstdio>
int main()
{
    Scene::Camera cam(glm::vec3(1.0f, 2.0f, 3.0f), glm::vec3(0.0f, 0.0f, 1.0f), 1.5f, 0.25f, 50.0f, 40.0f);
    cam.setUp(glm::vec3(0.0f, 1.0f, 0.0f));
    glm::vec3 pixels[6] = {}, variance[6] = {};
    uint32_t counts[6] = {};
    const Scene::RenderParams params{5u, 16u, 0.5f, 2u, 3u, true, false, pixels, counts, variance};
    const pico_camera c = pico_binding::to_pico_camera(cam, params);
    const pico_render_config r = pico_binding::to_render_config(params, PICO_ESTIMATOR_PHYSICAL, 99u);
    std::printf("%g %g %g %g %g %g %g %g %g %u %u %g %g %g %g\n", c.position[0], c.position[1], c.position[2],
                c.direction[0], c.direction[1], c.direction[2], c.up[0], c.up[1], c.up[2], c.resolution[0],
                c.resolution[1], c.aspect, c.near_plane, c.far_plane, c.fov);
    std::printf("%u %u %g %u %u %d %d %u %llu\n", r.max_ray_depth, r.max_samples, r.max_variance, r.height, r.width,
                r.tonemap, r.denoise, r.estimator, (unsigned long long)r.seed);
    pico_binding::SceneGpu gpu;   // no context opened: rendering returns an argument error
    std::printf("%d\n", pico_binding::render_scene_to_memory(gpu, cam, params, nullptr));
    return 0;
}
'''


def test_binding_compiles_links_and_converts_the_reference_types(tmp_path):
    import pico_oracle
    tree = pico_oracle.reference_tree()
    if tree is None:
        pytest.skip("the Pico source tree is not on this machine")
    lib = build.build()
    inc = [f"-I{p}" for p in (tree, tree / "Source", tree / "ThirdParty" / "glm",
                               tree / "ThirdParty" / "assimp-4.1.0" / "include", tree / "ThirdParty" / "stb_image",
                               tree / "ThirdParty" / "jsoncpp" / "include", ROOT / "include", BINDING)]
    flags = ["-std=c++20", "-O1", "-DGLM_ENABLE_EXPERIMENTAL", "-w", *inc]
    (tmp_path / "driver.cpp").write_text(DRIVER)
    for src, obj in ((BINDING / "pico_scene_binding.cpp", "binding.o"), (tmp_path / "driver.cpp", "driver.o")):
        r = subprocess.run(["g++", *flags, "-c", str(src), "-o", str(tmp_path / obj)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
    exe = tmp_path / "driver"
    r = subprocess.run(["g++", "-o", str(exe), str(tmp_path / "driver.o"), str(tmp_path / "binding.o"),
                        f"-L{lib.parent}", "-lpico_gpu", f"-Wl,-rpath,{lib.parent}", "-Wl,--no-undefined", "-pthread"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    cam, cfg, status = r.stdout.strip().splitlines()
    assert cam.split() == ["1", "2", "3", "0", "0", "1", "0", "1", "0", "3", "2", "1.5", "0.25", "50", "40"]
    assert cfg.split() == ["5", "16", "0.5", "2", "3", "1", "0", "1", "99"]
    assert int(status) == -1   # PICO_ERR_INVALID_ARG
