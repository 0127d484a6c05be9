// The reference-side binding of libpico_gpu: the code Pico's Scene runs in place of
// its tiled CPU integrator.  It is compiled inside the Pico tree, against Pico's own
// headers (Core/Scene.hpp, Core/Camera.hpp) and include/pico_gpu.h; a Scene that
// holds a SceneGpu member forwards Scene::render_scene_to_memory (Core/Scene.hpp:68,
// Core/Scene.cpp:143-235) to render_scene_to_memory below.  Converting the
// reference's own RenderParams and Camera here, in compiled code, is what makes a
// change on either side of the boundary (a renamed field, a changed signature or
// struct layout) a build error instead of a silent mismatch.
#pragma once

#include "Core/Scene.hpp"
#include "pico_gpu.h"

#include <cstdint>
#include <vector>

namespace pico_binding {

// What a Scene hands the library, in its insertion order (the reference's JSON loader
// adds instances from pool tasks in no fixed order, Core/Scene.cpp:66-80, so the
// order these vectors hold is the host's choice), and the uploaded scene.
struct SceneGpu {
    pico_gpu_ctx* ctx = nullptr;
    pico_gpu_scene* scene = nullptr;
    std::vector<pico_mesh> meshes;           // arrays kept alive by the Scene
    std::vector<pico_instance> instances;
    std::vector<pico_material> materials;
    bool has_sky = false;
    pico_sky sky{};
    uint32_t estimator = PICO_ESTIMATOR_REFERENCE;

    SceneGpu() = default;
    SceneGpu(const SceneGpu&) = delete;
    SceneGpu& operator=(const SceneGpu&) = delete;
    ~SceneGpu();
};

// Opens the context on `device`; returns a pico_status.
int open(SceneGpu& gpu, int device);

// The library's camera for a reference Camera rendering params' image size (the
// reference Camera has no resolution getter: the RenderParams size is the image's).
pico_camera to_pico_camera(const Scene::Camera& camera, const Scene::RenderParams& params);

// The library's render settings for the reference's RenderParams.
pico_render_config to_render_config(const Scene::RenderParams& params, uint32_t estimator, uint64_t seed);

// Scene::render_scene_to_memory on the GPU: uploads the scene on first use, then
// advances params' progressive buffers (mean, sample count, variance per pixel) in
// place, as the reference's loop does; *should_quit is honoured between sample
// batches.  Returns the library's status (PICO_ERR_CANCELLED after a cancel).
int render_scene_to_memory(SceneGpu& gpu, const Scene::Camera& camera, const Scene::RenderParams& params,
                           const bool* should_quit);

}  // namespace pico_binding
