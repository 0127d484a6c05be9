// See pico_scene_binding.hpp.
#include "pico_scene_binding.hpp"

#include <atomic>
#include <chrono>
#include <cstring>
#include <random>
#include <thread>

namespace pico_binding {

// The progressive buffers are handed over as flat float arrays.
static_assert(sizeof(glm::vec3) == 3 * sizeof(float), "RenderParams pixels must be packed float triples");

SceneGpu::~SceneGpu()
{
    if (scene) pico_gpu_scene_free(scene);
    if (ctx) pico_gpu_shutdown(ctx);
}

int open(SceneGpu& gpu, int device)
{
    return gpu.ctx ? PICO_OK : pico_gpu_init(device, &gpu.ctx);
}

pico_camera to_pico_camera(const Scene::Camera& camera, const Scene::RenderParams& params)
{
    pico_camera c{};
    std::memcpy(c.position, &camera.getPosition()[0], sizeof c.position);
    std::memcpy(c.direction, &camera.getDirection()[0], sizeof c.direction);
    const glm::vec3 up = camera.getUp();
    std::memcpy(c.up, &up[0], sizeof c.up);
    c.resolution[0] = params.m_Width;
    c.resolution[1] = params.m_Height;
    c.aspect = camera.getAspect();
    c.near_plane = camera.getNearPlane();
    c.far_plane = camera.getFarPlane();
    c.fov = camera.getFOV();
    return c;
}

pico_render_config to_render_config(const Scene::RenderParams& params, uint32_t estimator, uint64_t seed)
{
    pico_render_config cfg{};
    cfg.max_ray_depth = params.m_maxRayDepth;
    cfg.max_samples = params.m_maxSamples;
    cfg.max_variance = params.m_maxVariance;
    cfg.height = params.m_Height;
    cfg.width = params.m_Width;
    cfg.tonemap = params.m_tonemap ? 1 : 0;
    cfg.denoise = params.m_denoise ? 1 : 0;
    cfg.estimator = estimator;
    cfg.seed = seed;
    return cfg;
}

int render_scene_to_memory(SceneGpu& gpu, const Scene::Camera& camera, const Scene::RenderParams& params,
                           const bool* should_quit)
{
    if (!gpu.ctx) return PICO_ERR_INVALID_ARG;
    if (!gpu.scene) {
        pico_scene_desc d{};
        d.meshes = gpu.meshes.data();
        d.nmeshes = (uint32_t)gpu.meshes.size();
        d.instances = gpu.instances.data();
        d.ninstances = (uint32_t)gpu.instances.size();
        d.materials = gpu.materials.data();
        d.nmaterials = (uint32_t)gpu.materials.size();
        d.sky = gpu.has_sky ? &gpu.sky : nullptr;   // else the black sky (Core/Scene.cpp:683-690)
        const int st = pico_gpu_scene_upload(gpu.ctx, &d, &gpu.scene);
        if (st != PICO_OK) return st;
    }
    const pico_camera cam = to_pico_camera(camera, params);
    // the reference seeds each render from std::random_device (Core/Scene.cpp:203-204)
    const uint64_t seed = ((uint64_t)std::random_device{}() << 32) | std::random_device{}();
    const pico_render_config cfg = to_render_config(params, gpu.estimator, seed);
    // The library polls an int32 flag between sample batches; the reference's flag is a
    // bool the caller's thread writes, watched here until the render returns.
    volatile int32_t quit = 0;
    std::atomic<bool> done{false};
    std::thread watcher;
    if (should_quit) {
        watcher = std::thread([&] {
            while (!done.load(std::memory_order_relaxed)) {
                if (*static_cast<const volatile bool*>(should_quit)) {
                    quit = 1;
                    break;
                }
                std::this_thread::sleep_for(std::chrono::milliseconds(1));
            }
        });
    }
    const int st = pico_gpu_render(gpu.ctx, gpu.scene, &cam, &cfg, &params.m_Pixels[0].x, params.m_SampleCount,
                                   &params.m_variance[0].x, should_quit ? &quit : nullptr);
    done.store(true, std::memory_order_relaxed);
    if (watcher.joinable()) watcher.join();
    return st;
}

}  // namespace pico_binding
