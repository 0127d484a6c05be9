// Placeholder definitions for the entry points whose kernels are not built yet.
#include "capi_internal.h"

extern "C" {

int pico_gpu_render(pico_gpu_ctx* ctx, const pico_gpu_scene*, const pico_camera*, const pico_render_config*,
                    float*, uint32_t*, float*, const volatile int32_t*)
{
    return pico::set_error(ctx, PICO_ERR_UNSUPPORTED, "render not built");
}
int pico_gpu_denoiser_inputs(pico_gpu_ctx* ctx, const pico_gpu_scene*, const pico_camera*, float*, float*, float*)
{
    return pico::set_error(ctx, PICO_ERR_UNSUPPORTED, "denoiser inputs not built");
}
int pico_gpu_atrous(pico_gpu_ctx* ctx, const float*, const float*, const float*, const float*, uint32_t, uint32_t,
                    float*)
{
    return pico::set_error(ctx, PICO_ERR_UNSUPPORTED, "atrous not built");
}
int pico_gpu_atrous_device(pico_gpu_ctx* ctx, const float*, const float*, const float*, const float*, uint32_t,
                           uint32_t, float*, void*)
{
    return pico::set_error(ctx, PICO_ERR_UNSUPPORTED, "atrous not built");
}

}  // extern "C"
