// Batch evaluation of the device BSRDF routines (BSRDF::pdf / sample,
// Render/BSRDF.hpp:50-52, and direct_lighting_pdf, Render/Integrators.cpp:13-22)
// on caller-supplied inputs, so the shading code the integrator runs can be
// checked against the reference value by value.
#include "capi_internal.h"
#include "shade.cuh"

namespace pico {

__global__ void bsdf_eval_kernel(uint64_t n, const uint32_t* kinds, const GpuMaterial* mats, const float* V,
                                 const float* N, const float* H, const float* xi, float* pdf, float* L, float* P,
                                 float* energy, float* dl_pdf)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t kind = kinds[i];
    const GpuMaterial m = mats[i];
    const ex::V3 v = ex::v3(V[3 * i], V[3 * i + 1], V[3 * i + 2]);
    const ex::V3 nn = ex::v3(N[3 * i], N[3 * i + 1], N[3 * i + 2]);
    const ex::V3 h = ex::v3(H[3 * i], H[3 * i + 1], H[3 * i + 2]);
    pdf[i] = bsdf_pdf(kind, v, h, m.roughness, m.reflectance);
    int used = 0;
    auto next_xi = [&](float& a, float& b) {
        a = xi[4 * i + 2 * used];
        b = xi[4 * i + 2 * used + 1];
        ++used;
    };
    IorStack ior;   // a camera path's stack: {1.0}
    ior.n = 0;
    ior.push(1.0f);
    const BsdfSample s = sample_bsdf(kind, m, v, nn, next_xi, ior);
    L[3 * i] = s.L.x; L[3 * i + 1] = s.L.y; L[3 * i + 2] = s.L.z;
    P[i] = s.P;
    energy[3 * i] = s.energy.x; energy[3 * i + 1] = s.energy.y; energy[3 * i + 2] = s.energy.z;
    dl_pdf[i] = direct_lighting_pdf(kind, m, nn, v, s.L);
}

}  // namespace pico

using namespace pico;

extern "C" int pico_gpu_bsdf_eval(pico_gpu_ctx* ctx, uint64_t n, const uint32_t* kinds, const pico_material* mats,
                                  const float* V, const float* N, const float* H, const float* xi, float* pdf,
                                  float* L, float* P, float* energy, float* direct_pdf)
{
    if (!ctx || (n && (!kinds || !mats || !V || !N || !H || !xi || !pdf || !L || !P || !energy || !direct_pdf)))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (n == 0) return PICO_OK;
    cudaSetDevice(ctx->device);
    std::vector<GpuMaterial> gm(n);
    for (uint64_t i = 0; i < n; ++i) {
        const pico_material& m = mats[i];
        GpuMaterial g{};
        for (int a = 0; a < 3; ++a) {
            g.diffuse[a] = m.diffuse[a]; g.specular[a] = m.specular[a]; g.emissive[a] = m.emissive[a];
        }
        g.roughness = m.roughness;
        g.ior = m.index_of_refraction;
        const float s = std::sqrt((m.specular[0] * m.specular[0] + m.specular[1] * m.specular[1]) +
                                  m.specular[2] * m.specular[2]);
        const float d = std::sqrt((m.diffuse[0] * m.diffuse[0] + m.diffuse[1] * m.diffuse[1]) +
                                  m.diffuse[2] * m.diffuse[2]);
        g.reflectance = s / (s + d);
        gm[i] = g;
    }
    // one device block: [kinds | mats | V | N | H | xi | pdf | L | P | energy | dl]
    const size_t f = sizeof(float);
    const size_t sizes[] = {n * 4, n * sizeof(GpuMaterial), n * 3 * f, n * 3 * f, n * 3 * f, n * 4 * f,
                            n * f, n * 3 * f, n * f, n * 3 * f, n * f};
    size_t off[12] = {0};
    for (int k = 0; k < 11; ++k) off[k + 1] = off[k] + ((sizes[k] + 255) & ~size_t(255));
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, off[11]);
    if (e != cudaSuccess) return cuda_error(ctx, e, "bsdf eval buffers");
    char* b = static_cast<char*>(base);
    const void* src[] = {kinds, gm.data(), V, N, H, xi};
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) e = cudaMemcpy(b + off[k], src[k], sizes[k], cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        bsdf_eval_kernel<<<(unsigned)((n + 127) / 128), 128>>>(
            n, reinterpret_cast<uint32_t*>(b + off[0]), reinterpret_cast<GpuMaterial*>(b + off[1]),
            reinterpret_cast<float*>(b + off[2]), reinterpret_cast<float*>(b + off[3]),
            reinterpret_cast<float*>(b + off[4]), reinterpret_cast<float*>(b + off[5]),
            reinterpret_cast<float*>(b + off[6]), reinterpret_cast<float*>(b + off[7]),
            reinterpret_cast<float*>(b + off[8]), reinterpret_cast<float*>(b + off[9]),
            reinterpret_cast<float*>(b + off[10]));
        e = cudaGetLastError();
    }
    void* dst[] = {pdf, L, P, energy, direct_pdf};
    for (int k = 0; k < 5 && e == cudaSuccess; ++k) e = cudaMemcpy(dst[k], b + off[6 + k], sizes[6 + k], cudaMemcpyDeviceToHost);
    cudaFree(base);
    if (e != cudaSuccess) return cuda_error(ctx, e, "bsdf eval");
    return PICO_OK;
}
