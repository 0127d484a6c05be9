// Batch evaluation of the device BSRDF routines (BSRDF::pdf / sample,
// Render/BSRDF.hpp:50-52, and direct_lighting_pdf, Render/Integrators.cpp:13-22)
// on caller-supplied inputs, so the shading code the integrator runs can be
// checked against the reference value by value.
#include "capi_internal.h"
#include "physical.cuh"
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

// The physical estimator's BSDF on caller-supplied inputs, through the same
// device routines the physical shade kernel runs: f and pdf of (V, L) and one
// sample from three uniforms.
__global__ void phys_bsdf_kernel(uint64_t n, const uint32_t* kinds, const GpuMaterial* mats, const float* V,
                                 const float* N, const float* L, const float* u, float* f, float* pdf, float* sl,
                                 float* spdf, float* sw, uint32_t* sok)
{
    using namespace phys;
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Lobes lb = lobes_of(kinds[i], mats[i]);
    const Frame fr = frame_of(make_float3(N[3 * i], N[3 * i + 1], N[3 * i + 2]));
    const float3 vl = to_local(fr, make_float3(V[3 * i], V[3 * i + 1], V[3 * i + 2]));
    float3 fv;
    eval(lb, vl, to_local(fr, make_float3(L[3 * i], L[3 * i + 1], L[3 * i + 2])), fv, pdf[i]);
    f[3 * i] = fv.x; f[3 * i + 1] = fv.y; f[3 * i + 2] = fv.z;
    const Sample s = phys::sample(lb, vl, u[3 * i], u[3 * i + 1], u[3 * i + 2]);
    const float3 w = to_world(fr, s.l);
    sl[3 * i] = w.x; sl[3 * i + 1] = w.y; sl[3 * i + 2] = w.z;
    spdf[i] = s.pdf;
    sw[3 * i] = s.weight.x; sw[3 * i + 1] = s.weight.y; sw[3 * i + 2] = s.weight.z;
    sok[i] = s.ok ? 1u : 0u;
}

}  // namespace pico

using namespace pico;

extern "C" int pico_gpu_phys_bsdf_eval(pico_gpu_ctx* ctx, uint64_t n, const uint32_t* kinds,
                                       const pico_material* mats, const float* V, const float* N, const float* L,
                                       const float* u, float* f, float* pdf, float* sample_L, float* sample_pdf,
                                       float* sample_weight, uint32_t* sample_ok)
{
    if (!ctx || (n && (!kinds || !mats || !V || !N || !L || !u || !f || !pdf || !sample_L || !sample_pdf ||
                       !sample_weight || !sample_ok)))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (n == 0) return PICO_OK;
    for (uint64_t i = 0; i < n; ++i)
        if (kinds[i] != PICO_BSDF_DIFFUSE && kinds[i] != PICO_BSDF_SPECULAR && kinds[i] != PICO_BSDF_DIELECTRIC)
            return set_error(ctx, PICO_ERR_INVALID_ARG, "the physical BSDF covers Diffuse, Specular and Dielectric");
    const DeviceScope device_scope(ctx->device);
    std::vector<GpuMaterial> gm(n);
    for (uint64_t i = 0; i < n; ++i) {
        GpuMaterial g{};
        for (int a = 0; a < 3; ++a) {
            g.diffuse[a] = mats[i].diffuse[a]; g.specular[a] = mats[i].specular[a];
        }
        g.roughness = mats[i].roughness;
        gm[i] = g;
    }
    // one device block: [kinds | mats | V | N | L | u | f | pdf | sL | spdf | sw | sok]
    const size_t fl = sizeof(float);
    const size_t sizes[] = {n * 4, n * sizeof(GpuMaterial), n * 3 * fl, n * 3 * fl, n * 3 * fl, n * 3 * fl,
                            n * 3 * fl, n * fl, n * 3 * fl, n * fl, n * 3 * fl, n * 4};
    size_t off[13] = {0};
    for (int k = 0; k < 12; ++k) off[k + 1] = off[k] + ((sizes[k] + 255) & ~size_t(255));
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, off[12]);
    if (e != cudaSuccess) return cuda_error(ctx, e, "bsdf eval buffers");
    char* b = static_cast<char*>(base);
    const void* src[] = {kinds, gm.data(), V, N, L, u};
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) e = cudaMemcpy(b + off[k], src[k], sizes[k], cudaMemcpyHostToDevice);
    auto F = [&](int k) { return reinterpret_cast<float*>(b + off[k]); };
    if (e == cudaSuccess) {
        phys_bsdf_kernel<<<(unsigned)((n + 127) / 128), 128>>>(
            n, reinterpret_cast<uint32_t*>(b + off[0]), reinterpret_cast<GpuMaterial*>(b + off[1]), F(2), F(3),
            F(4), F(5), F(6), F(7), F(8), F(9), F(10), reinterpret_cast<uint32_t*>(b + off[11]));
        e = cudaGetLastError();
    }
    void* dst[] = {f, pdf, sample_L, sample_pdf, sample_weight, sample_ok};
    for (int k = 0; k < 6 && e == cudaSuccess; ++k) e = cudaMemcpy(dst[k], b + off[6 + k], sizes[6 + k], cudaMemcpyDeviceToHost);
    cudaFree(base);
    if (e != cudaSuccess) return cuda_error(ctx, e, "physical bsdf eval");
    return PICO_OK;
}

extern "C" int pico_gpu_bsdf_eval(pico_gpu_ctx* ctx, uint64_t n, const uint32_t* kinds, const pico_material* mats,
                                  const float* V, const float* N, const float* H, const float* xi, float* pdf,
                                  float* L, float* P, float* energy, float* direct_pdf)
{
    if (!ctx || (n && (!kinds || !mats || !V || !N || !H || !xi || !pdf || !L || !P || !energy || !direct_pdf)))
        return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    if (n == 0) return PICO_OK;
    const DeviceScope device_scope(ctx->device);
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
