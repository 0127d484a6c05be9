// Device building blocks of the neural radiance cache: tcgen05 / TMEM / mbarrier /
// bulk-copy wrappers (inline PTX for sm_103a) and the input encoding.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "nrc_layout.h"

namespace pico {
namespace nrc {

// A query record: 16 floats.  pad carries a payload (the path index in renders).
struct Query {
    float px, py, pz, dx, dy, dz, nx, ny, nz, rough, ax, ay, az;
    uint32_t pad;
};

__device__ __forceinline__ Query load_query(const float4* q)
{
    const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
    Query r;
    r.px = a.x; r.py = a.y; r.pz = a.z; r.dx = a.w;
    r.dy = b.x; r.dz = b.y; r.nx = b.z; r.ny = b.w;
    r.nz = c.x; r.rough = c.y; r.ax = c.z; r.ay = c.w;
    r.az = d.x; r.pad = __float_as_uint(d.y);
    return r;
}

__device__ __forceinline__ uint32_t grid_index(const GridGeometry& g, int l, uint32_t x, uint32_t y, uint32_t z)
{
    const uint32_t r = g.res1[l];
    if (r) return x + r * (y + r * z);
    return (x ^ (y * 2654435761u) ^ (z * 805459861u)) & g.table_mask;
}

// Cell and fractional position of a normalised point on level l.
__device__ __forceinline__ void grid_cell(const GridGeometry& g, int l, const float u[3], uint32_t c[3], float f[3])
{
    for (int a = 0; a < 3; ++a) {
        const float x = u[a] * g.scale[l];
        const float fl = floorf(x);
        c[a] = (uint32_t)fl;
        f[a] = x - fl;
    }
}

__device__ __forceinline__ void normalise_position(const GridGeometry& g, const Query& q, float u[3])
{
    u[0] = fminf(fmaxf((q.px - g.lo[0]) * g.inv_extent[0], 0.0f), 1.0f);
    u[1] = fminf(fmaxf((q.py - g.lo[1]) * g.inv_extent[1], 0.0f), 1.0f);
    u[2] = fminf(fmaxf((q.pz - g.lo[2]) * g.inv_extent[2], 0.0f), 1.0f);
}

// Real spherical harmonics of degrees 0-3 (16 values) of a unit direction, in the
// order (l, m) = (0,0), (1,-1), (1,0), (1,1), (2,-2) ... (3,3); the constants are the
// normalisations sqrt((2l+1)/(4 pi) (l-|m|)!/(l+|m|)!) (times sqrt(2) for m != 0)
// folded with the Legendre polynomial coefficients.
__device__ __forceinline__ void sh16(float x, float y, float z, float* o)
{
    const float xx = x * x, yy = y * y, zz = z * z;
    o[0] = 0.28209479177387814f;
    o[1] = -0.48860251190291987f * y;
    o[2] = 0.48860251190291987f * z;
    o[3] = -0.48860251190291987f * x;
    o[4] = 1.0925484305920792f * x * y;
    o[5] = -1.0925484305920792f * y * z;
    o[6] = 0.31539156525252005f * (3.0f * zz - 1.0f);
    o[7] = -1.0925484305920792f * x * z;
    o[8] = 0.54627421529603959f * (xx - yy);
    o[9] = -0.59004358992664352f * y * (3.0f * xx - yy);
    o[10] = 2.8906114426405538f * x * y * z;
    o[11] = -0.45704579946446572f * y * (5.0f * zz - 1.0f);
    o[12] = 0.3731763325901154f * z * (5.0f * zz - 3.0f);
    o[13] = -0.45704579946446572f * x * (5.0f * zz - 1.0f);
    o[14] = 1.4453057213202769f * z * (xx - yy);
    o[15] = -0.59004358992664352f * x * (xx - 3.0f * yy);
}

// The 64 network inputs of a query: 16 levels x 2 trilinearly interpolated
// hash-grid features, 16 SH values of the direction, normal, roughness,
// albedo, a constant 1 (the first layer's bias) and zero padding.
__device__ __forceinline__ void encode(const GridGeometry& g, const __half2* __restrict__ table, const Query& q,
                                       float* in)
{
    float u[3];
    normalise_position(g, q, u);
#pragma unroll
    for (int l = 0; l < kLevels; ++l) {
        uint32_t c[3];
        float f[3];
        grid_cell(g, l, u, c, f);
        const __half2* lv = table + ((size_t)l << g.log2_table);
        float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
            const float w = (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) * (dz ? f[2] : 1.0f - f[2]);
            const float2 v = __half22float2(lv[grid_index(g, l, c[0] + dx, c[1] + dy, c[2] + dz)]);
            a0 += w * v.x;
            a1 += w * v.y;
        }
        in[kInputHash + 2 * l] = a0;
        in[kInputHash + 2 * l + 1] = a1;
    }
    sh16(q.dx, q.dy, q.dz, in + kInputSH);
    in[kInputNormal] = q.nx; in[kInputNormal + 1] = q.ny; in[kInputNormal + 2] = q.nz;
    in[kInputRough] = q.rough;
    in[kInputAlbedo] = q.ax; in[kInputAlbedo + 1] = q.ay; in[kInputAlbedo + 2] = q.az;
    in[kInputBias] = 1.0f;
#pragma unroll
    for (int k = kInputBias + 1; k < kWidth; ++k) in[k] = 0.0f;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Writes 64 floats as one bf16 row of a swizzled tile (relu: negative values to 0).
template <bool kRelu>
__device__ __forceinline__ void store_row(uint8_t* tile, uint32_t row, const float* v)
{
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        float x[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = kRelu ? fmaxf(v[8 * c + k], 0.0f) : v[8 * c + k];
        uint4 w;
        w.x = pack_bf16(x[0], x[1]); w.y = pack_bf16(x[2], x[3]);
        w.z = pack_bf16(x[4], x[5]); w.w = pack_bf16(x[6], x[7]);
        *reinterpret_cast<uint4*>(tile + swz(row, c)) = w;
    }
}

// ---------------------------------------------------------------- PTX wrappers
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t globaltimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared-memory matrix descriptor: 128-byte swizzle (layout type 2), descriptor
// version 1, leading and stride byte offsets 1024.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(1024u >> 4) << 16) | ((uint64_t)(1024u >> 4) << 32) |
           (1ull << 46) | (2ull << 61);
}

// Instruction descriptor of kind::f16 with bf16 A and B, f32 accumulator:
// D format bits 4-5, A / B format bits 7-9 / 10-12, A / B major (1 = MN) bits 15 / 16,
// N >> 3 bits 17-22, M >> 4 bits 24-28.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t M, uint32_t N, bool a_mn, bool b_mn)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) | ((b_mn ? 1u : 0u) << 16) |
           ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(da), "l"(db), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive 32-bit columns of the warp's 32 TMEM lanes (one lane per thread),
// waited for inside the same statement so the registers are valid afterwards.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity to complete, for at most limit_ns
// nanoseconds of the global timer; false if it did not.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// One-dimensional bulk copy global -> shared, completing `bytes` on the barrier.
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

}  // namespace nrc
}  // namespace pico
