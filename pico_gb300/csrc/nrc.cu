// Neural radiance cache kernels (no counterpart in the reference): the input
// encoding, the fused network forward pass, the fused training step and the
// Adam optimiser, for sm_103a.
//
// The network: 64 inputs (nrc_device.cuh: encode) -> 5 hidden layers of 64
// ReLU units -> 3 linear outputs, no biases (the constant input gives the first
// layer one).  Weights and activations are bf16, products accumulate in fp32.
//
// Both network kernels work on tiles of 128 queries, one per thread of a
// warpgroup (4 warps), which is also one TMEM lane: the thread encodes its
// query into row `tid` of a swizzled shared-memory tile, the group's first
// thread issues the layer's tcgen05.mma (M = 128, N = 64 or 16, K = 64 as four
// K = 16 steps) with the accumulator in TMEM and commits it to an mbarrier, and
// every thread reads its row back with tcgen05.ld, applies ReLU and writes the
// next layer's input tile.  Inference CTAs hold 1, 2 or 4 such groups on their
// own tiles and TMEM columns; training CTAs hold one.  The weights (43 KB,
// bf16, already in the swizzled layout) reach shared memory once per CTA with
// one bulk copy.
//
// Training keeps the six layer inputs of a tile in shared memory.  The loss is
// relative L2, sum_c (y_c - t_c)^2 / (y_c^2 + 0.01) with the denominator held
// constant (Mueller et al. 2021), averaged over the batch and the three
// channels.  Backwards per layer l, with dY the gradient at the layer output:
//   dX = dY W_l      M = 128 rows, N = 64 inputs, K = outputs; W_l read MN-major
//   dW_l += dY^T X_l M = outputs (padded to 128), N = 64, K = 128 rows; both MN-major
// and the next dY is dX masked by X_l > 0.  dW_l accumulates in TMEM over all
// tiles of a CTA (6 x 64 columns) and is written once as a per-CTA partial,
// summed by the optimiser kernel in a fixed order, so the weight gradient is
// deterministic.  The first layer's input gradient flows into the hash grid:
// each of the 32 grid features scatters weight * gradient to its 8 corners
// with float2 atomics.
#include "kernels.h"
#include "nrc.h"
#include "nrc_device.cuh"

namespace pico {
namespace nrc {

namespace {

constexpr int kThreads = 128;
// Inference CTAs hold G warpgroups (128-row tiles in flight), G = 1, 2 or 4.
constexpr uint32_t infer_smem(int G) { return kWeightRegion + (uint32_t)G * kTileBytes + 64 + 1024; }
constexpr uint32_t infer_tmem_cols(int G) { return 64u * (uint32_t)G; }   // a power of two for G = 1, 2, 4
constexpr uint32_t kTrainSmem = kWeightRegion + 6 * kTileBytes + kTileBytes + kGuardBytes + 64 + 1024;
constexpr uint32_t kTrainTmemCols = 512;   // accumulator 0-63, dW_l at 64 + 64 l

__device__ __forceinline__ uint8_t* align1024(uint8_t* p)
{
    return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

__device__ __forceinline__ void set_error(int* err, int bit)
{
    if (err) atomicOr(err, bit);
}

constexpr int kErrTimeout = 1;

// Issues the MMAs of forward layer l: acc[0, N) = X_l * W_l^T.
__device__ __forceinline__ void issue_forward(uint32_t tmem, uint32_t x_addr, uint32_t w_addr, int l)
{
    const uint32_t id = idesc_bf16(128, l < kHidden ? 64 : kOutRows, false, false);
#pragma unroll
    for (uint32_t k = 0; k < 4; ++k) mma_bf16(tmem, sdesc(x_addr + 32 * k), sdesc(w_addr + 32 * k), id, k > 0);
}

}  // namespace

// ------------------------------------------------------------------ encoding
__global__ void __launch_bounds__(256) encode_kernel(GridGeometry g, const __half2* __restrict__ table,
                                                     const float4* __restrict__ queries, uint32_t n, float* out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const Query q = load_query(queries + 4 * (size_t)i);
        float in[kWidth];
        encode(g, table, q, in);
        float4* o = reinterpret_cast<float4*>(out + (size_t)kWidth * i);
#pragma unroll
        for (int k = 0; k < kWidth / 4; ++k) o[k] = make_float4(in[4 * k], in[4 * k + 1], in[4 * k + 2], in[4 * k + 3]);
    }
}

// ------------------------------------------------------------------ inference
struct InferArgs {
    GridGeometry g;
    const __half2* table;
    const uint8_t* weights;
    const float4* queries;
    uint32_t n;
    float* out_rgb;
    const float4* thr;
    float4* pay;
    int* err;
    const uint32_t* n_dev;
    WaitPolicy wait;
};

// G warpgroups per CTA share one copy of the weights; each runs its own 128-row
// tiles with its own shared-memory tile, TMEM columns (64 g .. 64 g + 63) and
// mbarrier, and synchronises on its own named barrier (1 + g), so that one
// group's encoding (hash-grid gathers) overlaps another's tensor-core layers.
template <int kId>
__device__ __forceinline__ bool bar_and(bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, %2, 128, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "n"(kId)
        : "memory");
    return r != 0;
}

// AND of v over warpgroup g's 128 threads on named barrier 1 + g; the barrier
// numbers are immediates, so a CTA reserves only the barriers it uses.
__device__ __forceinline__ bool group_sync_and(uint32_t g, bool v)
{
    switch (g) {
    case 0: return bar_and<1>(v);
    case 1: return bar_and<2>(v);
    case 2: return bar_and<3>(v);
    default: return bar_and<4>(v);
    }
}

template <int G>
__global__ void __launch_bounds__(128 * G) infer_kernel(InferArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = align1024(smem_raw);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, gtid = tid & 127u;
    uint8_t* W = sm;
    uint8_t* X = sm + kWeightRegion + g * kTileBytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sm + kWeightRegion + G * kTileBytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1 + G);
    const uint32_t bar_w = smem_addr(bars), bar_m = smem_addr(bars + 1 + g);
    if (tid == 0) {
        mbar_init(bar_w, 1);
        for (int k = 0; k < G; ++k) mbar_init(smem_addr(bars + 1 + k), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(smem_addr(tslot), infer_tmem_cols(G));
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot + 64u * g;
    if (tid == 0) {
        mbar_expect_tx(bar_w, kWeightBytes + a.wait.withheld_bytes);
        bulk_load(smem_addr(W), a.weights, kWeightBytes, bar_w);
    }
    bool ok = mbar_wait(bar_w, 0, a.wait.limit_ns);
    uint32_t phase = 0;
    const uint32_t lane_addr = tmem + (((warp & 3u) * 32u) << 16);
    const uint32_t x_addr = smem_addr(X), w_addr = smem_addr(W);
    const uint32_t n = a.n_dev ? min(*a.n_dev, a.n) : a.n;
    const uint32_t ntiles = (n + kRows - 1) / kRows;
    for (uint32_t t = blockIdx.x * G + g; t < ntiles; t += gridDim.x * G) {
        const uint32_t row = t * kRows + gtid;
        const bool valid = row < n;
        uint32_t payload = 0;
        {
            float in[kWidth];
            if (valid) {
                const Query q = load_query(a.queries + 4 * (size_t)row);
                payload = q.pad;
                encode(a.g, a.table, q, in);
            } else {
#pragma unroll
                for (int k = 0; k < kWidth; ++k) in[k] = 0.0f;
            }
            store_row<false>(X, gtid, in);
        }
        bool abort = false;
#pragma unroll 1
        for (int l = 0; l < kLayers; ++l) {
            fence_async_smem();
            tc_fence_before();
            if (!group_sync_and(g, ok)) { abort = true; break; }
            if (gtid == 0) {
                tc_fence_after();
                issue_forward(tmem, x_addr, w_addr + (uint32_t)l * kLayerBytes, l);
                mma_commit(bar_m);
            }
            ok = mbar_wait(bar_m, phase, a.wait.limit_ns);
            phase ^= 1u;
            tc_fence_after();
            if (l < kHidden) {
                float v[kWidth];
#pragma unroll
                for (int c = 0; c < 4; ++c) tmem_ld16(lane_addr + 16 * c, v + 16 * c);
                store_row<true>(X, gtid, v);
            } else {
                float v[16];
                tmem_ld16(lane_addr, v);
                if (valid && ok) {
                    if (a.pay) {
                        const float4 th = a.thr[payload];
                        float4 p = a.pay[payload];
                        p.x += th.x * fmaxf(v[0], 0.0f);
                        p.y += th.y * fmaxf(v[1], 0.0f);
                        p.z += th.z * fmaxf(v[2], 0.0f);
                        a.pay[payload] = p;
                    } else {
                        float* o = a.out_rgb + 3 * (size_t)row;
                        o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
                    }
                }
            }
        }
        if (abort) break;
    }
    if (!ok && gtid == 0) set_error(a.err, kErrTimeout);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(*tslot, infer_tmem_cols(G));
}

// ------------------------------------------------------------------ training
struct TrainArgs {
    GridGeometry g;
    const __half2* table;
    const uint8_t* weights;
    TrainBatch b;
    float loss_scale;      // 1 / (3 n)
    float2* grid_grad;
    float* partial;        // [gridDim.x][kMlpParams]
    float* loss;
    int* err;
    WaitPolicy wait;
};

__global__ void __launch_bounds__(kThreads, 1) train_kernel(TrainArgs a)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* sm = align1024(smem_raw);
    uint8_t* W = sm;
    uint8_t* X = sm + kWeightRegion;           // layer inputs X_0 .. X_5
    uint8_t* dY = X + 6 * kTileBytes;          // gradient at the current layer's output
    uint64_t* bars = reinterpret_cast<uint64_t*>(dY + kTileBytes + kGuardBytes);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t bar_w = smem_addr(bars), bar_m = smem_addr(bars + 1);
    if (tid == 0) {
        mbar_init(bar_w, 1);
        mbar_init(bar_m, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        tmem_alloc(smem_addr(tslot), kTrainTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;
    if (tid == 0) {
        mbar_expect_tx(bar_w, kWeightBytes);
        bulk_load(smem_addr(W), a.weights, kWeightBytes, bar_w);
    }
    bool ok = mbar_wait(bar_w, 0, a.wait.limit_ns);
    uint32_t phase = 0;
    const uint32_t lane_addr = tmem + ((warp * 32u) << 16);
    const uint32_t w_addr = smem_addr(W), x_addr = smem_addr(X), dy_addr = smem_addr(dY);
    const uint32_t ntiles = (a.b.n + kRows - 1) / kRows;
    bool first = true;
    float loss_sum = 0.0f;
    bool abort = false;
    for (uint32_t t = blockIdx.x; t < ntiles && !abort; t += gridDim.x) {
        const uint32_t row = t * kRows + tid;
        bool valid = row < a.b.n;
        float u[3] = {0.0f, 0.0f, 0.0f};
        float target[3] = {0.0f, 0.0f, 0.0f};
        {
            float in[kWidth];
            if (valid) {
                const size_t rec = a.b.offset + (size_t)row * a.b.stride;
                const Query q = load_query(a.b.queries + 4 * rec);
                const float4 tg = __ldg(a.b.targets + rec);
                target[0] = tg.x; target[1] = tg.y; target[2] = tg.z;
                valid = isfinite(tg.x) && isfinite(tg.y) && isfinite(tg.z);
                normalise_position(a.g, q, u);
                encode(a.g, a.table, q, in);
            } else {
#pragma unroll
                for (int k = 0; k < kWidth; ++k) in[k] = 0.0f;
            }
            store_row<false>(X, tid, in);
        }
        // forward
#pragma unroll 1
        for (int l = 0; l < kLayers; ++l) {
            fence_async_smem();
            tc_fence_before();
            if (!__syncthreads_and(ok)) { abort = true; break; }
            if (tid == 0) {
                tc_fence_after();
                issue_forward(tmem, x_addr + (uint32_t)l * kTileBytes, w_addr + (uint32_t)l * kLayerBytes, l);
                mma_commit(bar_m);
            }
            ok = mbar_wait(bar_m, phase, a.wait.limit_ns);
            phase ^= 1u;
            tc_fence_after();
            if (l < kHidden) {
                float v[kWidth];
#pragma unroll
                for (int c = 0; c < 4; ++c) tmem_ld16(lane_addr + 16 * c, v + 16 * c);
                store_row<true>(X + (l + 1) * kTileBytes, tid, v);
            } else {
                float v[16];
                tmem_ld16(lane_addr, v);
                float d[kWidth];
#pragma unroll
                for (int k = 0; k < kWidth; ++k) d[k] = 0.0f;
                if (valid) {
#pragma unroll
                    for (int c = 0; c < kOutputs; ++c) {
                        const float y = v[c], den = y * y + 0.01f, diff = y - target[c];
                        loss_sum += diff * diff / den * a.loss_scale;
                        d[c] = 2.0f * diff / den * a.loss_scale;
                    }
                }
                store_row<false>(dY, tid, d);
            }
        }
        if (abort) break;
        // backward
#pragma unroll 1
        for (int l = kLayers - 1; l >= 0; --l) {
            fence_async_smem();
            tc_fence_before();
            if (!__syncthreads_and(ok)) { abort = true; break; }
            if (tid == 0) {
                tc_fence_after();
                const uint32_t wl = w_addr + (uint32_t)l * kLayerBytes, xl = x_addr + (uint32_t)l * kTileBytes;
                const uint32_t kout = l < kHidden ? 4u : 1u;   // K = the layer's outputs, in steps of 16
                for (uint32_t k = 0; k < kout; ++k)
                    mma_bf16(tmem, sdesc(dy_addr + 32 * k), sdesc(wl + 2048 * k), idesc_bf16(128, 64, false, true),
                             k > 0);
                const uint32_t dw = tmem + 64u + 64u * (uint32_t)l;
                for (uint32_t k = 0; k < kRows / 16; ++k)
                    mma_bf16(dw, sdesc(dy_addr + 2048 * k), sdesc(xl + 2048 * k), idesc_bf16(128, 64, true, true),
                             (!first || k > 0) ? 1u : 0u);
                mma_commit(bar_m);
            }
            ok = mbar_wait(bar_m, phase, a.wait.limit_ns);
            phase ^= 1u;
            tc_fence_after();
            float v[kWidth];
#pragma unroll
            for (int c = 0; c < 4; ++c) tmem_ld16(lane_addr + 16 * c, v + 16 * c);
            if (l > 0) {
                const uint8_t* xl = X + l * kTileBytes;
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const uint4 w = *reinterpret_cast<const uint4*>(xl + swz(tid, c));
                    const uint32_t ws[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        // the ReLU passed the gradient where its output is positive
                        if ((ws[k] & 0x8000u) || !(ws[k] & 0x7fffu)) v[8 * c + 2 * k] = 0.0f;
                        if ((ws[k] & 0x80000000u) || !(ws[k] & 0x7fff0000u)) v[8 * c + 2 * k + 1] = 0.0f;
                    }
                }
                store_row<false>(dY, tid, v);
            } else if (valid) {
#pragma unroll 1
                for (int lev = 0; lev < kLevels; ++lev) {
                    uint32_t c[3];
                    float f[3];
                    grid_cell(a.g, lev, u, c, f);
                    const float g0 = v[kInputHash + 2 * lev], g1 = v[kInputHash + 2 * lev + 1];
                    float2* lv = a.grid_grad + ((size_t)lev << a.g.log2_table);
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const uint32_t dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
                        const float w = (dx ? f[0] : 1.0f - f[0]) * (dy ? f[1] : 1.0f - f[1]) *
                                        (dz ? f[2] : 1.0f - f[2]);
                        atomicAdd(lv + grid_index(a.g, lev, c[0] + dx, c[1] + dy, c[2] + dz),
                                  make_float2(w * g0, w * g1));
                    }
                }
            }
        }
        first = false;
    }
    // loss of the CTA
    for (int o = 16; o > 0; o >>= 1) loss_sum += __shfl_xor_sync(0xffffffffu, loss_sum, o);
    if (lane == 0 && loss_sum != 0.0f) atomicAdd(a.loss, loss_sum);
    // the CTA's weight-gradient partial: TMEM lanes = output rows
    tc_fence_before();
    const bool good = __syncthreads_and(ok && !abort);   // block-uniform: tcgen05.ld needs whole warps
    tc_fence_after();
    if (good && warp < 2) {
        float* part = a.partial + (size_t)blockIdx.x * kMlpParams;
        const uint32_t o = warp * 32u + lane;
        for (int l = 0; l < kLayers; ++l) {
            if (l == kHidden && warp > 0) break;   // the output layer has 16 rows
            float* dst = part + (size_t)l * kWidth * kWidth + (size_t)o * kWidth;
#pragma unroll 1
            for (int c = 0; c < 4; ++c) {
                float v[16];
                tmem_ld16(lane_addr + 64u + 64u * (uint32_t)l + 16u * c, v);
                float4* d4 = reinterpret_cast<float4*>(dst + 16 * c);
#pragma unroll
                for (int k = 0; k < 4; ++k) d4[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
            }
        }
    }
    if (!good && tid == 0) set_error(a.err, kErrTimeout);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, kTrainTmemCols);
}

// ------------------------------------------------------------------ optimiser
__global__ void __launch_bounds__(256) adam_mlp_kernel(const float* __restrict__ partial, uint32_t parts,
                                                      float* master, float* m, float* v, float* grad, uint8_t* image,
                                                      AdamStep s, bool apply)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kMlpParams) return;
    const uint32_t l = idx / (kWidth * kWidth), o = (idx / kWidth) % kWidth, i = idx % kWidth;
    if (l == kHidden && o >= (uint32_t)kOutputs) return;   // padding rows stay zero
    float g = 0.0f;
    for (uint32_t c = 0; c < parts; ++c) g += partial[(size_t)c * kMlpParams + idx];
    grad[idx] = g;
    if (!apply) return;
    const float mm = s.beta1 * m[idx] + (1.0f - s.beta1) * g;
    const float vv = s.beta2 * v[idx] + (1.0f - s.beta2) * g * g;
    m[idx] = mm;
    v[idx] = vv;
    const float p = master[idx] - s.lr * (mm * s.c1) / (sqrtf(vv * s.c2) + s.eps);
    master[idx] = p;
    *reinterpret_cast<__nv_bfloat16*>(image + weight_offset(l, o, i)) = __float2bfloat16_rn(p);
}

__global__ void __launch_bounds__(256) write_image_kernel(const float* __restrict__ master, uint8_t* image)
{
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= kMlpParams) return;
    const uint32_t l = idx / (kWidth * kWidth), o = (idx / kWidth) % kWidth, i = idx % kWidth;
    if (l == kHidden && o >= (uint32_t)kOutRows) return;
    const float p = (l == kHidden && o >= (uint32_t)kOutputs) ? 0.0f : master[idx];
    *reinterpret_cast<__nv_bfloat16*>(image + weight_offset(l, o, i)) = __float2bfloat16_rn(p);
}

__global__ void __launch_bounds__(256) adam_grid_kernel(const float4* __restrict__ grad, float4* master, float4* m,
                                                       float4* v, uint2* table, size_t n4, AdamStep s)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 g = grad[i];
        float4 mm = m[i], vv = v[i], p = master[i];
        float* gp = (float*)&g;
        float* mp = (float*)&mm;
        float* vp = (float*)&vv;
        float* pp = (float*)&p;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            mp[k] = s.beta1 * mp[k] + (1.0f - s.beta1) * gp[k];
            vp[k] = s.beta2 * vp[k] + (1.0f - s.beta2) * gp[k] * gp[k];
            pp[k] -= s.lr * (mp[k] * s.c1) / (sqrtf(vp[k] * s.c2) + s.eps);
        }
        m[i] = mm;
        v[i] = vv;
        master[i] = p;
        const __half2 h0 = __floats2half2_rn(p.x, p.y), h1 = __floats2half2_rn(p.z, p.w);
        table[i] = make_uint2(*reinterpret_cast<const uint32_t*>(&h0), *reinterpret_cast<const uint32_t*>(&h1));
    }
}

__global__ void __launch_bounds__(256) write_table_kernel(const float4* __restrict__ master, uint2* table, size_t n4)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 p = master[i];
        const __half2 h0 = __floats2half2_rn(p.x, p.y), h1 = __floats2half2_rn(p.z, p.w);
        table[i] = make_uint2(*reinterpret_cast<const uint32_t*>(&h0), *reinterpret_cast<const uint32_t*>(&h1));
    }
}

// ------------------------------------------------------------------ launchers
namespace {
unsigned elementwise_grid(size_t n, int threads)
{
    const size_t want = (n + threads - 1) / threads;
    const size_t cap = (size_t)sm_count() * 16;
    return (unsigned)(want < 1 ? 1 : (want > cap ? cap : want));
}
}  // namespace

uint32_t train_grid_size(uint32_t n)
{
    const uint32_t tiles = (n + kRows - 1) / kRows;
    const uint32_t sms = (uint32_t)sm_count();
    return tiles < 1 ? 1 : (tiles < sms ? tiles : sms);
}

cudaError_t launch_encode(const GridGeometry& g, const __half2* table, const float4* queries, uint32_t n, float* out,
                          cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    encode_kernel<<<elementwise_grid(n, 256), 256, 0, st>>>(g, table, queries, n, out);
    return cudaGetLastError();
}

template <int G>
static cudaError_t launch_infer_groups(const InferArgs& a, cudaStream_t st)
{
    static int per_sm = 0;
    if (!per_sm) {
        // no carveout preference: the hash-grid gathers live on the L1 left beside the shared memory
        cudaError_t e = cudaFuncSetAttribute(infer_kernel<G>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             infer_smem(G));
        if (e != cudaSuccess) return e;
        int occ = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, infer_kernel<G>, 128 * G, infer_smem(G));
        const int tmem_cap = (int)(512u / infer_tmem_cols(G));   // resident CTAs' columns fit the SM's 512
        per_sm = occ < 1 ? 1 : (occ > tmem_cap ? tmem_cap : occ);
    }
    const uint32_t tiles = (a.n + kRows - 1) / kRows;
    const uint32_t want = (tiles + G - 1) / G;
    const uint32_t cap = (uint32_t)(sm_count() * per_sm);
    infer_kernel<G><<<want < cap ? want : cap, 128 * G, infer_smem(G), st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_infer(const GridGeometry& g, const __half2* table, const uint8_t* weights, const float4* queries,
                         uint32_t n, float* out_rgb, const float4* thr, float4* pay, int* err, cudaStream_t st,
                         const uint32_t* n_dev, int groups, const WaitPolicy& wait)
{
    if (n == 0) return cudaSuccess;
    const InferArgs a{g, table, weights, queries, n, out_rgb, thr, pay, err, n_dev, wait};
    switch (groups) {
    case 1: return launch_infer_groups<1>(a, st);
    case 2: return launch_infer_groups<2>(a, st);
    default: return launch_infer_groups<4>(a, st);
    }
}

cudaError_t launch_train(const GridGeometry& g, const __half2* table, const uint8_t* weights, const TrainBatch& b,
                         float2* grid_grad, float* partial, uint32_t max_parts, uint32_t* parts, float* loss,
                         int* err, cudaStream_t st, const WaitPolicy& wait)
{
    *parts = 0;
    if (b.n == 0) return cudaSuccess;
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem);
        if (e != cudaSuccess) return e;
        configured = true;
    }
    uint32_t grid = train_grid_size(b.n);
    if (grid > max_parts) grid = max_parts;
    TrainArgs a{g, table, weights, b, 1.0f / (3.0f * (float)b.n), grid_grad, partial, loss, err, wait};
    train_kernel<<<grid, kThreads, kTrainSmem, st>>>(a);
    *parts = grid;
    return cudaGetLastError();
}

cudaError_t launch_adam_mlp(const float* partial, uint32_t parts, float* master, float* m, float* v, float* grad,
                            uint8_t* image, const AdamStep& s, bool apply, cudaStream_t st)
{
    adam_mlp_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(partial, parts, master, m, v, grad, image, s, apply);
    return cudaGetLastError();
}

cudaError_t launch_adam_grid(const float* grad, float* master, float* m, float* v, __half2* table, size_t nfloats,
                             const AdamStep& s, cudaStream_t st)
{
    const size_t n4 = nfloats / 4;
    adam_grid_kernel<<<elementwise_grid(n4, 256), 256, 0, st>>>(
        reinterpret_cast<const float4*>(grad), reinterpret_cast<float4*>(master), reinterpret_cast<float4*>(m),
        reinterpret_cast<float4*>(v), reinterpret_cast<uint2*>(table), n4, s);
    return cudaGetLastError();
}

cudaError_t launch_write_image(const float* master, uint8_t* image, cudaStream_t st)
{
    write_image_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(master, image);
    return cudaGetLastError();
}

cudaError_t launch_write_table(const float* master, __half2* table, size_t nfloats, cudaStream_t st)
{
    const size_t n4 = nfloats / 4;
    write_table_kernel<<<elementwise_grid(n4, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(master),
                                                                   reinterpret_cast<uint2*>(table), n4);
    return cudaGetLastError();
}

}  // namespace nrc
}  // namespace pico
