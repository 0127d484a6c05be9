// A-trous denoiser (Util::atrous_denoise, Util/Denoisers.cpp:107-126; blend_pixel :18-101).
//
// Five levels with tap spacing 1, 2, 4, 8, 16 over a 5x5 kernel (the reference's
// table, including its 0.09563 entry at index 17).  Each level runs two kernels:
//
//   stats  one CTA per 64x64 tile (the reference's Tiler tiles, clamped at the
//          right and bottom edges): the maximum luminance and the min / max
//          |position| over every pixel some tap of the tile reads.  That set is
//          rows x columns, each a union of five shifted copies of the tile's
//          range, clamped; the CTA walks the distinct members once instead of
//          25 taps per pixel.  max / min are exact, so the order is free, and
//          the selects keep std::max / std::min's NaN behaviour.
//   blend  one thread per pixel: 25 taps, weights
//          w = k[u] * min(exp(-|dn|^2/0.25),1) * min(exp(-|dp|^2/range^2),1)
//                   * min(exp(-|dalbedo|^2/white^2),1),
//          out = sum(w * c) / sum(w), in the reference's operation order.
//
// Arithmetic is exact IEEE except expf, which differs from the host libm by a
// few ulp; results agree with the reference to ~1e-6 relative.
#include "exact_math.cuh"
#include "kernels_render.h"

#include <algorithm>

namespace pico {

__constant__ float kAtrousWeights[25] = {
    0.00292f, 0.01306f, 0.02154f, 0.01306f, 0.00292f,
    0.01306f, 0.05855f, 0.09653f, 0.05855f, 0.01306f,
    0.02154f, 0.09653f, 0.15915f, 0.09653f, 0.02154f,
    0.01306f, 0.05855f, 0.09563f, 0.05855f, 0.01306f,
    0.00292f, 0.01306f, 0.02154f, 0.01306f, 0.00292f};

constexpr int kTile = 64;
constexpr int kStatsThreads = 256;

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Is raw coordinate c reached by some tap x + k*s, x in [a, b], k in [-2, 2]?
__device__ __forceinline__ bool tap_reaches(int c, int a, int b, int s)
{
#pragma unroll
    for (int k = -2; k <= 2; ++k) {
        const int x = c - k * s;
        if (x >= a && x <= b) return true;
    }
    return false;
}

__device__ __forceinline__ float luminance(float r, float g, float b)
{
    using namespace ex;
    return add(add(mul(r, 0.2126f), mul(g, 0.587f)), mul(b, 0.114f));
}

__global__ void __launch_bounds__(kStatsThreads) atrous_stats_kernel(const float* __restrict__ pix,
                                                                      const float* __restrict__ pos, uint32_t W,
                                                                      uint32_t H, int s, float2* __restrict__ stats)
{
    using namespace ex;
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const int tx = blockIdx.x % tiles_x, ty = blockIdx.x / tiles_x;
    const int x0 = tx * kTile, y0 = ty * kTile;
    const int x1 = min(x0 + kTile, (int)W) - 1, y1 = min(y0 + kTile, (int)H) - 1;
    // raw candidate ranges [x0 - 2s, x1 + 2s] (at most 64 + 64 wide for s <= 16)
    __shared__ int cols[kTile + 4 * 16 + 1], rows[kTile + 4 * 16 + 1];
    __shared__ int ncols, nrows;
    if (threadIdx.x == 0) {
        int n = 0;
        for (int c = x0 - 2 * s; c <= x1 + 2 * s; ++c)
            if (tap_reaches(c, x0, x1, s)) cols[n++] = clampi(c, 0, (int)W - 1);
        ncols = n;
        n = 0;
        for (int r = y0 - 2 * s; r <= y1 + 2 * s; ++r)
            if (tap_reaches(r, y0, y1, s)) rows[n++] = clampi(r, 0, (int)H - 1);
        nrows = n;
    }
    __syncthreads();
    const float kInf = __int_as_float(0x7f800000);
    float white = 0.0f, mind = kInf, maxd = -kInf;
    const int total = ncols * nrows;
    for (int k = threadIdx.x; k < total; k += blockDim.x) {
        const size_t f = (size_t)rows[k / ncols] * W + (size_t)cols[k % ncols];
        const float l = luminance(pix[3 * f], pix[3 * f + 1], pix[3 * f + 2]);
        white = (white < l) ? l : white;
        const float len = length(v3(pos[3 * f], pos[3 * f + 1], pos[3 * f + 2]));
        mind = (len < mind) ? len : mind;
        maxd = (maxd < len) ? len : maxd;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const float w2 = __shfl_down_sync(0xffffffffu, white, off);
        const float a2 = __shfl_down_sync(0xffffffffu, mind, off);
        const float b2 = __shfl_down_sync(0xffffffffu, maxd, off);
        white = (white < w2) ? w2 : white;
        mind = (a2 < mind) ? a2 : mind;
        maxd = (maxd < b2) ? b2 : maxd;
    }
    __shared__ float sw[kStatsThreads / 32], sa[kStatsThreads / 32], sb[kStatsThreads / 32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sw[warp] = white; sa[warp] = mind; sb[warp] = maxd; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kStatsThreads / 32; ++w) {
            white = (white < sw[w]) ? sw[w] : white;
            mind = (sa[w] < mind) ? sa[w] : mind;
            maxd = (maxd < sb[w]) ? sb[w] : maxd;
        }
        stats[blockIdx.x] = make_float2(white, sub(maxd, mind));
    }
}

__device__ __forceinline__ float min1(float e) { return (1.0f < e) ? 1.0f : e; }

__global__ void __launch_bounds__(256) atrous_blend_kernel(const float* __restrict__ src,
                                                           const float* __restrict__ nrm,
                                                           const float* __restrict__ pos,
                                                           const float* __restrict__ dif, uint32_t W, uint32_t H,
                                                           int s, const float2* __restrict__ stats,
                                                           float* __restrict__ dst)
{
    using namespace ex;
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const float2 st = stats[(y / kTile) * tiles_x + x / kTile];
    const float white = st.x, range = st.y;
    const float wden = mul(white, white), pden = mul(range, range);
    const size_t c = (size_t)y * W + x;
    const V3 nc = v3(nrm[3 * c], nrm[3 * c + 1], nrm[3 * c + 2]);
    const V3 pc = v3(pos[3 * c], pos[3 * c + 1], pos[3 * c + 2]);
    const V3 dc = v3(dif[3 * c], dif[3 * c + 1], dif[3 * c + 2]);
    float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, wsum = 0.0f;
#pragma unroll 5
    for (int u = 0; u < 25; ++u) {
        const int ix = clampi((int)x + (u % 5 - 2) * s, 0, (int)W - 1);
        const int iy = clampi((int)y + (u / 5 - 2) * s, 0, (int)H - 1);
        const size_t f = (size_t)iy * W + ix;
        V3 t = vsub(nc, v3(__ldg(nrm + 3 * f), __ldg(nrm + 3 * f + 1), __ldg(nrm + 3 * f + 2)));
        const float nw = min1(expf(div(-dot(t, t), 0.25f)));
        t = vsub(pc, v3(__ldg(pos + 3 * f), __ldg(pos + 3 * f + 1), __ldg(pos + 3 * f + 2)));
        const float pw = min1(expf(div(-dot(t, t), pden)));
        t = vsub(dc, v3(__ldg(dif + 3 * f), __ldg(dif + 3 * f + 1), __ldg(dif + 3 * f + 2)));
        const float dw = min1(expf(div(-dot(t, t), wden)));
        const float w = mul(mul(mul(kAtrousWeights[u], nw), pw), dw);
        r0 = add(r0, mul(__ldg(src + 3 * f), w));
        r1 = add(r1, mul(__ldg(src + 3 * f + 1), w));
        r2 = add(r2, mul(__ldg(src + 3 * f + 2), w));
        wsum = add(wsum, w);
    }
    dst[3 * c] = div(r0, wsum);
    dst[3 * c + 1] = div(r1, wsum);
    dst[3 * c + 2] = div(r2, wsum);
}

cudaError_t launch_atrous(const float* pixels, const float* normals, const float* positions, const float* diffuse,
                          uint32_t W, uint32_t H, float* scratch_a, float* scratch_b, float* tile_stats, float* out,
                          cudaStream_t st)
{
    if (W == 0 || H == 0) return cudaSuccess;
    const uint32_t tiles = ((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
    float2* stats = reinterpret_cast<float2*>(tile_stats);
    const float* src = pixels;
    for (int level = 0; level < 5; ++level) {
        // ping-pong: in -> A -> B -> A -> B -> out
        float* dst = level == 4 ? out : ((level % 2 == 0) ? scratch_a : scratch_b);
        const int s = 1 << level;
        atrous_stats_kernel<<<tiles, kStatsThreads, 0, st>>>(src, positions, W, H, s, stats);
        dim3 grid((W + 255) / 256, H);
        atrous_blend_kernel<<<grid, 256, 0, st>>>(src, normals, positions, diffuse, W, H, s, stats, dst);
        src = dst;
    }
    return cudaGetLastError();
}

}  // namespace pico

// ---------------------------------------------------------------------------
// Reinhard tone mapping (Util::reinhard_tone_mapping, Util/ToneMappers.cpp:12-44):
// a global white point = the largest luminance (from 0; NaN luminances are
// skipped, as std::max(white, lum) skips them), then per channel
// p * (1 + p / white^2) / (1 + p), in place.  Non-negative floats order like
// their bit patterns, so the maximum is an atomicMax on the bits.
namespace pico {

__global__ void __launch_bounds__(256) white_point_kernel(const float* __restrict__ pix, size_t npx,
                                                          unsigned* __restrict__ white_bits)
{
    float w = 0.0f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npx; i += (size_t)gridDim.x * blockDim.x) {
        const float l = luminance(pix[3 * i], pix[3 * i + 1], pix[3 * i + 2]);
        w = (w < l) ? l : w;
    }
    for (int off = 16; off > 0; off >>= 1) {
        const float o = __shfl_down_sync(0xffffffffu, w, off);
        w = (w < o) ? o : w;
    }
    if ((threadIdx.x & 31u) == 0) atomicMax(white_bits, __float_as_uint(w));
}

__global__ void __launch_bounds__(256) reinhard_kernel(float* __restrict__ pix, size_t n,
                                                       const unsigned* __restrict__ white_bits)
{
    using namespace ex;
    const float w = __uint_as_float(*white_bits);
    const float w2 = mul(w, w);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float p = pix[i];
        const float num = mul(p, add(1.0f, div(p, w2)));
        pix[i] = div(num, add(1.0f, p));
    }
}

cudaError_t launch_reinhard(float* pixels, uint32_t W, uint32_t H, unsigned* scratch, cudaStream_t st)
{
    const size_t npx = (size_t)W * H;
    if (npx == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned)std::min<size_t>((npx + 255) / 256, (size_t)sm_count() * 8);
    white_point_kernel<<<blocks, 256, 0, st>>>(pixels, npx, scratch);
    reinhard_kernel<<<blocks, 256, 0, st>>>(pixels, 3 * npx, scratch);
    return cudaGetLastError();
}

}  // namespace pico
