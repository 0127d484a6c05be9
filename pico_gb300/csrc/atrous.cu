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
//          out = sum(w * c) / sum(w), evaluated with one exponential per tap
//          (see the kernel).
//
// The statistics are exact; the blend agrees with the reference's arithmetic to
// about 1e-6 relative and keeps its NaN pattern.
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
constexpr int kStatsThreads = 512;
constexpr int kMaxSpan = kTile + 4 * 16;   // tap footprint of a tile along one axis, spacing <= 16

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Coordinates some tap x + k*s (x in [a, b], k in -2..2, clamped to [0, n-1])
// reaches: the union of the five clamped intervals, merged into at most five
// disjoint sorted spans.  Clamping is monotone, so each interval stays whole.
__device__ __forceinline__ int tap_spans(int a, int b, int s, int n, int* lo, int* hi)
{
    int m = 0;
#pragma unroll
    for (int k = -2; k <= 2; ++k) {
        const int l = clampi(a + k * s, 0, n - 1), h = clampi(b + k * s, 0, n - 1);
        if (m > 0 && l <= hi[m - 1] + 1) {
            hi[m - 1] = max(hi[m - 1], h);
        } else {
            lo[m] = l; hi[m] = h; ++m;
        }
    }
    return m;
}

// Lists the members of the spans in out[] with all threads; returns their count.
__device__ __forceinline__ int list_spans(const int* lo, const int* hi, int m, int* out)
{
    int total = 0;
    for (int i = 0; i < m; ++i) total += hi[i] - lo[i] + 1;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        int i = 0, base = 0;
        while (t - base > hi[i] - lo[i]) { base += hi[i] - lo[i] + 1; ++i; }
        out[t] = lo[i] + (t - base);
    }
    return total;
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
    __shared__ int cols[kMaxSpan], rows[kMaxSpan];
    __shared__ int span[4][5], nspan[2];
    if (threadIdx.x == 0) {
        nspan[0] = tap_spans(x0, x1, s, (int)W, span[0], span[1]);
        nspan[1] = tap_spans(y0, y1, s, (int)H, span[2], span[3]);
    }
    __syncthreads();
    const int ncols = list_spans(span[0], span[1], nspan[0], cols);
    const int nrows = list_spans(span[2], span[3], nspan[1], rows);
    __syncthreads();
    // maximum luminance and min / max |position| over the footprint; max / min are
    // exact, so the visiting order is free, and the selects keep std::max / std::min's
    // NaN behaviour
    const float kInf = __int_as_float(0x7f800000);
    float white = 0.0f, mind = kInf, maxd = -kInf;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int r = warp; r < nrows; r += kStatsThreads / 32) {
        const size_t rb = (size_t)rows[r] * W;
        for (int c = lane; c < ncols; c += 32) {
            const size_t f = rb + (size_t)cols[c];
            const float l = luminance(__ldg(pix + 3 * f), __ldg(pix + 3 * f + 1), __ldg(pix + 3 * f + 2));
            white = (white < l) ? l : white;
            const float len = length(v3(__ldg(pos + 3 * f), __ldg(pos + 3 * f + 1), __ldg(pos + 3 * f + 2)));
            mind = (len < mind) ? len : mind;
            maxd = (maxd < len) ? len : maxd;
        }
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

// One thread per pixel, 25 taps.  The reference's weight
//   k[u] * min(exp(-|dn|^2/0.25),1) * min(exp(-|dp|^2/range^2),1) * min(exp(-|da|^2/white^2),1)
// is evaluated as k[u] * exp(-(4|dn|^2 + |dp|^2 * (1/range^2) + |da|^2 * (1/white^2))): the
// arguments are never positive, so the min(., 1) clamps only pass NaN through, and a sum
// of -inf / NaN terms gives the same 0 / NaN as the product of exponentials.  One fast
// exponential per tap instead of three exact ones and three divides; the result stays
// within 1e-5 relative of the exact evaluation (the weights enter a normalised sum in
// which the centre tap, k = 0.159, always has exponent 0).
template <typename Idx>
__global__ void __launch_bounds__(256) atrous_blend_kernel(const float* __restrict__ src,
                                                           const float* __restrict__ nrm,
                                                           const float* __restrict__ pos,
                                                           const float* __restrict__ dif, uint32_t W, uint32_t H,
                                                           int s, const float2* __restrict__ stats,
                                                           float* __restrict__ dst)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const float2 st = stats[(y / kTile) * tiles_x + x / kTile];
    const float ip = __frcp_rn(__fmul_rn(st.y, st.y));   // 1 / range^2 (inf for a zero range)
    const float iw = __frcp_rn(__fmul_rn(st.x, st.x));   // 1 / white^2
    const Idx c = ((Idx)y * W + x) * 3;
    const float ncx = nrm[c], ncy = nrm[c + 1], ncz = nrm[c + 2];
    const float pcx = pos[c], pcy = pos[c + 1], pcz = pos[c + 2];
    const float dcx = dif[c], dcy = dif[c + 1], dcz = dif[c + 2];
    Idx col[5], row[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        col[k] = (Idx)clampi((int)x + (k - 2) * s, 0, (int)W - 1) * 3;
        row[k] = (Idx)clampi((int)y + (k - 2) * s, 0, (int)H - 1) * W * 3;
    }
    float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, wsum = 0.0f;
#pragma unroll
    for (int j = 0; j < 5; ++j) {
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const Idx f = row[j] + col[i];
            const float nx = ncx - __ldg(nrm + f), ny = ncy - __ldg(nrm + f + 1), nz = ncz - __ldg(nrm + f + 2);
            const float px = pcx - __ldg(pos + f), py = pcy - __ldg(pos + f + 1), pz = pcz - __ldg(pos + f + 2);
            const float ax = dcx - __ldg(dif + f), ay = dcy - __ldg(dif + f + 1), az = dcz - __ldg(dif + f + 2);
            const float dn = nx * nx + ny * ny + nz * nz;
            const float dp = px * px + py * py + pz * pz;
            const float da = ax * ax + ay * ay + az * az;
            const float w = kAtrousWeights[j * 5 + i] * __expf(-(4.0f * dn + dp * ip + da * iw));
            r0 += __ldg(src + f) * w;
            r1 += __ldg(src + f + 1) * w;
            r2 += __ldg(src + f + 2) * w;
            wsum += w;
        }
    }
    dst[c] = __fdiv_rn(r0, wsum);
    dst[c + 1] = __fdiv_rn(r1, wsum);
    dst[c + 2] = __fdiv_rn(r2, wsum);
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
        if ((uint64_t)W * H * 3 < (1ull << 32))
            atrous_blend_kernel<uint32_t><<<grid, 256, 0, st>>>(src, normals, positions, diffuse, W, H, s, stats, dst);
        else
            atrous_blend_kernel<size_t><<<grid, 256, 0, st>>>(src, normals, positions, diffuse, W, H, s, stats, dst);
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
