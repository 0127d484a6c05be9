// A-trous denoiser (Util::atrous_denoise, Util/Denoisers.cpp:107-126; blend_pixel :18-101).
//
// Five levels with tap spacing 1, 2, 4, 8, 16 over a 5x5 kernel (the reference's
// table, including its 0.09563 entry at index 17).  Per 64x64 tile (the
// reference's Tiler tiles, clamped at the right and bottom edges) and level the
// blend needs the maximum luminance and the min / max |position| over every
// pixel some tap of the tile reads.  That set is rows x columns, each a union of
// five shifted copies of the tile's range, clamped.  The positions are the same
// at every level, so two launches first reduce all five levels' |position|
// ranges, separably (per image row over each tile column's footprint columns,
// then per tile over its footprint rows), reading the positions once; then each
// level runs two kernels:
//
//   stats  the maximum luminance of the level's input colour over the tile's
//          footprint (four CTAs per tile, each a quarter of the footprint rows),
//          walking the distinct members once instead of 25 taps per pixel.
//          max / min are exact, so the order is free, and the selects keep
//          std::max / std::min's NaN behaviour.
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
constexpr int kStatsThreads = 256;
constexpr int kStatsSplit = 4;   // CTAs per tile; each reduces every fourth footprint row group
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

// Maximum luminance over this CTA's quarter of a tile's footprint rows (a partial
// record per CTA; tile_stats combines the four).
__global__ void __launch_bounds__(kStatsThreads) atrous_stats_kernel(const float* __restrict__ pix, uint32_t W,
                                                                      uint32_t H, int s, float* __restrict__ parts)
{
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const int tile = (int)(blockIdx.x / kStatsSplit), part = (int)(blockIdx.x % kStatsSplit);
    const int tx = tile % tiles_x, ty = tile / tiles_x;
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
    float white = 0.0f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int kWarps = kStatsThreads / 32;
    for (int r = part * kWarps + warp; r < nrows; r += kStatsSplit * kWarps) {
        const size_t rb = (size_t)rows[r] * W;
        for (int c = lane; c < ncols; c += 32) {
            const size_t f = rb + (size_t)cols[c];
            const float l = luminance(__ldg(pix + 3 * f), __ldg(pix + 3 * f + 1), __ldg(pix + 3 * f + 2));
            white = (white < l) ? l : white;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        const float w2 = __shfl_down_sync(0xffffffffu, white, off);
        white = (white < w2) ? w2 : white;
    }
    __shared__ float sw[kWarps];
    if (lane == 0) sw[warp] = white;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kWarps; ++w) white = (white < sw[w]) ? sw[w] : white;
        parts[blockIdx.x] = white;
    }
}

// The min / max |position| over each level's footprint of each tile, in two
// separable steps (the footprint is a set of rows times a set of columns):
//   row_range   one warp per (image row, tile column): |position| of the columns
//               any level's footprint of that tile column can reach ([x0 - 32,
//               x1 + 32], clamped) is read once, then reduced over each level's
//               column spans: rrow[(level * H + y) * tiles_x + tx] = (min, max);
//   tile_range  one warp per (tile, level): the row ranges reduced over the
//               level's row spans: range[level * tiles + tile] = (min, max).
// min / max are exact, so the grouping is free, and the selects keep std::min /
// std::max's NaN behaviour (a NaN |position| never replaces a bound).
constexpr int kRowWarps = 4;
// Whether column (or row) c is read by a tap of the stencil (offsets -2..2 times s, clamped to
// [0, n - 1]) from some pixel of [a, b]: the union tap_spans lists, tested tap by tap so that
// everything stays in registers (span arrays indexed at run time would live in local memory).
__device__ __forceinline__ bool tapped(int c, int a, int b, int s, int n)
{
    bool in = false;
#pragma unroll
    for (int k = -2; k <= 2; ++k) in |= clampi(a + k * s, 0, n - 1) <= c && c <= clampi(b + k * s, 0, n - 1);
    return in;
}

__global__ void __launch_bounds__(32 * kRowWarps) atrous_row_range_kernel(const float* __restrict__ pos, uint32_t W,
                                                                        uint32_t H, float2* __restrict__ rrow)
{
    using namespace ex;
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const int lane = threadIdx.x & 31;
    const long long task = (long long)blockIdx.x * kRowWarps + (threadIdx.x >> 5);
    if (task >= (long long)H * tiles_x) return;   // the whole warp leaves together
    const int y = (int)(task / tiles_x), tx = (int)(task % tiles_x);
    const int x0 = tx * kTile, x1 = min(x0 + kTile, (int)W) - 1;
    const int rx0 = max(x0 - 32, 0), rx1 = min(x1 + 32, (int)W - 1);
    // the span's positions (at most 128 pixels, 384 floats) staged through shared memory with
    // consecutive lanes reading consecutive floats, all twelve loads in flight before the first
    // store, then |position| of columns rx0 + lane + 32 k
    __shared__ float stage[kRowWarps][3 * 128];
    float* st = stage[threadIdx.x >> 5];
    const int nf = 3 * (rx1 - rx0 + 1);
    const float* row = pos + 3 * ((size_t)y * W + (size_t)rx0);
    float v[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) v[k] = (lane + 32 * k < nf) ? __ldg(row + lane + 32 * k) : 0.0f;
#pragma unroll
    for (int k = 0; k < 12; ++k) st[lane + 32 * k] = v[k];
    __syncwarp();
    float len[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int j = lane + 32 * k;
        len[k] = (rx0 + j <= rx1) ? length(v3(st[3 * j], st[3 * j + 1], st[3 * j + 2])) : 0.0f;
    }
    const float kInf = __int_as_float(0x7f800000);
    // A tile column at least 16 wide (all but a narrow last one) has overlapping taps at every
    // spacing up to 16: its columns are then the one range [x0 - 2 s, x1 + 2 s], clamped.
    const bool wide = x1 - x0 + 1 >= 16;
#pragma unroll
    for (int level = 0; level < 5; ++level) {
        const int s = 1 << level;
        const int lo = max(x0 - 2 * s, 0), hi = min(x1 + 2 * s, (int)W - 1);
        float mind = kInf, maxd = -kInf;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int c = rx0 + lane + 32 * k;
            if (c >= lo && c <= hi && (wide || tapped(c, x0, x1, s, (int)W))) {
                mind = (len[k] < mind) ? len[k] : mind;
                maxd = (maxd < len[k]) ? len[k] : maxd;
            }
        }
        for (int off = 16; off > 0; off >>= 1) {
            const float a2 = __shfl_down_sync(0xffffffffu, mind, off);
            const float b2 = __shfl_down_sync(0xffffffffu, maxd, off);
            mind = (a2 < mind) ? a2 : mind;
            maxd = (maxd < b2) ? b2 : maxd;
        }
        if (lane == 0) rrow[((size_t)level * H + y) * tiles_x + tx] = make_float2(mind, maxd);
    }
}

__global__ void __launch_bounds__(32 * 5) atrous_tile_range_kernel(const float2* __restrict__ rrow, uint32_t W,
                                                                   uint32_t H, float2* __restrict__ range)
{
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const int tiles = tiles_x * (int)((H + kTile - 1) / kTile);
    const int tile = (int)blockIdx.x, level = (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int tx = tile % tiles_x, y0 = (tile / tiles_x) * kTile;
    const int y1 = min(y0 + kTile, (int)H) - 1;
    const int s = 1 << level;
    const float kInf = __int_as_float(0x7f800000);
    float mind = kInf, maxd = -kInf;
    // the rows between the first and the last tap, those some tap reads
    for (int r = max(y0 - 2 * s, 0) + lane; r <= min(y1 + 2 * s, (int)H - 1); r += 32)
        if (tapped(r, y0, y1, s, (int)H)) {
            const float2 v = rrow[((size_t)level * H + r) * tiles_x + tx];
            mind = (v.x < mind) ? v.x : mind;
            maxd = (maxd < v.y) ? v.y : maxd;
        }
    for (int off = 16; off > 0; off >>= 1) {
        const float a2 = __shfl_down_sync(0xffffffffu, mind, off);
        const float b2 = __shfl_down_sync(0xffffffffu, maxd, off);
        mind = (a2 < mind) ? a2 : mind;
        maxd = (maxd < b2) ? b2 : maxd;
    }
    if (lane == 0) range[level * tiles + tile] = make_float2(mind, maxd);
}

// A tile's white point (from its kStatsSplit partial records) and |position| range.
__device__ __forceinline__ float2 tile_stats(const float* __restrict__ parts, const float2* __restrict__ range,
                                             int tile)
{
    float w = parts[tile * kStatsSplit];
#pragma unroll
    for (int k = 1; k < kStatsSplit; ++k) {
        const float p = parts[tile * kStatsSplit + k];
        w = (w < p) ? p : w;
    }
    const float2 r = range[tile];
    return make_float2(w, __fsub_rn(r.y, r.x));
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
                                                           int s, const float* __restrict__ stats,
                                                           const float2* __restrict__ range, float* __restrict__ dst)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const float2 st = tile_stats(stats, range, (int)((y / kTile) * tiles_x + x / kTile));
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

// The same blend with its taps staged in shared memory, for small spacings.  At
// spacing s every tap of a pixel lands on the pixel's own sub-lattice (x mod s,
// y mod s), so a CTA takes a kLatX x kLatY tile of one sub-lattice; the
// (kLatX + 4) x (kLatY + 4) lattice points its taps read (coordinates clamped
// exactly as the taps clamp them) are staged once as 48-byte records (normal,
// position, albedo, colour) and read back with 128-bit loads.  Each thread blends
// two horizontally adjacent lattice pixels, which share four of their five tap
// columns; the records of a footprint row are split into even and odd columns so
// that a warp's loads hit consecutive records.  The arithmetic per tap is the
// direct kernel's above, so the two kernels give identical results.
constexpr int kLatX = 64, kLatY = 8, kBlendThreads = (kLatX / 2) * kLatY;
constexpr int kFootX = kLatX + 4, kHalfX = kFootX / 2, kFootY = kLatY + 4;

__device__ __forceinline__ void blend_tap(const float4 t0, const float4 t1, const float4 t2, float k, const float* c,
                                          float ip, float iw, float* acc)
{
    const float nx = c[0] - t0.x, ny = c[1] - t0.y, nz = c[2] - t0.z;
    const float px = c[3] - t0.w, py = c[4] - t1.x, pz = c[5] - t1.y;
    const float ax = c[6] - t1.z, ay = c[7] - t1.w, az = c[8] - t2.x;
    const float dn = nx * nx + ny * ny + nz * nz;
    const float dp = px * px + py * py + pz * pz;
    const float da = ax * ax + ay * ay + az * az;
    const float w = k * __expf(-(4.0f * dn + dp * ip + da * iw));
    acc[0] += t2.y * w;
    acc[1] += t2.z * w;
    acc[2] += t2.w * w;
    acc[3] += w;
}

template <typename Idx>
__global__ void __launch_bounds__(kBlendThreads) atrous_blend_tiled_kernel(
    const float* __restrict__ src, const float* __restrict__ nrm, const float* __restrict__ pos,
    const float* __restrict__ dif, uint32_t W, uint32_t H, int s, const float* __restrict__ stats,
    const float2* __restrict__ range, float* __restrict__ dst)
{
    __shared__ float4 rec[kFootY * kFootX * 3];   // [row][column parity][column / 2] records
    const int rx = (int)(blockIdx.x % (uint32_t)s), tx = (int)(blockIdx.x / (uint32_t)s);
    const int ry = (int)(blockIdx.y % (uint32_t)s), ty = (int)(blockIdx.y / (uint32_t)s);
    const int lx0 = tx * kLatX - 2, ly0 = ty * kLatY - 2;   // lattice coordinate of footprint entry (0, 0)
    for (int e = threadIdx.x; e < kFootX * kFootY; e += blockDim.x) {
        const int ex = e % kFootX, ey = e / kFootX;
        const int x = clampi(rx + (lx0 + ex) * s, 0, (int)W - 1);
        const int y = clampi(ry + (ly0 + ey) * s, 0, (int)H - 1);
        const Idx f = ((Idx)y * W + (Idx)x) * 3;
        const int slot = 3 * ((ey * 2 + (ex & 1)) * kHalfX + (ex >> 1));
        rec[slot] = make_float4(__ldg(nrm + f), __ldg(nrm + f + 1), __ldg(nrm + f + 2), __ldg(pos + f));
        rec[slot + 1] = make_float4(__ldg(pos + f + 1), __ldg(pos + f + 2), __ldg(dif + f), __ldg(dif + f + 1));
        rec[slot + 2] = make_float4(__ldg(dif + f + 2), __ldg(src + f), __ldg(src + f + 1), __ldg(src + f + 2));
    }
    __syncthreads();
    const int h = (int)(threadIdx.x % (kLatX / 2)), b = (int)(threadIdx.x / (kLatX / 2));
    const int a = 2 * h;                                     // this thread's lattice pixels: a and a + 1
    const int y = ry + (ty * kLatY + b) * s;
    const int x0 = rx + (tx * kLatX + a) * s, x1 = x0 + s;
    if (y >= (int)H || x0 >= (int)W) return;
    const int tiles_x = (int)((W + kTile - 1) / kTile);
    const int x1c = x1 < (int)W ? x1 : x0;
    const float2 st0 = tile_stats(stats, range, (y / kTile) * tiles_x + x0 / kTile);
    const float2 st1 = tile_stats(stats, range, (y / kTile) * tiles_x + x1c / kTile);
    const float ip0 = __frcp_rn(__fmul_rn(st0.y, st0.y)), iw0 = __frcp_rn(__fmul_rn(st0.x, st0.x));
    const float ip1 = __frcp_rn(__fmul_rn(st1.y, st1.y)), iw1 = __frcp_rn(__fmul_rn(st1.x, st1.x));
    float c0[9], c1[9];
    {
        const int r0 = 3 * (((b + 2) * 2 + 0) * kHalfX + h + 1);   // column a + 2 (even)
        const int r1 = 3 * (((b + 2) * 2 + 1) * kHalfX + h + 1);   // column a + 3 (odd)
        const float4 p0 = rec[r0], p1 = rec[r0 + 1], p2 = rec[r0 + 2];
        const float4 q0 = rec[r1], q1 = rec[r1 + 1], q2 = rec[r1 + 2];
        c0[0] = p0.x; c0[1] = p0.y; c0[2] = p0.z; c0[3] = p0.w; c0[4] = p1.x; c0[5] = p1.y;
        c0[6] = p1.z; c0[7] = p1.w; c0[8] = p2.x;
        c1[0] = q0.x; c1[1] = q0.y; c1[2] = q0.z; c1[3] = q0.w; c1[4] = q1.x; c1[5] = q1.y;
        c1[6] = q1.z; c1[7] = q1.w; c1[8] = q2.x;
    }
    float acc0[4] = {0.0f, 0.0f, 0.0f, 0.0f}, acc1[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int j = 0; j < 5; ++j) {
#pragma unroll
        for (int q = 0; q < 6; ++q) {   // footprint column a + q
            const int r = 3 * (((b + j) * 2 + (q & 1)) * kHalfX + h + (q >> 1));
            const float4 t0 = rec[r], t1 = rec[r + 1], t2 = rec[r + 2];
            if (q <= 4) blend_tap(t0, t1, t2, kAtrousWeights[j * 5 + q], c0, ip0, iw0, acc0);
            if (q >= 1) blend_tap(t0, t1, t2, kAtrousWeights[j * 5 + q - 1], c1, ip1, iw1, acc1);
        }
    }
    const Idx o0 = ((Idx)y * W + (Idx)x0) * 3;
    dst[o0] = __fdiv_rn(acc0[0], acc0[3]);
    dst[o0 + 1] = __fdiv_rn(acc0[1], acc0[3]);
    dst[o0 + 2] = __fdiv_rn(acc0[2], acc0[3]);
    if (x1 < (int)W) {
        const Idx o1 = ((Idx)y * W + (Idx)x1) * 3;
        dst[o1] = __fdiv_rn(acc1[0], acc1[3]);
        dst[o1 + 1] = __fdiv_rn(acc1[1], acc1[3]);
        dst[o1 + 2] = __fdiv_rn(acc1[2], acc1[3]);
    }
}

// Spacings up to this use the tiled blend; wider ones gather their staged lattice
// points from scattered sectors and run faster as the direct kernel.
constexpr int kTiledMaxSpacing = 4;

cudaError_t launch_atrous(const float* pixels, const float* normals, const float* positions, const float* diffuse,
                          uint32_t W, uint32_t H, float* scratch_a, float* scratch_b, float* tile_stats, float* out,
                          cudaStream_t st)
{
    if (W == 0 || H == 0) return cudaSuccess;
    const uint32_t tiles = ((W + kTile - 1) / kTile) * ((H + kTile - 1) / kTile);
    // scratch (atrous_stats_floats): per tile kStatsSplit white-point partials, then five
    // (min, max) |position| ranges per tile, then five (min, max) per image row and tile column
    float* parts = tile_stats;
    float2* range = reinterpret_cast<float2*>(tile_stats + (size_t)tiles * kStatsSplit);
    float2* rrow = range + (size_t)5 * tiles;
    const uint32_t tiles_x = (W + kTile - 1) / kTile;
    const uint64_t row_tasks = (uint64_t)H * tiles_x;
    atrous_row_range_kernel<<<(unsigned)((row_tasks + kRowWarps - 1) / kRowWarps), 32 * kRowWarps, 0, st>>>(
        positions, W, H, rrow);
    atrous_tile_range_kernel<<<tiles, 32 * 5, 0, st>>>(rrow, W, H, range);
    const float* src = pixels;
    for (int level = 0; level < 5; ++level) {
        // ping-pong: in -> A -> B -> A -> B -> out
        float* dst = level == 4 ? out : ((level % 2 == 0) ? scratch_a : scratch_b);
        const int s = 1 << level;
        const float2* lrange = range + (size_t)level * tiles;
        atrous_stats_kernel<<<tiles * kStatsSplit, kStatsThreads, 0, st>>>(src, W, H, s, parts);
        const bool small = (uint64_t)W * H * 3 < (1ull << 32);
        if (s <= kTiledMaxSpacing) {
            // one CTA per kLatX x kLatY tile of each of the s x s sub-lattices
            const uint32_t lw = (W + s - 1) / s, lh = (H + s - 1) / s;
            dim3 grid(((lw + kLatX - 1) / kLatX) * s, ((lh + kLatY - 1) / kLatY) * s);
            if (small)
                atrous_blend_tiled_kernel<uint32_t><<<grid, kBlendThreads, 0, st>>>(src, normals, positions, diffuse,
                                                                                   W, H, s, parts, lrange, dst);
            else
                atrous_blend_tiled_kernel<size_t><<<grid, kBlendThreads, 0, st>>>(src, normals, positions, diffuse, W,
                                                                                 H, s, parts, lrange, dst);
        } else {
            dim3 grid((W + 255) / 256, H);
            if (small)
                atrous_blend_kernel<uint32_t><<<grid, 256, 0, st>>>(src, normals, positions, diffuse, W, H, s, parts,
                                                                    lrange, dst);
            else
                atrous_blend_kernel<size_t><<<grid, 256, 0, st>>>(src, normals, positions, diffuse, W, H, s, parts,
                                                                  lrange, dst);
        }
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
