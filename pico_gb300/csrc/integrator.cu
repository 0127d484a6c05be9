// Wavefront path tracer reproducing Monte_Carlo_Integrator (Render/Integrators.cpp:46-209)
// and the per-pixel sample loop of Scene::render_scene_to_memory (Core/Scene.cpp:164-198).
//
// A batch holds `npix` pixels x `spb` samples, one path per thread slot, with
// the path state in structure-of-arrays form in HBM.  Per bounce depth:
//   extend   closest hit for every queued path (traverse.cuh) and, in the
//            same launch, the NEE shadow rays the previous shade queued (a
//            light hit adds its radiance)
//   shade    BSRDF sample, emission, NEE setup, Russian roulette, next ray;
//            survivors and shadow rays are appended to queues with one
//            atomic per block and queue (block_append)
// then `accumulate` takes each payload as a sample value (NaN/Inf -> pink, as
// Integrators.cpp:145-146) and applies the reference's running mean / variance
// and early-exit rule per pixel, samples in order.
//
// The estimator is the reference's, including its non-physical choices: the
// NEE term is throughput * bsdf_pdf(L) * Le * albedo with no light pdf, any
// light hit by the shadow ray counts, Russian roulette runs from depth 0 with
// survival max(throughput), throughput is multiplied by the sample pdf, and
// rays leave surfaces 0.01 along the normal (or the light direction).
//
// The physical estimator (PICO_ESTIMATOR_PHYSICAL, physical.cuh) shares the
// batch, queues and extension kernels and replaces shade and the running mean.
#include "kernels_render.h"
#include "physical.cuh"
#include "shade.cuh"
#include "traverse.cuh"

namespace pico {

constexpr int kRenderThreads = 256;
// Resident blocks the shade kernels are compiled for: 4 (64 registers, a few spilled) against
// the 3 their natural 76-83 registers allow measured 1080p renders 0.4 % (reference
// estimator) and 1.7 % (physical) faster, with identical images.
constexpr int kShadeBlocksPerSm = 4;

__device__ __forceinline__ uint32_t warp_append(bool take, uint32_t* counter)
{
    const unsigned lane = threadIdx.x & 31u;
    const unsigned mask = __ballot_sync(0xffffffffu, take);
    uint32_t base = 0;
    if (lane == (unsigned)(__ffs(mask) - 1) && mask) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, mask ? __ffs(mask) - 1 : 0);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

// Queue appends with one atomic per block and queue (a same-address atomic per warp
// measured as the bound of raygen): each warp's count from a ballot, a prefix over
// the block's warps in shared memory, one atomicAdd per queue by one thread.  Every
// thread of the block calls it once per round of a loop whose round count is the same
// for the whole grid (it synchronises the block); blocks of kRenderThreads threads.
// The scratch alternates between rounds, so a round's writes never meet the previous
// round's reads.
struct AppendScratch {
    uint32_t warp_base[2][2][kRenderThreads / 32];   // [round parity][queue][warp]
    uint32_t base[2][2];
};

__device__ __forceinline__ void block_append(uint32_t round, bool a, uint32_t* counter_a, bool b, uint32_t* counter_b,
                                             AppendScratch& sh, uint32_t& at_a, uint32_t& at_b)
{
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const int par = (int)(round & 1u);
    const unsigned ma = __ballot_sync(0xffffffffu, a), mb = __ballot_sync(0xffffffffu, b);
    if (lane == 0) {
        sh.warp_base[par][0][warp] = (uint32_t)__popc(ma);
        sh.warp_base[par][1][warp] = (uint32_t)__popc(mb);
    }
    __syncthreads();
    if (threadIdx.x < 2) {
        const int q = (int)threadIdx.x;
        uint32_t total = 0;
        for (int w = 0; w < kRenderThreads / 32; ++w) {
            const uint32_t c = sh.warp_base[par][q][w];
            sh.warp_base[par][q][w] = total;
            total += c;
        }
        uint32_t* counter = q ? counter_b : counter_a;
        sh.base[par][q] = (total && counter) ? atomicAdd(counter, total) : 0u;
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
    at_a = sh.base[par][0] + sh.warp_base[par][0][warp] + (uint32_t)__popc(ma & below);
    at_b = sh.base[par][1] + sh.warp_base[par][1][warp] + (uint32_t)__popc(mb & below);
}

__global__ void __launch_bounds__(kRenderThreads) raygen_kernel(PathBatch b, CameraView cam, unsigned long long seed,
                                                               bool physical)
{
    __shared__ AppendScratch app;
    // whole blocks iterate together so the queue append can use block collectives
    const uint32_t n = b.plan ? b.plan->n : b.n, npix = b.plan ? b.plan->npix : b.npix;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t i = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool live = false;
        uint32_t pixel = 0, s = 0;
        if (i < n) {
            const uint32_t slot = i % npix;
            s = i / npix;
            pixel = b.pix_list[slot];
            live = b.done[pixel] == 0;
        }
        // a finished pixel's slots get no path: nothing reads their state
        if (live) {
            Pcg32 rng = path_rng(seed, pixel, b.count[pixel] + s);
            float x0, x1;
            if (physical) {
                // camera_ray halves its jitter (Camera.cpp:14-15): this covers the whole pixel
                x0 = 2.0f * rng.uniform();
                x1 = 2.0f * rng.uniform();
            } else {
                hammersley(rng, x0, x1);
            }
            float4 o, d;
            camera_ray(cam, x0, x1, pixel % b.width, pixel / b.width, o, d);
            b.org[i] = o;
            b.dir[i] = d;
            b.thr[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            b.pay[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            b.rng[i] = rng.state;
            b.depth[i] = 0;
            b.ior_n[i] = 1;   // Camera::generate_ray pushes 1.0 (Core/Camera.cpp:23)
            b.ior_lo[i] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
        }
        uint32_t at, unused;
        block_append(r, live, &b.counters[0], false, nullptr, app, at, unused);
        if (live) b.queue[0][at] = i;
    }
}

// Stores a path segment's hit, or adds what a shadow ray delivers.
__device__ __forceinline__ void extend_finish(const SceneView& sc, PathBatch& b, uint32_t i, const TraceHit& h,
                                              int s, bool shadow)
{
    const uint32_t rank = (s == kTraceOk) ? h.rank : kNoHit;
    if (shadow) {
        // a light hit adds (throughput * pdf) * Le * albedo (Integrators.cpp:109-117, 173-176);
        // a sun ray (senergy.w = 1) adds the sun colour when it escapes (Integrators.cpp:60-76)
        const float4 e = b.senergy[i];
        const float* le = nullptr;
        if (e.w != 0.0f) {
            if (rank == kNoHit && s == kTraceOk) le = sc.sun_col;
        } else if (rank != kNoHit) {
            const GpuInstanceShade is = sc.inst_shade[sc.insts[rank].inst_id];
            if (is.bsdf == PICO_BSDF_LIGHT) le = sc.materials[is.material].emissive;
        }
        if (le) {
            const float4 c = b.scontrib[i];
            float4 p = b.pay[i];
            p.x = p.x + (c.x * le[0]) * e.x;
            p.y = p.y + (c.y * le[1]) * e.y;
            p.z = p.z + (c.z * le[2]) * e.z;
            b.pay[i] = p;
        }
    } else {
        b.hit[i] = make_float4(h.t, h.u, h.v, __uint_as_float(rank));
        b.hit_tri[i] = h.tri;
    }
}

// The entries of an extension launch for walk_queue: the depth's path segments
// q[0, n0), then the shadow rays sq[0, n - n0); a lane's tag is its path index
// with the ray's kind in the top two bits (0 segment, 1 shadow ray, 2 occlusion
// query of the physical estimator).
struct ExtendRays {
    using Tag = uint32_t;
    using Index = uint32_t;   // at most 2^26 segments and 2^26 shadow rays
    const SceneView& sc;
    PathBatch& b;
    const uint32_t* q;
    const uint32_t* sq;
    uint32_t n0;
    int* err;

    __device__ __forceinline__ uint32_t load(uint32_t k, float4& o, float4& d, float& tmax, float& exit_below,
                                             bool& occlusion) const
    {
        const bool shadow = k >= n0;
        const uint32_t i = shadow ? sq[k - n0] : q[k];
        uint32_t kind = 0;
        tmax = INFINITY;
        exit_below = -INFINITY;
        occlusion = false;
        if (shadow) {
            o = b.sorg[i];
            d = b.sdir[i];
            const float ew = b.senergy[i].w;
            if (ew == 2.0f) {
                // physical estimator: an occlusion query bounded by the light sample's distance
                kind = 2;
                tmax = b.scontrib[i].w;
                occlusion = true;
            } else {
                // only whether the closest hit is a light (or, for a sun ray, nothing)
                // counts: the walk may stop at a hit nearer than every light
                kind = 1;
                exit_below = ew != 0.0f ? INFINITY : light_distance_bound(sc, o);
            }
        } else {
            o = b.org[i];
            d = b.dir[i];
        }
        return i | (kind << 30);
    }

    __device__ __forceinline__ void finish(uint32_t tag, const TraceHit& h, int s) const
    {
        const uint32_t i = tag & 0x3fffffffu, kind = tag >> 30;
        if (s != kTraceOk) atomicOr(err, s);
        if (kind == 2) {
            if (s == kTraceOk && h.tri == kNoHit) {
                const float4 c = b.scontrib[i];
                float4 p = b.pay[i];
                p.x += c.x; p.y += c.y; p.z += c.z;
                b.pay[i] = p;
            }
        } else {
            extend_finish(sc, b, i, h, s, kind == 1);
        }
    }
};

// Persistent: in the near-first order the warps walk the launch's entries with
// walk_queue (idle lanes refilled in batches); in the reference order each warp
// takes 32 entries at a time and each lane runs its ray to completion.  One
// launch traces two queues back to back: the paths' next segments q[0, *count)
// and, when sq is given, the shadow rays sq[0, *scount) the previous shade left
// (they write disjoint path fields and both finish before the next shade), so a
// depth pays one launch and one tail.  kThreads per CTA (64, 128 or 256): the
// block shape batched renders tune; the register budget is the same for every
// shape: 1024 threads (64 registers) per SM in the near-first order, where against
// 896 threads at 72 registers the 1080p renders measured 2 % faster with identical
// images (the extra warps hide more latency than the few spilled registers cost),
// and 896 threads in the reference's order, which spills more at 64.  kCount: the
// same traversal, also adding its work (nodes, triangles, instance entries) to
// `counters` (measurement only).
template <int kOrder>
constexpr int extend_threads_per_sm() { return (kOrder & kReferenceOrder) ? 896 : 1024; }
template <int kOrder, int kThreads, bool kCount = false>
__global__ void __launch_bounds__(kThreads, extend_threads_per_sm<kOrder>() / kThreads) extend_kernel(SceneView sc, PathBatch b, const uint32_t* q,
                                                       const uint32_t* count, const uint32_t* sq,
                                                       const uint32_t* scount, unsigned long long* work, int* err,
                                                       unsigned long long* tally, unsigned long long* stally,
                                                       unsigned long long* counters)
{
    TraceCounters cnt{0, 0, 0, 0};
    const unsigned lane = threadIdx.x & 31u;
    const uint32_t n0 = *count, n1 = sq ? *scount : 0u;
    const uint64_t n = (uint64_t)n0 + n1;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        atomicAdd(tally, (unsigned long long)n0);
        if (sq) atomicAdd(stally, (unsigned long long)n1);
    }
    if constexpr ((kOrder & kReferenceOrder) == 0) {
        ExtendRays rays{sc, b, q, sq, n0, err};
        walk_queue<kCount, (kOrder & kWithImplicit) != 0, (kOrder & kBounded) != 0, (kOrder & kWatertight) != 0>(
            sc, rays, (uint32_t)n, work, &cnt);
    } else {
        // the reference order: each lane runs its ray to completion, 32 rays per warp fetch
        for (;;) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(work, 32ull);
            base = __shfl_sync(0xffffffffu, base, 0);
            if (base >= n) break;
            const unsigned long long k = base + lane;
            if (k < n) {
                const bool shadow = k >= n0;
                const uint32_t i = shadow ? sq[k - n0] : q[k];
                if (shadow && b.senergy[i].w == 2.0f) {
                    // physical estimator: an occlusion query bounded by the light sample's distance
                    const float4 c = b.scontrib[i];
                    bool occluded = true;
                    const int s = trace_occluded<kOrder, kCount>(sc, b.sorg[i], b.sdir[i], c.w, occluded, &cnt);
                    if (s != kTraceOk) atomicOr(err, s);
                    if (s == kTraceOk && !occluded) {
                        float4 p = b.pay[i];
                        p.x += c.x; p.y += c.y; p.z += c.z;
                        b.pay[i] = p;
                    }
                } else {
                    // the reference order walks every shadow ray to its closest hit
                    TraceHit h;
                    const int s = trace_closest<kCount, kOrder>(sc, shadow ? b.sorg[i] : b.org[i],
                                                                shadow ? b.sdir[i] : b.dir[i], h, &cnt);
                    if (s != kTraceOk) atomicOr(err, s);
                    extend_finish(sc, b, i, h, s, shadow);
                }
            }
        }
    }
    if (kCount) flush_counters(cnt, counters);
}

__global__ void __launch_bounds__(kRenderThreads, kShadeBlocksPerSm) shade_kernel(SceneView sc, PathBatch b, int cur, uint32_t depth,
                                                              uint32_t max_depth, bool trace_last)
{
    __shared__ AppendScratch app;
    const uint32_t n = b.counters[cur];
    const uint32_t nxt = cur ^ 1;
    // whole blocks iterate together so the queue appends can use block collectives
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t k = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool cont = false, shadow = false;
        uint32_t i = 0;
        if (k < n) {
            i = b.queue[cur][k];
            const float4 hit = b.hit[i];
            const uint32_t rank = __float_as_uint(hit.w);
            float4 thr = b.thr[i], pay = b.pay[i];
            const float4 dir = b.dir[i];
            if (rank == kNoHit) {
                // sky on a miss (Integrators.cpp:152, 208)
                const float3 sk = sky_radiance(sc, dir.x, dir.y, dir.z);
                pay.x = ex::add(pay.x, ex::mul(thr.x, sk.x));
                pay.y = ex::add(pay.y, ex::mul(thr.y, sk.y));
                pay.z = ex::add(pay.z, ex::mul(thr.z, sk.z));
                b.pay[i] = pay;
            } else if (depth < max_depth) {
                Pcg32 rng{b.rng[i]};
                const Fragment f = make_fragment(sc, rank, b.hit_tri[i], hit.y, hit.z, b.org[i], dir);
                const GpuInstanceShade is = sc.inst_shade[f.inst];
                const GpuMaterial m = sc.materials[is.material];
                const ex::V3 V = ex::v3(-dir.x, -dir.y, -dir.z);
                auto next_xi = [&](float& a, float& c) { hammersley(rng, a, c); };
                // the path's index-of-refraction stack; only the BTDF lobes change it
                const bool btdf = is.bsdf == PICO_BSDF_BTDF || is.bsdf == PICO_BSDF_FRESNEL;
                IorStack ior;
                ior.n = b.ior_n[i];
                if (btdf) {
                    const float4 lo = b.ior_lo[i], hi = b.ior_hi[i];
                    ior.v[0] = lo.x; ior.v[1] = lo.y; ior.v[2] = lo.z; ior.v[3] = lo.w;
                    ior.v[4] = hi.x; ior.v[5] = hi.y; ior.v[6] = hi.z; ior.v[7] = hi.w;
                }
                const BsdfSample smp = sample_bsdf(is.bsdf, m, V, f.n, next_xi, ior);
                if (btdf) {
                    b.ior_n[i] = ior.n;
                    b.ior_lo[i] = make_float4(ior.v[0], ior.v[1], ior.v[2], ior.v[3]);
                    b.ior_hi[i] = make_float4(ior.v[4], ior.v[5], ior.v[6], ior.v[7]);
                }
                if (is.bsdf == PICO_BSDF_LIGHT) {
                    pay.x = pay.x + thr.x * smp.energy.x;
                    pay.y = pay.y + thr.y * smp.energy.y;
                    pay.z = pay.z + thr.z * smp.energy.z;
                }
                // next-event estimation towards one uniformly chosen light, the sun
                // counting as the last one (Integrators.cpp:54-76)
                const uint32_t nl = sc.nlights + (sc.use_sun ? 1u : 0u);
                uint32_t li = nl;
                if (is.bsdf != PICO_BSDF_LIGHT && !btdf && nl > 0) {
                    li = (uint32_t)(rng.uniform() * (float)nl);
                    if (li >= nl) li = nl - 1;
                }
                if (sc.use_sun && li == nl - 1) {
                    const ex::V3 ts = ex::v3(-sc.sun_dir[0], -sc.sun_dir[1], -sc.sun_dir[2]);
                    const float pdf = direct_lighting_pdf(is.bsdf, m, f.n, V, ts);
                    b.sorg[i] = make_float4(f.px + 0.01f * ts.x, f.py + 0.01f * ts.y, f.pz + 0.01f * ts.z,
                                            f.pw + 0.0f);
                    b.sdir[i] = make_float4(ts.x, ts.y, ts.z, 10000.0f);
                    b.scontrib[i] = make_float4(thr.x * pdf, thr.y * pdf, thr.z * pdf, 0.0f);
                    b.senergy[i] = make_float4(smp.energy.x, smp.energy.y, smp.energy.z, 1.0f);
                    shadow = true;
                } else if (li < sc.nlights) {
                    const GpuLight L = sc.lights[li];
                    float sx, sy, sz;
                    if (L.shape != PICO_SHAPE_TRIANGLES) {
                        implicit_light_point(L.shape, rng, sx, sy, sz);
                    } else {
                        const uint32_t bucket = rng.next() % L.ntris;
                        const float coin = (float)rng.next() / 4294967296.0f;
                        const uint32_t t = coin <= sc.light_alias_weight[L.tri_base + bucket]
                                               ? bucket
                                               : sc.light_alias_index[L.tri_base + bucket];
                        float x0, x1;
                        hammersley(rng, x0, x1);
                        const float su0 = ex::sqrt_(x0);
                        const float bx = 1.0f - su0, by = x1 * su0;
                        const float* lp = sc.light_positions + 9 * (size_t)(L.tri_base + t);
                        const float w0 = (1.0f - bx) - by;
                        sx = (w0 * lp[0] + bx * lp[3]) + by * lp[6];
                        sy = (w0 * lp[1] + bx * lp[4]) + by * lp[7];
                        sz = (w0 * lp[2] + bx * lp[5]) + by * lp[8];
                    }
                    const float4* lip = reinterpret_cast<const float4*>(sc.insts + sc.inst_rank[L.inst]);
                    const float4 r0 = __ldg(lip + 3), r1 = __ldg(lip + 4), r2 = __ldg(lip + 5);
                    const ex::V3 spw = ex::v3(ex::row4(r0, sx, sy, sz, 1.0f), ex::row4(r1, sx, sy, sz, 1.0f),
                                              ex::row4(r2, sx, sy, sz, 1.0f));
                    const ex::V3 tl = ex::normalize(ex::v3(spw.x - f.px, spw.y - f.py, spw.z - f.pz));
                    if (!(ex::dot(tl, f.n) < 0.0f)) {
                        const float pdf = direct_lighting_pdf(is.bsdf, m, f.n, V, tl);
                        b.sorg[i] = make_float4(f.px + 0.01f * tl.x, f.py + 0.01f * tl.y, f.pz + 0.01f * tl.z,
                                                f.pw + 0.0f);
                        b.sdir[i] = make_float4(tl.x, tl.y, tl.z, 10000.0f);
                        b.scontrib[i] = make_float4(thr.x * pdf, thr.y * pdf, thr.z * pdf, 0.0f);
                        b.senergy[i] = make_float4(smp.energy.x, smp.energy.y, smp.energy.z, 0.0f);
                        shadow = true;
                    }
                }
                b.pay[i] = pay;
                if (smp.P != 0.0f) {
                    // Russian roulette with survival max(throughput) (Integrators.cpp:185-193)
                    const float q = ex::smax(ex::smax(thr.x, thr.y), thr.z);
                    if (!(rng.uniform() > q)) {
                        const float iq = 1.0f / q;
                        thr.x = (thr.x * iq) * (smp.P * smp.energy.x);
                        thr.y = (thr.y * iq) * (smp.P * smp.energy.y);
                        thr.z = (thr.z * iq) * (smp.P * smp.energy.z);
                        b.thr[i] = thr;
                        // offset along N, or -N inside a transparent object (Integrators.cpp:199)
                        const float sgn = ior.inside() ? -0.01f : 0.01f;
                        b.org[i] = make_float4(f.px + sgn * f.n.x, f.py + sgn * f.n.y, f.pz + sgn * f.n.z,
                                               f.pw + 0.0f);
                        b.dir[i] = make_float4(smp.L.x, smp.L.y, smp.L.z, dir.w);
                        b.depth[i] = depth + 1;
                        // the ray after the last shaded vertex can only add sky radiance
                        const bool finite = isfinite(thr.x) && isfinite(thr.y) && isfinite(thr.z);
                        cont = depth + 1 < max_depth || trace_last || !finite;
                    }
                }
                b.rng[i] = rng.state;
            }
        }
        uint32_t at, sat;
        block_append(r, cont, &b.counters[nxt], shadow, &b.counters[2], app, at, sat);
        if (cont) b.queue[nxt][at] = i;
        if (shadow) b.shadow_queue[sat] = i;
    }
}

// The physical estimator's shade step.  Path state: thr.w is the density with
// which the current ray's direction was sampled (0 for camera rays and mirror
// bounces, whose emission is not weighted); a shadow record carries its finished
// contribution in scontrib.xyz, the distance from which a hit no longer occludes
// in scontrib.w, and senergy.w = 2.
// The radiance-cache query of a shading point (pico_nrc_query layout): position,
// direction towards the viewer, shading normal, roughness, albedo (diffuse +
// specular colour, at most 1), the path index as payload.
__device__ __forceinline__ void nrc_query(const Fragment& f, float3 nrm, float3 v, const GpuMaterial& m,
                                          uint32_t kind, uint32_t path, float4 (&q)[4])
{
    float a[3];
    if (kind == PICO_BSDF_DELTA) {
        for (int c = 0; c < 3; ++c) a[c] = m.specular[c];
    } else {
        const phys::Lobes lb = phys::lobes_of(kind, m);
        a[0] = lb.diffuse.x + lb.f0.x; a[1] = lb.diffuse.y + lb.f0.y; a[2] = lb.diffuse.z + lb.f0.z;
    }
    for (int c = 0; c < 3; ++c) a[c] = fminf(fmaxf(a[c], 0.0f), 1.0f);
    q[0] = make_float4(f.px, f.py, f.pz, v.x);
    q[1] = make_float4(v.y, v.z, nrm.x, nrm.y);
    q[2] = make_float4(nrm.z, kind == PICO_BSDF_DELTA ? 0.0f : m.roughness, a[0], a[1]);
    q[3] = make_float4(a[2], __uint_as_float(path), 0.0f, 0.0f);
}

__global__ void __launch_bounds__(kRenderThreads, kShadeBlocksPerSm) shade_physical_kernel(SceneView sc, PathBatch b, int cur,
                                                                       uint32_t depth, uint32_t max_depth,
                                                                       NrcShadeArgs nrc)
{
    using namespace phys;
    __shared__ AppendScratch app;
    const uint32_t n = b.counters[cur];
    const uint32_t nxt = cur ^ 1;
    const uint32_t nl = sc.nlights + (sc.use_sun ? 1u : 0u);
    const float4* light_geo = reinterpret_cast<const float4*>(sc.light_tri_geo);
    // whole blocks iterate together so the queue appends can use block collectives
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (n + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t k = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        bool cont = false, shadow = false, emit = false;
        float4 eq[4], et = make_float4(0.0f, 0.0f, 0.0f, 0.0f), ep = et;   // radiance-cache entry
        uint32_t i = 0;
        if (k < n) {
            i = b.queue[cur][k];
            const float4 hit = b.hit[i];
            const uint32_t rank = __float_as_uint(hit.w);
            float4 thr = b.thr[i], pay = b.pay[i];
            const float4 dir = b.dir[i];
            const bool terminal = nrc.mode == kNrcTerminate && rank != kNoHit &&
                                  (depth > nrc.bounces || (depth == nrc.bounces && nrc.prev_rough[i] >= 0.1f));
            if (rank == kNoHit) {
                const float3 sk = sky_radiance(sc, dir.x, dir.y, dir.z);
                pay.x += thr.x * sk.x; pay.y += thr.y * sk.y; pay.z += thr.z * sk.z;
                b.pay[i] = pay;
            } else if (terminal && sc.inst_shade[sc.insts[rank].inst_id].bsdf != PICO_BSDF_LIGHT) {
                // the path ends here in the radiance cache: query what this point reflects towards v
                const uint32_t inst = sc.insts[rank].inst_id;
                const GpuInstanceShade is = sc.inst_shade[inst];
                const GpuMaterial m = sc.materials[is.material];
                const Fragment f = make_fragment(sc, rank, b.hit_tri[i], hit.y, hit.z, b.org[i], dir);
                float3 nrm = normalize3(make_float3(f.n.x, f.n.y, f.n.z));
                const float3 v = make_float3(-dir.x, -dir.y, -dir.z);
                if (dot3(nrm, v) < 0.0f) nrm = make_float3(-nrm.x, -nrm.y, -nrm.z);
                nrc_query(f, nrm, v, m, is.bsdf, i, eq);
                emit = true;
            } else {
                const uint32_t inst = sc.insts[rank].inst_id;
                const GpuInstanceShade is = sc.inst_shade[inst];
                const GpuMaterial m = sc.materials[is.material];
                if (is.bsdf == PICO_BSDF_LIGHT) {
                    // emission, weighted against the light sample that could have reached this point
                    float w = 1.0f;
                    const uint32_t li = sc.light_of_inst[inst];
                    const uint32_t tri = b.hit_tri[i];
                    if (thr.w > 0.0f && li != ~0u && tri != kImplicitTri &&
                        sc.lights[li].shape == PICO_SHAPE_TRIANGLES) {
                        const float4 g = light_geo[sc.lights[li].tri_base + sc.tris[tri].prim];
                        const float cl = fabsf(g.x * dir.x + g.y * dir.y + g.z * dir.z);
                        const float pick = sc.light_pick[nl + li];
                        const float pl = g.w * hit.x * hit.x * pick / cl;   // +inf at cl = 0
                        w = mis_weight(thr.w, pl);
                    }
                    pay.x += thr.x * m.emissive[0] * w;
                    pay.y += thr.y * m.emissive[1] * w;
                    pay.z += thr.z * m.emissive[2] * w;
                    b.pay[i] = pay;
                } else if (depth < max_depth) {
                    Pcg32 rng{b.rng[i]};
                    const Fragment f = make_fragment(sc, rank, b.hit_tri[i], hit.y, hit.z, b.org[i], dir);
                    float3 nrm = normalize3(make_float3(f.n.x, f.n.y, f.n.z));
                    const float3 v = make_float3(-dir.x, -dir.y, -dir.z);
                    const bool front = !(dot3(nrm, v) < 0.0f);   // the viewer on the side the normal points to
                    if (!front) nrm = make_float3(-nrm.x, -nrm.y, -nrm.z);
                    if (nrc.mode == kNrcRecord) {
                        nrc_query(f, nrm, v, m, is.bsdf, i, eq);
                        et = thr;
                        ep = pay;
                        emit = true;
                    } else if (nrc.mode == kNrcTerminate) {
                        nrc.prev_rough[i] = is.bsdf == PICO_BSDF_DELTA ? 0.0f : m.roughness;   // a mirror is glossy
                    }
                    const float eps = ray_offset(f.px, f.py, f.pz);
                    float4 org = make_float4(f.px + eps * nrm.x, f.py + eps * nrm.y, f.pz + eps * nrm.z, f.pw);
                    float3 L, weight;
                    float pdf_next = 0.0f;
                    bool ok;
                    if (is.bsdf == PICO_BSDF_DELTA) {
                        // a mirror with Schlick reflectance; its emission is not weighted
                        const float c = dot3(nrm, v);
                        L = make_float3(2.0f * c * nrm.x - v.x, 2.0f * c * nrm.y - v.y, 2.0f * c * nrm.z - v.z);
                        weight = make_float3(schlick(m.specular[0], c), schlick(m.specular[1], c),
                                             schlick(m.specular[2], c));
                        ok = c > 0.0f;
                    } else if (is.bsdf == PICO_BSDF_BTDF || is.bsdf == PICO_BSDF_FRESNEL) {
                        // a rough dielectric interface between air and the material (entered where
                        // the viewer is on the normal's side); no next-event estimation, so the
                        // emission the continuation meets is not weighted
                        const Frame fr = frame_of(nrm);
                        const float ior = m.ior > 0.0f ? m.ior : 1.0f;
                        const float u0 = rng.uniform(), u1 = rng.uniform(), u2 = rng.uniform();
                        const DielectricSample ds =
                            sample_dielectric(to_local(fr, v), fmaxf(m.roughness * m.roughness, kMinAlpha),
                                              front ? 1.0f / ior : ior,
                                              make_float3(m.diffuse[0], m.diffuse[1], m.diffuse[2]),
                                              is.bsdf == PICO_BSDF_FRESNEL, u0, u1, u2);
                        ok = ds.ok;
                        L = to_world(fr, ds.l);
                        weight = ds.weight;
                        if (ds.refracted) org = make_float4(f.px - eps * nrm.x, f.py - eps * nrm.y, f.pz - eps * nrm.z, f.pw);
                    } else {
                        const Frame fr = frame_of(nrm);
                        const float3 vl = to_local(fr, v);
                        const Lobes lb = lobes_of(is.bsdf, m);
                        // next-event estimation towards one light (the sun last), picked by the
                        // scene's power-proportional table
                        if (nl > 0) {
                            // the first slot whose cumulative share exceeds up (the last
                            // slot otherwise), by bisection over the non-decreasing table
                            const float up = rng.uniform();
                            uint32_t li = 0, hi = nl - 1;
                            while (li < hi) {
                                const uint32_t mid = (li + hi) >> 1;
                                if (up >= sc.light_pick[mid]) li = mid + 1;
                                else hi = mid;
                            }
                            const float pick = sc.light_pick[nl + li];
                            float3 wi = make_float3(0.0f, 0.0f, 0.0f), c = wi;
                            float reach = 0.0f;
                            if (sc.use_sun && li == nl - 1) {
                                wi = normalize3(make_float3(-sc.sun_dir[0], -sc.sun_dir[1], -sc.sun_dir[2]));
                                const float3 wl = to_local(fr, wi);
                                if (wl.z > 0.0f) {
                                    float3 fv;
                                    float pb;
                                    eval(lb, vl, wl, fv, pb);
                                    const float kk = wl.z / pick;
                                    c = make_float3(thr.x * fv.x * sc.sun_col[0] * kk, thr.y * fv.y * sc.sun_col[1] * kk,
                                                    thr.z * fv.z * sc.sun_col[2] * kk);
                                    reach = __int_as_float(0x7f800000);   // only an escaping ray sees the sun
                                    shadow = true;
                                }
                            } else if (sc.lights[li].shape == PICO_SHAPE_TRIANGLES) {
                                const GpuLight Lt = sc.lights[li];
                                const uint32_t bucket = rng.next() % Lt.ntris;
                                const float coin = (float)rng.next() / 4294967296.0f;
                                const uint32_t t = coin <= sc.light_alias_weight[Lt.tri_base + bucket]
                                                       ? bucket
                                                       : sc.light_alias_index[Lt.tri_base + bucket];
                                const float su0 = sqrtf(rng.uniform()), x1 = rng.uniform();
                                const float bx = 1.0f - su0, by = x1 * su0, w0 = 1.0f - bx - by;
                                const float* lp = sc.light_positions + 9 * (size_t)(Lt.tri_base + t);
                                const float sx = w0 * lp[0] + bx * lp[3] + by * lp[6];
                                const float sy = w0 * lp[1] + bx * lp[4] + by * lp[7];
                                const float sz = w0 * lp[2] + bx * lp[5] + by * lp[8];
                                const float4* lip = reinterpret_cast<const float4*>(sc.insts + sc.inst_rank[Lt.inst]);
                                const float4 r0 = __ldg(lip + 3), r1 = __ldg(lip + 4), r2 = __ldg(lip + 5);
                                const float yx = r0.x * sx + r0.y * sy + r0.z * sz + r0.w;
                                const float yy = r1.x * sx + r1.y * sy + r1.z * sz + r1.w;
                                const float yz = r2.x * sx + r2.y * sy + r2.z * sz + r2.w;
                                const float3 dd = make_float3(yx - org.x, yy - org.y, yz - org.z);
                                const float dist2 = dot3(dd, dd), dist = sqrtf(dist2);
                                wi = make_float3(dd.x / dist, dd.y / dist, dd.z / dist);
                                const float4 g = light_geo[Lt.tri_base + t];
                                const float cl = fabsf(g.x * wi.x + g.y * wi.y + g.z * wi.z);
                                const float3 wl = to_local(fr, wi);
                                if (wl.z > 0.0f && cl > 0.0f && g.w > 0.0f && dist > 0.0f) {
                                    const float pl = g.w * dist2 * pick / cl;
                                    float3 fv;
                                    float pb;
                                    eval(lb, vl, wl, fv, pb);
                                    const float kk = wl.z * mis_weight(pl, pb) / pl;
                                    const float* le = sc.materials[sc.inst_shade[Lt.inst].material].emissive;
                                    c = make_float3(thr.x * fv.x * le[0] * kk, thr.y * fv.y * le[1] * kk,
                                                    thr.z * fv.z * le[2] * kk);
                                    reach = dist * (1.0f - 1e-4f);
                                    shadow = true;
                                }
                            }
                            if (shadow) {
                                b.sorg[i] = org;
                                b.sdir[i] = make_float4(wi.x, wi.y, wi.z, 10000.0f);
                                b.scontrib[i] = make_float4(c.x, c.y, c.z, reach);
                                b.senergy[i] = make_float4(0.0f, 0.0f, 0.0f, 2.0f);
                            }
                        }
                        const float u0 = rng.uniform(), u1 = rng.uniform(), u2 = rng.uniform();
                        const Sample smp = phys::sample(lb, vl, u0, u1, u2);
                        ok = smp.ok;
                        L = to_world(fr, smp.l);
                        weight = smp.weight;
                        pdf_next = smp.pdf;
                    }
                    if (ok) {
                        thr.x *= weight.x; thr.y *= weight.y; thr.z *= weight.z;
                        bool live = true;
                        if (depth >= 3) {   // Russian roulette from the fourth vertex
                            const float q = fminf(0.95f, fmaxf(thr.x, fmaxf(thr.y, thr.z)));
                            live = rng.uniform() < q;
                            if (live) { thr.x /= q; thr.y /= q; thr.z /= q; }
                        }
                        if (!(isfinite(thr.x) && isfinite(thr.y) && isfinite(thr.z))) {
                            pay.x = __int_as_float(0x7fffffff);   // shows as pink
                            b.pay[i] = pay;
                            live = false;
                        }
                        if (live) {
                            thr.w = pdf_next;
                            b.thr[i] = thr;
                            b.org[i] = org;
                            b.dir[i] = make_float4(L.x, L.y, L.z, dir.w);
                            b.depth[i] = depth + 1;
                            cont = true;
                        }
                    }
                    b.rng[i] = rng.state;
                }
            }
        }
        uint32_t at, sat;
        block_append(r, cont, &b.counters[nxt], shadow, &b.counters[2], app, at, sat);
        if (cont) b.queue[nxt][at] = i;
        if (shadow) b.shadow_queue[sat] = i;
        if (nrc.mode != kNrcOff) {
            const uint32_t ea = warp_append(emit, nrc.count);
            if (emit && ea < nrc.capacity) {
                float4* q = nrc.queries + 4 * (size_t)ea;
                q[0] = eq[0]; q[1] = eq[1]; q[2] = eq[2]; q[3] = eq[3];
                if (nrc.mode == kNrcRecord) {
                    nrc.rec_tp[2 * (size_t)ea] = et;
                    nrc.rec_tp[2 * (size_t)ea + 1] = ep;
                }
            }
        }
    }
}

// Pixel-pseudo-random camera paths that train the radiance cache: path j of pass
// `frame` starts at a uniformly drawn pixel with a jitter over the whole pixel.
__global__ void __launch_bounds__(kRenderThreads) train_raygen_kernel(PathBatch b, CameraView cam,
                                                                     unsigned long long seed, uint32_t frame,
                                                                     uint32_t W, uint32_t npx)
{
    __shared__ AppendScratch app;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (b.n + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t i = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool live = i < b.n;
        if (live) {
            Pcg32 rng = path_rng(seed, i, frame);
            const uint32_t pixel = rng.next() % npx;
            const float x0 = 2.0f * rng.uniform(), x1 = 2.0f * rng.uniform();
            float4 o, d;
            camera_ray(cam, x0, x1, pixel % W, pixel / W, o, d);
            b.org[i] = o;
            b.dir[i] = d;
            b.thr[i] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
            b.pay[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            b.rng[i] = rng.state;
            b.depth[i] = 0;
        }
        uint32_t at, unused;
        block_append(r, live, &b.counters[0], false, nullptr, app, at, unused);
        if (live) b.queue[0][at] = i;
    }
}

// Target of each training record: (final payload - payload on arrival) / throughput
// on arrival, per channel (0 where the throughput is 0); NaN for a path whose
// payload is not finite, which training skips.
__global__ void __launch_bounds__(kRenderThreads) nrc_targets_kernel(const float4* __restrict__ queries,
                                                                    const float4* __restrict__ rec_tp,
                                                                    const float4* __restrict__ pay,
                                                                    const uint32_t* count, uint32_t capacity,
                                                                    float4* targets)
{
    const uint32_t n = min(*count, capacity);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t path = __float_as_uint(queries[4 * (size_t)j + 3].y);
        const float4 T = rec_tp[2 * (size_t)j], P = rec_tp[2 * (size_t)j + 1], F = pay[path];
        float4 t;
        t.x = T.x > 0.0f ? (F.x - P.x) / T.x : 0.0f;
        t.y = T.y > 0.0f ? (F.y - P.y) / T.y : 0.0f;
        t.z = T.z > 0.0f ? (F.z - P.z) / T.z : 0.0f;
        t.w = 0.0f;
        if (!(isfinite(F.x) && isfinite(F.y) && isfinite(F.z))) t.x = __int_as_float(0x7fc00000);
        targets[j] = t;
    }
}

// Scene.cpp:173-198 for each pixel of the batch, samples in order, exact float ops.
// The physical estimator keeps a plain running mean (1 / (n + 1)) and never stops early.
__global__ void __launch_bounds__(kRenderThreads) accumulate_kernel(PathBatch b, uint32_t spb, uint32_t max_samples,
                                                                   float max_variance, bool physical)
{
    using namespace ex;
    const uint32_t npix = b.plan ? b.plan->npix : b.npix;
    if (b.plan) spb = b.plan->spb;
    if (spb == 0) return;   // an empty round (the whole grid leaves)
    uint32_t added = 0;   // samples this thread added to its pixels
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < npix; slot += gridDim.x * blockDim.x) {
        const uint32_t pixel = b.pix_list[slot];
        if (b.done[pixel]) continue;
        float* px = b.pixels + 3 * (size_t)pixel;
        float* var = b.variance + 3 * (size_t)pixel;
        // the pixel's mean and variance stay in registers for the batch; the payloads are
        // loaded two samples ahead of their use (the running mean is serial per pixel)
        float mean[3] = {px[0], px[1], px[2]}, vr[3] = {var[0], var[1], var[2]};
        uint32_t cnt = b.count[pixel];
        uint32_t taken = b.taken[pixel];
        const uint32_t taken0 = taken;
        const float4* pay = b.pay + slot;
        const float4 none = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        float4 ahead0 = pay[0], ahead1 = spb > 1 ? pay[npix] : none;
        for (uint32_t s = 0; s < spb && taken < max_samples; ++s) {
            // the path's payload is the sample; NaN / Inf becomes pink (Integrators.cpp:145-146)
            const float4 x4 = ahead0;
            ahead0 = ahead1;
            if (s + 2 < spb) ahead1 = pay[(size_t)(s + 2) * npix];
            const bool finite = isfinite(x4.x) && isfinite(x4.y) && isfinite(x4.z);
            float x[3] = {finite ? x4.x : 1.0f, finite ? x4.y : 0.4f, finite ? x4.z : 0.7f};
            const uint32_t prev = cnt;
            ++taken;
            if (prev < 1) {
                cnt = 1;
                vr[0] = vr[1] = vr[2] = 0.0f;
            } else {
                const float g = div(1.0f, (float)(prev + 1));
                const float f = physical ? g : div(1.0f, (float)prev);
                for (int c = 0; c < 3; ++c) {
                    const float pp = mean[c];
                    const float np = add(pp, mul(sub(x[c], pp), f));
                    vr[c] = mul(add(mul(vr[c], (float)prev), mul(sub(x[c], pp), sub(x[c], np))), g);
                    x[c] = np;
                }
                cnt = prev + 1;
            }
            mean[0] = x[0]; mean[1] = x[1]; mean[2] = x[2];
            if (!physical && prev > 4 && vr[0] <= max_variance && vr[1] <= max_variance &&
                vr[2] <= max_variance) {
                b.done[pixel] = 1;
                break;
            }
        }
        if (taken != taken0) {
            px[0] = mean[0]; px[1] = mean[1]; px[2] = mean[2];
            var[0] = vr[0]; var[1] = vr[1]; var[2] = vr[2];
        }
        if (taken >= max_samples) b.done[pixel] = 1;
        b.count[pixel] = cnt;
        b.taken[pixel] = taken;
        added += taken - taken0;
    }
    if (b.sample_tally) {
        // one atomic per warp: every thread of the block gets here
        const uint32_t warp_total = __reduce_add_sync(0xffffffffu, added);
        if ((threadIdx.x & 31u) == 0 && warp_total) atomicAdd(b.sample_tally, (unsigned long long)warp_total);
    }
}

// Exit-aware rounds (RoundPlan).  One thread sets the round from the pixels the
// previous compaction kept.
__global__ void plan_init_kernel(RoundPlan* p, uint32_t npix)
{
    *p = RoundPlan{0u, 0u, 0u, 0u, npix, {0u, 0u, 0u}};
}

__global__ void plan_round_kernel(RoundPlan* p, uint32_t max_samples, uint32_t first_cap, uint32_t cap,
                                  uint32_t max_paths)
{
    const uint32_t npix = p->next_npix;
    uint32_t spb = max_samples > p->scheduled ? max_samples - p->scheduled : 0u;
    spb = min(spb, npix ? max_paths / npix : 0u);
    if (p->scheduled == 0) spb = min(spb, first_cap);
    spb = min(spb, cap);
    p->npix = npix;
    p->spb = spb;
    p->n = npix * spb;
    p->scheduled += spb;
    p->next_npix = 0;
}

// The round's pixels that are still sampling, appended to `out` (block order is
// the atomics', order within a block is kept, so warps keep neighbouring pixels).
__global__ void __launch_bounds__(kRenderThreads) compact_pixels_kernel(RoundPlan* p, const uint32_t* in,
                                                                       const uint32_t* done, uint32_t* out)
{
    __shared__ AppendScratch app;
    const uint32_t npix = p->npix;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (npix + stride - 1) / stride;
    for (uint32_t r = 0; r < rounds; ++r) {
        const uint32_t k = r * stride + blockIdx.x * blockDim.x + threadIdx.x;
        uint32_t pixel = 0;
        bool keep = false;
        if (k < npix) {
            pixel = in[k];
            keep = done[pixel] == 0;
        }
        uint32_t at, unused;
        block_append(r, keep, &p->next_npix, false, nullptr, app, at, unused);
        if (keep) out[at] = pixel;
    }
}

// The image state of a render into caller buffers (pico_gpu_render_device).
__global__ void __launch_bounds__(kRenderThreads) prepare_image_kernel(const uint32_t* count, uint32_t npx,
                                                                      uint32_t max_samples, uint32_t* pix_list,
                                                                      uint32_t* done, uint32_t* taken)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += gridDim.x * blockDim.x) {
        pix_list[p] = p;
        done[p] = count[p] >= max_samples ? 1u : 0u;
        taken[p] = 0;
    }
}

// Scene::generate_denoiser_inputs: one primary ray per pixel with xi = (0, 0).
template <int kOrder>
__global__ void __launch_bounds__(128) gbuffer_kernel(SceneView sc, CameraView cam, uint32_t W, uint32_t H,
                                                     float* normals, float* positions, float* diffuse, int* err)
{
    using namespace ex;
    const uint32_t npx = W * H;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += gridDim.x * blockDim.x) {
        float4 o, d;
        camera_ray(cam, 0.0f, 0.0f, p % W, p / W, o, d);
        TraceHit h;
        const int s = trace_closest<false, kOrder>(sc, o, d, h, nullptr);
        if (s != kTraceOk) atomicOr(err, s);
        float n[3], pos[3], alb[3];
        if (s == kTraceOk && h.rank != kNoHit) {
            const Fragment f = make_fragment(sc, h.rank, h.tri, h.u, h.v, o, d);
            n[0] = f.n.x; n[1] = f.n.y; n[2] = f.n.z;
            const float* V = cam.view;
            for (int r = 0; r < 3; ++r)
                pos[r] = add(add(mul(V[0 * 4 + r], f.px), mul(V[1 * 4 + r], f.py)),
                             add(mul(V[2 * 4 + r], f.pz), mul(V[3 * 4 + r], f.pw)));
            const GpuMaterial& m = sc.materials[sc.inst_shade[f.inst].material];
            alb[0] = m.diffuse[0]; alb[1] = m.diffuse[1]; alb[2] = m.diffuse[2];
        } else {
            n[0] = -d.x; n[1] = -d.y; n[2] = -d.z;
            pos[0] = mul(d.x, d.w); pos[1] = mul(d.y, d.w); pos[2] = mul(d.z, d.w);
            const float3 sk = sky_radiance(sc, d.x, d.y, d.z);   // m_sky_box->sample4(ray.mDirection)
            alb[0] = sk.x; alb[1] = sk.y; alb[2] = sk.z;
        }
        for (int c = 0; c < 3; ++c) {
            normals[3 * (size_t)p + c] = n[c];
            positions[3 * (size_t)p + c] = pos[c];
            diffuse[3 * (size_t)p + c] = alb[c];
        }
    }
}

// ---------------------------------------------------------------- launchers
// Grid of a grid-stride loop over n items: enough blocks for the items, at most one
// full wave of the kernel's resident blocks.  Every block runs the same number of
// rounds, so a partial second wave would take as long as a full one.
template <class Kernel>
static unsigned grid_for(Kernel* kernel, uint32_t n, int threads)
{
    const uint64_t want = ((uint64_t)n + threads - 1) / threads;
    const uint64_t cap = (uint64_t)sm_count() * (uint64_t)resident_blocks((const void*)kernel, threads);
    return (unsigned)(want < 1 ? 1 : (want > cap ? cap : want));
}

// Persistent grid of a closest-hit launch: `ctas_per_sm` CTAs per SM (0 or more
// than fit: as many as fit).
template <int kOrder, int kThreads, bool kCount = false>
static unsigned extend_grid(uint32_t ctas_per_sm)
{
    static int per_sm = 0;
    if (!per_sm) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, extend_kernel<kOrder, kThreads, kCount>, kThreads, 0);
        if (per_sm < 1) per_sm = 1;
    }
    const int k = (ctas_per_sm > 0 && (int)ctas_per_sm < per_sm) ? (int)ctas_per_sm : per_sm;
    return (unsigned)(sm_count() * k);
}

// One closest-hit launch; with counters, the counting variant (128 threads per CTA).
template <int kOrder>
static void launch_extend(const SceneView& sc, PathBatch& b, const uint32_t* q, const uint32_t* count,
                          const uint32_t* sq, const uint32_t* scount, DeviceStatus* status,
                          unsigned long long* tally, unsigned long long* counters, cudaStream_t st)
{
    unsigned long long* stally = &status->rays[2];
    // the counting variant (measurement only) reads the bounds at run time; bounded walks
    // (a debugging aid) and watertight ones (opt-in) take 128-thread CTAs whatever the
    // block shape asked for
    if (counters) {
        extend_kernel<kOrder | kBounded, 128, true><<<extend_grid<kOrder | kBounded, 128, true>(b.extend_ctas), 128,
                                                     0, st>>>(sc, b, q, count, sq, scount, &status->work,
                                                              &status->trace_error, tally, stally, counters);
        return;
    }
    if constexpr ((kOrder & (kBounded | kWatertight)) != 0) {
        extend_kernel<kOrder, 128><<<extend_grid<kOrder, 128>(b.extend_ctas), 128, 0, st>>>(
            sc, b, q, count, sq, scount, &status->work, &status->trace_error, tally, stally, nullptr);
    } else {
        switch (b.extend_threads) {
        case 64:
            extend_kernel<kOrder, 64><<<extend_grid<kOrder, 64>(b.extend_ctas), 64, 0, st>>>(
                sc, b, q, count, sq, scount, &status->work, &status->trace_error, tally, stally, nullptr);
            break;
        case 256:
            extend_kernel<kOrder, 256><<<extend_grid<kOrder, 256>(b.extend_ctas), 256, 0, st>>>(
                sc, b, q, count, sq, scount, &status->work, &status->trace_error, tally, stally, nullptr);
            break;
        default:
            extend_kernel<kOrder, 128><<<extend_grid<kOrder, 128>(b.extend_ctas), 128, 0, st>>>(
                sc, b, q, count, sq, scount, &status->work, &status->trace_error, tally, stally, nullptr);
        }
    }
}

cudaError_t LaunchTimer::record(cudaStream_t st)
{
    if (used == events.size()) {
        cudaEvent_t ev = nullptr;
        const cudaError_t e = cudaEventCreate(&ev);
        if (e != cudaSuccess) return e;
        events.push_back(ev);
    }
    return cudaEventRecord(events[used++], st);
}

cudaError_t LaunchTimer::total(double& ms, uint64_t& launches) const
{
    ms = 0.0;
    launches = used / 2;
    for (size_t k = 0; k + 1 < used; k += 2) {
        float t = 0.0f;
        const cudaError_t e = cudaEventElapsedTime(&t, events[k], events[k + 1]);
        if (e != cudaSuccess) return e;
        ms += t;
    }
    return cudaSuccess;
}

LaunchTimer::~LaunchTimer()
{
    for (cudaEvent_t ev : events) cudaEventDestroy(ev);
}

__global__ void stamp_kernel(unsigned long long* dst)
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    *dst = t;
}

cudaError_t launch_stamp(unsigned long long* dst, cudaStream_t st)
{
    stamp_kernel<<<1, 1, 0, st>>>(dst);
    return cudaGetLastError();
}

// The extend / shade / shadow loop of one batch whose camera rays are queued.
static cudaError_t run_depth_loop(const SceneView& sc, PathBatch& b, uint32_t max_depth, bool physical,
                                  const NrcShadeArgs& nrc, DeviceStatus* status, int order, cudaStream_t st,
                                  const RenderProbe* probe = nullptr)
{
    LaunchTimer* timer = probe ? probe->timer : nullptr;
    LaunchTimer* shade_timer = probe ? probe->shade_timer : nullptr;
    unsigned long long* counters = probe ? probe->counters : nullptr;
    cudaError_t e = cudaSuccess;
    const bool trace_last =
        sc.sky_kind != PICO_SKY_CONSTANT || sc.sky[0] != 0.0f || sc.sky[1] != 0.0f || sc.sky[2] != 0.0f;
    int cur = 0;
    for (uint32_t depth = 0; depth <= max_depth; ++depth) {
        e = cudaMemsetAsync(&status->work, 0, sizeof(unsigned long long), st);
        if (e != cudaSuccess) return e;
        unsigned long long* tally = &status->rays[depth == 0 ? 0 : 1];
        // this depth's segments, and from depth 1 on the previous shade's shadow rays
        const uint32_t* sq = depth > 0 ? b.shadow_queue : nullptr;
        if (timer && (e = timer->record(st)) != cudaSuccess) return e;
        with_variant(order, sc, [&](auto v) {
            launch_extend<decltype(v)::value>(sc, b, b.queue[cur], &b.counters[cur], sq, &b.counters[2], status,
                                              tally, counters, st);
        });
        if (timer && (e = timer->record(st)) != cudaSuccess) return e;
        e = cudaMemsetAsync(&b.counters[cur ^ 1], 0, sizeof(uint32_t), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(&b.counters[2], 0, sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
        if (shade_timer && (e = shade_timer->record(st)) != cudaSuccess) return e;
        if (physical)
            shade_physical_kernel<<<grid_for(shade_physical_kernel, b.n, kRenderThreads), kRenderThreads, 0, st>>>(sc, b, cur, depth,
                                                                                         max_depth, nrc);
        else
            shade_kernel<<<grid_for(shade_kernel, b.n, kRenderThreads), kRenderThreads, 0, st>>>(sc, b, cur, depth, max_depth,
                                                                                    trace_last);
        if (shade_timer && (e = shade_timer->record(st)) != cudaSuccess) return e;
        cur ^= 1;
    }
    return cudaGetLastError();
}

cudaError_t launch_training_paths(const SceneView& sc, PathBatch& b, const CameraView& cam, unsigned long long seed,
                                  uint32_t frame, uint32_t n, uint32_t W, uint32_t H, uint32_t max_depth,
                                  const NrcShadeArgs& nrc, float4* targets, DeviceStatus* status, int order,
                                  cudaStream_t st)
{
    PathBatch t = b;
    t.n = n;
    cudaError_t e = cudaMemsetAsync(t.counters, 0, 4 * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(nrc.count, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    train_raygen_kernel<<<grid_for(train_raygen_kernel, n, kRenderThreads), kRenderThreads, 0, st>>>(t, cam, seed, frame, W, W * H);
    e = run_depth_loop(sc, t, max_depth, true, nrc, status, order, st);
    if (e != cudaSuccess) return e;
    nrc_targets_kernel<<<grid_for(nrc_targets_kernel, nrc.capacity, kRenderThreads), kRenderThreads, 0, st>>>(
        nrc.queries, nrc.rec_tp, t.pay, nrc.count, nrc.capacity, targets);
    return cudaGetLastError();
}

cudaError_t launch_render_batch(const SceneView& sc, PathBatch& b, const CameraView& cam, unsigned long long seed,
                                uint32_t spb, uint32_t max_depth, uint32_t max_samples, float max_variance,
                                int estimator, DeviceStatus* status, int order, cudaStream_t st,
                                const NrcShadeArgs* nrc, const RenderProbe* probe)
{
    b.sample_tally = &status->rays[3];
    const bool physical = estimator != PICO_ESTIMATOR_REFERENCE;
    NrcShadeArgs off{};
    off.mode = kNrcOff;
    const NrcShadeArgs& na = nrc ? *nrc : off;
    cudaError_t e = cudaMemsetAsync(b.counters, 0, 4 * sizeof(uint32_t), st);
    if (e == cudaSuccess && na.mode != kNrcOff) e = cudaMemsetAsync(na.count, 0, sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    raygen_kernel<<<grid_for(raygen_kernel, b.n, kRenderThreads), kRenderThreads, 0, st>>>(b, cam, seed, physical);
    e = run_depth_loop(sc, b, max_depth, physical, na, status, order, st, probe);
    if (e != cudaSuccess) return e;
    if (na.mode == kNrcTerminate) {
        e = nrc::launch_infer(na.geo, na.table, na.weights, na.queries, na.capacity, nullptr, b.thr, b.pay, na.err, st,
                              na.count, na.infer_groups, na.wait);
        if (e != cudaSuccess) return e;
    }
    accumulate_kernel<<<grid_for(accumulate_kernel, b.npix, kRenderThreads), kRenderThreads, 0, st>>>(b, spb, max_samples, max_variance,
                                                                                    physical);
    return cudaGetLastError();
}

cudaError_t launch_plan_init(RoundPlan* plan, uint32_t npix, cudaStream_t st)
{
    plan_init_kernel<<<1, 1, 0, st>>>(plan, npix);
    return cudaGetLastError();
}

cudaError_t launch_plan_round(RoundPlan* plan, uint32_t max_samples, uint32_t first_cap, uint32_t cap,
                              uint32_t max_paths, cudaStream_t st)
{
    plan_round_kernel<<<1, 1, 0, st>>>(plan, max_samples, first_cap, cap, max_paths);
    return cudaGetLastError();
}

cudaError_t launch_compact_pixels(RoundPlan* plan, const uint32_t* in, const uint32_t* done, uint32_t* out,
                                  uint32_t npix_bound, cudaStream_t st)
{
    compact_pixels_kernel<<<grid_for(compact_pixels_kernel, npix_bound, kRenderThreads), kRenderThreads, 0, st>>>(
        plan, in, done, out);
    return cudaGetLastError();
}

cudaError_t launch_prepare_image(const uint32_t* count, uint32_t npx, uint32_t max_samples, uint32_t* pix_list,
                                 uint32_t* done, uint32_t* taken, cudaStream_t st)
{
    if (npx == 0) return cudaSuccess;
    prepare_image_kernel<<<grid_for(prepare_image_kernel, npx, kRenderThreads), kRenderThreads, 0, st>>>(count, npx, max_samples, pix_list,
                                                                                  done, taken);
    return cudaGetLastError();
}

cudaError_t launch_gbuffer(const SceneView& sc, const CameraView& cam, uint32_t W, uint32_t H, float* normals,
                           float* positions, float* diffuse, DeviceStatus* status, int order, cudaStream_t st)
{
    with_variant(order, sc, [&](auto v) {
        gbuffer_kernel<decltype(v)::value><<<grid_for(gbuffer_kernel<decltype(v)::value>, W * H, 128), 128, 0, st>>>(sc, cam, W, H, normals, positions,
                                                                                 diffuse, &status->trace_error);
    });
    return cudaGetLastError();
}

}  // namespace pico
