// Device sampling and shading: the reference's camera, tangent frame, lobes,
// BSRDF sample / pdf and direct-lighting pdf.
//
//   Camera::generate_ray            Core/Camera.cpp:11-28 (exact operation order)
//   construct_world_to_tangent      Core/vectorUtils.cpp:9-35
//   glm::inverse(mat3)              glm/detail/func_matrix.inl:272-294
//   cosine lobe                     Render/Distributions.cpp:14-29
//   Beckmann lobe                   Render/Distributions.cpp:31-78
//   BSRDF sample / pdf              Render/BSRDF.cpp:11-214
//   direct_lighting_pdf             Render/Integrators.cpp:13-22
//   hammersley(i, 2^32-1)           Core/RandUtils.cpp:13-27, 87-90
//
// The geometric parts (camera ray, frame, inverse, reflection) keep glm's
// operation order through the exact helpers; the transcendental functions use
// CUDA's IEEE-accurate cosf/sinf/logf/expf (not the fast intrinsics), which
// agree with the host libm to a few ulp.  Random numbers come from a PCG32
// stream per path (O'Neill 2014) instead of the reference's xorshift and
// mt19937_64 draws: the estimator's distribution is the same, its stream is not.
#pragma once

#include "exact_math.cuh"
#include "kernels_render.h"
#include "layout.h"
#include "traverse.cuh"

namespace pico {

// ---------------------------------------------------------------- random numbers
struct Pcg32 {
    unsigned long long state;
    __device__ __forceinline__ uint32_t next()
    {
        const unsigned long long old = state;
        state = old * 6364136223846793005ull + 1442695040888963407ull;
        const uint32_t xorshifted = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    // uniform_real_distribution<float>(0, 1) stand-in: 24 random bits in [0, 1)
    __device__ __forceinline__ float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

// splitmix64 finaliser, used to derive independent PCG states from (seed, pixel, sample)
__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ Pcg32 path_rng(unsigned long long seed, uint32_t pixel, uint32_t sample)
{
    Pcg32 r;
    r.state = mix64(seed ^ mix64(((unsigned long long)pixel << 32) | sample));
    r.next();
    return r;
}

__device__ __forceinline__ float radical_inverse(uint32_t bits)
{
    return (float)__brev(bits) * 2.3283064365386963e-10f;
}

// Hammersley_Generator::next(): one 32-bit draw -> (i / 2^32, radical inverse of i).
__device__ __forceinline__ void hammersley(Pcg32& r, float& x, float& y)
{
    const uint32_t i = r.next();
    x = ex::div((float)i, 4294967296.0f);
    y = radical_inverse(i);
}

// ---------------------------------------------------------------- camera
__device__ __forceinline__ void camera_ray(const CameraView& c, float xi_x, float xi_y, uint32_t px, uint32_t py,
                                           float4& org, float4& dir)
{
    using namespace ex;
    const float rx = div(xi_x, 2.0f), ry = div(xi_y, 2.0f);
    const float dx = mul(sub(div(add((float)px, rx), c.res_x), 0.5f), c.aspect);
    const float dy = sub(div(add((float)py, ry), c.res_y), 0.5f);
    const V3 D = v3(c.dir[0], c.dir[1], c.dir[2]), U = v3(c.up[0], c.up[1], c.up[2]);
    const V3 R = v3(c.right[0], c.right[1], c.right[2]);
    const V3 d = normalize(vadd(vadd(vscale(D, 1.0f), vscale(U, dy)), vscale(R, dx)));
    org = make_float4(c.pos[0], c.pos[1], c.pos[2], 1.0f);
    dir = make_float4(d.x, d.y, d.z, c.far_plane);
}

// ---------------------------------------------------------------- tangent space
struct M3 { float m[3][3]; };   // column-major like glm: m[c][r]

__device__ __forceinline__ M3 tangent_frame(ex::V3 V, ex::V3 N)
{
    using namespace ex;
    V3 t;
    if (fabsf(dot(V, N)) > 0.95f) {
        const V3 vv = fabsf(N.z) > 0.99f ? v3(1, 0, 0) : v3(0, 0, 1);
        t = normalize(cross(N, vv));
    } else {
        t = normalize(cross(V, N));
    }
    const V3 b = normalize(cross(t, N));
    M3 m;   // transpose(mat3(t, b, N))
    m.m[0][0] = t.x; m.m[1][0] = t.y; m.m[2][0] = t.z;
    m.m[0][1] = b.x; m.m[1][1] = b.y; m.m[2][1] = b.z;
    m.m[0][2] = N.x; m.m[1][2] = N.y; m.m[2][2] = N.z;
    return m;
}

__device__ __forceinline__ ex::V3 m3_mul(const M3& m, ex::V3 v)
{
    using namespace ex;
    return v3(add(add(mul(m.m[0][0], v.x), mul(m.m[1][0], v.y)), mul(m.m[2][0], v.z)),
              add(add(mul(m.m[0][1], v.x), mul(m.m[1][1], v.y)), mul(m.m[2][1], v.z)),
              add(add(mul(m.m[0][2], v.x), mul(m.m[1][2], v.y)), mul(m.m[2][2], v.z)));
}

__device__ __forceinline__ M3 m3_inverse(const M3& a)
{
    using namespace ex;
    const float(*m)[3] = a.m;
    const float det = add(sub(mul(m[0][0], sub(mul(m[1][1], m[2][2]), mul(m[2][1], m[1][2]))),
                              mul(m[1][0], sub(mul(m[0][1], m[2][2]), mul(m[2][1], m[0][2])))),
                          mul(m[2][0], sub(mul(m[0][1], m[1][2]), mul(m[1][1], m[0][2]))));
    const float o = div(1.0f, det);
    M3 r;
    r.m[0][0] = mul(sub(mul(m[1][1], m[2][2]), mul(m[2][1], m[1][2])), o);
    r.m[1][0] = mul(-sub(mul(m[1][0], m[2][2]), mul(m[2][0], m[1][2])), o);
    r.m[2][0] = mul(sub(mul(m[1][0], m[2][1]), mul(m[2][0], m[1][1])), o);
    r.m[0][1] = mul(-sub(mul(m[0][1], m[2][2]), mul(m[2][1], m[0][2])), o);
    r.m[1][1] = mul(sub(mul(m[0][0], m[2][2]), mul(m[2][0], m[0][2])), o);
    r.m[2][1] = mul(-sub(mul(m[0][0], m[2][1]), mul(m[2][0], m[0][1])), o);
    r.m[0][2] = mul(sub(mul(m[0][1], m[1][2]), mul(m[1][1], m[0][2])), o);
    r.m[1][2] = mul(-sub(mul(m[0][0], m[1][2]), mul(m[1][0], m[0][2])), o);
    r.m[2][2] = mul(sub(mul(m[0][0], m[1][1]), mul(m[1][0], m[0][1])), o);
    return r;
}

// ---------------------------------------------------------------- lobes
constexpr double kPi = 3.14159265358979323846;

__device__ __forceinline__ ex::V3 cos_sample(float u1, float u2)
{
    using namespace ex;
    const float r = sqrt_(u1);
    const float phi = (float)((double)u2 * kPi * 2.0);
    const float om = sub(1.0f, u1);
    const float z = (float)sqrt((double)((0.0f < om) ? om : 0.0f));
    const double c = cos((double)phi), s = sin((double)phi);
    return normalize(v3((float)((double)r * c), (float)((double)r * s), z));
}

__device__ __forceinline__ float cos_pdf(ex::V3 H)
{
    const float c = ex::div(H.z, (float)kPi);
    return (0.0f < c) ? c : 0.0f;
}

__device__ __forceinline__ ex::V3 beckmann_sample(float x0, float x1, ex::V3 V, float R)
{
    using namespace ex;
    const float alpha = mul(R, R);
    float log_sample = logf(sub(1.0f, x0));
    if (isinf(log_sample)) log_sample = 0.0f;
    const float tan2 = mul(mul(-alpha, alpha), log_sample);
    const float phi = (float)((double)mul(x1, 2.0f) * kPi);
    const float cos_t = div(1.0f, sqrt_(add(1.0f, tan2)));
    const float s2 = sub(1.0f, mul(cos_t, cos_t));
    const float sin_t = sqrt_((0.0f < s2) ? s2 : 0.0f);
    V3 H = v3(mul(sin_t, cosf(phi)), mul(sin_t, sinf(phi)), cos_t);
    if (!(mul(V.z, H.z) > 0.0f)) H = vneg(H);
    return normalize(H);
}

__device__ __forceinline__ float roughness_to_alpha(float r)
{
    using namespace ex;
    r = (r < 1e-3f) ? 1e-3f : r;
    const float x = logf(r);
    return add(add(add(add(1.62142f, mul(0.819955f, x)), mul(mul(0.1734f, x), x)), mul(mul(mul(0.0171201f, x), x), x)),
               mul(mul(mul(mul(0.000640711f, x), x), x), x));
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

__device__ __forceinline__ float beckmann_D(ex::V3 w, float R)
{
    using namespace ex;
    const float ax = roughness_to_alpha(R);
    const float cos2 = mul(w.z, w.z);
    const float s2 = sub(1.0f, cos2);
    const float sin2 = (0.0f < s2) ? s2 : 0.0f;
    const float tan2 = div(sin2, cos2);
    if (isinf(tan2)) return 0.0f;
    const float cos4 = mul(cos2, cos2);
    const float sin_t = sqrt_(sin2);
    const float cphi = (sin_t == 0.0f) ? 1.0f : clampf(div(w.x, sin_t), -1.0f, 1.0f);
    const float sphi = (sin_t == 0.0f) ? 0.0f : clampf(div(w.y, sin_t), -1.0f, 1.0f);
    const float a2 = mul(ax, ax);
    const float e = expf(mul(-tan2, add(div(mul(cphi, cphi), a2), div(mul(sphi, sphi), a2))));
    return (float)((double)e / (kPi * (double)ax * (double)ax * (double)cos4));
}

__device__ __forceinline__ float beckmann_pdf(ex::V3 H, float R)
{
    const float d = clampf(beckmann_D(H, R), 0.0f, 1.0f);
    return ex::mul(d, fabsf(H.z));
}

__device__ __forceinline__ float bsdf_pdf(uint32_t kind, ex::V3 wo, ex::V3 H, float roughness, float refl)
{
    using namespace ex;
    switch (kind) {
    case PICO_BSDF_DIFFUSE:
    case PICO_BSDF_LIGHT: return cos_pdf(H);
    case PICO_BSDF_SPECULAR: return div(beckmann_pdf(H, roughness), mul(2.0f, dot(wo, H)));
    case PICO_BSDF_DIELECTRIC:
        return add(mul(cos_pdf(H), sub(1.0f, refl)), mul(div(beckmann_pdf(H, roughness), mul(2.0f, dot(wo, H))), refl));
    default: return 0.0f;
    }
}

__device__ __forceinline__ ex::V3 reflect3(ex::V3 I, ex::V3 N)
{
    using namespace ex;
    const float d = dot(N, I);
    return v3(sub(I.x, mul(mul(N.x, d), 2.0f)), sub(I.y, mul(mul(N.y, d), 2.0f)), sub(I.z, mul(mul(N.z, d), 2.0f)));
}

struct BsdfSample {
    ex::V3 L;
    float P;
    ex::V3 energy;
};

// Core::Ray's index-of-refraction stack (Core/AABB.cpp:54-81), 8 entries deep: a
// camera path starts with 1.0 and each Transparent_BTDF sample pushes the
// material's IoR on entering or pops on leaving.  Entries past the eighth are
// counted but not stored; popping an empty stack is ignored and reading one gives
// 1.0 (both undefined in the reference).
constexpr uint32_t kIorDepth = 8;
struct IorStack {
    float v[kIorDepth];
    uint32_t n;
    __device__ __forceinline__ void push(float x) { if (n < kIorDepth) v[n] = x; ++n; }
    __device__ __forceinline__ void pop() { if (n) --n; }
    __device__ __forceinline__ float top() const { return n ? v[(n < kIorDepth ? n : kIorDepth) - 1] : 1.0f; }
    __device__ __forceinline__ bool inside() const { return n > 1; }
};

// glm::refract (glm/detail/func_geometric.inl:119-127); the product with (k >= 0)
// keeps sqrt's NaN, so total internal reflection yields a NaN direction.
__device__ __forceinline__ ex::V3 refract3(ex::V3 I, ex::V3 N, float eta)
{
    using namespace ex;
    const float d = dot(N, I);
    const float k = sub(1.0f, mul(mul(eta, eta), sub(1.0f, mul(d, d))));
    const float s = add(mul(eta, d), sqrt_(k));
    const float g = (float)(k >= 0.0f);
    return v3(mul(sub(mul(eta, I.x), mul(s, N.x)), g), mul(sub(mul(eta, I.y), mul(s, N.y)), g),
              mul(sub(mul(eta, I.z), mul(s, N.z)), g));
}

// Transparent_BTDF::sample (Render/BSRDF.cpp:238-297).
template <class NextXi>
__device__ __forceinline__ BsdfSample transparent_sample(const GpuMaterial& m, ex::V3 V, ex::V3 N, IorStack& ior,
                                                         NextXi&& next_xi)
{
    using namespace ex;
    const M3 w2t = tangent_frame(V, N);
    const M3 t2w = m3_inverse(w2t);
    const V3 vt = normalize(m3_mul(w2t, V));
    const bool enter = vt.z >= 0.0f;
    float x0, x1;
    next_xi(x0, x1);
    const V3 H = beckmann_sample(x0, x1, vt, m.roughness);
    const float eta = div(1.0f, m.ior);
    if (enter) ior.push(m.ior); else ior.pop();
    const V3 L = refract3(vt, H, eta);
    BsdfSample s;
    s.L = normalize(m3_mul(t2w, L));
    const float pdf = beckmann_pdf(H, m.roughness);
    const V3 wh = normalize(vadd(vt, vscale(L, eta)));
    const float denom = add(dot(vt, wh), mul(eta, dot(L, wh)));
    const float dwh_dwi = fabsf(div(mul(mul(eta, eta), dot(L, wh)), mul(denom, denom)));
    s.P = mul(pdf, dwh_dwi);
    s.energy = v3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
    return s;
}

// Fresnel_BTDF::fresnel_factor (Render/BSRDF.cpp:395-421).
__device__ __forceinline__ float fresnel_factor(float cos_i, float eta_i, float eta_t)
{
    using namespace ex;
    cos_i = clampf(cos_i, -1.0f, 1.0f);
    if (!(cos_i > 0.0f)) {
        const float tmp = eta_i; eta_i = eta_t; eta_t = tmp;
        cos_i = fabsf(cos_i);
    }
    const float a = sub(1.0f, mul(cos_i, cos_i));
    const float sin_i = sqrt_((0.0f < a) ? a : 0.0f);
    const float sin_t = mul(div(eta_i, eta_t), sin_i);
    const float b = sub(1.0f, mul(sin_t, sin_t));
    const float cos_t = sqrt_((0.0f < b) ? b : 0.0f);
    const float rparl = div(sub(mul(eta_t, cos_i), mul(eta_i, cos_t)), add(mul(eta_t, cos_i), mul(eta_i, cos_t)));
    const float rperp = div(sub(mul(eta_i, cos_i), mul(eta_t, cos_t)), add(mul(eta_i, cos_i), mul(eta_t, cos_t)));
    return div(add(mul(rparl, rparl), mul(rperp, rperp)), 2.0f);
}

// Specular_BRDF::sample (Render/BSRDF.cpp:54-84).
template <class NextXi>
__device__ __forceinline__ BsdfSample specular_sample(const GpuMaterial& m, ex::V3 V, ex::V3 N, NextXi&& next_xi)
{
    using namespace ex;
    const M3 w2t = tangent_frame(V, N);
    const M3 t2w = m3_inverse(w2t);
    const V3 vt = normalize(m3_mul(w2t, V));
    float x0, x1;
    next_xi(x0, x1);
    const V3 H = beckmann_sample(x0, x1, vt, m.roughness);
    const V3 L = normalize(reflect3(vneg(vt), H));
    BsdfSample s;
    s.L = normalize(m3_mul(t2w, L));
    s.P = bsdf_pdf(PICO_BSDF_SPECULAR, vt, H, m.roughness, m.reflectance);
    s.energy = v3(m.specular[0], m.specular[1], m.specular[2]);
    return s;
}

// BSRDF::sample; `xi` yields the Hammersley points the lobe consumes in the reference's order.
template <class NextXi>
__device__ __forceinline__ BsdfSample sample_bsdf(uint32_t kind, const GpuMaterial& m, ex::V3 V, ex::V3 N, NextXi&& next_xi,
                                                  IorStack& ior)
{
    using namespace ex;
    if (kind == PICO_BSDF_DELTA) {   // Specular_Delta_BRDF (Render/BSRDF.cpp:216-229)
        BsdfSample s;
        s.energy = v3(m.specular[0], m.specular[1], m.specular[2]);
        s.L = reflect3(vneg(V), N);
        s.P = 1.0f;
        return s;
    }
    if (kind == PICO_BSDF_BTDF) return transparent_sample(m, V, N, ior, next_xi);
    if (kind == PICO_BSDF_FRESNEL) {   // Fresnel_BTDF::sample (Render/BSRDF.cpp:364-385)
        const M3 fw = tangent_frame(V, N);
        const V3 fvt = normalize(m3_mul(fw, V));
        float f0, f1;
        next_xi(f0, f1);
        const float F = fresnel_factor(fvt.z, m.ior, ior.top());
        if (f0 < F) {
            BsdfSample s = specular_sample(m, V, N, next_xi);
            s.P = mul(s.P, F);
            return s;
        }
        BsdfSample s = transparent_sample(m, V, N, ior, next_xi);
        s.P = mul(s.P, sub(1.0f, F));
        return s;
    }
    const M3 w2t = tangent_frame(V, N);
    const M3 t2w = m3_inverse(w2t);
    const V3 vt = normalize(m3_mul(w2t, V));
    BsdfSample s;
    float x0, x1;
    if (kind == PICO_BSDF_DIFFUSE || kind == PICO_BSDF_LIGHT) {
        next_xi(x0, x1);
        const V3 H = cos_sample(x0, x1);
        s.P = cos_pdf(H);
        s.L = normalize(m3_mul(t2w, H));
        s.energy = kind == PICO_BSDF_DIFFUSE ? v3(m.diffuse[0], m.diffuse[1], m.diffuse[2])
                                             : v3(m.emissive[0], m.emissive[1], m.emissive[2]);
    } else if (kind == PICO_BSDF_SPECULAR) {
        return specular_sample(m, V, N, next_xi);
    } else {
        next_xi(x0, x1);
        if (x1 >= m.reflectance) {
            next_xi(x0, x1);
            const V3 H = cos_sample(x0, x1);
            s.L = normalize(m3_mul(t2w, H));
            s.P = cos_pdf(H);
            s.energy = v3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
        } else {
            next_xi(x0, x1);
            const V3 H = beckmann_sample(x0, x1, vt, m.roughness);
            const V3 L = normalize(reflect3(vneg(vt), H));
            s.L = normalize(m3_mul(t2w, L));
            s.P = div(beckmann_pdf(H, m.roughness), mul(2.0f, dot(vt, H)));
            s.energy = v3(m.specular[0], m.specular[1], m.specular[2]);
        }
    }
    return s;
}

__device__ __forceinline__ float direct_lighting_pdf(uint32_t kind, const GpuMaterial& m, ex::V3 N, ex::V3 wi, ex::V3 wo)
{
    using namespace ex;
    const M3 t = tangent_frame(wi, N);
    const V3 two = m3_mul(t, wo);
    const V3 H = m3_mul(t, normalize(vadd(wi, wo)));
    return bsdf_pdf(kind, two, H, m.roughness, m.reflectance);
}

// ---------------------------------------------------------------- implicit lights
// sample_geometry of the implicit assets (Core/LowerLevelImplicitShapesBVH.cpp:59-67,
// 93-112): a uniform point on the radius-0.5 sphere (uniform_sample_sphere,
// Core/RandUtils.cpp:43-49) or on a face of the unit cube (a random corner, a random
// axis whose face offset is zero, two uniform offsets).
__device__ __forceinline__ void implicit_light_point(uint32_t shape, Pcg32& rng, float& x, float& y, float& z)
{
    using namespace ex;
    float a0, a1;
    hammersley(rng, a0, a1);
    if (shape == PICO_SHAPE_SPHERE) {
        const float zz = sub(1.0f, mul(2.0f, a0));
        const float q = sub(1.0f, mul(zz, zz));
        const float r = sqrt_((0.0f < q) ? q : 0.0f);
        const float phi = (float)(2.0 * kPi * (double)a1);
        x = mul(0.5f, mul(r, cosf(phi)));
        y = mul(0.5f, mul(r, sinf(phi)));
        z = mul(0.5f, zz);
        return;
    }
    float b0, b1, c0, c1;
    hammersley(rng, b0, b1);
    hammersley(rng, c0, c1);
    const float c[3] = {sub(a0, 0.5f), sub(a1, 0.5f), sub(b0, 0.5f)};
    float corner[3], face[3];
    for (int a = 0; a < 3; ++a) corner[a] = (float)((0.0f < c[a]) - (c[a] < 0.0f));
    uint32_t zero_axis = (uint32_t)mul(b1, 3.0f);
    if (zero_axis >= 3) zero_axis = 2;
    face[zero_axis] = 0.0f;
    face[(zero_axis + 1) % 3] = c0;
    face[(zero_axis + 2) % 3] = c1;
    x = add(mul(corner[0], 0.5f), mul(-corner[0], face[0]));
    y = add(mul(corner[1], 0.5f), mul(-corner[1], face[1]));
    z = add(mul(corner[2], 0.5f), mul(-corner[2], face[2]));
}

// ---------------------------------------------------------------- sky
// ImageCube::sample4 (Core/Image.cpp:361-397) of the scene's sky, xyz: the
// nearest texel of a 6-face RGBA8 cube (resolve_cubemap_UV, Image.cpp:428-455,
// texels / 255) or of an RGBA float equirectangular image (Image.cpp:457-464:
// (atan2(z, x), asin(y)) / (2 pi, pi) + 0.5 with v flipped); get_data_ptr
// (Image.cpp:400-425) truncates uv * size and wraps it modulo the size.  The
// constant kind returns sky_rgb.
__device__ __forceinline__ uint32_t sky_texel(float uv, uint32_t n)
{
    return __float2uint_rz(ex::mul(uv, (float)n)) % n;
}

__device__ __forceinline__ float3 sky_radiance(const SceneView& sc, float vx, float vy, float vz)
{
    using namespace ex;
    if (sc.sky_kind == PICO_SKY_CUBE_RGBA8) {
        const float ax = vx >= 0.0f ? vx : -vx, ay = vy >= 0.0f ? vy : -vy, az = vz >= 0.0f ? vz : -vz;
        uint32_t face;
        float ma, u, w;
        if (az >= ax && az >= ay) {
            face = vz < 0.0f ? 5 : 4;
            ma = div(0.5f, az);
            u = vz < 0.0f ? -vx : vx;
            w = -vy;
        } else if (ay >= ax) {
            face = vy < 0.0f ? 3 : 2;
            ma = div(0.5f, ay);
            u = vx;
            w = vy < 0.0f ? -vz : vz;
        } else {
            face = vx < 0.0f ? 1 : 0;
            ma = div(0.5f, ax);
            u = vx < 0.0f ? vz : -vz;
            w = -vy;
        }
        u = add(mul(u, ma), 0.5f);
        w = add(mul(w, ma), 0.5f);
        const uint32_t x = sky_texel(u, sc.sky_w), y = sky_texel(w, sc.sky_h);
        const uchar4 p = __ldg(static_cast<const uchar4*>(sc.sky_pixels) +
                               ((size_t)face * sc.sky_w * sc.sky_h + (size_t)y * sc.sky_w + x));
        return make_float3(div((float)p.x, 255.0f), div((float)p.y, 255.0f), div((float)p.z, 255.0f));
    }
    if (sc.sky_kind == PICO_SKY_EQUIRECT_RGBAF) {
        float u = (float)atan2((double)vz, (double)vx);
        float w = (float)asin((double)vy);
        u = mul(u, (float)(1.0 / (3.14159265358979323846 * 2.0f)));
        w = mul(w, (float)(1.0 / 3.14159265358979323846));
        u = add(u, 0.5f);
        w = sub(1.0f, add(w, 0.5f));
        const uint32_t x = sky_texel(u, sc.sky_w), y = sky_texel(w, sc.sky_h);
        const float4 p = __ldg(static_cast<const float4*>(sc.sky_pixels) + ((size_t)y * sc.sky_w + x));
        return make_float3(p.x, p.y, p.z);
    }
    return make_float3(sc.sky[0], sc.sky[1], sc.sky[2]);
}

// ---------------------------------------------------------------- hit fragments
struct Fragment {
    float px, py, pz, pw;   // world position (vec4)
    ex::V3 n;               // world normal
    uint32_t inst;          // original instance index
};

// interpolate_fragment + lower_level_intersector's world transform for a hit; an
// implicit hit (tri = kImplicitTri, object-space t in u) is rebuilt from the ray o, d.
__device__ __forceinline__ Fragment make_fragment(const SceneView& sc, uint32_t rank, uint32_t tri, float u, float v,
                                                  const float4 o, const float4 d)
{
    using namespace ex;
    if (tri == kImplicitTri) {
        const ObjectRay q = to_object(sc.insts + rank, o, d);
        const float t = u;
        float px, py, pz;
        V3 nobj;
        if (__float_as_uint(q.root_lo.w) == PICO_REF_SPHERE) {   // N = normalize(P.xyz)
            px = add(q.ox, mul(t, q.dx)); py = add(q.oy, mul(t, q.dy)); pz = add(q.oz, mul(t, q.dz));
            nobj = normalize(v3(px, py, pz));
        } else {   // the cube: the sign of the largest |component| (maximum_component_index)
            px = add(q.ox, mul(q.dx, t)); py = add(q.oy, mul(q.dy, t)); pz = add(q.oz, mul(q.dz, t));
            const float ax = px >= 0.0f ? px : -px, ay = py >= 0.0f ? py : -py, az = pz >= 0.0f ? pz : -pz;
            const int k = (ax >= ay && ax >= az) ? 0 : ((ay >= ax && ay >= az) ? 1 : 2);
            const float pk = k == 0 ? px : (k == 1 ? py : pz);
            const float sg = (float)((0.0f < pk) - (pk < 0.0f));
            nobj = v3(k == 0 ? sg : 0.0f, k == 1 ? sg : 0.0f, k == 2 ? sg : 0.0f);
        }
        const float4* ip = reinterpret_cast<const float4*>(sc.insts + rank);
        const float4 f0 = __ldg(ip + 3), f1 = __ldg(ip + 4), f2 = __ldg(ip + 5), f3 = __ldg(ip + 6);
        Fragment f;
        f.px = row4(f0, px, py, pz, 1.0f); f.py = row4(f1, px, py, pz, 1.0f);
        f.pz = row4(f2, px, py, pz, 1.0f); f.pw = row4(f3, px, py, pz, 1.0f);
        f.n = normalize(v3(row3(f0, nobj.x, nobj.y, nobj.z), row3(f1, nobj.x, nobj.y, nobj.z),
                           row3(f2, nobj.x, nobj.y, nobj.z)));
        f.inst = sc.insts[rank].inst_id;
        return f;
    }
    const float4* tp = reinterpret_cast<const float4*>(sc.tris + tri);
    const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
    const float4* np = reinterpret_cast<const float4*>(sc.tri_shade + tri);
    const float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
    const float w = sub(sub(1.0f, v), u);
    const float px = add(add(mul(w, a.x), mul(u, b.x)), mul(v, c.x));
    const float py = add(add(mul(w, a.y), mul(u, b.y)), mul(v, c.y));
    const float pz = add(add(mul(w, a.z), mul(u, b.z)), mul(v, c.z));
    const V3 nobj = normalize(v3(add(add(mul(w, na.x), mul(u, nb.x)), mul(v, nc.x)),
                                 add(add(mul(w, na.y), mul(u, nb.y)), mul(v, nc.y)),
                                 add(add(mul(w, na.z), mul(u, nb.z)), mul(v, nc.z))));
    const float4* ip = reinterpret_cast<const float4*>(sc.insts + rank);
    const float4 f0 = __ldg(ip + 3), f1 = __ldg(ip + 4), f2 = __ldg(ip + 5), f3 = __ldg(ip + 6);
    Fragment f;
    f.px = row4(f0, px, py, pz, 1.0f); f.py = row4(f1, px, py, pz, 1.0f);
    f.pz = row4(f2, px, py, pz, 1.0f); f.pw = row4(f3, px, py, pz, 1.0f);
    f.n = normalize(v3(row3(f0, nobj.x, nobj.y, nobj.z), row3(f1, nobj.x, nobj.y, nobj.z),
                       row3(f2, nobj.x, nobj.y, nobj.z)));
    f.inst = sc.insts[rank].inst_id;
    return f;
}

}  // namespace pico
