// The physical estimator (PICO_ESTIMATOR_PHYSICAL): no counterpart in the reference.
//
// BSDF at a shading point with unit normal n facing the viewer:
//   f(v, l) = diffuse / pi + F(v.h) D(h) G2(v, l) / (4 (n.v)(n.l))
// with GGX (Trowbridge-Reitz) D, alpha = max(roughness^2, 1e-3), the Smith
// height-correlated masking-shadowing G2 = 1 / (1 + Lambda(v) + Lambda(l)) and
// Schlick's Fresnel F = F0 + (1 - F0)(1 - v.h)^5 (Walter et al. 2007, "Microfacet
// models for refraction through rough surfaces"; Heitz 2014, "Understanding the
// masking-shadowing function in microfacet-based BRDFs").  Diffuse kinds have
// F0 = 0, Specular kinds no diffuse term, Dielectric kinds both; Transparent and
// Fresnel kinds are a rough dielectric interface (sample_dielectric).
//
// Sampling picks the GGX lobe with probability p = sum(F0) / (sum(F0) + sum(diffuse)),
// else the cosine lobe.  The GGX lobe samples a visible normal (Heitz 2018,
// "Sampling the GGX distribution of visible normals") and reflects v about it, so
// its density is pdf_s(l) = G1(v) D(h) / (4 n.v); the density of the sample is the
// mixture (1 - p) n.l / pi + p pdf_s(l), and the throughput weight f (n.l) / pdf.
// Directions are handled in an orthonormal frame around n (Duff et al. 2017,
// "Building an orthonormal basis, revisited").
#pragma once

#include "shade.cuh"

namespace pico {
namespace phys {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kMinAlpha = 1e-3f;

struct Frame {
    float3 t, b, n;
};

__device__ __forceinline__ Frame frame_of(float3 n)
{
    const float sign = copysignf(1.0f, n.z);
    const float a = -1.0f / (sign + n.z);
    const float b = n.x * n.y * a;
    Frame f;
    f.t = make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f.b = make_float3(b, sign + n.y * n.y * a, -n.y);
    f.n = n;
    return f;
}

__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

__device__ __forceinline__ float3 to_local(const Frame& f, float3 v)
{
    return make_float3(dot3(v, f.t), dot3(v, f.b), dot3(v, f.n));
}

__device__ __forceinline__ float3 to_world(const Frame& f, float3 v)
{
    return make_float3(v.x * f.t.x + v.y * f.b.x + v.z * f.n.x, v.x * f.t.y + v.y * f.b.y + v.z * f.n.y,
                       v.x * f.t.z + v.y * f.b.z + v.z * f.n.z);
}

__device__ __forceinline__ float3 normalize3(float3 v)
{
    const float r = rsqrtf(dot3(v, v));
    return make_float3(v.x * r, v.y * r, v.z * r);
}

struct Lobes {
    float3 diffuse, f0;
    float alpha, p_spec;
};

// The lobes of a supported BSRDF kind (Diffuse, Specular or Dielectric).
__device__ __forceinline__ Lobes lobes_of(uint32_t kind, const GpuMaterial& m)
{
    Lobes l;
    const bool diffuse = kind != PICO_BSDF_SPECULAR, spec = kind != PICO_BSDF_DIFFUSE;
    l.diffuse = diffuse ? make_float3(m.diffuse[0], m.diffuse[1], m.diffuse[2]) : make_float3(0.0f, 0.0f, 0.0f);
    l.f0 = spec ? make_float3(m.specular[0], m.specular[1], m.specular[2]) : make_float3(0.0f, 0.0f, 0.0f);
    l.alpha = fmaxf(m.roughness * m.roughness, kMinAlpha);
    const float s = l.f0.x + l.f0.y + l.f0.z, d = l.diffuse.x + l.diffuse.y + l.diffuse.z;
    l.p_spec = (s + d > 0.0f) ? s / (s + d) : 0.0f;
    return l;
}

// GGX distribution of a local half vector h (unit): alpha^2 / (pi (sin^2 + alpha^2 cos^2)^2),
// the sine taken from the tangential components so that it stays accurate near the pole.
__device__ __forceinline__ float ggx_d(float3 h, float a2)
{
    if (h.z <= 0.0f) return 0.0f;
    const float k = (h.x * h.x + h.y * h.y) + a2 * (h.z * h.z);
    return a2 / (kPi * k * k);
}

// Smith Lambda of a local direction w: (sqrt(1 + alpha^2 tan^2) - 1) / 2.
__device__ __forceinline__ float ggx_lambda(float3 w, float a2)
{
    const float c2 = w.z * w.z;
    const float t2 = (w.x * w.x + w.y * w.y) / c2;
    return 0.5f * (sqrtf(1.0f + a2 * t2) - 1.0f);
}

__device__ __forceinline__ float schlick(float f0, float c)
{
    const float m = fminf(fmaxf(1.0f - c, 0.0f), 1.0f);
    const float m2 = m * m;
    return f0 + (1.0f - f0) * (m2 * m2 * m);
}

// f(v, l) and the sampling density of l, both in the local frame (v.z > 0).
__device__ __forceinline__ void eval(const Lobes& lb, float3 v, float3 l, float3& f, float& pdf)
{
    f = make_float3(0.0f, 0.0f, 0.0f);
    pdf = 0.0f;
    if (v.z <= 0.0f || l.z <= 0.0f) return;
    const float inv_pi = 1.0f / kPi;
    f = make_float3(lb.diffuse.x * inv_pi, lb.diffuse.y * inv_pi, lb.diffuse.z * inv_pi);
    pdf = (1.0f - lb.p_spec) * l.z * inv_pi;
    if (lb.p_spec > 0.0f) {
        const float3 h = normalize3(make_float3(v.x + l.x, v.y + l.y, v.z + l.z));
        const float a2 = lb.alpha * lb.alpha;
        const float D = ggx_d(h, a2);
        const float lv = ggx_lambda(v, a2), ll = ggx_lambda(l, a2);
        const float vh = fmaxf(dot3(v, h), 0.0f);
        const float g = D / ((1.0f + lv + ll) * 4.0f * v.z * l.z);
        f.x += schlick(lb.f0.x, vh) * g;
        f.y += schlick(lb.f0.y, vh) * g;
        f.z += schlick(lb.f0.z, vh) * g;
        pdf += lb.p_spec * D / ((1.0f + lv) * 4.0f * v.z);
    }
}

// A visible normal of the GGX distribution seen from local v (Heitz 2018, isotropic alpha).
__device__ __forceinline__ float3 sample_vndf(float3 v, float alpha, float u1, float u2)
{
    const float3 vh = normalize3(make_float3(alpha * v.x, alpha * v.y, v.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    float3 t1 = make_float3(1.0f, 0.0f, 0.0f);
    if (lensq > 0.0f) {
        const float r = rsqrtf(lensq);
        t1 = make_float3(-vh.y * r, vh.x * r, 0.0f);
    }
    const float3 t2 = make_float3(vh.y * t1.z - vh.z * t1.y, vh.z * t1.x - vh.x * t1.z, vh.x * t1.y - vh.y * t1.x);
    const float r = sqrtf(u1);
    float sn, cs;
    sincosf(2.0f * kPi * u2, &sn, &cs);
    const float p1 = r * cs;
    float p2 = r * sn;
    const float s = 0.5f * (1.0f + vh.z);
    p2 = (1.0f - s) * sqrtf(fmaxf(1.0f - p1 * p1, 0.0f)) + s * p2;
    const float pz = sqrtf(fmaxf(1.0f - p1 * p1 - p2 * p2, 0.0f));
    const float3 nh = make_float3(p1 * t1.x + p2 * t2.x + pz * vh.x, p1 * t1.y + p2 * t2.y + pz * vh.y,
                                  p1 * t1.z + p2 * t2.z + pz * vh.z);
    return normalize3(make_float3(alpha * nh.x, alpha * nh.y, fmaxf(nh.z, 0.0f)));
}

struct Sample {
    float3 l;        // local direction
    float3 weight;   // f (n.l) / pdf
    float pdf;
    bool ok;
};

// One sample of the mixture from three uniforms in [0, 1).
__device__ __forceinline__ Sample sample(const Lobes& lb, float3 v, float u0, float u1, float u2)
{
    Sample s;
    s.ok = false;
    s.pdf = 0.0f;
    s.weight = make_float3(0.0f, 0.0f, 0.0f);
    s.l = make_float3(0.0f, 0.0f, 1.0f);
    if (v.z <= 0.0f || (lb.p_spec <= 0.0f && lb.diffuse.x + lb.diffuse.y + lb.diffuse.z <= 0.0f)) return s;
    if (u0 < lb.p_spec) {
        const float3 h = sample_vndf(v, lb.alpha, u1, u2);
        const float vh = dot3(v, h);
        s.l = make_float3(2.0f * vh * h.x - v.x, 2.0f * vh * h.y - v.y, 2.0f * vh * h.z - v.z);
    } else {
        const float r = sqrtf(u1);
        float sn, cs;
        sincosf(2.0f * kPi * u2, &sn, &cs);
        s.l = make_float3(r * cs, r * sn, sqrtf(fmaxf(1.0f - u1, 0.0f)));
    }
    if (s.l.z <= 0.0f) return s;
    float3 f;
    eval(lb, v, s.l, f, s.pdf);
    if (!(s.pdf > 0.0f)) return s;
    const float k = s.l.z / s.pdf;
    s.weight = make_float3(f.x * k, f.y * k, f.z * k);
    s.ok = true;
    return s;
}

// Exact dielectric Fresnel reflectance of unpolarised light at an interface with
// relative index eta = eta_i / eta_t, for cos_i > 0 the cosine on the incident side;
// 1 under total internal reflection.
__device__ __forceinline__ float fresnel_dielectric(float cos_i, float eta)
{
    const float sin2_t = eta * eta * fmaxf(1.0f - cos_i * cos_i, 0.0f);
    if (sin2_t >= 1.0f) return 1.0f;
    const float cos_t = sqrtf(1.0f - sin2_t);
    const float rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const float rp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return 0.5f * (rs * rs + rp * rp);
}

// The reference's Transparent and Fresnel kinds as a rough dielectric interface
// (Walter et al. 2007; GGX, visible-normal sampling).  v: local direction towards
// the viewer (v.z > 0); eta = eta_i / eta_t for the side v lies on.  A visible
// microfacet normal h is sampled; the Fresnel kind reflects about it with
// probability F(v.h) and refracts otherwise, the Transparent kind always refracts
// (it has no reflection lobe) but under total internal reflection, where both
// reflect.  With the sampling probabilities equal to the lobes' weights the
// throughput factor is G2(v, l) / G1(v) for a reflection and tint G2 / G1 eta^2
// for a refraction (eta^2: radiance transport across the interface).  The lobe
// is never evaluated: vertices on it take no next-event estimation, like mirrors.
struct DielectricSample {
    float3 l;        // local direction, l.z < 0 when refracted
    float3 weight;
    bool ok, refracted;
};

__device__ __forceinline__ DielectricSample sample_dielectric(float3 v, float alpha, float eta, float3 tint,
                                                              bool reflect_lobe, float u0, float u1, float u2)
{
    DielectricSample s;
    s.ok = false;
    s.refracted = false;
    s.weight = make_float3(0.0f, 0.0f, 0.0f);
    s.l = make_float3(0.0f, 0.0f, 1.0f);
    if (v.z <= 0.0f) return s;
    const float3 h = sample_vndf(v, alpha, u1, u2);
    const float vh = dot3(v, h);
    if (vh <= 0.0f) return s;
    const float F = fresnel_dielectric(vh, eta);
    const float a2 = alpha * alpha;
    const float lv = ggx_lambda(v, a2);
    if (F >= 1.0f || (reflect_lobe && u0 < F)) {
        s.l = make_float3(2.0f * vh * h.x - v.x, 2.0f * vh * h.y - v.y, 2.0f * vh * h.z - v.z);
        if (s.l.z <= 0.0f) return s;
        const float g = (1.0f + lv) / (1.0f + lv + ggx_lambda(s.l, a2));
        s.weight = make_float3(g, g, g);
    } else {
        const float cos_t = sqrtf(fmaxf(1.0f - eta * eta * (1.0f - vh * vh), 0.0f));
        const float k = eta * vh - cos_t;
        s.l = normalize3(make_float3(k * h.x - eta * v.x, k * h.y - eta * v.y, k * h.z - eta * v.z));
        if (s.l.z >= 0.0f) return s;
        const float g = (1.0f + lv) / (1.0f + lv + ggx_lambda(s.l, a2)) * eta * eta;
        s.weight = make_float3(tint.x * g, tint.y * g, tint.z * g);
        s.refracted = true;
    }
    s.ok = true;
    return s;
}

// Power-heuristic weight of a sample drawn with density a against a rival density b:
// a^2 / (a^2 + b^2), written so that very large densities cannot overflow.
__device__ __forceinline__ float mis_weight(float a, float b)
{
    if (!(a > 0.0f)) return 0.0f;
    const float r = b / a;
    return 1.0f / (1.0f + r * r);
}

// Offset of a new ray's origin along the shading normal: relative to the position's magnitude.
__device__ __forceinline__ float ray_offset(float px, float py, float pz)
{
    return 1e-4f * (1.0f + fmaxf(fmaxf(fabsf(px), fabsf(py)), fabsf(pz)));
}

}  // namespace phys
}  // namespace pico
