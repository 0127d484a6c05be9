/*
 * Oracle (test infrastructure only): sampling, shading and the integrator.
 *
 *   xorshift_random / Hammersley   Core/RandUtils.cpp:13-21, 27-33, 64-90
 *   std::mt19937_64 + uniform_real_distribution<float> (the Integrator's mGenerator,
 *   Render/Integrators.hpp:49-50): the published MT19937-64 recurrence and tempering,
 *   and libstdc++'s generate_canonical<float, 24> (one 64-bit draw scaled by 2^-64,
 *   clamped below 1)
 *   Camera::generate_ray           Core/Camera.cpp:11-28, Core/Camera.hpp:64-65
 *   tangent frame                  Core/vectorUtils.cpp:9-35, Core/vectorUtils.hpp:24-76
 *   distributions                  Render/Distributions.cpp:14-78
 *   BSRDF lobes                    Render/BSRDF.cpp:11-214
 *   reflectance                    Core/MaterialManager.hpp:30-45
 *   alias table                    Util/AliasTable.cpp:12-104
 *   light sampling                 Core/LowerLevelMeshBVH.cpp:92-132
 *   integrator                     Render/Integrators.cpp:13-22, 46-209
 *   per-pixel sample loop          Core/Scene.cpp:164-198
 *
 * Where the reference calls a double-precision libm routine on a float
 * (for example the unqualified cos/sin/sqrt of the cosine lobe, or sin() of
 * the degree-scaled angle in the triangle weights), the restatement does too.
 */
#include "po_internal.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------ threads */
typedef struct {
    size_t count, stride; char* items; void (*fn)(void*);
    size_t next; pthread_mutex_t lock;
} pf_ctx;

static void* pf_worker(void* p)
{
    pf_ctx* c = (pf_ctx*)p;
    for (;;) {
        pthread_mutex_lock(&c->lock);
        const size_t i = c->next++;
        pthread_mutex_unlock(&c->lock);
        if (i >= c->count) break;
        c->fn(c->items + i * c->stride);
    }
    return NULL;
}

void po_parallel_for(size_t count, void* items, size_t stride, void (*fn)(void*), int nthreads)
{
    if (nthreads <= 0) nthreads = (int)sysconf(_SC_NPROCESSORS_ONLN);
    if (nthreads < 1) nthreads = 1;
    if ((size_t)nthreads > count) nthreads = (int)(count ? count : 1);
    pf_ctx c;
    c.count = count; c.stride = stride; c.items = (char*)items; c.fn = fn; c.next = 0;
    pthread_mutex_init(&c.lock, NULL);
    if (nthreads == 1) {
        pf_worker(&c);
    } else {
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int i = 0; i < nthreads; ++i) pthread_create(&th[i], NULL, pf_worker, &c);
        for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
        free(th);
    }
    pthread_mutex_destroy(&c.lock);
}

/* ------------------------------------------------------------ random streams */
static uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

void po_xorshift_seed(uint32_t seed, uint32_t st[4])
{
    st[0] = rotl32(seed, 3); st[1] = rotl32(seed, 7);
    st[2] = rotl32(seed, 11); st[3] = rotl32(seed, 13);
}

uint32_t po_xorshift_next(uint32_t st[4])
{
    const uint32_t result = rotl32(st[0] + st[3], 7) + st[0];
    const uint32_t t = st[1] << 9;
    st[2] ^= st[0];
    st[3] ^= st[1];
    st[1] ^= st[2];
    st[0] ^= st[3];
    st[2] ^= t;
    st[3] = rotl32(st[3], 11);
    return result;
}

float po_radical_inverse(uint32_t bits)
{
    bits = (bits << 16u) | (bits >> 16u);
    bits = ((bits & 0x55555555u) << 1u) | ((bits & 0xAAAAAAAAu) >> 1u);
    bits = ((bits & 0x33333333u) << 2u) | ((bits & 0xCCCCCCCCu) >> 2u);
    bits = ((bits & 0x0F0F0F0Fu) << 4u) | ((bits & 0xF0F0F0F0u) >> 4u);
    bits = ((bits & 0x00FF00FFu) << 8u) | ((bits & 0xFF00FF00u) >> 8u);
    return (float)((double)(float)bits * 2.3283064365386963e-10);
}

/* hammersley(i, N) with N = 2^32 - 1 (RandUtils.cpp:23-27, 87-90). */
void po_hammersley_next(uint32_t st[4], float* xi)
{
    const uint32_t i = po_xorshift_next(st);
    xi[0] = (float)i / (float)4294967295u;
    xi[1] = po_radical_inverse(i);
}

void po_uniform_sample_triangle(const float* xi, float* out)
{
    const float su0 = sqrtf(xi[0]);
    out[0] = 1 - su0;
    out[1] = xi[1] * su0;
}

#define MT_N 312
#define MT_M 156
void po_mt64_seed(uint64_t* st, uint64_t seed)
{
    st[0] = seed;
    for (int i = 1; i < MT_N; ++i)
        st[i] = 6364136223846793005ULL * (st[i - 1] ^ (st[i - 1] >> 62)) + (uint64_t)i;
    st[MT_N] = MT_N;   /* index: forces a regeneration on the first draw */
}

static uint64_t mt64_next(uint64_t* st)
{
    const uint64_t upper = ~0ULL << 31, lower = ~upper, A = 0xb5026f5aa96619e9ULL;
    if (st[MT_N] >= MT_N) {
        int k;
        for (k = 0; k < MT_N - MT_M; ++k) {
            const uint64_t y = (st[k] & upper) | (st[k + 1] & lower);
            st[k] = st[k + MT_M] ^ (y >> 1) ^ ((y & 1ULL) ? A : 0ULL);
        }
        for (; k < MT_N - 1; ++k) {
            const uint64_t y = (st[k] & upper) | (st[k + 1] & lower);
            st[k] = st[k + (MT_M - MT_N)] ^ (y >> 1) ^ ((y & 1ULL) ? A : 0ULL);
        }
        const uint64_t y = (st[MT_N - 1] & upper) | (st[0] & lower);
        st[MT_N - 1] = st[MT_M - 1] ^ (y >> 1) ^ ((y & 1ULL) ? A : 0ULL);
        st[MT_N] = 0;
    }
    uint64_t z = st[st[MT_N]++];
    z ^= (z >> 29) & 0x5555555555555555ULL;
    z ^= (z << 17) & 0x71d67fffeda60000ULL;
    z ^= (z << 37) & 0xfff7eee000000000ULL;
    z ^= z >> 43;
    return z;
}

float po_mt64_uniform(uint64_t* st)
{
    const float sum = (float)mt64_next(st) * 1.0f;
    float r = sum / 18446744073709551616.0f;
    if (r >= 1.0f) r = nextafterf(1.0f, 0.0f);
    return r * (1.0f - 0.0f) + 0.0f;
}

/* ------------------------------------------------------------ camera */
void po_generate_ray(const po_camera* c, float xi_x, float xi_y, uint32_t px, uint32_t py, po_ray* out)
{
    const float rx = xi_x / 2.0f, ry = xi_y / 2.0f;
    const float dx = (((float)px + rx) / (float)c->resolution[0] - 0.5f) * c->aspect;
    const float dy = ((float)py + ry) / (float)c->resolution[1] - 0.5f;
    const float dz = 1.0f;
    const po_v3 D = v3(c->direction[0], c->direction[1], c->direction[2]);
    const po_v3 U = v3(c->up[0], c->up[1], c->up[2]);
    const po_v3 R = v3_cross(v3_normalize(D), U);
    const po_v3 d = v3_normalize(v3_add(v3_add(v3_scale(D, dz), v3_scale(U, dy)), v3_scale(R, dx)));
    out->org[0] = c->position[0]; out->org[1] = c->position[1]; out->org[2] = c->position[2];
    out->org[3] = 1.0f;
    out->dir[0] = d.x; out->dir[1] = d.y; out->dir[2] = d.z; out->dir[3] = c->far_plane;
}

/* ------------------------------------------------------------ tangent space */
static po_m3 tangent_frame(po_v3 V, po_v3 N)
{
    po_v3 t;
    if (fabsf(v3_dot(V, N)) > 0.95f) {
        const po_v3 vv = fabsf(N.z) > 0.99f ? v3(1, 0, 0) : v3(0, 0, 1);
        t = v3_normalize(v3_cross(N, vv));
    } else {
        t = v3_normalize(v3_cross(V, N));
    }
    const po_v3 b = v3_normalize(v3_cross(t, N));
    po_m3 m;   /* transpose(mat3(t, b, N)) */
    m.m[0][0] = t.x; m.m[1][0] = t.y; m.m[2][0] = t.z;
    m.m[0][1] = b.x; m.m[1][1] = b.y; m.m[2][1] = b.z;
    m.m[0][2] = N.x; m.m[1][2] = N.y; m.m[2][2] = N.z;
    return m;
}

void po_tangent_frame(const float* V, const float* N, float* out)
{
    po_m3 m = tangent_frame(v3(V[0], V[1], V[2]), v3(N[0], N[1], N[2]));
    memcpy(out, m.m, sizeof(float) * 9);
}

/* glm compute_inverse<3,3> (glm/detail/func_matrix.inl:272-294). */
static po_m3 m3_inverse(const po_m3* a)
{
    const float (*m)[3] = a->m;
    const float det = ((+m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]))
                       - m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]))
                      + m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
    const float o = 1.0f / det;
    po_m3 r;
    r.m[0][0] = +(m[1][1] * m[2][2] - m[2][1] * m[1][2]) * o;
    r.m[1][0] = -(m[1][0] * m[2][2] - m[2][0] * m[1][2]) * o;
    r.m[2][0] = +(m[1][0] * m[2][1] - m[2][0] * m[1][1]) * o;
    r.m[0][1] = -(m[0][1] * m[2][2] - m[2][1] * m[0][2]) * o;
    r.m[1][1] = +(m[0][0] * m[2][2] - m[2][0] * m[0][2]) * o;
    r.m[2][1] = -(m[0][0] * m[2][1] - m[2][0] * m[0][1]) * o;
    r.m[0][2] = +(m[0][1] * m[1][2] - m[1][1] * m[0][2]) * o;
    r.m[1][2] = -(m[0][0] * m[1][2] - m[1][0] * m[0][2]) * o;
    r.m[2][2] = +(m[0][0] * m[1][1] - m[1][0] * m[0][1]) * o;
    return r;
}

/* ------------------------------------------------------------ distributions */
static po_v3 cos_sample(const float* xi)
{
    const float u1 = xi[0], u2 = xi[1];
    const float r = sqrtf(u1);
    const float phi = (float)((double)u2 * M_PI * 2.0f);
    const float one_minus = (0.0f < 1.0f - u1) ? 1.0f - u1 : 0.0f;
    return v3_normalize(v3((float)((double)r * cos((double)phi)), (float)((double)r * sin((double)phi)),
                           (float)sqrt((double)one_minus)));
}
static float cos_pdf(po_v3 H)
{
    const float c = H.z / (float)M_PI;
    return (0.0f < c) ? c : 0.0f;
}

static po_v3 beckmann_sample(const float* xi, po_v3 V, float R)
{
    const float alpha = R * R;
    float log_sample = logf(1.0f - xi[0]);
    if (isinf(log_sample)) log_sample = 0;
    const float tan2 = -alpha * alpha * log_sample;
    const float phi = (float)((double)(xi[1] * 2.0f) * M_PI);
    const float cos_t = 1.0f / sqrtf(1.0f + tan2);
    const float s2 = 1.0f - cos_t * cos_t;
    const float sin_t = sqrtf((0.0f < s2) ? s2 : 0.0f);
    po_v3 H = v3(sin_t * cosf(phi), sin_t * sinf(phi), cos_t);
    if (!(V.z * H.z > 0.0f)) H = v3_neg(H);
    return v3_normalize(H);
}

static float roughness_to_alpha(float r)
{
    r = (r < (float)1e-3) ? (float)1e-3 : r;
    const float x = logf(r);
    return 1.62142f + 0.819955f * x + 0.1734f * x * x + 0.0171201f * x * x * x +
           0.000640711f * x * x * x * x;
}

static float clampf(float v, float lo, float hi) { return (v < lo) ? lo : ((hi < v) ? hi : v); }

static float beckmann_D(po_v3 w, float R)
{
    const float ax = roughness_to_alpha(R), ay = ax;
    const float cos2 = w.z * w.z;
    const float s2 = 1.0f - cos2;
    const float sin2 = (0.0f < s2) ? s2 : 0.0f;
    const float tan2 = sin2 / cos2;
    if (isinf(tan2)) return 0.0f;
    const float cos4 = cos2 * cos2;
    const float sin_t = sqrtf(sin2);
    const float cphi = (sin_t == 0) ? 1 : clampf(w.x / sin_t, -1.0f, 1.0f);
    const float sphi = (sin_t == 0) ? 0 : clampf(w.y / sin_t, -1.0f, 1.0f);
    const float cos2phi = cphi * cphi, sin2phi = sphi * sphi;
    const float e = expf(-tan2 * (cos2phi / (ax * ax) + sin2phi / (ay * ay)));
    return (float)((double)e / (M_PI * ax * ay * cos4));
}

static float beckmann_pdf(po_v3 H, float R)
{
    float d = beckmann_D(H, R);
    d = clampf(d, 0.0f, 1.0f);
    return d * fabsf(H.z);
}

void po_cos_sample(const float* xi, float* H) { po_v3 h = cos_sample(xi); H[0] = h.x; H[1] = h.y; H[2] = h.z; }
float po_cos_pdf(const float* H) { return cos_pdf(v3(H[0], H[1], H[2])); }
void po_beckmann_sample(const float* xi, const float* V, float R, float* H)
{
    po_v3 h = beckmann_sample(xi, v3(V[0], V[1], V[2]), R);
    H[0] = h.x; H[1] = h.y; H[2] = h.z;
}
float po_beckmann_pdf(const float* H, float R) { return beckmann_pdf(v3(H[0], H[1], H[2]), R); }

/* ------------------------------------------------------------ BSRDFs */
static float reflectance(const po_material* m)
{
    const float s = v3_length(v3(m->specular[0], m->specular[1], m->specular[2]));
    const float d = v3_length(v3(m->diffuse[0], m->diffuse[1], m->diffuse[2]));
    return s / (s + d);
}

static float bsdf_pdf(int type, po_v3 wo, po_v3 H, float roughness, float refl)
{
    switch (type) {
    case PO_DIFFUSE: return cos_pdf(H);
    case PO_SPECULAR: return beckmann_pdf(H, roughness) / (2.0f * v3_dot(wo, H));
    case PO_DIELECTRIC:
        return (cos_pdf(H) * (1 - refl)) + ((beckmann_pdf(H, roughness) / (2.0f * v3_dot(wo, H))) * refl);
    case PO_LIGHT: return cos_pdf(H);
    default: return 0.0f;
    }
}

float po_bsdf_pdf(int bsdf, const float* wo, const float* H, float roughness, float refl)
{
    return bsdf_pdf(bsdf, v3(wo[0], wo[1], wo[2]), v3(H[0], H[1], H[2]), roughness, refl);
}

static po_v3 reflect3(po_v3 I, po_v3 N)
{
    const float d = v3_dot(N, I);
    return v3(I.x - (N.x * d) * 2.0f, I.y - (N.y * d) * 2.0f, I.z - (N.z * d) * 2.0f);
}

typedef struct { po_v3 L; float P; po_v3 energy; } bsdf_sample;

/* next2() supplies successive Hammersley points; `ctx` is the generator. */
typedef void (*next2_fn)(void* ctx, float* xi);

/* Core::Ray's index-of-refraction stack (AABB.cpp:54-81): camera rays start with 1.0
 * (Camera.cpp:23).  Popping an empty stack or reading it empty is undefined in the
 * reference; here the pop is ignored and the read gives 1.0. */
#define PO_IOR_MAX 64
typedef struct { float v[PO_IOR_MAX]; uint32_t n; } po_ior_stack;
static void ior_push(po_ior_stack* s, float x) { if (s->n < PO_IOR_MAX) s->v[s->n] = x; s->n++; }
static void ior_pop(po_ior_stack* s) { if (s->n) s->n--; }
static float ior_top(const po_ior_stack* s)
{
    return s->n ? s->v[(s->n < PO_IOR_MAX ? s->n : PO_IOR_MAX) - 1] : 1.0f;
}
static int ior_inside(const po_ior_stack* s) { return s->n > 1; }

/* glm::refract (glm/detail/func_geometric.inl:119-127): the product with (k >= 0) keeps a
 * NaN from sqrt of a negative k, so total internal reflection gives a NaN vector. */
static po_v3 refract3(po_v3 I, po_v3 N, float eta)
{
    const float d = v3_dot(N, I);
    const float k = 1.0f - eta * eta * (1.0f - d * d);
    const float s = eta * d + sqrtf(k);
    const float g = (float)(k >= 0.0f);
    return v3((eta * I.x - s * N.x) * g, (eta * I.y - s * N.y) * g, (eta * I.z - s * N.z) * g);
}

/* Transparent_BTDF::sample (BSRDF.cpp:238-297). */
static bsdf_sample transparent_sample(const po_material* mat, po_v3 V, po_v3 N, po_ior_stack* ior,
                                      next2_fn next2, void* ctx)
{
    const po_m3 w2t = tangent_frame(V, N);
    const po_m3 t2w = m3_inverse(&w2t);
    const po_v3 vt = v3_normalize(m3_mul_v3(&w2t, V));
    const int enter = vt.z >= 0.0f;
    float xi[2];
    next2(ctx, xi);
    const po_v3 H = beckmann_sample(xi, vt, mat->roughness);
    const float eta = 1.0f / mat->index_of_refraction;
    if (enter) ior_push(ior, mat->index_of_refraction); else ior_pop(ior);
    const po_v3 L = refract3(vt, H, eta);
    bsdf_sample s;
    s.L = v3_normalize(m3_mul_v3(&t2w, L));
    const float pdf = beckmann_pdf(H, mat->roughness);
    const po_v3 wh = v3_normalize(v3_add(vt, v3_scale(L, eta)));
    const float denom = v3_dot(vt, wh) + eta * v3_dot(L, wh);
    const float dwh_dwi = fabsf((eta * eta * v3_dot(L, wh)) / (denom * denom));
    s.P = pdf * dwh_dwi;
    s.energy = v3(mat->diffuse[0], mat->diffuse[1], mat->diffuse[2]);
    return s;
}

/* Fresnel_BTDF::fresnel_factor (BSRDF.cpp:395-421). */
static float fresnel_factor(float cos_i, float eta_i, float eta_t)
{
    cos_i = clampf(cos_i, -1.0f, 1.0f);
    if (!(cos_i > 0.0f)) {
        const float tmp = eta_i; eta_i = eta_t; eta_t = tmp;
        cos_i = fabsf(cos_i);
    }
    const float sin_i = sqrtf((0.0f < 1.0f - cos_i * cos_i) ? 1.0f - cos_i * cos_i : 0.0f);
    const float sin_t = eta_i / eta_t * sin_i;
    const float cos_t = sqrtf((0.0f < 1.0f - sin_t * sin_t) ? 1.0f - sin_t * sin_t : 0.0f);
    const float rparl = ((eta_t * cos_i) - (eta_i * cos_t)) / ((eta_t * cos_i) + (eta_i * cos_t));
    const float rperp = ((eta_i * cos_i) - (eta_t * cos_t)) / ((eta_i * cos_i) + (eta_t * cos_t));
    return (rparl * rparl + rperp * rperp) / 2;
}

static bsdf_sample sample_bsdf(int type, const po_material* mat, po_v3 V, po_v3 N,
                               next2_fn next2, void* ctx, po_ior_stack* ior)
{
    if (type == PO_DELTA) {                                /* BSRDF.cpp:216-229 */
        bsdf_sample s;
        s.energy = v3(mat->specular[0], mat->specular[1], mat->specular[2]);
        s.L = reflect3(v3_neg(V), N);
        s.P = 1.0f;
        return s;
    }
    if (type == PO_BTDF) return transparent_sample(mat, V, N, ior, next2, ctx);
    if (type == PO_FRESNEL) {                              /* BSRDF.cpp:364-385 */
        const po_m3 w2t = tangent_frame(V, N);
        const po_v3 vt = v3_normalize(m3_mul_v3(&w2t, V));
        float xi[2];
        next2(ctx, xi);
        const float F = fresnel_factor(vt.z, mat->index_of_refraction, ior_top(ior));
        bsdf_sample s;
        if (xi[0] < F) {
            s = sample_bsdf(PO_SPECULAR, mat, V, N, next2, ctx, ior);
            s.P *= F;
        } else {
            s = transparent_sample(mat, V, N, ior, next2, ctx);
            s.P *= 1.0f - F;
        }
        return s;
    }
    const po_m3 w2t = tangent_frame(V, N);
    const po_m3 t2w = m3_inverse(&w2t);
    const po_v3 vt = v3_normalize(m3_mul_v3(&w2t, V));
    const po_v3 diffuse = v3(mat->diffuse[0], mat->diffuse[1], mat->diffuse[2]);
    const po_v3 specular = v3(mat->specular[0], mat->specular[1], mat->specular[2]);
    const po_v3 emissive = v3(mat->emissive[0], mat->emissive[1], mat->emissive[2]);
    bsdf_sample s;
    float xi[2];
    if (type == PO_DIFFUSE || type == PO_LIGHT) {          /* BSRDF.cpp:11-40, 173-202 */
        next2(ctx, xi);
        const po_v3 H = cos_sample(xi);
        s.P = cos_pdf(H);
        s.L = v3_normalize(m3_mul_v3(&t2w, H));
        s.energy = type == PO_DIFFUSE ? diffuse : emissive;
    } else if (type == PO_SPECULAR) {                      /* BSRDF.cpp:54-84 */
        next2(ctx, xi);
        const po_v3 H = beckmann_sample(xi, vt, mat->roughness);
        const po_v3 L = v3_normalize(reflect3(v3_neg(vt), H));
        s.L = v3_normalize(m3_mul_v3(&t2w, L));
        s.P = bsdf_pdf(PO_SPECULAR, vt, H, mat->roughness, reflectance(mat));
        s.energy = specular;
    } else {                                               /* BSRDF.cpp:100-149 */
        const float prop = reflectance(mat);
        next2(ctx, xi);
        if (xi[1] >= prop) {
            next2(ctx, xi);
            const po_v3 H = cos_sample(xi);
            s.L = v3_normalize(m3_mul_v3(&t2w, H));
            s.P = cos_pdf(H);
            s.energy = diffuse;
        } else {
            next2(ctx, xi);
            const po_v3 H = beckmann_sample(xi, vt, mat->roughness);
            const po_v3 L = v3_normalize(reflect3(v3_neg(vt), H));
            s.L = v3_normalize(m3_mul_v3(&t2w, L));
            s.P = beckmann_pdf(H, mat->roughness) / (2.0f * v3_dot(vt, H));
            s.energy = specular;
        }
    }
    return s;
}

typedef struct { const float* xi; int used; } fixed_xi;
static void fixed_next2(void* p, float* xi)
{
    fixed_xi* f = (fixed_xi*)p;
    xi[0] = f->xi[2 * f->used];
    xi[1] = f->xi[2 * f->used + 1];
    f->used++;
}

void po_bsdf_sample(int bsdf, const po_material* mat, const float* V, const float* N,
                    const float* xi, float* L, float* P, float* energy)
{
    fixed_xi f = {xi, 0};
    po_ior_stack ior = {{1.0f}, 1};
    bsdf_sample s = sample_bsdf(bsdf, mat, v3(V[0], V[1], V[2]), v3(N[0], N[1], N[2]), fixed_next2, &f, &ior);
    L[0] = s.L.x; L[1] = s.L.y; L[2] = s.L.z;
    *P = s.P;
    energy[0] = s.energy.x; energy[1] = s.energy.y; energy[2] = s.energy.z;
}

/* direct_lighting_pdf (Integrators.cpp:13-22). */
static float direct_pdf(int type, const po_material* mat, po_v3 N, po_v3 wi, po_v3 wo)
{
    const po_m3 t = tangent_frame(wi, N);
    const po_v3 two = m3_mul_v3(&t, wo);
    po_v3 H = v3_normalize(v3_add(wi, wo));
    H = m3_mul_v3(&t, H);
    return bsdf_pdf(type, two, H, mat->roughness, reflectance(mat));
}

float po_direct_lighting_pdf(int bsdf, const po_material* mat, const float* N, const float* wi, const float* wo)
{
    return direct_pdf(bsdf, mat, v3(N[0], N[1], N[2]), v3(wi[0], wi[1], wi[2]), v3(wo[0], wo[1], wo[2]));
}

/* ------------------------------------------------------------ light sampling */
void po_triangle_weights(const po_mesh_desc* m, float* w)
{
    for (uint32_t t = 0; t < m->ntris; ++t) {
        const float* pa = m->positions + 3 * m->indices[3 * t];
        const float* pb = m->positions + 3 * m->indices[3 * t + 1];
        const float* pc = m->positions + 3 * m->indices[3 * t + 2];
        const po_v3 a = v3(pa[0], pa[1], pa[2]), b = v3(pb[0], pb[1], pb[2]), c = v3(pc[0], pc[1], pc[2]);
        const po_v3 ac = v3_sub(a, c), bc = v3_sub(b, c);
        const float bc_len = v3_length(bc);
        const float base = v3_length(ac);
        const float theta = (float)sin((double)acosf(v3_dot(v3_normalize(ac), v3_normalize(bc))) *
                                       (180.0f / M_PI));
        const float height = theta * bc_len;
        w[t] = (base * height) / 2.0f;
    }
}

void po_alias_build(const float* weights, uint32_t n, float* bw, uint32_t* ba)
{
    double acc = 0.0;
    for (uint32_t i = 0; i < n; ++i) acc = acc + (double)weights[i];
    const float total = (float)acc;
    for (uint32_t i = 0; i < n; ++i) { bw[i] = weights[i] / total; ba[i] = 0; }
    float* over_p = (float*)malloc(sizeof(float) * (2 * n + 1));
    uint32_t* over_i = (uint32_t*)malloc(sizeof(uint32_t) * (2 * n + 1));
    float* under_p = (float*)malloc(sizeof(float) * (2 * n + 1));
    uint32_t* under_i = (uint32_t*)malloc(sizeof(uint32_t) * (2 * n + 1));
    uint32_t no = 0, nu = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const float p = bw[i] * (float)n;
        if (p < 1.0f) { under_p[nu] = p; under_i[nu++] = i; }
        else { over_p[no] = p; over_i[no++] = i; }
    }
    while (no && nu) {
        const float op = over_p[no - 1]; const uint32_t oi = over_i[no - 1]; --no;
        const float up = under_p[nu - 1]; const uint32_t ui = under_i[nu - 1]; --nu;
        bw[ui] = up;
        ba[ui] = oi;
        const float excess = up + op - 1.0f;
        if (excess < 1.0f) { under_p[nu] = excess; under_i[nu++] = oi; }
        else { over_p[no] = excess; over_i[no++] = oi; }
    }
    while (nu) { --nu; ba[under_i[nu]] = 0; bw[under_i[nu]] = 1.0f; }
    while (no) { --no; ba[over_i[no]] = 0; bw[over_i[no]] = 1.0f; }
    free(over_p); free(over_i); free(under_p); free(under_i);
}

void po_scene_build_light_tables(po_scene* s)
{
    for (uint32_t l = 0; l < s->nlights; ++l) {
        po_mesh* m = &s->meshes[s->instances[s->lights[l]].mesh];
        if (m->alias_weight || m->desc.shape != PO_SHAPE_TRIANGLES) continue;
        float* w = (float*)malloc(sizeof(float) * (m->desc.ntris ? m->desc.ntris : 1));
        po_triangle_weights(&m->desc, w);
        m->alias_n = m->desc.ntris;
        m->alias_weight = (float*)malloc(sizeof(float) * (m->alias_n ? m->alias_n : 1));
        m->alias_index = (uint32_t*)malloc(sizeof(uint32_t) * (m->alias_n ? m->alias_n : 1));
        po_alias_build(w, m->alias_n, m->alias_weight, m->alias_index);
        free(w);
    }
}

/* ------------------------------------------------------------ integrator */
typedef struct {
    const po_scene* s;
    uint64_t mt[MT_N + 1];
    uint32_t xs[4];        /* Hammersley_Generator's xorshift_random */
    uint32_t max_depth;
} integrator;

static void ham_next2(void* p, float* xi) { po_hammersley_next(((integrator*)p)->xs, xi); }

static const po_material* material_of(const po_scene* s, uint32_t inst)
{
    return &s->materials[s->instances[inst].material];
}

/* sample_geometry of the implicit shapes (LowerLevelImplicitShapesBVH.cpp:59-67, 93-112): a
 * uniform point on the radius-0.5 sphere (uniform_sample_sphere, RandUtils.cpp:43-49: phi in
 * double from M_PI, std::cos / std::sin of the float phi) or on a face of the unit cube. */
static po_v3 implicit_light_point(uint32_t shape, integrator* it)
{
    float xi[2];
    if (shape == PO_SHAPE_SPHERE) {
        po_hammersley_next(it->xs, xi);
        const float z = 1 - 2 * xi[0];
        const float r = sqrtf((0.0f < 1.0f - z * z) ? 1.0f - z * z : 0.0f);
        const float phi = (float)(2 * M_PI * (double)xi[1]);
        const po_v3 u = v3(r * cosf(phi), r * sinf(phi), z);
        return v3_scale(u, 0.5f);
    }
    float xj[2], xk[2];
    po_hammersley_next(it->xs, xi);
    po_hammersley_next(it->xs, xj);
    po_hammersley_next(it->xs, xk);
    const float c[3] = {xi[0] - 0.5f, xi[1] - 0.5f, xj[0] - 0.5f};
    float corner[3], face[3];
    for (int a = 0; a < 3; ++a) corner[a] = (float)((0.0f < c[a]) - (c[a] < 0.0f));
    uint32_t zero_axis = (uint32_t)(xj[1] * 3.0f);
    if (zero_axis == 3) zero_axis = 2;
    face[zero_axis] = 0.0f;
    face[(zero_axis + 1) % 3] = xk[0];
    face[(zero_axis + 2) % 3] = xk[1];
    return v3(corner[0] * 0.5f + -corner[0] * face[0], corner[1] * 0.5f + -corner[1] * face[1],
              corner[2] * 0.5f + -corner[2] * face[2]);
}

/* Monte_Carlo_Integrator::sample_direct_lighting (Integrators.cpp:46-128). */
static int direct_lighting(integrator* it, const po_fragment* f, po_v3 wi, po_v3* radiance, float* pdf)
{
    const po_scene* s = it->s;
    const int type = (int)s->instances[f->inst].bsdf;
    if (type == PO_BTDF || type == PO_FRESNEL || type == PO_LIGHT) return 0;   /* both BTDFs are kBTDF */
    const po_material* mat = material_of(s, f->inst);
    const int sun = s->sky.use_sun != 0;
    uint32_t light_count = s->nlights + (sun ? 1u : 0u);
    const uint32_t light_index = (uint32_t)(po_mt64_uniform(it->mt) * (float)light_count);
    if (light_index == light_count) light_count--;
    if (light_index >= light_count - 1 && sun) {
        /* the sun: a shadow ray against the light's direction (Integrators.cpp:60-76) */
        const po_v3 to_sun = v3(-s->sky.sun_direction[0], -s->sky.sun_direction[1], -s->sky.sun_direction[2]);
        const po_v3 off = v3_scale(to_sun, 0.01f);
        const po_v4 org = v4(f->position[0] + off.x, f->position[1] + off.y, f->position[2] + off.z,
                             f->position[3] + 0.0f);
        po_fragment hit;
        if (!po_closest_hit(s, org, to_sun, &hit, NULL)) {
            *pdf = direct_pdf(type, mat, v3(f->normal[0], f->normal[1], f->normal[2]), wi, to_sun);
            *radiance = v3(s->sky.sun_colour[0], s->sky.sun_colour[1], s->sky.sun_colour[2]);
            return 1;
        }
        return 0;
    }
    const po_instance* light = &s->instances[s->lights[light_index]];
    const po_mesh* lm = &s->meshes[light->mesh];
    po_v3 sp;
    if (lm->desc.shape != PO_SHAPE_TRIANGLES) {
        sp = implicit_light_point(lm->desc.shape, it);
    } else {
    /* AliasTable::sample (AliasTable.cpp:89-104) then a uniform triangle point. */
    const uint32_t bucket = po_xorshift_next(it->xs) % lm->alias_n;
    const float coin = (float)po_xorshift_next(it->xs) / (float)4294967295u;
    uint32_t tri;
    if (coin <= lm->alias_weight[bucket]) tri = bucket; else tri = lm->alias_index[bucket];
    float xi[2], bary[2];
    po_hammersley_next(it->xs, xi);
    po_uniform_sample_triangle(xi, bary);
    const float* p0 = lm->desc.positions + 3 * lm->desc.indices[3 * tri];
    const float* p1 = lm->desc.positions + 3 * lm->desc.indices[3 * tri + 1];
    const float* p2 = lm->desc.positions + 3 * lm->desc.indices[3 * tri + 2];
    const float w0 = (1.0f - bary[0]) - bary[1];
    sp = v3_add(v3_add(v3_scale(v3(p0[0], p0[1], p0[2]), w0), v3_scale(v3(p1[0], p1[1], p1[2]), bary[0])),
                v3_scale(v3(p2[0], p2[1], p2[2]), bary[1]));
    }
    sp = v3_of4(m4_mul_v4(&light->T, v4_of3(sp, 1.0f)));

    const po_v4 P = v4(f->position[0], f->position[1], f->position[2], f->position[3]);
    const po_v3 N = v3(f->normal[0], f->normal[1], f->normal[2]);
    const po_v3 to_light = v3_normalize(v3_sub(sp, v3_of4(P)));
    if (v3_dot(to_light, N) < 0.0f) return 0;
    const po_v3 off = v3_scale(to_light, 0.01f);
    const po_v4 org = v4(P.x + off.x, P.y + off.y, P.z + off.z, P.w + 0.0f);
    po_fragment hit;
    if (po_closest_hit(s, org, to_light, &hit, NULL)) {
        if (s->instances[hit.inst].bsdf == PO_LIGHT) {
            const po_material* lmat = material_of(s, hit.inst);
            *pdf = direct_pdf(type, mat, N, wi, to_light);
            *radiance = v3(lmat->emissive[0], lmat->emissive[1], lmat->emissive[2]);
            return 1;
        }
    }
    return 0;
}

typedef struct { po_v3 payload, throughput; po_v4 org; po_v3 dir; po_ior_stack ior; } path_state;

static po_v3 sky_colour(const po_scene* s, po_v3 d) { return v3_of4(po_sky_lookup(s, d)); }

/* Monte_Carlo_Integrator::trace_ray (Integrators.cpp:157-209) as a loop. */
static void trace_path(integrator* it, po_fragment frag, path_state* ray)
{
    const po_scene* s = it->s;
    for (uint32_t depth = 0;; ++depth) {
        if (depth == it->max_depth) return;
        const int type = (int)s->instances[frag.inst].bsdf;
        const po_material* mat = material_of(s, frag.inst);
        const po_v3 N = v3(frag.normal[0], frag.normal[1], frag.normal[2]);
        const bsdf_sample smp = sample_bsdf(type, mat, v3_neg(ray->dir), N, ham_next2, it, &ray->ior);
        if (type == PO_LIGHT)
            ray->payload = v3_add(ray->payload, v3_mul(ray->throughput, smp.energy));
        po_v3 rad; float pdf;
        if (direct_lighting(it, &frag, v3_neg(ray->dir), &rad, &pdf))
            ray->payload = v3_add(ray->payload,
                                  v3_mul(v3_mul(v3_scale(ray->throughput, pdf), rad), smp.energy));
        if (smp.P == 0.0f) return;
        const float q = f_max(f_max(ray->throughput.x, ray->throughput.y), ray->throughput.z);
        if (po_mt64_uniform(it->mt) > q) return;
        ray->throughput = v3_scale(ray->throughput, 1.0f / q);
        ray->throughput = v3_mul(ray->throughput, v3_scale(smp.energy, smp.P));
        const po_v3 off = v3_scale(ior_inside(&ray->ior) ? v3_neg(N) : N, 0.01f);   /* Integrators.cpp:199 */
        ray->org = v4(frag.position[0] + off.x, frag.position[1] + off.y, frag.position[2] + off.z,
                      frag.position[3] + 0.0f);
        ray->dir = smp.L;
        po_fragment next;
        if (po_closest_hit(s, ray->org, ray->dir, &next, NULL)) {
            frag = next;
        } else {
            ray->payload = v3_add(ray->payload, v3_mul(ray->throughput, sky_colour(s, smp.L)));
            return;
        }
    }
}

static void integrator_init(integrator* it, const po_scene* s, uint64_t seed, uint32_t max_depth)
{
    it->s = s;
    po_mt64_seed(it->mt, seed);
    po_xorshift_seed((uint32_t)seed, it->xs);
    it->max_depth = max_depth;
}

/* Monte_Carlo_Integrator::integrate_ray (Integrators.cpp:130-154). */
static po_v3 integrate(integrator* it, const po_camera* cam, uint32_t px, uint32_t py)
{
    float xi[2];
    po_hammersley_next(it->xs, xi);
    po_ray r;
    po_generate_ray(cam, xi[0], xi[1], px, py, &r);
    path_state ps;
    ps.org = v4(r.org[0], r.org[1], r.org[2], r.org[3]);
    ps.dir = v3(r.dir[0], r.dir[1], r.dir[2]);
    ps.payload = v3(0.0f, 0.0f, 0.0f);
    ps.throughput = v3(1.0f, 1.0f, 1.0f);
    ps.ior.n = 0;
    ior_push(&ps.ior, 1.0f);
    po_fragment f;
    if (po_closest_hit(it->s, ps.org, ps.dir, &f, NULL)) {
        trace_path(it, f, &ps);
        po_v3 res = ps.payload;
        if (isinf(res.x) || isinf(res.y) || isinf(res.z) || isnan(res.x) || isnan(res.y) || isnan(res.z))
            res = v3(1.0f, (float)0.4, (float)0.7);
        return res;
    }
    return sky_colour(it->s, ps.dir);
}

void po_integrate_ray(const po_scene* s, const po_camera* cam, uint32_t px, uint32_t py,
                      uint32_t max_depth, uint64_t seed, uint32_t nsamples, float* out)
{
    integrator* it = (integrator*)malloc(sizeof(integrator));
    integrator_init(it, s, seed, max_depth);
    for (uint32_t i = 0; i < nsamples; ++i) {
        const po_v3 c = integrate(it, cam, px, py);
        out[3 * i] = c.x; out[3 * i + 1] = c.y; out[3 * i + 2] = c.z;
    }
    free(it);
}

/* One step of the running mean / variance of Scene.cpp:173-198; returns 1 to stop. */
static int accumulate_step(po_v3 x, uint32_t max_samples, float max_variance,
                           float* pixel, uint32_t* count, float* variance)
{
    (void)max_samples;
    const uint32_t prev = *count;
    if (prev < 1) {
        *count = 1;
        variance[0] = variance[1] = variance[2] = 0.0f;
    } else {
        const po_v3 pp = v3(pixel[0], pixel[1], pixel[2]);
        const po_v3 pv = v3(variance[0], variance[1], variance[2]);
        const po_v3 np = v3_add(pp, v3_scale(v3_sub(x, pp), 1.0f / (float)prev));
        /* glm/gtx/scalar_multiplication.hpp: vec * uint multiplies by float(n),
         * vec / uint multiplies by 1.0f / float(n) */
        const po_v3 nv = v3_scale(v3_add(v3_scale(pv, (float)prev), v3_mul(v3_sub(x, pp), v3_sub(x, np))),
                                  1.0f / (float)(prev + 1));
        variance[0] = nv.x; variance[1] = nv.y; variance[2] = nv.z;
        *count = prev + 1;
        x = np;
    }
    pixel[0] = x.x; pixel[1] = x.y; pixel[2] = x.z;
    return prev > 4 && variance[0] <= max_variance && variance[1] <= max_variance &&
           variance[2] <= max_variance;
}

void po_accumulate(const float* samples, uint32_t n, uint32_t max_samples, float max_variance,
                   float* pixel, uint32_t* count, float* variance)
{
    if (*count >= max_samples) return;
    for (uint32_t i = 0; i < n && i < max_samples; ++i)
        if (accumulate_step(v3(samples[3 * i], samples[3 * i + 1], samples[3 * i + 2]), max_samples,
                            max_variance, pixel, count, variance))
            break;
}

typedef struct {
    const po_scene* s; const po_camera* cam;
    uint32_t max_depth, max_samples; float max_variance;
    uint32_t pixel; uint64_t seed;
    float* pixels; uint32_t* counts; float* variance;
} pixel_job;

static void pixel_job_run(void* p)
{
    pixel_job* j = (pixel_job*)p;
    const uint32_t flat = j->pixel;
    if (j->counts[flat] >= j->max_samples) return;
    const uint32_t W = j->cam->resolution[0];
    integrator* it = (integrator*)malloc(sizeof(integrator));
    integrator_init(it, j->s, j->seed, j->max_depth);
    for (uint32_t i = 0; i < j->max_samples; ++i) {
        const po_v3 x = integrate(it, j->cam, flat % W, flat / W);
        if (accumulate_step(x, j->max_samples, j->max_variance, j->pixels + 3 * flat, &j->counts[flat],
                            j->variance + 3 * flat))
            break;
    }
    free(it);
}

void po_render_pixels(const po_scene* s, const po_camera* cam, uint32_t max_depth,
                      uint32_t max_samples, float max_variance,
                      const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels,
                      float* pixels, uint32_t* sample_count, float* variance, int nthreads)
{
    pixel_job* jobs = (pixel_job*)malloc(sizeof(pixel_job) * (npixels ? npixels : 1));
    for (uint32_t i = 0; i < npixels; ++i) {
        pixel_job* j = &jobs[i];
        j->s = s; j->cam = cam; j->max_depth = max_depth; j->max_samples = max_samples;
        j->max_variance = max_variance; j->pixel = pixel_index[i]; j->seed = seeds[i];
        j->pixels = pixels; j->counts = sample_count; j->variance = variance;
    }
    po_parallel_for(npixels, jobs, sizeof(pixel_job), pixel_job_run, nthreads);
    free(jobs);
}
