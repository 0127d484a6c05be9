/* Oracle (test infrastructure only): double-precision restatement of the physical
 * estimator of the product (PICO_ESTIMATOR_PHYSICAL).  The reference has no such
 * estimator, so this file follows published methods, not reference code:
 *
 *   GGX / Trowbridge-Reitz distribution with Smith masking: Walter, Marschner, Li,
 *     Torrance 2007, "Microfacet models for refraction through rough surfaces";
 *     height-correlated G2: Heitz 2014, "Understanding the masking-shadowing
 *     function in microfacet-based BRDFs";
 *   visible-normal sampling: Heitz 2018, "Sampling the GGX distribution of visible
 *     normals" (JCGT 7(4));
 *   multiple importance sampling with the power heuristic: Veach and Guibas 1995;
 *   orthonormal basis: Duff et al. 2017, "Building an orthonormal basis, revisited".
 *
 * Geometry (closest hits, interpolated fragments, light alias tables, sky lookups)
 * comes from the rest of the oracle in float, as the product computes it; every
 * shading quantity here is double.  The path estimator can run with both light
 * strategies combined (MIS), next-event estimation alone or BSDF sampling alone:
 * all three converge to the same image, which pins the combination without a
 * reference implementation. */
#include "po_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double x, y, z; } d3;

static d3 d3v(double x, double y, double z) { d3 r = {x, y, z}; return r; }
static d3 d3_add(d3 a, d3 b) { return d3v(a.x + b.x, a.y + b.y, a.z + b.z); }
static d3 d3_sub(d3 a, d3 b) { return d3v(a.x - b.x, a.y - b.y, a.z - b.z); }
static d3 d3_scale(d3 a, double s) { return d3v(a.x * s, a.y * s, a.z * s); }
static d3 d3_mul(d3 a, d3 b) { return d3v(a.x * b.x, a.y * b.y, a.z * b.z); }
static double d3_dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static d3 d3_cross(d3 a, d3 b) { return d3v(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static d3 d3_norm(d3 a) { return d3_scale(a, 1.0 / sqrt(d3_dot(a, a))); }
static d3 d3_of(const float* p) { return d3v(p[0], p[1], p[2]); }

#define PHYS_PI 3.14159265358979323846
#define PHYS_MIN_ALPHA 1e-3

/* ------------------------------------------------------------------ BSDF */
typedef struct { d3 diffuse, f0; double alpha, p_spec; } lobes;

static lobes lobes_of(int kind, const po_material* m)
{
    lobes l;
    l.diffuse = kind == PO_SPECULAR ? d3v(0, 0, 0) : d3_of(m->diffuse);
    l.f0 = kind == PO_DIFFUSE ? d3v(0, 0, 0) : d3_of(m->specular);
    l.alpha = (double)m->roughness * (double)m->roughness;
    if (l.alpha < PHYS_MIN_ALPHA) l.alpha = PHYS_MIN_ALPHA;
    const double s = l.f0.x + l.f0.y + l.f0.z, d = l.diffuse.x + l.diffuse.y + l.diffuse.z;
    l.p_spec = (s + d > 0.0) ? s / (s + d) : 0.0;
    return l;
}

typedef struct { d3 t, b, n; } frame;

static frame frame_of(d3 n)
{
    const double sign = copysign(1.0, n.z);
    const double a = -1.0 / (sign + n.z);
    const double b = n.x * n.y * a;
    frame f;
    f.t = d3v(1.0 + sign * n.x * n.x * a, sign * b, -sign * n.x);
    f.b = d3v(b, sign + n.y * n.y * a, -n.y);
    f.n = n;
    return f;
}
static d3 to_local(const frame* f, d3 v) { return d3v(d3_dot(v, f->t), d3_dot(v, f->b), d3_dot(v, f->n)); }
static d3 to_world(const frame* f, d3 v)
{
    return d3_add(d3_add(d3_scale(f->t, v.x), d3_scale(f->b, v.y)), d3_scale(f->n, v.z));
}

static double ggx_d(d3 h, double a2)
{
    if (h.z <= 0.0) return 0.0;
    const double k = (h.x * h.x + h.y * h.y) + a2 * h.z * h.z;
    return a2 / (PHYS_PI * k * k);
}
static double ggx_lambda(d3 w, double a2)
{
    const double t2 = (w.x * w.x + w.y * w.y) / (w.z * w.z);
    return 0.5 * (sqrt(1.0 + a2 * t2) - 1.0);
}
static double schlick(double f0, double c)
{
    double m = 1.0 - c;
    if (m < 0.0) m = 0.0;
    if (m > 1.0) m = 1.0;
    return f0 + (1.0 - f0) * m * m * m * m * m;
}

/* f(v, l) and the mixture density of l, local frame. */
static void eval_local(const lobes* lb, d3 v, d3 l, d3* f, double* pdf)
{
    *f = d3v(0, 0, 0);
    *pdf = 0.0;
    if (v.z <= 0.0 || l.z <= 0.0) return;
    *f = d3_scale(lb->diffuse, 1.0 / PHYS_PI);
    *pdf = (1.0 - lb->p_spec) * l.z / PHYS_PI;
    if (lb->p_spec > 0.0) {
        const d3 h = d3_norm(d3_add(v, l));
        const double a2 = lb->alpha * lb->alpha;
        const double D = ggx_d(h, a2);
        const double lv = ggx_lambda(v, a2), ll = ggx_lambda(l, a2);
        double vh = d3_dot(v, h);
        if (vh < 0.0) vh = 0.0;
        const double g = D / ((1.0 + lv + ll) * 4.0 * v.z * l.z);
        *f = d3_add(*f, d3v(schlick(lb->f0.x, vh) * g, schlick(lb->f0.y, vh) * g, schlick(lb->f0.z, vh) * g));
        *pdf += lb->p_spec * D / ((1.0 + lv) * 4.0 * v.z);
    }
}

static d3 sample_vndf(d3 v, double alpha, double u1, double u2)
{
    const d3 vh = d3_norm(d3v(alpha * v.x, alpha * v.y, v.z));
    const double lensq = vh.x * vh.x + vh.y * vh.y;
    const d3 t1 = lensq > 0.0 ? d3_scale(d3v(-vh.y, vh.x, 0.0), 1.0 / sqrt(lensq)) : d3v(1, 0, 0);
    const d3 t2 = d3_cross(vh, t1);
    const double r = sqrt(u1), phi = 2.0 * PHYS_PI * u2;
    const double p1 = r * cos(phi);
    const double s = 0.5 * (1.0 + vh.z);
    const double p2 = (1.0 - s) * sqrt(fmax(1.0 - p1 * p1, 0.0)) + s * r * sin(phi);
    const double pz = sqrt(fmax(1.0 - p1 * p1 - p2 * p2, 0.0));
    const d3 nh = d3_add(d3_add(d3_scale(t1, p1), d3_scale(t2, p2)), d3_scale(vh, pz));
    return d3_norm(d3v(alpha * nh.x, alpha * nh.y, fmax(nh.z, 0.0)));
}

/* Exact dielectric Fresnel reflectance, eta = eta_i / eta_t, cos_i > 0; 1 under total
 * internal reflection. */
static double fresnel_dielectric(double cos_i, double eta)
{
    const double sin2_t = eta * eta * fmax(1.0 - cos_i * cos_i, 0.0);
    if (sin2_t >= 1.0) return 1.0;
    const double cos_t = sqrt(1.0 - sin2_t);
    const double rs = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const double rp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return 0.5 * (rs * rs + rp * rp);
}

/* Transparent / Fresnel kinds: a rough dielectric interface (Walter et al. 2007; GGX,
 * visible-normal sampling).  The Fresnel kind reflects about the sampled microfacet
 * normal with probability F(v.h), else refracts; the Transparent kind refracts unless
 * total internal reflection forces a reflection.  Weights: G2 / G1(v) for a
 * reflection, tint G2 / G1 eta^2 for a refraction.  Returns 0 when the direction
 * leaves on the wrong side; *refracted tells which. */
static int sample_dielectric(d3 v, double alpha, double eta, d3 tint, int reflect_lobe, const double* u, d3* l,
                             d3* weight, int* refracted)
{
    *refracted = 0;
    *weight = d3v(0, 0, 0);
    *l = d3v(0, 0, 1);
    if (v.z <= 0.0) return 0;
    const d3 h = sample_vndf(v, alpha, u[1], u[2]);
    const double vh = d3_dot(v, h);
    if (vh <= 0.0) return 0;
    const double F = fresnel_dielectric(vh, eta);
    const double a2 = alpha * alpha, lv = ggx_lambda(v, a2);
    if (F >= 1.0 || (reflect_lobe && u[0] < F)) {
        *l = d3_sub(d3_scale(h, 2.0 * vh), v);
        if (l->z <= 0.0) return 0;
        const double g = (1.0 + lv) / (1.0 + lv + ggx_lambda(*l, a2));
        *weight = d3v(g, g, g);
    } else {
        const double cos_t = sqrt(fmax(1.0 - eta * eta * (1.0 - vh * vh), 0.0));
        *l = d3_norm(d3_sub(d3_scale(h, eta * vh - cos_t), d3_scale(v, eta)));
        if (l->z >= 0.0) return 0;
        const double g = (1.0 + lv) / (1.0 + lv + ggx_lambda(*l, a2)) * eta * eta;
        *weight = d3_scale(tint, g);
        *refracted = 1;
    }
    return 1;
}

/* One sample from three uniforms; returns 0 when it leaves below the surface. */
static int sample_local(const lobes* lb, d3 v, const double* u, d3* l, double* pdf, d3* weight)
{
    *pdf = 0.0;
    *weight = d3v(0, 0, 0);
    *l = d3v(0, 0, 1);
    if (v.z <= 0.0 || (lb->p_spec <= 0.0 && lb->diffuse.x + lb->diffuse.y + lb->diffuse.z <= 0.0)) return 0;
    if (u[0] < lb->p_spec) {
        const d3 h = sample_vndf(v, lb->alpha, u[1], u[2]);
        *l = d3_sub(d3_scale(h, 2.0 * d3_dot(v, h)), v);
    } else {
        const double r = sqrt(u[1]), phi = 2.0 * PHYS_PI * u[2];
        *l = d3v(r * cos(phi), r * sin(phi), sqrt(fmax(1.0 - u[1], 0.0)));
    }
    if (l->z <= 0.0) return 0;
    d3 f;
    eval_local(lb, v, *l, &f, pdf);
    if (!(*pdf > 0.0)) return 0;
    *weight = d3_scale(f, l->z / *pdf);
    return 1;
}

void po_phys_bsdf_eval(int kind, const po_material* m, const double* V, const double* N, const double* L,
                       double* f, double* pdf)
{
    const lobes lb = lobes_of(kind, m);
    const frame fr = frame_of(d3v(N[0], N[1], N[2]));
    d3 fv;
    eval_local(&lb, to_local(&fr, d3v(V[0], V[1], V[2])), to_local(&fr, d3v(L[0], L[1], L[2])), &fv, pdf);
    f[0] = fv.x; f[1] = fv.y; f[2] = fv.z;
}

int po_phys_bsdf_sample(int kind, const po_material* m, const double* V, const double* N, const double* u,
                        double* L, double* pdf, double* weight)
{
    const lobes lb = lobes_of(kind, m);
    const frame fr = frame_of(d3v(N[0], N[1], N[2]));
    d3 l, w;
    const int ok = sample_local(&lb, to_local(&fr, d3v(V[0], V[1], V[2])), u, &l, pdf, &w);
    const d3 lw = to_world(&fr, l);
    L[0] = lw.x; L[1] = lw.y; L[2] = lw.z;
    weight[0] = w.x; weight[1] = w.y; weight[2] = w.z;
    return ok;
}

static double mis_weight(double a, double b)
{
    if (!(a > 0.0)) return 0.0;
    const double r = b / a;
    return 1.0 / (1.0 + r * r);
}

/* ------------------------------------------------------------------ lights */
typedef struct {
    const po_scene* s;
    uint32_t nl;               /* triangle and implicit lights, plus the sun */
    uint32_t* base;            /* per light: first triangle record */
    double* geo;               /* per light triangle: world unit normal, area density */
    uint32_t* light_of_inst;   /* instance -> light index or PO_INVALID */
    double* pick;              /* per slot (lights, then the sun): probability of the next-event pick */
} phys_scene;

static d3 xform_point(const po_m4* T, d3 p)
{
    return d3v(T->m[0][0] * p.x + T->m[1][0] * p.y + T->m[2][0] * p.z + T->m[3][0],
               T->m[0][1] * p.x + T->m[1][1] * p.y + T->m[2][1] * p.z + T->m[3][1],
               T->m[0][2] * p.x + T->m[1][2] * p.y + T->m[2][2] * p.z + T->m[3][2]);
}

static void phys_prepare(phys_scene* ps, const po_scene* s)
{
    ps->s = s;
    ps->nl = s->nlights + (s->sky.use_sun ? 1u : 0u);
    ps->base = (uint32_t*)calloc(s->nlights + 1, sizeof(uint32_t));
    ps->light_of_inst = (uint32_t*)malloc(sizeof(uint32_t) * (s->ninstances ? s->ninstances : 1));
    for (uint32_t i = 0; i < s->ninstances; ++i) ps->light_of_inst[i] = PO_INVALID;
    uint32_t total = 0;
    for (uint32_t l = 0; l < s->nlights; ++l) {
        ps->base[l] = total;
        ps->light_of_inst[s->lights[l]] = l;
        const po_mesh* m = &s->meshes[s->instances[s->lights[l]].mesh];
        if (m->desc.shape == PO_SHAPE_TRIANGLES) total += m->alias_n;
    }
    ps->base[s->nlights] = total;
    ps->geo = (double*)calloc(4 * (size_t)(total ? total : 1), sizeof(double));
    for (uint32_t l = 0; l < s->nlights; ++l) {
        const po_instance* in = &s->instances[s->lights[l]];
        const po_mesh* m = &s->meshes[in->mesh];
        if (m->desc.shape != PO_SHAPE_TRIANGLES) continue;
        const uint32_t n = m->alias_n;
        /* probability with which the alias table returns each triangle */
        double* p = (double*)calloc(n ? n : 1, sizeof(double));
        for (uint32_t b = 0; b < n; ++b) {
            double keep = m->alias_weight[b];
            if (keep < 0.0) keep = 0.0;
            if (keep > 1.0) keep = 1.0;
            p[b] += keep / n;
            if (m->alias_index[b] < n) p[m->alias_index[b]] += (1.0 - keep) / n;
        }
        for (uint32_t t = 0; t < n; ++t) {
            const uint32_t* ix = m->desc.indices + 3 * t;
            const d3 a = xform_point(&in->T, d3_of(m->desc.positions + 3 * ix[0]));
            const d3 b = xform_point(&in->T, d3_of(m->desc.positions + 3 * ix[1]));
            const d3 c = xform_point(&in->T, d3_of(m->desc.positions + 3 * ix[2]));
            const d3 cr = d3_cross(d3_sub(b, a), d3_sub(c, a));
            const double len = sqrt(d3_dot(cr, cr));
            double* g = ps->geo + 4 * (size_t)(ps->base[l] + t);
            if (len > 0.0) {
                g[0] = cr.x / len; g[1] = cr.y / len; g[2] = cr.z / len; g[3] = p[t] / (0.5 * len);
            } else {
                g[0] = 0; g[1] = 0; g[2] = 1; g[3] = 0;
            }
        }
        free(p);
    }
    /* Next-event pick: the sun keeps a uniform share 1 / nl; triangle lights share
     * the rest in proportion to their power (sum of the emitted radiance channels
     * times the world area), implicit lights are never picked. */
    ps->pick = (double*)calloc(ps->nl ? ps->nl : 1, sizeof(double));
    double power = 0.0;
    uint32_t ntri = 0;
    for (uint32_t l = 0; l < s->nlights; ++l) {
        const po_instance* in = &s->instances[s->lights[l]];
        const po_mesh* m = &s->meshes[in->mesh];
        if (m->desc.shape != PO_SHAPE_TRIANGLES) continue;
        ++ntri;
        double area = 0.0;
        for (uint32_t t = 0; t < m->desc.ntris; ++t) {
            const uint32_t* ix = m->desc.indices + 3 * t;
            const d3 a = xform_point(&in->T, d3_of(m->desc.positions + 3 * ix[0]));
            const d3 b = xform_point(&in->T, d3_of(m->desc.positions + 3 * ix[1]));
            const d3 c = xform_point(&in->T, d3_of(m->desc.positions + 3 * ix[2]));
            const d3 cr = d3_cross(d3_sub(b, a), d3_sub(c, a));
            area += 0.5 * sqrt(d3_dot(cr, cr));
        }
        const float* le = s->materials[in->material].emissive;
        const double pw = ((double)le[0] + (double)le[1] + (double)le[2]) * area;
        ps->pick[l] = (isfinite(pw) && pw > 0.0) ? pw : 0.0;
        power += ps->pick[l];
    }
    const double sun_share = s->sky.use_sun ? 1.0 / ps->nl : 0.0;
    for (uint32_t l = 0; l < s->nlights; ++l) {
        const po_mesh* m = &s->meshes[s->instances[s->lights[l]].mesh];
        if (m->desc.shape != PO_SHAPE_TRIANGLES) continue;
        ps->pick[l] = (1.0 - sun_share) * (power > 0.0 ? ps->pick[l] / power : 1.0 / ntri);
    }
    if (s->sky.use_sun) ps->pick[s->nlights] = ntri ? sun_share : 1.0;
}

/* The slot a uniform u picks from the next-event table. */
static uint32_t pick_light(const phys_scene* ps, double u)
{
    double acc = 0.0;
    uint32_t last = 0;
    for (uint32_t l = 0; l < ps->nl; ++l) {
        if (!(ps->pick[l] > 0.0)) continue;
        last = l;
        acc += ps->pick[l];
        if (u < acc) return l;
    }
    return last;
}

static void phys_release(phys_scene* ps)
{
    free(ps->base);
    free(ps->geo);
    free(ps->light_of_inst);
    free(ps->pick);
}

/* ------------------------------------------------------------------ paths */
typedef struct { uint64_t s; } prng;   /* splitmix64 */

static double rnd(prng* r)
{
    uint64_t z = (r->s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

enum { PHYS_MIS = 0, PHYS_NEE_ONLY = 1, PHYS_BSDF_ONLY = 2 };

static int trace(const po_scene* s, d3 o, double ow, d3 d, po_fragment* f)
{
    const po_v4 org = v4((float)o.x, (float)o.y, (float)o.z, (float)ow);
    return po_closest_hit(s, org, v3((float)d.x, (float)d.y, (float)d.z), f, NULL);
}

static d3 sky_of(const po_scene* s, d3 d)
{
    const po_v4 c = po_sky_lookup(s, v3((float)d.x, (float)d.y, (float)d.z));
    return d3v(c.x, c.y, c.z);
}

/* Density with which next-event estimation picks world point y on light triangle
 * record g of light slot li, seen from distance t along unit direction d (solid
 * angle measure). */
static double light_pdf(const phys_scene* ps, uint32_t li, const double* g, double t, d3 d)
{
    const double cl = fabs(g[0] * d.x + g[1] * d.y + g[2] * d.z);
    if (!(cl > 0.0)) return INFINITY;
    return g[3] * t * t * ps->pick[li] / cl;
}

/* One path of the physical estimator.  With `cache` (the radiance-cache form,
 * pico_gpu.h PICO_ESTIMATOR_RADIANCE_CACHE, here with a cache that answers the
 * constant radiance cache[0..2]): a path ends at its non-emitting vertex after
 * one bounce, or after two when the first vertex has roughness < 0.1 (a mirror
 * counts as roughness 0), adding throughput * cache there. */
static d3 phys_path(const phys_scene* ps, const po_camera* cam, uint32_t px, uint32_t py, uint32_t max_depth,
                    int strategy, const double* cache, prng* rng)
{
    double prev_rough = 0.0;
    const po_scene* s = ps->s;
    po_ray r;
    const float jx = (float)(2.0 * rnd(rng)), jy = (float)(2.0 * rnd(rng));
    po_generate_ray(cam, jx, jy, px, py, &r);
    d3 o = d3v(r.org[0], r.org[1], r.org[2]);
    double ow = r.org[3];
    d3 d = d3v(r.dir[0], r.dir[1], r.dir[2]);
    d3 thr = d3v(1, 1, 1), rad = d3v(0, 0, 0);
    double pdf_prev = 0.0;   /* 0: camera ray or mirror bounce, emission unweighted */
    for (uint32_t depth = 0;; ++depth) {
        po_fragment f;
        if (!trace(s, o, ow, d, &f)) {
            rad = d3_add(rad, d3_mul(thr, sky_of(s, d)));
            break;
        }
        const po_instance* in = &s->instances[f.inst];
        const po_material* m = &s->materials[in->material];
        if (in->bsdf == PO_LIGHT) {
            double w = 1.0;
            const uint32_t li = ps->light_of_inst[f.inst];
            const int tri_light = li != PO_INVALID && f.prim != PO_IMPLICIT_PRIM &&
                                  s->meshes[in->mesh].desc.shape == PO_SHAPE_TRIANGLES;
            if (pdf_prev > 0.0) {
                if (strategy == PHYS_NEE_ONLY && tri_light) w = 0.0;
                else if (strategy == PHYS_MIS && tri_light)
                    w = mis_weight(pdf_prev, light_pdf(ps, li, ps->geo + 4 * (size_t)(ps->base[li] + f.prim), f.t, d));
            }
            rad = d3_add(rad, d3_scale(d3_mul(thr, d3_of(m->emissive)), w));
            break;
        }
        if (cache && (depth >= 2 || (depth == 1 && prev_rough >= 0.1))) {
            rad = d3_add(rad, d3_mul(thr, d3v(cache[0], cache[1], cache[2])));
            break;
        }
        if (depth >= max_depth) break;
        prev_rough = in->bsdf == PO_DELTA ? 0.0 : m->roughness;   /* a mirror is glossy */
        d3 n = d3_norm(d3_of(f.normal));
        const d3 v = d3_scale(d, -1.0);
        const int front = !(d3_dot(n, v) < 0.0);   /* the viewer on the side the normal points to */
        if (!front) n = d3_scale(n, -1.0);
        const d3 P = d3v(f.position[0], f.position[1], f.position[2]);
        const double eps = 1e-4 * (1.0 + fmax(fmax(fabs(P.x), fabs(P.y)), fabs(P.z)));
        d3 org = d3_add(P, d3_scale(n, eps));
        d3 L, weight;
        double pdf_next = 0.0;
        int ok;
        if (in->bsdf == PO_DELTA) {
            const double c = d3_dot(n, v);
            L = d3_sub(d3_scale(n, 2.0 * c), v);
            weight = d3v(schlick(m->specular[0], c), schlick(m->specular[1], c), schlick(m->specular[2], c));
            ok = c > 0.0;
        } else if (in->bsdf == PO_BTDF || in->bsdf == PO_FRESNEL) {
            /* air outside, the material's index inside; no next-event estimation here */
            const frame fr = frame_of(n);
            const double ior = m->index_of_refraction > 0.0f ? m->index_of_refraction : 1.0;
            double u[3] = {rnd(rng), rnd(rng), rnd(rng)};
            d3 l;
            int refracted;
            ok = sample_dielectric(to_local(&fr, v), fmax((double)m->roughness * m->roughness, PHYS_MIN_ALPHA),
                                   front ? 1.0 / ior : ior, d3_of(m->diffuse), in->bsdf == PO_FRESNEL, u, &l, &weight,
                                   &refracted);
            L = to_world(&fr, l);
            if (refracted) org = d3_sub(P, d3_scale(n, eps));
        } else {
            const frame fr = frame_of(n);
            const d3 vl = to_local(&fr, v);
            const lobes lb = lobes_of((int)in->bsdf, m);
            if (ps->nl > 0 && strategy != PHYS_BSDF_ONLY) {
                const uint32_t li = pick_light(ps, rnd(rng));
                if (s->sky.use_sun && li == ps->nl - 1) {
                    const d3 wi = d3_norm(d3v(-s->sky.sun_direction[0], -s->sky.sun_direction[1],
                                              -s->sky.sun_direction[2]));
                    const d3 wl = to_local(&fr, wi);
                    po_fragment h;
                    if (wl.z > 0.0 && !trace(s, org, ow, wi, &h)) {
                        d3 fv; double pb;
                        eval_local(&lb, vl, wl, &fv, &pb);
                        rad = d3_add(rad, d3_scale(d3_mul(d3_mul(thr, fv), d3_of(s->sky.sun_colour)), wl.z / ps->pick[li]));
                    }
                } else {
                    const po_instance* lin = &s->instances[s->lights[li]];
                    const po_mesh* lm = &s->meshes[lin->mesh];
                    if (lm->desc.shape == PO_SHAPE_TRIANGLES) {
                        uint32_t bucket = (uint32_t)(rnd(rng) * lm->alias_n);
                        if (bucket >= lm->alias_n) bucket = lm->alias_n - 1;
                        const double coin = rnd(rng);
                        const uint32_t t = coin < lm->alias_weight[bucket] ? bucket : lm->alias_index[bucket];
                        const double su0 = sqrt(rnd(rng)), x1 = rnd(rng);
                        const double bx = 1.0 - su0, by = x1 * su0, w0 = 1.0 - bx - by;
                        const uint32_t* ix = lm->desc.indices + 3 * t;
                        const d3 a = d3_of(lm->desc.positions + 3 * ix[0]);
                        const d3 b = d3_of(lm->desc.positions + 3 * ix[1]);
                        const d3 c = d3_of(lm->desc.positions + 3 * ix[2]);
                        const d3 y = xform_point(&lin->T, d3_add(d3_add(d3_scale(a, w0), d3_scale(b, bx)),
                                                                 d3_scale(c, by)));
                        const d3 dd = d3_sub(y, org);
                        const double dist2 = d3_dot(dd, dd), dist = sqrt(dist2);
                        const d3 wi = d3_scale(dd, 1.0 / dist);
                        const double* g = ps->geo + 4 * (size_t)(ps->base[li] + t);
                        const double pl = light_pdf(ps, li, g, dist, wi);
                        const d3 wl = to_local(&fr, wi);
                        if (wl.z > 0.0 && isfinite(pl) && g[3] > 0.0 && dist > 0.0) {
                            po_fragment h;
                            const int hit = trace(s, org, ow, wi, &h);
                            if (!hit || h.t >= dist * (1.0 - 1e-4)) {
                                d3 fv; double pb;
                                eval_local(&lb, vl, wl, &fv, &pb);
                                const double w = strategy == PHYS_MIS ? mis_weight(pl, pb) : 1.0;
                                const po_material* lmat = &s->materials[lin->material];
                                rad = d3_add(rad, d3_scale(d3_mul(d3_mul(thr, fv), d3_of(lmat->emissive)),
                                                           wl.z * w / pl));
                            }
                        }
                    }
                }
            }
            double u[3] = {rnd(rng), rnd(rng), rnd(rng)};
            d3 l;
            ok = sample_local(&lb, vl, u, &l, &pdf_next, &weight);
            L = to_world(&fr, l);
        }
        if (!ok) break;
        thr = d3_mul(thr, weight);
        if (depth >= 3) {
            double q = fmax(fmax(thr.x, thr.y), thr.z);
            if (q > 0.95) q = 0.95;
            if (!(rnd(rng) < q)) break;
            thr = d3_scale(thr, 1.0 / q);
        }
        pdf_prev = pdf_next;
        o = org;
        d = L;
    }
    return rad;
}

typedef struct {
    const phys_scene* ps;
    const po_camera* cam;
    uint32_t max_depth, spp, pixel;
    int strategy;
    const double* cache;
    uint64_t seed;
    double *mean, *var;
} phys_job;

static void phys_job_run(void* p)
{
    phys_job* j = (phys_job*)p;
    const uint32_t W = j->cam->resolution[0];
    prng rng = {j->seed};
    double sum[3] = {0, 0, 0}, sq[3] = {0, 0, 0};
    for (uint32_t i = 0; i < j->spp; ++i) {
        const d3 x = phys_path(j->ps, j->cam, j->pixel % W, j->pixel / W, j->max_depth, j->strategy, j->cache, &rng);
        const double c[3] = {x.x, x.y, x.z};
        for (int a = 0; a < 3; ++a) { sum[a] += c[a]; sq[a] += c[a] * c[a]; }
    }
    for (int a = 0; a < 3; ++a) {
        const double m = sum[a] / j->spp;
        j->mean[a] = m;
        j->var[a] = j->spp > 1 ? (sq[a] - j->spp * m * m) / (j->spp - 1) : 0.0;
    }
}

static void render_mean(const po_scene* s, const po_camera* cam, uint32_t max_depth, uint32_t spp,
                        const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels, int strategy,
                        const double* cache, double* mean, double* var, int nthreads)
{
    phys_scene ps;
    phys_prepare(&ps, s);
    phys_job* jobs = (phys_job*)malloc(sizeof(phys_job) * (npixels ? npixels : 1));
    for (uint32_t i = 0; i < npixels; ++i) {
        phys_job* j = &jobs[i];
        j->ps = &ps; j->cam = cam; j->max_depth = max_depth; j->spp = spp; j->pixel = pixel_index[i];
        j->strategy = strategy; j->cache = cache; j->seed = seeds[i]; j->mean = mean + 3 * (size_t)i;
        j->var = var + 3 * (size_t)i;
    }
    po_parallel_for(npixels, jobs, sizeof(phys_job), phys_job_run, nthreads);
    free(jobs);
    phys_release(&ps);
}

void po_phys_render_mean(const po_scene* s, const po_camera* cam, uint32_t max_depth, uint32_t spp,
                         const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels, int strategy,
                         double* mean, double* var, int nthreads)
{
    render_mean(s, cam, max_depth, spp, pixel_index, seeds, npixels, strategy, NULL, mean, var, nthreads);
}

void po_phys_render_mean_cached(const po_scene* s, const po_camera* cam, uint32_t max_depth, uint32_t spp,
                                const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels,
                                const double* cache_rgb, double* mean, double* var, int nthreads)
{
    render_mean(s, cam, max_depth, spp, pixel_index, seeds, npixels, 0, cache_rgb, mean, var, nthreads);
}
