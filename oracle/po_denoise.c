/*
 * Oracle (test infrastructure only): denoiser inputs and the a-trous denoiser.
 *
 *   Scene::generate_denoiser_inputs   Core/Scene.cpp:248-294
 *   Camera::getViewMatrix             Core/Camera.cpp:90-93 (glm::lookAtRH,
 *                                     glm/gtc/matrix_transform.inl:754-774)
 *   Util::atrous_denoise              Util/Denoisers.cpp:107-126
 *   blend_pixel (per 64x64 tile)      Util/Denoisers.cpp:18-101
 *   Tiler tile walk                   Util/Tiler.hpp:20-49
 *   Util::reinhard_tone_mapping       Util/ToneMappers.cpp:12-44
 *
 * The 5x5 kernel table keeps the reference's 0.09563 entry at index 17.
 * std::min(std::exp(x), 1.0f) is restated as `(1 < e) ? 1 : e`, which keeps
 * a NaN weight NaN exactly as the reference does.
 */
#include "po_internal.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void po_view_matrix(const po_camera* c, float* out)
{
    const po_v3 eye = v3(c->position[0], c->position[1], c->position[2]);
    const po_v3 dir = v3(c->direction[0], c->direction[1], c->direction[2]);
    const po_v3 up = v3(c->up[0], c->up[1], c->up[2]);
    const po_v3 center = v3_add(eye, dir);
    const po_v3 f = v3_normalize(v3_sub(center, eye));
    const po_v3 s = v3_normalize(v3_cross(f, up));
    const po_v3 u = v3_cross(s, f);
    float m[4][4];
    memset(m, 0, sizeof m);
    m[0][0] = s.x; m[1][0] = s.y; m[2][0] = s.z;
    m[0][1] = u.x; m[1][1] = u.y; m[2][1] = u.z;
    m[0][2] = -f.x; m[1][2] = -f.y; m[2][2] = -f.z;
    m[3][0] = -v3_dot(s, eye); m[3][1] = -v3_dot(u, eye); m[3][2] = v3_dot(f, eye);
    m[3][3] = 1.0f;
    memcpy(out, m, sizeof m);
}

void po_denoiser_inputs(const po_scene* s, const po_camera* cam, uint32_t W, uint32_t H,
                        float* normals, float* positions, float* diffuse)
{
    po_m4 view;
    po_view_matrix(cam, &view.m[0][0]);
    for (uint32_t y = 0; y < H; ++y) {
        for (uint32_t x = 0; x < W; ++x) {
            const size_t flat = (size_t)y * W + x;
            po_ray r;
            po_generate_ray(cam, 0.0f, 0.0f, x, y, &r);
            const po_v3 d = v3(r.dir[0], r.dir[1], r.dir[2]);
            po_fragment f;
            if (po_closest_hit(s, v4(r.org[0], r.org[1], r.org[2], r.org[3]), d, &f, NULL)) {
                memcpy(normals + 3 * flat, f.normal, sizeof(float) * 3);
                const po_v4 p = m4_mul_v4(&view, v4(f.position[0], f.position[1], f.position[2], f.position[3]));
                positions[3 * flat] = p.x; positions[3 * flat + 1] = p.y; positions[3 * flat + 2] = p.z;
                memcpy(diffuse + 3 * flat, s->materials[s->instances[f.inst].material].diffuse, sizeof(float) * 3);
            } else {
                normals[3 * flat] = -d.x; normals[3 * flat + 1] = -d.y; normals[3 * flat + 2] = -d.z;
                positions[3 * flat] = d.x * r.dir[3];
                positions[3 * flat + 1] = d.y * r.dir[3];
                positions[3 * flat + 2] = d.z * r.dir[3];
                const po_v4 sky = po_sky_lookup(s, d);   /* m_sky_box->sample4(ray.mDirection) */
                diffuse[3 * flat] = sky.x; diffuse[3 * flat + 1] = sky.y; diffuse[3 * flat + 2] = sky.z;
            }
        }
    }
}

static const float kWeights[25] = {
    (float)0.00292, (float)0.01306, (float)0.02154, (float)0.01306, (float)0.00292,
    (float)0.01306, (float)0.05855, (float)0.09653, (float)0.05855, (float)0.01306,
    (float)0.02154, (float)0.09653, (float)0.15915, (float)0.09653, (float)0.02154,
    (float)0.01306, (float)0.05855, (float)0.09563, (float)0.05855, (float)0.01306,
    (float)0.00292, (float)0.01306, (float)0.02154, (float)0.01306, (float)0.00292};

static float lum(const float* c)
{
    return v3_dot(v3(c[0], c[1], c[2]), v3(0.2126f, 0.587f, 0.114f));
}
static int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
static float min1(float e) { return (1.0f < e) ? 1.0f : e; }

static void blend_tile(uint32_t x0, uint32_t y0, uint32_t tw, uint32_t th, uint32_t W, uint32_t H,
                       uint32_t level, const float* pix, const float* nrm, const float* pos,
                       const float* dif, float* out)
{
    const int scale = (int)pow(2, (double)level);
    float white = 0.0f, mind = INFINITY, maxd = -INFINITY;
    for (uint32_t x = x0; x < x0 + tw; ++x)
        for (uint32_t y = y0; y < y0 + th; ++y)
            for (int u = 0; u < 25; ++u) {
                const int ix = clampi((int)x + (u % 5 - 2) * scale, 0, (int)W - 1);
                const int iy = clampi((int)y + (u / 5 - 2) * scale, 0, (int)H - 1);
                const size_t f = (size_t)iy * W + (size_t)ix;
                white = f_max(white, lum(pix + 3 * f));
                const float len = v3_length(v3(pos[3 * f], pos[3 * f + 1], pos[3 * f + 2]));
                mind = f_min(mind, len);
                maxd = f_max(maxd, len);
            }
    const float range = maxd - mind;
    for (uint32_t x = x0; x < x0 + tw; ++x)
        for (uint32_t y = y0; y < y0 + th; ++y) {
            const size_t c = (size_t)y * W + x;
            float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, wsum = 0.0f;
            for (int u = 0; u < 25; ++u) {
                const int ix = clampi((int)x + (u % 5 - 2) * scale, 0, (int)W - 1);
                const int iy = clampi((int)y + (u / 5 - 2) * scale, 0, (int)H - 1);
                const size_t f = (size_t)iy * W + (size_t)ix;
                po_v3 t = v3_sub(v3(nrm[3 * c], nrm[3 * c + 1], nrm[3 * c + 2]),
                                 v3(nrm[3 * f], nrm[3 * f + 1], nrm[3 * f + 2]));
                float dist = v3_dot(t, t);
                const float nw = min1(expf(-dist / 0.25f));
                t = v3_sub(v3(pos[3 * c], pos[3 * c + 1], pos[3 * c + 2]), v3(pos[3 * f], pos[3 * f + 1], pos[3 * f + 2]));
                dist = v3_dot(t, t);
                const float pw = min1(expf(-dist / (range * range)));
                t = v3_sub(v3(dif[3 * c], dif[3 * c + 1], dif[3 * c + 2]), v3(dif[3 * f], dif[3 * f + 1], dif[3 * f + 2]));
                dist = v3_dot(t, t);
                const float dw = min1(expf(-dist / (white * white)));
                const float w = kWeights[u] * nw * pw * dw;
                r0 = r0 + pix[3 * f] * w;
                r1 = r1 + pix[3 * f + 1] * w;
                r2 = r2 + pix[3 * f + 2] * w;
                wsum = wsum + w;
            }
            out[3 * c] = r0 / wsum;
            out[3 * c + 1] = r1 / wsum;
            out[3 * c + 2] = r2 / wsum;
        }
}

void po_atrous_denoise(const float* pixels, const float* normals, const float* positions,
                       const float* diffuse, uint32_t W, uint32_t H, float* out)
{
    const size_t n = (size_t)W * H * 3;
    float* buf[2];
    buf[0] = (float*)malloc(sizeof(float) * (n ? n : 1));
    buf[1] = out;
    memcpy(buf[0], pixels, sizeof(float) * n);
    for (uint32_t level = 0; level < 5; ++level) {
        const float* src = buf[level % 2];
        float* dst = buf[(level + 1) % 2];
        for (uint32_t x = 0; x < W; x += 64)
            for (uint32_t y = 0; y < H; y += 64) {
                const uint32_t tw = (x + 64 > W) ? W - x : 64;
                const uint32_t th = (y + 64 > H) ? H - y : 64;
                blend_tile(x, y, tw, th, W, H, level, src, normals, positions, diffuse, dst);
            }
    }
    free(buf[0]);
}

/* Util::reinhard_tone_mapping (Util/ToneMappers.cpp:12-44): global white point
 * = max luminance (std::max from 0, so NaN luminances are skipped), then
 * p * (1 + p / w^2) / (1 + p) per channel, in place. */
void po_reinhard(float* pixels, uint32_t W, uint32_t H)
{
    const size_t n = (size_t)W * H;
    float white = 0.0f;
    for (size_t i = 0; i < n; ++i) white = f_max(white, lum(pixels + 3 * i));
    const float w2 = white * white;
    for (size_t i = 0; i < 3 * n; ++i) {
        const float p = pixels[i];
        const float num = p * (1.0f + (p / w2));
        pixels[i] = num / (1.0f + p);
    }
}

/* ---------------------------------------------------------------------------
 * Scene::render_scene_to_file's output step (Core/Scene.cpp:238-246): the flat
 * pixel array reversed (std::reverse, a 180-degree rotation), then written by
 * stb_image_write's stbi_write_hdr: the Radiance header, then per scanline the
 * RGBE encoding (frexp of the largest component), run-length coded per
 * component when 8 <= width < 32768 (runs of >= 3 equal bytes up to 127,
 * literal dumps up to 128).  Components that are NaN or negative make the
 * reference's float-to-byte conversion undefined; they are written as 0 here. */
void po_reverse_pixels(float* pixels, uint32_t n)
{
    for (uint32_t i = 0, j = n ? n - 1 : 0; i < j; ++i, --j)
        for (int c = 0; c < 3; ++c) {
            const float t = pixels[3 * i + c];
            pixels[3 * i + c] = pixels[3 * j + c];
            pixels[3 * j + c] = t;
        }
}

static unsigned char to_byte(float v) { return (v >= 0.0f && v < 256.0f) ? (unsigned char)v : 0; }

void po_rgbe(const float* c, unsigned char* out)
{
    const float m12 = (c[1] < c[2]) ? c[2] : c[1];
    const float maxcomp = (c[0] < m12) ? m12 : c[0];
    if (maxcomp < 1e-32f) {
        out[0] = out[1] = out[2] = out[3] = 0;
        return;
    }
    int e;
    const float normalize = (float)frexp(maxcomp, &e) * 256.0f / maxcomp;
    out[0] = to_byte(c[0] * normalize);
    out[1] = to_byte(c[1] * normalize);
    out[2] = to_byte(c[2] * normalize);
    out[3] = (unsigned char)(e + 128);
}

static size_t put(unsigned char* out, size_t at, size_t cap, const void* src, size_t n)
{
    if (out && at + n <= cap) memcpy(out + at, src, n);
    return at + n;
}

/* Returns the byte length of the file; writes it into `out` when it fits `cap`. */
size_t po_encode_hdr(const float* pixels, uint32_t W, uint32_t H, unsigned char* out, size_t cap)
{
    static const char header[] = "#?RADIANCE\n# Written by stb_image_write.h\nFORMAT=32-bit_rle_rgbe\n";
    char buf[128];
    size_t at = put(out, 0, cap, header, sizeof(header) - 1);
    const int len = snprintf(buf, sizeof buf, "EXPOSURE=          1.0000000000000\n\n-Y %d +X %d\n", (int)H, (int)W);
    at = put(out, at, cap, buf, (size_t)len);
    unsigned char* scratch = (unsigned char*)malloc((size_t)W * 4 + 4);
    for (uint32_t y = 0; y < H; ++y) {
        const float* line = pixels + (size_t)3 * W * y;
        if (W < 8 || W >= 32768) {
            for (uint32_t x = 0; x < W; ++x) {
                unsigned char rgbe[4];
                po_rgbe(line + 3 * x, rgbe);
                at = put(out, at, cap, rgbe, 4);
            }
            continue;
        }
        for (uint32_t x = 0; x < W; ++x) {
            unsigned char rgbe[4];
            po_rgbe(line + 3 * x, rgbe);
            for (int c = 0; c < 4; ++c) scratch[x + (size_t)W * c] = rgbe[c];
        }
        const unsigned char sh[4] = {2, 2, (unsigned char)((W & 0xff00) >> 8), (unsigned char)(W & 0xff)};
        at = put(out, at, cap, sh, 4);
        for (int c = 0; c < 4; ++c) {
            const unsigned char* comp = scratch + (size_t)W * c;
            uint32_t x = 0;
            while (x < W) {
                uint32_t r = x;   /* first run of three equal bytes at or after x */
                while (r + 2 < W) {
                    if (comp[r] == comp[r + 1] && comp[r] == comp[r + 2]) break;
                    ++r;
                }
                if (r + 2 >= W) r = W;
                while (x < r) {   /* literals up to the run */
                    uint32_t n = r - x;
                    if (n > 128) n = 128;
                    const unsigned char lb = (unsigned char)n;
                    at = put(out, at, cap, &lb, 1);
                    at = put(out, at, cap, comp + x, n);
                    x += n;
                }
                if (r + 2 < W) {   /* the run itself */
                    while (r < W && comp[r] == comp[x]) ++r;
                    while (x < r) {
                        uint32_t n = r - x;
                        if (n > 127) n = 127;
                        const unsigned char rb[2] = {(unsigned char)(n + 128), comp[x]};
                        at = put(out, at, cap, rb, 2);
                        x += n;
                    }
                }
            }
        }
    }
    free(scratch);
    return at;
}
