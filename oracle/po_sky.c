/*
 * Oracle (test infrastructure only): the sky of the reference.
 *
 * Scene::process_globals (Core/Scene.cpp:639-700) stores the sky as an
 * ImageCube: six RGBA8 faces ("Skybox" array of six files), one RGBA float
 * equirectangular image ("Skybox" as one HDRI file) or, without a GLOBALS
 * sky, a black 1x1 image.  ImageCube::sample4 (Core/Image.cpp:361-397) picks the
 * nearest texel: resolve_cubemap_UV (Image.cpp:428-466) maps the direction to a
 * face and (u, v), get_data_ptr (Image.cpp:400-425) truncates u*W and v*H and
 * wraps them modulo the size; RGBA8 texels are divided by 255.
 */
#include "po_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static size_t sky_bytes(const po_sky* k)
{
    if (k->kind == PO_SKY_CUBE_RGBA8) return (size_t)6 * k->width * k->height * 4;
    if (k->kind == PO_SKY_EQUIRECT_RGBAF) return (size_t)k->width * k->height * 4 * sizeof(float);
    return 0;
}

void po_scene_set_sky(po_scene* s, const po_sky* sky, const float* rgb)
{
    free(s->sky_pixels);
    s->sky_pixels = NULL;
    memset(&s->sky, 0, sizeof(s->sky));
    for (int c = 0; c < 3; ++c) s->sky_rgb[c] = rgb ? rgb[c] : 0.0f;
    if (!sky) return;
    s->sky = *sky;
    const size_t n = sky_bytes(sky);
    if (n) {
        s->sky_pixels = malloc(n);
        memcpy(s->sky_pixels, sky->pixels, n);
    }
    s->sky.pixels = s->sky_pixels;
}

/* Image::get_data_ptr: uint32_t(uv.x * width) % width (a float product, truncated). */
static uint32_t texel(float uv, uint32_t n) { return (uint32_t)(uv * (float)n) % n; }

static po_v4 sample4(const po_sky* k, const float* rgb, po_v3 v)
{
    if (k->kind == PO_SKY_CUBE_RGBA8) {
        /* ImageCube::resolve_cubemap_UV(v, face, uv), glm::abs is x >= 0 ? x : -x */
        const float ax = v.x >= 0.0f ? v.x : -v.x, ay = v.y >= 0.0f ? v.y : -v.y, az = v.z >= 0.0f ? v.z : -v.z;
        uint32_t face;
        float ma, u, w;
        if (az >= ax && az >= ay) {
            face = v.z < 0.0f ? 5 : 4;
            ma = 0.5f / az;
            u = v.z < 0.0f ? -v.x : v.x;
            w = -v.y;
        } else if (ay >= ax) {
            face = v.y < 0.0f ? 3 : 2;
            ma = 0.5f / ay;
            u = v.x;
            w = v.y < 0.0f ? -v.z : v.z;
        } else {
            face = v.x < 0.0f ? 1 : 0;
            ma = 0.5f / ax;
            u = v.x < 0.0f ? v.z : -v.z;
            w = -v.y;
        }
        u = u * ma + 0.5f;
        w = w * ma + 0.5f;
        const uint32_t x = texel(u, k->width), y = texel(w, k->height);
        const unsigned char* p = (const unsigned char*)k->pixels +
                                 4 * ((size_t)face * k->width * k->height + (size_t)y * k->width + x);
        return v4(p[0] / 255.0f, p[1] / 255.0f, p[2] / 255.0f, p[3] / 255.0f);
    }
    if (k->kind == PO_SKY_EQUIRECT_RGBAF) {
        /* ImageCube::resolve_cubemap_UV(v, uv): (atan2(z, x), asin(y)) / (2 pi, pi) + 0.5, v flipped */
        float u = atan2f(v.z, v.x);
        float w = (float)asin((double)v.y);
        u = u * (float)(1.0 / (3.14159265358979323846 * 2.0f));
        w = w * (float)(1.0 / 3.14159265358979323846);
        u = u + 0.5f;
        w = w + 0.5f;
        w = 1.0f - w;
        const uint32_t x = texel(u, k->width), y = texel(w, k->height);
        const float* p = (const float*)k->pixels + 4 * ((size_t)y * k->width + x);
        return v4(p[0], p[1], p[2], p[3]);
    }
    return v4(rgb[0], rgb[1], rgb[2], 0.0f);
}

po_v4 po_sky_lookup(const po_scene* s, po_v3 d) { return sample4(&s->sky, s->sky_rgb, d); }

void po_sky_sample(const po_sky* sky, const float* dirs, uint32_t n, float* rgba)
{
    static const float black[3] = {0.0f, 0.0f, 0.0f};
    for (uint32_t i = 0; i < n; ++i) {
        const po_v4 c = sample4(sky, black, v3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
        rgba[4 * i] = c.x; rgba[4 * i + 1] = c.y; rgba[4 * i + 2] = c.z; rgba[4 * i + 3] = c.w;
    }
}
