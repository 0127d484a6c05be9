// The reference's image output: Scene::render_scene_to_file (Core/Scene.cpp:238-246)
// reverses the flat pixel array and writes it with stb_image_write's
// stbi_write_hdr, a Radiance file of RGBE pixels, run-length coded per
// component on scanlines 8..32767 pixels wide.
//
// On the device: one thread per pixel encodes RGBE (frexp of the largest
// component; mantissa scaled by 256 / max, truncated), then one CTA per
// scanline run-length codes its four components, each into a slot of
// W + ceil(W / 128) bytes (the worst case: all literals).  The host writes
// the header and concatenates the slots.  NaN or negative components, whose
// conversion to a byte is undefined in the reference, are written as 0.
#include "capi_internal.h"
#include "kernels_render.h"

#include <cstdio>
#include <cstring>
#include <string>

namespace pico {
namespace {

__device__ __forceinline__ unsigned char to_byte(float v) { return (v >= 0.0f && v < 256.0f) ? (unsigned char)v : 0; }

__global__ void rgbe_kernel(const float* __restrict__ pix, size_t npx, uchar4* __restrict__ out)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < npx; i += (size_t)gridDim.x * blockDim.x) {
        const float r = pix[3 * i], g = pix[3 * i + 1], b = pix[3 * i + 2];
        const float m12 = (g < b) ? b : g;
        const float maxcomp = (r < m12) ? m12 : r;
        uchar4 o = make_uchar4(0, 0, 0, 0);
        if (!(maxcomp < 1e-32f)) {
            int e;
            const float m = frexpf(maxcomp, &e);
            const float normalize = __fdiv_rn(__fmul_rn(m, 256.0f), maxcomp);
            o = make_uchar4(to_byte(__fmul_rn(r, normalize)), to_byte(__fmul_rn(g, normalize)),
                            to_byte(__fmul_rn(b, normalize)), (unsigned char)(e + 128));
        }
        out[i] = o;
    }
}

size_t rle_slot(uint32_t W) { return (size_t)W + (W + 127) / 128; }

// The stbi_write_hdr run-length scheme, one CTA per scanline: the row's RGBE
// texels are staged in shared memory with coalesced loads, then four threads
// code the four components from shared memory (literal runs of up to 128
// bytes until the next run of three or more equal bytes, which is coded in
// pieces of up to 127).
__global__ void rle_row_kernel(const uchar4* __restrict__ rgbe, uint32_t W, uint32_t H, size_t slot,
                               unsigned char* __restrict__ out, uint32_t* __restrict__ lens)
{
    extern __shared__ uchar4 row_px[];
    const uint32_t row = blockIdx.x;
    const uchar4* line = rgbe + (size_t)row * W;
    for (uint32_t x = threadIdx.x; x < W; x += blockDim.x) row_px[x] = line[x];
    __syncthreads();
    const uint32_t c = threadIdx.x;
    if (c >= 4) return;
    auto at = [&](uint32_t x) -> unsigned char {
        const uchar4 v = row_px[x];
        return c == 0 ? v.x : (c == 1 ? v.y : (c == 2 ? v.z : v.w));
    };
    const uint32_t k = row * 4 + c;
    unsigned char* o = out + slot * k;
    uint32_t n = 0, x = 0;
    while (x < W) {
        uint32_t r = x;
        while (r + 2 < W) {
            const unsigned char a = at(r);
            if (a == at(r + 1) && a == at(r + 2)) break;
            ++r;
        }
        if (r + 2 >= W) r = W;
        while (x < r) {
            uint32_t len = r - x;
            if (len > 128) len = 128;
            o[n++] = (unsigned char)len;
            for (uint32_t i = 0; i < len; ++i) o[n++] = at(x + i);
            x += len;
        }
        if (r + 2 < W) {
            const unsigned char v = at(x);
            while (r < W && at(r) == v) ++r;
            while (x < r) {
                uint32_t len = r - x;
                if (len > 127) len = 127;
                o[n++] = (unsigned char)(len + 128);
                o[n++] = v;
                x += len;
            }
        }
    }
    lens[k] = n;
}

}  // namespace

size_t hdr_bound(uint32_t W, uint32_t H)
{
    return 256 + (size_t)H * (4 + 4 * rle_slot(W)) + (size_t)W * H * 4;
}

// Encodes device pixels into a Radiance file image in `out` (host); returns the length.
int encode_hdr(pico_gpu_ctx* ctx, const float* d_pixels, uint32_t W, uint32_t H, std::vector<unsigned char>& out)
{
    cudaStream_t st = ctx->stream;
    const size_t npx = (size_t)W * H;
    const bool rle = W >= 8 && W < 32768;
    const size_t slot = rle_slot(W);
    void* d_rgbe = nullptr;
    void* d_rle = nullptr;
    void* d_lens = nullptr;
    cudaError_t e = cudaMalloc(&d_rgbe, npx * 4 + 16);
    if (e == cudaSuccess && rle) e = cudaMalloc(&d_rle, slot * 4 * H + 16);
    if (e == cudaSuccess && rle) e = cudaMalloc(&d_lens, sizeof(uint32_t) * 4 * H + 16);
    std::vector<unsigned char> rgbe, body;
    std::vector<uint32_t> lens;
    if (e == cudaSuccess && npx) {
        const unsigned blocks = (unsigned)std::min<size_t>((npx + 255) / 256, (size_t)sm_count() * 8);
        rgbe_kernel<<<blocks, 256, 0, st>>>(d_pixels, npx, static_cast<uchar4*>(d_rgbe));
        e = cudaGetLastError();
        if (e == cudaSuccess && rle) {
            // rows are staged in shared memory (W < 32768 texels of 4 bytes)
            const size_t smem = (size_t)W * sizeof(uchar4);
            e = cudaFuncSetAttribute(rle_row_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess)
                rle_row_kernel<<<H, 128, smem, st>>>(static_cast<uchar4*>(d_rgbe), W, H, slot,
                                                     static_cast<unsigned char*>(d_rle),
                                                     static_cast<uint32_t*>(d_lens));
            e = cudaGetLastError();
            lens.resize(4 * (size_t)H);
            body.resize(slot * 4 * H);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(lens.data(), d_lens, lens.size() * 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(body.data(), d_rle, body.size(), cudaMemcpyDeviceToHost, st);
        } else if (e == cudaSuccess) {
            rgbe.resize(npx * 4);
            e = cudaMemcpyAsync(rgbe.data(), d_rgbe, npx * 4, cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(d_rgbe);
    cudaFree(d_rle);
    cudaFree(d_lens);
    if (e != cudaSuccess) return cuda_error(ctx, e, "hdr encode");
    static const char header[] = "#?RADIANCE\n# Written by stb_image_write.h\nFORMAT=32-bit_rle_rgbe\n";
    char res[128];
    const int n = std::snprintf(res, sizeof res, "EXPOSURE=          1.0000000000000\n\n-Y %d +X %d\n", (int)H, (int)W);
    out.assign(header, header + sizeof(header) - 1);
    out.insert(out.end(), res, res + n);
    for (uint32_t y = 0; y < H; ++y) {
        if (!rle) {
            out.insert(out.end(), rgbe.begin() + (size_t)4 * W * y, rgbe.begin() + (size_t)4 * W * (y + 1));
            continue;
        }
        const unsigned char sh[4] = {2, 2, (unsigned char)((W & 0xff00) >> 8), (unsigned char)(W & 0xff)};
        out.insert(out.end(), sh, sh + 4);
        for (uint32_t c = 0; c < 4; ++c) {
            const size_t k = (size_t)y * 4 + c;
            out.insert(out.end(), body.begin() + slot * k, body.begin() + slot * k + lens[k]);
        }
    }
    return PICO_OK;
}

}  // namespace pico

using namespace pico;

extern "C" {

size_t pico_gpu_hdr_bound(uint32_t width, uint32_t height) { return hdr_bound(width, height); }

int pico_gpu_encode_hdr(pico_gpu_ctx* ctx, const float* pixels, uint32_t W, uint32_t H, unsigned char* out,
                        size_t capacity, size_t* length)
{
    if (!ctx || !pixels || !length) return set_error(ctx, PICO_ERR_INVALID_ARG, "null argument");
    const DeviceScope device_scope(ctx->device);
    const size_t n3 = (size_t)W * H * 3;
    void* d = nullptr;
    cudaError_t e = cudaMalloc(&d, n3 * sizeof(float) + 16);
    if (e == cudaSuccess) e = cudaMemcpy(d, pixels, n3 * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(d);
        return cuda_error(ctx, e, "hdr upload");
    }
    std::vector<unsigned char> file;
    const int st = encode_hdr(ctx, static_cast<const float*>(d), W, H, file);
    cudaFree(d);
    if (st != PICO_OK) return st;
    *length = file.size();
    if (!out || capacity < file.size()) return set_error(ctx, PICO_ERR_INVALID_ARG, "output buffer too small");
    std::memcpy(out, file.data(), file.size());
    return PICO_OK;
}

int pico_gpu_render_to_file(pico_gpu_ctx* ctx, const pico_gpu_scene* scene, const pico_camera* camera,
                            const pico_render_config* config, float* pixels, uint32_t* sample_count,
                            float* variance, const char* path)
{
    if (!path) return set_error(ctx, PICO_ERR_INVALID_ARG, "null path");
    int32_t quit = 0;
    int st = pico_gpu_render(ctx, scene, camera, config, pixels, sample_count, variance, &quit);
    if (st != PICO_OK) return st;
    // flip the image (std::reverse of the flat array, Scene.cpp:243-244), in the caller's buffer too
    const size_t npx = (size_t)config->width * config->height;
    for (size_t i = 0, j = npx ? npx - 1 : 0; i < j; ++i, --j)
        for (int c = 0; c < 3; ++c) std::swap(pixels[3 * i + c], pixels[3 * j + c]);
    std::vector<unsigned char> file(hdr_bound(config->width, config->height));
    size_t len = 0;
    st = pico_gpu_encode_hdr(ctx, pixels, config->width, config->height, file.data(), file.size(), &len);
    if (st != PICO_OK) return st;
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_error(ctx, PICO_ERR_INVALID_ARG, std::string("cannot open ") + path);
    const size_t w = std::fwrite(file.data(), 1, len, f);
    std::fclose(f);
    if (w != len) return set_error(ctx, PICO_ERR_INVALID_ARG, std::string("short write to ") + path);
    return PICO_OK;
}

}  // extern "C"
