// post.cu — image post-processing (bloom, gray scale, tone mapping).
//
// Restates cr::post_processor::process (CRender
// src/render/post/post_processor.cpp:110-307) and its two compute shaders
// (assets/app/shaders/blur.comp, post_process.comp) as CUDA kernels on RGBA32F
// device images.  The passes and their order are the reference's:
//
//   bloom:  threshold (_brightness) -> 10 separable blur passes, horizontal
//           on even passes, ping-ponging between two images (_blur)
//   final:  source (+ bloom * strength) -> gray scale -> tone mapping
//
// Every float operation is written in the shader's order and compiled
// without contraction (-fmad=false), so results equal the oracle's CPU
// restatement bit for bit except where powf is involved (tone-mapping gamma).
//
// Each pixel of a pass costs 16 bytes read + 16 bytes written in HBM/L2; the
// 15-tap neighbourhoods are staged in shared memory (a row segment for the
// horizontal pass, a column tile for the vertical one), so each texel is read
// from global memory once per pass.
#include <algorithm>
#include <cstdint>

#include "crg_internal.h"

namespace crg {
namespace {

// blur.comp:11-19 (the GLSL float array)
__constant__ float kBlurW[8] = {0.19744746769063704f, 0.1746973469158936f, 0.12099884565428047f,
                                0.06560233156931679f, 0.027839605612666265f, 0.009246250740395456f,
                                0.002403157286908872f, 0.00048872837522002f};

struct PostDims {
    uint32_t w, h;   // image size
    uint32_t rw, rh; // region the reference's dispatches cover (8 * floor(n / 8) in FAITHFUL mode)
    uint32_t faithful;
    float threshold;
};

constexpr int kRowTile = 256;          // horizontal pass: pixels of a row per block
constexpr int kColW = 32, kColH = 32;  // vertical pass: tile of columns x rows per block
constexpr int kHalo = 7;

// _brightness (post_processor.cpp:296-307) visits pixel (i % w, i / h) for
// i < w*h.  Pixel (x, y) is visited iff some i = x + k*w lies in [y*h, y*h + h)
// and below w*h; visits are idempotent, so one visit decides.
__device__ __forceinline__ bool bright_visited(uint32_t x, uint32_t y, const PostDims &p) {
    if (!p.faithful) return true;
    const unsigned long long lo = (unsigned long long)y * p.h;
    const unsigned long long i0 = lo + ((unsigned long long)x + p.w - lo % p.w) % p.w;
    return i0 < lo + p.h && i0 < (unsigned long long)p.w * p.h;
}

__device__ __forceinline__ float4 bright(float4 c, uint32_t x, uint32_t y, const PostDims &p) {
    if (!bright_visited(x, y, p)) return c;
    // glm::dot(vec3, vec3(0.2126, 0.7152, 0.0722)): (x*bx + y*by) + z*bz
    const float l = (c.x * 0.2126f + c.y * 0.7152f) + c.z * 0.0722f;
    if (l < p.threshold) return make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    return c;
}

// blur.comp:21-44 for one pixel: centre * w0, then +i and -i for i = 1..7.
__device__ __forceinline__ float4 blur_taps(const float4 *s, int stride) {
    const float4 c = s[0];
    float r = c.x * kBlurW[0], g = c.y * kBlurW[0], b = c.z * kBlurW[0];
#pragma unroll
    for (int i = 1; i < 8; ++i) {
        const float4 a = s[i * stride];
        const float4 d = s[-i * stride];
        const float wi = kBlurW[i];
        r = r + a.x * wi;
        g = g + a.y * wi;
        b = b + a.z * wi;
        r = r + d.x * wi;
        g = g + d.y * wi;
        b = b + d.z * wi;
    }
    return make_float4(r, g, b, 1.0f);
}

// Horizontal pass.  BRIGHT: the source is the un-thresholded image and the
// threshold is applied to each staged texel (the first pass reads _brightness's
// output, which is never stored).  Pixels outside the covered region are
// written as zero, as the reference clears its target before each dispatch.
template <bool BRIGHT>
__global__ void __launch_bounds__(kRowTile) k_blur_h(const float4 *__restrict__ src, float4 *__restrict__ dst,
                                                     PostDims p) {
    __shared__ float4 row[kRowTile + 2 * kHalo];
    const uint32_t y = blockIdx.y;
    const int x0 = (int)(blockIdx.x * kRowTile);
    const float4 *srow = src + (size_t)y * p.w;
    for (int i = threadIdx.x; i < kRowTile + 2 * kHalo; i += kRowTile) {
        const int x = x0 + i - kHalo;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (x >= 0 && x < (int)p.w) {
            v = srow[x];
            if (BRIGHT) v = bright(v, (uint32_t)x, y, p);
        }
        row[i] = v;
    }
    __syncthreads();
    const uint32_t x = (uint32_t)x0 + threadIdx.x;
    if (x >= p.w) return;
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (x < p.rw && y < p.rh) out = blur_taps(&row[threadIdx.x + kHalo], 1);
    dst[(size_t)y * p.w + x] = out;
}

__global__ void __launch_bounds__(kColW * 8) k_blur_v(const float4 *__restrict__ src, float4 *__restrict__ dst,
                                                      PostDims p) {
    __shared__ float4 col[kColH + 2 * kHalo][kColW];
    const uint32_t x = blockIdx.x * kColW + threadIdx.x;
    const int y0 = (int)(blockIdx.y * kColH);
    for (int r = threadIdx.y; r < kColH + 2 * kHalo; r += 8) {
        const int y = y0 + r - kHalo;
        float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (x < p.w && y >= 0 && y < (int)p.h) v = src[(size_t)y * p.w + x];
        col[r][threadIdx.x] = v;
    }
    __syncthreads();
    if (x >= p.w) return;
    for (int k = threadIdx.y; k < kColH; k += 8) {
        const uint32_t y = (uint32_t)(y0 + k);
        if (y >= p.h) break;
        float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (x < p.rw && y < p.rh) out = blur_taps(&col[k + kHalo][threadIdx.x], kColW);
        dst[(size_t)y * p.w + x] = out;
    }
}

// post_process.comp:48-51 / 74-108 tone curves
__device__ __forceinline__ float uncharted_map(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}

__device__ __forceinline__ float gamma_of(float c, float inv_gamma) { return powf(c, inv_gamma); }

__device__ __forceinline__ float3 tonemap(float3 c, const crg_post_settings &s) {
    const float e = s.exposure;
    const float ig = 1.0f / s.gamma;
    switch (s.tonemap_type) {
    case CRG_TONEMAP_LINEAR:
        c = make_float3(c.x * e, c.y * e, c.z * e);
        return make_float3(gamma_of(c.x, ig), gamma_of(c.y, ig), gamma_of(c.z, ig));
    case CRG_TONEMAP_REINHARD:
        c = make_float3(c.x * e, c.y * e, c.z * e);
        c = make_float3(c.x / (c.x + 1.0f), c.y / (c.y + 1.0f), c.z / (c.z + 1.0f));
        return make_float3(gamma_of(c.x, ig), gamma_of(c.y, ig), gamma_of(c.z, ig));
    case CRG_TONEMAP_JIM_RICHARD: {
        c = make_float3(c.x * e, c.y * e, c.z * e);
        const float x = fmaxf(0.0f, c.x - 0.004f), y = fmaxf(0.0f, c.y - 0.004f), z = fmaxf(0.0f, c.z - 0.004f);
        return make_float3((x * (6.2f * x + 0.5f)) / (x * (6.2f * x + 1.7f) + 0.06f),
                           (y * (6.2f * y + 0.5f)) / (y * (6.2f * y + 1.7f) + 0.06f),
                           (z * (6.2f * z + 0.5f)) / (z * (6.2f * z + 1.7f) + 0.06f));
    }
    case CRG_TONEMAP_UNCHARTED: {
        c = make_float3(c.x * e, c.y * e, c.z * e);
        const float ws = 1.0f / uncharted_map(11.2f);
        c = make_float3(uncharted_map(2.0f * c.x) * ws, uncharted_map(2.0f * c.y) * ws, uncharted_map(2.0f * c.z) * ws);
        return make_float3(gamma_of(c.x, ig), gamma_of(c.y, ig), gamma_of(c.z, ig));
    }
    default:
        return c;
    }
}

// post_process.comp:116-136
__global__ void __launch_bounds__(256) k_post_final(const float4 *__restrict__ src, const float4 *__restrict__ bloom,
                                                    float4 *__restrict__ dst, PostDims p, crg_post_settings s) {
    const size_t n = (size_t)p.w * p.h;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t x = (uint32_t)(i % p.w), y = (uint32_t)(i / p.w);
        float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (x < p.rw && y < p.rh) {
            const float4 v = src[i];
            float3 f = make_float3(v.x, v.y, v.z);
            if (s.bloom) {
                const float4 b = bloom[i];
                const float k = s.bloom_strength;
                f = make_float3(f.x + b.x * k, f.y + b.y * k, f.z + b.z * k);
            }
            if (s.gray_scale) {
                const float g = (0.2126f * f.x + 0.7162f * f.y) + 0.0722f * f.z;
                f = make_float3(g, g, g);
            }
            if (s.tonemapping) f = tonemap(f, s);
            out = make_float4(f.x, f.y, f.z, 1.0f);
        }
        dst[i] = out;
    }
}

} // namespace
} // namespace crg

using namespace crg;

extern "C" crg_status crg_post_settings_default(crg_post_settings *s) {
    if (!s) return CRG_ERR_INVALID_ARG;
    *s = crg_post_settings{};
    s->bloom = 0;
    s->bloom_threshold = 0.7f;
    s->bloom_strength = 1.0f;
    s->gray_scale = 0;
    s->tonemapping = 0;
    s->tonemap_type = CRG_TONEMAP_LINEAR;
    s->exposure = 1.0f;
    s->gamma = 2.2f;
    s->mode = CRG_POST_FAITHFUL;
    return CRG_OK;
}

extern "C" crg_status crg_post_process(crg_context *ctx, const float *d_src, float *d_dst, uint32_t width,
                                       uint32_t height, const crg_post_settings *settings, crg_stream stream) {
    if (!ctx || !d_src || !d_dst || !settings) return set_error(ctx, CRG_ERR_INVALID_ARG, "null argument");
    if (width == 0 || height == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "empty image");
    if (width > 65536u * kRowTile || height > 65535u) return set_error(ctx, CRG_ERR_INVALID_ARG, "image too large");
    if (d_src == d_dst) return set_error(ctx, CRG_ERR_INVALID_ARG, "source and destination alias");
    const crg_post_settings &s = *settings;
    if (s.mode > CRG_POST_FULL) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad post-process mode");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t npix = (size_t)width * height;
    if (!s.bloom && !s.gray_scale && !s.tonemapping) {
        // post_processor.cpp:112-114: nothing enabled returns the input
        CRG_CUDA(ctx, cudaMemcpyAsync(d_dst, d_src, npix * 16, cudaMemcpyDeviceToDevice, st));
        return CRG_OK;
    }
    PostDims p;
    p.w = width;
    p.h = height;
    p.faithful = s.mode == CRG_POST_FAITHFUL;
    p.rw = p.faithful ? width / 8 * 8 : width;
    p.rh = p.faithful ? height / 8 * 8 : height;
    p.threshold = s.bloom_threshold;
    const float4 *src = (const float4 *)d_src;
    float4 *b0 = nullptr;
    if (s.bloom) {
        crg_status rc = dev_alloc(ctx, ctx->post_ws, npix * 32);
        if (rc != CRG_OK) return rc;
        b0 = (float4 *)ctx->post_ws.ptr;
        float4 *b1 = b0 + npix;
        const dim3 gh((width + kRowTile - 1) / kRowTile, height);
        const dim3 gv((width + kColW - 1) / kColW, (height + kColH - 1) / kColH);
        // _blur (post_processor.cpp:246-294): pass i reads buffers[i % 2] and
        // writes the other; even passes are horizontal; the result is buffers[0].
        // buffers[0] starts as the thresholded image, applied inside pass 0.
        k_blur_h<true><<<gh, kRowTile, 0, st>>>(src, b1, p);
        for (int i = 1; i < 10; ++i) {
            const float4 *from = (i % 2 == 0) ? b0 : b1;
            float4 *to = (i % 2 == 0) ? b1 : b0;
            if (i % 2 == 0) k_blur_h<false><<<gh, kRowTile, 0, st>>>(from, to, p);
            else k_blur_v<<<gv, dim3(kColW, 8), 0, st>>>(from, to, p);
        }
        CRG_CUDA(ctx, cudaGetLastError());
    }
    const unsigned blocks = (unsigned)std::min<size_t>((npix + 255) / 256, (size_t)std::max(ctx->sm_count, 1) * 8);
    k_post_final<<<blocks, 256, 0, st>>>(src, b0, (float4 *)d_dst, p, s);
    CRG_CUDA(ctx, cudaGetLastError());
    return CRG_OK;
}
