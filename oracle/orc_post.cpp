// orc_post.cpp — CPU restatement of CRender's post-processor.  TEST INFRASTRUCTURE ONLY.
//
// Follows cr::post_processor::process, _blur and _brightness
// (src/render/post/post_processor.cpp:110-307) and the shaders they dispatch
// (assets/app/shaders/blur.comp:1-44, post_process.comp:1-136) step by step,
// with the OpenGL textures replaced by host arrays:
//   - glClearTexImage(target, ..., nullptr) before each dispatch -> zero fill;
//   - glDispatchCompute(floor(W/8), floor(H/8)) with 8x8 groups -> only
//     x < 8*floor(W/8), y < 8*floor(H/8) are written (FAITHFUL mode);
//   - texelFetch outside the texture -> zero (GL leaves it undefined; robust
//     access returns zero, which is what the GPU kernels implement).
// Float operations are written in the shaders' order; the library is built
// with -ffp-contract=off so each rounds once.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "orc.h"

namespace {

struct Img {
    uint32_t w, h;
    std::vector<float> px; // RGBA

    Img(uint32_t w_, uint32_t h_) : w(w_), h(h_), px((size_t)w_ * h_ * 4, 0.0f) {}
    // texelFetch with zero outside the image
    void fetch(int x, int y, float out[4]) const {
        if (x < 0 || y < 0 || x >= (int)w || y >= (int)h) {
            out[0] = out[1] = out[2] = out[3] = 0.0f;
            return;
        }
        std::memcpy(out, &px[((size_t)y * w + x) * 4], 16);
    }
    float *at(uint32_t x, uint32_t y) { return &px[((size_t)y * w + x) * 4]; }
};

// blur.comp:11-19
const float kW[8] = {0.19744746769063704f, 0.1746973469158936f, 0.12099884565428047f, 0.06560233156931679f,
                     0.027839605612666265f, 0.009246250740395456f, 0.002403157286908872f, 0.00048872837522002f};

// blur.comp:21-44, one invocation
void blur_pixel(const Img &src, int x, int y, bool horizontal, float out[4]) {
    float c[4];
    src.fetch(x, y, c);
    float r = c[0] * kW[0], g = c[1] * kW[0], b = c[2] * kW[0];
    for (int i = 1; i < 8; ++i) {
        float a[4], d[4];
        if (horizontal) {
            src.fetch(x + i, y, a);
            src.fetch(x - i, y, d);
        } else {
            src.fetch(x, y + i, a);
            src.fetch(x, y - i, d);
        }
        r = r + a[0] * kW[i];
        g = g + a[1] * kW[i];
        b = b + a[2] * kW[i];
        r = r + d[0] * kW[i];
        g = g + d[1] * kW[i];
        b = b + d[2] * kW[i];
    }
    out[0] = r;
    out[1] = g;
    out[2] = b;
    out[3] = 1.0f;
}

// post_process.comp:74-85
float uncharted_map(float x) {
    const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
    return ((x * (A * x + C * B) + D * E) / (x * (A * x + B) + D * F)) - E / F;
}

// post_process.comp:49-108
void tonemap(float c[3], const crg_post_settings &s) {
    const float e = s.exposure, ig = 1.0f / s.gamma;
    switch (s.tonemap_type) {
    case CRG_TONEMAP_LINEAR:
        for (int k = 0; k < 3; ++k) c[k] = std::pow(c[k] * e, ig);
        return;
    case CRG_TONEMAP_REINHARD:
        for (int k = 0; k < 3; ++k) {
            const float v = c[k] * e;
            c[k] = std::pow(v / (v + 1.0f), ig);
        }
        return;
    case CRG_TONEMAP_JIM_RICHARD:
        for (int k = 0; k < 3; ++k) {
            const float v = c[k] * e;
            const float x = std::fmax(0.0f, v - 0.004f);
            c[k] = (x * (6.2f * x + 0.5f)) / (x * (6.2f * x + 1.7f) + 0.06f);
        }
        return;
    case CRG_TONEMAP_UNCHARTED: {
        const float ws = 1.0f / uncharted_map(11.2f);
        for (int k = 0; k < 3; ++k) c[k] = std::pow(uncharted_map(2.0f * (c[k] * e)) * ws, ig);
        return;
    }
    default:
        return;
    }
}

} // namespace

extern "C" int orc_post_process(const float *src, float *dst, uint32_t w, uint32_t h, const crg_post_settings *sp) {
    if (!src || !dst || !sp || w == 0 || h == 0) return 1;
    const crg_post_settings &s = *sp;
    const size_t n = (size_t)w * h;
    // post_processor.cpp:112-114
    if (!s.bloom && !s.gray_scale && !s.tonemapping) {
        std::memcpy(dst, src, n * 16);
        return 0;
    }
    const bool faithful = s.mode == CRG_POST_FAITHFUL;
    const uint32_t rw = faithful ? w / 8 * 8 : w, rh = faithful ? h / 8 * 8 : h;

    Img bloom(w, h);
    if (s.bloom) {
        // _brightness (post_processor.cpp:296-307)
        Img passed(w, h);
        std::memcpy(passed.px.data(), src, n * 16);
        for (uint64_t i = 0; i < (uint64_t)w * h; ++i) {
            const uint64_t x = i % w, y = faithful ? i / h : i / w;
            if (y >= h) continue; // out of bounds in the reference
            float *p = passed.at((uint32_t)x, (uint32_t)y);
            const float lum = (p[0] * 0.2126f + p[1] * 0.7152f) + p[2] * 0.0722f;
            if (lum < s.bloom_threshold) {
                p[0] = p[1] = p[2] = 0.0f;
                p[3] = 1.0f;
            }
        }
        // _blur (post_processor.cpp:246-294)
        Img buf[2] = {passed, Img(w, h)};
        for (int i = 0; i < 10; ++i) {
            const Img &from = buf[i % 2 == 0 ? 0 : 1];
            Img &to = buf[i % 2 != 0 ? 0 : 1];
            std::vector<float> out((size_t)w * h * 4, 0.0f);
            for (uint32_t y = 0; y < rh; ++y)
                for (uint32_t x = 0; x < rw; ++x) blur_pixel(from, (int)x, (int)y, i % 2 == 0, &out[((size_t)y * w + x) * 4]);
            to.px.swap(out);
        }
        bloom = buf[0];
    }
    // post_processor.cpp:160-233 and post_process.comp:116-136
    std::memset(dst, 0, n * 16);
    for (uint32_t y = 0; y < rh; ++y)
        for (uint32_t x = 0; x < rw; ++x) {
            const float *v = src + ((size_t)y * w + x) * 4;
            float f[3] = {v[0], v[1], v[2]};
            if (s.bloom) {
                const float *b = bloom.at(x, y);
                for (int k = 0; k < 3; ++k) f[k] = f[k] + b[k] * s.bloom_strength;
            }
            if (s.gray_scale) {
                const float g = (0.2126f * f[0] + 0.7162f * f[1]) + 0.0722f * f[2];
                f[0] = f[1] = f[2] = g;
            }
            if (s.tonemapping) tonemap(f, s);
            float *o = dst + ((size_t)y * w + x) * 4;
            o[0] = f[0];
            o[1] = f[1];
            o[2] = f[2];
            o[3] = 1.0f;
        }
    return 0;
}
