// crg_dev.cuh — device math of the render core (sm_103a).
//
// Compiled with -fmad=false: every float expression below rounds once per
// operation in the order written, so values that feed a decision (triangle
// hits, sampled directions, film sums) are bit-identical to a CPU evaluation
// of the same formulas.  Where an FMA is wanted (the conservative box test)
// it is written explicitly with __fmaf_rn.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace crg {

struct v3 {
    float x, y, z;
};
__device__ __forceinline__ v3 mk(float x, float y, float z) { return v3{x, y, z}; }
__device__ __forceinline__ v3 add(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ v3 sub(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ v3 mul(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ v3 mulv(v3 a, v3 b) { return v3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ v3 neg(v3 a) { return v3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
    return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// glm::normalize: v * (1 / sqrt(dot(v, v)))
__device__ __forceinline__ v3 normalize(v3 v) { return mul(v, 1.0f / sqrtf(dot(v, v))); }
// glm::reflect(I, N) = I - N * dot(N, I) * 2 (src/render/renderer.cpp:51, 83)
__device__ __forceinline__ v3 reflect(v3 i, v3 n) {
    const float d = dot(n, i);
    return sub(i, v3{(n.x * d) * 2.0f, (n.y * d) * 2.0f, (n.z * d) * 2.0f});
}
__device__ __forceinline__ float mx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float mn(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return mn(mx(x, lo), hi); }
__device__ __forceinline__ float absf(float x) { return x < 0.0f ? -x : x; }

// src/util/numbers.h:10-25
constexpr float kPi = 3.14159265359f;
constexpr float kTau = 6.28318530717f;
constexpr float kInvPi = 1.0f / 3.14159265359f;
constexpr float kInvTau = 1.0f / 6.28318530717f;

// ------------------------------------------------------------------ RNG
// pcg4d (Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 2020),
// keyed by (pixel, sample, dimension group, seed).
struct f4 {
    float x, y, z, w;
};
__device__ __forceinline__ float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ f4 rand4(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    uint32_t x = a * 1664525u + 1013904223u;
    uint32_t y = b * 1664525u + 1013904223u;
    uint32_t z = c * 1664525u + 1013904223u;
    uint32_t w = d * 1664525u + 1013904223u;
    x += y * w;
    y += z * x;
    z += x * y;
    w += y * z;
    x ^= x >> 16;
    y ^= y >> 16;
    z ^= z >> 16;
    w ^= w >> 16;
    x += y * w;
    y += z * x;
    z += x * y;
    w += y * z;
    return f4{u01(x), u01(y), u01(z), u01(w)};
}

// sin(2 pi u), cos(2 pi u): exact reduction to the nearest quarter turn, then
// the Taylor series of sin (to x^9) and cos (to x^10) on [-pi/4, pi/4].
__device__ __forceinline__ void sincos2pi(float u, float *s_out, float *c_out) {
    const float k = floorf(u * 4.0f + 0.5f);
    const float r = u - k * 0.25f;
    const int q = ((int)k) & 3;
    const float x = r * 6.28318548f;
    const float x2 = x * x;
    const float s = x * (1.0f + x2 * (-0.166666672f + x2 * (0.00833333377f + x2 * (-0.000198412701f + x2 * 2.75573188e-06f))));
    const float c = 1.0f + x2 * (-0.5f + x2 * (0.0416666679f + x2 * (-0.00138888892f + x2 * (2.48015876e-05f + x2 * -2.75573188e-07f))));
    float so, co;
    if (q == 0) { so = s; co = c; }
    else if (q == 1) { so = c; co = -s; }
    else if (q == 2) { so = -s; co = -c; }
    else { so = -c; co = s; }
    *s_out = so;
    *c_out = co;
}

// Duff et al. 2017 orthonormal basis, as cr::sampling::build_local (sampling.h:21-33)
struct onb {
    v3 n, t, b;
};
__device__ __forceinline__ onb build_local(v3 n) {
    const float s = (n.z < 0.0f) ? -1.0f : 1.0f;
    const float a = -1.0f / (s + n.z);
    const float b = n.x * n.y * a;
    onb o;
    o.n = n;
    o.t = v3{1.0f + s * n.x * n.x * a, s * b, -s * n.x};
    o.b = v3{b, s + n.y * n.y * a, -n.y};
    return o;
}

// ------------------------------------------------------------------ rays
struct RayPre {
    float ox, oy, oz;
    float ix, iy, iz; // 1 / dir (dir components below 2^-80 clamped)
    float Sx, Sy, Sz;
    float tmin;
    int kx, ky, kz;
    float dx, dy, dz;
};

__device__ __forceinline__ float comp(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ RayPre ray_prep(float ox, float oy, float oz, float dx, float dy, float dz, float tmin) {
    RayPre r;
    r.ox = ox; r.oy = oy; r.oz = oz;
    r.dx = dx; r.dy = dy; r.dz = dz;
    const float tiny = 8.27180613e-25f; // 2^-80
    const float ddx = fabsf(dx) < tiny ? copysignf(tiny, dx) : dx;
    const float ddy = fabsf(dy) < tiny ? copysignf(tiny, dy) : dy;
    const float ddz = fabsf(dz) < tiny ? copysignf(tiny, dz) : dz;
    r.ix = 1.0f / ddx;
    r.iy = 1.0f / ddy;
    r.iz = 1.0f / ddz;
    int kz = 0;
    if (fabsf(dy) > fabsf(dx)) kz = 1;
    if (fabsf(dz) > fabsf(comp(dx, dy, dz, kz))) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dkz = comp(dx, dy, dz, kz);
    if (dkz < 0.0f) { const int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = comp(dx, dy, dz, kx) / dkz;
    r.Sy = comp(dx, dy, dz, ky) / dkz;
    r.Sz = 1.0f / dkz;
    r.tmin = tmin;
    return r;
}

// Woop, Benthin & Wald 2013 watertight test (bit-identical to the CPU form).
__device__ __forceinline__ bool watertight(const RayPre &r, float4 a, float4 b, float4 c, float &t, float &u, float &v) {
    const float Ax_ = a.x - r.ox, Ay_ = a.y - r.oy, Az_ = a.z - r.oz;
    const float Bx_ = b.x - r.ox, By_ = b.y - r.oy, Bz_ = b.z - r.oz;
    const float Cx_ = c.x - r.ox, Cy_ = c.y - r.oy, Cz_ = c.z - r.oz;
    const float Akz = comp(Ax_, Ay_, Az_, r.kz), Bkz = comp(Bx_, By_, Bz_, r.kz), Ckz = comp(Cx_, Cy_, Cz_, r.kz);
    const float Ax = comp(Ax_, Ay_, Az_, r.kx) - r.Sx * Akz;
    const float Ay = comp(Ax_, Ay_, Az_, r.ky) - r.Sy * Akz;
    const float Bx = comp(Bx_, By_, Bz_, r.kx) - r.Sx * Bkz;
    const float By = comp(Bx_, By_, Bz_, r.ky) - r.Sy * Bkz;
    const float Cx = comp(Cx_, Cy_, Cz_, r.kx) - r.Sx * Ckz;
    const float Cy = comp(Cx_, Cy_, Cz_, r.ky) - r.Sy * Ckz;
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = (U + V) + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * Akz;
    const float Bz = r.Sz * Bkz;
    const float Cz = r.Sz * Ckz;
    const float T = (U * Az + V * Bz) + W * Cz;
    t = T / det;
    u = V / det;
    v = W / det;
    return true;
}

__device__ __forceinline__ bool accept_hit(float t, uint32_t prim, float tmin, float best_t, uint32_t best_prim) {
    if (!(t > tmin)) return false;
    if (t < best_t) return true;
    return t == best_t && best_prim != 0xFFFFFFFFu && prim < best_prim;
}

// ------------------------------------------------------------------ wide BVH
// Node of width W: 24-byte header {float p[3]; u8 e[3]; u8 imask; u32
// child_base; u32 tri_base}, then meta[W], qlo[3][W], qhi[3][W], padded to a
// multiple of 16 bytes.  Child box a-axis = p + 2^(e-127) * q.
template <int W> struct NodeLayout {
    static constexpr int BYTES = ((24 + 7 * W) + 15) / 16 * 16;
    static constexpr int WORDS = BYTES / 4;
    static constexpr int VEC = BYTES / 16;
};

template <int W> __device__ __forceinline__ uint32_t nbyte(const uint32_t *w, int b) {
    return (w[b >> 2] >> ((b & 3) * 8)) & 0xFFu;
}

struct TravStats {
    uint32_t nodes, tris;
};

constexpr int kStack = 64;

// Closest hit (ANY = false) or occlusion (ANY = true) through a W-wide
// compressed BVH.  Children are visited in the octant order of Ylitie et al.
// 2017: internal child with code c sets hit bit 24 + (c ^ oct); the highest
// bit is taken first.  Returns the error flag (stack overflow) in *err.
template <int W, bool ANY, bool COUNT>
__device__ __forceinline__ void traverse(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                         const RayPre &r, float tmax, float &best_t, uint32_t &best_prim,
                                         uint32_t &best_slot, float &best_u, float &best_v, bool &occluded,
                                         TravStats &st, uint32_t &err) {
    using L = NodeLayout<W>;
    const uint32_t oct = (r.dx < 0.0f ? 4u : 0u) | (r.dy < 0.0f ? 2u : 0u) | (r.dz < 0.0f ? 1u : 0u);
    best_t = tmax;
    best_prim = 0xFFFFFFFFu;
    best_slot = 0xFFFFFFFFu;
    occluded = false;
    uint2 stack[kStack];
    int sp = 0;
    // current node group {child_base, hits << 24 | imask}; the root is the
    // single internal child (code 0) of a virtual parent.
    uint2 ng = make_uint2(0u, (1u << (24 + (0u ^ oct))) | 1u);
    uint2 tg = make_uint2(0u, 0u);
    for (;;) {
        // triangles of the current group
        while (tg.y != 0u) {
            const int i = __ffs(tg.y) - 1;
            tg.y &= tg.y - 1u;
            const uint32_t slot = tg.x + (uint32_t)i;
            const float4 a = __ldg(&tris[slot * 3 + 0]);
            const float4 b = __ldg(&tris[slot * 3 + 1]);
            const float4 c = __ldg(&tris[slot * 3 + 2]);
            const uint32_t prim = __float_as_uint(a.w);
            if (COUNT) st.tris++;
            float t, u, v;
            if (!watertight(r, a, b, c, t, u, v)) continue;
            if (ANY) {
                if (t > r.tmin && t < tmax) { occluded = true; return; }
                continue;
            }
            if (accept_hit(t, prim, r.tmin, best_t, best_prim)) {
                best_t = t;
                best_prim = prim;
                best_slot = slot;
                best_u = u;
                best_v = v;
            }
        }
        // next internal child
        if ((ng.y >> 24) == 0u) {
            if (sp == 0) break;
            ng = stack[--sp];
        }
        const uint32_t hb = ng.y >> 24;
        const uint32_t pos = 31u - __clz(hb);
        const uint32_t code = pos ^ oct;
        ng.y &= ~(1u << (24 + pos));
        const uint32_t child = ng.x + __popc(ng.y & ((1u << code) - 1u) & 0xFFu);
        if ((ng.y >> 24) != 0u) {
            if (sp < kStack) stack[sp++] = ng;
            else err = 1u;
        }
        // load and decode the node
        uint32_t w[L::WORDS];
        const uint4 *np = nodes + (size_t)child * L::VEC;
#pragma unroll
        for (int k = 0; k < L::VEC; ++k) {
            const uint4 q = __ldg(np + k);
            w[4 * k + 0] = q.x;
            w[4 * k + 1] = q.y;
            w[4 * k + 2] = q.z;
            w[4 * k + 3] = q.w;
        }
        if (COUNT) st.nodes++;
        const float px = __uint_as_float(w[0]), py = __uint_as_float(w[1]), pz = __uint_as_float(w[2]);
        const uint32_t eb = w[3];
        const float sx = __uint_as_float((eb & 0xFFu) << 23) * r.ix;
        const float sy = __uint_as_float(((eb >> 8) & 0xFFu) << 23) * r.iy;
        const float sz = __uint_as_float(((eb >> 16) & 0xFFu) << 23) * r.iz;
        const float ox = (px - r.ox) * r.ix;
        const float oy = (py - r.oy) * r.iy;
        const float oz = (pz - r.oz) * r.iz;
        const uint32_t imask = eb >> 24;
        const uint32_t cbase = w[4], tbase = w[5];
        const float tfar_lim = best_t;
        uint32_t hit_int = 0u, hit_tri = 0u;
#pragma unroll
        for (int s = 0; s < W; ++s) {
            const uint32_t meta = nbyte<W>(w, 24 + s);
            if (meta == 0u) continue;
            const float qlx = (float)nbyte<W>(w, 24 + W + 0 * W + s);
            const float qly = (float)nbyte<W>(w, 24 + W + 1 * W + s);
            const float qlz = (float)nbyte<W>(w, 24 + W + 2 * W + s);
            const float qhx = (float)nbyte<W>(w, 24 + 4 * W + 0 * W + s);
            const float qhy = (float)nbyte<W>(w, 24 + 4 * W + 1 * W + s);
            const float qhz = (float)nbyte<W>(w, 24 + 4 * W + 2 * W + s);
            const float tx0 = __fmaf_rn(r.ix >= 0.0f ? qlx : qhx, sx, ox);
            const float tx1 = __fmaf_rn(r.ix >= 0.0f ? qhx : qlx, sx, ox);
            const float ty0 = __fmaf_rn(r.iy >= 0.0f ? qly : qhy, sy, oy);
            const float ty1 = __fmaf_rn(r.iy >= 0.0f ? qhy : qly, sy, oy);
            const float tz0 = __fmaf_rn(r.iz >= 0.0f ? qlz : qhz, sz, oz);
            const float tz1 = __fmaf_rn(r.iz >= 0.0f ? qhz : qlz, sz, oz);
            const float tn = fmaxf(fmaxf(tx0, ty0), fmaxf(tz0, r.tmin));
            const float tf = fminf(fminf(tx1, ty1), fminf(tz1, tfar_lim));
            if (!(tn <= tf * 1.00000095f)) continue;
            const uint32_t lo5 = meta & 31u;
            if (lo5 >= 24u) hit_int |= 1u << ((lo5 - 24u) ^ oct);
            else hit_tri |= (meta >> 5) << lo5;
        }
        ng = make_uint2(cbase, (hit_int << 24) | imask);
        tg = make_uint2(tbase, hit_tri);
    }
}

} // namespace crg
