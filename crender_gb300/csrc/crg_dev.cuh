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
    float okx, oky, okz; // origin permuted to (kx, ky, kz)
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
    r.okx = comp(ox, oy, oz, kx);
    r.oky = comp(ox, oy, oz, ky);
    r.okz = comp(ox, oy, oz, kz);
    r.tmin = tmin;
    return r;
}

// Woop, Benthin & Wald 2013 watertight test, bit-identical to the CPU form
// (scalar operations only: paired FP32 multiplies and adds may be fused into
// an FMA by the compiler, which would change the rounding).  Returns false
// unless the ray crosses the triangle; fills t and the scaled barycentrics
// (V, W, det) from which u = V / det and v = W / det are formed on acceptance.
struct TriHit {
    float t, V, W, det;
};
__device__ __forceinline__ bool watertight(const RayPre &r, float4 a, float4 b, float4 c, TriHit &h) {
    const float Akx = comp(a.x, a.y, a.z, r.kx) - r.okx, Aky = comp(a.x, a.y, a.z, r.ky) - r.oky;
    const float Akz = comp(a.x, a.y, a.z, r.kz) - r.okz;
    const float Bkx = comp(b.x, b.y, b.z, r.kx) - r.okx, Bky = comp(b.x, b.y, b.z, r.ky) - r.oky;
    const float Bkz = comp(b.x, b.y, b.z, r.kz) - r.okz;
    const float Ckx = comp(c.x, c.y, c.z, r.kx) - r.okx, Cky = comp(c.x, c.y, c.z, r.ky) - r.oky;
    const float Ckz = comp(c.x, c.y, c.z, r.kz) - r.okz;
    const float Ax = Akx - r.Sx * Akz;
    const float Ay = Aky - r.Sy * Akz;
    const float Bx = Bkx - r.Sx * Bkz;
    const float By = Bky - r.Sy * Bkz;
    const float Cx = Ckx - r.Sx * Ckz;
    const float Cy = Cky - r.Sy * Ckz;
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
    h.t = T / det;
    h.V = V;
    h.W = W;
    h.det = det;
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
// multiple of 16 bytes.  Child box a-axis = p + 2^(e-127) * q.  Empty slots
// carry the inverted box (qlo 255, qhi 0) and meta 0.
template <int W> struct NodeLayout {
    static constexpr int BYTES = ((24 + 7 * W) + 15) / 16 * 16;
    static constexpr int WORDS = BYTES / 4;
    static constexpr int VEC = BYTES / 16;
};

template <int W> __device__ __forceinline__ uint32_t nbyte(const uint32_t *w, int b) {
    return (w[b >> 2] >> ((b & 3) * 8)) & 0xFFu;
}

// Byte k of `word` as an exact float: 2^23 + q assembled by PRMT, minus 2^23.
__device__ __forceinline__ float2 qpair(uint32_t word, int k) {
    const float2 biased = make_float2(__uint_as_float(__byte_perm(word, 0x4B000000u, 0x7440u | k)),
                                      __uint_as_float(__byte_perm(word, 0x4B000000u, 0x7440u | (k + 1))));
    return __fadd2_rn(biased, make_float2(-8388608.0f, -8388608.0f));
}

struct TravStats {
    uint32_t nodes, tris;
};

// Slack on the best-hit bound when culling boxes: a triangle's computed t can
// sit below its exact t by more than slab rounding (t = T / det loses digits on
// large or grazing triangles; 2.8e-6 relative was seen on a floor coplanar with
// a box face), so a box is kept while its entry lies within best_t * (1 + 2^-12).
// The CPU oracle uses the same slack, so both find the closest computed t.
constexpr float kHitSlack = 1.000244140625f;

constexpr int kStack = 64;

// Per-ray traversal state (resumable).
struct Trav {
    uint2 ng; // {child_base, internal hits (traversal order) << 24 | imask}
    uint2 tg; // {tri_base, pending triangle bits}
    int sp;
    float best_t, tmax;
    uint32_t best_prim, best_slot;
    float best_V, best_W, best_det;
    uint32_t oct;
    bool occluded;
};

// `root` is the node index of the BVH's root: 0 for a scene of one model, the
// model's first node for a model of a multi-model scene.
__device__ __forceinline__ void trav_init(Trav &T, const RayPre &r, float tmax, uint32_t root = 0u) {
    T.oct = (r.dx < 0.0f ? 4u : 0u) | (r.dy < 0.0f ? 2u : 0u) | (r.dz < 0.0f ? 1u : 0u);
    T.ng = make_uint2(root, (1u << (24 + (0u ^ T.oct))) | 1u); // the root as child code 0 of a virtual parent
    T.tg = make_uint2(0u, 0u);
    T.sp = 0;
    T.best_t = tmax;
    T.tmax = tmax;
    T.best_prim = 0xFFFFFFFFu;
    T.best_slot = 0xFFFFFFFFu;
    T.best_V = T.best_W = 0.0f;
    T.best_det = 1.0f;
    T.occluded = false;
}

// Visits one wide node: returns its {internal group, triangle group}.
template <int W>
__device__ __forceinline__ void visit_node(const uint4 *__restrict__ nodes, uint32_t child, const RayPre &r, uint32_t oct,
                                           float tfar, uint2 &ng, uint2 &tg) {
    using L = NodeLayout<W>;
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
    const float px = __uint_as_float(w[0]), py = __uint_as_float(w[1]), pz = __uint_as_float(w[2]);
    const uint32_t eb = w[3];
    const float sx = __uint_as_float((eb & 0xFFu) << 23) * r.ix;
    const float sy = __uint_as_float(((eb >> 8) & 0xFFu) << 23) * r.iy;
    const float sz = __uint_as_float(((eb >> 16) & 0xFFu) << 23) * r.iz;
    const float ox = (px - r.ox) * r.ix;
    const float oy = (py - r.oy) * r.iy;
    const float oz = (pz - r.oz) * r.iz;
    const uint32_t imask = eb >> 24;
    uint32_t bits = 0u;
    if constexpr (W == 8 || W == 4) {
        // word-aligned quantized planes: pick near/far words once per axis
        constexpr int QW = W / 4; // words per axis row
        constexpr int LO = (24 + W) / 4, HI = (24 + 4 * W) / 4, ME = 24 / 4;
        const bool nxs = r.ix < 0.0f, nys = r.iy < 0.0f, nzs = r.iz < 0.0f;
        const float2 sx2 = make_float2(sx, sx), sy2 = make_float2(sy, sy), sz2 = make_float2(sz, sz);
        const float2 ox2 = make_float2(ox, ox), oy2 = make_float2(oy, oy), oz2 = make_float2(oz, oz);
#pragma unroll
        for (int p = 0; p < W / 2; ++p) {
            const int wi = (2 * p) >> 2, bo = (2 * p) & 3;
            const uint32_t lx = w[LO + 0 * QW + wi], hx = w[HI + 0 * QW + wi];
            const uint32_t ly = w[LO + 1 * QW + wi], hy = w[HI + 1 * QW + wi];
            const uint32_t lz = w[LO + 2 * QW + wi], hz = w[HI + 2 * QW + wi];
            const float2 txn = __ffma2_rn(qpair(nxs ? hx : lx, bo), sx2, ox2);
            const float2 txf = __ffma2_rn(qpair(nxs ? lx : hx, bo), sx2, ox2);
            const float2 tyn = __ffma2_rn(qpair(nys ? hy : ly, bo), sy2, oy2);
            const float2 tyf = __ffma2_rn(qpair(nys ? ly : hy, bo), sy2, oy2);
            const float2 tzn = __ffma2_rn(qpair(nzs ? hz : lz, bo), sz2, oz2);
            const float2 tzf = __ffma2_rn(qpair(nzs ? lz : hz, bo), sz2, oz2);
            const uint32_t mw = w[ME + wi];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const float tn = fmaxf(fmaxf(h ? txn.y : txn.x, h ? tyn.y : tyn.x), fmaxf(h ? tzn.y : tzn.x, r.tmin));
                const float tf = fminf(fminf(h ? txf.y : txf.x, h ? tyf.y : tyf.x), fminf(h ? tzf.y : tzf.x, tfar));
                const uint32_t meta = (mw >> (8 * (bo + h))) & 0xFFu;
                if (tn <= tf * 1.00000095f) bits |= (meta >> 5) << (meta & 31u);
            }
        }
    } else {
#pragma unroll
        for (int s = 0; s < W; ++s) {
            const uint32_t meta = nbyte<W>(w, 24 + s);
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
            const float tf = fminf(fminf(tx1, ty1), fminf(tz1, tfar));
            if (tn <= tf * 1.00000095f) bits |= (meta >> 5) << (meta & 31u);
        }
    }
    // internal hits by octant code -> traversal order (bit position code ^ oct)
    uint32_t m = bits >> 24;
    if (oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (oct & 4u) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    ng = make_uint2(w[4], (m << 24) | imask);
    tg = make_uint2(w[5], bits & 0x00FFFFFFu);
}

// Runs up to `iters` traversal iterations (each: the pending triangle group,
// then one node).  Returns true when the ray is finished.  Children are
// visited in the octant order of Ylitie et al. 2017: the highest set hit bit
// (position code ^ oct) first.  A full stack raises *err instead of trapping.
template <int W, bool ANY, bool COUNT>
__device__ __forceinline__ bool trav_step(Trav &T, uint2 *stack, const uint4 *__restrict__ nodes,
                                          const float4 *__restrict__ tris, const RayPre &r, int iters, TravStats &st,
                                          uint32_t &err) {
    for (int it = 0; it < iters; ++it) {
        while (T.tg.y != 0u) {
            const int i = __ffs(T.tg.y) - 1;
            T.tg.y &= T.tg.y - 1u;
            const uint32_t slot = T.tg.x + (uint32_t)i;
            const float4 a = __ldg(&tris[slot * 3 + 0]);
            const float4 b = __ldg(&tris[slot * 3 + 1]);
            const float4 c = __ldg(&tris[slot * 3 + 2]);
            if (COUNT) st.tris++;
            TriHit h;
            if (!watertight(r, a, b, c, h)) continue;
            if (ANY) {
                if (h.t > r.tmin && h.t < T.tmax) {
                    T.occluded = true;
                    return true;
                }
                continue;
            }
            const uint32_t prim = __float_as_uint(a.w);
            if (accept_hit(h.t, prim, r.tmin, T.best_t, T.best_prim)) {
                T.best_t = h.t;
                T.best_prim = prim;
                T.best_slot = slot;
                T.best_V = h.V;
                T.best_W = h.W;
                T.best_det = h.det;
            }
        }
        if ((T.ng.y >> 24) == 0u) {
            if (T.sp == 0) return true;
            T.ng = stack[--T.sp];
        }
        const uint32_t hb = T.ng.y >> 24;
        const uint32_t pos = 31u - __clz(hb);
        const uint32_t code = pos ^ T.oct;
        T.ng.y &= ~(1u << (24 + pos));
        const uint32_t child = T.ng.x + __popc(T.ng.y & ((1u << code) - 1u) & 0xFFu);
        if ((T.ng.y >> 24) != 0u) {
            if (T.sp < kStack) stack[T.sp++] = T.ng;
            else err = 1u;
        }
        if (COUNT) st.nodes++;
        visit_node<W>(nodes, child, r, T.oct, T.best_t * kHitSlack, T.ng, T.tg);
    }
    return false;
}

// Closest hit (ANY = false) or occlusion (ANY = true) of one ray, to completion.
template <int W, bool ANY, bool COUNT>
__device__ __forceinline__ void traverse(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                         const RayPre &r, float tmax, float &best_t, uint32_t &best_prim,
                                         uint32_t &best_slot, float &best_u, float &best_v, bool &occluded,
                                         TravStats &st, uint32_t &err, uint32_t root = 0u) {
    Trav T;
    uint2 stack[kStack];
    trav_init(T, r, tmax, root);
    while (!trav_step<W, ANY, COUNT>(T, stack, nodes, tris, r, 1 << 30, st, err)) {
    }
    best_t = T.best_t;
    best_prim = T.best_prim;
    best_slot = T.best_slot;
    best_u = T.best_V / T.best_det;
    best_v = T.best_W / T.best_det;
    occluded = T.occluded;
}

// Persistent traversal with per-lane ray refill (the "dynamic fetch" of Aila
// & Laine, "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009).
// A warp runs the loop with all lanes converged; a lane whose query is done
// takes the next index from *head (one atomic per refill, for all idle lanes
// at once) as soon as at least `min_refill` lanes are idle, so long queries
// no longer hold the short ones' lanes idle.  Between refill checks each busy
// lane advances its query by up to STEPS node visits.
//   fetch(idx, payload&, r&, tmax&, root&, nodes&, tris&) -> bool: loads query
//        idx and its first traversal (BVH root node); false = the query was
//        completed inside fetch (no traversal needed)
//   advance(payload, const Trav&, r&, tmax&, root&) -> bool: called when a
//        traversal ends; true = the query goes on with another traversal
//        (the next placement of a scene), set up in r, tmax and root
//   done(payload, const Trav&): consumes a finished query
template <int W, bool ANY, bool COUNT, int STEPS, class Fetch, class Advance, class Done>
__device__ __forceinline__ void dyn_traverse(unsigned int *head, unsigned int n, uint32_t min_refill, Fetch &&fetch,
                                             Advance &&advance, Done &&done, TravStats &st, uint32_t &err) {
    const uint32_t lane = threadIdx.x & 31u;
    bool has = false, exhausted = false;
    uint32_t payload = 0;
    RayPre r;
    Trav T;
    uint2 stack[kStack];
    const uint4 *nodes = nullptr;
    const float4 *tris = nullptr;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, !has);
        if (!exhausted && idle != 0u && ((uint32_t)__popc(idle) >= min_refill || idle == 0xFFFFFFFFu)) {
            const uint32_t cnt = (uint32_t)__popc(idle);
            unsigned int base = 0;
            if (lane == 0) base = atomicAdd(head, cnt);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + cnt >= n) exhausted = true;
            if (!has) {
                const unsigned int my = base + (unsigned int)__popc(idle & ((1u << lane) - 1u));
                if (my < n) {
                    float tmax;
                    uint32_t root = 0u;
                    if (fetch(my, payload, r, tmax, root, nodes, tris)) {
                        trav_init(T, r, tmax, root);
                        has = true;
                    }
                }
            }
        }
        if (!__any_sync(0xFFFFFFFFu, has)) {
            if (exhausted) break;
            continue;
        }
        if (has && trav_step<W, ANY, COUNT>(T, stack, nodes, tris, r, STEPS, st, err)) {
            float tmax;
            uint32_t root = 0u;
            if (advance(payload, T, r, tmax, root)) {
                trav_init(T, r, tmax, root);
            } else {
                has = false;
                done(payload, T);
            }
        }
    }
}

} // namespace crg
