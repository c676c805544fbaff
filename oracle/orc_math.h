/*
 * orc_math.h — scalar math of the CPU oracle.  TEST INFRASTRUCTURE ONLY: the
 * oracle is the checker for the GB300 kernels and is never linked into the
 * product library.
 *
 * Every float expression here is evaluated in IEEE binary32 with one rounding
 * per operation (the oracle is compiled with -ffp-contract=off and without
 * -ffast-math), in the operand order written.  The device code evaluates the
 * same formulas in the same order with FMA contraction disabled, so the two
 * agree bit for bit wherever they run the same algorithm.
 */
#ifndef ORC_MATH_H
#define ORC_MATH_H

#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

struct v3 {
    float x, y, z;
};
static inline v3 mk(float x, float y, float z) { return v3{x, y, z}; }
static inline v3 add(v3 a, v3 b) { return v3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline v3 sub(v3 a, v3 b) { return v3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline v3 mul(v3 a, float s) { return v3{a.x * s, a.y * s, a.z * s}; }
static inline v3 mulv(v3 a, v3 b) { return v3{a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline v3 neg(v3 a) { return v3{-a.x, -a.y, -a.z}; }
static inline float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 cross(v3 a, v3 b) {
    return v3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
/* glm::normalize: v * inversesqrt(dot(v, v)) with inversesqrt = 1/sqrt. */
static inline v3 normalize(v3 v) { return mul(v, 1.0f / std::sqrt(dot(v, v))); }
/* glm::reflect(I, N) = I - N * dot(N, I) * 2 (src/render/renderer.cpp:51, 83). */
static inline v3 reflect(v3 i, v3 n) {
    const float d = dot(n, i);
    return sub(i, v3{(n.x * d) * 2.0f, (n.y * d) * 2.0f, (n.z * d) * 2.0f});
}
static inline float maxf(float a, float b) { return a > b ? a : b; }
static inline float minf(float a, float b) { return a < b ? a : b; }
static inline float clampf(float x, float lo, float hi) { return minf(maxf(x, lo), hi); }
static inline float absf(float x) { return x < 0.0f ? -x : x; }

/* Constants of src/util/numbers.h:10-25. */
static const float kPi = 3.14159265359f;
static const float kTau = 6.28318530717f;
static const float kInvPi = 1.0f / 3.14159265359f;
static const float kInvTau = 1.0f / 6.28318530717f;

/* ---------------------------------------------------------------- RNG
 * Counter-based: pcg4d of Jarzynski & Olano, "Hash Functions for GPU
 * Rendering", JCGT 9(3), 2020.  Key = (pixel, sample, dimension group, seed);
 * each call yields four independent 32-bit values. */
struct u4 {
    uint32_t x, y, z, w;
};
static inline u4 pcg4d(u4 v) {
    v.x = v.x * 1664525u + 1013904223u;
    v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u;
    v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.w += v.y * v.z;
    v.x ^= v.x >> 16;
    v.y ^= v.y >> 16;
    v.z ^= v.z >> 16;
    v.w ^= v.w >> 16;
    v.x += v.y * v.w;
    v.y += v.z * v.x;
    v.z += v.x * v.y;
    v.w += v.y * v.z;
    return v;
}
/* Top 24 bits to a float in [0, 1) (exact). */
static inline float u01(uint32_t h) { return (float)(h >> 8) * (1.0f / 16777216.0f); }
struct f4 {
    float x, y, z, w;
};
static inline f4 rand4(uint32_t pixel, uint32_t sample, uint32_t group, uint32_t seed) {
    u4 h = pcg4d(u4{pixel, sample, group, seed});
    return f4{u01(h.x), u01(h.y), u01(h.z), u01(h.w)};
}

/* ---------------------------------------------------------------- sincos
 * sin(2*pi*u), cos(2*pi*u) for finite u >= 0 (used with u in [0, 1)).
 * Reduction to the nearest quarter turn is exact (Sterbenz); the remainder
 * x in [-pi/4, pi/4] goes through the Taylor series of sin (to x^9) and cos
 * (to x^10) in Horner form.  Truncation error < 2e-9; rounding ~1 ulp. */
static inline void sincos2pi(float u, float *s_out, float *c_out) {
    const float k = std::floor(u * 4.0f + 0.5f);
    const float r = u - k * 0.25f;
    const int q = ((int)k) & 3;
    const float x = r * 6.28318548f;
    const float x2 = x * x;
    const float s = x * (1.0f + x2 * (-0.166666672f + x2 * (0.00833333377f + x2 * (-0.000198412701f + x2 * 2.75573188e-06f))));
    const float c = 1.0f + x2 * (-0.5f + x2 * (0.0416666679f + x2 * (-0.00138888892f + x2 * (2.48015876e-05f + x2 * -2.75573188e-07f))));
    float so, co;
    switch (q) {
    case 0: so = s; co = c; break;
    case 1: so = c; co = -s; break;
    case 2: so = -s; co = -c; break;
    default: so = -c; co = s; break;
    }
    *s_out = so;
    *c_out = co;
}

/* Orthonormal basis around a unit normal, Duff et al., "Building an
 * Orthonormal Basis, Revisited", JCGT 2017, as written in
 * src/util/sampling.h:21-33 (cr::sampling::build_local). */
struct onb {
    v3 n, t, b;
};
static inline onb build_local(v3 n) {
    const float s = (n.z < 0.0f) ? -1.0f : 1.0f;
    const float a = -1.0f / (s + n.z);
    const float b = n.x * n.y * a;
    onb o;
    o.n = n;
    o.t = v3{1.0f + s * n.x * n.x * a, s * b, -s * n.x};
    o.b = v3{b, s + n.y * n.y * a, -n.y};
    return o;
}

} // namespace orc
#endif
