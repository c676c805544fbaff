// render.cu — one-thread-per-pixel path-tracing megakernel (sm_103a).
//
// The drop-in for cr::renderer's sample passes (CRender
// src/render/renderer.cpp:116-144, 240-384): each thread owns one pixel,
// draws settings.spp samples in order and adds them to the pixel's FP32 sum
// (and optional FP64 sum / sum of squares) in that order, so the film is
// bit-identical to a sequential CPU accumulation of the same samples.
//
// FAITHFUL follows process_hit / _sample_pixel (renderer.cpp:21-102,
// 258-384): Lambert = normalize(Ng + uniform sphere point), mirror metal,
// Fresnel-less glass, emission folded into the throughput, optional sun NEE
// with the reference's colour-squared weight.  EXTENDED adds emissive-
// triangle NEE with power-heuristic MIS, GGX (VNDF sampling), Fresnel
// dielectric and Russian roulette; Lambert still scatters into the geometric
// normal's hemisphere as the reference does.
//
// Random dimension groups: 0 = pixel jitter, 1 + 2i = BSDF at segment i,
// 2 + 2i = light sample at segment i (pcg4d keyed by pixel/sample/group/seed).
#include <cmath>

#include "crg_dev.cuh"
#include "crg_internal.h"

namespace crg {

CamDev camera_params(const crg_camera &c) {
    CamDev p;
    for (int a = 0; a < 3; ++a) p.pos[a] = c.position[a];
    const double k = 3.14159265358979323846 / 180.0;
    const double ax = c.rotation[0] * k, ay = c.rotation[1] * k, az = c.rotation[2] * k;
    const double Ry[3][3] = {{std::cos(ax), 0, std::sin(ax)}, {0, 1, 0}, {-std::sin(ax), 0, std::cos(ax)}};
    const double Rx[3][3] = {{1, 0, 0}, {0, std::cos(ay), -std::sin(ay)}, {0, std::sin(ay), std::cos(ay)}};
    const double Rz[3][3] = {{std::cos(az), -std::sin(az), 0}, {std::sin(az), std::cos(az), 0}, {0, 0, 1}};
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T[i][j] = 0;
            for (int m = 0; m < 3; ++m) T[i][j] += Ry[i][m] * Rx[m][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double r = 0;
            for (int m = 0; m < 3; ++m) r += T[i][m] * Rz[m][j];
            p.R[3 * i + j] = (float)r;
        }
    p.w = (float)(1.0 / std::tan(0.5 * (double)c.fov * k));
    p.mode = c.mode;
    p.scale = c.scale;
    return p;
}

namespace {

struct SceneDev {
    const uint4 *nodes;
    const float4 *tris;
    const uint32_t *mat_idx;
    const crg_material *mats;
    const uint32_t *light_prim;
    const float *light_cdf;
    const float *light_pdf;
    const float *mat_light_pdf;
    const float4 *sky;
    const float *verts;
    uint32_t nlights, ntri;
    uint32_t sky_w, sky_h;
    float sky_rot_u, sky_rot_v;
    int sun_on;
    float sun_frame[9]; // t, n, b
    float sun_cos, sun_pdf;
    float sun_neg_dir[3];
    float sun_rad[3];
    uint32_t *err;
    unsigned long long *counters;
};

struct FilmDev {
    float *sum;
    double *sum64, *sumsq64;
    float *aov_albedo, *aov_normal, *aov_depth;
    uint32_t width, height;
};

struct Hit {
    float t, u, v;
    uint32_t prim, slot;
};

struct PathCtx;

template <int W, bool CNT>
__device__ __forceinline__ bool closest(const SceneDev &S, v3 o, v3 d, float tmax, Hit &h, PathCtx &C);
template <int W, bool CNT>
__device__ __forceinline__ bool occluded(const SceneDev &S, v3 o, v3 d, float tmax, PathCtx &C);

__device__ __forceinline__ void slot_verts(const SceneDev &S, uint32_t slot, v3 &a, v3 &b, v3 &c) {
    const float4 x = __ldg(&S.tris[slot * 3 + 0]);
    const float4 y = __ldg(&S.tris[slot * 3 + 1]);
    const float4 z = __ldg(&S.tris[slot * 3 + 2]);
    a = mk(x.x, x.y, x.z);
    b = mk(y.x, y.y, y.z);
    c = mk(z.x, z.y, z.z);
}

__device__ __forceinline__ void prim_verts(const SceneDev &S, uint32_t prim, v3 &a, v3 &b, v3 &c) {
    const float *v = S.verts + (size_t)prim * 9;
    a = mk(__ldg(v + 0), __ldg(v + 1), __ldg(v + 2));
    b = mk(__ldg(v + 3), __ldg(v + 4), __ldg(v + 5));
    c = mk(__ldg(v + 6), __ldg(v + 7), __ldg(v + 8));
}

// image::get_uv (src/objects/image.h:104-109)
__device__ __forceinline__ uint32_t texel_index(float u, uint32_t n) {
    const float f = u * (float)n;
    unsigned long long i = 0;
    if (f >= 0.0f) i = f < 4.6e18f ? (unsigned long long)f : 0ull;
    return (uint32_t)(i % n);
}

__device__ __forceinline__ v3 sample_sky(const SceneDev &S, v3 d) {
    if (S.sky_w == 0) return mk(0, 0, 0);
    const float dy = clampf(d.y, -1.0f, 1.0f);
    const float u = 0.5f + atan2f(d.z, d.x) * kInvTau;
    const float v = 0.5f - asinf(dy) * kInvPi;
    const uint32_t x = texel_index(u + S.sky_rot_u, S.sky_w);
    const uint32_t y = texel_index(v + S.sky_rot_v, S.sky_h);
    const float4 t = __ldg(&S.sky[x + (size_t)y * S.sky_w]);
    return mk(t.x, t.y, t.z);
}

__device__ __forceinline__ v3 sphere(float u1, float u2) {
    const float cos_t = 2.0f * u1 - 1.0f;
    const float sin_t = sqrtf(1.0f - cos_t * cos_t);
    float sp, cp;
    sincos2pi(u2, &sp, &cp);
    return mk(sin_t * cp, cos_t, sin_t * sp);
}

struct Aov {
    v3 albedo, normal;
    float depth;
};

struct PathCtx {
    uint32_t pix, sample, seed;
    uint32_t segments, shadow;
    uint32_t err;
    unsigned long long nodes, tris; // traversal work, counted only in the instrumented variant
};

template <int W, bool CNT>
__device__ __forceinline__ bool closest(const SceneDev &S, v3 o, v3 d, float tmax, Hit &h, PathCtx &C) {
    const RayPre r = ray_prep(o.x, o.y, o.z, d.x, d.y, d.z, 1e-5f);
    bool occ;
    TravStats st{0, 0};
    traverse<W, false, CNT>(S.nodes, S.tris, r, tmax, h.t, h.prim, h.slot, h.u, h.v, occ, st, C.err);
    if (CNT) {
        C.nodes += st.nodes;
        C.tris += st.tris;
    }
    return h.prim != 0xFFFFFFFFu;
}

template <int W, bool CNT>
__device__ __forceinline__ bool occluded(const SceneDev &S, v3 o, v3 d, float tmax, PathCtx &C) {
    const RayPre r = ray_prep(o.x, o.y, o.z, d.x, d.y, d.z, 1e-5f);
    float t, u, v;
    uint32_t p, sl;
    bool occ;
    TravStats st{0, 0};
    traverse<W, true, CNT>(S.nodes, S.tris, r, tmax, t, p, sl, u, v, occ, st, C.err);
    if (CNT) {
        C.nodes += st.nodes;
        C.tris += st.tris;
    }
    return occ;
}

// ------------------------------------------------------------------ faithful
template <int W, bool CNT>
__device__ v3 trace_faithful(const SceneDev &S, const crg_settings &set, PathCtx &C, v3 o, v3 d, Aov &aov) {
    v3 T = mk(1, 1, 1), L = mk(0, 0, 0);
    for (uint32_t i = 0; i < set.max_bounces; ++i) {
        Hit h;
        C.segments++;
        if (!closest<W, CNT>(S, o, d, INFINITY, h, C)) {
            const v3 env = sample_sky(S, d);
            if (i == 0) aov.albedo = env;
            L = add(L, mulv(T, env));
            break;
        }
        const v3 p = add(o, mul(d, h.t));
        v3 a, b, c;
        slot_verts(S, h.slot, a, b, c);
        const v3 Ng = normalize(cross(sub(b, a), sub(c, a)));
        const crg_material &m = S.mats[__ldg(&S.mat_idx[h.prim])];
        const float c0 = m.colour[0], c1 = m.colour[1], c2 = m.colour[2], c3 = m.colour[3];
        if (c3 == 0.0f) {
            o = add(p, mul(d, 0.1f));
            continue;
        }
        v3 albedo = mk(c0, c1, c2);
        const f4 g = rand4(C.pix, C.sample, 1 + 2 * i, C.seed);
        v3 no, nd;
        const uint32_t shade = m.shade_type;
        if (shade == CRG_SHADE_GLASS) {
            const v3 reflected = reflect(d, Ng);
            v3 out_n = Ng;
            float eta = 1.0f / m.ior;
            if (dot(d, Ng) > 0.0f) {
                out_n = neg(Ng);
                eta = m.ior;
            }
            const v3 uv = normalize(d);
            const float dt = dot(uv, out_n);
            const float disc = 1.0f - (eta * eta) * (1.0f - dt * dt);
            no = add(p, mul(out_n, -0.0001f));
            if (disc > 0.0f) nd = sub(mul(sub(uv, mul(out_n, dt)), eta), mul(out_n, sqrtf(disc)));
            else nd = reflected;
        } else if (shade == CRG_SHADE_METAL) {
            no = add(p, mul(Ng, 0.0001f));
            nd = reflect(d, Ng);
            albedo = mul(albedo, m.reflectiveness);
        } else {
            const v3 hc = add(Ng, sphere(g.x, g.y));
            const float l2 = dot(hc, hc);
            nd = l2 > 0.0f ? mul(hc, 1.0f / sqrtf(l2)) : Ng;
            no = add(p, mul(Ng, 0.0001f));
        }
        if (i == 0) {
            aov.albedo = albedo;
            aov.normal = Ng;
            aov.depth = h.t;
        }
        T = mulv(T, albedo);
        L = add(L, mul(T, m.emission));
        if (S.sun_on) {
            v3 so = add(p, mul(Ng, 0.001f));
            const f4 g2 = rand4(C.pix, C.sample, 2 + 2 * i, C.seed);
            float sp, cp;
            sincos2pi(g2.x, &sp, &cp);
            const float ct = 1.0f - g2.y * (1.0f - S.sun_cos);
            const float st = sqrtf(1.0f - ct * ct);
            const v3 lv = mk(cp * st, ct, sp * st);
            const float *F = S.sun_frame;
            const v3 sd = mk((F[0] * lv.x + F[3] * lv.y) + F[6] * lv.z, (F[1] * lv.x + F[4] * lv.y) + F[7] * lv.z,
                             (F[2] * lv.x + F[5] * lv.y) + F[8] * lv.z);
            const float cosine = clampf(dot(Ng, sd), 0.0f, 1.0f);
            Hit sh;
            C.shadow++;
            bool blocked = closest<W, CNT>(S, so, sd, INFINITY, sh, C);
            while (blocked) {
                if (S.mats[__ldg(&S.mat_idx[sh.prim])].colour[3] != 0.0f) break;
                so = add(add(so, mul(sd, sh.t)), mul(sd, 0.1f));
                C.shadow++;
                blocked = closest<W, CNT>(S, so, sd, INFINITY, sh, C);
            }
            if (!blocked) {
                const v3 ms = mk(S.sun_neg_dir[0], S.sun_neg_dir[1], S.sun_neg_dir[2]);
                v3 sky = mk(0, 0, 0);
                if (dot(sd, ms) > S.sun_cos) sky = mk(S.sun_rad[0], S.sun_rad[1], S.sun_rad[2]);
                const v3 tc = mulv(T, mk(c0, c1, c2));
                L = add(L, mk(((tc.x * cosine) * sky.x) / S.sun_pdf, ((tc.y * cosine) * sky.y) / S.sun_pdf,
                              ((tc.z * cosine) * sky.z) / S.sun_pdf));
            }
        }
        o = no;
        d = nd;
        if (set.rr_depth > 0 && i + 1 >= set.rr_depth) {
            const float q = mn(mx(mx(T.x, T.y), T.z), 0.95f);
            if (g.w >= q) break;
            T = mk(T.x / q, T.y / q, T.z / q);
        }
    }
    return L;
}

// ------------------------------------------------------------------ extended
__device__ __forceinline__ float ggx_D(float nh, float a) {
    const float a2 = a * a;
    const float dd = (nh * a2 - nh) * nh + 1.0f;
    return a2 / ((dd * dd) * kPi);
}
__device__ __forceinline__ float ggx_lambda(v3 w, float a) {
    const float s2 = w.x * w.x + w.y * w.y;
    const float z2 = w.z * w.z;
    return (sqrtf(1.0f + ((a * a) * s2) / z2) - 1.0f) * 0.5f;
}
__device__ __forceinline__ v3 schlick(v3 f0, float c) {
    const float m = 1.0f - clampf(c, 0.0f, 1.0f);
    const float m2 = m * m;
    const float m5 = (m2 * m2) * m;
    return mk(f0.x + (1.0f - f0.x) * m5, f0.y + (1.0f - f0.y) * m5, f0.z + (1.0f - f0.z) * m5);
}
__device__ __forceinline__ v3 sample_vndf(v3 ve, float a, float u1, float u2) {
    const v3 vh = normalize(mk(a * ve.x, a * ve.y, ve.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const v3 t1v = lensq > 0.0f ? mul(mk(-vh.y, vh.x, 0.0f), 1.0f / sqrtf(lensq)) : mk(1, 0, 0);
    const v3 t2v = cross(vh, t1v);
    const float r = sqrtf(u1);
    float sp, cp;
    sincos2pi(u2, &sp, &cp);
    const float t1 = r * cp;
    float t2 = r * sp;
    const float sw = 0.5f * (1.0f + vh.z);
    t2 = (1.0f - sw) * sqrtf(1.0f - t1 * t1) + sw * t2;
    const v3 nh = add(add(mul(t1v, t1), mul(t2v, t2)), mul(vh, sqrtf(mx(0.0f, (1.0f - t1 * t1) - t2 * t2))));
    return normalize(mk(a * nh.x, a * nh.y, mx(0.0f, nh.z)));
}
__device__ __forceinline__ float fresnel_dielectric(float ci, float eta, float &st2_out) {
    ci = clampf(ci, 0.0f, 1.0f);
    const float st2 = (eta * eta) * (1.0f - ci * ci);
    st2_out = st2;
    if (st2 >= 1.0f) return 1.0f;
    const float ct = sqrtf(1.0f - st2);
    const float rs = (eta * ci - ct) / (eta * ci + ct);
    const float rp = (ci - eta * ct) / (ci + eta * ct);
    return 0.5f * (rs * rs + rp * rp);
}
__device__ __forceinline__ v3 to_local(const onb &F, v3 w) { return mk(dot(w, F.t), dot(w, F.b), dot(w, F.n)); }
__device__ __forceinline__ v3 from_local(const onb &F, v3 l) { return add(add(mul(F.t, l.x), mul(F.b, l.y)), mul(F.n, l.z)); }

__device__ __forceinline__ uint32_t pick_light(const SceneDev &S, float u) {
    uint32_t lo = 0, hi = S.nlights - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (u < __ldg(&S.light_cdf[mid])) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

template <int W, bool CNT>
__device__ v3 nee(const SceneDev &S, PathCtx &C, uint32_t i, v3 p, v3 n, v3 T, int bsdf, v3 albedo, const onb &F, v3 wol,
                  float alpha) {
    const f4 g = rand4(C.pix, C.sample, 2 + 2 * i, C.seed);
    const uint32_t j = pick_light(S, g.x);
    const uint32_t prim = __ldg(&S.light_prim[j]);
    v3 a, b, c;
    prim_verts(S, prim, a, b, c);
    const float su = sqrtf(g.y);
    const float b0 = 1.0f - su, b1 = su * (1.0f - g.z), b2 = su * g.z;
    const v3 pl = add(add(mul(a, b0), mul(b, b1)), mul(c, b2));
    const v3 po = add(p, mul(n, 1e-4f));
    const v3 w = sub(pl, po);
    const float d2 = dot(w, w);
    if (!(d2 > 0.0f)) return mk(0, 0, 0);
    const float dist = sqrtf(d2);
    const v3 wi = mul(w, 1.0f / dist);
    const float cos_s = dot(wi, n);
    if (!(cos_s > 0.0f)) return mk(0, 0, 0);
    const v3 Ngl = normalize(cross(sub(b, a), sub(c, a)));
    const float cos_l = absf(dot(Ngl, wi));
    if (!(cos_l > 0.0f)) return mk(0, 0, 0);
    C.shadow++;
    if (occluded<W, CNT>(S, po, wi, dist * 0.999f, C)) return mk(0, 0, 0);
    const crg_material &lm = S.mats[__ldg(&S.mat_idx[prim])];
    const v3 Le = mk(lm.colour[0] * lm.emission, lm.colour[1] * lm.emission, lm.colour[2] * lm.emission);
    const float p_light = (__ldg(&S.light_pdf[j]) * d2) / cos_l;
    v3 f;
    float p_bsdf, cos_i;
    if (bsdf == 0) {
        f = mul(albedo, kInvPi);
        p_bsdf = cos_s * kInvPi;
        cos_i = cos_s;
    } else {
        const v3 wil = to_local(F, wi);
        if (!(wil.z > 0.0f)) return mk(0, 0, 0);
        const v3 hv = normalize(add(wol, wil));
        const float woh = dot(wol, hv);
        const float D = ggx_D(hv.z, alpha);
        const float lo_ = ggx_lambda(wol, alpha), li = ggx_lambda(wil, alpha);
        const float G2 = 1.0f / ((1.0f + lo_) + li);
        const float G1 = 1.0f / (1.0f + lo_);
        const v3 Fr = schlick(albedo, woh);
        f = mul(Fr, (D * G2) / ((4.0f * wol.z) * wil.z));
        p_bsdf = (G1 * D) / (4.0f * wol.z);
        cos_i = wil.z;
    }
    const float w_mis = (p_light * p_light) / (p_light * p_light + p_bsdf * p_bsdf);
    return mul(mulv(mulv(T, f), Le), (cos_i * w_mis) / p_light);
}

template <int W, bool CNT>
__device__ v3 trace_extended(const SceneDev &S, const crg_settings &set, PathCtx &C, v3 o, v3 d, Aov &aov) {
    v3 T = mk(1, 1, 1), L = mk(0, 0, 0);
    float prev_pdf = 0.0f;
    bool prev_delta = true;
    for (uint32_t i = 0; i < set.max_bounces; ++i) {
        Hit h;
        C.segments++;
        if (!closest<W, CNT>(S, o, d, INFINITY, h, C)) {
            const v3 env = sample_sky(S, d);
            if (i == 0) aov.albedo = env;
            L = add(L, mulv(T, env));
            break;
        }
        const v3 p = add(o, mul(d, h.t));
        v3 a, b, c;
        slot_verts(S, h.slot, a, b, c);
        const v3 Ng = normalize(cross(sub(b, a), sub(c, a)));
        const uint32_t mi = __ldg(&S.mat_idx[h.prim]);
        const crg_material &m = S.mats[mi];
        const float c0 = m.colour[0], c1 = m.colour[1], c2 = m.colour[2], c3 = m.colour[3];
        if (c3 == 0.0f) {
            o = add(p, mul(d, 0.1f));
            continue;
        }
        const v3 rgb = mk(c0, c1, c2);
        const float cos_nd = dot(Ng, d);
        const v3 n = cos_nd < 0.0f ? Ng : neg(Ng);
        if (i == 0) {
            aov.albedo = rgb;
            aov.normal = Ng;
            aov.depth = h.t;
        }
        const float emission = m.emission;
        if (emission > 0.0f) {
            const v3 Le = mk(c0 * emission, c1 * emission, c2 * emission);
            if (prev_delta) {
                L = add(L, mulv(T, Le));
            } else {
                const float cos_l = absf(cos_nd);
                if (cos_l > 0.0f) {
                    const float pl = (__ldg(&S.mat_light_pdf[mi]) * (h.t * h.t)) / cos_l;
                    const float w = (prev_pdf * prev_pdf) / (prev_pdf * prev_pdf + pl * pl);
                    L = add(L, mul(mulv(T, Le), w));
                }
            }
        }
        const f4 g = rand4(C.pix, C.sample, 1 + 2 * i, C.seed);
        const v3 wo = neg(d);
        const bool have_lights = S.nlights > 0 && i + 1 < set.max_bounces;
        const uint32_t shade = m.shade_type;
        if (shade == CRG_SHADE_SMOOTH) {
            const onb F = build_local(Ng);
            if (have_lights) L = add(L, nee<W, CNT>(S, C, i, p, Ng, T, 0, rgb, F, mk(0, 0, 0), 0.0f));
            float sp, cp;
            sincos2pi(g.y, &sp, &cp);
            const float r = sqrtf(g.x);
            const v3 l = mk(r * cp, r * sp, sqrtf(mx(0.0f, 1.0f - g.x)));
            d = from_local(F, l);
            o = add(p, mul(Ng, 1e-4f));
            prev_pdf = l.z * kInvPi;
            prev_delta = false;
            T = mulv(T, rgb);
        } else if (shade == CRG_SHADE_METAL) {
            const v3 f0 = mul(rgb, m.reflectiveness);
            const float alpha = m.roughness;
            if (alpha < 1e-4f) {
                d = reflect(d, n);
                o = add(p, mul(n, 1e-4f));
                T = mulv(T, f0);
                prev_delta = true;
            } else {
                const onb F = build_local(n);
                const v3 wol = to_local(F, wo);
                if (!(wol.z > 0.0f)) break;
                if (have_lights) L = add(L, nee<W, CNT>(S, C, i, p, n, T, 1, f0, F, wol, alpha));
                const v3 hh = sample_vndf(wol, alpha, g.x, g.y);
                const float woh = dot(wol, hh);
                const float k2 = 2.0f * woh;
                const v3 wil = mk(hh.x * k2 - wol.x, hh.y * k2 - wol.y, hh.z * k2 - wol.z);
                if (!(wil.z > 0.0f)) break;
                const float lo_ = ggx_lambda(wol, alpha), li = ggx_lambda(wil, alpha);
                const float G1 = 1.0f / (1.0f + lo_);
                const float G2 = 1.0f / ((1.0f + lo_) + li);
                const v3 Fr = schlick(f0, woh);
                T = mulv(T, mul(Fr, G2 / G1));
                prev_pdf = (G1 * ggx_D(hh.z, alpha)) / (4.0f * wol.z);
                prev_delta = false;
                d = from_local(F, wil);
                o = add(p, mul(n, 1e-4f));
            }
        } else {
            const float eta = cos_nd < 0.0f ? 1.0f / m.ior : m.ior;
            const float ci = -dot(d, n);
            float st2;
            const float Fr = fresnel_dielectric(ci, eta, st2);
            if (g.z < Fr) {
                d = reflect(d, n);
                o = add(p, mul(n, 1e-4f));
            } else {
                const float cic = clampf(ci, 0.0f, 1.0f);
                const float ct = sqrtf(1.0f - st2);
                d = add(mul(d, eta), mul(n, eta * cic - ct));
                o = add(p, mul(n, -1e-4f));
            }
            T = mulv(T, rgb);
            prev_delta = true;
        }
        if (set.rr_depth > 0 && i + 1 >= set.rr_depth) {
            const float q = mn(mx(mx(T.x, T.y), T.z), 0.95f);
            if (g.w >= q) break;
            T = mk(T.x / q, T.y / q, T.z / q);
        }
    }
    return L;
}

// camera::get_ray (camera.cpp:14-39)
__device__ __forceinline__ void camera_ray(const CamDev &c, float x, float y, float aspect, v3 &o, v3 &d) {
    if (c.mode == CRG_CAMERA_ORTHOGRAPHIC) {
        const float u = 2.0f * x - 1.0f;
        const float v = 2.0f * y - 1.0f;
        const float su = c.scale * u, sv = c.scale * v;
        o = mk(((c.R[0] * su + c.R[1] * sv) + c.R[2] * 0.0f) + c.pos[0], ((c.R[3] * su + c.R[4] * sv) + c.R[5] * 0.0f) + c.pos[1],
               ((c.R[6] * su + c.R[7] * sv) + c.R[8] * 0.0f) + c.pos[2]);
        d = normalize(mk(c.R[2], c.R[5], c.R[8]));
        return;
    }
    const float u = (2.0f * x - 1.0f) * aspect;
    const float v = 2.0f * y - 1.0f;
    o = mk(c.pos[0], c.pos[1], c.pos[2]);
    d = normalize(mk((c.R[0] * u + c.R[1] * v) + c.R[2] * c.w, (c.R[3] * u + c.R[4] * v) + c.R[5] * c.w,
                     (c.R[6] * u + c.R[7] * v) + c.R[8] * c.w));
}

template <int W, int MODE, bool CNT>
__global__ void __launch_bounds__(128) k_render(SceneDev S, CamDev cam, crg_settings set, FilmDev F, uint64_t spp0) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t Wd = set.width, Hd = set.height;
    PathCtx C{pix, 0, set.seed, 0, 0, 0, 0ull, 0ull};
    if (pix < Wd * Hd) {
        const uint32_t px = pix % Wd, py = pix / Wd;
        const size_t fidx = (size_t)(Wd - 1 - px) + (size_t)(Hd - 1 - py) * Wd;
        float acc[3] = {F.sum[fidx * 3], F.sum[fidx * 3 + 1], F.sum[fidx * 3 + 2]};
        double a64[3] = {0, 0, 0}, q64[3] = {0, 0, 0};
        if (F.sum64) {
            a64[0] = F.sum64[fidx * 3]; a64[1] = F.sum64[fidx * 3 + 1]; a64[2] = F.sum64[fidx * 3 + 2];
            q64[0] = F.sumsq64[fidx * 3]; q64[1] = F.sumsq64[fidx * 3 + 1]; q64[2] = F.sumsq64[fidx * 3 + 2];
        }
        Aov aov;
        for (uint32_t s = 0; s < set.spp; ++s) {
            C.sample = (uint32_t)(spp0 + s);
            const f4 g0 = rand4(pix, C.sample, 0, set.seed);
            const float x = ((float)px + g0.x) / (float)Wd;
            const float y = ((float)py + g0.y) / (float)Hd;
            v3 o, d;
            camera_ray(cam, x, y, set.aspect, o, d);
            aov.albedo = mk(0, 0, 0);
            aov.normal = mk(0, 0, 0);
            aov.depth = 0.0f;
            const v3 L = MODE == CRG_MODE_EXTENDED ? trace_extended<W, CNT>(S, set, C, o, d, aov) : trace_faithful<W, CNT>(S, set, C, o, d, aov);
            acc[0] += L.x;
            acc[1] += L.y;
            acc[2] += L.z;
            if (F.sum64) {
                a64[0] += (double)L.x; a64[1] += (double)L.y; a64[2] += (double)L.z;
                q64[0] += (double)L.x * (double)L.x;
                q64[1] += (double)L.y * (double)L.y;
                q64[2] += (double)L.z * (double)L.z;
            }
        }
        F.sum[fidx * 3] = acc[0];
        F.sum[fidx * 3 + 1] = acc[1];
        F.sum[fidx * 3 + 2] = acc[2];
        if (F.sum64) {
            F.sum64[fidx * 3] = a64[0]; F.sum64[fidx * 3 + 1] = a64[1]; F.sum64[fidx * 3 + 2] = a64[2];
            F.sumsq64[fidx * 3] = q64[0]; F.sumsq64[fidx * 3 + 1] = q64[1]; F.sumsq64[fidx * 3 + 2] = q64[2];
        }
        if (F.aov_albedo && set.spp > 0) {
            reinterpret_cast<float4 *>(F.aov_albedo)[fidx] = make_float4(aov.albedo.x, aov.albedo.y, aov.albedo.z, 1.0f);
            reinterpret_cast<float4 *>(F.aov_normal)[fidx] =
                make_float4(aov.normal.x * 0.5f + 0.5f, aov.normal.y * 0.5f + 0.5f, aov.normal.z * 0.5f + 0.5f, 1.0f);
            const float dv = mn(aov.depth, 200.0f) / 200.0f;
            reinterpret_cast<float4 *>(F.aov_depth)[fidx] = make_float4(dv, dv, dv, 1.0f);
        }
    }
    if (C.err) atomicOr(S.err, C.err);
    if (CNT) {
        unsigned long long seg = C.segments, sh = C.shadow, nd = C.nodes, tr = C.tris;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            seg += __shfl_xor_sync(0xFFFFFFFFu, seg, off);
            sh += __shfl_xor_sync(0xFFFFFFFFu, sh, off);
            nd += __shfl_xor_sync(0xFFFFFFFFu, nd, off);
            tr += __shfl_xor_sync(0xFFFFFFFFu, tr, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&S.counters[1], seg);
            atomicAdd(&S.counters[2], sh);
            atomicAdd(&S.counters[3], nd);
            atomicAdd(&S.counters[4], tr);
        }
    }
}

template <int W>
void launch_w(const SceneDev &S, const CamDev &cam, const crg_settings &set, const FilmDev &F, uint64_t spp0,
              cudaStream_t st) {
    const uint32_t T = 128;
    const uint64_t npix = (uint64_t)set.width * set.height;
    const uint32_t blocks = (uint32_t)((npix + T - 1) / T);
    if (S.counters) {
        if (set.mode == CRG_MODE_EXTENDED) k_render<W, CRG_MODE_EXTENDED, true><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
        else k_render<W, CRG_MODE_FAITHFUL, true><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
    } else {
        if (set.mode == CRG_MODE_EXTENDED) k_render<W, CRG_MODE_EXTENDED, false><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
        else k_render<W, CRG_MODE_FAITHFUL, false><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
    }
}

} // namespace

crg_status launch_render(crg_scene *s, const CamDev &cam, const crg_settings &set, crg_film *film, cudaStream_t st) {
    SceneDev S{};
    S.nodes = (const uint4 *)s->wide.ptr;
    S.tris = (const float4 *)s->tris.ptr;
    S.mat_idx = (const uint32_t *)s->mat_idx.ptr;
    S.mats = (const crg_material *)s->mats.ptr;
    S.light_prim = (const uint32_t *)s->light_prim.ptr;
    S.light_cdf = (const float *)s->light_cdf.ptr;
    S.light_pdf = (const float *)s->light_pdf.ptr;
    S.mat_light_pdf = (const float *)s->mat_light_pdf.ptr;
    S.verts = (const float *)s->verts.ptr;
    S.nlights = s->nlights;
    S.ntri = s->ntri;
    S.sky = (const float4 *)s->sky.ptr;
    S.sky_w = s->sky.ptr ? s->sky_w : 0;
    S.sky_h = s->sky_h;
    S.sky_rot_u = s->sky_rot_u;
    S.sky_rot_v = s->sky_rot_v;
    S.sun_on = s->sun_enabled;
    for (int k = 0; k < 9; ++k) S.sun_frame[k] = s->sun_frame[k];
    S.sun_cos = s->sun_cos;
    S.sun_pdf = s->sun_pdf;
    for (int k = 0; k < 3; ++k) {
        S.sun_neg_dir[k] = -s->sun.direction[k];
        S.sun_rad[k] = s->sun.colour[k] * s->sun.intensity;
    }
    S.err = (uint32_t *)s->err.ptr;
    S.counters = s->counting ? (unsigned long long *)s->counters.ptr : nullptr;
    FilmDev F{(float *)film->sum.ptr,
              (double *)film->sum64.ptr,
              (double *)film->sumsq64.ptr,
              (float *)film->aov_albedo.ptr,
              (float *)film->aov_normal.ptr,
              (float *)film->aov_depth.ptr,
              film->width,
              film->height};
    if (s->ntri == 0) return set_error(s->ctx, CRG_ERR_INVALID_ARG, "crg_render: scene has no triangles");
    switch (s->width) {
    case 2: launch_w<2>(S, cam, set, F, film->spp, st); break;
    case 4: launch_w<4>(S, cam, set, F, film->spp, st); break;
    default: launch_w<8>(S, cam, set, F, film->spp, st); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(s->ctx, e, "k_render launch");
    return CRG_OK;
}

} // namespace crg
