// render_common.cuh — per-bounce path shading shared by the megakernel
// (render.cu) and the wavefront form (wavefront.cu), so both evaluate the
// same operations in the same order and produce bit-identical images.
//
// FAITHFUL follows process_hit / _sample_pixel (CRender
// src/render/renderer.cpp:21-102, 258-384); EXTENDED adds emissive-triangle
// NEE with power-heuristic MIS, GGX (VNDF sampling, Heitz 2018), a Fresnel
// dielectric and Russian roulette.  Random dimension groups: 0 = pixel
// jitter, 1 + 2i = BSDF at segment i, 2 + 2i = light sample at segment i.
#pragma once
#include <cmath>

#include "crg_dev.cuh"
#include "crg_internal.h"

namespace crg {
namespace rc {

struct SceneDev {
    const uint4 *nodes;
    const float4 *tris;
    const uint32_t *mat_idx;
    const crg_material *mats;
    const uint32_t *light_prim;
    const float2 *light_alias; // per emitter entry {prob, alias bits}
    const float *light_pdf;
    const float *mat_light_pdf;
    const float4 *sky;
    const float *verts;
    const float *uvs;       // float[ntri*6] per-corner texture coordinates, or null
    const float4 *texels;   // all textures' texels, concatenated
    const uint4 *tex_info;  // per texture: first texel (lo, hi), width, height
    uint32_t ntex;
    // instances (cr::entity::instances::transforms, model.cpp:99-126): per
    // instance 6 float4 rows: the inverse (3 rows of [A | t]) then the forward
    // transform; ninst = 0 means the mesh is used as is
    const float4 *inst;
    const uint32_t *inst_root;  // per placement: node index of its model's BVH root
    const float4 *tlas;         // top-level tree over the placements (4 float4 per node)
    uint32_t tlas_root;         // its root: a node index, or kTlasLeaf | placement
    const uint32_t *light_inst; // instance of each emitter entry (instanced scenes)
    // per emitter entry 4 float4: (v0, pdf), (v1, prim bits), (v2, material bits), (colour * emission,
    // textured flag bits); v0..v2 in world space
    const float4 *light_rec;
    uint32_t ninst;
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

// Device view of a built scene (defined in render.cu).
SceneDev scene_dev(const crg_scene *s);

struct FilmDev {
    float *sum;
    double *sum64, *sumsq64;
    float *aov_albedo, *aov_normal, *aov_depth;
    uint32_t width, height;
};

// Closest hit.  For an instanced scene t is the parameter along the
// instance's object-space ray (hit_geom turns it into the world point and
// distance) and inst the instance; otherwise inst = kNoInst and t is the
// world distance.
constexpr uint32_t kNoInst = 0xFFFFFFFFu;
struct Hit {
    float t, u, v;
    uint32_t prim, slot, inst;
};

struct PathCtx;

template <int W, bool CNT, bool INST>
__device__ __forceinline__ bool closest(const SceneDev &S, v3 o, v3 d, float tmax, Hit &h, PathCtx &C);
template <int W, bool CNT, bool INST>
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

// ------------------------------------------------------------------ textures
// process_hit takes the colour from the material's texture at the hit's
// interpolated texture coordinate when it has one (renderer.cpp:30-35,
// image::get_uv at image.h:104-109), else the material colour.
__device__ __forceinline__ bool textured(const SceneDev &S, const crg_material &m) {
    return m.tex >= 0 && (uint32_t)m.tex < S.ntex;
}

__device__ __forceinline__ float4 tex_lookup(const SceneDev &S, int32_t tex, float u, float v) {
    const uint4 ti = __ldg(&S.tex_info[tex]);
    const uint32_t x = texel_index(u, ti.z), y = texel_index(v, ti.w);
    const size_t base = ((size_t)ti.y << 32) | ti.x;
    return __ldg(&S.texels[base + x + (size_t)y * ti.z]);
}

// Barycentric interpolation of the per-corner coordinates (rtcInterpolate0 of
// the vertex attribute buffer, src/objects/model.cpp:39-47); (0, 0) without
// coordinates.
__device__ __forceinline__ void interp_uv(const SceneDev &S, uint32_t prim, float b1, float b2, float &u, float &v) {
    if (!S.uvs) {
        u = v = 0.0f;
        return;
    }
    const float *t = S.uvs + (size_t)prim * 6;
    const float b0 = (1.0f - b1) - b2;
    u = (b0 * __ldg(t + 0) + b1 * __ldg(t + 2)) + b2 * __ldg(t + 4);
    v = (b0 * __ldg(t + 1) + b1 * __ldg(t + 3)) + b2 * __ldg(t + 5);
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

// ------------------------------------------------------------------ instances
// Row-form affine transforms: x' = ((r.x * x + r.y * y) + r.z * z) + r.w.
__device__ __forceinline__ v3 xf_point(const float4 *R, v3 p) {
    const float4 a = __ldg(&R[0]), b = __ldg(&R[1]), c = __ldg(&R[2]);
    return mk(((a.x * p.x + a.y * p.y) + a.z * p.z) + a.w, ((b.x * p.x + b.y * p.y) + b.z * p.z) + b.w,
              ((c.x * p.x + c.y * p.y) + c.z * p.z) + c.w);
}
__device__ __forceinline__ v3 xf_vector(const float4 *R, v3 v) {
    const float4 a = __ldg(&R[0]), b = __ldg(&R[1]), c = __ldg(&R[2]);
    return mk((a.x * v.x + a.y * v.y) + a.z * v.z, (b.x * v.x + b.y * v.y) + b.z * v.z, (c.x * v.x + c.y * v.y) + c.z * v.z);
}

// model::intersect's object-space ray of instance j: inverse(T) * (o, 1) and
// normalize(inverse(T) * (d, 0)); len = |inverse(T) * d|.
__device__ __forceinline__ void inst_ray(const SceneDev &S, uint32_t j, v3 o, v3 d, v3 &oo, v3 &od, float &len) {
    const float4 *R = S.inst + 6 * (size_t)j;
    oo = xf_point(R, o);
    const v3 dr = xf_vector(R, d);
    len = sqrtf(dot(dr, dr));
    od = normalize(dr);
}

// World point T * (oo + od * t) of an object-space hit and its distance from
// the world origin o (model.cpp:117-121).
__device__ __forceinline__ v3 inst_point(const SceneDev &S, uint32_t j, v3 oo, v3 od, float t) {
    return xf_point(S.inst + 6 * (size_t)j + 3, add(oo, mul(od, t)));
}
__device__ __forceinline__ float vdist(v3 a, v3 b) {
    const v3 e = sub(a, b);
    return sqrtf(dot(e, e));
}

// Slack of the object-space bound that prunes an instance's traversal by the
// best world distance so far: the bound stays above the parameter at which
// the world distance reaches the best one, so pruning never changes the result
// of the reference's loop over instances.
constexpr float kInstSlack = 1.0001f;

// ------------------------------------------------------------------ top level
// Placements are the (model, instance) pairs of a scene in the order
// cr::scene::cast_ray and cr::model::intersect visit them (scene.cpp:79-98,
// model.cpp:99-126).  A binary tree over their world boxes (built on the
// host, 4 float4 per node: {lo_a, ref_a}, {hi_a, ref_b}, {lo_b, -}, {hi_b, -})
// orders and prunes them; the result is the reference loop's: the smallest
// world distance, ties to the earlier placement.  A subtree is skipped only
// when its box entry lies beyond the best distance by more than a generous
// margin (1e-3 relative plus 1e-3 of the origin's magnitude), far above the
// rounding of the world points, so pruning never changes the answer.
constexpr int kTlasStack = 48;

struct TlasRay {
    v3 o, inv;
    float dl;     // |d|
    float margin; // world-space widening of every box: 1e-4 of the origin's magnitude
    float slack;  // absolute slack of the pruning test: 1e-3 of the origin's magnitude (at least 1e-3)
    bool ahead;   // tmin >= 0: boxes wholly behind the origin cannot hold a hit
};
__device__ __forceinline__ TlasRay tlas_ray(v3 o, v3 d, float tmin) {
    TlasRay t;
    t.o = o;
    const float tiny = 8.27180613e-25f; // 2^-80
    t.inv = mk(1.0f / (fabsf(d.x) < tiny ? copysignf(tiny, d.x) : d.x), 1.0f / (fabsf(d.y) < tiny ? copysignf(tiny, d.y) : d.y),
               1.0f / (fabsf(d.z) < tiny ? copysignf(tiny, d.z) : d.z));
    t.dl = sqrtf(dot(d, d));
    const float om = fmaxf(fmaxf(fabsf(o.x), fabsf(o.y)), fabsf(o.z));
    t.margin = 1e-4f * om;
    t.slack = 1e-3f * (om + 1.0f);
    t.ahead = tmin >= 0.0f;
    return t;
}
// Entry parameter of the ray into a box widened by the margin, or +inf when it
// misses it (or, for tmin >= 0, when the box lies wholly behind the origin).
__device__ __forceinline__ float tlas_entry(const TlasRay &t, float4 lo, float4 hi) {
    const float m = t.margin;
    const float x0 = ((lo.x - m) - t.o.x) * t.inv.x, x1 = ((hi.x + m) - t.o.x) * t.inv.x;
    const float y0 = ((lo.y - m) - t.o.y) * t.inv.y, y1 = ((hi.y + m) - t.o.y) * t.inv.y;
    const float z0 = ((lo.z - m) - t.o.z) * t.inv.z, z1 = ((hi.z + m) - t.o.z) * t.inv.z;
    const float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fminf(z0, z1));
    const float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fmaxf(z0, z1));
    if (!(tn <= tf) || (t.ahead && tf < 0.0f)) return INFINITY;
    return tn;
}
// True while a subtree entered at parameter `entry` may still hold a hit whose
// world distance is at most `best`.
__device__ __forceinline__ bool tlas_keep(const TlasRay &t, float entry, float best) {
    return entry * t.dl <= best * 1.001f + t.slack;
}

// Visits the placements whose boxes the ray may reach, nearest box first;
// visit(k) returns the current bound (best world distance) after placement k,
// or a negative value to stop.  Returns false if the stack overflowed.
template <class Visit>
__device__ __forceinline__ bool tlas_walk(const SceneDev &S, const TlasRay &t, float bound, Visit &&visit) {
    uint32_t ref = S.tlas_root;
    uint32_t stack[kTlasStack];
    float sent[kTlasStack];
    int sp = 0;
    bool ok = true;
    for (;;) {
        if (ref & kTlasLeaf) {
            bound = visit(ref & ~kTlasLeaf);
            if (bound < 0.0f) return ok;
        } else {
            const float4 *n = S.tlas + 4 * (size_t)ref;
            const float4 la = __ldg(&n[0]), ha = __ldg(&n[1]), lb = __ldg(&n[2]), hb = __ldg(&n[3]);
            const float ea = tlas_entry(t, la, ha), eb = tlas_entry(t, lb, hb);
            const bool ka = ea < INFINITY && tlas_keep(t, ea, bound), kb = eb < INFINITY && tlas_keep(t, eb, bound);
            const uint32_t ra = __float_as_uint(la.w), rb = __float_as_uint(ha.w);
            if (ka && kb) {
                const bool a_first = ea <= eb;
                if (sp < kTlasStack) {
                    stack[sp] = a_first ? rb : ra;
                    sent[sp] = a_first ? eb : ea;
                    sp++;
                } else {
                    ok = false;
                }
                ref = a_first ? ra : rb;
                continue;
            }
            if (ka || kb) {
                ref = ka ? ra : rb;
                continue;
            }
        }
        // pop the next subtree that may still hold a closer hit
        bool found = false;
        while (sp > 0) {
            --sp;
            if (tlas_keep(t, sent[sp], bound)) {
                ref = stack[sp];
                found = true;
                break;
            }
        }
        if (!found) return ok;
    }
}

// The same walk, resumable: tlas_next returns the next placement whose box the
// ray may reach under `bound` (the best world distance so far), or kNoInst
// when the walk is over; the caller traces the placement between calls.
// Placements come in tlas_walk's order and with its pruning.
struct TlasWalk {
    uint32_t stack[kTlasStack];
    float sent[kTlasStack];
    uint32_t ref;
    int sp;
    bool pop; // the last placement returned: continue with the stack
    bool ok;  // false: the stack overflowed
};
__device__ __forceinline__ void tlas_begin(const SceneDev &S, TlasWalk &wk) {
    wk.ref = S.tlas_root;
    wk.sp = 0;
    wk.pop = false;
    wk.ok = true;
}
__device__ __forceinline__ uint32_t tlas_next(const SceneDev &S, const TlasRay &t, float bound, TlasWalk &wk) {
    for (;;) {
        if (!wk.pop) {
            const uint32_t ref = wk.ref;
            if (ref & kTlasLeaf) {
                wk.pop = true;
                return ref & ~kTlasLeaf;
            }
            const float4 *n = S.tlas + 4 * (size_t)ref;
            const float4 la = __ldg(&n[0]), ha = __ldg(&n[1]), lb = __ldg(&n[2]), hb = __ldg(&n[3]);
            const float ea = tlas_entry(t, la, ha), eb = tlas_entry(t, lb, hb);
            const bool ka = ea < INFINITY && tlas_keep(t, ea, bound), kb = eb < INFINITY && tlas_keep(t, eb, bound);
            const uint32_t ra = __float_as_uint(la.w), rb = __float_as_uint(ha.w);
            if (ka && kb) {
                const bool a_first = ea <= eb;
                if (wk.sp < kTlasStack) {
                    wk.stack[wk.sp] = a_first ? rb : ra;
                    wk.sent[wk.sp] = a_first ? eb : ea;
                    wk.sp++;
                } else {
                    wk.ok = false;
                }
                wk.ref = a_first ? ra : rb;
                continue;
            }
            if (ka || kb) {
                wk.ref = ka ? ra : rb;
                continue;
            }
        }
        // pop the next subtree that may still hold a closer hit
        wk.pop = false;
        bool found = false;
        while (wk.sp > 0) {
            --wk.sp;
            if (tlas_keep(t, wk.sent[wk.sp], bound)) {
                wk.ref = wk.stack[wk.sp];
                found = true;
                break;
            }
        }
        if (!found) return kNoInst;
    }
}

// Closest hit over the placements (the reference's loops over models and
// instances): h.t is the object-space parameter, h.inst the placement.
template <int W, bool CNT>
__device__ __forceinline__ void closest_placements(const SceneDev &S, v3 o, v3 d, float tmin, float tmax, Hit &h,
                                                TravStats &st, uint32_t &err) {
    const TlasRay tr = tlas_ray(o, d, tmin);
    float best = tmax;
    h.prim = 0xFFFFFFFFu;
    h.inst = kNoInst;
    const bool ok = tlas_walk(S, tr, tmax, [&](uint32_t k) {
        v3 oo, od;
        float len;
        inst_ray(S, k, o, d, oo, od, len);
        const float bound = best < INFINITY ? ((best * len) / tr.dl) * kInstSlack : INFINITY;
        const RayPre r = ray_prep(oo.x, oo.y, oo.z, od.x, od.y, od.z, tmin);
        Hit hk;
        bool occ;
        traverse<W, false, CNT>(S.nodes, S.tris, r, bound, hk.t, hk.prim, hk.slot, hk.u, hk.v, occ, st, err,
                                __ldg(&S.inst_root[k]));
        if (hk.prim != 0xFFFFFFFFu) {
            const float dist = vdist(inst_point(S, k, oo, od, hk.t), o);
            if (dist < best || (dist == best && h.inst != kNoInst && k < h.inst)) {
                best = dist;
                h = hk;
                h.inst = k;
            }
        }
        return best;
    });
    if (!ok) err = 1u;
}

// Any hit over the placements: a placement's hit counts when its object-space
// parameter is below tmax |inverse(T) d| / |d| (world distance below tmax).
template <int W, bool CNT>
__device__ __forceinline__ bool occluded_placements(const SceneDev &S, v3 o, v3 d, float tmin, float tmax, TravStats &st,
                                                 uint32_t &err) {
    const TlasRay tr = tlas_ray(o, d, tmin);
    bool occ = false;
    const bool ok = tlas_walk(S, tr, tmax, [&](uint32_t k) {
        v3 oo, od;
        float len;
        inst_ray(S, k, o, d, oo, od, len);
        const RayPre r = ray_prep(oo.x, oo.y, oo.z, od.x, od.y, od.z, tmin);
        float t, u, v;
        uint32_t p, sl;
        traverse<W, true, CNT>(S.nodes, S.tris, r, (tmax * len) / tr.dl, t, p, sl, u, v, occ, st, err,
                               __ldg(&S.inst_root[k]));
        return occ ? -1.0f : tmax;
    });
    if (!ok) err = 1u;
    return occ;
}

// Scenes with at most this many placements are traced by a plain loop over
// them in order (the reference's loops as written, each traversal pruned by
// the best world distance); larger ones through the top-level tree.
constexpr uint32_t kLoopPlacements = 4;

// Closest hit over a few placements, one after the other.
template <int W, bool CNT>
__device__ __forceinline__ void closest_placement_loop(const SceneDev &S, v3 o, v3 d, float tmin, float tmax, Hit &h,
                                                       TravStats &st, uint32_t &err) {
    bool occ;
    const float dl = sqrtf(dot(d, d));
    float best = tmax;
    h.prim = 0xFFFFFFFFu;
    h.inst = kNoInst;
    for (uint32_t j = 0; j < S.ninst; ++j) {
        v3 oo, od;
        float len;
        inst_ray(S, j, o, d, oo, od, len);
        const float bound = best < INFINITY ? ((best * len) / dl) * kInstSlack : INFINITY;
        const RayPre r = ray_prep(oo.x, oo.y, oo.z, od.x, od.y, od.z, tmin);
        Hit hj;
        traverse<W, false, CNT>(S.nodes, S.tris, r, bound, hj.t, hj.prim, hj.slot, hj.u, hj.v, occ, st, err,
                                __ldg(&S.inst_root[j]));
        if (hj.prim == 0xFFFFFFFFu) continue;
        const float dist = vdist(inst_point(S, j, oo, od, hj.t), o);
        if (dist < best) {
            best = dist;
            h = hj;
            h.inst = j;
        }
    }
}

// Any hit over a few placements, one after the other.
template <int W, bool CNT>
__device__ __forceinline__ bool occluded_placement_loop(const SceneDev &S, v3 o, v3 d, float tmin, float tmax,
                                                        TravStats &st, uint32_t &err) {
    float t, u, v;
    uint32_t p, sl;
    bool occ = false;
    const float dl = sqrtf(dot(d, d));
    for (uint32_t j = 0; j < S.ninst && !occ; ++j) {
        v3 oo, od;
        float len;
        inst_ray(S, j, o, d, oo, od, len);
        const RayPre r = ray_prep(oo.x, oo.y, oo.z, od.x, od.y, od.z, tmin);
        traverse<W, true, CNT>(S.nodes, S.tris, r, (tmax * len) / dl, t, p, sl, u, v, occ, st, err,
                               __ldg(&S.inst_root[j]));
    }
    return occ;
}

// Closest hit with tmin < t (object space for instances, as the reference's
// tnear) and world distance below tmax.  INST = false compiles the one-mesh
// path and the loop over a few placements; INST = true the top-level tree.
template <int W, bool CNT, bool INST>
__device__ __forceinline__ bool closest_t(const SceneDev &S, v3 o, v3 d, float tmin, float tmax, Hit &h, PathCtx &C) {
    bool occ;
    TravStats st{0, 0};
    if (S.ninst == 0) {
        const RayPre r = ray_prep(o.x, o.y, o.z, d.x, d.y, d.z, tmin);
        traverse<W, false, CNT>(S.nodes, S.tris, r, tmax, h.t, h.prim, h.slot, h.u, h.v, occ, st, C.err);
        h.inst = kNoInst;
    } else if (INST) {
        closest_placements<W, CNT>(S, o, d, tmin, tmax, h, st, C.err);
    } else {
        closest_placement_loop<W, CNT>(S, o, d, tmin, tmax, h, st, C.err);
    }
    if (CNT) {
        C.nodes += st.nodes;
        C.tris += st.tris;
    }
    return h.prim != 0xFFFFFFFFu;
}

template <int W, bool CNT, bool INST>
__device__ __forceinline__ bool closest(const SceneDev &S, v3 o, v3 d, float tmax, Hit &h, PathCtx &C) {
    return closest_t<W, CNT, INST>(S, o, d, 1e-5f, tmax, h, C);
}

// Any hit with tmin < t < tmax.  Instanced: any placement with a hit whose
// object-space parameter is below tmax * |inverse(T) d| / |d|.
template <int W, bool CNT, bool INST>
__device__ __forceinline__ bool occluded_t(const SceneDev &S, v3 o, v3 d, float tmin, float tmax, PathCtx &C) {
    float t, u, v;
    uint32_t p, sl;
    bool occ = false;
    TravStats st{0, 0};
    if (S.ninst == 0) {
        const RayPre r = ray_prep(o.x, o.y, o.z, d.x, d.y, d.z, tmin);
        traverse<W, true, CNT>(S.nodes, S.tris, r, tmax, t, p, sl, u, v, occ, st, C.err);
    } else if (INST) {
        occ = occluded_placements<W, CNT>(S, o, d, tmin, tmax, st, C.err);
    } else {
        occ = occluded_placement_loop<W, CNT>(S, o, d, tmin, tmax, st, C.err);
    }
    if (CNT) {
        C.nodes += st.nodes;
        C.tris += st.tris;
    }
    return occ;
}

template <int W, bool CNT, bool INST>
__device__ __forceinline__ bool occluded(const SceneDev &S, v3 o, v3 d, float tmax, PathCtx &C) {
    return occluded_t<W, CNT, INST>(S, o, d, 1e-5f, tmax, C);
}

// Geometry of a closest hit of the ray (o, d): world point, geometric normal,
// world distance, and the ray in the triangle's own space (for barycentrics).
// WORLD_N = false keeps the object-space normal of an instanced hit, as the
// reference does (model.cpp:117-121 maps only the point back).
struct HitGeom {
    v3 p, Ng;
    float dist;
    v3 ro, rd;
};
template <bool WORLD_N>
__device__ __forceinline__ HitGeom hit_geom(const SceneDev &S, const Hit &h, v3 o, v3 d) {
    HitGeom g;
    v3 a, b, c;
    slot_verts(S, h.slot, a, b, c);
    if (h.inst == kNoInst) {
        g.p = add(o, mul(d, h.t));
        g.dist = h.t;
        g.ro = o;
        g.rd = d;
    } else {
        float len;
        inst_ray(S, h.inst, o, d, g.ro, g.rd, len);
        g.p = inst_point(S, h.inst, g.ro, g.rd, h.t);
        g.dist = vdist(g.p, o);
        if (WORLD_N) {
            const float4 *F = S.inst + 6 * (size_t)h.inst + 3;
            a = xf_point(F, a);
            b = xf_point(F, b);
            c = xf_point(F, c);
        }
    }
    g.Ng = normalize(cross(sub(b, a), sub(c, a)));
    return g;
}

// Colour (RGBA) of the surface a ray (o, d) hit on triangle slot `slot`.  The
// barycentrics are recomputed with the traversal's watertight test, a pure
// function of ray and triangle, so every form of the renderer (and the CPU
// oracle) reads the same texel whatever produced the hit.
__device__ inline float4 hit_colour(const SceneDev &S, const crg_material &m, uint32_t prim, uint32_t slot, v3 o, v3 d) {
    // (o, d) is the ray in the triangle's space (HitGeom::ro / rd)
    if (!textured(S, m)) return make_float4(m.colour[0], m.colour[1], m.colour[2], m.colour[3]);
    const RayPre r = ray_prep(o.x, o.y, o.z, d.x, d.y, d.z, 1e-5f);
    TriHit th;
    float b1 = 0.0f, b2 = 0.0f;
    if (watertight(r, __ldg(&S.tris[slot * 3 + 0]), __ldg(&S.tris[slot * 3 + 1]), __ldg(&S.tris[slot * 3 + 2]), th)) {
        b1 = th.V / th.det;
        b2 = th.W / th.det;
    }
    float u, v;
    interp_uv(S, prim, b1, b2, u, v);
    return tex_lookup(S, m.tex, u, v);
}

// ------------------------------------------------------------------ path state
// One path between bounces.  Shading a bounce (shade_faithful / shade_extended)
// consumes the closest hit (or miss) of the current segment, updates the
// state, and may ask for one shadow test (NeeReq) whose contribution the
// caller adds to L if the test passes, before the next segment.
struct PathState {
    v3 o, d, T, L;
    float prev_pdf;
    uint32_t prev_delta;
};
struct NeeReq {
    v3 o, d, c;
    float tmax;
    uint32_t kind; // 0 none, 1 emitter (any hit below tmax), 2 sun (closest hit with alpha pass-through)
    // parameter factors of c beyond the path throughput (for the adjoint)
    uint32_t bsdf_mat, light_mat;
    v3 bsdf_dlog; // d log(BSDF factor) / d colour, per channel
};

// Records how a path's radiance depends on material parameters (adjoint).
// Every contribution to L is the throughput (a product of per-bounce factors,
// each depending on one material's colour) times emitter terms; the tape sees
// each factor and each contribution.  NullTape compiles to nothing.
struct NullTape {
    __device__ __forceinline__ void mult(uint32_t, v3) {}
    __device__ __forceinline__ void emit(v3, uint32_t) {}
    __device__ __forceinline__ void env(v3) {}
};

__device__ __forceinline__ v3 inv_or_zero(v3 c) {
    return mk(c.x > 0.0f ? 1.0f / c.x : 0.0f, c.y > 0.0f ? 1.0f / c.y : 0.0f, c.z > 0.0f ? 1.0f / c.z : 0.0f);
}

__device__ __forceinline__ void path_start(PathState &ps, v3 o, v3 d) {
    ps.o = o;
    ps.d = d;
    ps.T = mk(1, 1, 1);
    ps.L = mk(0, 0, 0);
    ps.prev_pdf = 0.0f;
    ps.prev_delta = 1u;
}

// ------------------------------------------------------------------ faithful
// process_hit + the bounce body of _sample_pixel (renderer.cpp:21-102, 272-355).
__device__ inline bool shade_faithful(const SceneDev &S, const crg_settings &set, const PathCtx &C, uint32_t i, PathState &ps,
                               bool found, const Hit &h, Aov &aov, NeeReq &nr) {
    nr.kind = 0;
    if (!found) {
        const v3 env = sample_sky(S, ps.d);
        if (i == 0) aov.albedo = env;
        ps.L = add(ps.L, mulv(ps.T, env));
        return false;
    }
    const HitGeom hg = hit_geom<false>(S, h, ps.o, ps.d);
    const v3 p = hg.p, Ng = hg.Ng;
    const crg_material &m = S.mats[__ldg(&S.mat_idx[h.prim])];
    const float4 col = hit_colour(S, m, h.prim, h.slot, hg.ro, hg.rd);
    const float c0 = col.x, c1 = col.y, c2 = col.z, c3 = col.w;
    if (c3 == 0.0f) {
        ps.o = add(p, mul(ps.d, 0.1f));
        return true;
    }
    v3 albedo = mk(c0, c1, c2);
    const f4 g = rand4(C.pix, C.sample, 1 + 2 * i, C.seed);
    v3 no, nd;
    const uint32_t shade = m.shade_type;
    if (shade == CRG_SHADE_GLASS) {
        const v3 reflected = reflect(ps.d, Ng);
        v3 out_n = Ng;
        float eta = 1.0f / m.ior;
        if (dot(ps.d, Ng) > 0.0f) {
            out_n = neg(Ng);
            eta = m.ior;
        }
        const v3 uv = normalize(ps.d);
        const float dt = dot(uv, out_n);
        const float disc = 1.0f - (eta * eta) * (1.0f - dt * dt);
        no = add(p, mul(out_n, -0.0001f));
        if (disc > 0.0f) nd = sub(mul(sub(uv, mul(out_n, dt)), eta), mul(out_n, sqrtf(disc)));
        else nd = reflected;
    } else if (shade == CRG_SHADE_METAL) {
        no = add(p, mul(Ng, 0.0001f));
        nd = reflect(ps.d, Ng);
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
        aov.depth = hg.dist;
    }
    ps.T = mulv(ps.T, albedo);
    ps.L = add(ps.L, mul(ps.T, m.emission));
    if (S.sun_on) {
        // renderer.cpp:315-354; the shadow ray is a closest-hit cast that steps
        // through alpha surfaces; the contribution is added when it escapes
        const v3 so = add(p, mul(Ng, 0.001f));
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
        const v3 ms = mk(S.sun_neg_dir[0], S.sun_neg_dir[1], S.sun_neg_dir[2]);
        v3 sky = mk(0, 0, 0);
        if (dot(sd, ms) > S.sun_cos) sky = mk(S.sun_rad[0], S.sun_rad[1], S.sun_rad[2]);
        const v3 tc = mulv(ps.T, mk(c0, c1, c2));
        nr.kind = 2;
        nr.o = so;
        nr.d = sd;
        nr.tmax = INFINITY;
        nr.c = mk(((tc.x * cosine) * sky.x) / S.sun_pdf, ((tc.y * cosine) * sky.y) / S.sun_pdf,
                  ((tc.z * cosine) * sky.z) / S.sun_pdf);
    }
    ps.o = no;
    ps.d = nd;
    if (set.rr_depth > 0 && i + 1 >= set.rr_depth) {
        const float q = mn(mx(mx(ps.T.x, ps.T.y), ps.T.z), 0.95f);
        if (g.w >= q) return false;
        ps.T = mk(ps.T.x / q, ps.T.y / q, ps.T.z / q);
    }
    return true;
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
__device__ __forceinline__ v3 schlick(v3 f0, float c, float *m5_out = nullptr) {
    const float m = 1.0f - clampf(c, 0.0f, 1.0f);
    const float m2 = m * m;
    const float m5 = (m2 * m2) * m;
    if (m5_out) *m5_out = m5;
    return mk(f0.x + (1.0f - f0.x) * m5, f0.y + (1.0f - f0.y) * m5, f0.z + (1.0f - f0.z) * m5);
}
// d log(Schlick F) / d colour for F0 = colour * reflectiveness
__device__ __forceinline__ v3 schlick_dlog(v3 Fr, float m5, float refl) {
    const float k = refl * (1.0f - m5);
    return mk(Fr.x > 0.0f ? k / Fr.x : 0.0f, Fr.y > 0.0f ? k / Fr.y : 0.0f, Fr.z > 0.0f ? k / Fr.z : 0.0f);
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

// Emitter entry with probability proportional to power: the alias table's
// column floor(u1 * n), kept when u2 < its probability, else its alias.
__device__ __forceinline__ uint32_t pick_light(const SceneDev &S, float u1, float u2) {
    uint32_t j = (uint32_t)(u1 * (float)S.nlights);
    if (j >= S.nlights) j = S.nlights - 1;
    const float2 e = __ldg(&S.light_alias[j]);
    return u2 < e.x ? j : __float_as_uint(e.y);
}

// Emissive-triangle NEE at p: fills nr (kind 1) with the shadow ray and the
// contribution it carries if unoccluded; bsdf 0 = Lambert (albedo), 1 = GGX.
__device__ inline void nee_prepare(const SceneDev &S, const PathCtx &C, uint32_t i, v3 p, v3 n, v3 T, int bsdf, v3 albedo,
                            const onb &F, v3 wol, float alpha, NeeReq &nr, uint32_t mat = 0, float refl = 1.0f) {
    nr.kind = 0;
    const f4 g = rand4(C.pix, C.sample, 2 + 2 * i, C.seed);
    const uint32_t j = pick_light(S, g.x, g.w);
    // the emitter entry's record: world-space corners, pdf, primitive, material, radiance
    const float4 r0 = __ldg(&S.light_rec[4 * (size_t)j + 0]), r1 = __ldg(&S.light_rec[4 * (size_t)j + 1]);
    const float4 r2 = __ldg(&S.light_rec[4 * (size_t)j + 2]), r3 = __ldg(&S.light_rec[4 * (size_t)j + 3]);
    const v3 a = mk(r0.x, r0.y, r0.z), b = mk(r1.x, r1.y, r1.z), c = mk(r2.x, r2.y, r2.z);
    const uint32_t prim = __float_as_uint(r1.w), lmi = __float_as_uint(r2.w);
    const float su = sqrtf(g.y);
    const float b0 = 1.0f - su, b1 = su * (1.0f - g.z), b2 = su * g.z;
    const v3 pl = add(add(mul(a, b0), mul(b, b1)), mul(c, b2));
    const v3 po = add(p, mul(n, 1e-4f));
    const v3 w = sub(pl, po);
    const float d2 = dot(w, w);
    if (!(d2 > 0.0f)) return;
    const float dist = sqrtf(d2);
    const v3 wi = mul(w, 1.0f / dist);
    const float cos_s = dot(wi, n);
    if (!(cos_s > 0.0f)) return;
    const v3 Ngl = normalize(cross(sub(b, a), sub(c, a)));
    const float cos_l = absf(dot(Ngl, wi));
    if (!(cos_l > 0.0f)) return;
    v3 Le = mk(r3.x, r3.y, r3.z); // colour * emission
    if (__float_as_uint(r3.w)) {   // textured emitter: texture colour at the sampled point * emission
        const crg_material &lm = S.mats[lmi];
        float tu, tv;
        interp_uv(S, prim, b1, b2, tu, tv);
        const float4 t = tex_lookup(S, lm.tex, tu, tv);
        Le = mk(t.x * lm.emission, t.y * lm.emission, t.z * lm.emission);
    }
    const float p_light = (r0.w * d2) / cos_l;
    v3 f;
    float p_bsdf, cos_i;
    if (bsdf == 0) {
        f = mul(albedo, kInvPi);
        p_bsdf = cos_s * kInvPi;
        cos_i = cos_s;
        nr.bsdf_dlog = inv_or_zero(albedo);
    } else {
        const v3 wil = to_local(F, wi);
        if (!(wil.z > 0.0f)) return;
        const v3 hv = normalize(add(wol, wil));
        const float woh = dot(wol, hv);
        const float D = ggx_D(hv.z, alpha);
        const float lo_ = ggx_lambda(wol, alpha), li = ggx_lambda(wil, alpha);
        const float G2 = 1.0f / ((1.0f + lo_) + li);
        const float G1 = 1.0f / (1.0f + lo_);
        float m5;
        const v3 Fr = schlick(albedo, woh, &m5);
        f = mul(Fr, (D * G2) / ((4.0f * wol.z) * wil.z));
        p_bsdf = (G1 * D) / (4.0f * wol.z);
        cos_i = wil.z;
        nr.bsdf_dlog = schlick_dlog(Fr, m5, refl);
    }
    const float w_mis = (p_light * p_light) / (p_light * p_light + p_bsdf * p_bsdf);
    nr.bsdf_mat = mat;
    nr.light_mat = lmi;
    nr.kind = 1;
    nr.o = po;
    nr.d = wi;
    nr.tmax = dist * 0.999f;
    nr.c = mul(mulv(mulv(T, f), Le), (cos_i * w_mis) / p_light);
}

// Extended estimator bounce: MIS-weighted emission, emissive-triangle NEE,
// Lambert (geometric-normal hemisphere) / GGX VNDF / Fresnel dielectric, RR.
template <class Tape = NullTape>
__device__ inline bool shade_extended(const SceneDev &S, const crg_settings &set, const PathCtx &C, uint32_t i, PathState &ps,
                                      bool found, const Hit &h, Aov &aov, NeeReq &nr, Tape *tape = nullptr) {
    nr.kind = 0;
    if (!found) {
        const v3 env = sample_sky(S, ps.d);
        if (i == 0) aov.albedo = env;
        const v3 contrib = mulv(ps.T, env);
        ps.L = add(ps.L, contrib);
        if (tape) tape->env(contrib);
        return false;
    }
    const HitGeom hg = hit_geom<true>(S, h, ps.o, ps.d);
    const v3 p = hg.p, Ng = hg.Ng;
    const uint32_t mi = __ldg(&S.mat_idx[h.prim]);
    const crg_material &m = S.mats[mi];
    const float4 col = hit_colour(S, m, h.prim, h.slot, hg.ro, hg.rd);
    const float c0 = col.x, c1 = col.y, c2 = col.z, c3 = col.w;
    if (c3 == 0.0f) {
        ps.o = add(p, mul(ps.d, 0.1f));
        return true;
    }
    const v3 rgb = mk(c0, c1, c2);
    const float cos_nd = dot(Ng, ps.d);
    const v3 n = cos_nd < 0.0f ? Ng : neg(Ng);
    if (i == 0) {
        aov.albedo = rgb;
        aov.normal = Ng;
        aov.depth = hg.dist;
    }
    const float emission = m.emission;
    if (emission > 0.0f) {
        const v3 Le = mk(c0 * emission, c1 * emission, c2 * emission);
        if (ps.prev_delta) {
            const v3 contrib = mulv(ps.T, Le);
            ps.L = add(ps.L, contrib);
            if (tape) tape->emit(contrib, mi);
        } else {
            const float cos_l = absf(cos_nd);
            if (cos_l > 0.0f) {
                const float pl = (__ldg(&S.mat_light_pdf[mi]) * (hg.dist * hg.dist)) / cos_l;
                const float w = (ps.prev_pdf * ps.prev_pdf) / (ps.prev_pdf * ps.prev_pdf + pl * pl);
                const v3 contrib = mul(mulv(ps.T, Le), w);
                ps.L = add(ps.L, contrib);
                if (tape) tape->emit(contrib, mi);
            }
        }
    }
    const f4 g = rand4(C.pix, C.sample, 1 + 2 * i, C.seed);
    const v3 wo = neg(ps.d);
    const bool have_lights = S.nlights > 0 && i + 1 < set.max_bounces;
    const uint32_t shade = m.shade_type;
    if (shade == CRG_SHADE_SMOOTH) {
        const onb F = build_local(Ng);
        if (have_lights) nee_prepare(S, C, i, p, Ng, ps.T, 0, rgb, F, mk(0, 0, 0), 0.0f, nr, mi);
        float sp, cp;
        sincos2pi(g.y, &sp, &cp);
        const float r = sqrtf(g.x);
        const v3 l = mk(r * cp, r * sp, sqrtf(mx(0.0f, 1.0f - g.x)));
        ps.d = from_local(F, l);
        ps.o = add(p, mul(Ng, 1e-4f));
        ps.prev_pdf = l.z * kInvPi;
        ps.prev_delta = 0u;
        ps.T = mulv(ps.T, rgb);
        if (tape) tape->mult(mi, inv_or_zero(rgb));
    } else if (shade == CRG_SHADE_METAL) {
        const v3 f0 = mul(rgb, m.reflectiveness);
        const float alpha = m.roughness;
        if (alpha < 1e-4f) {
            ps.d = reflect(ps.d, n);
            ps.o = add(p, mul(n, 1e-4f));
            ps.T = mulv(ps.T, f0);
            ps.prev_delta = 1u;
            if (tape) tape->mult(mi, inv_or_zero(rgb));
        } else {
            const onb F = build_local(n);
            const v3 wol = to_local(F, wo);
            if (!(wol.z > 0.0f)) return false;
            if (have_lights) nee_prepare(S, C, i, p, n, ps.T, 1, f0, F, wol, alpha, nr, mi, m.reflectiveness);
            const v3 hh = sample_vndf(wol, alpha, g.x, g.y);
            const float woh = dot(wol, hh);
            const float k2 = 2.0f * woh;
            const v3 wil = mk(hh.x * k2 - wol.x, hh.y * k2 - wol.y, hh.z * k2 - wol.z);
            if (!(wil.z > 0.0f)) return false;
            const float lo_ = ggx_lambda(wol, alpha), li = ggx_lambda(wil, alpha);
            const float G1 = 1.0f / (1.0f + lo_);
            const float G2 = 1.0f / ((1.0f + lo_) + li);
            float m5;
            const v3 Fr = schlick(f0, woh, &m5);
            ps.T = mulv(ps.T, mul(Fr, G2 / G1));
            if (tape) tape->mult(mi, schlick_dlog(Fr, m5, m.reflectiveness));
            ps.prev_pdf = (G1 * ggx_D(hh.z, alpha)) / (4.0f * wol.z);
            ps.prev_delta = 0u;
            ps.d = from_local(F, wil);
            ps.o = add(p, mul(n, 1e-4f));
        }
    } else {
        const float eta = cos_nd < 0.0f ? 1.0f / m.ior : m.ior;
        const float ci = -dot(ps.d, n);
        float st2;
        const float Fr = fresnel_dielectric(ci, eta, st2);
        if (g.z < Fr) {
            ps.d = reflect(ps.d, n);
            ps.o = add(p, mul(n, 1e-4f));
        } else {
            const float cic = clampf(ci, 0.0f, 1.0f);
            const float ct = sqrtf(1.0f - st2);
            ps.d = add(mul(ps.d, eta), mul(n, eta * cic - ct));
            ps.o = add(p, mul(n, -1e-4f));
        }
        ps.T = mulv(ps.T, rgb);
        ps.prev_delta = 1u;
        if (tape) tape->mult(mi, inv_or_zero(rgb));
    }
    if (set.rr_depth > 0 && i + 1 >= set.rr_depth) {
        const float q = mn(mx(mx(ps.T.x, ps.T.y), ps.T.z), 0.95f);
        if (g.w >= q) return false;
        ps.T = mk(ps.T.x / q, ps.T.y / q, ps.T.z / q);
    }
    return true;
}

// The shadow test a NeeReq asks for: kind 1 = any hit below tmax; kind 2 =
// closest hits stepping 0.1 past alpha-zero surfaces (renderer.cpp:330-345).
template <int W, bool CNT, bool INST>
__device__ __forceinline__ bool shadow_visible(const SceneDev &S, const NeeReq &nr, PathCtx &C) {
    if (nr.kind == 1) {
        C.shadow++;
        return !occluded<W, CNT, INST>(S, nr.o, nr.d, nr.tmax, C);
    }
    v3 so = nr.o;
    for (;;) {
        Hit sh;
        C.shadow++;
        if (!closest<W, CNT, INST>(S, so, nr.d, INFINITY, sh, C)) return true;
        const HitGeom hg = hit_geom<false>(S, sh, so, nr.d);
        if (hit_colour(S, S.mats[__ldg(&S.mat_idx[sh.prim])], sh.prim, sh.slot, hg.ro, hg.rd).w != 0.0f) return false;
        so = add(hg.p, mul(nr.d, 0.1f));
    }
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

} // namespace rc
} // namespace crg
