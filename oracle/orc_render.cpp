/*
 * orc_render.cpp — CPU oracle of the integrator.  TEST INFRASTRUCTURE ONLY.
 *
 * FAITHFUL mode restates cr::renderer::_sample_pixel and process_hit
 * (src/render/renderer.cpp:21-102, 258-384) with CRender's sampling helpers
 * (src/util/sampling.h:21-183) and camera (src/render/camera.cpp:14-68).
 * The only deliberate difference is the random number source: the reference
 * draws from a thread_local std::mt19937 whose stream depends on the thread
 * schedule (renderer.cpp:6-11); here every draw is a pure function of
 * (pixel, sample, dimension group, seed) so the GPU can reproduce it.
 *
 * EXTENDED mode keeps the same path space and adds power-heuristic MIS
 * between BSDF sampling and emissive-triangle next-event estimation, a GGX
 * microfacet metal sampled by visible normals (Heitz, "Sampling the GGX
 * Distribution of Visible Normals", JCGT 7(4), 2018; D as in
 * sampling.h:93-106), an exact unpolarised Fresnel dielectric, and Russian
 * roulette.  Lambertian surfaces scatter into the hemisphere of the geometric
 * normal as in the reference; GGX and glass use the normal facing the ray.
 * Its expectation equals the faithful estimator's on Lambertian scenes
 * without sun.
 *
 * Random dimension groups per sample: 0 = pixel jitter; 1 + 2i = BSDF at
 * segment i (x, y direction, z lobe, w roulette); 2 + 2i = light sample at
 * segment i (x light, y z point) — the faithful sun uses (x, y).
 */
#include "orc.h"
#include "orc_math.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <limits>
#include <thread>
#include <vector>

namespace orc_internal {
bool closest(const orc_bvh *b, const crg_ray &ray, crg_hit &hit);
bool any(const orc_bvh *b, const crg_ray &ray);
const float *verts(const orc_bvh *b);
} // namespace orc_internal

using namespace orc;

namespace {

const float kInf = std::numeric_limits<float>::infinity();

struct CamParams {
    float pos[3];
    float R[3][3]; /* row-major rotation Ry(x) * Rx(y) * Rz(z) */
    float w;       /* 1 / tan(fov / 2) */
    uint32_t mode;
    float scale;
};

CamParams camera_params(const crg_camera &c) {
    CamParams p;
    for (int a = 0; a < 3; ++a) p.pos[a] = c.position[a];
    const double k = 3.14159265358979323846 / 180.0;
    const double ax = c.rotation[0] * k, ay = c.rotation[1] * k, az = c.rotation[2] * k;
    const double Ry[3][3] = {{std::cos(ax), 0, std::sin(ax)}, {0, 1, 0}, {-std::sin(ax), 0, std::cos(ax)}};
    const double Rx[3][3] = {{1, 0, 0}, {0, std::cos(ay), -std::sin(ay)}, {0, std::sin(ay), std::cos(ay)}};
    const double Rz[3][3] = {{std::cos(az), -std::sin(az), 0}, {std::sin(az), std::cos(az), 0}, {0, 0, 1}};
    double T[3][3], R[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T[i][j] = 0;
            for (int m = 0; m < 3; ++m) T[i][j] += Ry[i][m] * Rx[m][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            R[i][j] = 0;
            for (int m = 0; m < 3; ++m) R[i][j] += T[i][m] * Rz[m][j];
            p.R[i][j] = (float)R[i][j];
        }
    p.w = (float)(1.0 / std::tan(0.5 * (double)c.fov * k));
    p.mode = c.mode;
    p.scale = c.scale;
    return p;
}

/* camera::get_ray (camera.cpp:14-39) */
void camera_ray(const CamParams &c, float x, float y, float aspect, v3 &o, v3 &d) {
    if (c.mode == CRG_CAMERA_ORTHOGRAPHIC) {
        const float u = 2.0f * x - 1.0f;
        const float v = 2.0f * y - 1.0f;
        const float su = c.scale * u, sv = c.scale * v;
        float org[3];
        for (int i = 0; i < 3; ++i) org[i] = ((c.R[i][0] * su + c.R[i][1] * sv) + c.R[i][2] * 0.0f) + c.pos[i];
        o = mk(org[0], org[1], org[2]);
        d = normalize(mk(c.R[0][2], c.R[1][2], c.R[2][2]));
        return;
    }
    const float u = (2.0f * x - 1.0f) * aspect;
    const float v = 2.0f * y - 1.0f;
    float dir[3];
    for (int i = 0; i < 3; ++i) dir[i] = (c.R[i][0] * u + c.R[i][1] * v) + c.R[i][2] * c.w;
    o = mk(c.pos[0], c.pos[1], c.pos[2]);
    d = normalize(mk(dir[0], dir[1], dir[2]));
}

struct Scene {
    Scene() = default;
    Scene(const Scene &) = delete;
    Scene &operator=(const Scene &) = delete;
    ~Scene() {
        for (orc_bvh *b : bvhs) orc_bvh_free(b);
    }
    const orc_bvh *bvh = nullptr; /* the BVH of a scene of one model */
    /* models (cr::registry entities): each its own BVH over its own triangles,
     * primitives [mfirst[m], mfirst[m] + its count) of the scene arrays */
    std::vector<orc_bvh *> bvhs;
    std::vector<uint32_t> mfirst;
    std::vector<uint32_t> place_model; /* model of each placement (instance) */
    const float *verts = nullptr;
    const uint32_t *mat_idx = nullptr;
    const crg_material *mats = nullptr;
    uint32_t nmat = 0;
    const float *sky = nullptr;
    uint32_t sky_w = 0, sky_h = 0;
    float sky_rot_u = 0, sky_rot_v = 0;
    bool sun_on = false;
    crg_sun sun{};
    onb sun_frame{};
    float sun_cos = 1, sun_pdf = 0;
    /* emissive triangles (extended mode) */
    std::vector<uint32_t> light_prim;
    std::vector<float> light_prob, light_pdf; /* alias table: probability and alias per entry */
    std::vector<uint32_t> light_alias;
    std::vector<float> mat_light_pdf;
    /* texture coordinates and textures */
    const float *uvs = nullptr;
    uint32_t ntex = 0;
    const float *const *tex_rgba = nullptr;
    const uint32_t *tex_w = nullptr, *tex_h = nullptr;
    /* instances: per instance 24 floats, the inverse's 3 rows [A | t] then the
     * forward transform's; empty = the mesh as is */
    uint32_t ninst = 0;
    std::vector<float> inst_rows;
    std::vector<uint32_t> light_inst;
};

constexpr uint32_t kNoInst = 0xFFFFFFFFu;

/* image::get_uv (src/objects/image.h:104-109): nearest texel, modulo wrap. */
uint64_t texel_index(float u, uint32_t n) {
    const float f = u * (float)n;
    uint64_t i = 0;
    if (f >= 0.0f) i = f < 4.6e18f ? (uint64_t)f : 0;
    return i % n;
}

v3 sample_sky(const Scene &S, v3 d) {
    if (!S.sky) return mk(0, 0, 0);
    const float dy = clampf(d.y, -1.0f, 1.0f);
    const float u = 0.5f + std::atan2(d.z, d.x) * kInvTau;
    const float v = 0.5f - std::asin(dy) * kInvPi;
    const uint64_t x = texel_index(u + S.sky_rot_u, S.sky_w);
    const uint64_t y = texel_index(v + S.sky_rot_v, S.sky_h);
    const float *t = S.sky + (x + y * S.sky_w) * 4;
    return mk(t[0], t[1], t[2]);
}

/* process_hit's colour (renderer.cpp:30-35): texture `tex` at the hit's
 * interpolated texture coordinate (rtcInterpolate0, model.cpp:39-47), nearest
 * texel with modulo wrap, else the material colour.  (b1, b2) are the
 * barycentrics of vertices 1 and 2. */
bool textured(const Scene &S, const crg_material &m) { return m.tex >= 0 && (uint32_t)m.tex < S.ntex; }

void interp_uv(const Scene &S, uint32_t prim, float b1, float b2, float &u, float &v) {
    if (!S.uvs) {
        u = v = 0.0f;
        return;
    }
    const float *t = S.uvs + (size_t)prim * 6;
    const float b0 = (1.0f - b1) - b2;
    u = (b0 * t[0] + b1 * t[2]) + b2 * t[4];
    v = (b0 * t[1] + b1 * t[3]) + b2 * t[5];
}

const float *tex_lookup(const Scene &S, int32_t tex, float u, float v) {
    const uint32_t w = S.tex_w[tex], h = S.tex_h[tex];
    const uint64_t x = texel_index(u, w), y = texel_index(v, h);
    return S.tex_rgba[tex] + (x + y * w) * 4;
}

/* RGBA colour of the surface at a closest hit. */
void hit_colour(const Scene &S, const crg_material &m, const crg_hit &h, float col[4]) {
    const float *c = m.colour;
    if (textured(S, m)) {
        float u, v;
        interp_uv(S, h.prim, h.u, h.v, u, v);
        c = tex_lookup(S, m.tex, u, v);
    }
    for (int k = 0; k < 4; ++k) col[k] = c[k];
}

/* sampling::sun::sample's direction (sampling.h:35-43, 72-80): the cone of
 * half-angle size around the sun, map_to_solid_angle with phi = 2 pi u1 and
 * cos(theta) = 1 - u2 (1 - cos(size)), turned by the sun frame's columns
 * (tangent, normal, bitangent; registry.cpp:44-48). */
v3 sun_direction(const onb &F, float sun_cos, float u1, float u2) {
    float sp, cp;
    sincos2pi(u1, &sp, &cp);
    const float ct = 1.0f - u2 * (1.0f - sun_cos);
    const float st = std::sqrt(1.0f - ct * ct);
    const v3 lv = mk(cp * st, ct, sp * st);
    return mk((F.t.x * lv.x + F.n.x * lv.y) + F.b.x * lv.z, (F.t.y * lv.x + F.n.y * lv.y) + F.b.y * lv.z,
              (F.t.z * lv.x + F.n.z * lv.y) + F.b.z * lv.z);
}

/* sampling::cos_hemp (sampling.h:174-183): cosine-weighted local direction,
 * radius sqrt(x) at angle 2 pi y. */
v3 cos_hemp(float x, float y) {
    float sp, cp;
    sincos2pi(y, &sp, &cp);
    const float r = std::sqrt(x);
    return mk(r * cp, r * sp, std::sqrt(maxf(0.0f, 1.0f - x)));
}

struct Ctx {
    const Scene *S;
    const crg_settings *set;
    uint32_t pix, sample;
    uint64_t segments = 0, shadow = 0;
};

/* ---- instances (cr::entity::instances, model::intersect at model.cpp:99-126) */
v3 xf_point(const float *R, v3 p) {
    return mk(((R[0] * p.x + R[1] * p.y) + R[2] * p.z) + R[3], ((R[4] * p.x + R[5] * p.y) + R[6] * p.z) + R[7],
              ((R[8] * p.x + R[9] * p.y) + R[10] * p.z) + R[11]);
}
v3 xf_vector(const float *R, v3 v) {
    return mk((R[0] * v.x + R[1] * v.y) + R[2] * v.z, (R[4] * v.x + R[5] * v.y) + R[6] * v.z,
              (R[8] * v.x + R[9] * v.y) + R[10] * v.z);
}
/* the object-space ray: inverse(T) (o, 1) and normalize(inverse(T) (d, 0)) */
void inst_ray(const Scene &S, uint32_t j, v3 o, v3 d, v3 &oo, v3 &od, float &len) {
    const float *R = &S.inst_rows[24 * (size_t)j];
    oo = xf_point(R, o);
    const v3 dr = xf_vector(R, d);
    len = std::sqrt(dot(dr, dr));
    od = normalize(dr);
}
v3 inst_point(const Scene &S, uint32_t j, v3 oo, v3 od, float t) {
    return xf_point(&S.inst_rows[24 * (size_t)j + 12], add(oo, mul(od, t)));
}
float vdist(v3 a, v3 b) {
    const v3 e = sub(a, b);
    return std::sqrt(dot(e, e));
}

/* Closest hit.  Instanced scenes run the reference's loop literally: each
 * instance traced to infinity in its object space, the world distance
 * |T p - o| recomputed, the smaller one kept (ties to the earlier instance);
 * h.t is then the object-space parameter and inst the instance. */
bool cast_query(const Scene &S, v3 o, v3 d, float tmin, float tmax, crg_hit &h, uint32_t &inst) {
    inst = kNoInst;
    if (S.ninst == 0) {
        crg_ray r{{o.x, o.y, o.z}, tmin, {d.x, d.y, d.z}, tmax};
        return orc_internal::closest(S.bvh, r, h);
    }
    /* the placements are scene.cpp:79-98's entities in order, each expanded
     * into model.cpp:99-126's instances in order; both loops keep a strictly
     * smaller distance, so one pass over the placements in order is their result */
    float best = tmax;
    bool found = false;
    for (uint32_t j = 0; j < S.ninst; ++j) {
        v3 oo, od;
        float len;
        inst_ray(S, j, o, d, oo, od, len);
        crg_ray r{{oo.x, oo.y, oo.z}, tmin, {od.x, od.y, od.z}, kInf};
        crg_hit hj;
        const uint32_t m = S.place_model[j];
        if (!orc_internal::closest(S.bvhs[m], r, hj)) continue;
        hj.prim += S.mfirst[m];
        const float dist = vdist(inst_point(S, j, oo, od, hj.t), o);
        if (dist < best) {
            best = dist;
            h = hj;
            inst = j;
            found = true;
        }
    }
    return found;
}

bool cast(const Scene &S, v3 o, v3 d, float tmax, crg_hit &h, uint32_t &inst) {
    return cast_query(S, o, d, 1e-5f, tmax, h, inst);
}

/* Any hit below tmax; instanced: any instance with a hit whose object-space
 * parameter is below tmax |inverse(T) d| / |d|. */
bool occluded_query(const Scene &S, v3 o, v3 d, float tmin, float tmax) {
    if (S.ninst == 0) {
        crg_ray r{{o.x, o.y, o.z}, tmin, {d.x, d.y, d.z}, tmax};
        return orc_internal::any(S.bvh, r);
    }
    const float dl = std::sqrt(dot(d, d));
    for (uint32_t j = 0; j < S.ninst; ++j) {
        v3 oo, od;
        float len;
        inst_ray(S, j, o, d, oo, od, len);
        crg_ray r{{oo.x, oo.y, oo.z}, tmin, {od.x, od.y, od.z}, (tmax * len) / dl};
        if (orc_internal::any(S.bvhs[S.place_model[j]], r)) return true;
    }
    return false;
}

bool occluded(const Scene &S, v3 o, v3 d, float tmax) { return occluded_query(S, o, d, 1e-5f, tmax); }

void tri_verts(const Scene &S, uint32_t prim, v3 &a, v3 &b, v3 &c) {
    const float *v = S.verts + (size_t)prim * 9;
    a = mk(v[0], v[1], v[2]);
    b = mk(v[3], v[4], v[5]);
    c = mk(v[6], v[7], v[8]);
}

/* World point, geometric normal and world distance of a closest hit.  The
 * faithful estimator keeps an instanced hit's object-space normal, as
 * model.cpp:117-121 maps only the point back; world_n transforms the
 * triangle first. */
struct Geom {
    v3 p, Ng;
    float dist;
};
Geom hit_geom(const Scene &S, const crg_hit &h, uint32_t inst, v3 o, v3 d, bool world_n) {
    Geom g;
    v3 a, b, c;
    tri_verts(S, h.prim, a, b, c);
    if (inst == kNoInst) {
        g.p = add(o, mul(d, h.t));
        g.dist = h.t;
    } else {
        v3 oo, od;
        float len;
        inst_ray(S, inst, o, d, oo, od, len);
        g.p = inst_point(S, inst, oo, od, h.t);
        g.dist = vdist(g.p, o);
        if (world_n) {
            const float *F = &S.inst_rows[24 * (size_t)inst + 12];
            a = xf_point(F, a);
            b = xf_point(F, b);
            c = xf_point(F, c);
        }
    }
    g.Ng = normalize(cross(sub(b, a), sub(c, a)));
    return g;
}

/* sampling.h:156-166 (cr::sampling::sphere) */
v3 sphere(float u1, float u2) {
    const float cos_t = 2.0f * u1 - 1.0f;
    const float sin_t = std::sqrt(1.0f - cos_t * cos_t);
    float sp, cp;
    sincos2pi(u2, &sp, &cp);
    return mk(sin_t * cp, cos_t, sin_t * sp);
}

struct Aov {
    v3 albedo{0, 0, 0}, normal{0, 0, 0};
    float depth = 0;
};

/* ------------------------------------------------------------ faithful */

v3 trace_faithful(Ctx &C, v3 o, v3 d, Aov &aov) {
    const Scene &S = *C.S;
    const crg_settings &set = *C.set;
    v3 T = mk(1, 1, 1), L = mk(0, 0, 0);
    for (uint32_t i = 0; i < set.max_bounces; ++i) {
        crg_hit h;
        uint32_t hinst;
        C.segments++;
        if (!cast(S, o, d, kInf, h, hinst)) {
            const v3 env = sample_sky(S, d);
            if (i == 0) aov.albedo = env;
            L = add(L, mulv(T, env));
            break;
        }
        const Geom hg = hit_geom(S, h, hinst, o, d, false);
        const v3 p = hg.p, Ng = hg.Ng;
        const crg_material &m = S.mats[S.mat_idx[h.prim]];
        float col[4];
        hit_colour(S, m, h, col);
        if (col[3] == 0.0f) {
            o = add(p, mul(d, 0.1f));
            continue;
        }
        v3 albedo = mk(col[0], col[1], col[2]);
        const f4 g = rand4(C.pix, C.sample, 1 + 2 * i, set.seed);
        v3 no, nd;
        if (m.shade_type == CRG_SHADE_GLASS) {
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
            if (disc > 0.0f) nd = sub(mul(sub(uv, mul(out_n, dt)), eta), mul(out_n, std::sqrt(disc)));
            else nd = reflected;
        } else if (m.shade_type == CRG_SHADE_METAL) {
            no = add(p, mul(Ng, 0.0001f));
            nd = reflect(d, Ng);
            albedo = mul(albedo, m.reflectiveness);
        } else {
            const v3 hc = add(Ng, sphere(g.x, g.y));
            const float l2 = dot(hc, hc);
            nd = l2 > 0.0f ? mul(hc, 1.0f / std::sqrt(l2)) : Ng;
            no = add(p, mul(Ng, 0.0001f));
        }
        if (i == 0) {
            aov.albedo = albedo;
            aov.normal = Ng;
            aov.depth = hg.dist;
        }
        T = mulv(T, albedo);
        L = add(L, mul(T, m.emission));
        if (S.sun_on) {
            /* renderer.cpp:315-354 */
            v3 so = add(p, mul(Ng, 0.001f));
            const f4 g2 = rand4(C.pix, C.sample, 2 + 2 * i, set.seed);
            const v3 sd = sun_direction(S.sun_frame, S.sun_cos, g2.x, g2.y);
            const float cosine = clampf(dot(Ng, sd), 0.0f, 1.0f);
            crg_hit sh;
            uint32_t sinst;
            C.shadow++;
            bool blocked = cast(S, so, sd, kInf, sh, sinst);
            while (blocked) {
                float scol[4];
                hit_colour(S, S.mats[S.mat_idx[sh.prim]], sh, scol);
                if (scol[3] != 0.0f) break;
                so = add(hit_geom(S, sh, sinst, so, sd, false).p, mul(sd, 0.1f));
                C.shadow++;
                blocked = cast(S, so, sd, kInf, sh, sinst);
            }
            if (!blocked) {
                const v3 ms = mk(-S.sun.direction[0], -S.sun.direction[1], -S.sun.direction[2]);
                v3 sky = mk(0, 0, 0);
                if (dot(sd, ms) > S.sun_cos)
                    sky = mk(S.sun.colour[0] * S.sun.intensity, S.sun.colour[1] * S.sun.intensity,
                             S.sun.colour[2] * S.sun.intensity);
                const v3 tc = mulv(T, mk(col[0], col[1], col[2]));
                L = add(L, mk(((tc.x * cosine) * sky.x) / S.sun_pdf, ((tc.y * cosine) * sky.y) / S.sun_pdf,
                              ((tc.z * cosine) * sky.z) / S.sun_pdf));
            }
        }
        o = no;
        d = nd;
        if (set.rr_depth > 0 && i + 1 >= set.rr_depth) {
            const float q = minf(maxf(maxf(T.x, T.y), T.z), 0.95f);
            if (g.w >= q) break;
            T = mk(T.x / q, T.y / q, T.z / q);
        }
    }
    return L;
}

/* ------------------------------------------------------------ adjoint tape
 * Records the parameter factors of a path (path-replay adjoint): every
 * contribution to L is the throughput (a product of per-bounce factors, each
 * depending on one material's colour) times emitter terms.  On each
 * contribution the gradient of <delta, L> is added for every factor:
 * delta * contribution * d log(factor) / d parameter, in double. */
struct Tape {
    std::vector<uint32_t> mat;
    std::vector<v3> dlog;
    double dx = 0, dy = 0, dz = 0;
    const crg_material *mats = nullptr;
    double *g_col = nullptr, *g_em = nullptr;
    void add_factor(uint32_t m, v3 d, double wx, double wy, double wz) {
        if (wx != 0.0 && d.x != 0.0f) g_col[3 * m + 0] += wx * (double)d.x;
        if (wy != 0.0 && d.y != 0.0f) g_col[3 * m + 1] += wy * (double)d.y;
        if (wz != 0.0 && d.z != 0.0f) g_col[3 * m + 2] += wz * (double)d.z;
    }
    void emitter(uint32_t m, double wx, double wy, double wz);
    void path(v3 C, double &wx, double &wy, double &wz) {
        wx = dx * (double)C.x;
        wy = dy * (double)C.y;
        wz = dz * (double)C.z;
        for (size_t k = 0; k < mat.size(); ++k) add_factor(mat[k], dlog[k], wx, wy, wz);
    }
    void mult(uint32_t m, v3 d) {
        mat.push_back(m);
        dlog.push_back(d);
    }
    void env(v3 C) {
        double wx, wy, wz;
        path(C, wx, wy, wz);
    }
    void emit(v3 C, uint32_t m) {
        double wx, wy, wz;
        path(C, wx, wy, wz);
        emitter(m, wx, wy, wz);
    }
    void nee(v3 C, uint32_t bsdf_mat, v3 bsdf_dlog, uint32_t light_mat) {
        double wx, wy, wz;
        path(C, wx, wy, wz);
        add_factor(bsdf_mat, bsdf_dlog, wx, wy, wz);
        emitter(light_mat, wx, wy, wz);
    }
};

v3 inv_or_zero(v3 c) {
    return mk(c.x > 0.0f ? 1.0f / c.x : 0.0f, c.y > 0.0f ? 1.0f / c.y : 0.0f, c.z > 0.0f ? 1.0f / c.z : 0.0f);
}

void Tape::emitter(uint32_t m, double wx, double wy, double wz) {
    const crg_material &em = mats[m];
    add_factor(m, inv_or_zero(mk(em.colour[0], em.colour[1], em.colour[2])), wx, wy, wz);
    if (em.emission > 0.0f) g_em[m] += (wx + wy + wz) / (double)em.emission;
}

/* ------------------------------------------------------------ extended */

float ggx_D(float nh, float a) { /* sampling.h:93-106 */
    const float a2 = a * a;
    const float dd = (nh * a2 - nh) * nh + 1.0f;
    return a2 / ((dd * dd) * kPi);
}
float ggx_lambda(v3 w, float a) {
    const float s2 = w.x * w.x + w.y * w.y;
    const float z2 = w.z * w.z;
    return (std::sqrt(1.0f + ((a * a) * s2) / z2) - 1.0f) * 0.5f;
}
v3 schlick(v3 f0, float c, float *m5_out = nullptr) {
    const float m = 1.0f - clampf(c, 0.0f, 1.0f);
    const float m2 = m * m;
    const float m5 = (m2 * m2) * m;
    if (m5_out) *m5_out = m5;
    return mk(f0.x + (1.0f - f0.x) * m5, f0.y + (1.0f - f0.y) * m5, f0.z + (1.0f - f0.z) * m5);
}
/* d log(Schlick F) / d colour for F0 = colour * reflectiveness */
v3 schlick_dlog(v3 Fr, float m5, float refl) {
    const float k = refl * (1.0f - m5);
    return mk(Fr.x > 0.0f ? k / Fr.x : 0.0f, Fr.y > 0.0f ? k / Fr.y : 0.0f, Fr.z > 0.0f ? k / Fr.z : 0.0f);
}
v3 sample_vndf(v3 ve, float a, float u1, float u2) {
    const v3 vh = normalize(mk(a * ve.x, a * ve.y, ve.z));
    const float lensq = vh.x * vh.x + vh.y * vh.y;
    const v3 t1v = lensq > 0.0f ? mul(mk(-vh.y, vh.x, 0.0f), 1.0f / std::sqrt(lensq)) : mk(1, 0, 0);
    const v3 t2v = cross(vh, t1v);
    const float r = std::sqrt(u1);
    float sp, cp;
    sincos2pi(u2, &sp, &cp);
    const float t1 = r * cp;
    float t2 = r * sp;
    const float sw = 0.5f * (1.0f + vh.z);
    t2 = (1.0f - sw) * std::sqrt(1.0f - t1 * t1) + sw * t2;
    const v3 nh = add(add(mul(t1v, t1), mul(t2v, t2)), mul(vh, std::sqrt(maxf(0.0f, (1.0f - t1 * t1) - t2 * t2))));
    return normalize(mk(a * nh.x, a * nh.y, maxf(0.0f, nh.z)));
}
float fresnel_dielectric(float ci, float eta, float *st2_out) {
    ci = clampf(ci, 0.0f, 1.0f);
    const float st2 = (eta * eta) * (1.0f - ci * ci);
    *st2_out = st2;
    if (st2 >= 1.0f) return 1.0f;
    const float ct = std::sqrt(1.0f - st2);
    const float rs = (eta * ci - ct) / (eta * ci + ct);
    const float rp = (ci - eta * ct) / (ci + eta * ct);
    return 0.5f * (rs * rs + rp * rp);
}
v3 to_local(const onb &F, v3 w) { return mk(dot(w, F.t), dot(w, F.b), dot(w, F.n)); }
v3 from_local(const onb &F, v3 l) { return add(add(mul(F.t, l.x), mul(F.b, l.y)), mul(F.n, l.z)); }

/* Walker's alias method: column floor(u1 * n), kept when u2 < its
 * probability, else its alias. */
uint32_t pick_light(const Scene &S, float u1, float u2) {
    const uint32_t n = (uint32_t)S.light_prim.size();
    uint32_t j = (uint32_t)(u1 * (float)n);
    if (j >= n) j = n - 1;
    return u2 < S.light_prob[j] ? j : S.light_alias[j];
}

/* Emissive-triangle NEE; bsdf 0 = Lambert (albedo), 1 = GGX (F0, alpha, frame, wol). */
v3 nee(Ctx &C, uint32_t i, v3 p, v3 n, v3 T, int bsdf, v3 albedo, const onb &F, v3 wol, float alpha,
       Tape *tape = nullptr, uint32_t bsdf_mat = 0, float refl = 1.0f) {
    const Scene &S = *C.S;
    const f4 g = rand4(C.pix, C.sample, 2 + 2 * i, C.set->seed);
    const uint32_t j = pick_light(S, g.x, g.w);
    const uint32_t prim = S.light_prim[j];
    v3 a, b, c;
    tri_verts(S, prim, a, b, c);
    if (S.ninst) {
        const float *F = &S.inst_rows[24 * (size_t)S.light_inst[j] + 12];
        a = xf_point(F, a);
        b = xf_point(F, b);
        c = xf_point(F, c);
    }
    const float su = std::sqrt(g.y);
    const float b0 = 1.0f - su, b1 = su * (1.0f - g.z), b2 = su * g.z;
    const v3 pl = add(add(mul(a, b0), mul(b, b1)), mul(c, b2));
    const v3 po = add(p, mul(n, 1e-4f));
    const v3 w = sub(pl, po);
    const float d2 = dot(w, w);
    if (!(d2 > 0.0f)) return mk(0, 0, 0);
    const float dist = std::sqrt(d2);
    const v3 wi = mul(w, 1.0f / dist);
    const float cos_s = dot(wi, n);
    if (!(cos_s > 0.0f)) return mk(0, 0, 0);
    const v3 Ngl = normalize(cross(sub(b, a), sub(c, a)));
    const float cos_l = absf(dot(Ngl, wi));
    if (!(cos_l > 0.0f)) return mk(0, 0, 0);
    C.shadow++;
    if (occluded(S, po, wi, dist * 0.999f)) return mk(0, 0, 0);
    const crg_material &lm = S.mats[S.mat_idx[prim]];
    const float *lc = lm.colour;
    if (textured(S, lm)) {
        float tu, tv;
        interp_uv(S, prim, b1, b2, tu, tv);
        lc = tex_lookup(S, lm.tex, tu, tv);
    }
    const v3 Le = mk(lc[0] * lm.emission, lc[1] * lm.emission, lc[2] * lm.emission);
    const float p_light = (S.light_pdf[j] * d2) / cos_l;
    v3 f, bsdf_dlog;
    float p_bsdf, cos_i;
    if (bsdf == 0) {
        f = mul(albedo, kInvPi);
        p_bsdf = cos_s * kInvPi;
        cos_i = cos_s;
        bsdf_dlog = inv_or_zero(albedo);
    } else {
        const v3 wil = to_local(F, wi);
        if (!(wil.z > 0.0f)) return mk(0, 0, 0);
        const v3 h = normalize(add(wol, wil));
        const float woh = dot(wol, h);
        const float D = ggx_D(h.z, alpha);
        const float lo_ = ggx_lambda(wol, alpha), li = ggx_lambda(wil, alpha);
        const float G2 = 1.0f / ((1.0f + lo_) + li);
        const float G1 = 1.0f / (1.0f + lo_);
        float m5;
        const v3 Fr = schlick(albedo, woh, &m5);
        f = mul(Fr, (D * G2) / ((4.0f * wol.z) * wil.z));
        p_bsdf = (G1 * D) / (4.0f * wol.z);
        cos_i = wil.z;
        bsdf_dlog = schlick_dlog(Fr, m5, refl);
    }
    const float w_mis = (p_light * p_light) / (p_light * p_light + p_bsdf * p_bsdf);
    const v3 c_out = mul(mulv(mulv(T, f), Le), (cos_i * w_mis) / p_light);
    if (tape) tape->nee(c_out, bsdf_mat, bsdf_dlog, S.mat_idx[prim]);
    return c_out;
}

v3 trace_extended(Ctx &C, v3 o, v3 d, Aov &aov, Tape *tape = nullptr) {
    const Scene &S = *C.S;
    const crg_settings &set = *C.set;
    v3 T = mk(1, 1, 1), L = mk(0, 0, 0);
    float prev_pdf = 0.0f;
    bool prev_delta = true;
    for (uint32_t i = 0; i < set.max_bounces; ++i) {
        crg_hit h;
        uint32_t hinst;
        C.segments++;
        if (!cast(S, o, d, kInf, h, hinst)) {
            const v3 env = sample_sky(S, d);
            if (i == 0) aov.albedo = env;
            L = add(L, mulv(T, env));
            if (tape) tape->env(mulv(T, env));
            break;
        }
        const Geom hg = hit_geom(S, h, hinst, o, d, true);
        const v3 p = hg.p, Ng = hg.Ng;
        const uint32_t mi = S.mat_idx[h.prim];
        const crg_material &m = S.mats[mi];
        float col[4];
        hit_colour(S, m, h, col);
        if (col[3] == 0.0f) {
            o = add(p, mul(d, 0.1f));
            continue;
        }
        const v3 rgb = mk(col[0], col[1], col[2]);
        const float cos_nd = dot(Ng, d);
        const v3 n = cos_nd < 0.0f ? Ng : neg(Ng);
        if (i == 0) {
            aov.albedo = rgb;
            aov.normal = Ng;
            aov.depth = hg.dist;
        }
        if (m.emission > 0.0f) {
            const v3 Le = mk(col[0] * m.emission, col[1] * m.emission, col[2] * m.emission);
            if (prev_delta) {
                L = add(L, mulv(T, Le));
                if (tape) tape->emit(mulv(T, Le), mi);
            } else {
                const float cos_l = absf(cos_nd);
                if (cos_l > 0.0f) {
                    const float pl = (S.mat_light_pdf[mi] * (hg.dist * hg.dist)) / cos_l;
                    const float w = (prev_pdf * prev_pdf) / (prev_pdf * prev_pdf + pl * pl);
                    L = add(L, mul(mulv(T, Le), w));
                    if (tape) tape->emit(mul(mulv(T, Le), w), mi);
                }
            }
        }
        const f4 g = rand4(C.pix, C.sample, 1 + 2 * i, set.seed);
        const v3 wo = neg(d);
        /* NEE at hit i estimates light arriving along segment i + 1, which
         * only exists when i + 1 < max_bounces. */
        const bool have_lights = !S.light_prim.empty() && i + 1 < set.max_bounces;
        if (m.shade_type == CRG_SHADE_SMOOTH) {
            /* Lambert scatters into the hemisphere of the geometric normal
             * whichever side was hit, as the reference does
             * (renderer.cpp:93-97): the same integral, estimated better. */
            const onb F = build_local(Ng);
            if (have_lights) L = add(L, nee(C, i, p, Ng, T, 0, rgb, F, mk(0, 0, 0), 0.0f, tape, mi));
            const v3 l = cos_hemp(g.x, g.y);
            d = from_local(F, l);
            o = add(p, mul(Ng, 1e-4f));
            prev_pdf = l.z * kInvPi;
            prev_delta = false;
            T = mulv(T, rgb);
            if (tape) tape->mult(mi, inv_or_zero(rgb));
        } else if (m.shade_type == CRG_SHADE_METAL) {
            const v3 f0 = mul(rgb, m.reflectiveness);
            const float alpha = m.roughness;
            if (alpha < 1e-4f) {
                d = reflect(d, n);
                o = add(p, mul(n, 1e-4f));
                T = mulv(T, f0);
                prev_delta = true;
                if (tape) tape->mult(mi, inv_or_zero(rgb));
            } else {
                const onb F = build_local(n);
                const v3 wol = to_local(F, wo);
                if (!(wol.z > 0.0f)) break;
                if (have_lights) L = add(L, nee(C, i, p, n, T, 1, f0, F, wol, alpha, tape, mi, m.reflectiveness));
                const v3 hh = sample_vndf(wol, alpha, g.x, g.y);
                const float woh = dot(wol, hh);
                const float k2 = 2.0f * woh;
                const v3 wil = mk(hh.x * k2 - wol.x, hh.y * k2 - wol.y, hh.z * k2 - wol.z);
                if (!(wil.z > 0.0f)) break;
                const float lo_ = ggx_lambda(wol, alpha), li = ggx_lambda(wil, alpha);
                const float G1 = 1.0f / (1.0f + lo_);
                const float G2 = 1.0f / ((1.0f + lo_) + li);
                float m5;
                const v3 Fr = schlick(f0, woh, &m5);
                T = mulv(T, mul(Fr, G2 / G1));
                if (tape) tape->mult(mi, schlick_dlog(Fr, m5, m.reflectiveness));
                prev_pdf = (G1 * ggx_D(hh.z, alpha)) / (4.0f * wol.z);
                prev_delta = false;
                d = from_local(F, wil);
                o = add(p, mul(n, 1e-4f));
            }
        } else {
            const float eta = cos_nd < 0.0f ? 1.0f / m.ior : m.ior;
            const float ci = -dot(d, n);
            float st2;
            const float Fr = fresnel_dielectric(ci, eta, &st2);
            if (g.z < Fr) {
                d = reflect(d, n);
                o = add(p, mul(n, 1e-4f));
            } else {
                const float cic = clampf(ci, 0.0f, 1.0f);
                const float ct = std::sqrt(1.0f - st2);
                d = add(mul(d, eta), mul(n, eta * cic - ct));
                o = add(p, mul(n, -1e-4f));
            }
            T = mulv(T, rgb);
            prev_delta = true;
            if (tape) tape->mult(mi, inv_or_zero(rgb));
        }
        if (set.rr_depth > 0 && i + 1 >= set.rr_depth) {
            const float q = minf(maxf(maxf(T.x, T.y), T.z), 0.95f);
            if (g.w >= q) break;
            T = mk(T.x / q, T.y / q, T.z / q);
        }
    }
    return L;
}

/* Alias table of the weights w (Walker 1977; Vose 1991's two worklists in
 * double, scanned in index order so the table is reproducible). */
void build_alias(const std::vector<double> &w, double total, std::vector<float> &prob_out,
                 std::vector<uint32_t> &alias) {
    const size_t n = w.size();
    std::vector<double> q(n), prob(n, 1.0);
    std::vector<uint32_t> small, large;
    alias.resize(n);
    for (size_t i = 0; i < n; ++i) {
        q[i] = (w[i] * (double)n) / total;
        alias[i] = (uint32_t)i;
        (q[i] < 1.0 ? small : large).push_back((uint32_t)i);
    }
    while (!small.empty() && !large.empty()) {
        const uint32_t l = small.back(), g = large.back();
        small.pop_back();
        large.pop_back();
        prob[l] = q[l];
        alias[l] = g;
        q[g] = (q[g] + q[l]) - 1.0;
        (q[g] < 1.0 ? small : large).push_back(g);
    }
    prob_out.assign(n, 0.0f);
    for (size_t i = 0; i < n; ++i) prob_out[i] = (float)prob[i];
}

/* Inverse of an affine 4x4 (column-major) in double, rounded once to rows
 * [A^-1 | -A^-1 t], followed by the forward rows [A | t] as given. */
void inverse_rows(const float *x, float rows[24]) {
    double a[3][3], t[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) a[r][c] = (double)x[4 * c + r];
        t[r] = (double)x[12 + r];
    }
    double inv[3][3];
    const double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    const double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    const double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    const double det = (a[0][0] * c00 + a[0][1] * c01) + a[0][2] * c02;
    inv[0][0] = c00 / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][0] = c01 / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][0] = c02 / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) rows[4 * r + c] = (float)inv[r][c];
        rows[4 * r + 3] = (float)-((inv[r][0] * t[0] + inv[r][1] * t[1]) + inv[r][2] * t[2]);
        for (int c = 0; c < 3; ++c) rows[12 + 4 * r + c] = x[4 * c + r];
        rows[12 + 4 * r + 3] = x[12 + r];
    }
}

void prepare(const orc_scene_desc &D, Scene &S) {
    /* models: one BVH each, over the model's own triangles (model-local ids) */
    const uint32_t nm = (D.nmodels && D.model_ntri) ? D.nmodels : 1;
    uint32_t first = 0;
    for (uint32_t m = 0; m < nm; ++m) {
        const uint32_t n = nm == 1 ? D.ntri : D.model_ntri[m];
        orc_bvh *b = nullptr;
        orc_bvh_build(D.verts + (size_t)first * 9, n, D.build, &b);
        S.bvhs.push_back(b);
        S.mfirst.push_back(first);
        first += n;
    }
    S.bvh = S.bvhs[0];
    S.verts = D.verts;
    S.mat_idx = D.mat_idx;
    S.mats = D.mats;
    S.nmat = D.nmat;
    S.sky = (D.skybox && D.sky_w && D.sky_h) ? D.skybox : nullptr;
    S.sky_w = D.sky_w;
    S.sky_h = D.sky_h;
    S.sky_rot_u = D.sky_rot_u;
    S.sky_rot_v = D.sky_rot_v;
    S.sun_on = D.sun_enabled != 0;
    S.sun = D.sun;
    S.uvs = D.uvs;
    S.ntex = (D.tex_rgba && D.tex_w && D.tex_h) ? D.ntex : 0;
    S.tex_rgba = D.tex_rgba;
    S.tex_w = D.tex_w;
    S.tex_h = D.tex_h;
    /* registry.cpp:44-48: sun frame = build_local(-direction) */
    S.sun_frame = build_local(mk(-D.sun.direction[0], -D.sun.direction[1], -D.sun.direction[2]));
    S.sun_cos = (float)std::cos((double)D.sun.size);
    S.sun_pdf = 1.0f / (kTau * (1.0f - S.sun_cos));
    /* emissive triangles, power weighted (area x luminance) */
    std::vector<double> lum(D.nmat, 0.0);
    for (uint32_t m = 0; m < D.nmat; ++m) {
        const crg_material &mm = D.mats[m];
        if (mm.emission > 0.0f) {
            const float r = mm.colour[0] * mm.emission, g = mm.colour[1] * mm.emission, b = mm.colour[2] * mm.emission;
            lum[m] = 0.2126 * (double)r + 0.7152 * (double)g + 0.0722 * (double)b;
        }
    }
    /* instances: inverse rows formed in double and rounded once; the emitter
     * table holds one entry per (instance, emissive triangle), instance-major,
     * weighed by the world area */
    /* placements: a scene of one model without instances is traced as is;
     * otherwise every model contributes its instances in order (one identity
     * instance when it has none, the registry's default, registry.cpp:73-74) */
    static const float kId[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    std::vector<const float *> pxf;
    if (nm == 1 && D.nmodels <= 1 && !(D.model_ninst && D.model_ninst[0])) {
        for (uint32_t j = 0; D.xforms && j < D.ninst; ++j) {
            pxf.push_back(D.xforms + 16 * (size_t)j);
            S.place_model.push_back(0);
        }
    } else {
        const float *x = D.xforms;
        for (uint32_t m = 0; m < nm; ++m) {
            /* without per-model counts every model takes the one list (crg_scene_set_instances) */
            if (!D.model_ninst) x = D.xforms;
            const uint32_t k = D.model_ninst ? D.model_ninst[m] : (D.xforms ? D.ninst : 0);
            if (k == 0) {
                pxf.push_back(kId);
                S.place_model.push_back(m);
            }
            for (uint32_t j = 0; j < k; ++j, x += 16) {
                pxf.push_back(x);
                S.place_model.push_back(m);
            }
        }
    }
    S.ninst = (uint32_t)pxf.size();
    S.inst_rows.assign(24 * (size_t)S.ninst, 0.0f);
    for (uint32_t j = 0; j < S.ninst; ++j) inverse_rows(pxf[j], &S.inst_rows[24 * (size_t)j]);
    std::vector<double> w;
    double total = 0.0;
    const uint32_t ncopy = S.ninst ? S.ninst : 1;
    for (uint32_t j = 0; j < ncopy; ++j) {
        const uint32_t mj = S.ninst ? S.place_model[j] : 0;
        const uint32_t p0 = S.ninst ? S.mfirst[mj] : 0;
        const uint32_t p1 = S.ninst ? (mj + 1 < nm ? S.mfirst[mj + 1] : D.ntri) : D.ntri;
        for (uint32_t p = p0; p < p1; ++p) {
            const uint32_t m = D.mat_idx[p];
            if (!(lum[m] > 0.0)) continue;
            double wv[3][3];
            for (int k = 0; k < 3; ++k) {
                const float *v = D.verts + (size_t)p * 9 + 3 * k;
                for (int r = 0; r < 3; ++r) {
                    if (S.ninst) {
                        const float *x = pxf[j];
                        wv[k][r] = (((double)x[r] * v[0] + (double)x[4 + r] * v[1]) + (double)x[8 + r] * v[2]) +
                                   (double)x[12 + r];
                    } else {
                        wv[k][r] = (double)v[r];
                    }
                }
            }
            double e1[3], e2[3];
            for (int a = 0; a < 3; ++a) {
                e1[a] = wv[1][a] - wv[0][a];
                e2[a] = wv[2][a] - wv[0][a];
            }
            const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                         cz = e1[0] * e2[1] - e1[1] * e2[0];
            const double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
            const double wt = area * lum[m];
            S.light_prim.push_back(p);
            S.light_inst.push_back(j);
            w.push_back(wt);
            total += wt;
        }
    }
    S.mat_light_pdf.assign(D.nmat, 0.0f);
    if (!(total > 0.0)) {
        S.light_prim.clear();
        return;
    }
    for (size_t j = 0; j < w.size(); ++j) S.light_pdf.push_back((float)(lum[D.mat_idx[S.light_prim[j]]] / total));
    build_alias(w, total, S.light_prob, S.light_alias);
    for (uint32_t m = 0; m < D.nmat; ++m) S.mat_light_pdf[m] = (float)(lum[m] / total);
}

} // namespace

extern "C" {

void orc_sincos2pi(float u, float *s, float *c) { sincos2pi(u, s, c); }

void orc_rand4(uint32_t pixel, uint32_t sample, uint32_t group, uint32_t seed, float *out4) {
    const f4 r = rand4(pixel, sample, group, seed);
    out4[0] = r.x;
    out4[1] = r.y;
    out4[2] = r.z;
    out4[3] = r.w;
}

void orc_camera_ray(const crg_camera *cam, const crg_settings *set, uint32_t px, uint32_t py, float jx, float jy,
                    float *org, float *dir) {
    const CamParams cp = camera_params(*cam);
    const float x = ((float)px + jx) / (float)set->width;
    const float y = ((float)py + jy) / (float)set->height;
    v3 o, d;
    camera_ray(cp, x, y, set->aspect, o, d);
    org[0] = o.x; org[1] = o.y; org[2] = o.z;
    dir[0] = d.x; dir[1] = d.y; dir[2] = d.z;
}

int orc_render_rows(const orc_scene_desc *desc, const crg_camera *cam, const crg_settings *set, orc_film *film,
                    uint32_t y0, uint32_t y1, int nthreads) {
    if (!desc || !cam || !set || !film || !film->sum_rgb) return CRG_ERR_INVALID_ARG;
    if (set->width != film->width || set->height != film->height) return CRG_ERR_INVALID_ARG;
    if (y1 > set->height) y1 = set->height;
    Scene S;
    prepare(*desc, S);
    const CamParams cp = camera_params(*cam);
    const uint32_t W = set->width, H = set->height;
    const uint64_t npix = (uint64_t)W * (y1 > y0 ? (y1 - y0) : 0);
    std::atomic<uint64_t> seg{0}, shad{0};
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::atomic<uint64_t> next{0};
    auto work = [&]() {
        uint64_t my_seg = 0, my_sh = 0;
        for (;;) {
            const uint64_t s0 = next.fetch_add(64);
            if (s0 >= npix) break;
            const uint64_t e0 = std::min<uint64_t>(npix, s0 + 64);
            for (uint64_t q = s0; q < e0; ++q) {
                const uint32_t px = (uint32_t)(q % W), py = y0 + (uint32_t)(q / W);
                const uint32_t pix = py * W + px;
                const uint64_t fidx = (uint64_t)(W - 1 - px) + (uint64_t)(H - 1 - py) * W;
                float acc[3] = {film->sum_rgb[fidx * 3], film->sum_rgb[fidx * 3 + 1], film->sum_rgb[fidx * 3 + 2]};
                Aov aov;
                for (uint32_t s = 0; s < set->spp; ++s) {
                    Ctx C{&S, set, pix, (uint32_t)(film->spp + s)};
                    const f4 g0 = rand4(pix, C.sample, 0, set->seed);
                    const float x = ((float)px + g0.x) / (float)W;
                    const float y = ((float)py + g0.y) / (float)H;
                    v3 o, d;
                    camera_ray(cp, x, y, set->aspect, o, d);
                    aov = Aov();
                    const v3 L = set->mode == CRG_MODE_EXTENDED ? trace_extended(C, o, d, aov)
                                                                : trace_faithful(C, o, d, aov);
                    acc[0] += L.x;
                    acc[1] += L.y;
                    acc[2] += L.z;
                    if (film->sum64) {
                        film->sum64[fidx * 3] += (double)L.x;
                        film->sum64[fidx * 3 + 1] += (double)L.y;
                        film->sum64[fidx * 3 + 2] += (double)L.z;
                    }
                    if (film->sumsq64) {
                        film->sumsq64[fidx * 3] += (double)L.x * (double)L.x;
                        film->sumsq64[fidx * 3 + 1] += (double)L.y * (double)L.y;
                        film->sumsq64[fidx * 3 + 2] += (double)L.z * (double)L.z;
                    }
                    my_seg += C.segments;
                    my_sh += C.shadow;
                }
                film->sum_rgb[fidx * 3] = acc[0];
                film->sum_rgb[fidx * 3 + 1] = acc[1];
                film->sum_rgb[fidx * 3 + 2] = acc[2];
                if (set->spp > 0) {
                    /* renderer.cpp:367-369 */
                    if (film->aov_albedo) {
                        float *t = film->aov_albedo + fidx * 4;
                        t[0] = aov.albedo.x; t[1] = aov.albedo.y; t[2] = aov.albedo.z; t[3] = 1.0f;
                    }
                    if (film->aov_normal) {
                        float *t = film->aov_normal + fidx * 4;
                        t[0] = aov.normal.x * 0.5f + 0.5f;
                        t[1] = aov.normal.y * 0.5f + 0.5f;
                        t[2] = aov.normal.z * 0.5f + 0.5f;
                        t[3] = 1.0f;
                    }
                    if (film->aov_depth) {
                        float *t = film->aov_depth + fidx * 4;
                        const float dv = minf(aov.depth, 200.0f) / 200.0f;
                        t[0] = dv; t[1] = dv; t[2] = dv; t[3] = 1.0f;
                    }
                }
            }
        }
        seg += my_seg;
        shad += my_sh;
    };
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work);
    for (auto &t : th) t.join();
    film->render_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    film->segments += seg.load();
    film->shadow_rays += shad.load();
    return CRG_OK;
}

int orc_adjoint(const orc_scene_desc *desc, const crg_camera *cam, const crg_settings *set, const float *adj,
                double *grad_colour, double *grad_emission, int nthreads) {
    if (!desc || !cam || !set || !adj || !grad_colour || !grad_emission) return CRG_ERR_INVALID_ARG;
    if (set->mode != CRG_MODE_EXTENDED) return CRG_ERR_UNSUPPORTED;
    Scene S;
    prepare(*desc, S);
    const CamParams cp = camera_params(*cam);
    const uint32_t W = set->width, H = set->height, nmat = desc->nmat;
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::vector<double>> gc(nthreads, std::vector<double>(3 * (size_t)nmat, 0.0)),
        ge(nthreads, std::vector<double>(nmat, 0.0));
    std::atomic<uint64_t> next{0};
    const uint64_t npix = (uint64_t)W * H;
    auto work = [&](int tid) {
        Tape tape;
        tape.mats = desc->mats;
        tape.g_col = gc[tid].data();
        tape.g_em = ge[tid].data();
        for (;;) {
            const uint64_t q = next.fetch_add(1);
            if (q >= npix) break;
            const uint32_t px = (uint32_t)(q % W), py = (uint32_t)(q / W);
            const uint32_t pix = py * W + px;
            const uint64_t fidx = (uint64_t)(W - 1 - px) + (uint64_t)(H - 1 - py) * W;
            const double inv = 1.0 / (double)set->spp;
            tape.dx = (double)adj[fidx * 3] * inv;
            tape.dy = (double)adj[fidx * 3 + 1] * inv;
            tape.dz = (double)adj[fidx * 3 + 2] * inv;
            if (tape.dx == 0.0 && tape.dy == 0.0 && tape.dz == 0.0) continue;
            for (uint32_t s = 0; s < set->spp; ++s) {
                Ctx C{&S, set, pix, s};
                const f4 g0 = rand4(pix, s, 0, set->seed);
                const float x = ((float)px + g0.x) / (float)W;
                const float y = ((float)py + g0.y) / (float)H;
                v3 o, d;
                camera_ray(cp, x, y, set->aspect, o, d);
                Aov aov;
                tape.mat.clear();
                tape.dlog.clear();
                trace_extended(C, o, d, aov, &tape);
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(work, t);
    for (auto &t : th) t.join();
    for (int t = 0; t < nthreads; ++t) {
        for (size_t k = 0; k < 3 * (size_t)nmat; ++k) grad_colour[k] += gc[t][k];
        for (size_t k = 0; k < nmat; ++k) grad_emission[k] += ge[t][k];
    }
    return CRG_OK;
}

int orc_render(const orc_scene_desc *desc, const crg_camera *cam, const crg_settings *set, orc_film *film,
               int nthreads) {
    const int rc = orc_render_rows(desc, cam, set, film, 0, set ? set->height : 0, nthreads);
    if (rc == CRG_OK) film->spp += set->spp;
    return rc;
}

/* Draft preview (cr::draft_renderer, draft_renderer.cpp:150-271): the unlit
 * colour of the nearest surface at each pixel centre, within the
 * rasteriser's near / far planes, over the skybox; film pixel layout. */
int orc_draft_render(const orc_scene_desc *desc, const crg_camera *cam, uint32_t w, uint32_t h, float aspect,
                     float *rgba) {
    if (!desc || !cam || !rgba || w == 0 || h == 0) return CRG_ERR_INVALID_ARG;
    Scene S;
    prepare(*desc, S);
    const CamParams cp = camera_params(*cam);
    const v3 fwd = mk(cp.R[0][2], cp.R[1][2], cp.R[2][2]);
    const float zn = cam->mode == CRG_CAMERA_ORTHOGRAPHIC ? 0.01f : 0.1f;
    for (uint32_t py = 0; py < h; ++py)
        for (uint32_t px = 0; px < w; ++px) {
            const float x = ((float)px + 0.5f) / (float)w, y = ((float)py + 0.5f) / (float)h;
            v3 o, d;
            camera_ray(cp, x, y, aspect, o, d);
            const float cz = dot(d, fwd);
            crg_hit hit;
            uint32_t inst = kNoInst;
            float c[4];
            if (cz > 0.0f && cast_query(S, o, d, zn / cz, 10000.0f / cz, hit, inst)) {
                const crg_material &m = S.mats[S.mat_idx[hit.prim]];
                hit_colour(S, m, hit, c);
                if (!textured(S, m)) c[3] = 1.0f;
            } else {
                const v3 e = sample_sky(S, d);
                c[0] = e.x;
                c[1] = e.y;
                c[2] = e.z;
                c[3] = 1.0f;
            }
            float *out = rgba + ((size_t)(w - 1 - px) + (size_t)(h - 1 - py) * w) * 4;
            for (int k = 0; k < 4; ++k) out[k] = c[k];
        }
    return CRG_OK;
}

void orc_alias_table(const double *w, uint32_t n, float *prob, uint32_t *alias) {
    std::vector<double> ww(w, w + n);
    double total = 0.0;
    for (uint32_t i = 0; i < n; ++i) total += w[i];
    std::vector<float> p;
    std::vector<uint32_t> a;
    build_alias(ww, total, p, a);
    for (uint32_t i = 0; i < n; ++i) {
        prob[i] = p[i];
        alias[i] = a[i];
    }
}

int orc_scene_intersect(const orc_scene_desc *desc, const crg_ray *rays, crg_hit *hits, uint32_t *occluded,
                        uint64_t n) {
    if (!desc || !rays || (!hits && !occluded)) return CRG_ERR_INVALID_ARG;
    Scene S;
    prepare(*desc, S);
    for (uint64_t i = 0; i < n; ++i) {
        const crg_ray &r = rays[i];
        const v3 o = mk(r.org[0], r.org[1], r.org[2]), d = mk(r.dir[0], r.dir[1], r.dir[2]);
        if (occluded) {
            occluded[i] = occluded_query(S, o, d, r.tmin, r.tmax) ? 1u : 0u;
            continue;
        }
        crg_hit h;
        uint32_t inst;
        if (cast_query(S, o, d, r.tmin, r.tmax, h, inst)) {
            if (inst != kNoInst) {
                v3 oo, od;
                float len;
                inst_ray(S, inst, o, d, oo, od, len);
                h.t = vdist(inst_point(S, inst, oo, od, h.t), o);
            }
            hits[i] = h;
        } else {
            hits[i] = crg_hit{kInf, 0xFFFFFFFFu, 0.0f, 0.0f};
        }
    }
    return CRG_OK;
}

/* The faithful estimator's sun sample: direction, pdf and cosine with the
 * normal, from a sun (crg_sun's direction and size) and the two uniforms. */
void orc_sun_sample(const crg_sun *sun, const float *normal3, float u1, float u2, float *dir3, float *pdf, float *cosine) {
    const onb F = build_local(mk(-sun->direction[0], -sun->direction[1], -sun->direction[2]));
    const float sun_cos = (float)std::cos((double)sun->size);
    const v3 d = sun_direction(F, sun_cos, u1, u2);
    dir3[0] = d.x; dir3[1] = d.y; dir3[2] = d.z;
    *pdf = 1.0f / (kTau * (1.0f - sun_cos));
    *cosine = clampf(dot(mk(normal3[0], normal3[1], normal3[2]), d), 0.0f, 1.0f);
}
/* The faithful estimator's sun disc test (dot(d, -sun.direction) > cos(size)). */
int orc_sun_visible(const crg_sun *sun, const float *dir3) {
    const v3 ms = mk(-sun->direction[0], -sun->direction[1], -sun->direction[2]);
    return dot(mk(dir3[0], dir3[1], dir3[2]), ms) > (float)std::cos((double)sun->size) ? 1 : 0;
}
void orc_cos_hemp(float x, float y, float *out3) {
    const v3 v = cos_hemp(x, y);
    out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}

/* Sampling helpers exported for known-answer and distribution tests. */
void orc_sample_sphere(float u1, float u2, float *out3) {
    const v3 v = sphere(u1, u2);
    out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}
void orc_build_local(const float *n3, float *t3, float *b3) {
    const onb F = build_local(mk(n3[0], n3[1], n3[2]));
    t3[0] = F.t.x; t3[1] = F.t.y; t3[2] = F.t.z;
    b3[0] = F.b.x; b3[1] = F.b.y; b3[2] = F.b.z;
}
float orc_ggx_d(float nh, float alpha) { return ggx_D(nh, alpha); }
float orc_ggx_lambda(const float *w3, float alpha) { return ggx_lambda(mk(w3[0], w3[1], w3[2]), alpha); }
void orc_sample_vndf(const float *wo3, float alpha, float u1, float u2, float *h3) {
    const v3 h = sample_vndf(mk(wo3[0], wo3[1], wo3[2]), alpha, u1, u2);
    h3[0] = h.x; h3[1] = h.y; h3[2] = h.z;
}
float orc_fresnel_dielectric(float ci, float eta) {
    float st2;
    return fresnel_dielectric(ci, eta, &st2);
}

} /* extern "C" */
