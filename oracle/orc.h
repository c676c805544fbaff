/*
 * orc.h — CPU oracle of the render hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A C++ restatement, for checking the GB300 kernels, of:
 *   - CRender's integrator (src/render/renderer.cpp:21-102, 258-384), its
 *     sampling helpers (src/util/sampling.h:21-183) and camera
 *     (src/render/camera.cpp:14-68) — the "faithful" estimator;
 *   - the extensions the GPU path adds (emissive-triangle NEE with MIS, GGX,
 *     Fresnel dielectric, Russian roulette) — the "extended" estimator;
 *   - the acceleration structure that replaces Embree 3 (rtcCommitScene /
 *     rtcIntersect1, src/objects/model.cpp:5-97): a Karras (2012) LBVH with
 *     optional Karras & Aila (2013) treelet restructuring, collapsed to a
 *     quantized wide BVH, and the Woop/Benthin/Wald (2013) watertight
 *     ray/triangle test.
 *
 * Parity status: the reference ships no tests, golden vectors or fixtures, and
 * it cannot be built here (Embree 3, TBB, OIDN, glm and GLFW are absent), so
 * this oracle is PARITY UNPINNED against the reference itself.  It is pinned
 * instead by analytic known answers (furnace and ray/triangle cases), an FP64
 * brute-force intersector, and golden fixtures generated from it.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * this library; the product never does.
 */
#ifndef ORC_H
#define ORC_H

#include "../include/crg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_bvh orc_bvh;

/* Builds the LBVH (+ optional treelets) and its wide collapse on the CPU. */
int orc_bvh_build(const float *verts, uint32_t ntri, const crg_build_opts *opts, orc_bvh **out);
void orc_bvh_free(orc_bvh *b);
void orc_bvh_info(const orc_bvh *b, crg_bvh_info *info);
/* Same layouts as crg_scene_bvh_download. */
void orc_bvh_download(const orc_bvh *b, float *bvh2, uint32_t *order, void *wide, float *tris);

/* Closest / any hit through the binary LBVH with the watertight test.
 * nthreads <= 0 means all hardware threads. */
void orc_intersect_closest(const orc_bvh *b, const crg_ray *rays, crg_hit *hits, uint64_t n, int nthreads);
void orc_intersect_any(const orc_bvh *b, const crg_ray *rays, uint32_t *occluded, uint64_t n, int nthreads);
/* Brute force over all triangles, with the same FP32 watertight test. */
void orc_intersect_closest_brute(const float *verts, uint32_t ntri, const crg_ray *rays, crg_hit *hits,
                                 uint64_t n);
/* FP64 brute force (Moller-Trumbore in double) for classifying ties: returns t64
 * and the prim, plus min distance of the hit to a triangle edge in barycentric
 * units (edge_dist). */
void orc_intersect_closest_f64(const float *verts, uint32_t ntri, const crg_ray *rays, double *t64,
                               uint32_t *prim, double *edge_dist, uint64_t n);

/* ---- rendering ---- */
typedef struct orc_scene_desc {
    const float *verts;      /* ntri*9 */
    uint32_t ntri;
    const uint32_t *mat_idx; /* ntri */
    const crg_material *mats;
    uint32_t nmat;
    const float *skybox;     /* RGBA [h][w][4] or NULL */
    uint32_t sky_w, sky_h;
    float sky_rot_u, sky_rot_v;
    int sun_enabled;
    crg_sun sun;
    const crg_build_opts *build; /* BVH options (NULL = defaults) */
    const float *uvs;            /* ntri*6 per-corner texture coordinates, or NULL */
    uint32_t ntex;               /* textures (crg_scene_set_textures) */
    const float *const *tex_rgba;
    const uint32_t *tex_w, *tex_h;
    const float *xforms;         /* ninst*16 column-major affine transforms (crg_scene_set_instances), or NULL;
                                    with models: every model's list, concatenated in model order */
    uint32_t ninst;
    /* models (crg_scene_add_model): nmodels consecutive primitive ranges of
     * model_ntri[m] triangles, model m with model_ninst[m] transforms (0 = one
     * identity instance; model_ninst = NULL: every model takes the xforms
     * list, as crg_scene_set_instances gives it); nmodels = 0 or model_ntri =
     * NULL: one model */
    uint32_t nmodels;
    const uint32_t *model_ntri;
    const uint32_t *model_ninst;
} orc_scene_desc;

typedef struct orc_film {
    uint32_t width, height;
    float *sum_rgb;     /* W*H*3, accumulated into (not cleared) */
    double *sum64;      /* optional */
    double *sumsq64;    /* optional */
    float *aov_albedo;  /* optional W*H*4 */
    float *aov_normal;
    float *aov_depth;
    uint64_t spp;       /* in: samples already accumulated (sample index offset); out: += spp */
    uint64_t segments;  /* out: segments traced (reference ray count) */
    uint64_t shadow_rays;
    double render_seconds; /* out: wall time of the pixel loop (BVH build excluded) */
} orc_film;

int orc_render(const orc_scene_desc *scene, const crg_camera *cam, const crg_settings *set, orc_film *film,
               int nthreads);
/* Renders only pixels [y0, y1) of each row range (used for bounded CPU timing). */
int orc_render_rows(const orc_scene_desc *scene, const crg_camera *cam, const crg_settings *set,
                    orc_film *film, uint32_t y0, uint32_t y1, int nthreads);

/* FP64 gradient of sum_p <adj[p], mean of spp samples> (extended estimator,
 * samples 0..spp-1 under set->seed) w.r.t. every material's colour and
 * emission, accumulated into grad_colour[nmat*3] and grad_emission[nmat]. */
int orc_adjoint(const orc_scene_desc *scene, const crg_camera *cam, const crg_settings *set, const float *adj,
                double *grad_colour, double *grad_emission, int nthreads);

/* Post-processing (bloom, gray scale, tone mapping) of an RGBA32F image
 * [h][w][4], restating cr::post_processor::process step by step
 * (src/render/post/post_processor.cpp:110-307). */
int orc_post_process(const float *src, float *dst, uint32_t w, uint32_t h, const crg_post_settings *s);

/* Batched queries on a scene description, instances included (the semantics
 * of crg_intersect_closest / crg_intersect_any): hits (t = world distance) or,
 * when occluded is non-NULL, any-hit flags. */
int orc_scene_intersect(const orc_scene_desc *scene, const crg_ray *rays, crg_hit *hits, uint32_t *occluded,
                        uint64_t n);

/* Draft preview (crg_draft_render semantics) into rgba[h*w*4]. */
int orc_draft_render(const orc_scene_desc *scene, const crg_camera *cam, uint32_t w, uint32_t h, float aspect,
                     float *rgba);

/* The emitter alias table of weights w[n] (for unit tests). */
void orc_alias_table(const double *w, uint32_t n, float *prob, uint32_t *alias);

/* Camera ray of pixel (px, py) with jitter (jx, jy) (for unit tests). */
void orc_camera_ray(const crg_camera *cam, const crg_settings *set, uint32_t px, uint32_t py, float jx,
                    float jy, float *org, float *dir);
/* Scalar helpers exported for known-answer tests. */
void orc_sincos2pi(float u, float *s, float *c);
void orc_rand4(uint32_t pixel, uint32_t sample, uint32_t group, uint32_t seed, float *out4);
uint32_t orc_morton3(float x, float y, float z); /* x,y,z already in [0,1024) */
/* Sampling helpers of the estimators (for distribution tests): uniform sphere
 * (sampling.h:156-166), orthonormal frame around a unit normal (sampling.h:21-33),
 * GGX D and Smith Lambda in the local frame (sampling.h:93-140), visible-normal
 * sampling (Heitz 2018), exact unpolarised dielectric Fresnel (eta = n_i / n_t). */
void orc_sample_sphere(float u1, float u2, float *out3);
void orc_build_local(const float *n3, float *t3, float *b3);
float orc_ggx_d(float nh, float alpha);
float orc_ggx_lambda(const float *w3, float alpha);
void orc_sample_vndf(const float *wo3, float alpha, float u1, float u2, float *h3);
float orc_fresnel_dielectric(float ci, float eta);
/* The faithful estimator's sun sample (sampling.h:72-80 with the registry's
 * sun frame): direction, pdf and clamped cosine with normal3, from uniforms
 * (u1, u2); its sun disc test; the extended Lambert's local cosine-weighted
 * direction (sampling.h:174-183).  For the cross-check with the reference's
 * own compiled code (oracle/ref_bridge.cpp). */
void orc_sun_sample(const crg_sun *sun, const float *normal3, float u1, float u2, float *dir3, float *pdf, float *cosine);
int orc_sun_visible(const crg_sun *sun, const float *dir3);
void orc_cos_hemp(float x, float y, float *out3);

#ifdef __cplusplus
}
#endif
#endif
