/*
 * crg.h — C ABI of the GB300 render core (BVH build, closest/any-hit traversal,
 * path-traced rendering with BSDF sampling, next-event estimation and film
 * accumulation).
 *
 * This is the drop-in boundary for CRender's render hot path.  Each entry point
 * names the reference interface it replaces (paths relative to the CRender
 * source tree).  Every call returns a crg_status; nothing throws across the ABI
 * and nothing calls exit().  Device pointers are plain CUDA device addresses;
 * `crg_stream` is a cudaStream_t (NULL = legacy default stream).
 *
 * Threading: a built scene may be queried concurrently from several host
 * threads (queries only read it).  Mutating calls (create/build/destroy,
 * set_skybox, set_sun) need external synchronisation, as the reference only
 * mutates the scene while the renderer is paused (src/render/renderer.cpp:185-192).
 */
#ifndef CRG_H
#define CRG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CRG_ABI_VERSION 1

typedef struct CUstream_st *crg_stream; /* == cudaStream_t */

typedef enum crg_status {
    CRG_OK = 0,
    CRG_ERR_INVALID_ARG = 1, /* null pointer, bad size, bad enum */
    CRG_ERR_OOM = 2,         /* device or host allocation failed */
    CRG_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    CRG_ERR_TIMEOUT = 4,     /* a bounded device wait ran out */
    CRG_ERR_NOT_BUILT = 5,   /* query on a scene whose BVH is not built */
    CRG_ERR_UNSUPPORTED = 6, /* valid request the call does not support (e.g. the adjoint of a textured scene) */
    CRG_ERR_DEVICE = 7       /* a kernel reported an internal error word */
} crg_status;

/* ------------------------------------------------------------------ POD types */

/* One ray, 32 bytes, two float4 loads.  Mirrors the fields the reference fills
 * in RTCRayHit (src/objects/model.cpp:10-27: org, tnear = 1e-5, dir, tfar = +inf). */
typedef struct crg_ray {
    float org[3];
    float tmin;
    float dir[3];
    float tmax;
} crg_ray;

/* Closest-hit record, 16 bytes.  prim = CRG_INVALID_PRIM and t = +inf on a miss.
 * u, v are the barycentrics of vertices 1 and 2 (Embree's convention, used by
 * rtcInterpolate0 at src/objects/model.cpp:39-47). */
typedef struct crg_hit {
    float t;
    uint32_t prim;
    float u;
    float v;
} crg_hit;
#define CRG_INVALID_PRIM 0xFFFFFFFFu

/* Material record; field meaning and defaults follow
 * cr::material::information (src/render/material/material.h:31-41). */
typedef enum crg_shade_type {
    CRG_SHADE_METAL = 0,  /* material.h: metal  */
    CRG_SHADE_SMOOTH = 1, /* material.h: smooth (Lambertian) */
    CRG_SHADE_GLASS = 2   /* material.h: glass  */
} crg_shade_type;

typedef struct crg_material {
    uint32_t shade_type; /* crg_shade_type; default SMOOTH */
    float ior;           /* default 1.5 */
    float roughness;     /* default 0.5 (GGX alpha in the extended estimator) */
    float reflectiveness;/* default 1   */
    float emission;      /* scalar emission, default 0; radiance = colour.rgb * emission */
    float colour[4];     /* RGBA, default (1,1,1,1); alpha 0 = pass-through */
    int32_t tex;         /* texture index into crg_scene_set_textures, -1 = none */
    uint32_t pad_[2];
} crg_material; /* 48 bytes */

/* Sun light; defaults follow cr::entity::sun (src/render/entities/components.h:23-29). */
typedef struct crg_sun {
    float size;         /* angular radius in radians, default pi/48 */
    float intensity;    /* default 100 */
    float direction[3]; /* default normalize(0.8, -1, 0) */
    float colour[3];    /* default (1, 0.9, 0.7) */
} crg_sun;

/* Camera; mirrors cr::camera (src/render/camera.h:12-41): position, Euler
 * rotation in degrees (applied as Ry(x)*Rx(y)*Rz(z), camera.cpp:54-68),
 * vertical fov in degrees, projection mode and orthographic scale. */
typedef enum crg_camera_mode { CRG_CAMERA_PERSPECTIVE = 0, CRG_CAMERA_ORTHOGRAPHIC = 1 } crg_camera_mode;
typedef struct crg_camera {
    float position[3];
    float rotation[3];
    float fov;
    uint32_t mode;
    float scale;
    uint32_t pad_;
} crg_camera;

/* Estimator selection.
 *  FAITHFUL  — the reference estimator of renderer.cpp:21-102 and 258-384
 *              (Lambert via normal+sphere, mirror metal, Fresnel-less glass,
 *              emission folded into throughput, optional sun NEE, no MIS).
 *  EXTENDED  — same path space with emissive-triangle NEE + power-heuristic MIS,
 *              GGX (VNDF) metal, Fresnel dielectric, two-sided shading normal. */
typedef enum crg_mode { CRG_MODE_FAITHFUL = 0, CRG_MODE_EXTENDED = 1 } crg_mode;

typedef struct crg_settings {
    uint32_t width, height; /* film resolution (renderer::set_resolution) */
    uint32_t spp;           /* samples per pixel added by this call */
    uint32_t max_bounces;   /* segments per path (renderer::set_max_bounces) */
    uint32_t rr_depth;      /* Russian roulette from this segment on; 0 = off */
    uint32_t mode;          /* crg_mode */
    uint32_t seed;          /* RNG stream key */
    float aspect;           /* horizontal scale of the image plane; the reference
                               uses 1 until set_resolution() sets W/H (renderer.cpp:199) */
} crg_settings;

/* BVH build options (the knob set the autotuner searches). */
typedef struct crg_build_opts {
    uint32_t width;        /* wide-BVH branching factor: 2, 4 or 8 (default 8) */
    uint32_t treelet;      /* 1 = binned-SAH treelet restructuring passes on the LBVH */
    uint32_t leaf_max;     /* max triangles per wide leaf slot, 1..3 (default 3) */
    uint32_t treelet_rounds; /* restructuring rounds (default 3) */
} crg_build_opts;

/* Film flags. */
#define CRG_FILM_F64 1u  /* also keep FP64 sum and FP64 sum of squares per channel */
#define CRG_FILM_AOV 2u  /* keep first-hit albedo / normal / depth AOVs */

typedef struct crg_context crg_context;
typedef struct crg_scene crg_scene;
typedef struct crg_film crg_film;

/* ------------------------------------------------------------------ context */

/* Creates a context on CUDA device `device` (the thread pool of
 * src/objects/thread_pool.cpp:3-24 is replaced by kernel launches). */
crg_status crg_context_create(int device, crg_context **out);
crg_status crg_context_destroy(crg_context *ctx);
/* Last error message of this context (never NULL): a copy owned by the calling
 * thread, valid until that thread calls crg_last_error_string again. */
const char *crg_last_error_string(const crg_context *ctx);
const char *crg_status_string(crg_status s);
uint32_t crg_abi_version(void);

/* Allocation fault injection, for testing callers' error paths (no reference
 * counterpart: the reference ends the process with cr::exit on any fatal
 * error, src/util/exception.h:9-13).  After crg_debug_fail_allocation(n), the
 * n-th next allocation the library makes (n = 0: the very next one), device or
 * host, fails as if memory were exhausted: the call that made it returns
 * CRG_ERR_OOM with a message naming the injected fault, frees what it had
 * allocated, and leaves its context usable.  The fault fires once, then the
 * hook disarms; n < 0 disarms it.  Process-wide and thread-safe; the GPU is
 * never made to fault.  crg_debug_allocation_stats reports the allocations
 * made since the library loaded, the faults fired, and the countdown (-1 =
 * disarmed); any pointer may be NULL. */
crg_status crg_debug_fail_allocation(int64_t nth);
crg_status crg_debug_allocation_stats(uint64_t *allocations, uint32_t *injected, int64_t *armed);

/* Device memory helpers for callers without their own allocator (no reference
 * counterpart: the reference keeps everything in host memory). */
crg_status crg_device_alloc(crg_context *ctx, size_t bytes, void **dptr);
crg_status crg_device_free(crg_context *ctx, void *dptr);
crg_status crg_memcpy_h2d(crg_context *ctx, void *dst, const void *src, size_t bytes, crg_stream stream);
crg_status crg_memcpy_d2h(crg_context *ctx, void *dst, const void *src, size_t bytes, crg_stream stream);
crg_status crg_stream_sync(crg_context *ctx, crg_stream stream);
/* Page-locked host memory (fast, asynchronous host<->device copies). */
crg_status crg_host_alloc(crg_context *ctx, size_t bytes, void **hptr);
crg_status crg_host_free(crg_context *ctx, void *hptr);

/* ------------------------------------------------------------------ scene */

/* Creates a scene from de-indexed triangles, as cr::registry::register_model
 * stores them after persist_and_expand (src/render/entities/registry.cpp:51-97):
 *   verts   : host float[ntri*9] (v0.xyz v1.xyz v2.xyz per triangle)
 *   uvs     : optional host float[ntri*6] per-corner texture coordinates
 *   mat_idx : host uint32[ntri] per-primitive material index
 *             (cr::entity::model_materials::indices, components.h:82-97)
 *   mats    : host crg_material[nmat]
 * The data are copied to the device; the caller keeps its host arrays.
 * Replaces cr::model::instance_geometry's shared Embree buffers
 * (src/objects/model.cpp:52-97) and the material table of the registry. */
crg_status crg_scene_create(crg_context *ctx, const float *verts, uint32_t ntri, const float *uvs,
                            const uint32_t *mat_idx, const crg_material *mats, uint32_t nmat,
                            crg_scene **out);
/* Same, with verts already resident on the device (float[ntri*9] device pointer). */
crg_status crg_scene_create_device(crg_context *ctx, const float *d_verts, uint32_t ntri,
                                   const uint32_t *mat_idx, const crg_material *mats, uint32_t nmat,
                                   crg_scene **out);
/* Same, from indexed geometry as the OBJ loader returns it
 * (cr::asset_loader::model_data, src/util/asset_loader.cpp:182-303), expanded
 * on the device instead of on the host (persist_and_expand in
 * cr::registry::register_model, src/render/entities/registry.cpp:13-24, 51-66):
 *   positions      host float[npos*3]
 *   vertex_indices host uint32[ntri*3], each < npos
 *   texcoords      optional host float[ntc*2]
 *   tex_indices    optional host int32[ntri*3]; NULL = no texture coordinates;
 *                  -1 or >= ntc gives (0, 0) (the reference would read out of bounds)
 *   mat_idx, mats  as crg_scene_create
 * Triangle p is (positions[vertex_indices[3p + k]], k = 0..2). */
crg_status crg_scene_create_indexed(crg_context *ctx, const float *positions, uint32_t npos,
                                    const uint32_t *vertex_indices, uint32_t ntri, const float *texcoords,
                                    uint32_t ntc, const int32_t *tex_indices, const uint32_t *mat_idx,
                                    const crg_material *mats, uint32_t nmat, crg_scene **out);
crg_status crg_scene_destroy(crg_scene *scene);

/* Builds the acceleration structure: LBVH (Morton codes, radix sort, Karras
 * hierarchy, optional treelet restructuring) collapsed to a compressed wide BVH,
 * one per model (crg_scene_add_model).  Replaces rtcCommitScene
 * (src/objects/model.cpp:94).  Only models whose BVH is missing or was built
 * with other options are (re)built, so adding a model to a built scene builds
 * that model alone.  opts may be NULL (defaults). */
crg_status crg_scene_build(crg_scene *scene, const crg_build_opts *opts, crg_stream stream);

/* Equirectangular skybox, host RGBA32F [h][w][4]; replaces cr::scene::set_skybox
 * and set_skybox_rotation (src/render/scene.cpp:36-65).  A 1x1 image is a
 * constant environment.  w = h = 0 removes it (misses return black). */
crg_status crg_scene_set_skybox(crg_scene *scene, const float *rgba, uint32_t w, uint32_t h,
                                float rot_u, float rot_v);
/* Sun light for the faithful estimator; replaces cr::scene::set_sun_enabled
 * and cr::registry::set_sun (scene.cpp:113-121, registry.cpp:248-256). sun may be NULL (defaults). */
crg_status crg_scene_set_sun(crg_scene *scene, int enabled, const crg_sun *sun);
/* Textures: `count` host RGBA32F images rgba[i] of widths[i] x heights[i]
 * ([h][w][4], cr::image layout), replacing any earlier set.  A material with
 * 0 <= tex < count takes its RGBA colour from texture `tex` at the hit's
 * texture coordinate — the per-corner uvs of crg_scene_create interpolated
 * with the hit's barycentrics, (0, 0) without uvs — by nearest texel with
 * modulo wrap, as process_hit and image::get_uv do (src/render/renderer.cpp:30-35,
 * src/objects/image.h:104-109); alpha 0 there is a pass-through surface.  An
 * emissive textured material emits texture colour x emission.  Other tex
 * values mean "no texture".  count = 0 removes the textures. */
crg_status crg_scene_set_textures(crg_scene *scene, uint32_t count, const float *const *rgba,
                                  const uint32_t *widths, const uint32_t *heights);

/* Instances: `ninst` affine 4x4 transforms, 16 floats each, column-major as
 * glm::mat4 stores them (last row 0 0 0 1), given to EVERY model of the scene
 * (crg_scene_set_model_instances sets one model's list).  Replaces
 * cr::entity::instances::transforms and the per-instance loop of
 * cr::model::intersect (src/objects/model.cpp:99-126, registry.cpp:73-74):
 * a ray is transformed into each instance's object space (origin by
 * inverse(T), direction by inverse(T) and renormalised), traced there with
 * tnear 1e-5, and the hit whose world point T * p is closest to the ray
 * origin wins (ties to the earlier instance).  The faithful estimator keeps
 * the reference's object-space normal (model.cpp maps only the point back);
 * the extended estimator shades with the world-space normal, and its emitter
 * table holds one copy of every emissive triangle per instance, weighed by
 * world area.  Inverses are formed once here (in double), not per ray.
 * ninst = 0 on a scene of one model (the default) traces the mesh as is,
 * without any transform.  The BVHs are not rebuilt.  Instanced batches run
 * the wavefront form without per-lane refill. */
crg_status crg_scene_set_instances(crg_scene *scene, const float *xforms, uint32_t ninst);

/* ------------------------------------------------------------------ models
 *
 * A scene holds one or more models.  Each model is one entity of the
 * reference's registry (cr::registry::register_model,
 * src/render/entities/registry.cpp:51-97): its own triangles, its own BVH
 * (the bottom level) and its own instance list (cr::entity::instances,
 * src/render/entities/components.h:18-21).  Model 0 holds the triangles the
 * scene was created with.  A scene of more than one model, or with an
 * instance list, is traced through its PLACEMENTS, every (model, instance)
 * pair in model order then instance order (a model without a list has one
 * identity instance, the registry's default, registry.cpp:73-74); a top-level
 * tree over their world boxes prunes them, and the answer is that of
 * cr::scene::cast_ray's loop over entities around cr::model::intersect's loop
 * over instances (scene.cpp:79-98, model.cpp:99-126): the hit of smallest
 * world distance |T p - o|, ties to the earlier placement.  Primitive indices
 * (crg_hit::prim, the material table) are scene-wide: a model's triangles
 * follow those of the models added before it. */

/* Appends a model, as cr::scene::add_model -> registry::register_model does:
 * arguments as crg_scene_create (host arrays, copied); its material indices
 * index its own `mats`, which are appended to the scene's material table.
 * *model (may be NULL) receives the model's index.  The scene must be built
 * again (only the new model's BVH is built). */
crg_status crg_scene_add_model(crg_scene *scene, const float *verts, uint32_t ntri, const float *uvs,
                               const uint32_t *mat_idx, const crg_material *mats, uint32_t nmat, uint32_t *model);
/* Same from indexed geometry, expanded on the device (arguments as
 * crg_scene_create_indexed). */
crg_status crg_scene_add_model_indexed(crg_scene *scene, const float *positions, uint32_t npos,
                                       const uint32_t *vertex_indices, uint32_t ntri, const float *texcoords, uint32_t ntc,
                                       const int32_t *tex_indices, const uint32_t *mat_idx, const crg_material *mats,
                                       uint32_t nmat, uint32_t *model);
/* One model's instance list (transforms as crg_scene_set_instances); ninst = 0
 * gives it one identity instance (the mesh as is when it is the scene's only
 * model).  Replaces editing one entity's cr::entity::instances
 * (src/ui/ui.h:1105-1193).  No BVH is rebuilt. */
crg_status crg_scene_set_model_instances(crg_scene *scene, uint32_t model, const float *xforms, uint32_t ninst);
crg_status crg_scene_model_count(const crg_scene *scene, uint32_t *count);

typedef struct crg_model_info {
    uint32_t first_prim;   /* the model's triangles are scene primitives [first_prim, first_prim + ntri) */
    uint32_t ntri;
    uint32_t node_base;    /* first node of its wide BVH in crg_scene_bvh_download's node array */
    uint32_t n_wide_nodes; /* its wide nodes (0 until built) */
    uint32_t depth;
    uint32_t ninst;        /* transforms in its instance list (0 = one identity instance) */
    uint32_t built;        /* 1 when its BVH is current */
    float sah_cost;
} crg_model_info;
crg_status crg_scene_model_info(const crg_scene *scene, uint32_t model, crg_model_info *info);

/* Introspection of the built structure (for parity checks against a CPU build). */
typedef struct crg_bvh_info {
    uint32_t ntri;
    uint32_t width;
    uint32_t n_bvh2_nodes;   /* internal nodes of the binary LBVH (ntri-1, or 0) */
    uint32_t n_wide_nodes;
    uint32_t node_bytes;     /* bytes per wide node */
    uint32_t n_tri_slots;    /* triangles in the wide-BVH triangle array */
    uint32_t depth;          /* wide-BVH depth (levels) */
    float sah_cost;          /* SAH cost of the binary tree (Ci=1.2, Ct=1) */
    uint32_t leaf_max;       /* the build's crg_build_opts::leaf_max */
    uint32_t treelet;        /* the build's crg_build_opts::treelet */
} crg_bvh_info;
crg_status crg_scene_bvh_info(const crg_scene *scene, crg_bvh_info *info);
/* Copies to host: bvh2 = float[n_bvh2_nodes*8] (lo.xyz,left, hi.xyz,right; child
 * ints stored as raw bits, leaves tagged with bit 31), order = uint32[ntri] sorted
 * primitive order, wide = bytes[n_wide_nodes*node_bytes], tris = float[n_tri_slots*12].
 * Any pointer may be NULL.  On a scene of several models the arrays hold every
 * model's structure: model m's binary nodes at 2 * node_base (model-local
 * indices), its order at first_prim (model-local indices), its wide nodes at
 * node_base (child and triangle indices scene-wide, unused nodes zero) and its
 * triangle slots at first_prim (primitive ids scene-wide); n_bvh2_nodes and
 * n_wide_nodes then give the arrays' full length (crg_scene_model_info). */
crg_status crg_scene_bvh_download(const crg_scene *scene, float *bvh2, uint32_t *order, void *wide,
                                  float *tris);

/* ------------------------------------------------------------------ build without allocation */

/* Largest triangle count crg_build_bvh_noalloc accepts. */
#define CRG_NOALLOC_MAX_TRIS 16384u

/* Message of the calling thread's last failed crg_build_bvh_noalloc call
 * ("" after a call that succeeded); that call has no context, so
 * crg_last_error_string does not describe it.  Valid until the thread's next
 * crg_build_bvh_noalloc call. */
const char *crg_noalloc_last_error(void);

/* Builds the same wide BVH as crg_scene_create + crg_scene_build, for callers
 * that cannot allocate device memory themselves: a host application whose own
 * pool owns the GPU's memory, or an interactive loop that must not pay the
 * device-wide synchronisation of cudaMalloc/cudaFree when a model is added.
 * This entry point calls no cudaMalloc, cudaFree or other allocating routine;
 * it runs the same build pipeline as crg_scene_build, with its scratch taken
 * from the fixed array described below.  It has no counterpart in the
 * reference.
 *
 *   d_verts    : device float[ntri*9], de-indexed triangles
 *   ntri       : at most CRG_NOALLOC_MAX_TRIS (larger counts return
 *                CRG_ERR_INVALID_ARG without touching the device)
 *   opts       : as crg_scene_build (NULL = defaults)
 *   d_wide     : device buffer of at least node_bytes * max(1, ntri - 1) bytes,
 *                node_bytes = 80 / 64 / 48 for width 8 / 4 / 2 (wide_bytes
 *                gives its size)
 *   d_tris     : device float[ntri*12] (triangle array in wide-leaf order)
 *   d_order    : device uint32[ntri] (Morton order of the primitives)
 *   info       : optional; filled like crg_scene_bvh_info
 *
 * Scratch (sort keys, tree arrays, collapse levels) lives in one fixed device
 * array inside the library, about 2.5 MB, which every GPU that loads the
 * library holds until the process exits.  All calls share it and it keeps the
 * last call's contents: the call clears what must start at zero, but two calls
 * whose work overlaps on the GPU (different streams or threads at once) race
 * on it and must be serialised by the caller.  The array's device address is
 * looked up (cudaGetSymbolAddress) once per device with that device current:
 * by crg_context_create on its device, else by the first call on a device no
 * context was created on — that first call may load the library's device code
 * and reserve the array (a driver-side allocation and a synchronisation), so
 * make it before any stream capture, or create a context on the device first.
 * The call synchronises `stream` once per BVH level, as crg_scene_build does;
 * when it fails after queueing work it waits for that work to finish before
 * returning.  Errors are described by crg_noalloc_last_error. */
crg_status crg_build_bvh_noalloc(const float *d_verts, uint32_t ntri, const crg_build_opts *opts,
                                 void *d_wide, size_t wide_bytes, float *d_tris, uint32_t *d_order,
                                 crg_bvh_info *info, crg_stream stream);

/* ------------------------------------------------------------------ queries */

/* Batched closest hit.  Replaces cr::scene::cast_ray -> cr::model::intersect
 * -> rtcIntersect1 (src/render/scene.cpp:79-98, src/objects/model.cpp:5-49).
 * d_rays/d_hits are device arrays of n records.  Ties at equal t go to the
 * smaller primitive index. */
crg_status crg_intersect_closest(const crg_scene *scene, const crg_ray *d_rays, crg_hit *d_hits,
                                 uint64_t n, crg_stream stream);
/* Batched any hit (occlusion): d_occluded[i] = 1 if some triangle is hit with
 * tmin < t < tmax.  The reference traces its shadow rays with closest hit
 * (src/render/renderer.cpp:330-345); this is the rtcOccluded1 equivalent. */
crg_status crg_intersect_any(const crg_scene *scene, const crg_ray *d_rays, uint32_t *d_occluded,
                             uint64_t n, crg_stream stream);
/* Instrumented closest hit: also returns per-ray counts of wide nodes visited and
 * triangles tested (device uint32 arrays, may be NULL). */
crg_status crg_intersect_closest_counted(const crg_scene *scene, const crg_ray *d_rays, crg_hit *d_hits,
                                         uint32_t *d_nodes, uint32_t *d_tris, uint64_t n,
                                         crg_stream stream);

/* Traversal schemes of the batched queries (the results are the same):
 *   THREAD: one ray per thread, its group stack in local memory (the default
 *           of crg_intersect_closest / crg_intersect_any);
 *   WARP:   W lanes per ray (W = the BVH width), 32 / W rays per warp: the
 *           ray's node is read with 16-byte vector loads by its lanes into
 *           shared memory, each lane tests one child box, pending triangles
 *           are tested W at a time, and each ray's group stack lives in its
 *           warp's shared memory.  Scenes traced through placements use
 *           THREAD. */
typedef enum crg_traversal { CRG_TRAVERSAL_THREAD = 0, CRG_TRAVERSAL_WARP = 1 } crg_traversal;
/* crg_intersect_closest / crg_intersect_any with an explicit traversal scheme. */
crg_status crg_intersect_closest_with(const crg_scene *scene, const crg_ray *d_rays, crg_hit *d_hits, uint64_t n,
                                      crg_traversal traversal, crg_stream stream);
crg_status crg_intersect_any_with(const crg_scene *scene, const crg_ray *d_rays, uint32_t *d_occluded, uint64_t n,
                                  crg_traversal traversal, crg_stream stream);

/* Reads and clears the scene's device error word, which a kernel sets instead
 * of trapping when a traversal stack would overflow.  Returns CRG_ERR_DEVICE
 * when it was set.  Synchronises with the device. */
crg_status crg_scene_poll_error(crg_scene *scene);

/* ------------------------------------------------------------------ film */

/* Film: FP32 RGB running sum (renderer.h:85 _raw_buffer), pixel (x, y) stored
 * at ((W-1-x) + (H-1-y)*W) as renderer.cpp:358-362 does; optional FP64 sum and
 * sum of squares; optional AOVs (albedo, normal*0.5+0.5, min(depth,200)/200 as
 * renderer.cpp:367-369). */
crg_status crg_film_create(crg_context *ctx, uint32_t width, uint32_t height, uint32_t flags,
                           crg_film **out);
crg_status crg_film_destroy(crg_film *film);
/* Zeroes the sums and the sample count (renderer::start, renderer.cpp:154-170). */
crg_status crg_film_reset(crg_film *film, crg_stream stream);
/* Samples per pixel accumulated so far (renderer::current_sample_count). */
crg_status crg_film_spp(const crg_film *film, uint64_t *spp);
/* Copies to host; any pointer may be NULL.  sum_rgb float[W*H*3]; sum64,
 * sumsq64 double[W*H*3]; aov_* float[W*H*4] RGBA as cr::image stores them. */
crg_status crg_film_download(crg_film *film, float *sum_rgb, double *sum64, double *sumsq64,
                             float *aov_albedo, float *aov_normal, float *aov_depth, crg_stream stream);
/* crg_film_download without the wait: the copies are only enqueued on
 * `stream`, so the downloads of many films cost one synchronisation
 * (crg_stream_sync) instead of one each.  The host arrays must stay valid
 * until the stream has reached them; page-locked arrays (crg_host_alloc) make
 * the copies asynchronous. */
crg_status crg_film_download_async(crg_film *film, float *sum_rgb, double *sum64, double *sumsq64,
                                   float *aov_albedo, float *aov_normal, float *aov_depth, crg_stream stream);
/* Device pointers of the film arrays (valid until crg_film_destroy). */
crg_status crg_film_device_ptrs(crg_film *film, float **sum_rgb, double **sum64, double **sumsq64);
/* Display transform clamp(sum/spp, 0, 1)^(1/2.2) into a device RGBA32F
 * buffer (renderer.cpp:371-383, the image behind renderer::current_progress). */
crg_status crg_film_display(crg_film *film, float *d_rgba, crg_stream stream);

/* ------------------------------------------------------------------ post-processing */

/* Tone-mapping operators of the reference's post-process shader
 * (assets/app/shaders/post_process.comp:49-108, selected by tonemapping_type). */
typedef enum crg_tonemap {
    CRG_TONEMAP_LINEAR = 0,      /* exposure, then gamma */
    CRG_TONEMAP_REINHARD = 1,    /* c / (c + 1), then gamma */
    CRG_TONEMAP_JIM_RICHARD = 2, /* Hejl-Burgess-Dawson filmic curve (gamma built in) */
    CRG_TONEMAP_UNCHARTED = 3    /* Hable's Uncharted 2 curve, white point 11.2, then gamma */
} crg_tonemap;

/* FAITHFUL reproduces two coverage quirks of cr::post_processor:
 *  - its compute dispatches are floor(W/8) x floor(H/8) groups of 8x8
 *    (post_processor.cpp:219-222, 280-283), so pixels with x >= 8*floor(W/8) or
 *    y >= 8*floor(H/8) come out as zero (the cleared target texture);
 *  - the bloom brightness pass visits pixel (i % W, i / H) for i < W*H
 *    (post_processor.cpp:296-307): on a non-square image some pixels are never
 *    thresholded (visits with i / H >= H, an out-of-bounds access in the
 *    reference, are skipped).
 * FULL processes every pixel and thresholds every pixel once. */
typedef enum crg_post_mode { CRG_POST_FAITHFUL = 0, CRG_POST_FULL = 1 } crg_post_mode;

/* Fields and defaults follow cr::post_processor::bloom_settings,
 * gray_scale_settings and tonemapping_settings
 * (src/render/post/post_processor.h:20-40); crg_post_settings_default fills them. */
typedef struct crg_post_settings {
    uint32_t bloom;        /* default 0 */
    float bloom_threshold; /* luminance below which a pixel does not bloom, default 0.7 */
    float bloom_strength;  /* default 1 */
    uint32_t gray_scale;   /* default 0 */
    uint32_t tonemapping;  /* default 0 */
    int32_t tonemap_type;  /* crg_tonemap, default LINEAR; other values leave the colour as is */
    float exposure;        /* default 1 */
    float gamma;           /* default 2.2 */
    uint32_t mode;         /* crg_post_mode, default FAITHFUL */
    uint32_t pad_;
} crg_post_settings; /* 40 bytes */

crg_status crg_post_settings_default(crg_post_settings *settings);

/* Post-processes a device RGBA32F image [height][width][4] (typically the
 * output of crg_film_display) into d_dst (same shape; must not alias d_src).
 * Replaces cr::post_processor::process (src/render/post/post_processor.cpp:110-244)
 * with its OpenGL compute passes restated as CUDA kernels:
 *   bloom      threshold on luminance dot(rgb, (0.2126, 0.7152, 0.0722))
 *              (_brightness, :296-307), then 10 separable 15-tap Gaussian passes
 *              alternating horizontal / vertical (_blur, :246-294; blur.comp),
 *              added with bloom_strength;
 *   gray_scale 0.2126 r + 0.7162 g + 0.0722 b (post_process.comp:110-114, as written);
 *   tonemapping one of crg_tonemap with exposure and gamma.
 * Texels outside the image read as zero.  With no effect enabled the image is
 * copied unchanged, as the reference returns its input.  The blur's two
 * ping-pong images live in a grow-only workspace of the context (2 x W x H x
 * 16 bytes); calls on one context must not overlap. */
crg_status crg_post_process(crg_context *ctx, const float *d_src, float *d_dst, uint32_t width, uint32_t height,
                            const crg_post_settings *settings, crg_stream stream);

/* ------------------------------------------------------------------ draft preview */

/* Draft-mode preview: the unlit colour of the nearest surface at every pixel
 * centre (the material colour, or its texture at the hit's texture coordinate
 * with its alpha) over the skybox, into a device RGBA32F image [height][width][4]
 * in the film's pixel layout.  Replaces cr::draft_renderer::render's OpenGL
 * passes (src/render/draft/draft_renderer.cpp:150-271, draft_mode.vert/.frag,
 * draft_mode_background.comp) with one ray per pixel through the built BVH;
 * the rasteriser's near / far planes (0.1 / 10000 along the view axis, 0.01
 * for orthographic) bound the rays.  `aspect` as crg_settings::aspect. */
crg_status crg_draft_render(crg_scene *scene, const crg_camera *camera, uint32_t width, uint32_t height, float aspect,
                            float *d_rgba, crg_stream stream);

/* ------------------------------------------------------------------ render */

/* Renders settings->spp more samples per pixel into the film with the
 * one-thread-per-pixel megakernel.  Replaces one or more passes of the
 * renderer's management loop (src/render/renderer.cpp:116-144, 240-384).
 * Sample indices continue from the film's current count, so repeated calls
 * draw fresh, reproducible random numbers. */
crg_status crg_render(crg_scene *scene, const crg_camera *camera, const crg_settings *settings,
                      crg_film *film, crg_stream stream);

/* ------------------------------------------------------------------ batched wavefront */

/* One view of a batch: a camera over scenes[scene] with its own resolution,
 * spp, depth, estimator and seed (settings), rendered into its own film. */
typedef struct crg_view {
    uint32_t scene;
    uint32_t pad_;
    crg_camera camera;
    crg_settings settings;
} crg_view;

/* Wavefront knobs (the autotuner's search space besides the BVH width).
 * Zero fields take the defaults. */
typedef struct crg_wavefront_opts {
    uint32_t path_pool;     /* paths in flight (default 134,217,728; at most the chunk's samples;
                               about 156 bytes of path state each) */
    uint32_t chunk_samples; /* samples resolved into the films per chunk (default 134,217,728) */
    uint32_t block_size;    /* threads per block of the persistent kernels: 64, 128 or 256 (default 128) */
    uint32_t fetch;         /* queue entries a warp takes per atomic, multiple of 32 (default 32) */
    uint32_t max_iterations;/* cap on the device-side loop (0 = a bound derived from the batch);
                               reaching it ends the frame with CRG_ERR_TIMEOUT */
    uint32_t count_work;    /* 1 = instrumented kernels: crg_batch_stats_get also reports
                               nodes visited and triangles tested */
    uint32_t host_loop;     /* 1 = drive the loop from the host instead of one graph with a
                               device-side condition (same kernels; for profilers); 2 = the
                               same, timing every stage with CUDA events on the stream
                               (crg_batch_stage_times_get) */
    uint32_t fuse;          /* stage fusion (films are identical for every value; default 1):
                               1 = separate extend / shade / shadow kernels and queues;
                               2 = the shadow test runs inside shade (no shadow queue);
                               3 = extend + shade + shadow in one kernel per bounce */
    uint32_t refill;        /* traversal stages (extend, shadow): 1..32 = per-lane refill: a
                               lane whose ray is done takes a new one as soon as this many
                               lanes of its warp are idle (dynamic fetch; default 16);
                               0xFFFFFFFF = off: each warp takes `fetch` queue entries and
                               runs them to completion */
} crg_wavefront_opts;

/* Renders every view of a batch in one launch of the wavefront form (one CUDA
 * graph per frame with a device-side loop): generate / extend / shade / shadow
 * queues driven by persistent kernels with atomic work fetch.  Films receive
 * exactly the samples crg_render would add (same random numbers, same order):
 * with the same settings the FP32 and FP64 sums are bit-identical to the
 * megakernel's.  AOV planes are not written.  All scenes must be built with the
 * same width and context; films must be distinct.  Replaces the per-pass loop
 * of the renderer (src/render/renderer.cpp:116-144) for many cameras at once.
 * Calls on one context must not overlap (they share its workspace).  This call
 * waits for the batch (crg_render_batch_async does not). */
crg_status crg_render_batch(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views,
                            crg_film *const *films, uint32_t nviews, const crg_wavefront_opts *opts,
                            crg_stream stream);

/* Stream-ordered form of crg_render_batch: enqueues the batch on `stream` and
 * returns without waiting for it, so the host prepares the next batch (or
 * other work) while this one renders.  The instantiated graph of the loop is
 * kept by the context and relaunched for every later batch of the same shape
 * (views, segments, chunks, path pool, options): only the plan it reads is
 * copied, through pinned staging buffers.  Film sample counts advance at
 * once; the films' contents follow the stream.  Errors found on the device
 * (iteration cap, stack overflow) are reported by crg_batch_wait, which also
 * makes crg_batch_stats_get describe the last batch.  Batches of one context
 * must be enqueued on one stream (they share its workspace); the host waits
 * only when it is two batches ahead of the device.  No reference counterpart
 * (the reference's loop, renderer.cpp:116-144, runs one pass at a time). */
crg_status crg_render_batch_async(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views,
                                  crg_film *const *films, uint32_t nviews, const crg_wavefront_opts *opts,
                                  crg_stream stream);
/* Waits for every batch enqueued on ctx; returns the first error among them. */
crg_status crg_batch_wait(crg_context *ctx);

/* Autotuner of the wavefront form.  Renders a reduced copy of the batch (each
 * view's spp scaled down so the trial holds about sample_budget samples, into
 * scratch films) under candidate settings and keeps the fastest by device
 * time: BVH width (the scenes are rebuilt with their build options at each
 * width tried, and left built at the winner), each scene's leaf size, stage
 * fusion, per-lane refill,
 * queue fetch size, block size and path pool, searched one knob at a time
 * from the defaults.  Every candidate renders identical films, so the choice
 * only trades speed.  Results are cached in the context by batch shape. */
typedef struct crg_autotune_opts {
    uint64_t sample_budget; /* samples per trial batch (0 = 134,217,728) */
    uint32_t widths;        /* BVH widths to try, bit mask of 2 | 4 | 8 (0 = keep the scenes' width) */
    uint32_t reuse;         /* 1 = return the cached result for a batch of the same shape */
    uint32_t leaves;        /* leaf sizes (crg_build_opts::leaf_max) to try for each scene on its own,
                               bit mask of 1 << 1 | 1 << 2 | 1 << 3 (0 = keep the scenes' leaf sizes);
                               the scenes are left built with the winners */
    uint32_t pad_;
} crg_autotune_opts;

typedef struct crg_autotune_trial {
    crg_wavefront_opts opts;
    uint32_t width;
    float ms;               /* device time of the trial batch */
    float msamples_per_s;
    uint32_t pad_;
} crg_autotune_trial;

/* No reference counterpart (the reference has no tunable launch shape).
 * Writes the best options to *best and the BVH width to *best_width (scenes
 * are left built at it); up to trials_cap trials to `trials` (may be NULL)
 * and their count to *ntrials (may be NULL; 0 when the cache answered). */
crg_status crg_autotune_batch(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views, uint32_t nviews,
                              const crg_autotune_opts *opts, crg_wavefront_opts *best, uint32_t *best_width,
                              crg_autotune_trial *trials, uint32_t trials_cap, uint32_t *ntrials,
                              crg_stream stream);

/* The context's autotuner cache outlives the process through a text file: one
 * header line, a line naming the device the answers were measured on (name and
 * SM count), then one line per batch shape (shape key, BVH width, the nine
 * crg_wavefront_opts fields, the scenes' leaf sizes).  crg_autotune_cache_save
 * writes every cached answer (an empty cache writes the two header lines).
 * crg_autotune_cache_load adds a file's answers to the cache, replacing
 * answers for the same shapes, and stores how many it read in *count (may be
 * NULL).  A file written on another kind of device reads nothing (CRG_OK,
 * *count = 0): the answers are timings of that device.  A file that cannot be
 * opened or a malformed line fails with CRG_ERR_INVALID_ARG, and then nothing
 * of the file is added. */
crg_status crg_autotune_cache_save(crg_context *ctx, const char *path);
crg_status crg_autotune_cache_load(crg_context *ctx, const char *path, uint32_t *count);

/* ------------------------------------------------------------------ differentiation */

/* Replaces the material table (same count, e.g. after an optimiser step)
 * without rebuilding the BVH; the emitter table is rebuilt.  The reference
 * edits cr::material::information in place while the renderer is paused
 * (src/render/material/material.h:31-41, renderer.cpp:185-192). */
crg_status crg_scene_set_materials(crg_scene *scene, const crg_material *mats, uint32_t nmat);

/* Backward half of a forward/backward pair whose forward half is crg_render
 * (extended estimator): the path-replay adjoint (Vicini, Speierer & Jakob,
 * SIGGRAPH 2021).  Re-traces settings->spp fresh samples per pixel (sample
 * indices 0..spp-1 under settings->seed; use a seed different from the
 * forward pass for an unbiased gradient) and ADDS to
 *   d_grad_colour   device double[nmat*3]: d/d colour of every material
 *   d_grad_emission device double[nmat]  : d/d emission of every material
 * the gradient of sum_p <d_adjoint[p], I[p]>, where I[p] is the pixel's mean
 * radiance over these samples and d_adjoint is a device float[W*H*3] image in
 * film layout (typically dLoss/dI of the forward image).  Random decisions
 * (Russian roulette included) are held fixed, so the result is the exact
 * derivative of the estimator for those samples: it matches central finite
 * differences with common random numbers when roulette is off.  No path is
 * stored.  Requires mode EXTENDED, max_bounces <= 32, sun off. */
crg_status crg_backward(crg_scene *scene, const crg_camera *camera, const crg_settings *settings,
                        const float *d_adjoint, double *d_grad_colour, double *d_grad_emission,
                        crg_stream stream);

/* Image loss of a forward pass, the link between crg_render and crg_backward:
 * with I = film sum / film spp (FP32 sum plane) and T = d_target (device
 * float[W*H*3], film layout),
 *   *d_loss    = mean over the W*H*3 values of (I - T)^2       (device double, overwritten)
 *   d_adjoint  = dLoss/dI = 2 (I - T) / (W*H*3)               (device float[W*H*3], overwritten)
 * No reference counterpart (the reference renderer has no differentiation). */
crg_status crg_film_loss_l2(crg_film *film, const float *d_target, float *d_adjoint, double *d_loss,
                            crg_stream stream);

/* Statistics of the last render on this scene (renderer::current_stats,
 * renderer.cpp:396-404): segments traced (the reference's ray count,
 * renderer.cpp:271-272/356) and shadow rays traced. */
typedef struct crg_render_stats {
    uint64_t samples;
    uint64_t segments;
    uint64_t shadow_rays;
    uint64_t nodes_visited; /* wide nodes loaded by all traversals (counting mode) */
    uint64_t tris_tested;   /* triangles tested by all traversals (counting mode) */
    uint64_t iterations;    /* device-loop iterations of the last batch (wavefront only) */
} crg_render_stats;
crg_status crg_render_stats_get(const crg_scene *scene, crg_render_stats *stats);
/* Statistics of the last crg_render_batch on this context. */
crg_status crg_batch_stats_get(const crg_context *ctx, crg_render_stats *stats);

/* Device time of each stage of the last crg_render_batch run with
 * host_loop = 2 (all zero otherwise), summed over its loop iterations from
 * CUDA events on the launching stream: extend (closest hits), shade, shadow
 * (NEE any hits; zero when fused into shade), and the control / resolve /
 * generate kernels.  With count_work, the shadow stage's share of
 * crg_render_stats::nodes_visited / tris_tested (the rest is extend's).
 * No reference counterpart (the reference's timer, src/render/timer.h, times
 * whole passes). */
typedef struct crg_stage_times {
    double extend_ms, shade_ms, shadow_ms, other_ms;
    uint64_t iterations;
    uint64_t shadow_nodes, shadow_tris;
} crg_stage_times;
crg_status crg_batch_stage_times_get(const crg_context *ctx, crg_stage_times *times);
/* Turn on per-launch counting of segments, shadow rays, nodes visited and
 * triangles tested for crg_render (runs an instrumented kernel variant). */
crg_status crg_scene_set_counting(crg_scene *scene, int enabled);

#ifdef __cplusplus
}
#endif
#endif /* CRG_H */
