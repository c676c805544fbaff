// crg_internal.h — host-side objects behind the C ABI handles.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/crg.h"

namespace crg {
struct BatchState; // wavefront.cu
}

// Device buffer owned by a scene, film or context.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
};

struct crg_context {
    int device = 0;
    std::string last_error;     // guarded by error_mutex: concurrent queries may fail at once
    mutable std::mutex error_mutex;
    int sm_count = 0;
    DevBuf wf_ws; // wavefront workspace (path pool, queues, sample slots), grow-only
    DevBuf post_ws; // post-process ping-pong images, grow-only
    crg_render_stats batch_stats{};
    crg_stage_times stage_times{}; // of the last crg_render_batch run with host_loop 2
    crg::BatchState *batch = nullptr; // wavefront graphs, pinned staging, batches in flight (wavefront.cu)
    struct Tuned {
        crg_wavefront_opts opts;
        uint32_t width;
        std::vector<uint32_t> leaf; // per scene
    };
    std::map<std::string, Tuned> tune_cache; // autotuner results by batch shape
};

// One model of a scene (cr::registry::register_model, src/render/entities/registry.cpp:51-97):
// a contiguous range of the scene's primitives with its own BVH (BLAS) and its
// own instance list (cr::entity::instances::transforms, components.h:18-21).
struct crg_model_rec {
    uint32_t first = 0, ntri = 0; // primitives [first, first + ntri) of the scene arrays
    uint32_t node_base = 0;       // first node of its BVH in the scene's node arrays
    uint32_t node_cap = 1;        // nodes reserved for it: max(1, ntri - 1)
    bool built = false;           // its BVH is current for the scene's build options
    uint32_t n_wide = 0, depth = 0;
    float sah = 0.0f;
    float box[6] = {0, 0, 0, 0, 0, 0}; // object-space bounds of its vertices (lo.xyz, hi.xyz)
    bool box_valid = false;       // box computed (done when the scene first needs placements)
    std::vector<float> xf;        // 16 floats per instance as given; empty = one identity instance
                                  // (the mesh as is when the scene has this one model only)
};

struct crg_scene {
    crg_context *ctx = nullptr;
    uint32_t ntri = 0;
    uint32_t nmat = 0;
    // geometry and materials (original primitive order)
    DevBuf verts;   // float[ntri*9]
    DevBuf mat_idx; // uint32[ntri]
    DevBuf mats;    // crg_material[nmat]
    std::vector<crg_material> host_mats;
    std::vector<uint32_t> host_mat_idx;
    // texture coordinates and textures (cr::image entities referenced by crg_material::tex)
    DevBuf uvs;       // float[ntri*6] per-corner (u, v), primitive order; empty = none
    DevBuf texels;    // float4 texels of all textures, concatenated
    DevBuf tex_info;  // uint4 per texture: {first texel (low 32 bits), first texel (high 32 bits), width, height}
    uint32_t ntex = 0;
    // models (at least one; model 0 holds the triangles the scene was created with)
    std::vector<crg_model_rec> models;
    // placements: every (model, instance) pair in model order then instance
    // order, the order in which cr::scene::cast_ray and cr::model::intersect
    // visit them (scene.cpp:79-98, model.cpp:99-126).  ninst = 0 when the scene
    // is one model without an instance list: the mesh is traced as is.
    uint32_t ninst = 0;
    std::vector<float> host_xf;   // 16 floats per placement (identity for a model without a list)
    std::vector<float> host_rows; // 24 floats per placement (the device layout)
    std::vector<uint32_t> place_model; // model of each placement
    std::vector<double> inst_area; // world area of each placement's triangles, placement-major
    std::vector<size_t> inst_area_off; // first inst_area entry of each placement
    DevBuf inst;       // float4[6 * ninst]
    DevBuf inst_root;  // uint32 per placement: node index of its model's BVH root
    DevBuf tlas;       // float4[4] per top-level node over the placements' world boxes
    uint32_t tlas_root = 0; // top-level root: node index, or kTlasLeaf | placement
    uint32_t tlas_nodes = 0;
    DevBuf light_inst; // uint32 per emitter entry (instanced scenes): its placement
    // emissive triangles (power-weighted alias table)
    uint32_t nlights = 0;
    std::vector<double> tri_area; // per-triangle area (host), for rebuilding the emitter table
    DevBuf light_prim, light_alias, light_pdf, mat_light_pdf; // light_alias: float2 {prob, alias bits}
    DevBuf light_rec; // float4[4] per emitter entry: world corners, pdf, prim, material, radiance
    // environment / sun
    DevBuf sky;
    uint32_t sky_w = 0, sky_h = 0;
    float sky_rot_u = 0, sky_rot_v = 0;
    int sun_enabled = 0;
    crg_sun sun{};
    float sun_frame[9] = {0}; // tangent, normal, bitangent of build_local(-direction)
    float sun_cos = 1.0f, sun_pdf = 0.0f;
    // acceleration structure
    bool built = false;
    crg_build_opts opts{8, 0, 3, 3};
    uint32_t width = 8, node_bytes = 80, n_wide = 0, depth = 0;
    float sah = 0.0f;
    uint32_t node_cap = 0; // sum of the models' node_cap: the node arrays' length
    DevBuf bvh2;   // float4[2*node_cap]: each model's binary LBVH at 2 * node_base, model-local indices
    DevBuf order;  // uint32[ntri]: each model's sorted primitive order at first, model-local indices
    DevBuf wide;   // node_bytes * node_cap: each model's wide BVH at node_base (indices scene-global)
    DevBuf tris;   // float4[3*ntri]: each model's triangle slots at first (primitive ids scene-global)
    DevBuf err;    // uint32 device error word
    DevBuf qhead;  // uint32 work counter of the persistent query kernels
    // statistics
    int counting = 0;
    DevBuf counters; // unsigned long long[4]: samples, segments, shadow rays
    crg_render_stats last_stats{};
};

struct crg_film {
    crg_context *ctx = nullptr;
    uint32_t width = 0, height = 0, flags = 0;
    uint64_t spp = 0;
    DevBuf sum;      // float[W*H*3]
    DevBuf sum64;    // double[W*H*3]
    DevBuf sumsq64;  // double[W*H*3]
    DevBuf aov_albedo, aov_normal, aov_depth; // float[W*H*4]
};

namespace crg {

// Allocation fault injection (crg_debug_fail_allocation): true when the
// allocation about to be made must fail as if the device or host were out of
// memory.  Every allocation site of the library asks once per allocation.
bool fault_injected();

crg_status set_error(crg_context *ctx, crg_status s, const std::string &msg);
crg_status cuda_error(crg_context *ctx, cudaError_t e, const char *what);
crg_status dev_alloc(crg_context *ctx, DevBuf &b, size_t bytes);
void dev_free(DevBuf &b);

// bvh_build.cu
// Builds the BVH of every model that is not built for options o (all of them
// when o differs from the scene's current options).
crg_status build_bvh(crg_scene *s, const crg_build_opts &o, cudaStream_t stream);
// Looks the no-allocation build's scratch array up on the current device
// (called once per context so that crg_build_bvh_noalloc never loads anything).
void noalloc_prepare();

// top-level tree over a scene's placements (crg_api.cu)
constexpr uint32_t kTlasLeaf = 0x80000000u;

// traverse.cu
crg_status launch_intersect(const crg_scene *s, const crg_ray *rays, crg_hit *hits, uint32_t *occluded,
                            uint32_t *nodes, uint32_t *tris, uint64_t n, bool any, cudaStream_t stream,
                            int traversal = CRG_TRAVERSAL_THREAD);

// render.cu
struct CamDev {
    float pos[3];
    float R[9];
    float w;
    uint32_t mode;
    float scale;
};
CamDev camera_params(const crg_camera &c);
crg_status launch_render(crg_scene *s, const CamDev &cam, const crg_settings &set, crg_film *film,
                         cudaStream_t stream);
crg_status build_light_records(crg_scene *s);

// draft.cu
crg_status launch_draft(crg_scene *s, const CamDev &cam, uint32_t w, uint32_t h, float aspect, float *d_rgba,
                        cudaStream_t stream);

// adjoint.cu
crg_status launch_backward(crg_scene *s, const CamDev &cam, const crg_settings &set, const float *adj, double *g_col,
                           double *g_em, cudaStream_t stream);
crg_status launch_loss_l2(crg_film *f, const float *target, float *adj, double *loss, cudaStream_t stream);

// wavefront.cu
// Enqueues a batch on `stream` (wait = false) or runs it to completion (wait = true).
crg_status render_batch(crg_context *ctx, crg_scene *const *scenes, uint32_t nscenes, const crg_view *views,
                        crg_film *const *films, uint32_t nviews, const crg_wavefront_opts &o, cudaStream_t stream,
                        bool wait);
// Waits for the batches enqueued on ctx; the first error among them, and their statistics.
crg_status batch_wait(crg_context *ctx);
void batch_state_free(crg_context *ctx);

} // namespace crg

#define CRG_CUDA(ctx, call)                                                                                            \
    do {                                                                                                               \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess) return crg::cuda_error((ctx), e_, #call);                                               \
    } while (0)
