// crg_host.h — C++ host adapter over the C ABI (include/crg.h) with the
// interface of CRender's cr::scene, cr::camera and cr::renderer, so the code
// that drives the reference renderer (its UI, src/ui/ui.h) keeps calling the
// same names while the samples come from the GB300 kernels.
//
//   crg::host::scene     <- cr::scene    (src/render/scene.h:17-55)
//   crg::host::camera    <- cr::camera   (src/render/camera.h:10-44)
//   crg::host::renderer  <- cr::renderer (src/render/renderer.h:22-111)
//   crg::host::model_data, material_information, image, ray,
//   intersection_record  <- cr::asset_loader::model_data (src/util/asset_loader.h:16-30),
//                           cr::material::information (src/render/material/material.h:31-41),
//                           cr::image (src/objects/image.h), cr::ray (src/render/ray.h:9-35)
//
// The adapter holds no compute of its own: geometry goes to crg_scene_create /
// crg_scene_build, every render pass is one crg_render call on the context's
// stream, and progress / AOV images are film downloads.  Errors from the ABI
// are thrown as crg::host::error carrying crg_last_error_string (the reference
// calls cr::exit instead).  Only this header and include/crg.h are needed to
// use it; link libcrg_host.so and libcrg.so.
#pragma once

#include <array>
#include <atomic>
#include <cmath>
#include <limits>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <functional>
#include <mutex>
#include <optional>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/crg.h"

namespace crg::host {

struct vec2 {
    float x = 0, y = 0;
};
struct vec3 {
    float x = 0, y = 0, z = 0;
};

class error : public std::runtime_error {
public:
    error(crg_status s, const std::string &what) : std::runtime_error(what), status(s) {}
    crg_status status;
};

// cr::material::information without the GL texture plumbing: `tex` indexes
// model_data::textures (sampled on the GPU, crg_scene_set_textures).
struct material_information {
    enum type : unsigned char { metal = CRG_SHADE_METAL, smooth = CRG_SHADE_SMOOTH, glass = CRG_SHADE_GLASS };
    type shade_type = smooth;
    float ior = 1.5f;
    float roughness = 0.5f;
    float reflectiveness = 1.0f;
    float emission = 0.0f;
    float colour[4] = {1, 1, 1, 1};
    std::string name = "ERROR - Report";
    std::optional<uint32_t> tex;
};

// RGBA float image (cr::image layout: width * height * 4).
class image {
public:
    image() = default;
    image(uint64_t width, uint64_t height);
    image(const std::vector<float> &data, uint64_t width, uint64_t height);
    float *data() noexcept { return data_.data(); }
    const float *data() const noexcept { return data_.data(); }
    uint64_t width() const noexcept { return width_; }
    uint64_t height() const noexcept { return height_; }
    bool valid() const noexcept { return width_ != 0 && height_ != 0; }
    // Nearest texel at (u, v) in [0,1]^2, wrapping like cr::image::get_uv.
    vec3 get_uv(float u, float v) const noexcept;

private:
    uint64_t width_ = 0, height_ = 0;
    std::vector<float> data_;
};

struct model_data {
    std::string name;
    std::vector<vec3> vertices;
    std::vector<material_information> materials;
    std::vector<vec2> texture_coords;
    std::vector<vec3> normals;
    std::vector<image> textures;
    std::vector<uint32_t> vertex_indices;   // 3 per triangle
    std::vector<uint32_t> material_indices; // 1 per triangle, into materials
    std::vector<uint32_t> texture_indices;  // 3 per triangle or empty; 0xFFFFFFFF = none
    std::vector<uint32_t> normal_indices;
    std::vector<std::string> texture_names; // map_Kd of each material ("" = none), as the MTL gave them
};

// Loads a Wavefront OBJ (and the MTL files it names, relative to `folder`,
// default the OBJ's own folder) the way cr::asset_loader::load_model does
// through tinyobjloader (src/util/asset_loader.cpp:182-303): positions,
// texture coordinates and normals as listed; faces in file order,
// triangulated (triangles as given, quads split along the shorter diagonal as
// tinyobjloader does, larger polygons as a fan from their first corner);
// 1-based or negative (relative) indices; one material per face from
// `usemtl` (colour = Kd with alpha 1, smooth, no emission).  Faces before any
// `usemtl`, or naming an unknown material, get an extra default material at
// the end of the table (tinyobjloader reports -1 there, which the reference
// would index out of bounds).  Image files named by map_Kd are recorded in
// texture_names but not decoded (no image codec here): the material keeps its
// Kd colour, as the reference does when a texture fails to load.  Throws
// crg::host::error on unreadable files or malformed records.
model_data load_model(const std::string &file, const std::string &folder = "");

struct ray {
    vec3 origin, direction;
};

struct intersection_record {
    uint32_t prim_id = 0; // triangle index in add_model order over all models
    float distance = std::numeric_limits<float>::infinity();
    const material_information *material = nullptr;
    vec2 uv;
    vec3 normal;             // geometric normal (e1 x e2, normalised)
    vec3 intersection_point;
};

class camera {
public:
    enum class mode { perspective, orthographic };
    explicit camera(vec3 position = {5, 5, 0}, float fov = 75, mode camera_mode = mode::perspective);
    // Moves along the camera's own axes: position = M * (t, 1) with M the
    // matrix of the last translate / rotate (camera.cpp:48-52).
    void translate(const vec3 &translation);
    // Adds degrees (yaw about +y, pitch about +x clamped to [-90, 90], roll
    // about +z) and refreshes the matrix (camera.cpp:54-59).
    void rotate(const vec3 &rotation);
    // What a render pass sees: rays use the matrix of the last translate /
    // rotate (identity until the first), as cr::camera::get_ray does.
    crg_camera to_crg() const noexcept;

    float fov;
    float scale = 1.0f;
    mode current_mode;
    vec3 position{};
    vec3 rotation{};

private:
    void update_cache();
    vec3 cached_position_{};
    vec3 cached_rotation_{};
};

class scene {
public:
    // A scene on `device`; owns its crg_context.
    explicit scene(int device = 0);
    ~scene();
    scene(const scene &) = delete;
    scene &operator=(const scene &) = delete;

    // Registers the model (registry.cpp:51-97) as one more model of the
    // library scene, with its own BVH and instance list; at the next render or
    // query it is de-indexed on the device and only its BVH is built
    // (rtcCommitScene's role).  Returns the model's index.
    size_t add_model(const model_data &model);
    // One model's instance transforms (its cr::entity::instances::transforms,
    // edited per entity by the UI, src/ui/ui.h:1105-1193); empty = one
    // identity instance, the registry's default (registry.cpp:73-74).
    void set_model_instances(size_t model, const std::vector<std::array<float, 16>> &transforms);
    size_t model_count() const noexcept { return models_.size(); }
    void set_skybox(image &&skybox);
    void set_skybox_rotation(const vec2 &rotation);
    void set_sun_enabled(bool value);
    void set_sun(const crg_sun &sun);
    vec3 sample_skybox(float x, float y) const noexcept;
    // Closest hit of one ray over all models (scene.cpp:79-98), through
    // crg_intersect_closest.  cast_rays is the batched form.
    intersection_record cast_ray(const ray &r);
    std::vector<intersection_record> cast_rays(const std::vector<ray> &rays);
    class camera *camera() noexcept { return &camera_; }
    vec2 skybox_rotation() const noexcept { return sky_rot_; }
    bool is_sun_enabled() const noexcept { return sun_enabled_; }
    // BVH options used by the next commit (default: width 8, treelets on).
    void set_build_options(const crg_build_opts &opts);
    // Instance transforms (cr::entity::instances::transforms, model.cpp:99-126),
    // 16 floats each, column-major as glm::mat4; given to every model of this
    // scene (crg_scene_set_instances).  Empty = the models as added.
    void set_instances(const std::vector<std::array<float, 16>> &transforms);

    // ABI handles (the scene is committed first).
    crg_context *context() noexcept { return ctx_; }
    crg_scene *handle();
    uint64_t triangle_count() const noexcept { return mat_idx_.size(); }

private:
    void check(crg_status s) const;
    void commit();
    crg_context *ctx_ = nullptr;
    crg_scene *scene_ = nullptr;
    bool dirty_ = true;
    crg_build_opts opts_{8, 1, 3, 3};
    // one library model per add_model call, kept indexed: the library expands
    // it on the device (crg_scene_create_indexed / crg_scene_add_model_indexed),
    // so the host never holds the de-indexed copy
    struct model_rec {
        std::vector<float> positions;  // 3 per vertex
        std::vector<uint32_t> vidx;    // 3 per triangle, into positions
        std::vector<float> texcoords;  // 2 per coordinate
        std::vector<int32_t> tidx;     // 3 per triangle, into texcoords (-1 = none); empty = no coordinates
        std::vector<uint32_t> mat_idx; // into materials
        std::vector<crg_material> materials; // textures rebased onto the scene's texture list
        std::vector<material_information> infos; // the same, as cast_ray's records point to them
        std::vector<std::array<float, 16>> instances;
        bool added = false;            // present in the library scene
        bool instances_dirty = false;
    };
    std::vector<model_rec> models_;
    std::vector<uint32_t> mat_idx_;  // model-local material index per triangle, all models (triangle_count)
    std::vector<size_t> first_;      // first scene triangle of each model
    std::vector<image> textures_;    // all models' textures
    size_t textures_sent_ = 0;
    std::optional<image> skybox_;
    vec2 sky_rot_;
    bool sun_enabled_ = true;
    crg_sun sun_{};
    bool sun_set_ = false;
    class camera camera_;
    std::mutex mutex_;
    friend class renderer;
};

class renderer {
public:
    struct renderer_stats {
        uint64_t rays_per_second;
        uint64_t samples_per_second;
        uint64_t total_rays;
        double running_time;
    };
    struct options {
        uint32_t mode = CRG_MODE_FAITHFUL; // FAITHFUL = the reference estimator
        uint32_t samples_per_pass = 1;     // reference: one sample per pixel per pass
        uint32_t rr_depth = 0;
        uint32_t seed = 1;
        bool aov = true;                   // normals / albedos / depths planes
        bool count_rays = true;            // fills renderer_stats::total_rays
        uint64_t target_spp = 0;           // initial set_target_spp (0 = render until paused)
    };

    // Starts the management thread (renderer.cpp:105-144); rendering begins
    // at once, one crg_render pass after another, until the target spp.
    renderer(uint64_t res_x, uint64_t res_y, uint64_t bounces, scene *s);
    renderer(uint64_t res_x, uint64_t res_y, uint64_t bounces, scene *s, const options &opts);
    ~renderer();
    renderer(const renderer &) = delete;
    renderer &operator=(const renderer &) = delete;

    // Resumes after pause(): clears the film, the timer and the counters.
    bool start();
    // Blocks until the pass in flight has finished.
    bool pause();
    // pause(); update(); start() (renderer.cpp:182-189).
    void update(const std::function<void()> &update);
    void set_resolution(int x, int y);
    void set_max_bounces(int bounces);
    void set_target_spp(uint64_t target);
    renderer_stats current_stats();
    uint64_t current_sample_count() const noexcept { return sample_.load(); }
    std::pair<int, int> current_resolution() const noexcept { return {(int)res_x_, (int)res_y_}; }
    // Display image clamp(sum/spp, 0, 1)^(1/2.2), RGBA, refreshed on each call.
    image *current_progress();
    image *current_normals();
    image *current_albedos();
    image *current_depths();
    // Not in the reference: waits until the target spp is reached (false on timeout).
    bool wait_for_target(double seconds);
    // Not in the reference: raw film sums (float[W*H*3], film layout) and the film handle.
    std::vector<float> current_sums();
    crg_film *film() noexcept { return film_; }

private:
    void loop();
    void pass();
    void check(crg_status s) const;
    void make_film();
    bool want_work() const;

    scene *scene_;
    options opts_;
    uint64_t res_x_, res_y_;
    std::atomic<uint64_t> max_bounces_;
    std::atomic<uint64_t> target_{0};
    std::atomic<uint64_t> sample_{0};
    std::atomic<uint64_t> total_rays_{0};
    crg_film *film_ = nullptr;
    float *d_rgba_ = nullptr;
    image progress_, normals_, albedos_, depths_;
    std::chrono::steady_clock::time_point t0_;

    std::mutex gpu_;  // serialises ABI calls on the context's stream
    std::mutex m_;
    std::condition_variable cv_start_, cv_idle_;
    bool run_ = true, paused_ = false, idle_ = false;
    std::string thread_error_;
    std::thread thread_;
};

// cr::post_processor (src/render/post/post_processor.h:10-62) over
// crg_post_process: the same settings structs and process(image) -> image,
// with the GL compute passes run as CUDA kernels on the scene's device.
class post_processor {
public:
    struct bloom_settings {
        bool enabled = false;
        float threshold = 0.7f;
        float strength = 1.0f;
    };
    struct gray_scale_settings {
        bool enabled = false;
    };
    struct tonemapping_settings {
        bool enabled = false;
        int type = 0;
        float exposure = 1.f;
        float gamma_correction = 2.2f;
    };
    // Runs on the context of `owner` (its device); `faithful` reproduces the
    // reference's 8x8-dispatch coverage and brightness indexing (crg.h).
    explicit post_processor(scene *owner, bool faithful = true);
    ~post_processor();
    post_processor(const post_processor &) = delete;
    post_processor &operator=(const post_processor &) = delete;
    image process(const image &img);
    void submit_bloom_settings(const bloom_settings &s) { bloom_ = s; }
    void submit_gray_scale_settings(const gray_scale_settings &s) { gray_ = s; }
    void submit_tonemapping_settings(const tonemapping_settings &s) { tone_ = s; }

private:
    scene *scene_;
    bool faithful_;
    bloom_settings bloom_;
    gray_scale_settings gray_;
    tonemapping_settings tone_;
    float *d_src_ = nullptr, *d_dst_ = nullptr;
    size_t bytes_ = 0;
};

// cr::draft_renderer (src/render/draft/draft_renderer.h) over crg_draft_render:
// the unlit preview of the scene from its camera, as an RGBA image in the
// film's pixel layout.
class draft_renderer {
public:
    draft_renderer(scene *s, uint64_t res_x, uint64_t res_y);
    ~draft_renderer();
    draft_renderer(const draft_renderer &) = delete;
    draft_renderer &operator=(const draft_renderer &) = delete;
    void set_resolution(uint64_t res_x, uint64_t res_y);
    image *render();

private:
    scene *scene_;
    uint64_t res_x_, res_y_;
    float *d_rgba_ = nullptr;
    image out_;
};

} // namespace crg::host
