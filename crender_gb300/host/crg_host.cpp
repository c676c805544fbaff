// crg_host.cpp — C++ adapter with the interface of cr::scene / cr::camera /
// cr::renderer over the C ABI.  See crg_host.h.
#include "crg_host.h"

#include <algorithm>
#include <cmath>

namespace crg::host {

namespace {

[[noreturn]] void raise(crg_context *ctx, crg_status s, const char *what) {
    std::string msg = std::string(what) + ": " + crg_status_string(s);
    if (ctx) msg += std::string(" (") + crg_last_error_string(ctx) + ")";
    throw error(s, msg);
}

// image::get_uv texel index (src/objects/image.h:104-109): truncation, modulo wrap.
uint64_t texel(float u, uint64_t n) {
    const float f = u * (float)n;
    uint64_t i = 0;
    if (f >= 0.0f) i = f < 4.6e18f ? (uint64_t)f : 0;
    return i % n;
}

// Ry(a) * Rx(b) * Rz(c), degrees (camera.cpp:62-68), in double.
void rotation_matrix(const vec3 &r, double M[3][3]) {
    const double k = 3.14159265358979323846 / 180.0;
    const double ax = r.x * k, ay = r.y * k, az = r.z * k;
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
            M[i][j] = 0;
            for (int m = 0; m < 3; ++m) M[i][j] += T[i][m] * Rz[m][j];
        }
}

crg_material to_crg(const material_information &m) {
    crg_material c{};
    c.shade_type = (uint32_t)m.shade_type;
    c.ior = m.ior;
    c.roughness = m.roughness;
    c.reflectiveness = m.reflectiveness;
    c.emission = m.emission;
    for (int k = 0; k < 4; ++k) c.colour[k] = m.colour[k];
    c.tex = m.tex ? (int32_t)*m.tex : -1;
    return c;
}

} // namespace

// ------------------------------------------------------------------ image
image::image(uint64_t width, uint64_t height)
    : width_(width), height_(height), data_(width * height * 4, std::numeric_limits<float>::max()) {}

image::image(const std::vector<float> &data, uint64_t width, uint64_t height) : width_(width), height_(height) {
    if (data.size() != width * height * 4) throw error(CRG_ERR_INVALID_ARG, "image: data is not width*height*4 floats");
    data_ = data;
}

vec3 image::get_uv(float u, float v) const noexcept {
    if (!valid()) return {};
    const float *t = data_.data() + (texel(u, width_) + texel(v, height_) * width_) * 4;
    return {t[0], t[1], t[2]};
}

// ------------------------------------------------------------------ camera
camera::camera(vec3 position_, float fov_, mode camera_mode) : fov(fov_), current_mode(camera_mode), position(position_) {}

void camera::update_cache() {
    cached_position_ = position;
    cached_rotation_ = rotation;
}

void camera::translate(const vec3 &t) {
    double M[3][3];
    rotation_matrix(cached_rotation_, M);
    const vec3 p = cached_position_;
    position = {(float)(M[0][0] * t.x + M[0][1] * t.y + M[0][2] * t.z + p.x),
                (float)(M[1][0] * t.x + M[1][1] * t.y + M[1][2] * t.z + p.y),
                (float)(M[2][0] * t.x + M[2][1] * t.y + M[2][2] * t.z + p.z)};
    update_cache();
}

void camera::rotate(const vec3 &r) {
    rotation.x += r.x;
    rotation.y = std::clamp(rotation.y + r.y, -90.0f, 90.0f);
    rotation.z += r.z;
    update_cache();
}

crg_camera camera::to_crg() const noexcept {
    crg_camera c{};
    // perspective rays start at the live position; orthographic origins go through the cached matrix
    const vec3 p = current_mode == mode::perspective ? position : cached_position_;
    c.position[0] = p.x;
    c.position[1] = p.y;
    c.position[2] = p.z;
    c.rotation[0] = cached_rotation_.x;
    c.rotation[1] = cached_rotation_.y;
    c.rotation[2] = cached_rotation_.z;
    c.fov = fov;
    c.mode = current_mode == mode::perspective ? CRG_CAMERA_PERSPECTIVE : CRG_CAMERA_ORTHOGRAPHIC;
    c.scale = scale;
    return c;
}

// ------------------------------------------------------------------ scene
scene::scene(int device) {
    const crg_status s = crg_context_create(device, &ctx_);
    if (s != CRG_OK) raise(nullptr, s, "crg_context_create");
}

scene::~scene() {
    if (scene_) crg_scene_destroy(scene_);
    if (ctx_) crg_context_destroy(ctx_);
}

void scene::check(crg_status s) const {
    if (s != CRG_OK) raise(ctx_, s, "crg");
}

size_t scene::add_model(const model_data &m) {
    std::lock_guard<std::mutex> g(mutex_);
    const size_t ni = m.vertex_indices.size();
    if (ni % 3) throw error(CRG_ERR_INVALID_ARG, "add_model: vertex_indices is not a multiple of 3");
    const size_t ntri = ni / 3;
    if (m.material_indices.size() != ntri) throw error(CRG_ERR_INVALID_ARG, "add_model: one material index per triangle");
    const bool have_uv = !m.texture_indices.empty();
    if (have_uv && m.texture_indices.size() != ni) throw error(CRG_ERR_INVALID_ARG, "add_model: texture_indices size");
    for (uint32_t k : m.vertex_indices)
        if (k >= m.vertices.size()) throw error(CRG_ERR_INVALID_ARG, "add_model: vertex index out of range");
    for (uint32_t k : m.material_indices)
        if (k >= m.materials.size()) throw error(CRG_ERR_INVALID_ARG, "add_model: material index out of range");
    for (const material_information &mi : m.materials)
        if (mi.tex && *mi.tex >= m.textures.size()) throw error(CRG_ERR_INVALID_ARG, "add_model: texture index out of range");
    // register_model (registry.cpp:51-97) keeps the model's own index space; only
    // texture indices are rebased onto the scene's texture list
    model_rec r;
    const uint32_t tex_base = (uint32_t)textures_.size();
    for (const vec3 &v : m.vertices) r.positions.insert(r.positions.end(), {v.x, v.y, v.z});
    for (const vec2 &t : m.texture_coords) r.texcoords.insert(r.texcoords.end(), {t.x, t.y});
    r.vidx.assign(m.vertex_indices.begin(), m.vertex_indices.end());
    if (have_uv)
        for (size_t i = 0; i < ni; ++i) {
            const uint32_t t = m.texture_indices[i];
            r.tidx.push_back(t < m.texture_coords.size() ? (int32_t)t : -1);
        }
    r.mat_idx.assign(m.material_indices.begin(), m.material_indices.end());
    for (material_information mi : m.materials) {
        if (mi.tex) mi.tex = tex_base + *mi.tex;
        r.materials.push_back(to_crg(mi));
        r.infos.push_back(mi);
    }
    first_.push_back(mat_idx_.size());
    for (size_t t = 0; t < ntri; ++t) mat_idx_.push_back(m.material_indices[t]);
    textures_.insert(textures_.end(), m.textures.begin(), m.textures.end());
    models_.push_back(std::move(r));
    dirty_ = true;
    return models_.size() - 1;
}

void scene::set_instances(const std::vector<std::array<float, 16>> &transforms) {
    std::lock_guard<std::mutex> g(mutex_);
    for (model_rec &r : models_) {
        r.instances = transforms;
        r.instances_dirty = false;
    }
    if (scene_) check(crg_scene_set_instances(scene_, transforms.empty() ? nullptr : transforms[0].data(),
                                              (uint32_t)transforms.size()));
}

void scene::set_model_instances(size_t model, const std::vector<std::array<float, 16>> &transforms) {
    std::lock_guard<std::mutex> g(mutex_);
    if (model >= models_.size()) throw error(CRG_ERR_INVALID_ARG, "set_model_instances: no such model");
    model_rec &r = models_[model];
    r.instances = transforms;
    r.instances_dirty = true;
    if (scene_ && r.added) {
        check(crg_scene_set_model_instances(scene_, (uint32_t)model, transforms.empty() ? nullptr : transforms[0].data(),
                                            (uint32_t)transforms.size()));
        r.instances_dirty = false;
    }
}

void scene::set_skybox(image &&sky) {
    std::lock_guard<std::mutex> g(mutex_);
    skybox_ = std::move(sky);
    if (scene_) check(crg_scene_set_skybox(scene_, skybox_->data(), (uint32_t)skybox_->width(),
                                           (uint32_t)skybox_->height(), sky_rot_.x, sky_rot_.y));
}

void scene::set_skybox_rotation(const vec2 &r) {
    std::lock_guard<std::mutex> g(mutex_);
    sky_rot_ = r;
    if (scene_ && skybox_)
        check(crg_scene_set_skybox(scene_, skybox_->data(), (uint32_t)skybox_->width(), (uint32_t)skybox_->height(),
                                   sky_rot_.x, sky_rot_.y));
}

void scene::set_sun_enabled(bool v) {
    std::lock_guard<std::mutex> g(mutex_);
    sun_enabled_ = v;
    if (scene_) check(crg_scene_set_sun(scene_, v ? 1 : 0, sun_set_ ? &sun_ : nullptr));
}

void scene::set_sun(const crg_sun &s) {
    std::lock_guard<std::mutex> g(mutex_);
    sun_ = s;
    sun_set_ = true;
    if (scene_) check(crg_scene_set_sun(scene_, sun_enabled_ ? 1 : 0, &sun_));
}

void scene::set_build_options(const crg_build_opts &o) {
    std::lock_guard<std::mutex> g(mutex_);
    opts_ = o;
    dirty_ = true;
}

vec3 scene::sample_skybox(float x, float y) const noexcept {
    if (!skybox_) return {};
    return skybox_->get_uv(x + sky_rot_.x, y + sky_rot_.y);
}

void scene::commit() {
    if (!dirty_ && scene_) return;
    if (models_.empty() || mat_idx_.empty()) throw error(CRG_ERR_INVALID_ARG, "scene has no triangles");
    auto indexed = [](const model_rec &r, auto &&call) {
        return call(r.positions.data(), (uint32_t)(r.positions.size() / 3), r.vidx.data(), (uint32_t)(r.vidx.size() / 3),
                    r.texcoords.empty() ? nullptr : r.texcoords.data(), (uint32_t)(r.texcoords.size() / 2),
                    r.tidx.empty() ? nullptr : r.tidx.data(), r.mat_idx.data(), r.materials.data(),
                    (uint32_t)r.materials.size());
    };
    crg_status s = CRG_OK;
    bool fresh = false;
    if (!scene_) {
        // model 0 creates the library scene (crg_scene_create_indexed)
        crg_scene *sc = nullptr;
        s = indexed(models_[0], [&](auto... a) { return crg_scene_create_indexed(ctx_, a..., &sc); });
        if (s != CRG_OK) raise(ctx_, s, "scene commit");
        scene_ = sc;
        models_[0].added = true;
        models_[0].instances_dirty = !models_[0].instances.empty();
        textures_sent_ = 0;
        fresh = true;
    }
    // every later model: appended with its own BVH region (crg_scene_add_model_indexed)
    for (size_t k = 0; k < models_.size() && s == CRG_OK; ++k) {
        model_rec &r = models_[k];
        if (r.added) continue;
        uint32_t idx = 0;
        s = indexed(r, [&](auto... a) { return crg_scene_add_model_indexed(scene_, a..., &idx); });
        if (s == CRG_OK && idx != k) s = CRG_ERR_INVALID_ARG;
        r.added = s == CRG_OK;
        r.instances_dirty = !r.instances.empty();
    }
    if (s == CRG_OK && textures_sent_ != textures_.size()) {
        std::vector<const float *> px;
        std::vector<uint32_t> w, h;
        for (const image &t : textures_) {
            px.push_back(t.data());
            w.push_back((uint32_t)t.width());
            h.push_back((uint32_t)t.height());
        }
        s = crg_scene_set_textures(scene_, (uint32_t)px.size(), px.data(), w.data(), h.data());
        if (s == CRG_OK) textures_sent_ = textures_.size();
    }
    for (size_t k = 0; k < models_.size() && s == CRG_OK; ++k) {
        model_rec &r = models_[k];
        if (!r.instances_dirty) continue;
        s = crg_scene_set_model_instances(scene_, (uint32_t)k, r.instances.empty() ? nullptr : r.instances[0].data(),
                                          (uint32_t)r.instances.size());
        r.instances_dirty = false;
    }
    // only models without a BVH for these options are built
    if (s == CRG_OK) s = crg_scene_build(scene_, &opts_, nullptr);
    if (s == CRG_OK && fresh && skybox_)
        s = crg_scene_set_skybox(scene_, skybox_->data(), (uint32_t)skybox_->width(), (uint32_t)skybox_->height(),
                                 sky_rot_.x, sky_rot_.y);
    if (s == CRG_OK && fresh) s = crg_scene_set_sun(scene_, sun_enabled_ ? 1 : 0, sun_set_ ? &sun_ : nullptr);
    if (s == CRG_OK) s = crg_stream_sync(ctx_, nullptr);
    if (s != CRG_OK) {
        // a failed commit leaves no half-made library scene behind: the next one starts over
        crg_scene_destroy(scene_);
        scene_ = nullptr;
        for (model_rec &r : models_) r.added = false;
        raise(ctx_, s, "scene commit");
    }
    dirty_ = false;
}

crg_scene *scene::handle() {
    std::lock_guard<std::mutex> g(mutex_);
    commit();
    return scene_;
}

std::vector<intersection_record> scene::cast_rays(const std::vector<ray> &rays) {
    std::lock_guard<std::mutex> g(mutex_);
    commit();
    std::vector<intersection_record> out(rays.size());
    if (rays.empty()) return out;
    std::vector<crg_ray> rr(rays.size());
    for (size_t i = 0; i < rays.size(); ++i) {
        const ray &r = rays[i];
        // RTCRayHit as model.cpp:10-27 fills it: tnear 1e-5, tfar +inf
        rr[i] = crg_ray{{r.origin.x, r.origin.y, r.origin.z}, 1e-5f, {r.direction.x, r.direction.y, r.direction.z}, INFINITY};
    }
    void *d_rays = nullptr, *d_hits = nullptr;
    std::vector<crg_hit> hits(rays.size());
    crg_status s = crg_device_alloc(ctx_, rr.size() * sizeof(crg_ray), &d_rays);
    if (s == CRG_OK) s = crg_device_alloc(ctx_, rr.size() * sizeof(crg_hit), &d_hits);
    if (s == CRG_OK) s = crg_memcpy_h2d(ctx_, d_rays, rr.data(), rr.size() * sizeof(crg_ray), nullptr);
    if (s == CRG_OK)
        s = crg_intersect_closest(scene_, (const crg_ray *)d_rays, (crg_hit *)d_hits, rr.size(), nullptr);
    if (s == CRG_OK) s = crg_memcpy_d2h(ctx_, hits.data(), d_hits, hits.size() * sizeof(crg_hit), nullptr);
    if (s == CRG_OK) s = crg_stream_sync(ctx_, nullptr);
    if (s == CRG_OK) s = crg_scene_poll_error(scene_);
    if (d_rays) crg_device_free(ctx_, d_rays);
    if (d_hits) crg_device_free(ctx_, d_hits);
    if (s != CRG_OK) raise(ctx_, s, "cast_rays");
    for (size_t i = 0; i < rays.size(); ++i) {
        const crg_hit &h = hits[i];
        intersection_record &rec = out[i];
        if (h.prim == CRG_INVALID_PRIM) continue;
        rec.prim_id = h.prim;
        rec.distance = h.t;
        // the model holding the triangle, and its index there
        const size_t mdl = (size_t)(std::upper_bound(first_.begin(), first_.end(), (size_t)h.prim) - first_.begin()) - 1;
        const model_rec &mr = models_[mdl];
        const size_t p = h.prim - first_[mdl];
        rec.material = &mr.infos[mr.mat_idx[p]];
        float v[9];
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) v[3 * k + a] = mr.positions[3 * (size_t)mr.vidx[3 * p + k] + a];
        const double e1[3] = {(double)v[3] - v[0], (double)v[4] - v[1], (double)v[5] - v[2]};
        const double e2[3] = {(double)v[6] - v[0], (double)v[7] - v[1], (double)v[8] - v[2]};
        double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        if (len > 0) rec.normal = {(float)(n[0] / len), (float)(n[1] / len), (float)(n[2] / len)};
        float uv[6] = {0, 0, 0, 0, 0, 0};
        for (int k = 0; k < 3 && !mr.tidx.empty(); ++k) {
            const int32_t t = mr.tidx[3 * p + k];
            if (t >= 0) {
                uv[2 * k] = mr.texcoords[2 * (size_t)t];
                uv[2 * k + 1] = mr.texcoords[2 * (size_t)t + 1];
            }
        }
        const float w0 = 1.0f - h.u - h.v;
        rec.uv = {w0 * uv[0] + h.u * uv[2] + h.v * uv[4], w0 * uv[1] + h.u * uv[3] + h.v * uv[5]};
        const ray &r = rays[i];
        rec.intersection_point = {r.origin.x + r.direction.x * h.t, r.origin.y + r.direction.y * h.t,
                                  r.origin.z + r.direction.z * h.t};
    }
    return out;
}

intersection_record scene::cast_ray(const ray &r) { return cast_rays({r})[0]; }

// ------------------------------------------------------------------ renderer
renderer::renderer(uint64_t res_x, uint64_t res_y, uint64_t bounces, scene *s)
    : renderer(res_x, res_y, bounces, s, options()) {}

renderer::renderer(uint64_t res_x, uint64_t res_y, uint64_t bounces, scene *s, const options &opts)
    : scene_(s), opts_(opts), res_x_(res_x), res_y_(res_y), max_bounces_(bounces) {
    if (!s) throw error(CRG_ERR_INVALID_ARG, "renderer: null scene");
    if (res_x == 0 || res_y == 0) throw error(CRG_ERR_INVALID_ARG, "renderer: empty resolution");
    if (opts_.samples_per_pass == 0) opts_.samples_per_pass = 1;
    target_ = opts_.target_spp;
    make_film();
    t0_ = std::chrono::steady_clock::now();
    thread_ = std::thread([this] { loop(); });
}

renderer::~renderer() {
    {
        std::lock_guard<std::mutex> g(m_);
        run_ = false;
    }
    cv_start_.notify_all();
    if (thread_.joinable()) thread_.join();
    if (d_rgba_) crg_device_free(scene_->context(), d_rgba_);
    if (film_) crg_film_destroy(film_);
}

void renderer::check(crg_status s) const {
    if (s != CRG_OK) raise(scene_->context(), s, "renderer");
}

void renderer::make_film() {
    if (d_rgba_) crg_device_free(scene_->context(), d_rgba_);
    d_rgba_ = nullptr;
    if (film_) crg_film_destroy(film_);
    film_ = nullptr;
    check(crg_film_create(scene_->context(), (uint32_t)res_x_, (uint32_t)res_y_, opts_.aov ? CRG_FILM_AOV : 0u, &film_));
    void *p = nullptr;
    check(crg_device_alloc(scene_->context(), res_x_ * res_y_ * 16, &p));
    d_rgba_ = (float *)p;
    progress_ = image(res_x_, res_y_);
    normals_ = image(res_x_, res_y_);
    albedos_ = image(res_x_, res_y_);
    depths_ = image(res_x_, res_y_);
}

bool renderer::want_work() const {
    const uint64_t t = target_.load();
    return !paused_ && (t == 0 || sample_.load() < t);
}

void renderer::pass() {
    std::lock_guard<std::mutex> g(gpu_);
    crg_scene *sc = scene_->handle();
    const crg_camera cam = scene_->camera()->to_crg();
    uint32_t spp = opts_.samples_per_pass;
    const uint64_t t = target_.load();
    if (t) spp = (uint32_t)std::min<uint64_t>(spp, t - std::min(t, sample_.load()));
    if (spp == 0) return;
    crg_settings s{};
    s.width = (uint32_t)res_x_;
    s.height = (uint32_t)res_y_;
    s.spp = spp;
    s.max_bounces = (uint32_t)max_bounces_.load();
    s.rr_depth = opts_.rr_depth;
    s.mode = opts_.mode;
    s.seed = opts_.seed;
    s.aspect = (float)res_x_ / (float)res_y_; // renderer::set_resolution's aspect correction
    check(crg_scene_set_counting(sc, opts_.count_rays ? 1 : 0));
    check(crg_render(sc, &cam, &s, film_, nullptr));
    check(crg_stream_sync(scene_->context(), nullptr));
    crg_render_stats st{};
    check(crg_render_stats_get(sc, &st));
    total_rays_ += st.segments + st.shadow_rays;
    sample_ += spp;
}

void renderer::loop() {
    std::unique_lock<std::mutex> lk(m_);
    while (run_) {
        if (want_work()) {
            lk.unlock();
            try {
                pass();
            } catch (const std::exception &e) {
                lk.lock();
                thread_error_ = e.what();
                paused_ = true; // stop until start() after the caller has seen the error
                continue;
            }
            lk.lock();
            continue;
        }
        idle_ = true;
        cv_idle_.notify_all();
        cv_start_.wait(lk, [this] { return !run_ || want_work(); });
        idle_ = false;
    }
    idle_ = true;
    cv_idle_.notify_all();
}

bool renderer::start() {
    std::unique_lock<std::mutex> lk(m_);
    if (!paused_) return false;
    {
        std::lock_guard<std::mutex> g(gpu_);
        check(crg_film_reset(film_, nullptr));
    }
    sample_ = 0;
    total_rays_ = 0;
    thread_error_.clear();
    t0_ = std::chrono::steady_clock::now();
    paused_ = false;
    if (want_work()) idle_ = false; // so a wait that follows sees the work, not the old idle state
    lk.unlock();
    cv_start_.notify_all();
    return true;
}

bool renderer::pause() {
    std::unique_lock<std::mutex> lk(m_);
    if (paused_) return false;
    paused_ = true;
    cv_idle_.wait(lk, [this] { return idle_; });
    return true;
}

void renderer::update(const std::function<void()> &fn) {
    pause();
    fn();
    start();
}

void renderer::set_resolution(int x, int y) {
    if (x <= 0 || y <= 0) throw error(CRG_ERR_INVALID_ARG, "set_resolution: empty resolution");
    std::unique_lock<std::mutex> lk(m_);
    const bool was_paused = paused_;
    paused_ = true;
    cv_idle_.wait(lk, [this] { return idle_; });
    {
        std::lock_guard<std::mutex> g(gpu_);
        res_x_ = (uint64_t)x;
        res_y_ = (uint64_t)y;
        make_film();
    }
    sample_ = 0;
    paused_ = was_paused;
    if (want_work()) idle_ = false;
    lk.unlock();
    cv_start_.notify_all();
}

void renderer::set_max_bounces(int bounces) { max_bounces_ = (uint64_t)std::max(bounces, 0); }

void renderer::set_target_spp(uint64_t target) {
    std::unique_lock<std::mutex> lk(m_);
    target_ = target;
    if (want_work()) idle_ = false;
    lk.unlock();
    cv_start_.notify_all();
}

bool renderer::wait_for_target(double seconds) {
    std::unique_lock<std::mutex> lk(m_);
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(seconds);
    const bool ok = cv_idle_.wait_until(lk, until, [this] { return idle_ || !thread_error_.empty(); });
    if (!thread_error_.empty()) throw error(CRG_ERR_CUDA, thread_error_);
    return ok && target_.load() != 0 && sample_.load() >= target_.load();
}

renderer::renderer_stats renderer::current_stats() {
    const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    renderer_stats s{};
    s.total_rays = total_rays_.load();
    s.running_time = t;
    s.rays_per_second = t > 0 ? (uint64_t)((double)s.total_rays / t) : 0;
    s.samples_per_second = t > 0 ? (uint64_t)((double)sample_.load() / t) : 0;
    return s;
}

image *renderer::current_progress() {
    std::lock_guard<std::mutex> g(gpu_);
    if (sample_.load() == 0) return &progress_;
    check(crg_film_display(film_, d_rgba_, nullptr));
    check(crg_memcpy_d2h(scene_->context(), progress_.data(), d_rgba_, res_x_ * res_y_ * 16, nullptr));
    check(crg_stream_sync(scene_->context(), nullptr));
    return &progress_;
}

image *renderer::current_normals() {
    std::lock_guard<std::mutex> g(gpu_);
    if (opts_.aov) check(crg_film_download(film_, nullptr, nullptr, nullptr, nullptr, normals_.data(), nullptr, nullptr));
    return &normals_;
}

image *renderer::current_albedos() {
    std::lock_guard<std::mutex> g(gpu_);
    if (opts_.aov) check(crg_film_download(film_, nullptr, nullptr, nullptr, albedos_.data(), nullptr, nullptr, nullptr));
    return &albedos_;
}

image *renderer::current_depths() {
    std::lock_guard<std::mutex> g(gpu_);
    if (opts_.aov) check(crg_film_download(film_, nullptr, nullptr, nullptr, nullptr, nullptr, depths_.data(), nullptr));
    return &depths_;
}

std::vector<float> renderer::current_sums() {
    std::lock_guard<std::mutex> g(gpu_);
    std::vector<float> out(res_x_ * res_y_ * 3);
    check(crg_film_download(film_, out.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr));
    return out;
}

// ------------------------------------------------------------------ post_processor
post_processor::post_processor(scene *owner, bool faithful) : scene_(owner), faithful_(faithful) {
    if (!owner) throw error(CRG_ERR_INVALID_ARG, "post_processor: null scene");
}

post_processor::~post_processor() {
    if (d_src_) crg_device_free(scene_->context(), d_src_);
    if (d_dst_) crg_device_free(scene_->context(), d_dst_);
}

image post_processor::process(const image &img) {
    if (!img.valid()) throw error(CRG_ERR_INVALID_ARG, "post_processor: empty image");
    crg_context *ctx = scene_->context();
    const size_t bytes = img.width() * img.height() * 16;
    if (bytes > bytes_) {
        if (d_src_) crg_device_free(ctx, d_src_);
        if (d_dst_) crg_device_free(ctx, d_dst_);
        d_src_ = d_dst_ = nullptr;
        bytes_ = 0;
        void *a = nullptr, *b = nullptr;
        crg_status s = crg_device_alloc(ctx, bytes, &a);
        if (s == CRG_OK) s = crg_device_alloc(ctx, bytes, &b);
        if (s != CRG_OK) {
            if (a) crg_device_free(ctx, a);
            raise(ctx, s, "post_processor");
        }
        d_src_ = (float *)a;
        d_dst_ = (float *)b;
        bytes_ = bytes;
    }
    crg_post_settings ps;
    crg_post_settings_default(&ps);
    ps.bloom = bloom_.enabled;
    ps.bloom_threshold = bloom_.threshold;
    ps.bloom_strength = bloom_.strength;
    ps.gray_scale = gray_.enabled;
    ps.tonemapping = tone_.enabled;
    ps.tonemap_type = tone_.type;
    ps.exposure = tone_.exposure;
    ps.gamma = tone_.gamma_correction;
    ps.mode = faithful_ ? CRG_POST_FAITHFUL : CRG_POST_FULL;
    image out(img.width(), img.height());
    crg_status s = crg_memcpy_h2d(ctx, d_src_, img.data(), bytes, nullptr);
    if (s == CRG_OK) s = crg_post_process(ctx, d_src_, d_dst_, (uint32_t)img.width(), (uint32_t)img.height(), &ps, nullptr);
    if (s == CRG_OK) s = crg_memcpy_d2h(ctx, out.data(), d_dst_, bytes, nullptr);
    if (s == CRG_OK) s = crg_stream_sync(ctx, nullptr);
    if (s != CRG_OK) raise(ctx, s, "post_processor::process");
    return out;
}

// ------------------------------------------------------------------ draft_renderer
draft_renderer::draft_renderer(scene *s, uint64_t res_x, uint64_t res_y) : scene_(s), res_x_(0), res_y_(0) {
    if (!s) throw error(CRG_ERR_INVALID_ARG, "draft_renderer: null scene");
    set_resolution(res_x, res_y);
}

draft_renderer::~draft_renderer() {
    if (d_rgba_) crg_device_free(scene_->context(), d_rgba_);
}

void draft_renderer::set_resolution(uint64_t res_x, uint64_t res_y) {
    if (res_x == 0 || res_y == 0) throw error(CRG_ERR_INVALID_ARG, "draft_renderer: empty resolution");
    if (d_rgba_) crg_device_free(scene_->context(), d_rgba_);
    d_rgba_ = nullptr;
    void *p = nullptr;
    const crg_status s = crg_device_alloc(scene_->context(), res_x * res_y * 16, &p);
    if (s != CRG_OK) raise(scene_->context(), s, "draft_renderer");
    d_rgba_ = (float *)p;
    res_x_ = res_x;
    res_y_ = res_y;
    out_ = image(res_x, res_y);
}

image *draft_renderer::render() {
    crg_scene *sc = scene_->handle();
    const crg_camera cam = scene_->camera()->to_crg();
    crg_context *ctx = scene_->context();
    crg_status s = crg_draft_render(sc, &cam, (uint32_t)res_x_, (uint32_t)res_y_, (float)res_x_ / (float)res_y_,
                                    d_rgba_, nullptr);
    if (s == CRG_OK) s = crg_memcpy_d2h(ctx, out_.data(), d_rgba_, res_x_ * res_y_ * 16, nullptr);
    if (s == CRG_OK) s = crg_stream_sync(ctx, nullptr);
    if (s != CRG_OK) raise(ctx, s, "draft_renderer::render");
    return &out_;
}

} // namespace crg::host
