/*
 * ref_bridge.cpp — C entry points over CRender's OWN sampling and camera code,
 * compiled unmodified from the reference tree (src/util/sampling.h,
 * src/render/camera.cpp, src/render/ray.cpp) against the project-written glm
 * stand-in in oracle/refshim/.  TEST INFRASTRUCTURE ONLY: tests/ compare the
 * oracle's restatement (orc_render.cpp) with these functions.  Built by
 * oracle/Makefile's `ref` target into oracle/_ref/libref.so, only where the
 * reference sources are present; nothing on the product path loads it.
 */
#include <cstdint>
#include <deque>

#include <render/camera.h>
#include <util/sampling.h>

namespace {
// The reference's randf (declared in sampling.h, defined in renderer.cpp with
// a thread_local mt19937) is replaced by a queue the caller fills, so each
// draw is a known number.
thread_local std::deque<float> g_draws;
float randf() noexcept {
    if (g_draws.empty()) return 0.0f;
    const float u = g_draws.front();
    g_draws.pop_front();
    return u;
}
} // namespace

extern "C" {

/* cr::sampling::build_local (sampling.h:21-33) */
void ref_build_local(const float *n3, float *t3, float *b3) {
    const cr::sampling::local_coords c = cr::sampling::build_local(glm::vec3(n3[0], n3[1], n3[2]));
    t3[0] = c.tangent.x; t3[1] = c.tangent.y; t3[2] = c.tangent.z;
    b3[0] = c.bi_tangent.x; b3[1] = c.bi_tangent.y; b3[2] = c.bi_tangent.z;
}

/* cr::sampling::sphere (sampling.h:156-166) */
void ref_sphere(float u1, float u2, float *out3) {
    const glm::vec3 v = cr::sampling::sphere(glm::vec2(u1, u2));
    out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}

/* cr::sampling::hemp_cos (sampling.h:168-172): the faithful Lambert direction before normalisation */
void ref_hemp_cos(const float *n3, float u1, float u2, float *out3) {
    const glm::vec3 v = cr::sampling::hemp_cos(glm::vec3(n3[0], n3[1], n3[2]), glm::vec2(u1, u2));
    out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}

/* cr::sampling::cook_torrence::specular_d (sampling.h:93-107) */
float ref_specular_d(float noh, float roughness) { return cr::sampling::cook_torrence::specular_d(noh, roughness); }

/* cr::sampling::cos_hemp (sampling.h:174-183) */
void ref_cos_hemp(float x, float y, float *out3) {
    const glm::vec3 v = cr::sampling::cos_hemp(x, y);
    out3[0] = v.x; out3[1] = v.y; out3[2] = v.z;
}

/* cr::sampling::sun::sample (sampling.h:72-80) with the sun transform of
 * cr::registry (registry.cpp:44-48): the two draws are `first` then `second`
 * (the order in which the compiler evaluates the two randf() arguments of
 * map_to_solid_angle's vec2 is unspecified; the caller finds it out).
 * Writes the direction, the pdf and the cosine with `normal`. */
void ref_sun_sample(const float *sun_dir3, float sun_size, const float *normal3, float first, float second, float *dir3,
                    float *pdf, float *cosine) {
    cr::entity::sun sun;
    sun.direction = glm::vec3(sun_dir3[0], sun_dir3[1], sun_dir3[2]);
    sun.size = sun_size;
    const cr::sampling::local_coords lc = cr::sampling::build_local(-sun.direction);
    cr::sampling::sun::incoming in;
    in.normal = glm::vec3(normal3[0], normal3[1], normal3[2]);
    in.sun_transform = glm::mat3(lc.tangent, lc.normal, lc.bi_tangent);
    in.sun = sun;
    g_draws.clear();
    g_draws.push_back(first);
    g_draws.push_back(second);
    const cr::sampling::sun::pdf_cos s = cr::sampling::sun::sample(in);
    dir3[0] = s.dir.x; dir3[1] = s.dir.y; dir3[2] = s.dir.z;
    *pdf = s.pdf;
    *cosine = s.cosine;
}

/* cr::sampling::sun::sky_colour (sampling.h:53-57): 1 when the direction sees the sun disc */
int ref_sun_visible(const float *dir3, const float *sun_dir3, float sun_size) {
    cr::entity::sun sun;
    sun.direction = glm::vec3(sun_dir3[0], sun_dir3[1], sun_dir3[2]);
    sun.size = sun_size;
    sun.intensity = 1.0f;
    sun.colour = glm::vec3(1.0f);
    const glm::vec3 c = cr::sampling::sun::sky_colour(glm::vec3(dir3[0], dir3[1], dir3[2]), sun);
    return c.x != 0.0f ? 1 : 0;
}

/* cr::camera::rotate + get_ray (camera.cpp:14-68): a camera at `pos` turned by
 * `rot` degrees (one rotate call from zero, as the UI's first edit), vertical
 * fov, mode 0 perspective / 1 orthographic with `scale`. */
void ref_camera_ray(const float *pos3, const float *rot3, float fov, int mode, float scale, float x, float y,
                    float aspect, float *org3, float *dir3) {
    cr::camera cam(glm::vec3(pos3[0], pos3[1], pos3[2]), fov,
                   mode ? cr::camera::mode::orthographic : cr::camera::mode::perspective);
    cam.scale = scale;
    cam.rotate(glm::vec3(rot3[0], rot3[1], rot3[2]));
    const cr::ray r = cam.get_ray(x, y, aspect);
    org3[0] = r.origin.x; org3[1] = r.origin.y; org3[2] = r.origin.z;
    dir3[0] = r.direction.x; dir3[1] = r.direction.y; dir3[2] = r.direction.z;
}

} /* extern "C" */
