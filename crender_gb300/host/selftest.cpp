// selftest.cpp — drives crg::host::scene / renderer the way the reference's
// UI drives cr::scene / cr::renderer, on a scene read from a file, and writes
// what it saw for the tests to compare with direct ABI calls.
//
//   crg_host_selftest <in> <out>
// in : u32 magic 0x54475243, ntri, nmat, W, H, spp, bounces, mode, nrays, nsplit;
//      float verts[ntri*9]; u32 mat_idx[ntri]; crg_material mats[nmat];
//      crg_camera cam; crg_ray rays[nrays]
//      (triangles [0, nsplit) and [nsplit, ntri) go in as two models, indexed)
// out: u64 spp1; float sums1[W*H*3]; u64 spp2; float sums2[W*H*3];
//      u64 total_rays; per ray: u32 prim, float distance, float normal[3]
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "crg_host.h"

using namespace crg::host;

namespace {

template <class T> bool rd(FILE *f, T *p, size_t n) { return n == 0 || std::fread(p, sizeof(T), n, f) == n; }
template <class T> void wr(FILE *f, const T *p, size_t n) { if (n) std::fwrite(p, sizeof(T), n, f); }

model_data make_model(const std::vector<float> &v, const std::vector<uint32_t> &mi, const std::vector<crg_material> &mats,
                      size_t t0, size_t t1) {
    model_data m;
    m.name = "part";
    // indexed the way an OBJ loader produces it: vertices listed in reverse, indices pointing back
    const size_t nt = t1 - t0;
    m.vertices.resize(nt * 3);
    for (size_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k) {
            const float *p = &v[(t0 + t) * 9 + k * 3];
            m.vertices[nt * 3 - 1 - (t * 3 + k)] = vec3{p[0], p[1], p[2]};
            m.vertex_indices.push_back((uint32_t)(nt * 3 - 1 - (t * 3 + k)));
        }
    for (const crg_material &c : mats) {
        material_information info;
        info.shade_type = (material_information::type)c.shade_type;
        info.ior = c.ior;
        info.roughness = c.roughness;
        info.reflectiveness = c.reflectiveness;
        info.emission = c.emission;
        std::memcpy(info.colour, c.colour, sizeof(info.colour));
        m.materials.push_back(info);
    }
    for (size_t t = t0; t < t1; ++t) m.material_indices.push_back(mi[t]);
    return m;
}

// crg_host_selftest obj <file.obj> <out>: load_model only (no device).
// out: u32 npos, ntc, ntri, nmat; float positions[npos*3]; float texcoords[ntc*2];
//      u32 vertex_indices[ntri*3]; u32 texture_indices[ntri*3] (0xFFFFFFFF = none);
//      u32 material_indices[ntri]; float colours[nmat*4]
int obj_parse(const char *file, const char *out) {
    try {
        const model_data m = load_model(file);
        FILE *g = std::fopen(out, "wb");
        if (!g) return 2;
        const uint32_t ntri = (uint32_t)(m.vertex_indices.size() / 3);
        const uint32_t h[4] = {(uint32_t)m.vertices.size(), (uint32_t)m.texture_coords.size(), ntri,
                               (uint32_t)m.materials.size()};
        wr(g, h, 4);
        for (const vec3 &v : m.vertices) wr(g, &v.x, 3);
        for (const vec2 &t : m.texture_coords) wr(g, &t.x, 2);
        wr(g, m.vertex_indices.data(), m.vertex_indices.size());
        std::vector<uint32_t> ti(m.texture_indices);
        if (ti.empty()) ti.assign(m.vertex_indices.size(), 0xFFFFFFFFu);
        wr(g, ti.data(), ti.size());
        wr(g, m.material_indices.data(), m.material_indices.size());
        for (const material_information &mi : m.materials) wr(g, mi.colour, 4);
        std::fclose(g);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "selftest: %s\n", e.what());
        return 1;
    }
    return 0;
}

// crg_host_selftest objrender <file.obj> <out> <W> <H> <spp>: load_model ->
// scene::add_model (indexed, expanded on the device) -> faithful renderer with
// the default sun, camera at (0, 0.5, -3) looking down +z, 60 degrees.
// out: u64 spp; float sums[W*H*3]
int obj_render(const char *file, const char *out, uint32_t W, uint32_t H, uint32_t spp) {
    try {
        scene sc(0);
        sc.add_model(load_model(file));
        camera *c = sc.camera();
        c->fov = 60.0f;
        c->rotate(vec3{0, 0, 0});
        c->position = vec3{0.0f, 0.5f, -3.0f};
        renderer::options o;
        o.mode = CRG_MODE_FAITHFUL;
        o.target_spp = spp;
        renderer r(W, H, 6, &sc, o);
        if (!r.wait_for_target(120.0)) return 1;
        const uint64_t n = r.current_sample_count();
        const std::vector<float> s1 = r.current_sums();
        FILE *g = std::fopen(out, "wb");
        if (!g) return 2;
        wr(g, &n, 1);
        wr(g, s1.data(), s1.size());
        std::fclose(g);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "selftest: %s\n", e.what());
        return 1;
    }
    return 0;
}

// crg_host_selftest extras <in> <out>: the same input as the main mode; drives
// draft_renderer, post_processor (bloom + Reinhard on a FULL-coverage
// processor) on the progress image of a short render, and scene::set_instances.
// out: float draft[W*H*4]; float progress[W*H*4]; float post[W*H*4];
//      per ray: u32 prim, float distance (two instances: identity and +0.25 in x)
int extras(const char *in, const char *out_path) {
    FILE *f = std::fopen(in, "rb");
    if (!f) return 2;
    uint32_t h[10];
    if (!rd(f, h, 10) || h[0] != 0x54475243u) return 2;
    const uint32_t ntri = h[1], nmat = h[2], W = h[3], H = h[4], spp = h[5], bounces = h[6], mode = h[7], nrays = h[8];
    std::vector<float> verts((size_t)ntri * 9);
    std::vector<uint32_t> mat_idx(ntri);
    std::vector<crg_material> mats(nmat);
    crg_camera cam;
    std::vector<crg_ray> rays(nrays);
    if (!rd(f, verts.data(), verts.size()) || !rd(f, mat_idx.data(), ntri) || !rd(f, mats.data(), nmat) ||
        !rd(f, &cam, 1) || !rd(f, rays.data(), nrays))
        return 2;
    std::fclose(f);
    try {
        scene sc(0);
        sc.add_model(make_model(verts, mat_idx, mats, 0, ntri));
        sc.set_sun_enabled(false);
        camera *c = sc.camera();
        c->fov = cam.fov;
        c->rotate(vec3{cam.rotation[0], cam.rotation[1], cam.rotation[2]});
        c->position = vec3{cam.position[0], cam.position[1], cam.position[2]};
        draft_renderer dr(&sc, W, H);
        const image draft = *dr.render();
        renderer::options o;
        o.mode = mode;
        o.target_spp = spp;
        renderer r(W, H, bounces, &sc, o);
        if (!r.wait_for_target(120.0)) return 1;
        const image progress = *r.current_progress();
        post_processor pp(&sc, false);
        pp.submit_bloom_settings({true, 0.6f, 0.8f});
        pp.submit_tonemapping_settings({true, 1, 1.2f, 2.2f});
        const image post = pp.process(progress);
        std::array<float, 16> id{}, moved{};
        for (int k = 0; k < 4; ++k) id[5 * k] = moved[5 * k] = 1.0f;
        moved[12] = 0.25f;
        sc.set_instances({id, moved});
        std::vector<ray> rr(nrays);
        for (uint32_t i = 0; i < nrays; ++i)
            rr[i] = ray{vec3{rays[i].org[0], rays[i].org[1], rays[i].org[2]},
                        vec3{rays[i].dir[0], rays[i].dir[1], rays[i].dir[2]}};
        const std::vector<intersection_record> recs = sc.cast_rays(rr);
        FILE *g = std::fopen(out_path, "wb");
        if (!g) return 2;
        wr(g, draft.data(), (size_t)W * H * 4);
        wr(g, progress.data(), (size_t)W * H * 4);
        wr(g, post.data(), (size_t)W * H * 4);
        for (const intersection_record &rec : recs) {
            const uint32_t prim = rec.material ? rec.prim_id : CRG_INVALID_PRIM;
            wr(g, &prim, 1);
            wr(g, &rec.distance, 1);
        }
        std::fclose(g);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "selftest: %s\n", e.what());
        return 1;
    }
    return 0;
}

} // namespace

int main(int argc, char **argv) {
    if (argc == 4 && std::strcmp(argv[1], "extras") == 0) return extras(argv[2], argv[3]);
    if (argc == 4 && std::strcmp(argv[1], "obj") == 0) return obj_parse(argv[2], argv[3]);
    if (argc == 7 && std::strcmp(argv[1], "objrender") == 0)
        return obj_render(argv[2], argv[3], (uint32_t)std::atoi(argv[4]), (uint32_t)std::atoi(argv[5]),
                          (uint32_t)std::atoi(argv[6]));
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <in> <out> | obj <file.obj> <out> | objrender <file.obj> <out> <W> <H> <spp>\n",
                     argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    uint32_t h[10];
    if (!rd(f, h, 10) || h[0] != 0x54475243u) return 2;
    const uint32_t ntri = h[1], nmat = h[2], W = h[3], H = h[4], spp = h[5], bounces = h[6], mode = h[7], nrays = h[8],
                   nsplit = h[9];
    std::vector<float> verts((size_t)ntri * 9);
    std::vector<uint32_t> mat_idx(ntri);
    std::vector<crg_material> mats(nmat);
    crg_camera cam;
    std::vector<crg_ray> rays(nrays);
    if (!rd(f, verts.data(), verts.size()) || !rd(f, mat_idx.data(), ntri) || !rd(f, mats.data(), nmat) ||
        !rd(f, &cam, 1) || !rd(f, rays.data(), nrays))
        return 2;
    std::fclose(f);
    try {
        scene sc(0);
        // the second model's material indices are relative to its own table
        std::vector<uint32_t> mi2(mat_idx);
        sc.add_model(make_model(verts, mat_idx, mats, 0, nsplit));
        if (nsplit < ntri) sc.add_model(make_model(verts, mi2, mats, nsplit, ntri));
        sc.set_sun_enabled(false);
        camera *c = sc.camera();
        c->fov = cam.fov;
        c->current_mode = cam.mode == CRG_CAMERA_PERSPECTIVE ? camera::mode::perspective : camera::mode::orthographic;
        c->scale = cam.scale;
        c->rotate(vec3{cam.rotation[0], cam.rotation[1], cam.rotation[2]});
        c->position = vec3{cam.position[0], cam.position[1], cam.position[2]};

        renderer::options o;
        o.mode = mode;
        o.target_spp = spp;
        renderer r(W, H, bounces, &sc, o);
        if (!r.wait_for_target(120.0)) {
            std::fprintf(stderr, "target spp not reached\n");
            return 1;
        }
        const uint64_t spp1 = r.current_sample_count();
        const std::vector<float> s1 = r.current_sums();
        const image *prog = r.current_progress();
        if (!prog->valid()) {
            std::fprintf(stderr, "no progress image\n");
            return 1;
        }
        // update(): pause, change the depth, restart from an empty film
        r.update([&] { r.set_max_bounces((int)bounces / 2); });
        if (!r.wait_for_target(120.0)) {
            std::fprintf(stderr, "target spp not reached after update()\n");
            return 1;
        }
        const uint64_t spp2 = r.current_sample_count();
        const std::vector<float> s2 = r.current_sums();
        const uint64_t total_rays = r.current_stats().total_rays;

        std::vector<ray> rr(nrays);
        for (uint32_t i = 0; i < nrays; ++i)
            rr[i] = ray{vec3{rays[i].org[0], rays[i].org[1], rays[i].org[2]},
                        vec3{rays[i].dir[0], rays[i].dir[1], rays[i].dir[2]}};
        const std::vector<intersection_record> recs = sc.cast_rays(rr);
        FILE *g = std::fopen(argv[2], "wb");
        if (!g) return 2;
        wr(g, &spp1, 1);
        wr(g, s1.data(), s1.size());
        wr(g, &spp2, 1);
        wr(g, s2.data(), s2.size());
        wr(g, &total_rays, 1);
        for (const intersection_record &rec : recs) {
            const uint32_t prim = rec.material ? rec.prim_id : CRG_INVALID_PRIM;
            const float row[4] = {rec.distance, rec.normal.x, rec.normal.y, rec.normal.z};
            wr(g, &prim, 1);
            wr(g, row, 4);
        }
        std::fclose(g);
    } catch (const std::exception &e) {
        std::fprintf(stderr, "selftest: %s\n", e.what());
        return 1;
    }
    return 0;
}
