// obj_loader.cpp — Wavefront OBJ / MTL reader for crg::host::load_model, the
// counterpart of cr::asset_loader::load_model (src/util/asset_loader.cpp:182-303,
// which reads through tinyobjloader).  Host-side I/O only: it fills a
// model_data whose indexed arrays crg::host::scene hands to
// crg_scene_create_indexed, so the de-indexing happens on the device.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <unordered_map>

#include "crg_host.h"

namespace crg::host {

namespace {

struct corner {
    int64_t v = 0, vt = 0, vn = 0; // as written (1-based, negative = relative, 0 = absent)
};

[[noreturn]] void bad(const std::string &file, size_t line, const std::string &what) {
    throw error(CRG_ERR_INVALID_ARG, file + ":" + std::to_string(line) + ": " + what);
}

// "v", "v/vt", "v//vn", "v/vt/vn"
bool parse_corner(const std::string &tok, corner &c) {
    const size_t s1 = tok.find('/');
    auto num = [](const std::string &x, int64_t &out) {
        if (x.empty()) {
            out = 0;
            return true;
        }
        char *end = nullptr;
        out = std::strtoll(x.c_str(), &end, 10);
        return end && *end == '\0' && out != 0;
    };
    if (s1 == std::string::npos) return num(tok, c.v) && c.v != 0;
    const size_t s2 = tok.find('/', s1 + 1);
    if (!num(tok.substr(0, s1), c.v) || c.v == 0) return false;
    if (s2 == std::string::npos) return num(tok.substr(s1 + 1), c.vt);
    return num(tok.substr(s1 + 1, s2 - s1 - 1), c.vt) && num(tok.substr(s2 + 1), c.vn);
}

// 1-based / negative OBJ index -> 0-based, or -1 when absent or out of range.
int64_t resolve(int64_t i, size_t count) {
    if (i > 0) return (size_t)i <= count ? i - 1 : -1;
    if (i < 0) return (int64_t)count + i >= 0 ? (int64_t)count + i : -1;
    return -1;
}

std::string trim(const std::string &s) {
    const size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    const size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

std::string join_path(const std::string &folder, const std::string &name) {
    if (folder.empty() || (!name.empty() && name[0] == '/')) return name;
    return folder.back() == '/' ? folder + name : folder + "/" + name;
}

// newmtl / Kd / map_Kd of an MTL file, in file order (tinyobjloader's material order).
void read_mtl(const std::string &path, std::vector<material_information> &mats, std::vector<std::string> &tex,
              std::unordered_map<std::string, uint32_t> &by_name) {
    std::ifstream in(path);
    if (!in) return; // a missing MTL leaves the faces on the default material, as tinyobjloader warns and goes on
    std::string line;
    size_t ln = 0;
    while (std::getline(in, line)) {
        ++ln;
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key) || key[0] == '#') continue;
        if (key == "newmtl") {
            std::string name;
            std::getline(ss, name);
            name = trim(name);
            material_information m;
            m.name = name;
            m.shade_type = material_information::smooth;
            m.emission = 0.0f;
            by_name[name] = (uint32_t)mats.size();
            mats.push_back(m);
            tex.emplace_back();
        } else if (key == "Kd" && !mats.empty()) {
            float r = 0, g = 0, b = 0;
            if (!(ss >> r)) bad(path, ln, "Kd without a value");
            if (!(ss >> g >> b)) g = b = r; // a single value sets all three channels
            mats.back().colour[0] = r;
            mats.back().colour[1] = g;
            mats.back().colour[2] = b;
            mats.back().colour[3] = 1.0f;
        } else if (key == "map_Kd" && !mats.empty()) {
            std::string rest, last;
            while (ss >> rest) last = rest; // options come first, the file name last
            tex.back() = last;
        }
    }
}

} // namespace

model_data load_model(const std::string &file, const std::string &folder_in) {
    std::ifstream in(file);
    if (!in) throw error(CRG_ERR_INVALID_ARG, "load_model: cannot open " + file);
    const size_t slash = file.find_last_of('/');
    const std::string folder = !folder_in.empty() ? folder_in : (slash == std::string::npos ? "" : file.substr(0, slash));
    model_data m;
    {
        const std::string base = slash == std::string::npos ? file : file.substr(slash + 1);
        const size_t dot = base.find_last_of('.');
        m.name = dot == std::string::npos ? base : base.substr(0, dot);
    }
    std::unordered_map<std::string, uint32_t> by_name;
    std::vector<std::string> tex_names;
    int64_t current = -1; // material of the faces that follow
    std::vector<int64_t> face_mat;
    std::string line;
    size_t ln = 0;
    std::vector<corner> poly;
    while (std::getline(in, line)) {
        ++ln;
        std::istringstream ss(line);
        std::string key;
        if (!(ss >> key) || key[0] == '#') continue;
        if (key == "v") {
            vec3 p;
            if (!(ss >> p.x >> p.y >> p.z)) bad(file, ln, "vertex needs three coordinates");
            m.vertices.push_back(p);
        } else if (key == "vt") {
            vec2 t;
            if (!(ss >> t.x)) bad(file, ln, "texture coordinate needs a value");
            if (!(ss >> t.y)) t.y = 0.0f;
            m.texture_coords.push_back(t);
        } else if (key == "vn") {
            vec3 n;
            if (!(ss >> n.x >> n.y >> n.z)) bad(file, ln, "normal needs three coordinates");
            m.normals.push_back(n);
        } else if (key == "f") {
            poly.clear();
            std::string tok;
            while (ss >> tok) {
                corner c;
                if (!parse_corner(tok, c)) bad(file, ln, "bad face corner '" + tok + "'");
                poly.push_back(c);
            }
            if (poly.size() < 3) continue; // degenerate face, skipped as tinyobjloader does
            std::vector<int64_t> vi(poly.size()), ti(poly.size()), ni(poly.size());
            bool ok = true;
            for (size_t k = 0; k < poly.size(); ++k) {
                vi[k] = resolve(poly[k].v, m.vertices.size());
                ti[k] = resolve(poly[k].vt, m.texture_coords.size());
                ni[k] = resolve(poly[k].vn, m.normals.size());
                if (vi[k] < 0) ok = false;
            }
            if (!ok) continue; // invalid vertex index: the face is skipped (tinyobjloader warns likewise)
            std::vector<size_t> tri; // corners, 3 per triangle
            if (poly.size() == 3) {
                tri = {0, 1, 2};
            } else if (poly.size() == 4) {
                // the shorter diagonal splits the quad (tinyobjloader's rule, float arithmetic)
                const vec3 &p0 = m.vertices[vi[0]], &p1 = m.vertices[vi[1]], &p2 = m.vertices[vi[2]],
                           &p3 = m.vertices[vi[3]];
                const float ax = p2.x - p0.x, ay = p2.y - p0.y, az = p2.z - p0.z;
                const float bx = p3.x - p1.x, by = p3.y - p1.y, bz = p3.z - p1.z;
                const float d02 = (ax * ax + ay * ay) + az * az, d13 = (bx * bx + by * by) + bz * bz;
                if (d02 < d13) tri = {0, 1, 2, 0, 2, 3};
                else tri = {0, 1, 3, 1, 2, 3};
            } else {
                for (size_t k = 1; k + 1 < poly.size(); ++k) tri.insert(tri.end(), {0, k, k + 1});
            }
            for (size_t c : tri) {
                m.vertex_indices.push_back((uint32_t)vi[c]);
                m.texture_indices.push_back(ti[c] >= 0 ? (uint32_t)ti[c] : 0xFFFFFFFFu);
                m.normal_indices.push_back(ni[c] >= 0 ? (uint32_t)ni[c] : 0xFFFFFFFFu);
            }
            for (size_t t = 0; t < tri.size() / 3; ++t) face_mat.push_back(current);
        } else if (key == "mtllib") {
            std::string name;
            while (ss >> name) read_mtl(join_path(folder, name), m.materials, tex_names, by_name);
        } else if (key == "usemtl") {
            std::string name;
            std::getline(ss, name);
            const auto it = by_name.find(trim(name));
            current = it == by_name.end() ? -1 : (int64_t)it->second;
        }
        // o, g, s, l, p and unknown records carry nothing the renderer uses
    }
    bool need_default = false;
    for (int64_t f : face_mat) need_default |= f < 0;
    const uint32_t fallback = (uint32_t)m.materials.size();
    if (need_default) {
        material_information d;
        d.name = "default";
        m.materials.push_back(d);
        tex_names.emplace_back();
    }
    for (int64_t f : face_mat) m.material_indices.push_back(f < 0 ? fallback : (uint32_t)f);
    m.texture_names = tex_names;
    bool any_uv = false;
    for (uint32_t t : m.texture_indices) any_uv |= t != 0xFFFFFFFFu;
    if (!any_uv) m.texture_indices.clear();
    return m;
}

} // namespace crg::host
