// crg_api.cu — the C ABI of include/crg.h.
//
// Handles own their device memory; every call returns a crg_status and
// records a message in the context.  Nothing here computes rays or samples:
// the host side only validates arguments, copies inputs, prepares the
// emissive-triangle table and launches kernels.
#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "crg_internal.h"

namespace crg {

namespace {
// Countdown of the armed allocation fault: -1 = disarmed, else the number of
// allocations still to succeed before one fails.
std::atomic<int64_t> g_fault_countdown{-1};
std::atomic<uint64_t> g_alloc_seen{0};
std::atomic<uint32_t> g_fault_fired{0};
} // namespace

bool fault_injected() {
    g_alloc_seen.fetch_add(1, std::memory_order_relaxed);
    int64_t c = g_fault_countdown.load(std::memory_order_relaxed);
    while (c >= 0) {
        if (g_fault_countdown.compare_exchange_weak(c, c - 1, std::memory_order_relaxed)) {
            if (c == 0) {
                g_fault_fired.fetch_add(1, std::memory_order_relaxed);
                return true;
            }
            return false;
        }
    }
    return false;
}

crg_status set_error(crg_context *ctx, crg_status s, const std::string &msg) {
    if (ctx) {
        std::lock_guard<std::mutex> lock(ctx->error_mutex);
        ctx->last_error = msg;
    }
    return s;
}

crg_status cuda_error(crg_context *ctx, cudaError_t e, const char *what) {
    const crg_status s = (e == cudaErrorMemoryAllocation) ? CRG_ERR_OOM : CRG_ERR_CUDA;
    return set_error(ctx, s, std::string(what) + ": " + cudaGetErrorString(e));
}

crg_status dev_alloc(crg_context *ctx, DevBuf &b, size_t bytes) {
    if (b.ptr && b.bytes >= bytes) return CRG_OK;
    dev_free(b);
    if (bytes == 0) return CRG_OK;
    if (fault_injected()) return set_error(ctx, CRG_ERR_OOM, "device allocation of " + std::to_string(bytes) +
                                                                 " bytes failed (injected fault)");
    void *p = nullptr;
    const cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return cuda_error(ctx, e, "cudaMalloc");
    }
    b.ptr = p;
    b.bytes = bytes;
    return CRG_OK;
}

void dev_free(DevBuf &b) {
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = nullptr;
    b.bytes = 0;
}

namespace {

// cr::sampling::build_local (src/util/sampling.h:21-33), host form.
void build_local_host(const float n[3], float t[3], float b[3]) {
    const float s = (n[2] < 0.0f) ? -1.0f : 1.0f;
    const float a = -1.0f / (s + n[2]);
    const float bb = n[0] * n[1] * a;
    t[0] = 1.0f + s * n[0] * n[0] * a;
    t[1] = s * bb;
    t[2] = -s * n[0];
    b[0] = bb;
    b[1] = s + n[1] * n[1] * a;
    b[2] = -n[1];
}

crg_sun default_sun() {
    // cr::entity::sun (src/render/entities/components.h:23-29)
    crg_sun s;
    s.size = 3.14159265359f / 48.0f;
    s.intensity = 100.0f;
    const float d[3] = {0.8f, -1.0f, 0.0f};
    const float inv = 1.0f / std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    s.direction[0] = d[0] * inv;
    s.direction[1] = d[1] * inv;
    s.direction[2] = d[2] * inv;
    s.colour[0] = 1.0f;
    s.colour[1] = 0.9f;
    s.colour[2] = 0.7f;
    return s;
}

void apply_sun(crg_scene *s, const crg_sun &sun) {
    s->sun = sun;
    const float n[3] = {-sun.direction[0], -sun.direction[1], -sun.direction[2]};
    float t[3], b[3];
    build_local_host(n, t, b);
    for (int k = 0; k < 3; ++k) {
        s->sun_frame[k] = t[k];
        s->sun_frame[3 + k] = n[k];
        s->sun_frame[6 + k] = b[k];
    }
    s->sun_cos = (float)std::cos((double)sun.size);
    s->sun_pdf = 1.0f / (6.28318530717f * (1.0f - s->sun_cos));
}

__global__ void k_fill_f32(float *a, size_t n, float v) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) a[i] = v;
}

__global__ void k_display(const float *__restrict__ sum, float4 *__restrict__ out, size_t npix, float inv_n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += (size_t)gridDim.x * blockDim.x) {
        const float r = fminf(fmaxf(sum[3 * i] * inv_n, 0.0f), 1.0f);
        const float g = fminf(fmaxf(sum[3 * i + 1] * inv_n, 0.0f), 1.0f);
        const float b = fminf(fmaxf(sum[3 * i + 2] * inv_n, 0.0f), 1.0f);
        out[i] = make_float4(powf(r, 1.0f / 2.2f), powf(g, 1.0f / 2.2f), powf(b, 1.0f / 2.2f), 1.0f);
    }
}

// persist_and_expand (registry.cpp:13-24) on the device: corner c of the
// de-indexed mesh takes position vidx[c] and texture coordinate tidx[c]
// ((0, 0) for -1 or an index past the coordinates).  Gathers 12 + 8 bytes and
// writes 12 + 8 bytes per corner.
__global__ void k_expand(const float *__restrict__ pos, const uint32_t *__restrict__ vidx, const float *__restrict__ tc,
                         const int32_t *__restrict__ tidx, uint32_t ntc, float *__restrict__ verts, float *__restrict__ uvs,
                         size_t ncorner) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncorner; c += (size_t)gridDim.x * blockDim.x) {
        const size_t k = vidx[c];
        verts[3 * c + 0] = pos[3 * k + 0];
        verts[3 * c + 1] = pos[3 * k + 1];
        verts[3 * c + 2] = pos[3 * k + 2];
        if (uvs) {
            const int32_t t = tidx ? tidx[c] : -1;
            float u = 0.0f, v = 0.0f;
            if (t >= 0 && (uint32_t)t < ntc) {
                u = tc[2 * (size_t)t];
                v = tc[2 * (size_t)t + 1];
            }
            uvs[2 * c + 0] = u;
            uvs[2 * c + 1] = v;
        }
    }
}

// Per-triangle areas in double from the float vertices (kept on the host so
// the emitter table can be rebuilt when materials change).
double tri_area_of(const float *v) {
    double e1[3], e2[3];
    for (int a = 0; a < 3; ++a) {
        e1[a] = (double)v[3 + a] - (double)v[a];
        e2[a] = (double)v[6 + a] - (double)v[a];
    }
    const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
    return 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
}

// Runs fn(begin, end) over [0, n) in contiguous ranges on up to 16 host
// threads (one range when n is small); each index is computed once, by the
// same code, so the results do not depend on the split.
template <class Fn>
void parallel_ranges(size_t n, Fn fn) {
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const size_t nt = n < (1u << 16) ? 1 : std::min<size_t>(std::min(16u, hw), n);
    if (nt <= 1) {
        fn((size_t)0, n);
        return;
    }
    std::vector<std::thread> pool;
    const size_t step = (n + nt - 1) / nt;
    try {
        for (size_t t = 1; t < nt; ++t) {
            const size_t b = t * step, e = std::min(n, b + step);
            if (b < e) pool.emplace_back(fn, b, e);
        }
    } catch (...) { // no thread could be started: the rest on this one
        const size_t done = (pool.size() + 1) * step;
        if (done < n) fn(done, n);
    }
    fn((size_t)0, std::min(n, step));
    for (auto &th : pool) th.join();
}

void compute_areas(crg_scene *s, const float *verts) {
    s->tri_area.assign(s->ntri, 0.0);
    double *a = s->tri_area.data();
    parallel_ranges(s->ntri, [a, verts](size_t b, size_t e) {
        for (size_t p = b; p < e; ++p) a[p] = tri_area_of(verts + p * 9);
    });
}

// Alias table (Walker 1977, built with Vose's 1991 two-worklist method in
// double, worklists scanned in index order so the table is reproducible) of
// the weights w: entry j = {prob_j, alias_j}; picking j = floor(u1 * n) and
// keeping it when u2 < prob_j, else taking alias_j, selects entry k with
// probability w_k / total in two loads instead of a binary search.
std::vector<float> alias_table(const std::vector<double> &w, double total) {
    const size_t n = w.size();
    std::vector<double> q(n);
    std::vector<uint32_t> small, large, alias(n);
    std::vector<double> prob(n, 1.0);
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
    std::vector<float> out(2 * n);
    for (size_t i = 0; i < n; ++i) {
        out[2 * i] = (float)prob[i];
        std::memcpy(&out[2 * i + 1], &alias[i], 4);
    }
    return out;
}

// Emissive triangles weighted by area x luminance of colour*emission (double
// sums in primitive order; CDF and pdfs rounded to float once).
crg_status prepare_lights(crg_scene *s) {
    const uint32_t nmat = s->nmat;
    std::vector<double> lum(nmat, 0.0);
    for (uint32_t m = 0; m < nmat; ++m) {
        const crg_material &mm = s->host_mats[m];
        if (mm.emission > 0.0f) {
            const float r = mm.colour[0] * mm.emission, g = mm.colour[1] * mm.emission, b = mm.colour[2] * mm.emission;
            lum[m] = 0.2126 * (double)r + 0.7152 * (double)g + 0.0722 * (double)b;
        }
    }
    std::vector<uint32_t> &mat_idx = s->host_mat_idx;
    std::vector<uint32_t> prim, inst;
    std::vector<double> w;
    double total = 0.0;
    // entries in placement-major, primitive order; an instanced scene holds one
    // copy of every emissive triangle of a placement's model, weighed by its world area
    const uint32_t ncopy = s->ninst ? s->ninst : 1;
    for (uint32_t j = 0; j < ncopy; ++j) {
        const uint32_t p0 = s->ninst ? s->models[s->place_model[j]].first : 0;
        const uint32_t p1 = s->ninst ? p0 + s->models[s->place_model[j]].ntri : s->ntri;
        for (uint32_t p = p0; p < p1; ++p) {
            const uint32_t m = mat_idx[p];
            if (!(lum[m] > 0.0)) continue;
            const double area = s->ninst ? s->inst_area[s->inst_area_off[j] + (p - p0)] : s->tri_area[p];
            const double wt = area * lum[m];
            prim.push_back(p);
            inst.push_back(j);
            w.push_back(wt);
            total += wt;
        }
    }
    std::vector<float> mpdf(nmat, 0.0f);
    s->nlights = 0;
    if (total > 0.0) {
        std::vector<float> pdf;
        for (size_t j = 0; j < w.size(); ++j) pdf.push_back((float)(lum[mat_idx[prim[j]]] / total));
        const std::vector<float> alias = alias_table(w, total);
        for (uint32_t m = 0; m < nmat; ++m) mpdf[m] = (float)(lum[m] / total);
        s->nlights = (uint32_t)prim.size();
        crg_status rc;
        if ((rc = dev_alloc(s->ctx, s->light_prim, 4 * prim.size())) != CRG_OK) return rc;
        if ((rc = dev_alloc(s->ctx, s->light_alias, 4 * alias.size())) != CRG_OK) return rc;
        if ((rc = dev_alloc(s->ctx, s->light_pdf, 4 * pdf.size())) != CRG_OK) return rc;
        CRG_CUDA(s->ctx, cudaMemcpy(s->light_prim.ptr, prim.data(), 4 * prim.size(), cudaMemcpyHostToDevice));
        CRG_CUDA(s->ctx, cudaMemcpy(s->light_alias.ptr, alias.data(), 4 * alias.size(), cudaMemcpyHostToDevice));
        CRG_CUDA(s->ctx, cudaMemcpy(s->light_pdf.ptr, pdf.data(), 4 * pdf.size(), cudaMemcpyHostToDevice));
        if (s->ninst) {
            if ((rc = dev_alloc(s->ctx, s->light_inst, 4 * inst.size())) != CRG_OK) return rc;
            CRG_CUDA(s->ctx, cudaMemcpy(s->light_inst.ptr, inst.data(), 4 * inst.size(), cudaMemcpyHostToDevice));
        }
    }
    crg_status rc;
    if ((rc = dev_alloc(s->ctx, s->mat_light_pdf, 4 * (size_t)(nmat ? nmat : 1))) != CRG_OK) return rc;
    if (nmat) CRG_CUDA(s->ctx, cudaMemcpy(s->mat_light_pdf.ptr, mpdf.data(), 4 * nmat, cudaMemcpyHostToDevice));
    return build_light_records(s);
}

// Affine 4x4 (column-major, glm::mat4 layout) -> device rows {inverse, forward}.
// The inverse is formed in double from the float entries (adjugate / det of
// the 3x3 part, t' = -A^-1 t) and rounded once.  False if the matrix is not
// affine or not invertible.
bool instance_rows(const float *x, float rows[24]) {
    if (x[3] != 0.0f || x[7] != 0.0f || x[11] != 0.0f || x[15] != 1.0f) return false;
    double a[3][3], t[3];
    for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) a[r][c] = (double)x[4 * c + r];
        t[r] = (double)x[12 + r];
    }
    const double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    const double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    const double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    const double det = (a[0][0] * c00 + a[0][1] * c01) + a[0][2] * c02;
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    double inv[3][3];
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
        const double ti = -((inv[r][0] * t[0] + inv[r][1] * t[1]) + inv[r][2] * t[2]);
        for (int c = 0; c < 3; ++c) rows[4 * r + c] = (float)inv[r][c];
        rows[4 * r + 3] = (float)ti;
        for (int c = 0; c < 3; ++c) rows[12 + 4 * r + c] = x[4 * c + r];
        rows[12 + 4 * r + 3] = x[12 + r];
    }
    for (int k = 0; k < 24; ++k)
        if (!std::isfinite(rows[k])) return false;
    return true;
}

// World areas (double) of every triangle of each placement's model under its transform.
void instance_areas(crg_scene *s, const float *verts) {
    s->inst_area.clear();
    s->inst_area_off.assign(s->ninst, 0);
    for (uint32_t j = 0; j < s->ninst; ++j) {
        const float *x = &s->host_xf[16 * (size_t)j];
        const crg_model_rec &md = s->models[s->place_model[j]];
        s->inst_area_off[j] = s->inst_area.size();
        for (uint32_t p = md.first; p < md.first + md.ntri; ++p) {
            double w[3][3];
            for (int k = 0; k < 3; ++k) {
                const float *v = verts + (size_t)p * 9 + 3 * k;
                for (int r = 0; r < 3; ++r)
                    w[k][r] = (((double)x[r] * v[0] + (double)x[4 + r] * v[1]) + (double)x[8 + r] * v[2]) + (double)x[12 + r];
            }
            double e1[3], e2[3];
            for (int r = 0; r < 3; ++r) {
                e1[r] = w[1][r] - w[0][r];
                e2[r] = w[2][r] - w[0][r];
            }
            const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                         cz = e1[0] * e2[1] - e1[1] * e2[0];
            s->inst_area.push_back(0.5 * std::sqrt(cx * cx + cy * cy + cz * cz));
        }
    }
}

// Object-space bounds of ntri de-indexed triangles (host float[ntri*9]).
void mesh_box(const float *v, uint32_t ntri, float box[6]) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t k = 0; k < 3 * (size_t)ntri; ++k) {
        const float *p = v + 3 * k;
        for (int a = 0; a < 3; ++a) {
            lo[a] = p[a] < lo[a] ? p[a] : lo[a];
            hi[a] = p[a] > hi[a] ? p[a] : hi[a];
        }
    }
    for (int a = 0; a < 3; ++a) {
        box[a] = ntri ? lo[a] : 0.0f;
        box[3 + a] = ntri ? hi[a] : 0.0f;
    }
}

const float kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

// World box of a model's object box under a column-major affine transform,
// from its 8 corners in double, widened outwards by 1e-5 of its size and of
// its distance from the origin so that every rounded world point of a hit
// lies inside it.
void world_box(const float box[6], const float *x, double out[6]) {
    for (int a = 0; a < 3; ++a) {
        out[a] = INFINITY;
        out[3 + a] = -INFINITY;
    }
    for (int c = 0; c < 8; ++c) {
        const double p[3] = {box[(c & 1) ? 3 : 0], box[(c & 2) ? 4 : 1], box[(c & 4) ? 5 : 2]};
        for (int r = 0; r < 3; ++r) {
            const double w = (((double)x[r] * p[0] + (double)x[4 + r] * p[1]) + (double)x[8 + r] * p[2]) + (double)x[12 + r];
            out[r] = std::min(out[r], w);
            out[3 + r] = std::max(out[3 + r], w);
        }
    }
    double mag = 0.0, ext = 0.0;
    for (int a = 0; a < 3; ++a) {
        mag = std::max(mag, std::max(std::fabs(out[a]), std::fabs(out[3 + a])));
        ext = std::max(ext, out[3 + a] - out[a]);
    }
    const double pad = 1e-5 * (mag + ext) + 1e-30;
    for (int a = 0; a < 3; ++a) {
        out[a] -= pad;
        out[3 + a] += pad;
    }
}

// Top-level tree over the placements' world boxes: a binary tree split at the
// median placement along the widest axis of the box centres (ties by placement
// index), nodes in pre-order.  Node i is 4 float4: {lo_a.xyz, ref_a},
// {hi_a.xyz, ref_b}, {lo_b.xyz, 0}, {hi_b.xyz, 0}; a ref is a node index, or
// kTlasLeaf | placement.  Boxes are rounded outwards to float.
struct TlasBuilder {
    const std::vector<std::array<double, 6>> &box;
    std::vector<float> nodes; // 16 floats per node
    std::array<double, 6> bounds(const std::vector<uint32_t> &ids, size_t b, size_t e) const {
        std::array<double, 6> r{INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        for (size_t i = b; i < e; ++i)
            for (int a = 0; a < 3; ++a) {
                r[a] = std::min(r[a], box[ids[i]][a]);
                r[3 + a] = std::max(r[3 + a], box[ids[i]][3 + a]);
            }
        return r;
    }
    static float down(double v) {
        float f = (float)v;
        if ((double)f > v) f = std::nextafter(f, -INFINITY);
        return f;
    }
    static float up(double v) {
        float f = (float)v;
        if ((double)f < v) f = std::nextafter(f, INFINITY);
        return f;
    }
    // returns the ref of the subtree over ids[b, e)
    uint32_t build(std::vector<uint32_t> &ids, size_t b, size_t e) {
        if (e - b == 1) return kTlasLeaf | ids[b];
        const uint32_t me = (uint32_t)(nodes.size() / 16);
        nodes.resize(nodes.size() + 16, 0.0f);
        double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (size_t i = b; i < e; ++i)
            for (int a = 0; a < 3; ++a) {
                const double c = 0.5 * (box[ids[i]][a] + box[ids[i]][3 + a]);
                clo[a] = std::min(clo[a], c);
                chi[a] = std::max(chi[a], c);
            }
        int ax = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[ax] - clo[ax]) ax = a;
        std::sort(ids.begin() + b, ids.begin() + e, [&](uint32_t p, uint32_t q) {
            const double cp = box[p][ax] + box[p][3 + ax], cq = box[q][ax] + box[q][3 + ax];
            return cp < cq || (cp == cq && p < q);
        });
        const size_t mid = b + (e - b) / 2;
        const std::array<double, 6> la = bounds(ids, b, mid), lb = bounds(ids, mid, e);
        const uint32_t ra = build(ids, b, mid);
        const uint32_t rb = build(ids, mid, e);
        float *n = &nodes[16 * (size_t)me];
        for (int a = 0; a < 3; ++a) {
            n[a] = down(la[a]);
            n[4 + a] = up(la[3 + a]);
            n[8 + a] = down(lb[a]);
            n[12 + a] = up(lb[3 + a]);
        }
        std::memcpy(&n[3], &ra, 4);
        std::memcpy(&n[7], &rb, 4);
        return me;
    }
};

// Rebuilds the placement list of a scene from its models' instance lists:
// device transform rows, BVH roots, the top-level tree and the world areas of
// emitter copies.  A scene of one model without a list has no placements.
crg_status update_placements(crg_scene *s) {
    crg_context *ctx = s->ctx;
    const bool flat = s->models.size() == 1 && s->models[0].xf.empty();
    s->ninst = 0;
    s->host_xf.clear();
    s->host_rows.clear();
    s->place_model.clear();
    s->inst_area.clear();
    s->inst_area_off.clear();
    s->tlas_root = 0;
    s->tlas_nodes = 0;
    dev_free(s->inst);
    dev_free(s->inst_root);
    dev_free(s->tlas);
    dev_free(s->light_inst);
    if (flat) return CRG_OK;
    // the vertices come back to the host once: model boxes (for the top-level
    // tree) and the world areas of emitter copies
    std::vector<float> hv((size_t)s->ntri * 9);
    if (s->ntri) CRG_CUDA(ctx, cudaMemcpy(hv.data(), s->verts.ptr, sizeof(float) * hv.size(), cudaMemcpyDeviceToHost));
    for (crg_model_rec &md : s->models)
        if (!md.box_valid) {
            mesh_box(hv.data() + (size_t)md.first * 9, md.ntri, md.box);
            md.box_valid = true;
        }
    std::vector<uint32_t> roots;
    std::vector<std::array<double, 6>> boxes;
    for (uint32_t m = 0; m < (uint32_t)s->models.size(); ++m) {
        const crg_model_rec &md = s->models[m];
        const uint32_t count = md.xf.empty() ? 1u : (uint32_t)(md.xf.size() / 16);
        for (uint32_t j = 0; j < count; ++j) {
            const float *x = md.xf.empty() ? kIdentity : &md.xf[16 * (size_t)j];
            float rows[24];
            if (!instance_rows(x, rows)) return set_error(ctx, CRG_ERR_INVALID_ARG, "instance transform is not invertible");
            s->host_xf.insert(s->host_xf.end(), x, x + 16);
            s->host_rows.insert(s->host_rows.end(), rows, rows + 24);
            s->place_model.push_back(m);
            roots.push_back(md.node_base);
            std::array<double, 6> wb;
            world_box(md.box, x, wb.data());
            boxes.push_back(wb);
        }
    }
    const uint32_t np = (uint32_t)s->place_model.size();
    if (np > (1u << 20)) return set_error(ctx, CRG_ERR_INVALID_ARG, "more than 2^20 placements");
    TlasBuilder tb{boxes, {}};
    std::vector<uint32_t> ids(np);
    for (uint32_t k = 0; k < np; ++k) ids[k] = k;
    const uint32_t root = tb.build(ids, 0, np);
    crg_status rc;
    if ((rc = dev_alloc(ctx, s->inst, sizeof(float) * s->host_rows.size())) != CRG_OK) return rc;
    if ((rc = dev_alloc(ctx, s->inst_root, sizeof(uint32_t) * np)) != CRG_OK) return rc;
    if (!tb.nodes.empty() && (rc = dev_alloc(ctx, s->tlas, sizeof(float) * tb.nodes.size())) != CRG_OK) return rc;
    CRG_CUDA(ctx, cudaMemcpy(s->inst.ptr, s->host_rows.data(), sizeof(float) * s->host_rows.size(), cudaMemcpyHostToDevice));
    CRG_CUDA(ctx, cudaMemcpy(s->inst_root.ptr, roots.data(), sizeof(uint32_t) * np, cudaMemcpyHostToDevice));
    if (!tb.nodes.empty())
        CRG_CUDA(ctx, cudaMemcpy(s->tlas.ptr, tb.nodes.data(), sizeof(float) * tb.nodes.size(), cudaMemcpyHostToDevice));
    s->tlas_root = root;
    s->tlas_nodes = (uint32_t)(tb.nodes.size() / 16);
    s->ninst = np;
    instance_areas(s, hv.data());
    return CRG_OK;
}

// Copies the first `keep` bytes of src into a fresh buffer of `bytes` bytes.
crg_status copy_grow(crg_context *ctx, const DevBuf &src, size_t keep, size_t bytes, DevBuf &out) {
    crg_status rc = dev_alloc(ctx, out, bytes);
    if (rc != CRG_OK) return rc;
    if (src.ptr && keep) CRG_CUDA(ctx, cudaMemcpy(out.ptr, src.ptr, keep, cudaMemcpyDeviceToDevice));
    return CRG_OK;
}

// cr::registry::register_model (registry.cpp:51-97) for a scene that already
// exists: the model's triangles are appended to the scene's arrays (its
// material indices rebased onto the appended materials) and it gets its own
// BVH region; only its BVH is built by the next crg_scene_build.  fill(d_verts,
// d_uvs, box, areas) writes the model's de-indexed vertices (and texture
// coordinates when d_uvs is not null), its object box and its triangle areas.
// The scene is left unchanged when a step fails.
template <class Fill>
crg_status append_model(crg_scene *s, uint32_t ntri, const uint32_t *mat_idx, const crg_material *mats, uint32_t nmat,
                        uint32_t *model, Fill &&fill, bool model_uv) {
    crg_context *ctx = s->ctx;
    if (ntri > 0 && (!mat_idx || !mats || nmat == 0))
        return set_error(ctx, CRG_ERR_INVALID_ARG, "triangles need mat_idx and a non-empty material table");
    if ((uint64_t)s->ntri + ntri > (1u << 30)) return set_error(ctx, CRG_ERR_INVALID_ARG, "more than 2^30 triangles");
    if (s->models.size() >= (1u << 16)) return set_error(ctx, CRG_ERR_INVALID_ARG, "more than 65536 models");
    for (uint32_t p = 0; p < ntri; ++p)
        if (mat_idx[p] >= nmat) return set_error(ctx, CRG_ERR_INVALID_ARG, "material index out of range");
    for (uint32_t m = 0; m < nmat; ++m)
        if (mats[m].shade_type > CRG_SHADE_GLASS) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad shade_type");
    const uint32_t n0 = s->ntri, m0 = s->nmat, n1 = n0 + ntri, m1 = m0 + nmat;
    const bool uv = s->uvs.ptr != nullptr || model_uv;
    DevBuf verts, uvs, midx, dmats;
    std::vector<uint32_t> shifted(mat_idx, mat_idx + ntri);
    for (uint32_t &k : shifted) k += m0;
    crg_model_rec rec;
    rec.first = n0;
    rec.ntri = ntri;
    rec.node_base = 0;
    for (const crg_model_rec &m : s->models) rec.node_base = std::max(rec.node_base, m.node_base + m.node_cap);
    rec.node_cap = ntri >= 2 ? ntri - 1 : 1;
    std::vector<double> areas;
    crg_status rc = copy_grow(ctx, s->verts, sizeof(float) * 9 * (size_t)n0, sizeof(float) * 9 * (size_t)std::max(n1, 1u), verts);
    if (rc == CRG_OK && uv) {
        rc = copy_grow(ctx, s->uvs, s->uvs.ptr ? sizeof(float) * 6 * (size_t)n0 : 0, sizeof(float) * 6 * (size_t)std::max(n1, 1u), uvs);
        if (rc == CRG_OK && !s->uvs.ptr && n0) {
            const cudaError_t e = cudaMemset(uvs.ptr, 0, sizeof(float) * 6 * (size_t)n0);
            if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaMemset(uvs)");
        }
    }
    if (rc == CRG_OK) rc = copy_grow(ctx, s->mat_idx, sizeof(uint32_t) * n0, sizeof(uint32_t) * std::max(n1, 1u), midx);
    if (rc == CRG_OK) rc = copy_grow(ctx, s->mats, sizeof(crg_material) * m0, sizeof(crg_material) * std::max(m1, 1u), dmats);
    if (rc == CRG_OK && ntri) {
        const cudaError_t e = cudaMemcpy((uint32_t *)midx.ptr + n0, shifted.data(), sizeof(uint32_t) * ntri, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaMemcpy(mat_idx)");
    }
    if (rc == CRG_OK && nmat) {
        const cudaError_t e = cudaMemcpy((crg_material *)dmats.ptr + m0, mats, sizeof(crg_material) * nmat, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaMemcpy(materials)");
    }
    if (rc == CRG_OK) rc = fill((float *)verts.ptr + 9 * (size_t)n0, uv ? (float *)uvs.ptr + 6 * (size_t)n0 : nullptr, rec.box, areas);
    if (rc != CRG_OK) {
        dev_free(verts);
        dev_free(uvs);
        dev_free(midx);
        dev_free(dmats);
        return rc;
    }
    dev_free(s->verts);
    s->verts = verts;
    if (uv) {
        dev_free(s->uvs);
        s->uvs = uvs;
    }
    dev_free(s->mat_idx);
    s->mat_idx = midx;
    dev_free(s->mats);
    s->mats = dmats;
    s->host_mat_idx.insert(s->host_mat_idx.end(), shifted.begin(), shifted.end());
    s->host_mats.insert(s->host_mats.end(), mats, mats + nmat);
    s->tri_area.insert(s->tri_area.end(), areas.begin(), areas.end());
    s->models.push_back(rec);
    s->ntri = n1;
    s->nmat = m1;
    s->built = false;
    if (model) *model = (uint32_t)(s->models.size() - 1);
    rc = update_placements(s);
    if (rc == CRG_OK) rc = prepare_lights(s);
    return rc;
}

crg_status scene_common(crg_context *ctx, uint32_t ntri, const uint32_t *mat_idx, const crg_material *mats, uint32_t nmat,
                        crg_scene **out, crg_scene *&s) {
    if (!ctx || !out) return set_error(ctx, CRG_ERR_INVALID_ARG, "null context or output handle");
    if (ntri > 0 && (!mat_idx || !mats || nmat == 0))
        return set_error(ctx, CRG_ERR_INVALID_ARG, "triangles need mat_idx and a non-empty material table");
    if (ntri > (1u << 30)) return set_error(ctx, CRG_ERR_INVALID_ARG, "more than 2^30 triangles");
    for (uint32_t p = 0; p < ntri; ++p)
        if (mat_idx[p] >= nmat) return set_error(ctx, CRG_ERR_INVALID_ARG, "material index out of range");
    for (uint32_t m = 0; m < nmat; ++m)
        if (mats[m].shade_type > CRG_SHADE_GLASS) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad shade_type");
    s = fault_injected() ? nullptr : new (std::nothrow) crg_scene();
    if (!s) return set_error(ctx, CRG_ERR_OOM, "host allocation of the scene failed");
    s->ctx = ctx;
    s->ntri = ntri;
    s->nmat = nmat;
    s->host_mats.assign(mats, mats + nmat);
    s->host_mat_idx.assign(mat_idx, mat_idx + ntri);
    crg_model_rec m0;
    m0.first = 0;
    m0.ntri = ntri;
    m0.node_base = 0;
    m0.node_cap = ntri >= 2 ? ntri - 1 : 1;
    s->models.push_back(m0);
    apply_sun(s, default_sun());
    s->sun_enabled = 0;
    crg_status rc;
    if ((rc = dev_alloc(ctx, s->mat_idx, sizeof(uint32_t) * (size_t)(ntri ? ntri : 1))) != CRG_OK) return rc;
    if ((rc = dev_alloc(ctx, s->mats, sizeof(crg_material) * (size_t)(nmat ? nmat : 1))) != CRG_OK) return rc;
    if ((rc = dev_alloc(ctx, s->err, 64)) != CRG_OK) return rc;
    if ((rc = dev_alloc(ctx, s->counters, 64)) != CRG_OK) return rc;
    if ((rc = dev_alloc(ctx, s->qhead, 64)) != CRG_OK) return rc;
    CRG_CUDA(ctx, cudaMemset(s->err.ptr, 0, 64));
    CRG_CUDA(ctx, cudaMemset(s->counters.ptr, 0, 64));
    if (ntri) CRG_CUDA(ctx, cudaMemcpy(s->mat_idx.ptr, mat_idx, sizeof(uint32_t) * ntri, cudaMemcpyHostToDevice));
    if (nmat) CRG_CUDA(ctx, cudaMemcpy(s->mats.ptr, mats, sizeof(crg_material) * nmat, cudaMemcpyHostToDevice));
    return CRG_OK;
}

void scene_free(crg_scene *s) {
    if (!s) return;
    DevBuf *bufs[] = {&s->verts, &s->mat_idx, &s->mats, &s->light_prim, &s->light_alias, &s->light_pdf, &s->mat_light_pdf,
                      &s->sky, &s->bvh2, &s->order, &s->wide, &s->tris, &s->err, &s->counters, &s->qhead,
                      &s->uvs, &s->texels, &s->tex_info, &s->inst, &s->light_inst, &s->light_rec,
                      &s->inst_root, &s->tlas};
    for (DevBuf *b : bufs) dev_free(*b);
    delete s;
}

bool valid_opts(const crg_build_opts &o) {
    return (o.width == 2 || o.width == 4 || o.width == 8) && o.leaf_max >= 1 && o.leaf_max <= 3 && o.treelet_rounds <= 8;
}

} // namespace
} // namespace crg

using namespace crg;

extern "C" {

uint32_t crg_abi_version(void) { return CRG_ABI_VERSION; }

crg_status crg_debug_fail_allocation(int64_t nth) {
    g_fault_countdown.store(nth < 0 ? -1 : nth, std::memory_order_relaxed);
    return CRG_OK;
}

crg_status crg_debug_allocation_stats(uint64_t *allocations, uint32_t *injected, int64_t *armed) {
    if (allocations) *allocations = g_alloc_seen.load(std::memory_order_relaxed);
    if (injected) *injected = g_fault_fired.load(std::memory_order_relaxed);
    if (armed) *armed = g_fault_countdown.load(std::memory_order_relaxed);
    return CRG_OK;
}

const char *crg_status_string(crg_status s) {
    switch (s) {
    case CRG_OK: return "OK";
    case CRG_ERR_INVALID_ARG: return "INVALID_ARG";
    case CRG_ERR_OOM: return "OOM";
    case CRG_ERR_CUDA: return "CUDA";
    case CRG_ERR_TIMEOUT: return "TIMEOUT";
    case CRG_ERR_NOT_BUILT: return "NOT_BUILT";
    case CRG_ERR_UNSUPPORTED: return "UNSUPPORTED";
    case CRG_ERR_DEVICE: return "DEVICE";
    }
    return "UNKNOWN";
}

crg_status crg_context_create(int device, crg_context **out) {
    if (!out) return CRG_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || device < 0 || device >= count) {
        (void)cudaGetLastError();
        return e != cudaSuccess ? CRG_ERR_CUDA : CRG_ERR_INVALID_ARG;
    }
    if ((e = cudaSetDevice(device)) != cudaSuccess) return CRG_ERR_CUDA;
    crg_context *ctx = fault_injected() ? nullptr : new (std::nothrow) crg_context();
    if (!ctx) return CRG_ERR_OOM;
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    // crg_build_bvh_noalloc's scratch array: its module is loaded and its address
    // looked up here, so that the no-allocation build itself loads nothing
    noalloc_prepare();
    *out = ctx;
    return CRG_OK;
}

crg_status crg_context_destroy(crg_context *ctx) {
    if (!ctx) return CRG_ERR_INVALID_ARG;
    batch_state_free(ctx);
    dev_free(ctx->wf_ws);
    dev_free(ctx->post_ws);
    delete ctx;
    return CRG_OK;
}

const char *crg_last_error_string(const crg_context *ctx) {
    if (!ctx) return "null context";
    // a copy per calling thread: the context's message may be replaced by another thread's error
    thread_local std::string copy;
    std::lock_guard<std::mutex> lock(ctx->error_mutex);
    copy = ctx->last_error;
    return copy.c_str();
}

crg_status crg_device_alloc(crg_context *ctx, size_t bytes, void **dptr) {
    if (!ctx || !dptr) return set_error(ctx, CRG_ERR_INVALID_ARG, "null argument");
    *dptr = nullptr;
    if (bytes == 0) return CRG_OK;
    if (fault_injected()) return set_error(ctx, CRG_ERR_OOM, "crg_device_alloc failed (injected fault)");
    CRG_CUDA(ctx, cudaMalloc(dptr, bytes));
    return CRG_OK;
}

crg_status crg_device_free(crg_context *ctx, void *dptr) {
    if (!ctx) return CRG_ERR_INVALID_ARG;
    if (dptr) CRG_CUDA(ctx, cudaFree(dptr));
    return CRG_OK;
}

crg_status crg_memcpy_h2d(crg_context *ctx, void *dst, const void *src, size_t bytes, crg_stream stream) {
    if (!ctx || (bytes && (!dst || !src))) return set_error(ctx, CRG_ERR_INVALID_ARG, "null argument");
    if (bytes) CRG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    return CRG_OK;
}

crg_status crg_memcpy_d2h(crg_context *ctx, void *dst, const void *src, size_t bytes, crg_stream stream) {
    if (!ctx || (bytes && (!dst || !src))) return set_error(ctx, CRG_ERR_INVALID_ARG, "null argument");
    if (bytes) CRG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    return CRG_OK;
}

crg_status crg_host_alloc(crg_context *ctx, size_t bytes, void **hptr) {
    if (!ctx || !hptr) return set_error(ctx, CRG_ERR_INVALID_ARG, "null argument");
    *hptr = nullptr;
    if (bytes == 0) return CRG_OK;
    if (fault_injected()) return set_error(ctx, CRG_ERR_OOM, "crg_host_alloc failed (injected fault)");
    CRG_CUDA(ctx, cudaHostAlloc(hptr, bytes, cudaHostAllocDefault));
    return CRG_OK;
}

crg_status crg_host_free(crg_context *ctx, void *hptr) {
    if (!ctx) return CRG_ERR_INVALID_ARG;
    if (hptr) CRG_CUDA(ctx, cudaFreeHost(hptr));
    return CRG_OK;
}

crg_status crg_stream_sync(crg_context *ctx, crg_stream stream) {
    if (!ctx) return CRG_ERR_INVALID_ARG;
    CRG_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
    return CRG_OK;
}

crg_status crg_scene_create(crg_context *ctx, const float *verts, uint32_t ntri, const float *uvs, const uint32_t *mat_idx,
                            const crg_material *mats, uint32_t nmat, crg_scene **out) {
    if (ntri > 0 && !verts) return set_error(ctx, CRG_ERR_INVALID_ARG, "null vertex array");
    if (out) *out = nullptr;
    crg_scene *s = nullptr;
    crg_status rc = scene_common(ctx, ntri, mat_idx, mats, nmat, out, s);
    if (rc == CRG_OK) rc = dev_alloc(ctx, s->verts, sizeof(float) * 9 * (size_t)(ntri ? ntri : 1));
    if (rc == CRG_OK && ntri) {
        const cudaError_t e = cudaMemcpy(s->verts.ptr, verts, sizeof(float) * 9 * (size_t)ntri, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaMemcpy(verts)");
    }
    // per-corner texture coordinates (the ATTRIBUTE buffer of model.cpp:80-90)
    if (rc == CRG_OK && ntri && uvs) rc = dev_alloc(ctx, s->uvs, sizeof(float) * 6 * (size_t)ntri);
    if (rc == CRG_OK && ntri && uvs) {
        const cudaError_t e = cudaMemcpy(s->uvs.ptr, uvs, sizeof(float) * 6 * (size_t)ntri, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaMemcpy(uvs)");
    }
    if (rc == CRG_OK) {
        compute_areas(s, verts);
        rc = prepare_lights(s);
    }
    if (rc != CRG_OK) {
        scene_free(s);
        return rc;
    }
    *out = s;
    return CRG_OK;
}

crg_status crg_scene_create_indexed(crg_context *ctx, const float *positions, uint32_t npos, const uint32_t *vertex_indices,
                                    uint32_t ntri, const float *texcoords, uint32_t ntc, const int32_t *tex_indices,
                                    const uint32_t *mat_idx, const crg_material *mats, uint32_t nmat, crg_scene **out) {
    if (ntri > 0 && (!positions || !vertex_indices)) return set_error(ctx, CRG_ERR_INVALID_ARG, "null positions or indices");
    if (ntc > 0 && !texcoords) return set_error(ctx, CRG_ERR_INVALID_ARG, "null texture coordinates");
    if (out) *out = nullptr;
    for (size_t c = 0; c < 3 * (size_t)ntri; ++c)
        if (vertex_indices[c] >= npos) return set_error(ctx, CRG_ERR_INVALID_ARG, "vertex index out of range");
    crg_scene *s = nullptr;
    crg_status rc = scene_common(ctx, ntri, mat_idx, mats, nmat, out, s);
    const bool want_uv = tex_indices != nullptr;
    DevBuf dpos, didx, dtc, dti;
    const size_t nc = 3 * (size_t)ntri;
    if (rc == CRG_OK) rc = dev_alloc(ctx, s->verts, sizeof(float) * 9 * (size_t)(ntri ? ntri : 1));
    if (rc == CRG_OK && ntri) {
        if (rc == CRG_OK) rc = dev_alloc(ctx, dpos, sizeof(float) * 3 * (size_t)npos);
        if (rc == CRG_OK) rc = dev_alloc(ctx, didx, sizeof(uint32_t) * nc);
        if (rc == CRG_OK && want_uv) rc = dev_alloc(ctx, s->uvs, sizeof(float) * 6 * (size_t)ntri);
        if (rc == CRG_OK && want_uv) rc = dev_alloc(ctx, dti, sizeof(int32_t) * nc);
        if (rc == CRG_OK && want_uv && ntc) rc = dev_alloc(ctx, dtc, sizeof(float) * 2 * (size_t)ntc);
        cudaError_t e = cudaSuccess;
        if (rc == CRG_OK) e = cudaMemcpy(dpos.ptr, positions, sizeof(float) * 3 * (size_t)npos, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess) e = cudaMemcpy(didx.ptr, vertex_indices, sizeof(uint32_t) * nc, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess && want_uv)
            e = cudaMemcpy(dti.ptr, tex_indices, sizeof(int32_t) * nc, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess && want_uv && ntc)
            e = cudaMemcpy(dtc.ptr, texcoords, sizeof(float) * 2 * (size_t)ntc, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess) {
            const unsigned blocks = (unsigned)std::min<size_t>((nc + 255) / 256, (size_t)std::max(ctx->sm_count, 1) * 8);
            k_expand<<<blocks, 256>>>((const float *)dpos.ptr, (const uint32_t *)didx.ptr, (const float *)dtc.ptr,
                                      (const int32_t *)dti.ptr, want_uv ? ntc : 0, (float *)s->verts.ptr,
                                      want_uv ? (float *)s->uvs.ptr : nullptr, nc);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
        }
        if (rc == CRG_OK && e != cudaSuccess) rc = cuda_error(ctx, e, "k_expand");
    }
    dev_free(dpos);
    dev_free(didx);
    dev_free(dtc);
    dev_free(dti);
    if (rc == CRG_OK) {
        // emitter areas from the same float positions the device copied
        float tv[9];
        s->tri_area.assign(ntri, 0.0);
        for (uint32_t p = 0; p < ntri; ++p) {
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) tv[3 * k + a] = positions[3 * (size_t)vertex_indices[3 * (size_t)p + k] + a];
            s->tri_area[p] = tri_area_of(tv);
        }
        rc = prepare_lights(s);
    }
    if (rc != CRG_OK) {
        scene_free(s);
        return rc;
    }
    *out = s;
    return CRG_OK;
}

crg_status crg_scene_create_device(crg_context *ctx, const float *d_verts, uint32_t ntri, const uint32_t *mat_idx,
                                   const crg_material *mats, uint32_t nmat, crg_scene **out) {
    if (ntri > 0 && !d_verts) return set_error(ctx, CRG_ERR_INVALID_ARG, "null vertex array");
    if (out) *out = nullptr;
    crg_scene *s = nullptr;
    crg_status rc = scene_common(ctx, ntri, mat_idx, mats, nmat, out, s);
    if (rc == CRG_OK) rc = dev_alloc(ctx, s->verts, sizeof(float) * 9 * (size_t)(ntri ? ntri : 1));
    std::vector<float> hv;
    if (rc == CRG_OK && ntri) {
        cudaError_t e = cudaMemcpy(s->verts.ptr, d_verts, sizeof(float) * 9 * (size_t)ntri, cudaMemcpyDeviceToDevice);
        if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaMemcpy(verts)");
        // the emissive-triangle table needs the vertices of emitters only; a
        // host copy keeps its construction identical to crg_scene_create
        if (rc == CRG_OK) {
            hv.resize((size_t)ntri * 9);
            e = cudaMemcpy(hv.data(), d_verts, sizeof(float) * 9 * (size_t)ntri, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaMemcpy(verts to host)");
        }
    }
    if (rc == CRG_OK) {
        compute_areas(s, hv.data());
        rc = prepare_lights(s);
    }
    if (rc != CRG_OK) {
        scene_free(s);
        return rc;
    }
    *out = s;
    return CRG_OK;
}

crg_status crg_scene_destroy(crg_scene *scene) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    scene_free(scene);
    return CRG_OK;
}

crg_status crg_scene_build(crg_scene *scene, const crg_build_opts *opts, crg_stream stream) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    crg_build_opts o{8, 0, 3, 3};
    if (opts) o = *opts;
    if (!valid_opts(o)) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "build options: width 2/4/8, leaf_max 1..3");
    const crg_status rc = build_bvh(scene, o, (cudaStream_t)stream);
    if (rc != CRG_OK) scene->built = false;
    return rc;
}

crg_status crg_scene_set_skybox(crg_scene *scene, const float *rgba, uint32_t w, uint32_t h, float rot_u, float rot_v) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if ((w == 0) != (h == 0) || (w && !rgba)) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "bad skybox size");
    scene->sky_rot_u = rot_u;
    scene->sky_rot_v = rot_v;
    if (w == 0) {
        dev_free(scene->sky);
        scene->sky_w = scene->sky_h = 0;
        return CRG_OK;
    }
    const size_t bytes = sizeof(float) * 4 * (size_t)w * h;
    crg_status rc = dev_alloc(scene->ctx, scene->sky, bytes);
    if (rc != CRG_OK) return rc;
    CRG_CUDA(scene->ctx, cudaMemcpy(scene->sky.ptr, rgba, bytes, cudaMemcpyHostToDevice));
    scene->sky_w = w;
    scene->sky_h = h;
    return CRG_OK;
}

crg_status crg_scene_set_sun(crg_scene *scene, int enabled, const crg_sun *sun) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    apply_sun(scene, sun ? *sun : default_sun());
    scene->sun_enabled = enabled ? 1 : 0;
    return CRG_OK;
}

crg_status crg_scene_set_textures(crg_scene *scene, uint32_t count, const float *const *rgba, const uint32_t *widths,
                                  const uint32_t *heights) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = scene->ctx;
    if (count > 0 && (!rgba || !widths || !heights)) return set_error(ctx, CRG_ERR_INVALID_ARG, "null texture arrays");
    std::vector<uint32_t> info(4 * (size_t)count);
    size_t total = 0;
    for (uint32_t i = 0; i < count; ++i) {
        if (!rgba[i] || widths[i] == 0 || heights[i] == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "empty texture");
        info[4 * i + 0] = (uint32_t)(total & 0xFFFFFFFFu);
        info[4 * i + 1] = (uint32_t)(total >> 32);
        info[4 * i + 2] = widths[i];
        info[4 * i + 3] = heights[i];
        total += (size_t)widths[i] * heights[i];
    }
    dev_free(scene->texels);
    dev_free(scene->tex_info);
    scene->ntex = 0;
    if (count == 0) return build_light_records(scene);
    crg_status rc;
    if ((rc = dev_alloc(ctx, scene->texels, 16 * total)) != CRG_OK) return rc;
    if ((rc = dev_alloc(ctx, scene->tex_info, 16 * (size_t)count)) != CRG_OK) return rc;
    for (uint32_t i = 0; i < count; ++i) {
        const size_t first = ((size_t)info[4 * i + 1] << 32) | info[4 * i];
        CRG_CUDA(ctx, cudaMemcpy((float *)scene->texels.ptr + 4 * first, rgba[i], 16 * (size_t)widths[i] * heights[i],
                                 cudaMemcpyHostToDevice));
    }
    CRG_CUDA(ctx, cudaMemcpy(scene->tex_info.ptr, info.data(), 16 * (size_t)count, cudaMemcpyHostToDevice));
    scene->ntex = count;
    return build_light_records(scene); // emitters' textured flags follow the texture count
}

crg_status crg_scene_set_instances(crg_scene *scene, const float *xforms, uint32_t ninst) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = scene->ctx;
    if (ninst > 0 && !xforms) return set_error(ctx, CRG_ERR_INVALID_ARG, "null transform array");
    if (ninst > (1u << 16)) return set_error(ctx, CRG_ERR_INVALID_ARG, "more than 65536 instances");
    float rows[24];
    for (uint32_t j = 0; j < ninst; ++j)
        if (!instance_rows(xforms + 16 * (size_t)j, rows))
            return set_error(ctx, CRG_ERR_INVALID_ARG, "instance transform is not an invertible affine matrix");
    for (crg_model_rec &m : scene->models) m.xf.assign(xforms, xforms + 16 * (size_t)ninst);
    crg_status rc = update_placements(scene);
    if (rc == CRG_OK) rc = prepare_lights(scene);
    return rc;
}

crg_status crg_scene_set_model_instances(crg_scene *scene, uint32_t model, const float *xforms, uint32_t ninst) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = scene->ctx;
    if (model >= scene->models.size()) return set_error(ctx, CRG_ERR_INVALID_ARG, "model index out of range");
    if (ninst > 0 && !xforms) return set_error(ctx, CRG_ERR_INVALID_ARG, "null transform array");
    if (ninst > (1u << 16)) return set_error(ctx, CRG_ERR_INVALID_ARG, "more than 65536 instances");
    float rows[24];
    for (uint32_t j = 0; j < ninst; ++j)
        if (!instance_rows(xforms + 16 * (size_t)j, rows))
            return set_error(ctx, CRG_ERR_INVALID_ARG, "instance transform is not an invertible affine matrix");
    scene->models[model].xf.assign(xforms, xforms + 16 * (size_t)ninst);
    crg_status rc = update_placements(scene);
    if (rc == CRG_OK) rc = prepare_lights(scene);
    return rc;
}

crg_status crg_scene_add_model(crg_scene *scene, const float *verts, uint32_t ntri, const float *uvs,
                               const uint32_t *mat_idx, const crg_material *mats, uint32_t nmat, uint32_t *model) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if (ntri > 0 && !verts) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "null vertex array");
    return append_model(scene, ntri, mat_idx, mats, nmat, model,
                        [&](float *d_verts, float *d_uvs, float *box, std::vector<double> &areas) {
        cudaError_t e = cudaSuccess;
        if (ntri) e = cudaMemcpy(d_verts, verts, sizeof(float) * 9 * (size_t)ntri, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && d_uvs && ntri) {
            if (uvs) e = cudaMemcpy(d_uvs, uvs, sizeof(float) * 6 * (size_t)ntri, cudaMemcpyHostToDevice);
            else e = cudaMemset(d_uvs, 0, sizeof(float) * 6 * (size_t)ntri);
        }
        if (e != cudaSuccess) return cuda_error(scene->ctx, e, "cudaMemcpy(model)");
        areas.resize(ntri);
        for (uint32_t p = 0; p < ntri; ++p) areas[p] = tri_area_of(verts + (size_t)p * 9);
        (void)box; // computed from the device copy when the placements are rebuilt
        return CRG_OK;
    }, uvs != nullptr);
}

crg_status crg_scene_add_model_indexed(crg_scene *scene, const float *positions, uint32_t npos,
                                       const uint32_t *vertex_indices, uint32_t ntri, const float *texcoords, uint32_t ntc,
                                       const int32_t *tex_indices, const uint32_t *mat_idx, const crg_material *mats,
                                       uint32_t nmat, uint32_t *model) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = scene->ctx;
    if (ntri > 0 && (!positions || !vertex_indices)) return set_error(ctx, CRG_ERR_INVALID_ARG, "null positions or indices");
    if (ntc > 0 && !texcoords) return set_error(ctx, CRG_ERR_INVALID_ARG, "null texture coordinates");
    for (size_t c = 0; c < 3 * (size_t)ntri; ++c)
        if (vertex_indices[c] >= npos) return set_error(ctx, CRG_ERR_INVALID_ARG, "vertex index out of range");
    const bool want_uv = tex_indices != nullptr;
    return append_model(scene, ntri, mat_idx, mats, nmat, model,
                        [&](float *d_verts, float *d_uvs, float *box, std::vector<double> &areas) {
        if (ntri == 0) return CRG_OK;
        const size_t nc = 3 * (size_t)ntri;
        DevBuf dpos, didx, dtc, dti;
        crg_status rc = dev_alloc(ctx, dpos, sizeof(float) * 3 * (size_t)npos);
        if (rc == CRG_OK) rc = dev_alloc(ctx, didx, sizeof(uint32_t) * nc);
        if (rc == CRG_OK && d_uvs && want_uv) rc = dev_alloc(ctx, dti, sizeof(int32_t) * nc);
        if (rc == CRG_OK && d_uvs && want_uv && ntc) rc = dev_alloc(ctx, dtc, sizeof(float) * 2 * (size_t)ntc);
        cudaError_t e = cudaSuccess;
        if (rc == CRG_OK) e = cudaMemcpy(dpos.ptr, positions, sizeof(float) * 3 * (size_t)npos, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess) e = cudaMemcpy(didx.ptr, vertex_indices, sizeof(uint32_t) * nc, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess && dti.ptr)
            e = cudaMemcpy(dti.ptr, tex_indices, sizeof(int32_t) * nc, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess && dtc.ptr)
            e = cudaMemcpy(dtc.ptr, texcoords, sizeof(float) * 2 * (size_t)ntc, cudaMemcpyHostToDevice);
        if (rc == CRG_OK && e == cudaSuccess) {
            const unsigned blocks = (unsigned)std::min<size_t>((nc + 255) / 256, (size_t)std::max(ctx->sm_count, 1) * 8);
            k_expand<<<blocks, 256>>>((const float *)dpos.ptr, (const uint32_t *)didx.ptr, (const float *)dtc.ptr,
                                      (const int32_t *)dti.ptr, dtc.ptr ? ntc : 0, d_verts, d_uvs, nc);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaDeviceSynchronize();
        }
        dev_free(dpos);
        dev_free(didx);
        dev_free(dtc);
        dev_free(dti);
        if (rc != CRG_OK) return rc;
        if (e != cudaSuccess) return cuda_error(ctx, e, "k_expand(model)");
        float tv[9];
        (void)box; // computed from the device copy when the placements are rebuilt
        for (uint32_t p = 0; p < ntri; ++p) {
            for (int k = 0; k < 3; ++k)
                for (int a = 0; a < 3; ++a) tv[3 * k + a] = positions[3 * (size_t)vertex_indices[3 * (size_t)p + k] + a];
            areas.push_back(tri_area_of(tv));
        }
        return CRG_OK;
    }, want_uv);
}

crg_status crg_scene_model_count(const crg_scene *scene, uint32_t *count) {
    if (!scene || !count) return CRG_ERR_INVALID_ARG;
    *count = (uint32_t)scene->models.size();
    return CRG_OK;
}

crg_status crg_scene_model_info(const crg_scene *scene, uint32_t model, crg_model_info *info) {
    if (!scene || !info) return CRG_ERR_INVALID_ARG;
    if (model >= scene->models.size()) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "model index out of range");
    const crg_model_rec &m = scene->models[model];
    *info = crg_model_info{};
    info->first_prim = m.first;
    info->ntri = m.ntri;
    info->node_base = m.node_base;
    info->n_wide_nodes = m.built ? m.n_wide : 0;
    info->depth = m.built ? m.depth : 0;
    info->ninst = (uint32_t)(m.xf.size() / 16);
    info->built = m.built ? 1u : 0u;
    info->sah_cost = m.built ? m.sah : 0.0f;
    return CRG_OK;
}

crg_status crg_scene_bvh_info(const crg_scene *scene, crg_bvh_info *info) {
    if (!scene || !info) return CRG_ERR_INVALID_ARG;
    if (!scene->built) return CRG_ERR_NOT_BUILT;
    const bool one = scene->models.size() == 1;
    info->ntri = scene->ntri;
    info->width = scene->width;
    info->n_bvh2_nodes = one ? (scene->ntri >= 2 ? scene->ntri - 1 : 0) : scene->node_cap;
    info->n_wide_nodes = scene->n_wide;
    info->node_bytes = scene->node_bytes;
    info->n_tri_slots = scene->ntri;
    info->depth = scene->depth;
    info->sah_cost = scene->sah;
    info->leaf_max = scene->opts.leaf_max;
    info->treelet = scene->opts.treelet;
    return CRG_OK;
}

crg_status crg_scene_bvh_download(const crg_scene *scene, float *bvh2, uint32_t *order, void *wide, float *tris) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if (!scene->built) return CRG_ERR_NOT_BUILT;
    crg_context *ctx = scene->ctx;
    const uint32_t n = scene->ntri;
    if (n == 0) return CRG_OK;
    const size_t n2 = scene->models.size() == 1 ? (n >= 2 ? n - 1 : 0) : scene->node_cap;
    if (bvh2 && n2) CRG_CUDA(ctx, cudaMemcpy(bvh2, scene->bvh2.ptr, sizeof(float) * 8 * n2, cudaMemcpyDeviceToHost));
    if (order) CRG_CUDA(ctx, cudaMemcpy(order, scene->order.ptr, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost));
    if (wide) CRG_CUDA(ctx, cudaMemcpy(wide, scene->wide.ptr, (size_t)scene->node_bytes * scene->n_wide, cudaMemcpyDeviceToHost));
    if (tris) CRG_CUDA(ctx, cudaMemcpy(tris, scene->tris.ptr, sizeof(float) * 12 * (size_t)n, cudaMemcpyDeviceToHost));
    return CRG_OK;
}

crg_status crg_intersect_closest(const crg_scene *scene, const crg_ray *d_rays, crg_hit *d_hits, uint64_t n, crg_stream stream) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if (!scene->built) return set_error(scene->ctx, CRG_ERR_NOT_BUILT, "scene not built");
    if (n && (!d_rays || !d_hits)) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "null ray or hit array");
    return launch_intersect(scene, d_rays, d_hits, nullptr, nullptr, nullptr, n, false, (cudaStream_t)stream);
}

crg_status crg_intersect_any(const crg_scene *scene, const crg_ray *d_rays, uint32_t *d_occluded, uint64_t n, crg_stream stream) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if (!scene->built) return set_error(scene->ctx, CRG_ERR_NOT_BUILT, "scene not built");
    if (n && (!d_rays || !d_occluded)) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "null ray or output array");
    return launch_intersect(scene, d_rays, nullptr, d_occluded, nullptr, nullptr, n, true, (cudaStream_t)stream);
}

crg_status crg_intersect_closest_with(const crg_scene *scene, const crg_ray *d_rays, crg_hit *d_hits, uint64_t n,
                                      crg_traversal traversal, crg_stream stream) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if (!scene->built) return set_error(scene->ctx, CRG_ERR_NOT_BUILT, "scene not built");
    if (n && (!d_rays || !d_hits)) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "null ray or hit array");
    if (traversal != CRG_TRAVERSAL_THREAD && traversal != CRG_TRAVERSAL_WARP)
        return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "unknown traversal scheme");
    return launch_intersect(scene, d_rays, d_hits, nullptr, nullptr, nullptr, n, false, (cudaStream_t)stream, traversal);
}

crg_status crg_intersect_any_with(const crg_scene *scene, const crg_ray *d_rays, uint32_t *d_occluded, uint64_t n,
                                  crg_traversal traversal, crg_stream stream) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if (!scene->built) return set_error(scene->ctx, CRG_ERR_NOT_BUILT, "scene not built");
    if (n && (!d_rays || !d_occluded)) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "null ray or output array");
    if (traversal != CRG_TRAVERSAL_THREAD && traversal != CRG_TRAVERSAL_WARP)
        return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "unknown traversal scheme");
    return launch_intersect(scene, d_rays, nullptr, d_occluded, nullptr, nullptr, n, true, (cudaStream_t)stream, traversal);
}

crg_status crg_intersect_closest_counted(const crg_scene *scene, const crg_ray *d_rays, crg_hit *d_hits, uint32_t *d_nodes,
                                         uint32_t *d_tris, uint64_t n, crg_stream stream) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    if (!scene->built) return set_error(scene->ctx, CRG_ERR_NOT_BUILT, "scene not built");
    if (n && (!d_rays || !d_hits)) return set_error(scene->ctx, CRG_ERR_INVALID_ARG, "null ray or hit array");
    if (!d_nodes && !d_tris) return launch_intersect(scene, d_rays, d_hits, nullptr, nullptr, nullptr, n, false, (cudaStream_t)stream);
    return launch_intersect(scene, d_rays, d_hits, nullptr, d_nodes, d_tris, n, false, (cudaStream_t)stream);
}

crg_status crg_scene_poll_error(crg_scene *scene) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    uint32_t e = 0;
    CRG_CUDA(scene->ctx, cudaMemcpy(&e, scene->err.ptr, 4, cudaMemcpyDeviceToHost));
    if (e) {
        CRG_CUDA(scene->ctx, cudaMemset(scene->err.ptr, 0, 4));
        return set_error(scene->ctx, CRG_ERR_DEVICE, "traversal stack overflow reported by a kernel");
    }
    return CRG_OK;
}

crg_status crg_film_create(crg_context *ctx, uint32_t width, uint32_t height, uint32_t flags, crg_film **out) {
    if (!ctx || !out) return set_error(ctx, CRG_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (width == 0 || height == 0 || (uint64_t)width * height > (1ull << 31))
        return set_error(ctx, CRG_ERR_INVALID_ARG, "film size must be positive and at most 2^31 pixels");
    crg_film *f = fault_injected() ? nullptr : new (std::nothrow) crg_film();
    if (!f) return set_error(ctx, CRG_ERR_OOM, "host allocation of the film failed");
    f->ctx = ctx;
    f->width = width;
    f->height = height;
    f->flags = flags;
    const size_t npix = (size_t)width * height;
    crg_status rc = dev_alloc(ctx, f->sum, sizeof(float) * 3 * npix);
    if (rc == CRG_OK && (flags & CRG_FILM_F64)) {
        rc = dev_alloc(ctx, f->sum64, sizeof(double) * 3 * npix);
        if (rc == CRG_OK) rc = dev_alloc(ctx, f->sumsq64, sizeof(double) * 3 * npix);
    }
    if (rc == CRG_OK && (flags & CRG_FILM_AOV)) {
        rc = dev_alloc(ctx, f->aov_albedo, sizeof(float) * 4 * npix);
        if (rc == CRG_OK) rc = dev_alloc(ctx, f->aov_normal, sizeof(float) * 4 * npix);
        if (rc == CRG_OK) rc = dev_alloc(ctx, f->aov_depth, sizeof(float) * 4 * npix);
        // cr::image starts filled with FLT_MAX (src/objects/image.h:30-33)
        if (rc == CRG_OK) {
            k_fill_f32<<<152 * 4, 256>>>((float *)f->aov_albedo.ptr, 4 * npix, FLT_MAX);
            k_fill_f32<<<152 * 4, 256>>>((float *)f->aov_normal.ptr, 4 * npix, FLT_MAX);
            k_fill_f32<<<152 * 4, 256>>>((float *)f->aov_depth.ptr, 4 * npix, FLT_MAX);
        }
    }
    if (rc == CRG_OK) rc = crg_film_reset(f, nullptr);
    if (rc == CRG_OK) {
        const cudaError_t e = cudaStreamSynchronize(nullptr);
        if (e != cudaSuccess) rc = cuda_error(ctx, e, "film init");
    }
    if (rc != CRG_OK) {
        crg_film_destroy(f);
        return rc;
    }
    *out = f;
    return CRG_OK;
}

crg_status crg_film_destroy(crg_film *film) {
    if (!film) return CRG_ERR_INVALID_ARG;
    DevBuf *bufs[] = {&film->sum, &film->sum64, &film->sumsq64, &film->aov_albedo, &film->aov_normal, &film->aov_depth};
    for (DevBuf *b : bufs) dev_free(*b);
    delete film;
    return CRG_OK;
}

crg_status crg_film_reset(crg_film *film, crg_stream stream) {
    if (!film) return CRG_ERR_INVALID_ARG;
    const size_t npix = (size_t)film->width * film->height;
    cudaStream_t st = (cudaStream_t)stream;
    CRG_CUDA(film->ctx, cudaMemsetAsync(film->sum.ptr, 0, sizeof(float) * 3 * npix, st));
    if (film->sum64.ptr) {
        CRG_CUDA(film->ctx, cudaMemsetAsync(film->sum64.ptr, 0, sizeof(double) * 3 * npix, st));
        CRG_CUDA(film->ctx, cudaMemsetAsync(film->sumsq64.ptr, 0, sizeof(double) * 3 * npix, st));
    }
    film->spp = 0;
    return CRG_OK;
}

crg_status crg_film_spp(const crg_film *film, uint64_t *spp) {
    if (!film || !spp) return CRG_ERR_INVALID_ARG;
    *spp = film->spp;
    return CRG_OK;
}

crg_status crg_film_download(crg_film *film, float *sum_rgb, double *sum64, double *sumsq64, float *aov_albedo,
                             float *aov_normal, float *aov_depth, crg_stream stream) {
    const crg_status rc = crg_film_download_async(film, sum_rgb, sum64, sumsq64, aov_albedo, aov_normal, aov_depth, stream);
    if (rc != CRG_OK) return rc;
    CRG_CUDA(film->ctx, cudaStreamSynchronize((cudaStream_t)stream));
    return CRG_OK;
}

crg_status crg_film_download_async(crg_film *film, float *sum_rgb, double *sum64, double *sumsq64, float *aov_albedo,
                                   float *aov_normal, float *aov_depth, crg_stream stream) {
    if (!film) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = film->ctx;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t npix = (size_t)film->width * film->height;
    if ((sum64 || sumsq64) && !film->sum64.ptr) return set_error(ctx, CRG_ERR_INVALID_ARG, "film has no FP64 planes");
    if ((aov_albedo || aov_normal || aov_depth) && !film->aov_albedo.ptr)
        return set_error(ctx, CRG_ERR_INVALID_ARG, "film has no AOV planes");
    if (sum_rgb) CRG_CUDA(ctx, cudaMemcpyAsync(sum_rgb, film->sum.ptr, sizeof(float) * 3 * npix, cudaMemcpyDeviceToHost, st));
    if (sum64) CRG_CUDA(ctx, cudaMemcpyAsync(sum64, film->sum64.ptr, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, st));
    if (sumsq64) CRG_CUDA(ctx, cudaMemcpyAsync(sumsq64, film->sumsq64.ptr, sizeof(double) * 3 * npix, cudaMemcpyDeviceToHost, st));
    if (aov_albedo) CRG_CUDA(ctx, cudaMemcpyAsync(aov_albedo, film->aov_albedo.ptr, sizeof(float) * 4 * npix, cudaMemcpyDeviceToHost, st));
    if (aov_normal) CRG_CUDA(ctx, cudaMemcpyAsync(aov_normal, film->aov_normal.ptr, sizeof(float) * 4 * npix, cudaMemcpyDeviceToHost, st));
    if (aov_depth) CRG_CUDA(ctx, cudaMemcpyAsync(aov_depth, film->aov_depth.ptr, sizeof(float) * 4 * npix, cudaMemcpyDeviceToHost, st));
    return CRG_OK;
}

crg_status crg_film_device_ptrs(crg_film *film, float **sum_rgb, double **sum64, double **sumsq64) {
    if (!film) return CRG_ERR_INVALID_ARG;
    if (sum_rgb) *sum_rgb = (float *)film->sum.ptr;
    if (sum64) *sum64 = (double *)film->sum64.ptr;
    if (sumsq64) *sumsq64 = (double *)film->sumsq64.ptr;
    return CRG_OK;
}

crg_status crg_film_display(crg_film *film, float *d_rgba, crg_stream stream) {
    if (!film || !d_rgba) return set_error(film ? film->ctx : nullptr, CRG_ERR_INVALID_ARG, "null argument");
    const size_t npix = (size_t)film->width * film->height;
    const float inv = film->spp ? 1.0f / (float)film->spp : 0.0f;
    k_display<<<152 * 4, 256, 0, (cudaStream_t)stream>>>((const float *)film->sum.ptr, (float4 *)d_rgba, npix, inv);
    CRG_CUDA(film->ctx, cudaGetLastError());
    return CRG_OK;
}

crg_status crg_draft_render(crg_scene *scene, const crg_camera *camera, uint32_t width, uint32_t height, float aspect,
                            float *d_rgba, crg_stream stream) {
    if (!scene || !camera || !d_rgba) return set_error(scene ? scene->ctx : nullptr, CRG_ERR_INVALID_ARG, "null argument");
    crg_context *ctx = scene->ctx;
    if (!scene->built) return set_error(ctx, CRG_ERR_NOT_BUILT, "scene not built");
    if (width == 0 || height == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "empty image");
    if ((uint64_t)width * height >= (1ull << 32)) return set_error(ctx, CRG_ERR_INVALID_ARG, "image too large");
    if (camera->mode > CRG_CAMERA_ORTHOGRAPHIC) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad camera mode");
    if (scene->ntri == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "scene has no triangles");
    return launch_draft(scene, camera_params(*camera), width, height, aspect, d_rgba, (cudaStream_t)stream);
}

crg_status crg_render(crg_scene *scene, const crg_camera *camera, const crg_settings *settings, crg_film *film, crg_stream stream) {
    if (!scene || !camera || !settings || !film) return set_error(scene ? scene->ctx : nullptr, CRG_ERR_INVALID_ARG, "null argument");
    crg_context *ctx = scene->ctx;
    if (film->ctx != ctx) return set_error(ctx, CRG_ERR_INVALID_ARG, "film and scene belong to different contexts");
    if (!scene->built) return set_error(ctx, CRG_ERR_NOT_BUILT, "scene not built");
    const crg_settings &s = *settings;
    if (s.width != film->width || s.height != film->height) return set_error(ctx, CRG_ERR_INVALID_ARG, "settings resolution differs from the film");
    if (s.mode > CRG_MODE_EXTENDED) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad estimator mode");
    if (camera->mode > CRG_CAMERA_ORTHOGRAPHIC) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad camera mode");
    if (s.max_bounces > 1024) return set_error(ctx, CRG_ERR_INVALID_ARG, "max_bounces above 1024");
    if (film->spp + s.spp > 0xFFFFFFFFull) return set_error(ctx, CRG_ERR_INVALID_ARG, "sample index would exceed 2^32");
    cudaStream_t st = (cudaStream_t)stream;
    if (scene->counting) CRG_CUDA(ctx, cudaMemsetAsync(scene->counters.ptr, 0, 64, st));
    const CamDev cam = camera_params(*camera);
    crg_status rc = launch_render(scene, cam, s, film, st);
    if (rc != CRG_OK) return rc;
    film->spp += s.spp;
    scene->last_stats.samples = (uint64_t)s.spp * s.width * s.height;
    if (scene->counting) {
        unsigned long long c[8];
        CRG_CUDA(ctx, cudaMemcpyAsync(c, scene->counters.ptr, sizeof(c), cudaMemcpyDeviceToHost, st));
        CRG_CUDA(ctx, cudaStreamSynchronize(st));
        scene->last_stats.segments = c[1];
        scene->last_stats.shadow_rays = c[2];
        scene->last_stats.nodes_visited = c[3];
        scene->last_stats.tris_tested = c[4];
    }
    return CRG_OK;
}

namespace {
crg_status batch_call(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views, crg_film *const *films,
                      uint32_t nviews, const crg_wavefront_opts *opts, crg_stream stream, bool wait) {
    if (!scenes || nscenes == 0 || !scenes[0]) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = scenes[0]->ctx;
    if (!views || !films || nviews == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "empty batch");
    if (nviews > 65535) return set_error(ctx, CRG_ERR_INVALID_ARG, "at most 65535 views per batch");
    for (uint32_t i = 0; i < nscenes; ++i) {
        if (!scenes[i] || scenes[i]->ctx != ctx) return set_error(ctx, CRG_ERR_INVALID_ARG, "scenes must share one context");
        if (!scenes[i]->built) return set_error(ctx, CRG_ERR_NOT_BUILT, "scene not built");
        if (scenes[i]->width != scenes[0]->width) return set_error(ctx, CRG_ERR_INVALID_ARG, "scenes must share one BVH width");
        if (scenes[i]->ntri == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "scene has no triangles");
    }
    for (uint32_t v = 0; v < nviews; ++v) {
        const crg_settings &s = views[v].settings;
        if (views[v].scene >= nscenes) return set_error(ctx, CRG_ERR_INVALID_ARG, "view scene index out of range");
        if (!films[v] || films[v]->ctx != ctx) return set_error(ctx, CRG_ERR_INVALID_ARG, "null film or film of another context");
        if (s.width != films[v]->width || s.height != films[v]->height)
            return set_error(ctx, CRG_ERR_INVALID_ARG, "view resolution differs from its film");
        if (s.mode > CRG_MODE_EXTENDED || views[v].camera.mode > CRG_CAMERA_ORTHOGRAPHIC)
            return set_error(ctx, CRG_ERR_INVALID_ARG, "bad estimator or camera mode");
        if (s.max_bounces > 1023) return set_error(ctx, CRG_ERR_INVALID_ARG, "max_bounces above 1023");
        if (films[v]->spp + s.spp > 0xFFFFFFFFull) return set_error(ctx, CRG_ERR_INVALID_ARG, "sample index would exceed 2^32");
        for (uint32_t u = 0; u < v; ++u)
            if (films[u] == films[v]) return set_error(ctx, CRG_ERR_INVALID_ARG, "films must be distinct");
    }
    // defaults: up to 128M paths in flight (about 20 GB of path state for a batch that large; a
    // frame never holds more paths than its largest chunk's samples), 128M-sample chunks (2 GB of
    // sample slots), split stages with per-lane refill in the traversal stages
    crg_wavefront_opts o{1u << 27, 1u << 27, 128, 32, 0, 0, 0, 1, 16};
    if (opts) {
        if (opts->path_pool) o.path_pool = opts->path_pool;
        if (opts->chunk_samples) o.chunk_samples = opts->chunk_samples;
        if (opts->block_size) o.block_size = opts->block_size;
        if (opts->fetch) o.fetch = opts->fetch;
        o.max_iterations = opts->max_iterations;
        o.count_work = opts->count_work;
        o.host_loop = opts->host_loop;
        if (opts->fuse) o.fuse = opts->fuse;
        if (opts->refill) o.refill = opts->refill == 0xFFFFFFFFu ? 0u : opts->refill;
    }
    if ((o.block_size != 64 && o.block_size != 128 && o.block_size != 256) || o.fetch % 32 || o.fetch > 4096 ||
        o.path_pool > (1u << 28) || o.fuse > 3 || o.refill > 32 || o.host_loop > 2)
        return set_error(ctx, CRG_ERR_INVALID_ARG,
                         "wavefront options: block_size 64/128/256, fetch a multiple of 32, path_pool <= 2^28, fuse <= 3, "
                         "refill <= 32, host_loop <= 2");
    return render_batch(ctx, scenes, nscenes, views, films, nviews, o, (cudaStream_t)stream, wait);
}
} // namespace

crg_status crg_render_batch(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views, crg_film *const *films,
                            uint32_t nviews, const crg_wavefront_opts *opts, crg_stream stream) {
    return batch_call(scenes, nscenes, views, films, nviews, opts, stream, true);
}

crg_status crg_render_batch_async(crg_scene *const *scenes, uint32_t nscenes, const crg_view *views,
                                  crg_film *const *films, uint32_t nviews, const crg_wavefront_opts *opts,
                                  crg_stream stream) {
    return batch_call(scenes, nscenes, views, films, nviews, opts, stream, false);
}

crg_status crg_batch_wait(crg_context *ctx) {
    if (!ctx) return CRG_ERR_INVALID_ARG;
    return batch_wait(ctx);
}

crg_status crg_batch_stats_get(const crg_context *ctx, crg_render_stats *stats) {
    if (!ctx || !stats) return CRG_ERR_INVALID_ARG;
    *stats = ctx->batch_stats;
    return CRG_OK;
}

crg_status crg_batch_stage_times_get(const crg_context *ctx, crg_stage_times *times) {
    if (!ctx || !times) return CRG_ERR_INVALID_ARG;
    *times = ctx->stage_times;
    return CRG_OK;
}

crg_status crg_scene_set_materials(crg_scene *scene, const crg_material *mats, uint32_t nmat) {
    if (!scene || !mats) return CRG_ERR_INVALID_ARG;
    crg_context *ctx = scene->ctx;
    if (nmat != scene->nmat) return set_error(ctx, CRG_ERR_INVALID_ARG, "material count differs from the scene's");
    for (uint32_t m = 0; m < nmat; ++m)
        if (mats[m].shade_type > CRG_SHADE_GLASS) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad shade_type");
    scene->host_mats.assign(mats, mats + nmat);
    CRG_CUDA(ctx, cudaMemcpy(scene->mats.ptr, mats, sizeof(crg_material) * nmat, cudaMemcpyHostToDevice));
    return prepare_lights(scene);
}

crg_status crg_backward(crg_scene *scene, const crg_camera *camera, const crg_settings *settings, const float *d_adjoint,
                        double *d_grad_colour, double *d_grad_emission, crg_stream stream) {
    if (!scene || !camera || !settings || !d_adjoint || !d_grad_colour || !d_grad_emission)
        return set_error(scene ? scene->ctx : nullptr, CRG_ERR_INVALID_ARG, "null argument");
    crg_context *ctx = scene->ctx;
    if (!scene->built) return set_error(ctx, CRG_ERR_NOT_BUILT, "scene not built");
    if (scene->ntri == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "scene has no triangles");
    const crg_settings &s = *settings;
    if (s.mode != CRG_MODE_EXTENDED) return set_error(ctx, CRG_ERR_UNSUPPORTED, "the adjoint differentiates the extended estimator");
    if (s.max_bounces > 32) return set_error(ctx, CRG_ERR_INVALID_ARG, "adjoint: max_bounces above 32");
    if (s.width == 0 || s.height == 0 || s.spp == 0) return set_error(ctx, CRG_ERR_INVALID_ARG, "empty adjoint pass");
    if (camera->mode > CRG_CAMERA_ORTHOGRAPHIC) return set_error(ctx, CRG_ERR_INVALID_ARG, "bad camera mode");
    if (scene->sun_enabled) return set_error(ctx, CRG_ERR_UNSUPPORTED, "adjoint: the sun belongs to the faithful estimator");
    for (const crg_material &m : scene->host_mats)
        if (m.tex >= 0 && (uint32_t)m.tex < scene->ntex)
            return set_error(ctx, CRG_ERR_UNSUPPORTED, "adjoint: textured materials have no colour parameter");
    return launch_backward(scene, camera_params(*camera), s, d_adjoint, d_grad_colour, d_grad_emission, (cudaStream_t)stream);
}

crg_status crg_film_loss_l2(crg_film *film, const float *d_target, float *d_adjoint, double *d_loss, crg_stream stream) {
    if (!film || !d_target || !d_adjoint || !d_loss)
        return set_error(film ? film->ctx : nullptr, CRG_ERR_INVALID_ARG, "null argument");
    if (film->spp == 0) return set_error(film->ctx, CRG_ERR_INVALID_ARG, "film holds no samples");
    return launch_loss_l2(film, d_target, d_adjoint, d_loss, (cudaStream_t)stream);
}

crg_status crg_render_stats_get(const crg_scene *scene, crg_render_stats *stats) {
    if (!scene || !stats) return CRG_ERR_INVALID_ARG;
    *stats = scene->last_stats;
    return CRG_OK;
}

crg_status crg_scene_set_counting(crg_scene *scene, int enabled) {
    if (!scene) return CRG_ERR_INVALID_ARG;
    scene->counting = enabled ? 1 : 0;
    return CRG_OK;
}

} /* extern "C" */
