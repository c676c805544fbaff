/*
 * orc_bvh.cpp — CPU oracle of the acceleration structure.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates, for checking the GPU builder bit for bit:
 *   1. triangle bounds and AABB-centre centroids;
 *   2. 30-bit Morton codes over the centroid bounds (10 bits per axis,
 *      q = min(max((c - lo) * (1024 / extent), 0), 1023));
 *   3. sort by (code, primitive index);
 *   4. the Karras 2012 hierarchy ("Maximizing Parallelism in the Construction
 *      of BVHs, Octrees, and k-d Trees", HPG 2012, Fig. 4) with the index
 *      tie-break for equal codes;
 *   5. bottom-up boxes and primitive counts;
 *   6. optional treelet restructuring (Karras & Aila, "Fast Parallel
 *      Construction of High-Quality Bounding Volume Hierarchies", HPG 2013):
 *      7-leaf treelets grown by largest surface area, exact SAH dynamic
 *      programming over the 127 leaf subsets, bottom-up over nodes whose
 *      subtree holds at least gamma primitives, gamma = 7, 14, 28, ...;
 *   7. greedy collapse to a W-wide BVH (largest-area child expanded first),
 *      child slots assigned to the 8 octant directions as in Ylitie, Karras &
 *      Laine, "Efficient Incoherent Ray Traversal on GPUs Through Compressed
 *      Wide BVHs", HPG 2017, with 8-bit quantized child boxes (empty slots
 *      carry the inverted box lo = 255, hi = 0, which no ray can hit).
 * This replaces what rtcCommitScene does for CRender (src/objects/model.cpp:52-97).
 *
 * Queries use the binary tree with a conservative slab test (tmax scaled by
 * 1 + 2*gamma(3), Ize 2013 / pbrt-v3) and the watertight ray/triangle test of
 * Woop, Benthin & Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013.
 * Ray defaults follow _intersect (src/objects/model.cpp:5-49): tnear 1e-5,
 * tfar +inf; the geometric normal convention is cross(v1 - v0, v2 - v0).
 */
#include "orc.h"
#include "orc_math.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <limits>
#include <thread>
#include <vector>

namespace {

const uint32_t LEAF = 0x80000000u;

struct Box {
    float lo[3], hi[3];
};
inline float fmn(float a, float b) { return a < b ? a : b; }
inline float fmx(float a, float b) { return a > b ? a : b; }

Box tri_box(const float *v) {
    Box b;
    for (int a = 0; a < 3; ++a) {
        b.lo[a] = fmn(fmn(v[a], v[3 + a]), v[6 + a]);
        b.hi[a] = fmx(fmx(v[a], v[3 + a]), v[6 + a]);
    }
    return b;
}
Box merge(const Box &a, const Box &b) {
    Box r;
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = fmn(a.lo[k], b.lo[k]);
        r.hi[k] = fmx(a.hi[k], b.hi[k]);
    }
    return r;
}
float area(const Box &b) {
    const float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    return 2.0f * ((dx * dy + dy * dz) + dz * dx);
}

uint32_t spread10(uint32_t v) {
    uint32_t r = 0;
    for (int i = 0; i < 10; ++i) r |= ((v >> i) & 1u) << (3 * i);
    return r;
}

int delta(const uint32_t *k, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    const uint32_t a = k[i], b = k[j];
    if (a != b) return __builtin_clz(a ^ b);
    return 32 + __builtin_clz((uint32_t)i ^ (uint32_t)j);
}

/* Smallest e with 2^e >= x (x > 0), from the exact binary exponent. */
int ceil_log2(double x) {
    int k;
    const double m = std::frexp(x, &k); /* x = m * 2^k, m in [0.5, 1) */
    return (m == 0.5) ? k - 1 : k;
}
int floor_log2(double x) {
    int k;
    std::frexp(x, &k);
    return k - 1;
}

} // namespace

struct orc_bvh {
    uint32_t ntri = 0;
    crg_build_opts opts{};
    std::vector<float> verts;
    std::vector<uint32_t> order;          /* sorted position -> primitive */
    std::vector<uint32_t> left, right;    /* internal children (LEAF | j for leaves) */
    std::vector<uint32_t> parent;         /* internal node parents (root: 0xFFFFFFFF) */
    std::vector<uint32_t> leaf_parent;    /* sorted position -> internal parent */
    std::vector<Box> nbox, lbox;
    std::vector<uint32_t> count;          /* primitives under an internal node */
    uint32_t width = 8, node_bytes = 80, n_wide = 0, depth = 0;
    std::vector<uint8_t> wide;
    std::vector<float> tris;
    float sah = 0.0f;

    uint32_t root() const { return ntri >= 2 ? 0u : (LEAF | 0u); }
    const Box &box_of(uint32_t r) const { return (r & LEAF) ? lbox[r & ~LEAF] : nbox[r]; }
    uint32_t count_of(uint32_t r) const { return (r & LEAF) ? 1u : count[r]; }
};

namespace {

/* ------------------------------------------------------------ treelets */

const float kCi = 1.2f, kCt = 1.0f; /* SAH constants of Karras & Aila 2013 */

/* Restructures the treelet rooted at internal node r (all descendants already
 * processed).  Returns nothing; node arrays are updated in place. */
void optimize_treelet(orc_bvh &B, uint32_t r, std::vector<float> &cost) {
    /* refresh this node's cost from its (already final) children */
    {
        auto c = [&](uint32_t ref) { return (ref & LEAF) ? kCt * area(B.lbox[ref & ~LEAF]) : cost[ref]; };
        cost[r] = kCi * area(B.nbox[r]) + (c(B.left[r]) + c(B.right[r]));
    }
    /* Grow: leaves start as the two children; expand the internal leaf with
     * the largest area (first on ties) until 7 leaves or none expandable. */
    uint32_t leaves[7];
    int nl = 2;
    leaves[0] = B.left[r];
    leaves[1] = B.right[r];
    uint32_t internals[6];
    int ni = 0;
    while (nl < 7) {
        int best = -1;
        float best_a = -1.0f;
        for (int j = 0; j < nl; ++j) {
            if (leaves[j] & LEAF) continue;
            const float a = area(B.nbox[leaves[j]]);
            if (a > best_a) { best_a = a; best = j; }
        }
        if (best < 0) break;
        const uint32_t x = leaves[best];
        internals[ni++] = x;
        leaves[best] = B.left[x];
        leaves[nl++] = B.right[x];
    }
    if (nl < 3) return; /* nothing to rearrange */
    const int nsub = 1 << nl;
    float aS[128], cS[128];
    int pS[128];
    Box bS[128];
    for (int s = 1; s < nsub; ++s) {
        Box b{};
        bool first = true;
        for (int j = 0; j < nl; ++j)
            if (s & (1 << j)) {
                const Box &lb = B.box_of(leaves[j]);
                b = first ? lb : merge(b, lb);
                first = false;
            }
        bS[s] = b;
        aS[s] = area(b);
    }
    auto leaf_cost = [&](uint32_t ref) -> float {
        return (ref & LEAF) ? kCt * area(B.lbox[ref & ~LEAF]) : cost[ref];
    };
    for (int j = 0; j < nl; ++j) {
        cS[1 << j] = leaf_cost(leaves[j]);
        pS[1 << j] = 0;
    }
    /* Subsets in increasing size so that all proper subsets are ready. */
    for (int k = 2; k <= nl; ++k) {
        for (int s = 1; s < nsub; ++s) {
            if (__builtin_popcount((unsigned)s) != k) continue;
            float best = FLT_MAX;
            int bp = 0;
            /* partitions (P, S\P), P containing the lowest set bit of S */
            const int low = s & -s;
            const int rest = s ^ low;
            for (int q = rest;; q = (q - 1) & rest) {
                const int P = q | low;
                if (P != s) {
                    const float c = cS[P] + cS[s ^ P];
                    if (c < best) { best = c; bp = P; }
                }
                if (q == 0) break;
            }
            cS[s] = kCi * aS[s] + best;
            pS[s] = bp;
        }
    }
    const int full = nsub - 1;
    if (!(cS[full] < cost[r])) return;
    /* Rebuild: internal nodes reused in formation order; root stays r. */
    int next = 0;
    struct Item { int s; uint32_t node; };
    std::vector<Item> stack;
    stack.push_back({full, r});
    std::vector<std::pair<int, uint32_t>> post; /* (subset, node) for bottom-up refresh */
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        const int P = pS[it.s];
        const int Q = it.s ^ P;
        uint32_t kids[2];
        const int parts[2] = {P, Q};
        for (int c = 0; c < 2; ++c) {
            const int sub = parts[c];
            if (__builtin_popcount((unsigned)sub) == 1) {
                kids[c] = leaves[__builtin_ctz((unsigned)sub)];
            } else {
                kids[c] = internals[next++];
            }
        }
        B.left[it.node] = kids[0];
        B.right[it.node] = kids[1];
        for (int c = 0; c < 2; ++c) {
            if (kids[c] & LEAF) B.leaf_parent[kids[c] & ~LEAF] = it.node;
            else B.parent[kids[c]] = it.node;
        }
        post.push_back({it.s, it.node});
        /* push right then left so left is expanded first (pre-order) */
        for (int c = 1; c >= 0; --c)
            if (!(kids[c] & LEAF) && __builtin_popcount((unsigned)parts[c]) > 1) stack.push_back({parts[c], kids[c]});
    }
    for (auto it = post.rbegin(); it != post.rend(); ++it) {
        const uint32_t x = it->second;
        B.nbox[x] = bS[it->first];
        B.count[x] = B.count_of(B.left[x]) + B.count_of(B.right[x]);
        cost[x] = cS[it->first];
    }
}

void treelet_pass(orc_bvh &B, uint32_t gamma, std::vector<float> &cost) {
    const uint32_t n = B.ntri;
    std::vector<uint32_t> visits(n - 1, 0);
    for (uint32_t j = 0; j < n; ++j) {
        uint32_t x = B.leaf_parent[j];
        while (x != 0xFFFFFFFFu) {
            if (++visits[x] < 2) break;
            if (B.count[x] >= gamma) optimize_treelet(B, x, cost);
            x = B.parent[x];
        }
    }
}

void compute_costs(orc_bvh &B, std::vector<float> &cost) {
    const uint32_t n = B.ntri;
    cost.assign(n - 1, 0.0f);
    std::vector<uint32_t> visits(n - 1, 0);
    for (uint32_t j = 0; j < n; ++j) {
        uint32_t x = B.leaf_parent[j];
        while (x != 0xFFFFFFFFu) {
            if (++visits[x] < 2) break;
            auto c = [&](uint32_t ref) { return (ref & LEAF) ? kCt * area(B.lbox[ref & ~LEAF]) : cost[ref]; };
            cost[x] = kCi * area(B.nbox[x]) + (c(B.left[x]) + c(B.right[x]));
            x = B.parent[x];
        }
    }
}

/* ------------------------------------------------------------ wide collapse */

void put_f32(uint8_t *p, float v) { std::memcpy(p, &v, 4); }
void put_u32(uint8_t *p, uint32_t v) { std::memcpy(p, &v, 4); }

void collapse(orc_bvh &B) {
    const uint32_t W = B.width;
    const uint32_t leaf_max = B.opts.leaf_max;
    B.node_bytes = ((24 + 7 * W) + 15) / 16 * 16;
    B.wide.clear();
    B.tris.clear();
    B.n_wide = 0;
    B.depth = 0;
    if (B.ntri == 0) return;
    std::vector<uint32_t> level{B.root()};
    uint32_t next_node = 1, tri_next = 0;
    while (!level.empty()) {
        const size_t L = level.size();
        std::vector<std::vector<uint32_t>> ents(L);
        std::vector<uint32_t> ic(L), tc(L);
        for (size_t k = 0; k < L; ++k) {
            const uint32_t r = level[k];
            std::vector<uint32_t> &e = ents[k];
            if (r & LEAF) {
                e.push_back(r);
            } else {
                e.push_back(B.left[r]);
                e.push_back(B.right[r]);
                while (e.size() < W) {
                    int best = -1;
                    float best_a = -1.0f;
                    for (size_t j = 0; j < e.size(); ++j) {
                        if (e[j] & LEAF) continue;
                        const float a = area(B.nbox[e[j]]);
                        if (a > best_a) { best_a = a; best = (int)j; }
                    }
                    if (best < 0) break;
                    const uint32_t x = e[best];
                    e[best] = B.left[x];
                    e.push_back(B.right[x]);
                }
            }
            uint32_t ni = 0, nt = 0;
            for (uint32_t x : e) {
                const uint32_t c = B.count_of(x);
                if ((x & LEAF) || c <= leaf_max) nt += c;
                else ni++;
            }
            ic[k] = ni;
            tc[k] = nt;
        }
        uint32_t sum_ic = 0, sum_tc = 0;
        std::vector<uint32_t> cbase(L), tbase(L);
        for (size_t k = 0; k < L; ++k) {
            cbase[k] = next_node + sum_ic;
            tbase[k] = tri_next + sum_tc;
            sum_ic += ic[k];
            sum_tc += tc[k];
        }
        const uint32_t node_start = next_node - (uint32_t)L;
        B.wide.resize((size_t)(node_start + L) * B.node_bytes, 0);
        B.tris.resize((size_t)(tri_next + sum_tc) * 12, 0.0f);
        std::vector<uint32_t> next_level(sum_ic);
        for (size_t k = 0; k < L; ++k) {
            const std::vector<uint32_t> &e = ents[k];
            const int m = (int)e.size();
            /* node box and centroid */
            Box nb = B.box_of(e[0]);
            for (int j = 1; j < m; ++j) nb = merge(nb, B.box_of(e[j]));
            float pc[3];
            for (int a = 0; a < 3; ++a) pc[a] = (nb.lo[a] + nb.hi[a]) * 0.5f;
            /* greedy octant assignment: highest score first, ties by child then code */
            float score[8][8];
            for (int i = 0; i < m; ++i) {
                const Box &cb = B.box_of(e[i]);
                float off[3];
                for (int a = 0; a < 3; ++a) off[a] = (cb.lo[a] + cb.hi[a]) * 0.5f - pc[a];
                for (int c = 0; c < 8; ++c) {
                    const float sx = (c & 4) ? -1.0f : 1.0f, sy = (c & 2) ? -1.0f : 1.0f, sz = (c & 1) ? -1.0f : 1.0f;
                    score[i][c] = (off[0] * sx + off[1] * sy) + off[2] * sz;
                }
            }
            int code_of[8];
            bool used_i[8] = {false}, used_c[8] = {false};
            for (int it = 0; it < m; ++it) {
                int bi = -1, bc = -1;
                float bs = 0.0f;
                for (int i = 0; i < m; ++i) {
                    if (used_i[i]) continue;
                    for (int c = 0; c < 8; ++c) {
                        if (used_c[c]) continue;
                        if (bi < 0 || score[i][c] > bs) { bs = score[i][c]; bi = i; bc = c; }
                    }
                }
                used_i[bi] = true;
                used_c[bc] = true;
                code_of[bi] = bc;
            }
            /* slots in ascending code order; for W = 8 slot == code */
            int child_at_code[8];
            for (int c = 0; c < 8; ++c) child_at_code[c] = -1;
            for (int i = 0; i < m; ++i) child_at_code[code_of[i]] = i;
            int slot_child[8];
            int ns = 0;
            for (int c = 0; c < 8; ++c) {
                if (W == 8) slot_child[c] = child_at_code[c];
                else if (child_at_code[c] >= 0) slot_child[ns++] = child_at_code[c];
            }
            if (W != 8)
                for (int s = ns; s < (int)W; ++s) slot_child[s] = -1;
            /* quantization grid (double, deterministic) */
            int ex[3];
            float p[3];
            for (int a = 0; a < 3; ++a) {
                const double lo = nb.lo[a], hi = nb.hi[a];
                const double ext = hi - lo;
                const double mag = std::max(std::fabs(lo), std::fabs(hi));
                int e = -126;
                if (ext > 0.0) e = std::max(e, ceil_log2(ext / 252.0));
                if (mag > 0.0) e = std::max(e, floor_log2(mag) - 21);
                if (e > 100) e = 100;
                ex[a] = e;
                const double pd = lo - std::ldexp(1.0, e);
                float pf = (float)pd;
                if ((double)pf > pd) pf = std::nextafter(pf, -std::numeric_limits<float>::infinity());
                p[a] = pf;
            }
            uint8_t *nd = &B.wide[(size_t)(node_start + k) * B.node_bytes];
            for (int a = 0; a < 3; ++a) put_f32(nd + 4 * a, p[a]);
            for (int a = 0; a < 3; ++a) nd[12 + a] = (uint8_t)(ex[a] + 127);
            uint8_t imask = 0;
            put_u32(nd + 16, cbase[k]);
            put_u32(nd + 20, tbase[k]);
            uint32_t toff = 0, crank = 0;
            /* internal children in ascending code order -> child array order */
            for (int c = 0; c < 8; ++c) {
                const int i = child_at_code[c];
                if (i < 0) continue;
                const uint32_t x = e[i];
                const bool leafslot = (x & LEAF) || B.count_of(x) <= leaf_max;
                if (!leafslot) {
                    imask |= (uint8_t)(1u << c);
                    next_level[cbase[k] - next_node + crank] = x;
                    crank++;
                }
            }
            nd[15] = imask;
            for (int s = 0; s < (int)W; ++s) {
                const int i = slot_child[s];
                if (i < 0) {
                    /* empty slot: inverted box (lo 255, hi 0) fails every slab test */
                    for (int a = 0; a < 3; ++a) nd[24 + W + a * W + s] = 255;
                    continue;
                }
                const uint32_t x = e[i];
                const Box &cb = B.box_of(x);
                const bool leafslot = (x & LEAF) || B.count_of(x) <= leaf_max;
                uint8_t meta;
                if (!leafslot) {
                    meta = (uint8_t)(0x20 | (24 + code_of[i]));
                } else {
                    const uint32_t cnt = B.count_of(x);
                    meta = (uint8_t)((((1u << cnt) - 1u) << 5) | toff);
                    /* gather triangles of this subtree, left first */
                    std::vector<uint32_t> st{x};
                    while (!st.empty()) {
                        const uint32_t y = st.back();
                        st.pop_back();
                        if (y & LEAF) {
                            const uint32_t prim = B.order[y & ~LEAF];
                            float *t = &B.tris[(size_t)(tbase[k] + toff) * 12];
                            const float *v = &B.verts[(size_t)prim * 9];
                            t[0] = v[0]; t[1] = v[1]; t[2] = v[2];
                            std::memcpy(&t[3], &prim, 4);
                            t[4] = v[3]; t[5] = v[4]; t[6] = v[5]; t[7] = 0.0f;
                            t[8] = v[6]; t[9] = v[7]; t[10] = v[8]; t[11] = 0.0f;
                            toff++;
                        } else {
                            st.push_back(B.right[y]);
                            st.push_back(B.left[y]);
                        }
                    }
                }
                nd[24 + s] = meta;
                for (int a = 0; a < 3; ++a) {
                    const double sc = std::ldexp(1.0, -ex[a]);
                    double ql = std::floor(((double)cb.lo[a] - (double)p[a]) * sc) - 1.0;
                    double qh = std::ceil(((double)cb.hi[a] - (double)p[a]) * sc) + 1.0;
                    if (ql < 0.0) ql = 0.0;
                    if (qh > 255.0) qh = 255.0;
                    nd[24 + W + a * W + s] = (uint8_t)ql;
                    nd[24 + 4 * W + a * W + s] = (uint8_t)qh;
                }
            }
        }
        B.n_wide = next_node + sum_ic;
        next_node += sum_ic;
        tri_next += sum_tc;
        B.depth++;
        level.swap(next_level);
    }
    B.wide.resize((size_t)B.n_wide * B.node_bytes, 0);
}

/* ------------------------------------------------------------ ray/triangle */

struct RayPre {
    float o[3], d[3], invd[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float tmin, tmax;
};

RayPre prep(const crg_ray &r) {
    RayPre p;
    for (int a = 0; a < 3; ++a) {
        p.o[a] = r.org[a];
        p.d[a] = r.dir[a];
        float dd = r.dir[a];
        if (std::fabs(dd) < 8.27180613e-25f) dd = std::copysign(8.27180613e-25f, dd); /* 2^-80 */
        p.invd[a] = 1.0f / dd;
    }
    int kz = 0;
    if (std::fabs(p.d[1]) > std::fabs(p.d[kz])) kz = 1;
    if (std::fabs(p.d[2]) > std::fabs(p.d[kz])) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    if (p.d[kz] < 0.0f) std::swap(kx, ky);
    p.kx = kx; p.ky = ky; p.kz = kz;
    p.Sx = p.d[kx] / p.d[kz];
    p.Sy = p.d[ky] / p.d[kz];
    p.Sz = 1.0f / p.d[kz];
    p.tmin = r.tmin;
    p.tmax = r.tmax;
    return p;
}

/* Watertight test; returns true and fills t,u,v when the ray crosses the triangle. */
bool watertight(const RayPre &r, const float *v0, const float *v1, const float *v2, float &t, float &u,
                float &v) {
    const float A[3] = {v0[0] - r.o[0], v0[1] - r.o[1], v0[2] - r.o[2]};
    const float Bv[3] = {v1[0] - r.o[0], v1[1] - r.o[1], v1[2] - r.o[2]};
    const float C[3] = {v2[0] - r.o[0], v2[1] - r.o[1], v2[2] - r.o[2]};
    const float Ax = A[r.kx] - r.Sx * A[r.kz];
    const float Ay = A[r.ky] - r.Sy * A[r.kz];
    const float Bx = Bv[r.kx] - r.Sx * Bv[r.kz];
    const float By = Bv[r.ky] - r.Sy * Bv[r.kz];
    const float Cx = C[r.kx] - r.Sx * C[r.kz];
    const float Cy = C[r.ky] - r.Sy * C[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float Wt = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || Wt == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        Wt = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || Wt < 0.0f) && (U > 0.0f || V > 0.0f || Wt > 0.0f)) return false;
    const float det = (U + V) + Wt;
    if (det == 0.0f) return false;
    const float Az = r.Sz * A[r.kz];
    const float Bz = r.Sz * Bv[r.kz];
    const float Cz = r.Sz * C[r.kz];
    const float T = (U * Az + V * Bz) + Wt * Cz;
    t = T / det;
    u = V / det;
    v = Wt / det;
    return true;
}

inline bool accept(float t, uint32_t prim, float tmin, float best_t, uint32_t best_prim) {
    if (!(t > tmin)) return false;
    if (t < best_t) return true;
    return t == best_t && best_prim != CRG_INVALID_PRIM && prim < best_prim;
}

/* Slack on the best-hit bound: a triangle's computed t can sit below its exact
 * t by more than slab rounding (t = T / det on large or grazing triangles), so
 * a box is kept while its entry lies within best_t * (1 + 2^-12); the GPU
 * traversal uses the same slack, so both find the closest computed t. */
constexpr float kHitSlack = 1.000244140625f;

bool slab(const RayPre &r, const Box &b, float tmax, float *tnear = nullptr) {
    float t0 = r.tmin, t1 = tmax * kHitSlack;
    for (int a = 0; a < 3; ++a) {
        float tn = (b.lo[a] - r.o[a]) * r.invd[a];
        float tf = (b.hi[a] - r.o[a]) * r.invd[a];
        if (tn > tf) std::swap(tn, tf);
        tf = tf * 1.00000036f; /* 1 + 2*gamma(3) */
        t0 = tn > t0 ? tn : t0;
        t1 = tf < t1 ? tf : t1;
        if (t0 > t1) return false;
    }
    if (tnear) *tnear = t0;
    return true;
}

template <bool ANY>
void trace(const orc_bvh &B, const crg_ray &ray, crg_hit &hit, bool &occl) {
    hit.t = std::numeric_limits<float>::infinity();
    hit.prim = CRG_INVALID_PRIM;
    hit.u = hit.v = 0.0f;
    occl = false;
    if (B.ntri == 0) return;
    const RayPre r = prep(ray);
    float best_t = r.tmax;
    uint32_t best_prim = CRG_INVALID_PRIM;
    /* front-to-back: children are tested on push, the nearer one popped first;
     * entries carry their entry distance and are skipped once beyond best_t */
    uint32_t stack[128];
    float stack_t[128];
    int sp = 0;
    {
        float t0;
        if (!slab(r, B.box_of(B.root()), best_t, &t0)) return;
        stack[sp] = B.root();
        stack_t[sp++] = t0;
    }
    while (sp > 0) {
        --sp;
        const uint32_t x = stack[sp];
        if (stack_t[sp] > best_t * kHitSlack) continue;
        if (x & LEAF) {
            const uint32_t prim = B.order[x & ~LEAF];
            const float *v = &B.verts[(size_t)prim * 9];
            float t, u, vv;
            if (!watertight(r, v, v + 3, v + 6, t, u, vv)) continue;
            if (ANY) {
                if (t > r.tmin && t < r.tmax) { occl = true; return; }
                continue;
            }
            if (accept(t, prim, r.tmin, best_t, best_prim)) {
                best_t = t;
                best_prim = prim;
                hit.t = t;
                hit.prim = prim;
                hit.u = u;
                hit.v = vv;
            }
        } else {
            if (sp + 2 > 128) continue; /* cannot happen for n < 2^30 */
            float tl = 0.0f, tr = 0.0f;
            const bool hl = slab(r, B.box_of(B.left[x]), best_t, &tl);
            const bool hr = slab(r, B.box_of(B.right[x]), best_t, &tr);
            if (hl && hr) {
                const bool left_first = tl <= tr;
                stack[sp] = left_first ? B.right[x] : B.left[x];
                stack_t[sp++] = left_first ? tr : tl;
                stack[sp] = left_first ? B.left[x] : B.right[x];
                stack_t[sp++] = left_first ? tl : tr;
            } else if (hl) {
                stack[sp] = B.left[x];
                stack_t[sp++] = tl;
            } else if (hr) {
                stack[sp] = B.right[x];
                stack_t[sp++] = tr;
            }
        }
    }
}

template <typename F>
void parallel_for(uint64_t n, int nthreads, F f) {
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    if ((uint64_t)nthreads > n) nthreads = (int)std::max<uint64_t>(1, n);
    if (nthreads == 1) {
        for (uint64_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> th;
    std::atomic<uint64_t> next{0};
    for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&]() {
            for (;;) {
                const uint64_t s = next.fetch_add(1024);
                if (s >= n) break;
                const uint64_t e = std::min<uint64_t>(n, s + 1024);
                for (uint64_t i = s; i < e; ++i) f(i);
            }
        });
    for (auto &t : th) t.join();
}

} // namespace

/* ------------------------------------------------------------ exported */

extern "C" {

uint32_t orc_morton3(float x, float y, float z) {
    return (spread10((uint32_t)x) << 2) | (spread10((uint32_t)y) << 1) | spread10((uint32_t)z);
}

int orc_bvh_build(const float *verts, uint32_t ntri, const crg_build_opts *opts, orc_bvh **out) {
    if (!out || (ntri > 0 && !verts)) return CRG_ERR_INVALID_ARG;
    orc_bvh *B = new orc_bvh();
    crg_build_opts o{8, 0, 3, 3};
    if (opts) o = *opts;
    if (o.width != 2 && o.width != 4 && o.width != 8) { delete B; return CRG_ERR_INVALID_ARG; }
    if (o.leaf_max < 1 || o.leaf_max > 3) { delete B; return CRG_ERR_INVALID_ARG; }
    B->opts = o;
    B->width = o.width;
    B->ntri = ntri;
    B->verts.assign(verts, verts + (size_t)ntri * 9);
    const uint32_t n = ntri;
    if (n == 0) { *out = B; return CRG_OK; }
    /* 1. bounds */
    std::vector<Box> tb(n);
    std::vector<float> cen((size_t)n * 3);
    float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = 0; i < n; ++i) {
        tb[i] = tri_box(&verts[(size_t)i * 9]);
        for (int a = 0; a < 3; ++a) {
            const float c = (tb[i].lo[a] + tb[i].hi[a]) * 0.5f;
            cen[(size_t)i * 3 + a] = c;
            clo[a] = fmn(clo[a], c);
            chi[a] = fmx(chi[a], c);
        }
    }
    /* 2. Morton codes */
    float scale[3];
    for (int a = 0; a < 3; ++a) {
        const float ext = chi[a] - clo[a];
        scale[a] = ext > 0.0f ? 1024.0f / ext : 0.0f;
    }
    std::vector<uint64_t> keys(n);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            const float f = (cen[(size_t)i * 3 + a] - clo[a]) * scale[a];
            q[a] = (uint32_t)fmn(fmx(f, 0.0f), 1023.0f);
        }
        const uint32_t code = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
        keys[i] = ((uint64_t)code << 32) | i;
    }
    /* 3. sort */
    std::sort(keys.begin(), keys.end());
    std::vector<uint32_t> code(n);
    B->order.resize(n);
    for (uint32_t j = 0; j < n; ++j) {
        code[j] = (uint32_t)(keys[j] >> 32);
        B->order[j] = (uint32_t)(keys[j] & 0xFFFFFFFFu);
    }
    B->lbox.resize(n);
    for (uint32_t j = 0; j < n; ++j) B->lbox[j] = tb[B->order[j]];
    B->leaf_parent.assign(n, 0xFFFFFFFFu);
    if (n >= 2) {
        /* 4. Karras hierarchy */
        B->left.resize(n - 1);
        B->right.resize(n - 1);
        B->parent.assign(n - 1, 0xFFFFFFFFu);
        const int N = (int)n;
        for (int i = 0; i < N - 1; ++i) {
            const int d = (delta(code.data(), N, i, i + 1) - delta(code.data(), N, i, i - 1)) >= 0 ? 1 : -1;
            const int dmin = delta(code.data(), N, i, i - d);
            int lmax = 2;
            while (delta(code.data(), N, i, i + lmax * d) > dmin) lmax *= 2;
            int l = 0;
            for (int t = lmax / 2; t >= 1; t /= 2)
                if (delta(code.data(), N, i, i + (l + t) * d) > dmin) l += t;
            const int j = i + l * d;
            const int dnode = delta(code.data(), N, i, j);
            int s = 0, t = l;
            do {
                t = (t + 1) >> 1;
                if (delta(code.data(), N, i, i + (s + t) * d) > dnode) s += t;
            } while (t > 1);
            const int g = i + s * d + std::min(d, 0);
            const uint32_t lc = (std::min(i, j) == g) ? (LEAF | (uint32_t)g) : (uint32_t)g;
            const uint32_t rc = (std::max(i, j) == g + 1) ? (LEAF | (uint32_t)(g + 1)) : (uint32_t)(g + 1);
            B->left[i] = lc;
            B->right[i] = rc;
            if (lc & LEAF) B->leaf_parent[lc & ~LEAF] = (uint32_t)i; else B->parent[lc] = (uint32_t)i;
            if (rc & LEAF) B->leaf_parent[rc & ~LEAF] = (uint32_t)i; else B->parent[rc] = (uint32_t)i;
        }
        /* 5. bottom-up boxes and counts (second visitor computes, as on the GPU) */
        B->nbox.resize(n - 1);
        B->count.assign(n - 1, 0);
        std::vector<uint32_t> visits(n - 1, 0);
        for (uint32_t j = 0; j < n; ++j) {
            uint32_t x = B->leaf_parent[j];
            while (x != 0xFFFFFFFFu) {
                if (++visits[x] < 2) break;
                B->nbox[x] = merge(B->box_of(B->left[x]), B->box_of(B->right[x]));
                B->count[x] = B->count_of(B->left[x]) + B->count_of(B->right[x]);
                x = B->parent[x];
            }
        }
        /* 6. treelets */
        std::vector<float> cost;
        compute_costs(*B, cost);
        if (o.treelet) {
            uint32_t gamma = 7;
            for (uint32_t round = 0; round < o.treelet_rounds; ++round) {
                treelet_pass(*B, gamma, cost);
                gamma *= 2;
            }
        }
        compute_costs(*B, cost);
        const float root_area = area(B->nbox[0]);
        B->sah = root_area > 0.0f ? cost[0] / root_area : 0.0f;
    }
    /* 7. wide collapse */
    collapse(*B);
    *out = B;
    return CRG_OK;
}

void orc_bvh_free(orc_bvh *b) { delete b; }

void orc_bvh_info(const orc_bvh *b, crg_bvh_info *info) {
    info->ntri = b->ntri;
    info->width = b->width;
    info->n_bvh2_nodes = b->ntri >= 2 ? b->ntri - 1 : 0;
    info->n_wide_nodes = b->n_wide;
    info->node_bytes = b->node_bytes;
    info->n_tri_slots = (uint32_t)(b->tris.size() / 12);
    info->depth = b->depth;
    info->sah_cost = b->sah;
    info->leaf_max = b->opts.leaf_max;
    info->treelet = b->opts.treelet;
}

void orc_bvh_download(const orc_bvh *b, float *bvh2, uint32_t *order, void *wide, float *tris) {
    if (bvh2 && b->ntri >= 2) {
        for (uint32_t i = 0; i + 1 < b->ntri; ++i) {
            float *o = bvh2 + (size_t)i * 8;
            o[0] = b->nbox[i].lo[0]; o[1] = b->nbox[i].lo[1]; o[2] = b->nbox[i].lo[2];
            std::memcpy(&o[3], &b->left[i], 4);
            o[4] = b->nbox[i].hi[0]; o[5] = b->nbox[i].hi[1]; o[6] = b->nbox[i].hi[2];
            std::memcpy(&o[7], &b->right[i], 4);
        }
    }
    if (order) std::copy(b->order.begin(), b->order.end(), order);
    if (wide) std::memcpy(wide, b->wide.data(), b->wide.size());
    if (tris) std::memcpy(tris, b->tris.data(), b->tris.size() * sizeof(float));
}

void orc_intersect_closest(const orc_bvh *b, const crg_ray *rays, crg_hit *hits, uint64_t n, int nthreads) {
    parallel_for(n, nthreads, [&](uint64_t i) {
        bool o;
        trace<false>(*b, rays[i], hits[i], o);
    });
}

void orc_intersect_any(const orc_bvh *b, const crg_ray *rays, uint32_t *occluded, uint64_t n, int nthreads) {
    parallel_for(n, nthreads, [&](uint64_t i) {
        crg_hit h;
        bool o;
        trace<true>(*b, rays[i], h, o);
        occluded[i] = o ? 1u : 0u;
    });
}

void orc_intersect_closest_brute(const float *verts, uint32_t ntri, const crg_ray *rays, crg_hit *hits,
                                 uint64_t n) {
    parallel_for(n, 0, [&](uint64_t i) {
        const RayPre r = prep(rays[i]);
        crg_hit h{std::numeric_limits<float>::infinity(), CRG_INVALID_PRIM, 0.0f, 0.0f};
        float best_t = r.tmax;
        uint32_t best_prim = CRG_INVALID_PRIM;
        for (uint32_t p = 0; p < ntri; ++p) {
            const float *v = verts + (size_t)p * 9;
            float t, u, vv;
            if (!watertight(r, v, v + 3, v + 6, t, u, vv)) continue;
            if (accept(t, p, r.tmin, best_t, best_prim)) {
                best_t = t;
                best_prim = p;
                h = crg_hit{t, p, u, vv};
            }
        }
        hits[i] = h;
    });
}

void orc_intersect_closest_f64(const float *verts, uint32_t ntri, const crg_ray *rays, double *t64,
                               uint32_t *prim, double *edge_dist, uint64_t n) {
    parallel_for(n, 0, [&](uint64_t i) {
        const crg_ray &r = rays[i];
        double best = std::numeric_limits<double>::infinity();
        uint32_t bp = CRG_INVALID_PRIM;
        double bed = 0.0;
        const double o[3] = {r.org[0], r.org[1], r.org[2]}, d[3] = {r.dir[0], r.dir[1], r.dir[2]};
        for (uint32_t p = 0; p < ntri; ++p) {
            const float *v = verts + (size_t)p * 9;
            double e1[3], e2[3], s[3], pv[3], qv[3];
            for (int a = 0; a < 3; ++a) {
                e1[a] = (double)v[3 + a] - v[a];
                e2[a] = (double)v[6 + a] - v[a];
                s[a] = o[a] - v[a];
            }
            pv[0] = d[1] * e2[2] - d[2] * e2[1];
            pv[1] = d[2] * e2[0] - d[0] * e2[2];
            pv[2] = d[0] * e2[1] - d[1] * e2[0];
            const double det = e1[0] * pv[0] + e1[1] * pv[1] + e1[2] * pv[2];
            if (det == 0.0) continue;
            const double inv = 1.0 / det;
            const double u = (s[0] * pv[0] + s[1] * pv[1] + s[2] * pv[2]) * inv;
            qv[0] = s[1] * e1[2] - s[2] * e1[1];
            qv[1] = s[2] * e1[0] - s[0] * e1[2];
            qv[2] = s[0] * e1[1] - s[1] * e1[0];
            const double vv = (d[0] * qv[0] + d[1] * qv[1] + d[2] * qv[2]) * inv;
            const double t = (e2[0] * qv[0] + e2[1] * qv[1] + e2[2] * qv[2]) * inv;
            const double w = 1.0 - u - vv;
            const double ed = std::min(std::min(u, vv), w);
            if (ed < -1e-9) continue;
            if (!(t > r.tmin) || !(t < r.tmax)) continue;
            if (t < best) { best = t; bp = p; bed = ed; }
        }
        t64[i] = best;
        prim[i] = bp;
        edge_dist[i] = bed;
    });
}

} /* extern "C" */

/* internal accessors for orc_render.cpp */
namespace orc_internal {
bool closest(const orc_bvh *b, const crg_ray &ray, crg_hit &hit) {
    bool o;
    trace<false>(*b, ray, hit, o);
    return hit.prim != CRG_INVALID_PRIM;
}
bool any(const orc_bvh *b, const crg_ray &ray) {
    crg_hit h;
    bool o;
    trace<true>(*b, ray, h, o);
    return o;
}
const float *verts(const orc_bvh *b) { return b->verts.data(); }
} // namespace orc_internal
