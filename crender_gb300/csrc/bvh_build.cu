// bvh_build.cu — GPU LBVH builder and wide-BVH collapse (sm_103a).
//
// Replaces rtcCommitScene (CRender src/objects/model.cpp:52-97).  Pipeline:
//   k_bounds        triangle boxes + centroid bounds (order-preserving int atomics)
//   k_morton        30-bit Morton codes of AABB centres
//   radix sort      stable LSD, 8-bit digits, 4 passes: hist / scan / scatter
//                   (warp match_any ranking keeps equal digits in input order,
//                   so the result is the unique (code, index) order)
//   k_karras        Karras 2012 hierarchy, one thread per internal node
//   k_bottom_up     boxes and primitive counts, second arrival computes
//   k_costs         SAH cost per node (Ci = 1.2, Ct = 1), same bottom-up order
//   k_treelet       optional Karras & Aila 2013 treelet restructuring
//   k_collapse_*    level-by-level greedy collapse to a W-wide quantized BVH
// Every float decision is evaluated in the same order as the CPU form, so the
// binary tree, the wide nodes and the triangle array are bit-identical to a
// CPU run of the same algorithm.
#include <cfloat>
#include <cmath>
#include <mutex>

#include "crg_dev.cuh"
#include "crg_internal.h"

namespace crg {
namespace {

constexpr uint32_t LEAF = 0x80000000u;
constexpr uint32_t NONE = 0xFFFFFFFFu;

__device__ __forceinline__ float fmn(float a, float b) { return a < b ? a : b; }
__device__ __forceinline__ float fmx(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ uint32_t f2key(float f) {
    const uint32_t i = __float_as_uint(f);
    return (i & 0x80000000u) ? ~i : (i | 0x80000000u);
}
__device__ __forceinline__ float key2f(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
__device__ __forceinline__ float area3(float dx, float dy, float dz) { return 2.0f * ((dx * dy + dy * dz) + dz * dx); }

struct Box {
    float lo[3], hi[3];
};
__device__ __forceinline__ Box merge(const Box &a, const Box &b) {
    Box r;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        r.lo[k] = fmn(a.lo[k], b.lo[k]);
        r.hi[k] = fmx(a.hi[k], b.hi[k]);
    }
    return r;
}
__device__ __forceinline__ float area(const Box &b) {
    return area3(b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]);
}

// ----------------------------------------------------------------- bounds
__global__ void k_bounds(const float *__restrict__ v, uint32_t n, float4 *__restrict__ tbox, uint32_t *__restrict__ cb) {
    float mn3[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx3[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float *p = v + (size_t)i * 9;
        float lo[3], hi[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float x0 = p[a], x1 = p[3 + a], x2 = p[6 + a];
            lo[a] = fmn(fmn(x0, x1), x2);
            hi[a] = fmx(fmx(x0, x1), x2);
            const float c = (lo[a] + hi[a]) * 0.5f;
            mn3[a] = fminf(mn3[a], c);
            mx3[a] = fmaxf(mx3[a], c);
        }
        tbox[2 * (size_t)i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        tbox[2 * (size_t)i + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            mn3[a] = fminf(mn3[a], __shfl_xor_sync(0xFFFFFFFFu, mn3[a], off));
            mx3[a] = fmaxf(mx3[a], __shfl_xor_sync(0xFFFFFFFFu, mx3[a], off));
        }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(&cb[a], f2key(mn3[a]));
            atomicMax(&cb[3 + a], f2key(mx3[a]));
        }
    }
}

// Standard 10-bit interleave (Karras, "Thinking Parallel III", 2012).
__device__ __forceinline__ uint32_t expand10(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

__global__ void k_morton(const float4 *__restrict__ tbox, uint32_t n, const uint32_t *__restrict__ cb,
                         uint32_t *__restrict__ keys, uint32_t *__restrict__ vals) {
    float clo[3], scale[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        clo[a] = key2f(cb[a]);
        const float ext = key2f(cb[3 + a]) - clo[a];
        scale[a] = ext > 0.0f ? 1024.0f / ext : 0.0f;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 lo = tbox[2 * (size_t)i], hi = tbox[2 * (size_t)i + 1];
        const float c[3] = {(lo.x + hi.x) * 0.5f, (lo.y + hi.y) * 0.5f, (lo.z + hi.z) * 0.5f};
        uint32_t q[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) q[a] = (uint32_t)fmn(fmx((c[a] - clo[a]) * scale[a], 0.0f), 1023.0f);
        keys[i] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
        vals[i] = i;
    }
}

// ----------------------------------------------------------------- radix sort
constexpr int kSortThreads = 256;
constexpr int kSortTile = 4096; // 8 warps x 512 consecutive keys

__global__ void __launch_bounds__(kSortThreads) k_hist(const uint32_t *__restrict__ keys, uint32_t n, int shift,
                                                       uint32_t *__restrict__ hist) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile;
    for (int k = 0; k < kSortTile / kSortThreads; ++k) {
        const uint32_t i = base + k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m words in place, one block of 1024 threads; optionally
// stores the total in *total.
__global__ void __launch_bounds__(1024) k_scan(uint32_t *__restrict__ a, uint32_t m, uint32_t *__restrict__ total) {
    __shared__ uint32_t part[1024];
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(m, b + per);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += a[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const uint32_t x = threadIdx.x >= (uint32_t)off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (uint32_t i = b; i < e; ++i) {
        const uint32_t x = a[i];
        a[i] = run;
        run += x;
    }
    if (total && threadIdx.x == 1023) *total = part[1023];
}

__global__ void __launch_bounds__(kSortThreads) k_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
                                                          uint32_t n, int shift, const uint32_t *__restrict__ hist,
                                                          uint32_t *__restrict__ kout, uint32_t *__restrict__ vout) {
    __shared__ uint32_t wcnt[8][256];
    __shared__ uint32_t goff[256];
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
#pragma unroll
    for (int k = 0; k < 8; ++k) wcnt[k][tid] = 0;
    goff[tid] = hist[tid * gridDim.x + blockIdx.x];
    __syncthreads();
    const uint32_t base = blockIdx.x * kSortTile + w * 512;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t kk[16], vv[16], rk[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const uint32_t i = base + r * 32 + lane;
        const bool valid = i < n;
        const uint32_t key = valid ? kin[i] : 0u;
        const uint32_t val = valid ? vin[i] : 0u;
        const uint32_t d = (key >> shift) & 255u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, valid ? d : 256u + lane);
        const uint32_t before = valid ? wcnt[w][d] : 0u;
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) wcnt[w][d] += __popc(peers);
        __syncwarp();
        kk[r] = key;
        vv[r] = val;
        rk[r] = before + __popc(peers & lt);
    }
    __syncthreads();
    {
        uint32_t run = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const uint32_t c = wcnt[k][tid];
            wcnt[k][tid] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 16; ++r) {
        const uint32_t i = base + r * 32 + lane;
        if (i < n) {
            const uint32_t d = (kk[r] >> shift) & 255u;
            const uint32_t pos = goff[d] + wcnt[w][d] + rk[r];
            kout[pos] = kk[r];
            vout[pos] = vv[r];
        }
    }
}

// ----------------------------------------------------------------- hierarchy
__device__ __forceinline__ int kdelta(const uint32_t *__restrict__ code, int n, int i, int j) {
    if (j < 0 || j > n - 1) return -1;
    const uint32_t a = code[i], b = code[j];
    if (a != b) return __clz(a ^ b);
    return 32 + __clz((uint32_t)i ^ (uint32_t)j);
}

__global__ void k_karras(const uint32_t *__restrict__ code, int n, float4 *__restrict__ nbox,
                         uint32_t *__restrict__ parent, uint32_t *__restrict__ leaf_parent) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n - 1; i += gridDim.x * blockDim.x) {
        const int d = (kdelta(code, n, i, i + 1) - kdelta(code, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = kdelta(code, n, i, i - d);
        int lmax = 2;
        while (kdelta(code, n, i, i + lmax * d) > dmin) lmax *= 2;
        int l = 0;
        for (int t = lmax / 2; t >= 1; t /= 2)
            if (kdelta(code, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        const int dnode = kdelta(code, n, i, j);
        int s = 0, t = l;
        do {
            t = (t + 1) >> 1;
            if (kdelta(code, n, i, i + (s + t) * d) > dnode) s += t;
        } while (t > 1);
        const int g = i + s * d + min(d, 0);
        const uint32_t lc = (min(i, j) == g) ? (LEAF | (uint32_t)g) : (uint32_t)g;
        const uint32_t rc = (max(i, j) == g + 1) ? (LEAF | (uint32_t)(g + 1)) : (uint32_t)(g + 1);
        nbox[2 * (size_t)i] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(lc));
        nbox[2 * (size_t)i + 1] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(rc));
        if (lc & LEAF) leaf_parent[lc & ~LEAF] = (uint32_t)i; else parent[lc] = (uint32_t)i;
        if (rc & LEAF) leaf_parent[rc & ~LEAF] = (uint32_t)i; else parent[rc] = (uint32_t)i;
        if (i == 0) parent[0] = NONE;
    }
}

struct Tree {
    const float4 *tbox;
    const uint32_t *order;
    float4 *nbox;
    uint32_t *parent;
    uint32_t *leaf_parent;
    uint32_t *count;
    float *cost;
};

// Coherent (L2) reads of data written by other threads of the same kernel.
__device__ __forceinline__ Box box_of_cg(const Tree &T, uint32_t r) {
    float4 lo, hi;
    if (r & LEAF) {
        const uint32_t prim = T.order[r & ~LEAF];
        lo = T.tbox[2 * (size_t)prim];
        hi = T.tbox[2 * (size_t)prim + 1];
    } else {
        lo = __ldcg(&T.nbox[2 * (size_t)r]);
        hi = __ldcg(&T.nbox[2 * (size_t)r + 1]);
    }
    return Box{{lo.x, lo.y, lo.z}, {hi.x, hi.y, hi.z}};
}
__device__ __forceinline__ uint32_t left_of(const Tree &T, uint32_t x) { return __float_as_uint(__ldcg(&T.nbox[2 * (size_t)x]).w); }
__device__ __forceinline__ uint32_t right_of(const Tree &T, uint32_t x) { return __float_as_uint(__ldcg(&T.nbox[2 * (size_t)x + 1]).w); }
__device__ __forceinline__ uint32_t count_of_cg(const Tree &T, uint32_t r) { return (r & LEAF) ? 1u : __ldcg(&T.count[r]); }

constexpr float kCi = 1.2f, kCt = 1.0f;

__device__ __forceinline__ float cost_of_cg(const Tree &T, uint32_t r) {
    if (r & LEAF) {
        const Box b = box_of_cg(T, r);
        return kCt * area(b);
    }
    return __ldcg(&T.cost[r]);
}

// mode 0: boxes + counts; mode 1: SAH costs.
__global__ void k_bottom_up(Tree T, uint32_t n, uint32_t *__restrict__ visits, int mode) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        uint32_t x = T.leaf_parent[j];
        while (x != NONE) {
            __threadfence();
            if (atomicAdd(&visits[x], 1u) == 0u) break;
            __threadfence();
            const uint32_t lc = left_of(T, x), rc = right_of(T, x);
            if (mode == 0) {
                const Box b = merge(box_of_cg(T, lc), box_of_cg(T, rc));
                T.nbox[2 * (size_t)x] = make_float4(b.lo[0], b.lo[1], b.lo[2], __uint_as_float(lc));
                T.nbox[2 * (size_t)x + 1] = make_float4(b.hi[0], b.hi[1], b.hi[2], __uint_as_float(rc));
                T.count[x] = count_of_cg(T, lc) + count_of_cg(T, rc);
            } else {
                const Box b = box_of_cg(T, x);
                T.cost[x] = kCi * area(b) + (cost_of_cg(T, lc) + cost_of_cg(T, rc));
            }
            x = __ldcg(&T.parent[x]);
        }
    }
}

// ----------------------------------------------------------------- treelets
// A warp's working set for one treelet, in shared memory.
struct TreeletWork {
    float aS[128], cS[128]; // subset areas and costs
    uint8_t pS[128];        // best partition of each subset
    uint32_t leaves[7], internals[6];
    float lb[7][6];         // the treelet leaves' boxes (lo.xyz, hi.xyz)
};

// The 7-leaf treelet rooted at r is restructured (Karras & Aila 2013) by the
// 32 lanes of a warp, with the same result as the CPU form: growth by largest
// area (first maximum), DP over subsets in increasing size with partitions
// containing the lowest set bit, first minimum kept (in the CPU's
// enumeration, q = rest, (q - 1) & rest, ...: the larger partition wins a
// tie), internal nodes reused in formation order, pre-order rebuild.  The
// growth step's areas, the subset areas and the DP are split over the lanes;
// the owning lane `leader` (the one whose arrival at r made it ready) writes
// the rebuilt nodes.
__device__ void optimize_treelet(const Tree &T, uint32_t r, bool leader, TreeletWork &w) {
    const uint32_t lane = threadIdx.x & 31u;
    float cost_r;
    {
        const Box b = box_of_cg(T, r);
        cost_r = kCi * area(b) + (cost_of_cg(T, left_of(T, r)) + cost_of_cg(T, right_of(T, r)));
        if (leader) T.cost[r] = cost_r;
    }
    int nl = 2, ni = 0;
    if (lane == 0u) {
        w.leaves[0] = left_of(T, r);
        w.leaves[1] = right_of(T, r);
    }
    __syncwarp();
    while (nl < 7) {
        // the internal leaf of largest area (lowest index on ties); none: the treelet is complete
        const uint32_t lj = (int)lane < nl ? w.leaves[lane] : LEAF;
        float a = -1.0f;
        if (!(lj & LEAF)) {
            a = area(box_of_cg(T, lj));
            if (!(a > -1.0f)) a = -1.0f; // NaN: never chosen
        }
        int bj = (int)lane;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const float oa = __shfl_xor_sync(0xFFFFFFFFu, a, off);
            const int oj = __shfl_xor_sync(0xFFFFFFFFu, bj, off);
            if (oa > a || (oa == a && oj < bj)) { a = oa; bj = oj; }
        }
        if (!(a > -1.0f)) break;
        const uint32_t x = __shfl_sync(0xFFFFFFFFu, lj, bj);
        if (lane == 0u) {
            w.internals[ni] = x;
            w.leaves[bj] = left_of(T, x);
            w.leaves[nl] = right_of(T, x);
        }
        ++ni;
        ++nl;
        __syncwarp();
    }
    if (nl < 3) {
        __syncwarp();
        return;
    }
    const int nsub = 1 << nl;
    if ((int)lane < nl) {
        const uint32_t lj = w.leaves[lane];
        const Box b = box_of_cg(T, lj);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            w.lb[lane][k] = b.lo[k];
            w.lb[lane][3 + k] = b.hi[k];
        }
        w.cS[1 << lane] = (lj & LEAF) ? kCt * area(b) : __ldcg(&T.cost[lj]);
        w.pS[1 << lane] = 0;
    }
    __syncwarp();
    for (int s = (int)lane + 1; s < nsub; s += 32) {
        const int j0 = __ffs(s) - 1;
        Box b{{w.lb[j0][0], w.lb[j0][1], w.lb[j0][2]}, {w.lb[j0][3], w.lb[j0][4], w.lb[j0][5]}};
        for (int j = j0 + 1; j < nl; ++j)
            if (s & (1 << j)) b = merge(b, Box{{w.lb[j][0], w.lb[j][1], w.lb[j][2]}, {w.lb[j][3], w.lb[j][4], w.lb[j][5]}});
        w.aS[s] = area(b);
    }
    __syncwarp();
    for (int k = 2; k <= nl; ++k) {
        if (k <= 5) {
            // a subset per lane (at most 15 partitions each), in the CPU's partition order
            for (int s = (int)lane + 1; s < nsub; s += 32) {
                if (__popc(s) != k) continue;
                float best = FLT_MAX;
                int bp = 0;
                const int low = s & -s;
                const int rest = s ^ low;
                for (int q = rest;; q = (q - 1) & rest) {
                    const int P = q | low;
                    if (P != s) {
                        const float c = w.cS[P] + w.cS[s ^ P];
                        if (c < best) { best = c; bp = P; }
                    }
                    if (q == 0) break;
                }
                w.cS[s] = kCi * w.aS[s] + best;
                w.pS[s] = (uint8_t)bp;
            }
        } else {
            // subsets of 6 or 7 leaves one at a time, their 31 / 63 partitions over the lanes
            for (int s = 1; s < nsub; ++s) {
                if (__popc(s) != k) continue;
                const int low = s & -s;
                const int rest = s ^ low;
                const int npart = (1 << (k - 1)) - 1; // q = rest (P == s) excluded
                float best = INFINITY;
                int bp = -1;
                for (int t = (int)lane; t < npart; t += 32) {
                    int q = 0, bit = 0; // deposit t's bits into rest's set bits
                    for (int rr = rest; rr; rr &= rr - 1, ++bit)
                        if (t & (1 << bit)) q |= rr & -rr;
                    const int P = q | low;
                    const float c = w.cS[P] + w.cS[s ^ P];
                    if (c < best || (c == best && P > bp)) { best = c; bp = P; }
                }
#pragma unroll
                for (int off = 16; off >= 1; off >>= 1) {
                    const float oc = __shfl_xor_sync(0xFFFFFFFFu, best, off);
                    const int op = __shfl_xor_sync(0xFFFFFFFFu, bp, off);
                    if (oc < best || (oc == best && op > bp)) { best = oc; bp = op; }
                }
                if (lane == 0u) {
                    w.cS[s] = kCi * w.aS[s] + best;
                    w.pS[s] = (uint8_t)bp;
                }
            }
        }
        __syncwarp();
    }
    const int full = nsub - 1;
    if (!(w.cS[full] < cost_r)) {
        __syncwarp();
        return;
    }
    if (leader) {
        // pre-order rebuild with an explicit stack; record (subset, node) pairs
        int st_s[8];
        uint32_t st_n[8];
        int sp = 0, next = 0;
        int post_s[6 + 1];
        uint32_t post_n[6 + 1];
        int np = 0;
        st_s[sp] = full;
        st_n[sp] = r;
        sp++;
        while (sp > 0) {
            --sp;
            const int S = st_s[sp];
            const uint32_t node = st_n[sp];
            const int P = w.pS[S];
            const int parts[2] = {P, S ^ P};
            uint32_t kids[2];
            for (int c = 0; c < 2; ++c) {
                if (__popc(parts[c]) == 1) kids[c] = w.leaves[__ffs(parts[c]) - 1];
                else kids[c] = w.internals[next++];
            }
            // children pointers (.w of the node's float4 pair); box written below
            T.nbox[2 * (size_t)node].w = __uint_as_float(kids[0]);
            T.nbox[2 * (size_t)node + 1].w = __uint_as_float(kids[1]);
            for (int c = 0; c < 2; ++c) {
                if (kids[c] & LEAF) T.leaf_parent[kids[c] & ~LEAF] = node;
                else T.parent[kids[c]] = node;
            }
            post_s[np] = S;
            post_n[np] = node;
            np++;
            for (int c = 1; c >= 0; --c)
                if (!(kids[c] & LEAF) && __popc(parts[c]) > 1) {
                    st_s[sp] = parts[c];
                    st_n[sp] = kids[c];
                    sp++;
                }
        }
        for (int q = np - 1; q >= 0; --q) {
            const int S = post_s[q];
            const uint32_t x = post_n[q];
            const int j0 = __ffs(S) - 1;
            Box b{{w.lb[j0][0], w.lb[j0][1], w.lb[j0][2]}, {w.lb[j0][3], w.lb[j0][4], w.lb[j0][5]}};
            for (int j = j0 + 1; j < nl; ++j)
                if (S & (1 << j)) b = merge(b, Box{{w.lb[j][0], w.lb[j][1], w.lb[j][2]}, {w.lb[j][3], w.lb[j][4], w.lb[j][5]}});
            const uint32_t lc = __float_as_uint(T.nbox[2 * (size_t)x].w), rc = __float_as_uint(T.nbox[2 * (size_t)x + 1].w);
            T.nbox[2 * (size_t)x] = make_float4(b.lo[0], b.lo[1], b.lo[2], __uint_as_float(lc));
            T.nbox[2 * (size_t)x + 1] = make_float4(b.hi[0], b.hi[1], b.hi[2], __uint_as_float(rc));
            T.count[x] = count_of_cg(T, lc) + count_of_cg(T, rc);
            T.cost[x] = w.cS[S];
        }
    }
    __syncwarp(); // the warp's next treelet reuses the working set
}

// Bottom-up pass over the tree by warps of 32 leaves: a lane goes on to a
// node's parent only on the node's second arrival (both subtrees final); the
// nodes of at least `gamma` leaves that the lanes reach in a step are
// restructured one after another by the whole warp.  Launched with 128
// threads per block.
__global__ void __launch_bounds__(128) k_treelet(Tree T, uint32_t n, uint32_t *__restrict__ visits, uint32_t gamma) {
    __shared__ TreeletWork s_w[4];
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t base = (blockIdx.x * (blockDim.x >> 5) + wib) * 32u; base < n; base += nwarps * 32u) {
        const uint32_t j = base + lane;
        uint32_t x = j < n ? __ldcg(&T.leaf_parent[j]) : NONE;
        bool active = x != NONE;
        while (__any_sync(0xFFFFFFFFu, active)) {
            bool need = false;
            if (active) {
                __threadfence();
                if (atomicAdd(&visits[x], 1u) == 0u) {
                    active = false;
                } else {
                    __threadfence();
                    need = __ldcg(&T.count[x]) >= gamma;
                }
            }
            uint32_t m;
            while ((m = __ballot_sync(0xFFFFFFFFu, need)) != 0u) {
                const int leader = __ffs(m) - 1;
                const uint32_t r = __shfl_sync(0xFFFFFFFFu, x, leader);
                optimize_treelet(T, r, (int)lane == leader, s_w[wib]);
                if ((int)lane == leader) need = false;
            }
            if (active) {
                x = __ldcg(&T.parent[x]);
                if (x == NONE) active = false;
            }
        }
    }
}

// ----------------------------------------------------------------- collapse
struct Collapse {
    Tree T;
    const float *verts;  // the BVH's own triangles (model-local indexing)
    uint32_t W, leaf_max, node_bytes;
    uint32_t prim_base;  // added to the primitive index stored in a triangle slot (scene-global ids)
};

__global__ void k_collapse_count(Collapse C, const uint32_t *__restrict__ level, uint32_t L, uint32_t *__restrict__ ents,
                                 uint32_t *__restrict__ nent, uint32_t *__restrict__ ic, uint32_t *__restrict__ tc) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
        const uint32_t r = level[k];
        uint32_t e[8];
        uint32_t m;
        if (r & LEAF) {
            e[0] = r;
            m = 1;
        } else {
            e[0] = left_of(C.T, r);
            e[1] = right_of(C.T, r);
            m = 2;
            while (m < C.W) {
                int best = -1;
                float best_a = -1.0f;
                for (uint32_t j = 0; j < m; ++j) {
                    if (e[j] & LEAF) continue;
                    const float a = area(box_of_cg(C.T, e[j]));
                    if (a > best_a) { best_a = a; best = (int)j; }
                }
                if (best < 0) break;
                const uint32_t x = e[best];
                e[best] = left_of(C.T, x);
                e[m++] = right_of(C.T, x);
            }
        }
        uint32_t ni = 0, nt = 0;
        for (uint32_t j = 0; j < m; ++j) {
            const uint32_t c = count_of_cg(C.T, e[j]);
            if ((e[j] & LEAF) || c <= C.leaf_max) nt += c;
            else ni++;
            ents[(size_t)k * 8 + j] = e[j];
        }
        nent[k] = m;
        ic[k] = ni;
        tc[k] = nt;
    }
}

__device__ __forceinline__ int ceil_log2(double x) {
    int k;
    const double m = frexp(x, &k);
    return (m == 0.5) ? k - 1 : k;
}
__device__ __forceinline__ int floor_log2(double x) {
    int k;
    frexp(x, &k);
    return k - 1;
}
__device__ __forceinline__ void put_byte(uint32_t *w, int b, uint32_t v) { w[b >> 2] |= (v & 0xFFu) << ((b & 3) * 8); }

__global__ void k_collapse_emit(Collapse C, const uint32_t *__restrict__ level, uint32_t L, const uint32_t *__restrict__ ents,
                                const uint32_t *__restrict__ nent, const uint32_t *__restrict__ cbase_rel,
                                const uint32_t *__restrict__ tbase_rel, uint32_t node_start, uint32_t next_start,
                                uint32_t tri_start, uint8_t *__restrict__ wide, float4 *__restrict__ tris,
                                uint32_t *__restrict__ next_level) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
        const int m = (int)nent[k];
        uint32_t e[8];
        Box cb[8];
        for (int j = 0; j < m; ++j) {
            e[j] = ents[(size_t)k * 8 + j];
            cb[j] = box_of_cg(C.T, e[j]);
        }
        Box nb = cb[0];
        for (int j = 1; j < m; ++j) nb = merge(nb, cb[j]);
        float pc[3];
        for (int a = 0; a < 3; ++a) pc[a] = (nb.lo[a] + nb.hi[a]) * 0.5f;
        float score[8][8];
        for (int i = 0; i < m; ++i) {
            float off[3];
            for (int a = 0; a < 3; ++a) off[a] = (cb[i].lo[a] + cb[i].hi[a]) * 0.5f - pc[a];
            for (int c = 0; c < 8; ++c) {
                const float sx = (c & 4) ? -1.0f : 1.0f, sy = (c & 2) ? -1.0f : 1.0f, sz = (c & 1) ? -1.0f : 1.0f;
                score[i][c] = (off[0] * sx + off[1] * sy) + off[2] * sz;
            }
        }
        int code_of[8];
        uint32_t used_i = 0, used_c = 0;
        for (int it = 0; it < m; ++it) {
            int bi = -1, bc = -1;
            float bs = 0.0f;
            for (int i = 0; i < m; ++i) {
                if (used_i & (1u << i)) continue;
                for (int c = 0; c < 8; ++c) {
                    if (used_c & (1u << c)) continue;
                    if (bi < 0 || score[i][c] > bs) { bs = score[i][c]; bi = i; bc = c; }
                }
            }
            used_i |= 1u << bi;
            used_c |= 1u << bc;
            code_of[bi] = bc;
        }
        int child_at_code[8];
        for (int c = 0; c < 8; ++c) child_at_code[c] = -1;
        for (int i = 0; i < m; ++i) child_at_code[code_of[i]] = i;
        int slot_child[8];
        int ns = 0;
        for (int c = 0; c < 8; ++c) {
            if (C.W == 8) slot_child[c] = child_at_code[c];
            else if (child_at_code[c] >= 0) slot_child[ns++] = child_at_code[c];
        }
        if (C.W != 8)
            for (int s = ns; s < (int)C.W; ++s) slot_child[s] = -1;
        int ex[3];
        float p[3];
        for (int a = 0; a < 3; ++a) {
            const double lo = nb.lo[a], hi = nb.hi[a];
            const double ext = hi - lo;
            const double mag = fmax(fabs(lo), fabs(hi));
            int eh = -126;
            if (ext > 0.0) eh = max(eh, ceil_log2(ext / 252.0));
            if (mag > 0.0) eh = max(eh, floor_log2(mag) - 21);
            if (eh > 100) eh = 100;
            ex[a] = eh;
            const double pd = lo - ldexp(1.0, eh);
            float pf = (float)pd;
            if ((double)pf > pd) pf = nextafterf(pf, -INFINITY);
            p[a] = pf;
        }
        uint32_t w[20];
        for (int q = 0; q < 20; ++q) w[q] = 0u;
        w[0] = __float_as_uint(p[0]);
        w[1] = __float_as_uint(p[1]);
        w[2] = __float_as_uint(p[2]);
        const uint32_t cbase = next_start + cbase_rel[k];
        const uint32_t tbase = tri_start + tbase_rel[k];
        w[4] = cbase;
        w[5] = tbase;
        uint32_t imask = 0, crank = 0;
        for (int c = 0; c < 8; ++c) {
            const int i = child_at_code[c];
            if (i < 0) continue;
            const uint32_t x = e[i];
            const bool leafslot = (x & LEAF) || count_of_cg(C.T, x) <= C.leaf_max;
            if (!leafslot) {
                imask |= 1u << c;
                next_level[cbase_rel[k] + crank] = x;
                crank++;
            }
        }
        w[3] = (uint32_t)(ex[0] + 127) | ((uint32_t)(ex[1] + 127) << 8) | ((uint32_t)(ex[2] + 127) << 16) | (imask << 24);
        const int W = (int)C.W;
        uint32_t toff = 0;
        for (int s = 0; s < W; ++s) {
            const int i = slot_child[s];
            if (i < 0) {
                // empty slot: inverted box (lo 255, hi 0) fails every slab test
                for (int a = 0; a < 3; ++a) put_byte(w, 24 + W + a * W + s, 255u);
                continue;
            }
            const uint32_t x = e[i];
            const bool leafslot = (x & LEAF) || count_of_cg(C.T, x) <= C.leaf_max;
            uint32_t meta;
            if (!leafslot) {
                meta = 0x20u | (24u + (uint32_t)code_of[i]);
            } else {
                const uint32_t cnt = count_of_cg(C.T, x);
                meta = (((1u << cnt) - 1u) << 5) | toff;
                uint32_t st[8];
                int sp = 0;
                st[sp++] = x;
                while (sp > 0) {
                    const uint32_t y = st[--sp];
                    if (y & LEAF) {
                        const uint32_t prim = C.T.order[y & ~LEAF];
                        const float *v = C.verts + (size_t)prim * 9;
                        float4 *t = tris + (size_t)(tbase + toff) * 3;
                        t[0] = make_float4(v[0], v[1], v[2], __uint_as_float(prim + C.prim_base));
                        t[1] = make_float4(v[3], v[4], v[5], 0.0f);
                        t[2] = make_float4(v[6], v[7], v[8], 0.0f);
                        toff++;
                    } else {
                        st[sp++] = right_of(C.T, y);
                        st[sp++] = left_of(C.T, y);
                    }
                }
            }
            put_byte(w, 24 + s, meta);
            for (int a = 0; a < 3; ++a) {
                const double sc = ldexp(1.0, -ex[a]);
                double ql = floor(((double)cb[i].lo[a] - (double)p[a]) * sc) - 1.0;
                double qh = ceil(((double)cb[i].hi[a] - (double)p[a]) * sc) + 1.0;
                if (ql < 0.0) ql = 0.0;
                if (qh > 255.0) qh = 255.0;
                put_byte(w, 24 + W + a * W + s, (uint32_t)ql);
                put_byte(w, 24 + 4 * W + a * W + s, (uint32_t)qh);
            }
        }
        uint4 *dst = reinterpret_cast<uint4 *>(wide + (size_t)(node_start + k) * C.node_bytes);
        for (uint32_t q = 0; q < C.node_bytes / 16; ++q) dst[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
    }
}

__global__ void k_fill(uint32_t *a, uint32_t n, uint32_t v) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = v;
}

inline uint32_t grid_for(uint64_t n, uint32_t threads, uint32_t cap = 152 * 32) {
    uint64_t g = (n + threads - 1) / threads;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (uint32_t)g;
}

// Where a build's scratch arrays come from: stream-ordered allocations for
// crg_scene_build, a fixed device array for crg_build_bvh_noalloc.  get()
// returns a 256-byte aligned block, or nullptr when none is available.
struct ScratchSource {
    virtual void *get(size_t bytes) = 0;
    virtual ~ScratchSource() = default;
};

// Scratch owned for the duration of one build (stream-ordered allocations).
struct AsyncScratch final : ScratchSource {
    cudaStream_t st;
    std::vector<void *> ptrs;
    cudaError_t err = cudaSuccess;
    explicit AsyncScratch(cudaStream_t s) : st(s) {}
    void *get(size_t bytes) override {
        void *p = nullptr;
        if (fault_injected()) {
            err = cudaErrorMemoryAllocation;
            return nullptr;
        }
        const cudaError_t e = cudaMallocAsync(&p, bytes + 16, st);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            err = e;
            return nullptr;
        }
        ptrs.push_back(p);
        return p;
    }
    ~AsyncScratch() override {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
};

// One BVH of n triangles written into a region of a scene's node arrays.
struct BvhTarget {
    const float *verts;  // float[n*9], the BVH's triangles
    uint32_t n;
    float4 *nbox;        // binary nodes float4[2*max(1, n-1)]; nullptr = take them from the scratch
    uint32_t *order;     // uint32[n]: sorted primitive order (BVH-local indices)
    uint8_t *wide;       // node array; this BVH's nodes start at node_base
    float4 *tris;        // triangle slot array; this BVH's slots start at slot_base
    uint32_t node_base, node_cap; // region of the node array reserved for this BVH
    uint32_t slot_base, prim_base;
};

struct BvhResult {
    uint32_t n_wide = 0, depth = 0;
    float sah = 0.0f;
};

// The build pipeline of this file's header comment, for one BVH.  Synchronises
// the stream once per wide-BVH level.  On failure *msg names the failing step.
crg_status build_pipeline(const BvhTarget &t, const crg_build_opts &o, ScratchSource &src, cudaStream_t st,
                          BvhResult &res, std::string *msg) {
    const uint32_t n = t.n;
    res = BvhResult{};
    if (n == 0) return CRG_OK;
    const uint32_t nint = n >= 2 ? n - 1 : 1;
    const uint32_t node_bytes = ((24 + 7 * o.width) + 15) / 16 * 16;
    const uint32_t nblk = (n + kSortTile - 1) / kSortTile;
    auto fail = [&](crg_status s, const std::string &m) {
        if (msg) *msg = m;
        return s;
    };
    auto cuda_fail = [&](cudaError_t e, const char *what) {
        (void)cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? CRG_ERR_OOM : CRG_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
    };
#define BP_CHECK(call)                                                                                                 \
    do {                                                                                                               \
        const cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);                                                            \
    } while (0)
    auto take = [&](size_t bytes) { return src.get((bytes + 255) / 256 * 256); };
    float4 *tbox = (float4 *)take(sizeof(float4) * 2 * (size_t)n);
    float4 *nbox = t.nbox ? t.nbox : (float4 *)take(sizeof(float4) * 2 * (size_t)nint);
    uint32_t *cb = (uint32_t *)take(sizeof(uint32_t) * 8);
    uint32_t *k0 = (uint32_t *)take(sizeof(uint32_t) * n), *v0 = (uint32_t *)take(sizeof(uint32_t) * n);
    uint32_t *k1 = (uint32_t *)take(sizeof(uint32_t) * n), *v1 = (uint32_t *)take(sizeof(uint32_t) * n);
    uint32_t *hist = (uint32_t *)take(sizeof(uint32_t) * 256 * (size_t)nblk);
    uint32_t *parent = (uint32_t *)take(sizeof(uint32_t) * nint), *leaf_parent = (uint32_t *)take(sizeof(uint32_t) * n);
    uint32_t *count = (uint32_t *)take(sizeof(uint32_t) * nint), *visits = (uint32_t *)take(sizeof(uint32_t) * nint);
    float *cost = (float *)take(sizeof(float) * nint);
    uint32_t *lvl0 = (uint32_t *)take(sizeof(uint32_t) * (n + 1)), *lvl1 = (uint32_t *)take(sizeof(uint32_t) * (n + 1));
    uint32_t *ents = (uint32_t *)take(sizeof(uint32_t) * 8 * (size_t)(n + 1));
    uint32_t *nent = (uint32_t *)take(sizeof(uint32_t) * (n + 1)), *ic = (uint32_t *)take(sizeof(uint32_t) * (n + 1));
    uint32_t *tc = (uint32_t *)take(sizeof(uint32_t) * (n + 1)), *totals = (uint32_t *)take(sizeof(uint32_t) * 2);
    if (!tbox || !nbox || !cb || !k0 || !v0 || !k1 || !v1 || !hist || !parent || !leaf_parent || !count || !visits ||
        !cost || !lvl0 || !lvl1 || !ents || !nent || !ic || !tc || !totals)
        return fail(CRG_ERR_OOM, "BVH build: no room for the build's scratch arrays");

    // centroid bounds start at the identities of min / max
    BP_CHECK(cudaMemsetAsync(cb, 0xFF, 3 * sizeof(uint32_t), st));
    BP_CHECK(cudaMemsetAsync(cb + 3, 0x00, 3 * sizeof(uint32_t), st));
    const uint32_t T = 256;
    k_bounds<<<grid_for(n, T), T, 0, st>>>(t.verts, n, tbox, cb);
    k_morton<<<grid_for(n, T), T, 0, st>>>(tbox, n, cb, k0, v0);
    // 4 passes: k0/v0 -> k1/v1 -> k0/v0 -> k1/v1 -> k0/v0: the sorted data ends in k0 / v0
    {
        uint32_t *ki = k0, *vi = v0, *ko = k1, *vo = v1;
        for (int pass = 0; pass < 4; ++pass) {
            k_hist<<<nblk, kSortThreads, 0, st>>>(ki, n, pass * 8, hist);
            k_scan<<<1, 1024, 0, st>>>(hist, 256 * nblk, nullptr);
            k_scatter<<<nblk, kSortThreads, 0, st>>>(ki, vi, n, pass * 8, hist, ko, vo);
            std::swap(ki, ko);
            std::swap(vi, vo);
        }
        BP_CHECK(cudaMemcpyAsync(t.order, v0, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st));
    }
    Tree Tr{tbox, t.order, nbox, parent, leaf_parent, count, cost};
    if (n >= 2) {
        k_karras<<<grid_for(n - 1, T), T, 0, st>>>(k0, (int)n, nbox, parent, leaf_parent);
        BP_CHECK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * nint, st));
        k_bottom_up<<<grid_for(n, T), T, 0, st>>>(Tr, n, visits, 0);
        BP_CHECK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * nint, st));
        k_bottom_up<<<grid_for(n, T), T, 0, st>>>(Tr, n, visits, 1);
        if (o.treelet) {
            uint32_t gamma = 7;
            for (uint32_t round = 0; round < o.treelet_rounds; ++round) {
                BP_CHECK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * nint, st));
                k_treelet<<<grid_for(n, 128), 128, 0, st>>>(Tr, n, visits, gamma);
                gamma *= 2;
            }
            BP_CHECK(cudaMemsetAsync(visits, 0, sizeof(uint32_t) * nint, st));
            k_bottom_up<<<grid_for(n, T), T, 0, st>>>(Tr, n, visits, 1);
        }
    } else {
        k_fill<<<1, 32, 0, st>>>(leaf_parent, 1, NONE);
    }
    BP_CHECK(cudaGetLastError());

    // level-by-level collapse into the target region
    Collapse Cc{Tr, t.verts, o.width, o.leaf_max, node_bytes, t.prim_base};
    k_fill<<<1, 32, 0, st>>>(lvl0, 1, n >= 2 ? 0u : LEAF);
    uint32_t L = 1, node_start = 0, next_start = 1, tri_start = 0, depth = 0;
    uint32_t *cur = lvl0, *nxt = lvl1;
    while (L > 0) {
        k_collapse_count<<<grid_for(L, 128), 128, 0, st>>>(Cc, cur, L, ents, nent, ic, tc);
        k_scan<<<1, 1024, 0, st>>>(ic, L, totals);
        k_scan<<<1, 1024, 0, st>>>(tc, L, totals + 1);
        k_collapse_emit<<<grid_for(L, 64), 64, 0, st>>>(Cc, cur, L, ents, nent, ic, tc, t.node_base + node_start,
                                                       t.node_base + next_start, t.slot_base + tri_start, t.wide,
                                                       t.tris, nxt);
        uint32_t h[2];
        BP_CHECK(cudaMemcpyAsync(h, totals, sizeof(h), cudaMemcpyDeviceToHost, st));
        BP_CHECK(cudaStreamSynchronize(st));
        BP_CHECK(cudaGetLastError());
        depth++;
        node_start = next_start;
        next_start += h[0];
        tri_start += h[1];
        L = h[0];
        std::swap(cur, nxt);
        // the next level writes nodes [node_start, next_start): stop before it would leave the region
        if (next_start > t.node_cap) return fail(CRG_ERR_DEVICE, "wide BVH node count exceeded capacity");
    }
    if (tri_start != n) return fail(CRG_ERR_DEVICE, "wide BVH triangle count mismatch");
    res.n_wide = next_start;
    res.depth = depth;
    if (n >= 2) {
        float c0 = 0.0f;
        float4 r[2];
        BP_CHECK(cudaMemcpyAsync(&c0, cost, sizeof(float), cudaMemcpyDeviceToHost, st));
        BP_CHECK(cudaMemcpyAsync(r, nbox, sizeof(r), cudaMemcpyDeviceToHost, st));
        BP_CHECK(cudaStreamSynchronize(st));
        const float dx = r[1].x - r[0].x, dy = r[1].y - r[0].y, dz = r[1].z - r[0].z;
        const float ra = 2.0f * ((dx * dy + dy * dz) + dz * dx);
        res.sah = ra > 0.0f ? c0 / ra : 0.0f;
    }
#undef BP_CHECK
    (void)node_bytes;
    return CRG_OK;
}

// Grows b to `bytes`, keeping its first `keep` bytes (device to device).
crg_status grow_keep(crg_context *ctx, DevBuf &b, size_t bytes, size_t keep, cudaStream_t st) {
    if (b.ptr && b.bytes >= bytes) return CRG_OK;
    DevBuf nb;
    crg_status rc = dev_alloc(ctx, nb, bytes);
    if (rc != CRG_OK) return rc;
    if (b.ptr && keep) {
        const cudaError_t e = cudaMemcpyAsync(nb.ptr, b.ptr, std::min(keep, b.bytes), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) (void)cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            dev_free(nb);
            return cuda_error(ctx, e, "cudaMemcpyAsync(grow)");
        }
    }
    dev_free(b);
    b = nb;
    return CRG_OK;
}

} // namespace

crg_status build_bvh(crg_scene *s, const crg_build_opts &o, cudaStream_t st) {
    crg_context *ctx = s->ctx;
    const bool same = s->opts.width == o.width && s->opts.treelet == o.treelet && s->opts.leaf_max == o.leaf_max &&
                      s->opts.treelet_rounds == o.treelet_rounds;
    if (!same)
        for (crg_model_rec &m : s->models) m.built = false;
    s->built = false;
    s->opts = o;
    s->width = o.width;
    s->node_bytes = ((24 + 7 * o.width) + 15) / 16 * 16;
    // node arrays: each model's region at node_base (fixed by the triangle counts)
    uint32_t cap = 0;
    for (const crg_model_rec &m : s->models) cap = std::max(cap, m.node_base + m.node_cap);
    const uint32_t old_cap = s->node_cap;
    const size_t keep_nodes = same ? old_cap : 0;
    crg_status rc;
    if (s->ntri > 0) {
        if ((rc = grow_keep(ctx, s->bvh2, sizeof(float4) * 2 * (size_t)cap, sizeof(float4) * 2 * keep_nodes, st)) != CRG_OK)
            return rc;
        if ((rc = grow_keep(ctx, s->wide, (size_t)s->node_bytes * cap, (size_t)s->node_bytes * keep_nodes, st)) != CRG_OK)
            return rc;
        size_t kept_prims = 0;
        for (const crg_model_rec &m : s->models)
            if (m.built) kept_prims = std::max<size_t>(kept_prims, (size_t)m.first + m.ntri);
        if ((rc = grow_keep(ctx, s->order, sizeof(uint32_t) * s->ntri, sizeof(uint32_t) * kept_prims, st)) != CRG_OK)
            return rc;
        if ((rc = grow_keep(ctx, s->tris, sizeof(float4) * 3 * s->ntri, sizeof(float4) * 3 * kept_prims, st)) != CRG_OK)
            return rc;
        if (cap > old_cap || !same) // unused node slots read as zero (deterministic downloads)
            CRG_CUDA(ctx, cudaMemsetAsync((uint8_t *)s->wide.ptr + (size_t)s->node_bytes * keep_nodes, 0,
                                          (size_t)s->node_bytes * (cap - keep_nodes), st));
    }
    s->node_cap = cap;
    for (crg_model_rec &m : s->models) {
        if (m.built) continue;
        BvhTarget t{(const float *)s->verts.ptr + (size_t)m.first * 9,
                    m.ntri,
                    (float4 *)s->bvh2.ptr + 2 * (size_t)m.node_base,
                    (uint32_t *)s->order.ptr + m.first,
                    (uint8_t *)s->wide.ptr,
                    (float4 *)s->tris.ptr,
                    m.node_base,
                    m.node_base + m.node_cap,
                    m.first,
                    m.first};
        AsyncScratch src(st);
        BvhResult res;
        std::string msg;
        rc = build_pipeline(t, o, src, st, res, &msg);
        if (rc != CRG_OK) {
            if (src.err != cudaSuccess) return cuda_error(ctx, src.err, "cudaMallocAsync(build scratch)");
            return set_error(ctx, rc, msg);
        }
        m.n_wide = res.n_wide;
        m.depth = res.depth;
        m.sah = res.sah;
        m.built = true;
    }
    // whole-scene figures: the single model's, or the sums / maxima over the models
    s->n_wide = 0;
    s->depth = 0;
    s->sah = 0.0f;
    for (const crg_model_rec &m : s->models) {
        s->depth = std::max(s->depth, m.depth);
        s->sah += m.sah;
    }
    s->n_wide = s->models.size() == 1 ? s->models[0].n_wide : cap;
    s->built = true;
    return CRG_OK;
}

} // namespace crg

// ----------------------------------------------------------------- build without allocation
// crg_build_bvh_noalloc: build_pipeline with its scratch carved from one
// file-scope __device__ array sized for CRG_NOALLOC_MAX_TRIS triangles; every
// GPU that loads this library holds it until the process exits.
namespace crg {
namespace {

constexpr size_t kNaN = CRG_NOALLOC_MAX_TRIS; // max triangles
constexpr size_t kNaBlk = (kNaN + kSortTile - 1) / kSortTile;
constexpr size_t na_round(size_t b) { return (b + 255) / 256 * 256; }
// the blocks build_pipeline takes for kNaN triangles, each rounded to 256 bytes
constexpr size_t kNaBytes = 2 * na_round(sizeof(float4) * 2 * kNaN) +    // triangle boxes, binary nodes
                            na_round(sizeof(uint32_t) * 8) +               // centroid bounds
                            4 * na_round(sizeof(uint32_t) * kNaN) +        // sort keys and values
                            na_round(sizeof(uint32_t) * 256 * kNaBlk) +    // digit histograms
                            5 * na_round(sizeof(uint32_t) * kNaN) +        // parent, leaf parent, count, visits, cost
                            2 * na_round(sizeof(uint32_t) * (kNaN + 1)) +  // collapse levels
                            na_round(sizeof(uint32_t) * 8 * (kNaN + 1)) +  // collapse entries
                            3 * na_round(sizeof(uint32_t) * (kNaN + 1)) +  // entry / internal / triangle counts
                            na_round(sizeof(uint32_t) * 2);                // level totals

__device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

// Device address of g_noalloc_scratch per device, fetched once with that
// device current (in host code the symbol's name is only a stand-in).
constexpr int kNaMaxDevices = 64;
unsigned char *g_noalloc_ptr[kNaMaxDevices] = {nullptr};
std::mutex g_noalloc_mutex;

crg_status noalloc_scratch(unsigned char **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) {
        (void)cudaGetLastError();
        return CRG_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
            (void)cudaGetLastError();
            return CRG_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = (unsigned char *)p;
    }
    *out = g_noalloc_ptr[dev];
    return CRG_OK;
}

// Bump allocation over the fixed array; never more than kNaBytes.
struct FixedScratch final : ScratchSource {
    unsigned char *base;
    size_t used = 0;
    explicit FixedScratch(unsigned char *b) : base(b) {}
    void *get(size_t bytes) override {
        if (bytes > kNaBytes - used) return nullptr;
        void *p = base + used;
        used += bytes;
        return p;
    }
};

// Message of this thread's last failed crg_build_bvh_noalloc call.
thread_local std::string g_noalloc_error;

crg_status noalloc_fail(crg_status s, const std::string &m) {
    g_noalloc_error = m;
    return s;
}

} // namespace

void noalloc_prepare() {
    unsigned char *p = nullptr;
    (void)noalloc_scratch(&p);
}

} // namespace crg

extern "C" const char *crg_noalloc_last_error(void) { return crg::g_noalloc_error.c_str(); }

extern "C" crg_status crg_build_bvh_noalloc(const float *d_verts, uint32_t ntri, const crg_build_opts *opts,
                                            void *d_wide, size_t wide_bytes, float *d_tris, uint32_t *d_order,
                                            crg_bvh_info *info, crg_stream stream) {
    using namespace crg;
    g_noalloc_error.clear();
    crg_build_opts o{8, 0, 3, 3};
    if (opts) o = *opts;
    if (!((o.width == 2 || o.width == 4 || o.width == 8) && o.leaf_max >= 1 && o.leaf_max <= 3 && o.treelet_rounds <= 8))
        return noalloc_fail(CRG_ERR_INVALID_ARG, "build options: width 2/4/8, leaf_max 1..3, treelet_rounds <= 8");
    if (ntri > CRG_NOALLOC_MAX_TRIS)
        return noalloc_fail(CRG_ERR_INVALID_ARG, "more triangles than CRG_NOALLOC_MAX_TRIS");
    const uint32_t n = ntri;
    const uint32_t node_bytes = ((24 + 7 * o.width) + 15) / 16 * 16;
    const uint32_t nint = n >= 2 ? n - 1 : 1;
    if (n > 0 && (!d_verts || !d_wide || !d_tris || !d_order)) return noalloc_fail(CRG_ERR_INVALID_ARG, "null buffer");
    if (n > 0 && wide_bytes < (size_t)node_bytes * nint)
        return noalloc_fail(CRG_ERR_INVALID_ARG, "node buffer smaller than node_bytes * max(1, ntri - 1)");
    if (info) {
        *info = crg_bvh_info{};
        info->ntri = n;
        info->width = o.width;
        info->leaf_max = o.leaf_max;
        info->treelet = o.treelet;
        info->node_bytes = node_bytes;
        info->n_bvh2_nodes = n >= 2 ? n - 1 : 0;
        info->n_tri_slots = n;
    }
    if (n == 0) return CRG_OK;
    unsigned char *base = nullptr;
    if (noalloc_scratch(&base) != CRG_OK) return noalloc_fail(CRG_ERR_CUDA, "cudaGetSymbolAddress(scratch array) failed");
    // an error left pending by the caller's earlier work is not this call's
    (void)cudaGetLastError();
    cudaStream_t st = (cudaStream_t)stream;
    FixedScratch src(base);
    BvhTarget t{d_verts, n, nullptr, d_order, (uint8_t *)d_wide, (float4 *)d_tris, 0, nint, 0, 0};
    BvhResult res;
    std::string msg;
    const crg_status rc = build_pipeline(t, o, src, st, res, &msg);
    if (rc != CRG_OK) {
        // kernels queued before the failure may still use the shared array:
        // let them finish so the caller's next call does not race with them
        (void)cudaStreamSynchronize(st);
        (void)cudaGetLastError();
        return noalloc_fail(rc, msg);
    }
    if (info) {
        info->n_wide_nodes = res.n_wide;
        info->depth = res.depth;
        info->sah_cost = res.sah;
    }
    return CRG_OK;
}
