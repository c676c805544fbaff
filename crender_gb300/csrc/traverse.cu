// traverse.cu — batched closest-hit / any-hit queries (the rtcIntersect1 /
// rtcOccluded1 replacements, CRender src/objects/model.cpp:5-49).
//
// One thread per ray; rays are two 16-byte loads, hits one 16-byte store.
// The wide nodes are read with 16-byte vector loads through the read-only
// path; per-thread group stack of 64 entries (overflow raises the scene's
// error word instead of trapping).
#include <algorithm>

#include "render_common.cuh"

namespace crg {
namespace {

// Queries on an instanced scene: model::intersect's loop over the instances
// (model.cpp:99-126) through the shared closest / any-hit functions.  The
// ray's tmin applies in each instance's object space (the reference's tnear);
// t is the world distance of the hit point.
template <int W, bool ANY>
__global__ void __launch_bounds__(128) k_intersect_inst(rc::SceneDev S, const float4 *__restrict__ rays,
                                                       float4 *__restrict__ hits, uint32_t *__restrict__ occluded,
                                                       uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 r0 = __ldg(&rays[2 * i]);
    const float4 r1 = __ldg(&rays[2 * i + 1]);
    const v3 o = mk(r0.x, r0.y, r0.z), d = mk(r1.x, r1.y, r1.z);
    rc::PathCtx C{0, 0, 0, 0, 0, 0, 0ull, 0ull};
    if (ANY) {
        occluded[i] = rc::occluded_t<W, false, true>(S, o, d, r0.w, r1.w, C) ? 1u : 0u;
    } else {
        rc::Hit h;
        if (rc::closest_t<W, false, true>(S, o, d, r0.w, r1.w, h, C)) {
            v3 oo, od;
            float len;
            rc::inst_ray(S, h.inst, o, d, oo, od, len);
            const float t = rc::vdist(rc::inst_point(S, h.inst, oo, od, h.t), o);
            hits[i] = make_float4(t, __uint_as_float(h.prim), h.u, h.v);
        } else {
            hits[i] = make_float4(INFINITY, __uint_as_float(0xFFFFFFFFu), 0.0f, 0.0f);
        }
    }
    if (C.err) atomicOr(S.err, C.err);
}

// One thread per ray.  (A persistent-block variant that refilled idle lanes
// from a shared-memory counter between traversal slices measured 21% slower
// on the 1M-triangle soup: its extra state cost occupancy.)
template <int W, bool ANY, bool COUNT>
__global__ void __launch_bounds__(128, 8) k_intersect(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                                   const float4 *__restrict__ rays, float4 *__restrict__ hits,
                                                   uint32_t *__restrict__ occluded, uint32_t *__restrict__ ncount,
                                                   uint32_t *__restrict__ tcount, uint64_t n, uint32_t ntri,
                                                   uint32_t *__restrict__ err) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 r0 = __ldg(&rays[2 * i]);
    const float4 r1 = __ldg(&rays[2 * i + 1]);
    float best_t = INFINITY, bu = 0.0f, bv = 0.0f;
    uint32_t best_prim = 0xFFFFFFFFu, best_slot;
    bool occ = false;
    TravStats st{0, 0};
    if (ntri > 0) {
        const RayPre r = ray_prep(r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r0.w);
        uint32_t e = 0;
        traverse<W, ANY, COUNT>(nodes, tris, r, r1.w, best_t, best_prim, best_slot, bu, bv, occ, st, e);
        if (e) atomicOr(err, e);
    }
    if (ANY) {
        occluded[i] = occ ? 1u : 0u;
    } else {
        if (best_prim == 0xFFFFFFFFu) {
            best_t = INFINITY;
            bu = bv = 0.0f;
        }
        hits[i] = make_float4(best_t, __uint_as_float(best_prim), bu, bv);
    }
    if (COUNT) {
        if (ncount) ncount[i] = st.nodes;
        if (tcount) tcount[i] = st.tris;
    }
}

// Persistent variant with per-lane ray refill (dyn_traverse): a lane whose
// ray is done takes the next ray index from *head while its warp's other
// lanes are still traversing.
template <int W, bool ANY>
__global__ void __launch_bounds__(128) k_intersect_dyn(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                                     const float4 *__restrict__ rays, float4 *__restrict__ hits,
                                                     uint32_t *__restrict__ occluded, unsigned int *head, uint32_t n,
                                                     uint32_t refill, uint32_t *__restrict__ err) {
    TravStats st{0, 0};
    uint32_t e = 0;
    dyn_traverse<W, ANY, false, 4>(
        head, n, refill,
        [&](unsigned int i, uint32_t &payload, RayPre &r, float &tmax, uint32_t &root, const uint4 *&nd,
            const float4 *&tr) {
            payload = i;
            root = 0u;
            const float4 r0 = __ldg(&rays[2 * (size_t)i]);
            const float4 r1 = __ldg(&rays[2 * (size_t)i + 1]);
            r = ray_prep(r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r0.w);
            tmax = r1.w;
            nd = nodes;
            tr = tris;
            return true;
        },
        [](uint32_t, const Trav &, RayPre &, float &, uint32_t &) { return false; },
        [&](uint32_t i, const Trav &T) {
            if (ANY) {
                occluded[i] = T.occluded ? 1u : 0u;
            } else if (T.best_prim == 0xFFFFFFFFu) {
                hits[i] = make_float4(INFINITY, __uint_as_float(0xFFFFFFFFu), 0.0f, 0.0f);
            } else {
                hits[i] = make_float4(T.best_t, __uint_as_float(T.best_prim), T.best_V / T.best_det, T.best_W / T.best_det);
            }
        },
        st, e);
    if (e) atomicOr(err, e);
}

// Warp-cooperative traversal: G = W lanes per ray, 32 / W rays per warp.  A
// ray's node is read with 16-byte vector loads by its lanes into shared
// memory, each lane tests one child box against the ray, and the hit bits are
// OR-reduced over the lanes; its pending triangles are tested G at a time (one
// per lane, 16-byte loads) and the lexicographic minimum (t, primitive) of
// the lanes' hits is reduced by shuffles, so the closest hit equals the
// per-thread traversal's (accept_hit's order, conservative culling).  Each
// ray keeps its group stack in the warp's shared memory; an idle group takes
// the next ray index with one atomic per warp for all idle groups.
template <int W>
struct WarpShared {
    static constexpr int R = 32 / W;
    uint4 node[4][R][NodeLayout<W>::VEC];
    uint2 stack[4][R][kStack];
};

// One iteration for the group in `gmask` (c = lane in group): the pending
// triangles, then one node.  Returns true when the ray is finished.
template <int W, bool ANY>
__device__ __forceinline__ bool warp_step(Trav &T, uint2 *stack, uint4 *nbuf, const uint4 *__restrict__ nodes,
                                          const float4 *__restrict__ tris, const RayPre &r, uint32_t gmask, uint32_t c,
                                          uint32_t &err) {
    using L = NodeLayout<W>;
    constexpr int G = W;
    while (T.tg.y != 0u) {
        const uint32_t pend = T.tg.y;
        const uint32_t pos = __fns(pend, 0, (int)c + 1);  // this lane's triangle: the (c+1)-th pending bit
        const uint32_t last = __fns(pend, 0, G);          // the G-th pending bit: all up to it are taken now
        T.tg.y = last == 0xFFFFFFFFu ? 0u : pend & ~((2u << last) - 1u);
        bool hit = false;
        float ct = INFINITY;
        uint32_t cp = 0xFFFFFFFFu, slot = 0u;
        TriHit h{0.0f, 0.0f, 0.0f, 1.0f};
        if (pos != 0xFFFFFFFFu) {
            slot = T.tg.x + pos;
            const float4 a = __ldg(&tris[slot * 3 + 0]);
            const float4 b = __ldg(&tris[slot * 3 + 1]);
            const float4 cc = __ldg(&tris[slot * 3 + 2]);
            hit = watertight(r, a, b, cc, h);
            if (ANY) {
                hit = hit && h.t > r.tmin && h.t < T.tmax;
            } else if (hit && h.t > r.tmin) {
                ct = h.t;
                cp = __float_as_uint(a.w);
            }
        }
        if (ANY) {
            if (__ballot_sync(gmask, hit) != 0u) {
                T.occluded = true;
                return true;
            }
            continue;
        }
        float mt = ct;
        uint32_t mp = cp;
#pragma unroll
        for (int off = G / 2; off >= 1; off >>= 1) {
            const float ot = __shfl_xor_sync(gmask, mt, off, G);
            const uint32_t op = __shfl_xor_sync(gmask, mp, off, G);
            if (ot < mt || (ot == mt && op < mp)) {
                mt = ot;
                mp = op;
            }
        }
        if (mp != 0xFFFFFFFFu && accept_hit(mt, mp, r.tmin, T.best_t, T.best_prim)) {
            const uint32_t win = (uint32_t)__ffs(__ballot_sync(gmask, cp == mp && ct == mt)) - 1u;
            T.best_t = mt;
            T.best_prim = mp;
            T.best_slot = __shfl_sync(gmask, slot, win);
            T.best_V = __shfl_sync(gmask, h.V, win);
            T.best_W = __shfl_sync(gmask, h.W, win);
            T.best_det = __shfl_sync(gmask, h.det, win);
        }
    }
    if ((T.ng.y >> 24) == 0u) {
        if (T.sp == 0) return true;
        T.ng = stack[--T.sp];
    }
    const uint32_t hb = T.ng.y >> 24;
    const uint32_t pos = 31u - __clz(hb);
    const uint32_t code = pos ^ T.oct;
    T.ng.y &= ~(1u << (24 + pos));
    const uint32_t child = T.ng.x + __popc(T.ng.y & ((1u << code) - 1u) & 0xFFu);
    if ((T.ng.y >> 24) != 0u) {
        if (T.sp < kStack) {
            if (c == 0u) stack[T.sp] = T.ng;
            T.sp++;
        } else {
            err = 1u;
        }
    }
    const uint4 *np = nodes + (size_t)child * L::VEC;
    for (int k = (int)c; k < L::VEC; k += G) nbuf[k] = __ldg(np + k);
    __syncwarp(gmask);
    const uint4 h0 = nbuf[0];
    const uint2 h1 = *reinterpret_cast<const uint2 *>(&nbuf[1]);
    const uint8_t *nb = reinterpret_cast<const uint8_t *>(nbuf);
    const uint32_t meta = nb[24 + c];
    const float qlx = (float)nb[24 + W + c], qly = (float)nb[24 + 2 * W + c], qlz = (float)nb[24 + 3 * W + c];
    const float qhx = (float)nb[24 + 4 * W + c], qhy = (float)nb[24 + 5 * W + c], qhz = (float)nb[24 + 6 * W + c];
    const uint32_t eb = h0.w;
    const float sx = __uint_as_float((eb & 0xFFu) << 23) * r.ix;
    const float sy = __uint_as_float(((eb >> 8) & 0xFFu) << 23) * r.iy;
    const float sz = __uint_as_float(((eb >> 16) & 0xFFu) << 23) * r.iz;
    const float ox = (__uint_as_float(h0.x) - r.ox) * r.ix;
    const float oy = (__uint_as_float(h0.y) - r.oy) * r.iy;
    const float oz = (__uint_as_float(h0.z) - r.oz) * r.iz;
    const float tx0 = __fmaf_rn(r.ix >= 0.0f ? qlx : qhx, sx, ox);
    const float tx1 = __fmaf_rn(r.ix >= 0.0f ? qhx : qlx, sx, ox);
    const float ty0 = __fmaf_rn(r.iy >= 0.0f ? qly : qhy, sy, oy);
    const float ty1 = __fmaf_rn(r.iy >= 0.0f ? qhy : qly, sy, oy);
    const float tz0 = __fmaf_rn(r.iz >= 0.0f ? qlz : qhz, sz, oz);
    const float tz1 = __fmaf_rn(r.iz >= 0.0f ? qhz : qlz, sz, oz);
    const float tn = fmaxf(fmaxf(tx0, ty0), fmaxf(tz0, r.tmin));
    const float tf = fminf(fminf(tx1, ty1), fminf(tz1, T.best_t * kHitSlack));
    const uint32_t mine = tn <= tf * 1.00000095f ? (meta >> 5) << (meta & 31u) : 0u;
    const uint32_t bits = __reduce_or_sync(gmask, mine);
    uint32_t m = bits >> 24;
    if (T.oct & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (T.oct & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (T.oct & 4u) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    T.ng = make_uint2(h1.x, (m << 24) | (eb >> 24));
    T.tg = make_uint2(h1.y, bits & 0x00FFFFFFu);
    __syncwarp(gmask); // every lane has read the node before the group's next one overwrites it
    return false;
}

template <int W, bool ANY>
__global__ void __launch_bounds__(128) k_intersect_warp(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                                      const float4 *__restrict__ rays, float4 *__restrict__ hits,
                                                      uint32_t *__restrict__ occluded, unsigned int *head, uint32_t n,
                                                      uint32_t *__restrict__ err) {
    constexpr int G = W;
    __shared__ WarpShared<W> sh;
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5;
    const uint32_t g = lane / G, c = lane % G;
    const uint32_t gmask = ((1u << G) - 1u) << (g * G);
    uint4 *nbuf = sh.node[wib][g];
    uint2 *stack = sh.stack[wib][g];
    bool has = false, exhausted = false;
    uint32_t ray = 0, e = 0;
    RayPre r;
    Trav T;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, c == 0u && !has); // one bit per idle group
        if (!exhausted && idle != 0u) {
            const uint32_t cnt = (uint32_t)__popc(idle);
            unsigned int base = 0;
            if (lane == 0) base = atomicAdd(head, cnt);
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + cnt >= n) exhausted = true;
            if (!has) {
                const unsigned int my = base + (unsigned int)__popc(idle & ((1u << (g * G)) - 1u));
                if (my < n) {
                    const float4 r0 = __ldg(&rays[2 * (size_t)my]);
                    const float4 r1 = __ldg(&rays[2 * (size_t)my + 1]);
                    r = ray_prep(r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r0.w);
                    trav_init(T, r, r1.w);
                    ray = my;
                    has = true;
                }
            }
        }
        if (!__any_sync(0xFFFFFFFFu, has)) {
            if (exhausted) break;
            continue;
        }
        if (has) {
            bool done = false;
            for (int it = 0; it < 4 && !done; ++it) done = warp_step<W, ANY>(T, stack, nbuf, nodes, tris, r, gmask, c, e);
            if (done) {
                if (c == 0u) {
                    if (ANY) occluded[ray] = T.occluded ? 1u : 0u;
                    else if (T.best_prim == 0xFFFFFFFFu)
                        hits[ray] = make_float4(INFINITY, __uint_as_float(0xFFFFFFFFu), 0.0f, 0.0f);
                    else
                        hits[ray] = make_float4(T.best_t, __uint_as_float(T.best_prim), T.best_V / T.best_det,
                                                T.best_W / T.best_det);
                }
                has = false;
            }
        }
    }
    if (e) atomicOr(err, e);
}

// Any-hit queries use the refill kernel (threshold 4 idle lanes): on the
// 1M-triangle soup with 16M shadow rays it measured 1862 against 1364 Mrays/s
// for one thread per ray.  Closest-hit queries stay one thread per ray (813
// against 781 Mrays/s).
constexpr uint32_t kAnyRefill = 4;

template <int W>
void launch_warp(const crg_scene *s, const crg_ray *rays, crg_hit *hits, uint32_t *occluded, uint64_t n, bool any,
                 cudaStream_t st) {
    int per_sm = 0;
    if (any) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_intersect_warp<W, true>, 128, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_intersect_warp<W, false>, 128, 0);
    const uint32_t grid = (uint32_t)(std::max(s->ctx->sm_count, 1) * std::max(per_sm, 1));
    unsigned int *head = (unsigned int *)s->qhead.ptr;
    cudaMemsetAsync(head, 0, sizeof(unsigned int), st);
    const uint4 *nd = (const uint4 *)s->wide.ptr;
    const float4 *tr = (const float4 *)s->tris.ptr;
    if (any)
        k_intersect_warp<W, true><<<grid, 128, 0, st>>>(nd, tr, (const float4 *)rays, nullptr, occluded, head, (uint32_t)n,
                                                       (uint32_t *)s->err.ptr);
    else
        k_intersect_warp<W, false><<<grid, 128, 0, st>>>(nd, tr, (const float4 *)rays, (float4 *)hits, nullptr, head,
                                                        (uint32_t)n, (uint32_t *)s->err.ptr);
}

template <int W>
void launch_w(const crg_scene *s, const crg_ray *rays, crg_hit *hits, uint32_t *occluded, uint32_t *nodes, uint32_t *tris,
              uint64_t n, bool any, cudaStream_t st) {
    if (s->ninst && s->ntri > 0) {
        const rc::SceneDev S = rc::scene_dev(s);
        const uint64_t blocks = (n + 127) / 128;
        if (any) k_intersect_inst<W, true><<<blocks, 128, 0, st>>>(S, (const float4 *)rays, nullptr, occluded, n);
        else k_intersect_inst<W, false><<<blocks, 128, 0, st>>>(S, (const float4 *)rays, (float4 *)hits, nullptr, n);
        if (nodes) cudaMemsetAsync(nodes, 0, 4 * n, st);
        if (tris) cudaMemsetAsync(tris, 0, 4 * n, st);
        return;
    }
    if (any && n >= (1u << 16) && n < 0xFFFF0000ull && s->ntri > 0) {
        int per_sm = 0;
        if (any) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_intersect_dyn<W, true>, 128, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_intersect_dyn<W, false>, 128, 0);
        const uint32_t grid = (uint32_t)(std::max(s->ctx->sm_count, 1) * std::max(per_sm, 1));
        unsigned int *head = (unsigned int *)s->qhead.ptr;
        cudaMemsetAsync(head, 0, sizeof(unsigned int), st);
        const uint4 *nd = (const uint4 *)s->wide.ptr;
        const float4 *tr = (const float4 *)s->tris.ptr;
        if (any)
            k_intersect_dyn<W, true><<<grid, 128, 0, st>>>(nd, tr, (const float4 *)rays, nullptr, occluded, head,
                                                           (uint32_t)n, kAnyRefill, (uint32_t *)s->err.ptr);
        else
            k_intersect_dyn<W, false><<<grid, 128, 0, st>>>(nd, tr, (const float4 *)rays, (float4 *)hits, nullptr, head,
                                                            (uint32_t)n, kAnyRefill, (uint32_t *)s->err.ptr);
        return;
    }
    const uint32_t T = 128;
    const uint64_t blocks = (n + T - 1) / T;
    const uint4 *nd = (const uint4 *)s->wide.ptr;
    const float4 *tr = (const float4 *)s->tris.ptr;
    uint32_t *err = (uint32_t *)s->err.ptr;
    const bool count = nodes || tris;
    if (any)
        k_intersect<W, true, false><<<blocks, T, 0, st>>>(nd, tr, (const float4 *)rays, nullptr, occluded, nullptr, nullptr, n,
                                                           s->ntri, err);
    else if (count)
        k_intersect<W, false, true><<<blocks, T, 0, st>>>(nd, tr, (const float4 *)rays, (float4 *)hits, nullptr, nodes, tris, n,
                                                           s->ntri, err);
    else
        k_intersect<W, false, false><<<blocks, T, 0, st>>>(nd, tr, (const float4 *)rays, (float4 *)hits, nullptr, nullptr,
                                                            nullptr, n, s->ntri, err);
}

} // namespace

crg_status launch_intersect(const crg_scene *s, const crg_ray *rays, crg_hit *hits, uint32_t *occluded, uint32_t *nodes,
                            uint32_t *tris, uint64_t n, bool any, cudaStream_t st, int traversal) {
    if (n == 0) return CRG_OK;
    if (traversal == CRG_TRAVERSAL_WARP && s->ninst == 0 && s->ntri > 0 && !nodes && !tris) {
        if (n >= 0xFFFF0000ull) return set_error(s->ctx, CRG_ERR_INVALID_ARG, "warp traversal: at most 2^32 - 2^16 rays per call");
        switch (s->width) {
        case 2: launch_warp<2>(s, rays, hits, occluded, n, any, st); break;
        case 4: launch_warp<4>(s, rays, hits, occluded, n, any, st); break;
        default: launch_warp<8>(s, rays, hits, occluded, n, any, st); break;
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_error(s->ctx, e, "k_intersect_warp launch");
        return CRG_OK;
    }
    switch (s->width) {
    case 2: launch_w<2>(s, rays, hits, occluded, nodes, tris, n, any, st); break;
    case 4: launch_w<4>(s, rays, hits, occluded, nodes, tris, n, any, st); break;
    default: launch_w<8>(s, rays, hits, occluded, nodes, tris, n, any, st); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(s->ctx, e, "k_intersect launch");
    return CRG_OK;
}

} // namespace crg
