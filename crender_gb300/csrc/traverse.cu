// traverse.cu — batched closest-hit / any-hit queries (the rtcIntersect1 /
// rtcOccluded1 replacements, CRender src/objects/model.cpp:5-49).
//
// Persistent blocks pull rays from their own range; rays are two 16-byte
// loads, hits one 16-byte store.
// The wide nodes are read with 16-byte vector loads through the read-only
// path; per-thread group stack of 64 entries (overflow raises the scene's
// error word instead of trapping).
#include <algorithm>

#include "crg_dev.cuh"
#include "crg_internal.h"

namespace crg {
namespace {

// Persistent blocks with dynamic fetch: each block owns a contiguous range of
// rays; its warps take kBatch indices at a time from a shared-memory counter
// and refill idle lanes between bounded traversal slices, so lanes whose rays
// finish early get new rays instead of idling until the warp's longest ray
// ends.  No global state: concurrent launches on one scene do not interact.
constexpr uint32_t kBatch = 64;
constexpr int kSlice = 4; // traversal iterations between refills

template <int W, bool ANY, bool COUNT>
__global__ void __launch_bounds__(256) k_intersect(const uint4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                                   const float4 *__restrict__ rays, float4 *__restrict__ hits,
                                                   uint32_t *__restrict__ occluded, uint32_t *__restrict__ ncount,
                                                   uint32_t *__restrict__ tcount, uint64_t n, uint32_t ntri,
                                                   uint32_t *__restrict__ err) {
    __shared__ unsigned long long blk_next;
    const uint64_t per_block = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t blk_begin = (uint64_t)blockIdx.x * per_block;
    const uint64_t blk_end = blk_begin + per_block < n ? blk_begin + per_block : n;
    if (threadIdx.x == 0) blk_next = blk_begin;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt = (1u << lane) - 1u;
    bool active = false;
    uint64_t idx = 0;
    RayPre r;
    Trav T;
    uint2 stack[kStack];
    TravStats st{0, 0};
    uint32_t e = 0;
    uint64_t pool = 0, pool_end = 0; // warp-uniform
    bool exhausted = false;         // warp-uniform
    for (;;) {
        const uint32_t need = __ballot_sync(0xFFFFFFFFu, !active);
        if (need && !(exhausted && pool >= pool_end)) {
            if (pool >= pool_end) {
                unsigned long long b = 0;
                if (lane == 0) b = atomicAdd(&blk_next, (unsigned long long)kBatch);
                b = __shfl_sync(0xFFFFFFFFu, b, 0);
                pool = b;
                pool_end = b + kBatch < blk_end ? b + kBatch : blk_end;
                if (b + kBatch >= blk_end) exhausted = true;
            }
            const uint64_t avail = pool < pool_end ? pool_end - pool : 0;
            const uint32_t rank = __popc(need & lt);
            if (!active && rank < avail) {
                idx = pool + rank;
                const float4 r0 = __ldg(&rays[2 * idx]);
                const float4 r1 = __ldg(&rays[2 * idx + 1]);
                r = ray_prep(r0.x, r0.y, r0.z, r1.x, r1.y, r1.z, r0.w);
                trav_init(T, r, r1.w);
                st = TravStats{0, 0};
                active = true;
                if (ntri == 0) T.ng.y = 0u; // empty scene: nothing to visit
            }
            const uint64_t taken = __popc(need) < avail ? __popc(need) : avail;
            pool += taken;
        }
        if (__ballot_sync(0xFFFFFFFFu, active) == 0u) {
            if (exhausted && pool >= pool_end) break;
            continue;
        }
        if (active && trav_step<W, ANY, COUNT>(T, stack, nodes, tris, r, kSlice, st, e)) {
            if (ANY) {
                occluded[idx] = T.occluded ? 1u : 0u;
            } else if (T.best_prim == 0xFFFFFFFFu) {
                hits[idx] = make_float4(INFINITY, __uint_as_float(0xFFFFFFFFu), 0.0f, 0.0f);
            } else {
                hits[idx] = make_float4(T.best_t, __uint_as_float(T.best_prim), T.best_V / T.best_det, T.best_W / T.best_det);
            }
            if (COUNT) {
                if (ncount) ncount[idx] = st.nodes;
                if (tcount) tcount[idx] = st.tris;
            }
            active = false;
        }
    }
    if (e) atomicOr(err, e);
}

template <int W>
void launch_w(const crg_scene *s, const crg_ray *rays, crg_hit *hits, uint32_t *occluded, uint32_t *nodes, uint32_t *tris,
              uint64_t n, bool any, cudaStream_t st) {
    const uint32_t T = 256;
    // persistent grid: enough resident warps to fill every SM, never more blocks than work
    const uint64_t want = (uint64_t)(s->ctx->sm_count > 0 ? s->ctx->sm_count : 152) * 4;
    const uint64_t blocks = std::min<uint64_t>(want, (n + T - 1) / T);
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
                            uint32_t *tris, uint64_t n, bool any, cudaStream_t st) {
    if (n == 0) return CRG_OK;
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
