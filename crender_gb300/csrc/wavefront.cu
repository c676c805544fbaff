// wavefront.cu — batched wavefront path tracer (sm_103a).
//
// Many views (cameras over one or more scenes, each with its own resolution
// and spp) are rendered in one CUDA-graph launch.  Paths live in a pool of P
// slots (structure of arrays in HBM) and move through queues:
//
//   extend   closest hit for every path in the input queue
//   shade    one bounce of the shared shading code (render_common.cuh): a path
//            that continues goes to the output queue, an NEE shadow request
//            to the shadow queue; a finished path writes its sample and the
//            slot immediately takes the next sample of the batch
//   shadow   the shadow tests; a visible contribution is added to the path
//   control  swaps the queues, detects a drained chunk, and sets the graph's
//            WHILE condition (bounded by an iteration cap that raises
//            CRG_ERR_TIMEOUT instead of looping forever)
//   resolve  adds a drained chunk's per-sample radiance to the films in sample
//            order, so films are bit-identical to the megakernel's
//   generate seeds the pool with the next chunk's first samples
//
// A new sample stores only its meta word: extend and shade derive its camera
// ray, throughput and radiance.  The traversal stages refill idle lanes ray
// by ray and trace a ray through a scene's placements themselves.
//
// extend / shade / shadow are persistent kernels: a fixed grid whose warps
// take `fetch` queue entries at a time with one atomic.  The order in which L
// receives contributions (emission of bounce i, then NEE of bounce i, then
// bounce i + 1) is the megakernel's, because the shadow kernel of bounce i
// runs before the shade kernel of bounce i + 1.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "render_common.cuh"

namespace crg {
using namespace rc;
namespace {

struct ViewDev {
    CamDev cam;
    crg_settings set;
    uint32_t scene;
    uint32_t npix;
    uint64_t spp0; // film sample count before this batch (sample index offset)
    float *sum;
    double *sum64, *sumsq64;
};

struct Segment {            // samples [s0, s1) of one view, contiguous in gid order
    unsigned long long gid; // first gid of the segment
    uint32_t view, s0, s1;
    uint32_t pix_base;      // prefix of npix over the chunk's segments (resolve work index)
};

struct Chunk {
    unsigned long long gid_begin, gid_end;
    uint32_t seg_begin, seg_end;
    uint32_t resolve_items; // sum of npix over the chunk's segments
    uint32_t pad_;
};

struct Ctrl {
    unsigned int in_count, out_count, sh_count;
    unsigned int head_ext, head_shade, head_sh;
    unsigned int parity;
    unsigned int chunk;          // chunk being rendered
    unsigned int resolve_chunk;  // chunk to resolve this iteration, or ~0u
    unsigned int generate;       // 1: seed the pool with `chunk`
    unsigned int done;
    unsigned int error;
    unsigned int iterations, max_iterations;
    unsigned long long issued;   // next gid to issue in `chunk`
    unsigned long long segments, shadow;
    unsigned long long nodes, tris; // traversal work (instrumented variant only): closest hits
    unsigned long long nodes_sh, tris_sh; // the same for the shadow tests (split and shade+shadow stages)
};

constexpr uint32_t kFinish = 1u << 31;    // meta.x flag: finish after the shadow test
constexpr uint32_t kPrevDelta = 1u << 30; // meta.x flag: previous bounce was a delta lobe
constexpr uint32_t kFresh = 1u << 29;     // meta.x flag: a new sample whose camera ray, throughput and
                                          // radiance are not stored (derived from view, pixel and sample)

struct Wf {
    Ctrl *ctrl;
    const SceneDev *scenes;
    const ViewDev *views;
    const Segment *segs;
    const Chunk *chunks;
    uint32_t nchunks, P, fetch;
    uint32_t refill;       // extend: 0 = static fetch of `fetch` entries, else the per-lane refill threshold
    uint32_t refill_sh;    // shadow: the same (0 when a batch can produce sun requests)
    uint32_t placed;       // placements in the batch: 0 none, 1 at most kLoopPlacements per scene, 2 more
    uint32_t pad_[2];
    float4 *o, *d, *T, *L; // T.w = prev_pdf
    uint4 *meta;           // x: view | depth << 16 | flags; y: pixel; z: sample; w: offset in the chunk
    float4 *hit;           // t, prim bits, triangle slot bits, found
    float4 *sh_o, *sh_d, *sh_c;
    uint32_t *qa, *qb, *qsh;
    float4 *slots;         // radiance per sample of the current chunk
};

// hit.w of a path slot: 0 = miss, 1 = hit on the plain mesh, 2 + j = hit on instance j.
__device__ __forceinline__ float pack_found(bool found, uint32_t inst) {
    return __uint_as_float(found ? (inst == kNoInst ? 1u : inst + 2u) : 0u);
}

__device__ __forceinline__ uint32_t *q_in(const Wf &w, const Ctrl &c) { return c.parity ? w.qb : w.qa; }
__device__ __forceinline__ uint32_t *q_out(const Wf &w, const Ctrl &c) { return c.parity ? w.qa : w.qb; }

// Warp-cooperative fetch of `fetch` entries; returns the first index (all
// lanes of the active mask agree).
__device__ __forceinline__ unsigned int warp_fetch(unsigned int *head, uint32_t fetch) {
    unsigned int b = 0;
    if ((threadIdx.x & 31) == 0) b = atomicAdd(head, fetch);
    return __shfl_sync(0xFFFFFFFFu, b, 0);
}

// Warp-aggregated append of flagged lanes to a queue.
__device__ __forceinline__ void warp_push(bool want, uint32_t value, uint32_t *queue, unsigned int *count) {
    const uint32_t active = __activemask();
    const uint32_t m = __ballot_sync(active, want);
    if (!m) return;
    const uint32_t lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    unsigned int base = 0;
    if ((int)lane == leader) base = atomicAdd(count, (unsigned int)__popc(m));
    base = __shfl_sync(active, base, leader);
    if (want) queue[base + __popc(m & ((1u << lane) - 1u))] = value;
}

// The camera ray of `sample` at pixel `pix` of view V, exactly as the
// megakernel starts a sample.
__device__ __forceinline__ void sample_ray(const ViewDev &V, uint32_t pix, uint32_t sample, v3 &o, v3 &d) {
    const uint32_t Wd = V.set.width, Hd = V.set.height;
    const uint32_t px = pix % Wd, py = pix / Wd;
    const f4 g0 = rand4(pix, sample, 0, V.set.seed);
    const float x = ((float)px + g0.x) / (float)Wd;
    const float y = ((float)py + g0.y) / (float)Hd;
    camera_ray(V.cam, x, y, V.set.aspect, o, d);
}

// The ray a path traces next: a new sample's camera ray (recomputed), else
// the stored one.
__device__ __forceinline__ void path_ray(const Wf &w, uint32_t slot, const uint4 &m, float4 &o, float4 &d) {
    if (m.x & kFresh) {
        v3 a, b;
        sample_ray(w.views[m.x & 0xFFFFu], m.y, m.z, a, b);
        o = make_float4(a.x, a.y, a.z, 0.0f);
        d = make_float4(b.x, b.y, b.z, 0.0f);
    } else {
        o = w.o[slot];
        d = w.d[slot];
    }
}

// Starts sample `gid` of the batch in path slot `slot`: only its meta word is
// written (kFresh: camera ray, unit throughput and zero radiance are implied;
// extend and shade derive them).
__device__ void start_sample(const Wf &w, uint32_t slot, unsigned long long gid, const Chunk &ch) {
    uint32_t lo = ch.seg_begin, hi = ch.seg_end - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (w.segs[mid].gid <= gid) lo = mid;
        else hi = mid - 1;
    }
    const Segment sg = w.segs[lo];
    const ViewDev &V = w.views[sg.view];
    const unsigned long long rel = gid - sg.gid;
    const uint32_t s = sg.s0 + (uint32_t)(rel / V.npix);
    const uint32_t pix = (uint32_t)(rel % V.npix);
    const uint32_t sample = (uint32_t)(V.spp0 + s);
    w.meta[slot] = make_uint4(sg.view | kPrevDelta | kFresh, pix, sample, (uint32_t)(gid - ch.gid_begin));
}

// Writes a finished sample and, if the chunk has more, starts the next one
// in the same slot (pushed to the output queue).
__device__ __forceinline__ void finish_and_refill(const Wf &w, Ctrl *c, bool finishing, uint32_t slot, float4 Lv,
                                                  uint32_t off) {
    if (finishing) w.slots[off] = Lv;
    const uint32_t active = __activemask();
    const uint32_t m = __ballot_sync(active, finishing);
    bool refill = false;
    unsigned long long gid = 0;
    const Chunk ch = w.chunks[c->chunk];
    if (m) {
        const uint32_t lane = threadIdx.x & 31;
        const int leader = __ffs(m) - 1;
        unsigned long long base = 0;
        if ((int)lane == leader) base = atomicAdd(&c->issued, (unsigned long long)__popc(m));
        base = __shfl_sync(active, base, leader);
        gid = base + __popc(m & ((1u << lane) - 1u));
        refill = finishing && gid < ch.gid_end;
    }
    if (refill) start_sample(w, slot, gid, ch);
    warp_push(refill, slot, q_out(w, *c), &c->out_count);
}

template <int W, bool CNT, bool INST>
__global__ void __launch_bounds__(256) k_wf_extend(Wf w) {
    unsigned long long nodes = 0, tris = 0;
    Ctrl *c = w.ctrl;
    const unsigned int n = c->in_count;
    const uint32_t *in = q_in(w, *c);
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        const unsigned int base = warp_fetch(&c->head_ext, w.fetch);
        if (base >= n) break;
        for (uint32_t k = lane; k < w.fetch; k += 32) {
            const unsigned int qi = base + k;
            if (qi >= n) break;
            const uint32_t slot = in[qi];
            const uint4 m = w.meta[slot];
            const SceneDev &S = w.scenes[w.views[m.x & 0xFFFFu].scene];
            float4 o, d;
            path_ray(w, slot, m, o, d);
            PathCtx C{0, 0, 0, 0, 0, 0, 0ull, 0ull};
            Hit h;
            const bool found = closest<W, CNT, INST>(S, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), INFINITY, h, C);
            w.hit[slot] = make_float4(h.t, __uint_as_float(h.prim), __uint_as_float(h.slot), pack_found(found, h.inst));
            if (C.err) atomicOr(&c->error, 1u);
            if (CNT) {
                nodes += C.nodes;
                tris += C.tris;
            }
        }
    }
    if (CNT) {
        atomicAdd(&c->nodes, nodes);
        atomicAdd(&c->tris, tris);
    }
}

// Warp-aggregated count of flagged lanes (shadow rays traced inside a fused shade kernel).
__device__ __forceinline__ void warp_count(bool want, unsigned int *count) {
    const uint32_t active = __activemask();
    const uint32_t m = __ballot_sync(active, want);
    if (m && (threadIdx.x & 31) == (uint32_t)(__ffs(m) - 1)) atomicAdd(count, (unsigned int)__popc(m));
}

// FUSE 0: shade only (hits from k_wf_extend, shadow rays to the shadow queue)
// FUSE 1: shade + the NEE shadow test in the same thread (no shadow queue)
// FUSE 2: closest hit + shade + shadow test (one kernel per bounce)
// Contributions reach L in the same order in every form: emission of bounce
// i, its NEE, then bounce i + 1.
template <int W, int FUSE, bool CNT, bool INST>
__global__ void __launch_bounds__(256, FUSE == 0 ? 3 : 2) k_wf_shade(Wf w) {
    unsigned long long nodes = 0, tris = 0;
    Ctrl *c = w.ctrl;
    const unsigned int n = c->in_count;
    const uint32_t *in = q_in(w, *c);
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        const unsigned int base = warp_fetch(&c->head_shade, w.fetch);
        if (base >= n) break;
        for (uint32_t k0 = 0; k0 < w.fetch; k0 += 32) {
            if (base + k0 >= n) break;
            const unsigned int qi = base + k0 + lane;
            const bool valid = qi < n && k0 + lane < w.fetch;
            uint32_t slot = 0;
            bool cont = false, finishing = false, shadow = false;
            float4 Lv = make_float4(0, 0, 0, 0);
            uint32_t off = 0;
            if (valid) {
                slot = in[qi];
                uint4 m = w.meta[slot];
                const uint32_t view = m.x & 0xFFFFu, depth = (m.x >> 16) & 0x3FFu;
                const ViewDev &V = w.views[view];
                const SceneDev &S = w.scenes[V.scene];
                float4 o, d, T, L;
                path_ray(w, slot, m, o, d);
                if (m.x & kFresh) {
                    T = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
                    L = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                } else {
                    T = w.T[slot];
                    L = w.L[slot];
                }
                PathCtx C{m.y, m.z, V.set.seed, 0, 0, 0, 0ull, 0ull};
                float4 h4;
                if (FUSE >= 2) {
                    Hit hh;
                    const bool f = closest<W, CNT, INST>(S, mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), INFINITY, hh, C);
                    h4 = make_float4(hh.t, __uint_as_float(hh.prim), __uint_as_float(hh.slot), pack_found(f, hh.inst));
                } else {
                    h4 = w.hit[slot];
                }
                PathState ps;
                ps.o = mk(o.x, o.y, o.z);
                ps.d = mk(d.x, d.y, d.z);
                ps.T = mk(T.x, T.y, T.z);
                ps.L = mk(L.x, L.y, L.z);
                ps.prev_pdf = T.w;
                ps.prev_delta = (m.x & kPrevDelta) ? 1u : 0u;
                Hit h;
                h.t = h4.x;
                h.prim = __float_as_uint(h4.y);
                h.slot = __float_as_uint(h4.z);
                h.u = h.v = 0.0f;
                const uint32_t fw = __float_as_uint(h4.w);
                h.inst = fw >= 2u ? fw - 2u : kNoInst;
                Aov aov;
                NeeReq nr;
                nr.kind = 0;
                if (depth >= V.set.max_bounces) {
                    cont = false; // max_bounces == 0: the megakernel traces nothing for this sample
                } else {
                    cont = V.set.mode == CRG_MODE_EXTENDED
                               ? shade_extended(S, V.set, C, depth, ps, fw != 0u, h, aov, nr)
                               : shade_faithful(S, V.set, C, depth, ps, fw != 0u, h, aov, nr);
                }
                if (cont && depth + 1 >= V.set.max_bounces) cont = false;
                shadow = nr.kind != 0;
                if (FUSE >= 1 && shadow && shadow_visible<W, CNT, INST>(S, nr, C)) ps.L = add(ps.L, nr.c);
                if (C.err) atomicOr(&c->error, 1u);
                if (CNT) {
                    nodes += C.nodes;
                    tris += C.tris;
                }
                Lv = make_float4(ps.L.x, ps.L.y, ps.L.z, 0.0f);
                off = m.w;
                finishing = !cont && (FUSE >= 1 || !shadow);
                if (FUSE == 0 && shadow) {
                    w.sh_o[slot] = make_float4(nr.o.x, nr.o.y, nr.o.z, nr.tmax);
                    w.sh_d[slot] = make_float4(nr.d.x, nr.d.y, nr.d.z, __uint_as_float(nr.kind));
                    w.sh_c[slot] = make_float4(nr.c.x, nr.c.y, nr.c.z, 0.0f);
                }
                uint32_t mx_ = (m.x & 0xFFFFu) | ((depth + 1) << 16) | (ps.prev_delta ? kPrevDelta : 0u);
                if (FUSE == 0 && !cont && shadow) mx_ |= kFinish;
                m.x = mx_;
                if (!finishing) { // a finishing path's radiance goes to its sample slot; its state is dead
                    w.L[slot] = Lv;
                    w.meta[slot] = m;
                }
                if (cont) {
                    w.o[slot] = make_float4(ps.o.x, ps.o.y, ps.o.z, 0.0f);
                    w.d[slot] = make_float4(ps.d.x, ps.d.y, ps.d.z, 0.0f);
                    w.T[slot] = make_float4(ps.T.x, ps.T.y, ps.T.z, ps.prev_pdf);
                }
            }
            if (FUSE == 0) warp_push(valid && shadow, slot, w.qsh, &c->sh_count);
            else warp_count(valid && shadow, &c->sh_count);
            warp_push(valid && cont, slot, q_out(w, *c), &c->out_count);
            finish_and_refill(w, c, valid && finishing, slot, Lv, off);
        }
    }
    if (CNT && FUSE >= 1) { // FUSE 1: the shadow test's work; FUSE 2: closest hit and shadow test together
        atomicAdd(FUSE == 1 ? &c->nodes_sh : &c->nodes, nodes);
        atomicAdd(FUSE == 1 ? &c->tris_sh : &c->tris, tris);
    }
}

template <int W, bool CNT, bool INST>
__global__ void __launch_bounds__(256) k_wf_shadow(Wf w) {
    unsigned long long nodes = 0, tris = 0;
    Ctrl *c = w.ctrl;
    const unsigned int n = c->sh_count;
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        const unsigned int base = warp_fetch(&c->head_sh, w.fetch);
        if (base >= n) break;
        for (uint32_t k0 = 0; k0 < w.fetch; k0 += 32) {
            if (base + k0 >= n) break;
            const unsigned int qi = base + k0 + lane;
            const bool valid = qi < n && k0 + lane < w.fetch;
            uint32_t slot = 0, off = 0;
            bool finishing = false;
            float4 Lv = make_float4(0, 0, 0, 0);
            if (valid) {
                slot = w.qsh[qi];
                uint4 m = w.meta[slot];
                const ViewDev &V = w.views[m.x & 0xFFFFu];
                const SceneDev &S = w.scenes[V.scene];
                const float4 so = w.sh_o[slot], sd = w.sh_d[slot], sc = w.sh_c[slot];
                NeeReq nr;
                nr.o = mk(so.x, so.y, so.z);
                nr.d = mk(sd.x, sd.y, sd.z);
                nr.c = mk(sc.x, sc.y, sc.z);
                nr.tmax = so.w;
                nr.kind = __float_as_uint(sd.w);
                PathCtx C{0, 0, 0, 0, 0, 0, 0ull, 0ull};
                Lv = w.L[slot];
                if (shadow_visible<W, CNT, INST>(S, nr, C)) {
                    const v3 L = add(mk(Lv.x, Lv.y, Lv.z), nr.c);
                    Lv = make_float4(L.x, L.y, L.z, 0.0f);
                    w.L[slot] = Lv;
                }
                if (C.err) atomicOr(&c->error, 1u);
                if (CNT) {
                    nodes += C.nodes;
                    tris += C.tris;
                }
                finishing = (m.x & kFinish) != 0u;
                off = m.w;
            }
            finish_and_refill(w, c, valid && finishing, slot, Lv, off);
        }
    }
    if (CNT) {
        atomicAdd(&c->nodes_sh, nodes);
        atomicAdd(&c->tris_sh, tris);
    }
}

// Extend with per-lane ray refill (dyn_traverse): the same hits as k_wf_extend.
// PL: the scenes' placements.  0: none (one mesh per scene).  1: at most
// kLoopPlacements per scene, traced one after the other as
// closest_placement_loop does.  2: placements through the top-level tree, as
// closest_placements does (the walk is resumed between placements).  Each
// placement is a traversal of its own that the lane resumes between refill
// checks; the lane keeps the world ray, the walk and the best hit so far.  A
// ray that reaches no placement box runs one empty traversal (tmax below
// tmin) so that every query passes through done.
template <int W, bool CNT, int PL>
__global__ void __launch_bounds__(256, 5) k_wf_extend_dyn(Wf w) {
    Ctrl *c = w.ctrl;
    const unsigned int n = c->in_count;
    const uint32_t *in = q_in(w, *c);
    TravStats st{0, 0};
    uint32_t err = 0;
    // per-lane state of a ray through placements
    const SceneDev *Sp = nullptr;
    v3 wo = mk(0.0f, 0.0f, 0.0f), wd = wo, oo = wo, od = wo;
    float dl = 0.0f, best = INFINITY, bt = 0.0f;
    uint32_t k = 0, bprim = 0xFFFFFFFFu, bslot = 0u, binst = kNoInst;
    TlasRay tr;
    TlasWalk wk;
    // sets up placement k's traversal under the current best world distance
    auto place = [&](RayPre &r, float &tmax, uint32_t &root) {
        float len;
        inst_ray(*Sp, k, wo, wd, oo, od, len);
        tmax = best < INFINITY ? ((best * len) / dl) * kInstSlack : INFINITY;
        r = ray_prep(oo.x, oo.y, oo.z, od.x, od.y, od.z, 1e-5f);
        root = __ldg(&Sp->inst_root[k]);
    };
    dyn_traverse<W, false, CNT, 8>(
        &c->head_ext, n, w.refill,
        [&](unsigned int qi, uint32_t &slot, RayPre &r, float &tmax, uint32_t &root, const uint4 *&nodes,
            const float4 *&tris) {
            slot = in[qi];
            const uint4 m = w.meta[slot];
            const SceneDev &S = w.scenes[w.views[m.x & 0xFFFFu].scene];
            nodes = S.nodes;
            tris = S.tris;
            float4 o, d;
            path_ray(w, slot, m, o, d);
            tmax = INFINITY;
            root = 0u;
            if (PL) Sp = &S;
            if (PL == 0 || S.ninst == 0) {
                r = ray_prep(o.x, o.y, o.z, d.x, d.y, d.z, 1e-5f);
                return true;
            }
            wo = mk(o.x, o.y, o.z);
            wd = mk(d.x, d.y, d.z);
            dl = sqrtf(dot(wd, wd));
            best = INFINITY;
            bprim = 0xFFFFFFFFu;
            binst = kNoInst;
            if (PL == 2) {
                tr = tlas_ray(wo, wd, 1e-5f);
                tlas_begin(S, wk);
                k = tlas_next(S, tr, best, wk);
                if (k == kNoInst) { // no placement box on the ray: one empty traversal
                    r = ray_prep(wo.x, wo.y, wo.z, wd.x, wd.y, wd.z, 1e-5f);
                    tmax = -1.0f;
                    root = __ldg(&S.inst_root[0]);
                    return true;
                }
            } else {
                k = 0;
            }
            place(r, tmax, root);
            return true;
        },
        [&](uint32_t, const Trav &T, RayPre &r, float &tmax, uint32_t &root) {
            if (PL == 0 || Sp->ninst == 0 || k == kNoInst) return false;
            if (T.best_prim != 0xFFFFFFFFu) {
                const float dist = vdist(inst_point(*Sp, k, oo, od, T.best_t), wo);
                if (dist < best || (PL == 2 && dist == best && binst != kNoInst && k < binst)) {
                    best = dist;
                    bt = T.best_t;
                    bprim = T.best_prim;
                    bslot = T.best_slot;
                    binst = k;
                }
            }
            if (PL == 2) {
                k = tlas_next(*Sp, tr, best, wk);
                if (k == kNoInst) return false;
            } else if (++k >= Sp->ninst) {
                return false;
            }
            place(r, tmax, root);
            return true;
        },
        [&](uint32_t slot, const Trav &T) {
            if (PL != 0 && Sp->ninst != 0) {
                if (PL == 2 && !wk.ok) err = 1u;
                w.hit[slot] = make_float4(bt, __uint_as_float(bprim), __uint_as_float(bslot),
                                          pack_found(bprim != 0xFFFFFFFFu, binst));
                return;
            }
            const bool found = T.best_prim != 0xFFFFFFFFu;
            w.hit[slot] = make_float4(T.best_t, __uint_as_float(T.best_prim), __uint_as_float(T.best_slot),
                                      pack_found(found, kNoInst));
        },
        st, err);
    if (err) atomicOr(&c->error, 1u);
    if (CNT) {
        atomicAdd(&c->nodes, (unsigned long long)st.nodes);
        atomicAdd(&c->tris, (unsigned long long)st.tris);
    }
}

// Shadow tests with per-lane ray refill, for batches whose shadow requests
// are all emitter tests (any hit below tmax); sun requests (faithful
// estimator with the sun on) go through k_wf_shadow.  PL: as k_wf_extend_dyn
// (occluded_placement_loop, occluded_placements), stopping at the first
// placement that occludes.
template <int W, bool CNT, int PL>
__global__ void __launch_bounds__(256, 5) k_wf_shadow_dyn(Wf w) {
    Ctrl *c = w.ctrl;
    const unsigned int n = c->sh_count;
    TravStats st{0, 0};
    uint32_t err = 0;
    const SceneDev *Sp = nullptr;
    v3 wo = mk(0.0f, 0.0f, 0.0f), wd = wo;
    float dl = 0.0f, tw = 0.0f;
    uint32_t k = 0;
    TlasRay tr;
    TlasWalk wk;
    auto place = [&](RayPre &r, float &tmax, uint32_t &root) {
        v3 oo, od;
        float len;
        inst_ray(*Sp, k, wo, wd, oo, od, len);
        r = ray_prep(oo.x, oo.y, oo.z, od.x, od.y, od.z, 1e-5f);
        tmax = (tw * len) / dl;
        root = __ldg(&Sp->inst_root[k]);
    };
    dyn_traverse<W, true, CNT, 8>(
        &c->head_sh, n, w.refill_sh,
        [&](unsigned int qi, uint32_t &slot, RayPre &r, float &tmax, uint32_t &root, const uint4 *&nodes,
            const float4 *&tris) {
            slot = w.qsh[qi];
            const SceneDev &S = w.scenes[w.views[w.meta[slot].x & 0xFFFFu].scene];
            const float4 so = w.sh_o[slot], sd = w.sh_d[slot];
            nodes = S.nodes;
            tris = S.tris;
            root = 0u;
            if (PL) Sp = &S;
            if (PL == 0 || S.ninst == 0) {
                r = ray_prep(so.x, so.y, so.z, sd.x, sd.y, sd.z, 1e-5f);
                tmax = so.w;
                return true;
            }
            wo = mk(so.x, so.y, so.z);
            wd = mk(sd.x, sd.y, sd.z);
            dl = sqrtf(dot(wd, wd));
            tw = so.w;
            if (PL == 2) {
                tr = tlas_ray(wo, wd, 1e-5f);
                dl = tr.dl;
                tlas_begin(S, wk);
                k = tlas_next(S, tr, tw, wk);
                if (k == kNoInst) { // no placement box on the ray: one empty traversal
                    r = ray_prep(wo.x, wo.y, wo.z, wd.x, wd.y, wd.z, 1e-5f);
                    tmax = -1.0f;
                    root = __ldg(&S.inst_root[0]);
                    return true;
                }
            } else {
                k = 0;
            }
            place(r, tmax, root);
            return true;
        },
        [&](uint32_t, const Trav &T, RayPre &r, float &tmax, uint32_t &root) {
            if (PL == 0 || Sp->ninst == 0 || k == kNoInst || T.occluded) return false;
            if (PL == 2) {
                k = tlas_next(*Sp, tr, tw, wk);
                if (k == kNoInst) return false;
            } else if (++k >= Sp->ninst) {
                return false;
            }
            place(r, tmax, root);
            return true;
        },
        [&](uint32_t slot, const Trav &T) {
            if (PL == 2 && Sp->ninst != 0 && !wk.ok) err = 1u;
            const uint4 m = w.meta[slot];
            float4 Lv = w.L[slot];
            if (!T.occluded) {
                const float4 sc = w.sh_c[slot];
                const v3 L = add(mk(Lv.x, Lv.y, Lv.z), mk(sc.x, sc.y, sc.z));
                Lv = make_float4(L.x, L.y, L.z, 0.0f);
                w.L[slot] = Lv;
            }
            finish_and_refill(w, c, (m.x & kFinish) != 0u, slot, Lv, m.w);
        },
        st, err);
    if (err) atomicOr(&c->error, 1u);
    if (CNT) {
        atomicAdd(&c->nodes_sh, (unsigned long long)st.nodes);
        atomicAdd(&c->tris_sh, (unsigned long long)st.tris);
    }
}

__global__ void k_wf_control(Wf w, cudaGraphConditionalHandle handle, int in_graph) {
    if (threadIdx.x != 0) return;
    Ctrl *c = w.ctrl;
    if (c->done) { // iterations after the end (host-driven loop) change nothing
        c->resolve_chunk = 0xFFFFFFFFu;
        c->generate = 0;
        if (in_graph) cudaGraphSetConditional(handle, 0u);
        return;
    }
    c->segments += c->in_count;
    c->shadow += c->sh_count;
    c->parity ^= 1u;
    c->in_count = c->out_count;
    c->out_count = 0;
    c->sh_count = 0;
    c->head_ext = c->head_shade = c->head_sh = 0;
    c->resolve_chunk = 0xFFFFFFFFu;
    c->generate = 0;
    if (c->in_count == 0) {
        // chunk drained: resolve it, then seed the next one or stop
        c->resolve_chunk = c->chunk;
        if (c->chunk + 1 < w.nchunks) {
            c->chunk += 1;
            c->generate = 1;
        } else {
            c->done = 1;
        }
    }
    c->iterations += 1;
    if (c->iterations >= c->max_iterations && !c->done) {
        c->error |= 2u; // bounded loop ran out
        c->done = 1;
    }
    if (in_graph) cudaGraphSetConditional(handle, c->done ? 0u : 1u);
}

__global__ void k_wf_resolve(Wf w) {
    const Ctrl *c = w.ctrl;
    const uint32_t k = c->resolve_chunk;
    if (k == 0xFFFFFFFFu) return;
    const Chunk ch = w.chunks[k];
    for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < ch.resolve_items; item += gridDim.x * blockDim.x) {
        uint32_t lo = ch.seg_begin, hi = ch.seg_end - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (w.segs[mid].pix_base <= item) lo = mid;
            else hi = mid - 1;
        }
        const Segment sg = w.segs[lo];
        const ViewDev &V = w.views[sg.view];
        const uint32_t pix = item - sg.pix_base;
        const uint32_t px = pix % V.set.width, py = pix / V.set.width;
        const size_t fidx = (size_t)(V.set.width - 1 - px) + (size_t)(V.set.height - 1 - py) * V.set.width;
        float acc[3] = {V.sum[fidx * 3], V.sum[fidx * 3 + 1], V.sum[fidx * 3 + 2]};
        double a64[3] = {0, 0, 0}, q64[3] = {0, 0, 0};
        if (V.sum64) {
            for (int k3 = 0; k3 < 3; ++k3) {
                a64[k3] = V.sum64[fidx * 3 + k3];
                q64[k3] = V.sumsq64[fidx * 3 + k3];
            }
        }
        const unsigned long long first = sg.gid - ch.gid_begin + pix;
        for (uint32_t s = sg.s0; s < sg.s1; ++s) {
            const float4 L = w.slots[first + (unsigned long long)(s - sg.s0) * V.npix];
            acc[0] += L.x;
            acc[1] += L.y;
            acc[2] += L.z;
            if (V.sum64) {
                a64[0] += (double)L.x; a64[1] += (double)L.y; a64[2] += (double)L.z;
                q64[0] += (double)L.x * (double)L.x;
                q64[1] += (double)L.y * (double)L.y;
                q64[2] += (double)L.z * (double)L.z;
            }
        }
        V.sum[fidx * 3] = acc[0];
        V.sum[fidx * 3 + 1] = acc[1];
        V.sum[fidx * 3 + 2] = acc[2];
        if (V.sum64) {
            for (int k3 = 0; k3 < 3; ++k3) {
                V.sum64[fidx * 3 + k3] = a64[k3];
                V.sumsq64[fidx * 3 + k3] = q64[k3];
            }
        }
    }
}

// Seeds the pool with the first min(P, chunk size) samples of the chunk.
__global__ void k_wf_generate(Wf w, int first) {
    Ctrl *c = w.ctrl;
    if (!first && !c->generate) return;
    const Chunk ch = w.chunks[c->chunk];
    const unsigned long long total = ch.gid_end - ch.gid_begin;
    const uint32_t count = (uint32_t)(total < w.P ? total : w.P);
    uint32_t *in = q_in(w, *c);
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < count; slot += gridDim.x * blockDim.x) {
        start_sample(w, slot, ch.gid_begin + slot, ch);
        in[slot] = slot;
    }
}

// Sets the counts after a generate (one thread; runs after k_wf_generate).
__global__ void k_wf_generated(Wf w, int first) {
    if (threadIdx.x != 0) return;
    Ctrl *c = w.ctrl;
    if (!first && !c->generate) return;
    const Chunk ch = w.chunks[c->chunk];
    const unsigned long long total = ch.gid_end - ch.gid_begin;
    const uint32_t count = (uint32_t)(total < w.P ? total : w.P);
    c->in_count = count;
    c->issued = ch.gid_begin + count;
    c->generate = 0;
}

__global__ void k_wf_start(Ctrl *c, unsigned int max_iterations) {
    if (threadIdx.x != 0) return;
    Ctrl z{};
    z.resolve_chunk = 0xFFFFFFFFu;
    z.max_iterations = max_iterations;
    *c = z;
}

struct Workspace {
    DevBuf buf;
};

size_t align_up(size_t x) { return (x + 255) / 256 * 256; }

// Persistent grids: each per-bounce kernel fills every SM with as many of its
// own blocks as fit (the traversal kernels need fewer registers than shading,
// so they get more warps to hide memory latency); work is fetched atomically,
// so any grid size is correct.
struct Grids {
    uint32_t ext, shade, shadow;
};

template <class K>
uint32_t resident_grid(K kernel, uint32_t block, int sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, (int)block, 0) != cudaSuccess) {
        (void)cudaGetLastError();
        per_sm = 1;
    }
    return (uint32_t)(std::max(sms, 1) * std::max(per_sm, 1));
}

// INST: kernels for batches with a scene traced through the top-level tree
// (split stages only; with refill, the traversal stages keep the walk per
// lane); batches whose scenes have at most kLoopPlacements placements run the
// placement loop.
template <int W, int FUSE, bool CNT, bool INST>
Grids bounce_grids(const Wf &wf, uint32_t block, int sms) {
    Grids g{0, 0, 0};
    if (FUSE <= 1)
        g.ext = wf.refill ? (INST ? resident_grid(k_wf_extend_dyn<W, CNT, 2>, block, sms)
                                  : wf.placed ? resident_grid(k_wf_extend_dyn<W, CNT, 1>, block, sms)
                                              : resident_grid(k_wf_extend_dyn<W, CNT, 0>, block, sms))
                          : resident_grid(k_wf_extend<W, CNT, INST>, block, sms);
    g.shade = resident_grid(k_wf_shade<W, FUSE, CNT, INST>, block, sms);
    if (FUSE == 0)
        g.shadow = wf.refill_sh ? (INST ? resident_grid(k_wf_shadow_dyn<W, CNT, 2>, block, sms)
                                        : wf.placed ? resident_grid(k_wf_shadow_dyn<W, CNT, 1>, block, sms)
                                                    : resident_grid(k_wf_shadow_dyn<W, CNT, 0>, block, sms))
                                : resident_grid(k_wf_shadow<W, CNT, INST>, block, sms);
    return g;
}

// The traversal stages with per-lane refill: through the top-level tree (INST),
// the placement loop (a scene with placements) or one mesh per scene.
template <int W, bool CNT, bool INST>
void launch_extend_dyn(const Wf &wf, uint32_t grid, uint32_t block, cudaStream_t st) {
    if (INST) k_wf_extend_dyn<W, CNT, 2><<<grid, block, 0, st>>>(wf);
    else if (wf.placed) k_wf_extend_dyn<W, CNT, 1><<<grid, block, 0, st>>>(wf);
    else k_wf_extend_dyn<W, CNT, 0><<<grid, block, 0, st>>>(wf);
}
template <int W, bool CNT, bool INST>
void launch_shadow_dyn(const Wf &wf, uint32_t grid, uint32_t block, cudaStream_t st) {
    if (INST) k_wf_shadow_dyn<W, CNT, 2><<<grid, block, 0, st>>>(wf);
    else if (wf.placed) k_wf_shadow_dyn<W, CNT, 1><<<grid, block, 0, st>>>(wf);
    else k_wf_shadow_dyn<W, CNT, 0><<<grid, block, 0, st>>>(wf);
}

// The per-bounce kernels of one loop iteration for a fusion level.
template <int W, int FUSE, bool CNT, bool INST>
void launch_bounce(const Wf &wf, const Grids &g, uint32_t block, cudaStream_t st) {
    if (FUSE <= 1) {
        if (wf.refill) launch_extend_dyn<W, CNT, INST>(wf, g.ext, block, st);
        else k_wf_extend<W, CNT, INST><<<g.ext, block, 0, st>>>(wf);
    }
    k_wf_shade<W, FUSE, CNT, INST><<<g.shade, block, 0, st>>>(wf);
    if (FUSE == 0) {
        if (wf.refill_sh) launch_shadow_dyn<W, CNT, INST>(wf, g.shadow, block, st);
        else k_wf_shadow<W, CNT, INST><<<g.shadow, block, 0, st>>>(wf);
    }
}

// Host-driven loop: the same kernels launched from the host, which polls the
// done flag every 8 iterations (for profilers that cannot see into graphs
// with conditional nodes, and for runtimes without them).  With `times`, CUDA
// events on the stream bracket every stage of every iteration and the device
// time of each stage is summed into it: extend, shade, shadow, and the
// control / resolve / generate kernels.
template <int W, int FUSE, bool CNT, bool INST>
crg_status run_host(crg_context *ctx, const Wf &wf, uint32_t grid, const Grids &bg, uint32_t block, uint32_t max_iters,
                    cudaStream_t st, crg_stage_times *times) {
    unsigned int *done_h = nullptr;
    if (fault_injected()) return set_error(ctx, CRG_ERR_OOM, "host-driven loop: pinned flag allocation failed (injected fault)");
    CRG_CUDA(ctx, cudaHostAlloc(&done_h, sizeof(unsigned int), cudaHostAllocDefault));
    constexpr int kWin = 8, kMarks = 5; // iterations between polls; events per iteration
    cudaEvent_t ev[kWin * kMarks] = {};
    crg_status rc = CRG_OK;
    if (times) {
        *times = crg_stage_times{};
        for (int k = 0; k < kWin * kMarks && rc == CRG_OK; ++k) {
            const cudaError_t e = cudaEventCreate(&ev[k]);
            if (e != cudaSuccess) rc = cuda_error(ctx, e, "cudaEventCreate");
        }
    }
    auto mark = [&](uint32_t it, int m) {
        if (times) cudaEventRecord(ev[(it % kWin) * kMarks + m], st);
    };
    for (uint32_t it = 0; rc == CRG_OK && it < max_iters + 8; ++it) {
        mark(it, 0);
        if (FUSE <= 1) {
            if (wf.refill) launch_extend_dyn<W, CNT, INST>(wf, bg.ext, block, st);
            else k_wf_extend<W, CNT, INST><<<bg.ext, block, 0, st>>>(wf);
        }
        mark(it, 1);
        k_wf_shade<W, FUSE, CNT, INST><<<bg.shade, block, 0, st>>>(wf);
        mark(it, 2);
        if (FUSE == 0) {
            if (wf.refill_sh) launch_shadow_dyn<W, CNT, INST>(wf, bg.shadow, block, st);
            else k_wf_shadow<W, CNT, INST><<<bg.shadow, block, 0, st>>>(wf);
        }
        mark(it, 3);
        k_wf_control<<<1, 32, 0, st>>>(wf, 0, 0);
        k_wf_resolve<<<grid, 256, 0, st>>>(wf);
        k_wf_generate<<<grid, 256, 0, st>>>(wf, 0);
        k_wf_generated<<<1, 32, 0, st>>>(wf, 0);
        mark(it, 4);
        if ((it % kWin) == kWin - 1) {
            cudaError_t e = cudaMemcpyAsync(done_h, &wf.ctrl->done, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                rc = cuda_error(ctx, e, "wavefront host loop");
                break;
            }
            if (times)
                for (int k = 0; k < kWin; ++k) {
                    float ms[4] = {0, 0, 0, 0};
                    for (int m = 0; m < 4; ++m) cudaEventElapsedTime(&ms[m], ev[k * kMarks + m], ev[k * kMarks + m + 1]);
                    // a stage this fusion level does not launch keeps 0 (its empty event gap
                    // goes to the control stage)
                    times->extend_ms += FUSE <= 1 ? ms[0] : 0.0;
                    times->shade_ms += ms[1];
                    times->shadow_ms += FUSE == 0 ? ms[2] : 0.0;
                    times->other_ms += ms[3] + (FUSE <= 1 ? 0.0 : ms[0]) + (FUSE == 0 ? 0.0 : ms[2]);
                    times->iterations++;
                }
            if (*done_h) break;
        }
    }
    for (int k = 0; k < kWin * kMarks; ++k)
        if (ev[k]) cudaEventDestroy(ev[k]);
    cudaFreeHost(done_h);
    return rc;
}

// Wavefront graphs are kept per context: a graph's kernel nodes hold the Wf
// argument by value, so a batch whose Wf (workspace pointers, pool size,
// chunk count, options) and launch shape equal an earlier batch's relaunches
// that batch's instantiated graph; only the plan arrays it reads change.
struct GraphEntry {
    std::string key;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done = nullptr; // recorded after the entry's last launch
    uint64_t used = 0;
};
constexpr size_t kMaxGraphs = 8;

} // namespace

// Per-context state of the batched form: cached graphs, the pinned staging
// buffers of the host-side plan (two, alternating, each guarded by the event
// of its last copy), and the control blocks of batches in flight (two pinned
// slots, each with the event of its readback).
struct BatchState {
    std::vector<GraphEntry> graphs;
    uint64_t tick = 0;
    void *stage[2] = {nullptr, nullptr};
    size_t stage_cap[2] = {0, 0};
    cudaEvent_t stage_ev[2] = {nullptr, nullptr};
    int stage_next = 0;
    void *ctrl[2] = {nullptr, nullptr}; // a Ctrl each
    cudaEvent_t ctrl_ev[2] = {nullptr, nullptr};
    bool busy[2] = {false, false};
    uint64_t seq[2] = {0, 0}, next_seq = 1;
    crg_render_stats stats[2] = {};
    uint32_t loop_mode[2] = {0, 0}; // crg_wavefront_opts::host_loop of the slot's batch
    // occupancy answers (resident blocks per SM) by kernel set and block size: the
    // runtime's occupancy queries cost tens of microseconds each, every call
    std::vector<std::pair<uint64_t, uint32_t>> occupancy;
    int ctrl_next = 0;
    crg_status sticky = CRG_OK; // first error of the batches collected since the last wait
    std::string sticky_msg;
};

namespace {

crg_status state_of(crg_context *ctx, BatchState *&b) {
    if (!ctx->batch) {
        if (fault_injected()) return set_error(ctx, CRG_ERR_OOM, "batch state allocation failed (injected fault)");
        ctx->batch = new (std::nothrow) BatchState();
        if (!ctx->batch) return set_error(ctx, CRG_ERR_OOM, "batch state allocation failed");
    }
    b = ctx->batch;
    return CRG_OK;
}

// The instantiated graph of one loop body, from the cache or built now.
template <int W, int FUSE, bool CNT, bool INST>
crg_status cached_graph(crg_context *ctx, const Wf &wf, const Grids &bg, uint32_t grid, uint32_t block, GraphEntry *&out) {
    BatchState *B = nullptr;
    crg_status rc = state_of(ctx, B);
    if (rc != CRG_OK) return rc;
    const uint32_t shape[9] = {(uint32_t)W, (uint32_t)FUSE, CNT ? 1u : 0u, INST ? 1u : 0u, grid, block,
                               bg.ext,      bg.shade,       bg.shadow};
    std::string key((const char *)&wf, sizeof(Wf));
    key.append((const char *)shape, sizeof(shape));
    for (GraphEntry &g : B->graphs)
        if (g.key == key) {
            g.used = ++B->tick;
            out = &g;
            return CRG_OK;
        }
    if (B->graphs.size() >= kMaxGraphs) { // evict the least recently used, once its last launch is done
        size_t lru = 0;
        for (size_t k = 1; k < B->graphs.size(); ++k)
            if (B->graphs[k].used < B->graphs[lru].used) lru = k;
        GraphEntry &g = B->graphs[lru];
        cudaEventSynchronize(g.done);
        cudaEventDestroy(g.done);
        cudaGraphExecDestroy(g.exec);
        cudaGraphDestroy(g.graph);
        B->graphs.erase(B->graphs.begin() + (long)lru);
    }
    // one graph: WHILE (not done) { extend, shade, shadow, control, resolve, generate }
    GraphEntry e;
    e.key = key;
    cudaStream_t cap = nullptr;
    do {
        cudaError_t er;
        if ((er = cudaGraphCreate(&e.graph, 0)) != cudaSuccess) { rc = cuda_error(ctx, er, "cudaGraphCreate"); break; }
        cudaGraphConditionalHandle handle;
        if ((er = cudaGraphConditionalHandleCreate(&handle, e.graph, 1, cudaGraphCondAssignDefault)) != cudaSuccess) {
            rc = cuda_error(ctx, er, "cudaGraphConditionalHandleCreate");
            break;
        }
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = handle;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        if ((er = cudaGraphAddNode(&node, e.graph, nullptr, nullptr, 0, &cp)) != cudaSuccess) {
            rc = cuda_error(ctx, er, "cudaGraphAddNode(while)");
            break;
        }
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        if ((er = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess) {
            rc = cuda_error(ctx, er, "cudaStreamCreate");
            break;
        }
        if ((er = cudaStreamBeginCaptureToGraph(cap, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) != cudaSuccess) {
            rc = cuda_error(ctx, er, "cudaStreamBeginCaptureToGraph");
            break;
        }
        launch_bounce<W, FUSE, CNT, INST>(wf, bg, block, cap);
        k_wf_control<<<1, 32, 0, cap>>>(wf, handle, 1);
        k_wf_resolve<<<grid, 256, 0, cap>>>(wf);
        k_wf_generate<<<grid, 256, 0, cap>>>(wf, 0);
        k_wf_generated<<<1, 32, 0, cap>>>(wf, 0);
        er = cudaStreamEndCapture(cap, &body);
        if (er != cudaSuccess) { rc = cuda_error(ctx, er, "cudaStreamEndCapture"); break; }
        if ((er = cudaGraphInstantiate(&e.exec, e.graph, 0)) != cudaSuccess) {
            rc = cuda_error(ctx, er, "cudaGraphInstantiate");
            break;
        }
        if ((er = cudaEventCreateWithFlags(&e.done, cudaEventDisableTiming)) != cudaSuccess) {
            rc = cuda_error(ctx, er, "cudaEventCreate");
            break;
        }
    } while (0);
    if (cap) cudaStreamDestroy(cap);
    if (rc != CRG_OK) {
        if (e.exec) cudaGraphExecDestroy(e.exec);
        if (e.graph) cudaGraphDestroy(e.graph);
        return rc;
    }
    e.used = ++B->tick;
    B->graphs.push_back(e);
    out = &B->graphs.back();
    return CRG_OK;
}

template <int W, int FUSE, bool CNT, bool INST>
crg_status run(crg_context *ctx, const Wf &wf, uint32_t grid, uint32_t block, uint32_t max_iters, cudaStream_t st,
               uint32_t host_loop) {
    // prologue on the caller's stream
    k_wf_start<<<1, 32, 0, st>>>(wf.ctrl, max_iters);
    k_wf_generate<<<grid, 256, 0, st>>>(wf, 1);
    k_wf_generated<<<1, 32, 0, st>>>(wf, 1);
    CRG_CUDA(ctx, cudaGetLastError());
    Grids bg{0, 0, 0};
    {
        // resident grids of this kernel set, cached per context
        BatchState *B = nullptr;
        crg_status rc0 = state_of(ctx, B);
        if (rc0 != CRG_OK) return rc0;
        const uint64_t key = (uint64_t)W | (uint64_t)FUSE << 8 | (uint64_t)CNT << 12 | (uint64_t)INST << 13 |
                             (uint64_t)(wf.refill != 0) << 14 | (uint64_t)(wf.refill_sh != 0) << 15 | (uint64_t)block << 16 |
                             (uint64_t)wf.placed << 36;
        uint32_t found = 0;
        for (const auto &e : B->occupancy)
            if (e.first == (key | 1ull << 40) || e.first == (key | 2ull << 40) || e.first == (key | 3ull << 40)) found++;
        if (found == 3) {
            for (const auto &e : B->occupancy) {
                if (e.first == (key | 1ull << 40)) bg.ext = e.second;
                if (e.first == (key | 2ull << 40)) bg.shade = e.second;
                if (e.first == (key | 3ull << 40)) bg.shadow = e.second;
            }
        } else {
            bg = bounce_grids<W, FUSE, CNT, INST>(wf, block, ctx->sm_count);
            B->occupancy.push_back({key | 1ull << 40, bg.ext});
            B->occupancy.push_back({key | 2ull << 40, bg.shade});
            B->occupancy.push_back({key | 3ull << 40, bg.shadow});
        }
    }
    {
        // a pool smaller than a resident grid's threads needs fewer blocks: in a small batch the
        // others would only start, find the queue empty and exit, every stage of every bounce
        const uint32_t need = std::max<uint32_t>(1u, (uint32_t)(((uint64_t)wf.P + block - 1) / block));
        bg.ext = std::min(bg.ext, need);
        bg.shade = std::min(bg.shade, need);
        bg.shadow = std::min(bg.shadow, need);
    }
    if (host_loop)
        return run_host<W, FUSE, CNT, INST>(ctx, wf, grid, bg, block, max_iters, st,
                                            host_loop == 2 ? &ctx->stage_times : nullptr);
    GraphEntry *g = nullptr;
    const crg_status rc = cached_graph<W, FUSE, CNT, INST>(ctx, wf, bg, grid, block, g);
    if (rc != CRG_OK) return rc;
    CRG_CUDA(ctx, cudaGraphLaunch(g->exec, st));
    CRG_CUDA(ctx, cudaEventRecord(g->done, st));
    return CRG_OK;
}

template <int W, int FUSE>
int occupancy_of(int block) {
    int a = 0, b = 0, c = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_wf_shade<W, FUSE, false, false>, block, 0);
    a = b;
    if (FUSE <= 1 && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_wf_extend<W, false, false>, block, 0) == cudaSuccess)
        a = std::min(a, c);
    if (FUSE <= 1 && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_wf_extend_dyn<W, false, 0>, block, 0) == cudaSuccess)
        a = std::min(a, c);
    if (FUSE == 0 && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_wf_shadow<W, false, false>, block, 0) == cudaSuccess)
        a = std::min(a, c);
    if (FUSE == 0 && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_wf_shadow_dyn<W, false, 0>, block, 0) == cudaSuccess)
        a = std::min(a, c);
    cudaGetLastError();
    return std::max(a, 1);
}

int occupancy(uint32_t width, uint32_t fuse, int block) {
    switch (width * 4 + fuse) {
    case 8: return occupancy_of<2, 0>(block);
    case 9: return occupancy_of<2, 1>(block);
    case 10: return occupancy_of<2, 2>(block);
    case 16: return occupancy_of<4, 0>(block);
    case 17: return occupancy_of<4, 1>(block);
    case 18: return occupancy_of<4, 2>(block);
    case 32: return occupancy_of<8, 0>(block);
    case 33: return occupancy_of<8, 1>(block);
    default: return occupancy_of<8, 2>(block);
    }
}

template <int W>
crg_status dispatch_w(crg_context *ctx, const Wf &wf, uint32_t fuse, bool cnt, bool inst, uint32_t grid, uint32_t block,
                      uint32_t max_iters, cudaStream_t st, uint32_t hl) {
    if (inst) // batches with placements run the split stages
        return cnt ? run<W, 0, true, true>(ctx, wf, grid, block, max_iters, st, hl)
                   : run<W, 0, false, true>(ctx, wf, grid, block, max_iters, st, hl);
    switch (fuse * 2 + (cnt ? 1 : 0)) {
    case 0: return run<W, 0, false, false>(ctx, wf, grid, block, max_iters, st, hl);
    case 1: return run<W, 0, true, false>(ctx, wf, grid, block, max_iters, st, hl);
    case 2: return run<W, 1, false, false>(ctx, wf, grid, block, max_iters, st, hl);
    case 3: return run<W, 1, true, false>(ctx, wf, grid, block, max_iters, st, hl);
    case 4: return run<W, 2, false, false>(ctx, wf, grid, block, max_iters, st, hl);
    default: return run<W, 2, true, false>(ctx, wf, grid, block, max_iters, st, hl);
    }
}

crg_status dispatch(crg_context *ctx, const Wf &wf, uint32_t width, uint32_t fuse, bool cnt, bool inst, uint32_t grid,
                    uint32_t block, uint32_t max_iters, cudaStream_t st, uint32_t hl) {
    switch (width) {
    case 2: return dispatch_w<2>(ctx, wf, fuse, cnt, inst, grid, block, max_iters, st, hl);
    case 4: return dispatch_w<4>(ctx, wf, fuse, cnt, inst, grid, block, max_iters, st, hl);
    default: return dispatch_w<8>(ctx, wf, fuse, cnt, inst, grid, block, max_iters, st, hl);
    }
}

std::string ctx_message(const crg_context *ctx) {
    std::lock_guard<std::mutex> lock(ctx->error_mutex);
    return ctx->last_error;
}

// Reads back the control block of the batch in `slot` (waiting for it), turns
// its error word into a status, and keeps its statistics.
crg_status collect(crg_context *ctx, BatchState *B, int slot) {
    if (!B->busy[slot]) return CRG_OK;
    B->busy[slot] = false;
    CRG_CUDA(ctx, cudaEventSynchronize(B->ctrl_ev[slot]));
    const Ctrl &c = *(const Ctrl *)B->ctrl[slot];
    crg_render_stats &s = B->stats[slot];
    s.segments = c.segments;
    s.shadow_rays = c.shadow;
    s.nodes_visited = c.nodes + c.nodes_sh;
    s.tris_tested = c.tris + c.tris_sh;
    s.iterations = c.iterations;
    ctx->batch_stats = s;
    if (B->loop_mode[slot] == 2) {
        ctx->stage_times.shadow_nodes = c.nodes_sh;
        ctx->stage_times.shadow_tris = c.tris_sh;
    }
    if (c.error & 2u) return set_error(ctx, CRG_ERR_TIMEOUT, "wavefront: iteration cap reached before the batch drained");
    if (c.error & 1u) return set_error(ctx, CRG_ERR_DEVICE, "wavefront: traversal stack overflow");
    return CRG_OK;
}

} // namespace

crg_status batch_wait(crg_context *ctx) {
    BatchState *B = ctx->batch;
    if (!B) return CRG_OK;
    // oldest first, so the statistics left are the last batch's
    const int first = (B->busy[0] && B->busy[1]) ? (B->seq[0] < B->seq[1] ? 0 : 1) : (B->busy[0] ? 0 : 1);
    for (int k = 0; k < 2; ++k) {
        const crg_status rc = collect(ctx, B, first ^ k);
        if (rc != CRG_OK && !B->sticky) {
            B->sticky = rc;
            B->sticky_msg = ctx_message(ctx);
        }
    }
    const crg_status rc = B->sticky;
    if (rc != CRG_OK) set_error(ctx, rc, B->sticky_msg);
    B->sticky = CRG_OK;
    B->sticky_msg.clear();
    return rc;
}

void batch_state_free(crg_context *ctx) {
    BatchState *B = ctx->batch;
    if (!B) return;
    cudaDeviceSynchronize();
    for (GraphEntry &g : B->graphs) {
        if (g.done) cudaEventDestroy(g.done);
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.graph) cudaGraphDestroy(g.graph);
    }
    for (int k = 0; k < 2; ++k) {
        if (B->stage[k]) cudaFreeHost(B->stage[k]);
        if (B->stage_ev[k]) cudaEventDestroy(B->stage_ev[k]);
        if (B->ctrl[k]) cudaFreeHost(B->ctrl[k]);
        if (B->ctrl_ev[k]) cudaEventDestroy(B->ctrl_ev[k]);
    }
    delete B;
    ctx->batch = nullptr;
}

crg_status render_batch(crg_context *ctx, crg_scene *const *scenes, uint32_t nscenes, const crg_view *views,
                        crg_film *const *films, uint32_t nviews, const crg_wavefront_opts &o, cudaStream_t st,
                        bool wait) {
    // ---- host-side plan: views, segments, chunks
    const uint32_t width = scenes[0]->width;
    std::vector<SceneDev> sdev(nscenes);
    for (uint32_t i = 0; i < nscenes; ++i) sdev[i] = scene_dev(scenes[i]);
    std::vector<ViewDev> vdev(nviews);
    unsigned long long total = 0;
    for (uint32_t v = 0; v < nviews; ++v) {
        ViewDev &V = vdev[v];
        V.cam = camera_params(views[v].camera);
        V.set = views[v].settings;
        V.scene = views[v].scene;
        V.npix = V.set.width * V.set.height;
        V.spp0 = films[v]->spp;
        V.sum = (float *)films[v]->sum.ptr;
        V.sum64 = (double *)films[v]->sum64.ptr;
        V.sumsq64 = (double *)films[v]->sumsq64.ptr;
        total += (unsigned long long)V.npix * V.set.spp;
    }
    if (total == 0) { // nothing to trace: films and their sample counts stay as they are
        ctx->batch_stats = crg_render_stats{};
        return CRG_OK;
    }
    const unsigned long long C = o.chunk_samples;
    std::vector<Segment> segs;
    std::vector<Chunk> chunks;
    {
        unsigned long long gid = 0, chunk_fill = 0;
        Chunk cur{0, 0, 0, 0, 0, 0};
        for (uint32_t v = 0; v < nviews; ++v) {
            const uint32_t npix = vdev[v].npix;
            uint32_t s = 0;
            while (s < vdev[v].set.spp) {
                if (chunk_fill + npix > C && chunk_fill > 0) { // close the chunk
                    cur.gid_end = gid;
                    cur.seg_end = (uint32_t)segs.size();
                    chunks.push_back(cur);
                    cur = Chunk{gid, 0, (uint32_t)segs.size(), 0, 0, 0};
                    chunk_fill = 0;
                }
                const unsigned long long room = C > chunk_fill ? (C - chunk_fill) / npix : 0;
                uint32_t take = (uint32_t)std::min<unsigned long long>(vdev[v].set.spp - s, std::max<unsigned long long>(room, 1));
                Segment sg{gid, v, s, s + take, cur.resolve_items};
                segs.push_back(sg);
                cur.resolve_items += npix;
                gid += (unsigned long long)take * npix;
                chunk_fill += (unsigned long long)take * npix;
                s += take;
            }
        }
        cur.gid_end = gid;
        cur.seg_end = (uint32_t)segs.size();
        if (cur.seg_end > cur.seg_begin) chunks.push_back(cur);
    }
    unsigned long long max_chunk = 0;
    for (const Chunk &ch : chunks) max_chunk = std::max(max_chunk, ch.gid_end - ch.gid_begin);
    const uint32_t P = (uint32_t)std::min<unsigned long long>(o.path_pool, max_chunk);
    // ---- device workspace (grow-only, owned by the context)
    const size_t n_sc = align_up(sizeof(SceneDev) * nscenes), n_vd = align_up(sizeof(ViewDev) * nviews);
    const size_t n_sg = align_up(sizeof(Segment) * segs.size()), n_ch = align_up(sizeof(Chunk) * chunks.size());
    const size_t n_ctrl = align_up(sizeof(Ctrl));
    const size_t n_f4 = align_up(sizeof(float4) * (size_t)P), n_u4 = align_up(sizeof(uint4) * (size_t)P);
    const size_t n_q = align_up(sizeof(uint32_t) * (size_t)P);
    const size_t n_slots = align_up(sizeof(float4) * (size_t)max_chunk);
    const size_t bytes = n_sc + n_vd + n_sg + n_ch + n_ctrl + 8 * n_f4 + n_u4 + 3 * n_q + n_slots;
    crg_status rc = dev_alloc(ctx, ctx->wf_ws, bytes);
    if (rc != CRG_OK) return rc;
    char *p = (char *)ctx->wf_ws.ptr;
    auto take = [&](size_t b) {
        char *r = p;
        p += b;
        return r;
    };
    Wf wf{};
    SceneDev *d_sc = (SceneDev *)take(n_sc);
    ViewDev *d_vd = (ViewDev *)take(n_vd);
    Segment *d_sg = (Segment *)take(n_sg);
    Chunk *d_ch = (Chunk *)take(n_ch);
    wf.ctrl = (Ctrl *)take(n_ctrl);
    wf.scenes = d_sc;
    wf.views = d_vd;
    wf.segs = d_sg;
    wf.chunks = d_ch;
    wf.nchunks = (uint32_t)chunks.size();
    wf.P = P;
    wf.fetch = o.fetch;
    // per-lane refill resumes a traversal: of one mesh, or of one placement of a
    // scene (the refill kernels keep the placement loop or the top-level walk)
    bool instanced = false, tree = false; // placements; more of them than the plain loop takes
    for (uint32_t i = 0; i < nscenes; ++i) {
        if (scenes[i]->ninst) instanced = true;
        if (scenes[i]->ninst > kLoopPlacements) tree = true;
    }
    wf.refill = o.refill;
    wf.placed = instanced ? (tree ? 2u : 1u) : 0u;
    bool sun_requests = false; // the faithful estimator's sun test steps through alpha surfaces
    for (uint32_t v = 0; v < nviews; ++v)
        if (vdev[v].set.mode == CRG_MODE_FAITHFUL && scenes[vdev[v].scene]->sun_enabled) sun_requests = true;
    wf.refill_sh = sun_requests ? 0u : o.refill;
    wf.o = (float4 *)take(n_f4);
    wf.d = (float4 *)take(n_f4);
    wf.T = (float4 *)take(n_f4);
    wf.L = (float4 *)take(n_f4);
    wf.hit = (float4 *)take(n_f4);
    wf.sh_o = (float4 *)take(n_f4);
    wf.sh_d = (float4 *)take(n_f4);
    wf.sh_c = (float4 *)take(n_f4);
    wf.meta = (uint4 *)take(n_u4);
    wf.qa = (uint32_t *)take(n_q);
    wf.qb = (uint32_t *)take(n_q);
    wf.qsh = (uint32_t *)take(n_q);
    wf.slots = (float4 *)take(n_slots);
    // the plan goes to the device through a pinned staging buffer (a copy from pageable memory
    // would wait for the stream), alternating between two so that the host can prepare the next
    // batch while this one's copy is pending
    BatchState *B = nullptr;
    if ((rc = state_of(ctx, B)) != CRG_OK) return rc;
    {
        const int k = B->stage_next;
        B->stage_next ^= 1;
        const size_t plan = n_sc + n_vd + n_sg + n_ch;
        if (B->stage_ev[k]) CRG_CUDA(ctx, cudaEventSynchronize(B->stage_ev[k]));
        else CRG_CUDA(ctx, cudaEventCreateWithFlags(&B->stage_ev[k], cudaEventDisableTiming));
        if (B->stage_cap[k] < plan) {
            if (B->stage[k]) cudaFreeHost(B->stage[k]);
            B->stage[k] = nullptr;
            B->stage_cap[k] = 0;
            if (fault_injected()) return set_error(ctx, CRG_ERR_OOM, "pinned plan staging failed (injected fault)");
            CRG_CUDA(ctx, cudaHostAlloc(&B->stage[k], plan, cudaHostAllocDefault));
            B->stage_cap[k] = plan;
        }
        char *h = (char *)B->stage[k];
        std::memcpy(h, sdev.data(), sizeof(SceneDev) * nscenes);
        std::memcpy(h + n_sc, vdev.data(), sizeof(ViewDev) * nviews);
        std::memcpy(h + n_sc + n_vd, segs.data(), sizeof(Segment) * segs.size());
        std::memcpy(h + n_sc + n_vd + n_sg, chunks.data(), sizeof(Chunk) * chunks.size());
        CRG_CUDA(ctx, cudaMemcpyAsync(d_sc, h, plan, cudaMemcpyHostToDevice, st)); // d_sc .. d_ch are contiguous
        CRG_CUDA(ctx, cudaEventRecord(B->stage_ev[k], st));
    }
    // persistent grid: resident blocks of the launched kernels on every SM
    const uint32_t fuse = instanced ? 0u : (o.fuse ? o.fuse - 1 : 0); // fusion level 0..2 (split with placements)
    int per_sm = 0;
    {
        const uint64_t key = (uint64_t)width | (uint64_t)fuse << 8 | (uint64_t)o.block_size << 16 | 4ull << 40;
        for (const auto &e : B->occupancy)
            if (e.first == key) per_sm = (int)e.second;
        if (!per_sm) {
            per_sm = occupancy(width, fuse, (int)o.block_size);
            B->occupancy.push_back({key, (uint32_t)per_sm});
        }
    }
    const uint32_t grid = (uint32_t)(std::max(ctx->sm_count, 1) * per_sm);
    // every chunk needs at most (samples / P + 1) refills of max_bounces + 1 iterations
    unsigned long long iters = 16;
    uint32_t maxb = 1;
    for (uint32_t v = 0; v < nviews; ++v) maxb = std::max(maxb, vdev[v].set.max_bounces);
    for (const Chunk &ch : chunks) iters += ((ch.gid_end - ch.gid_begin) / std::max<uint32_t>(P, 1) + 2) * (maxb + 2) * 4;
    uint32_t max_iters = (uint32_t)std::min<unsigned long long>(iters, 0x7FFFFFFFull);
    if (o.max_iterations) max_iters = o.max_iterations;
    const bool cnt = o.count_work != 0;
    const uint32_t hl = o.host_loop;
    // the control block comes back through a pinned slot, read when the batch is waited for
    const int slot = B->ctrl_next;
    if (B->busy[slot]) { // the slot's earlier batch: collect it first
        if ((rc = collect(ctx, B, slot)) != CRG_OK && !B->sticky) {
            B->sticky = rc;
            B->sticky_msg = ctx_message(ctx);
        }
    }
    if (!B->ctrl[slot]) {
        if (fault_injected()) return set_error(ctx, CRG_ERR_OOM, "pinned control block failed (injected fault)");
        CRG_CUDA(ctx, cudaHostAlloc(&B->ctrl[slot], sizeof(Ctrl), cudaHostAllocDefault));
        CRG_CUDA(ctx, cudaEventCreateWithFlags(&B->ctrl_ev[slot], cudaEventDisableTiming));
    }
    rc = dispatch(ctx, wf, width, fuse, cnt, tree, grid, o.block_size, max_iters, st, hl);
    if (rc != CRG_OK) return rc;
    CRG_CUDA(ctx, cudaMemcpyAsync(B->ctrl[slot], wf.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, st));
    CRG_CUDA(ctx, cudaEventRecord(B->ctrl_ev[slot], st));
    B->busy[slot] = true;
    B->seq[slot] = B->next_seq++;
    B->stats[slot] = crg_render_stats{};
    B->stats[slot].samples = total;
    B->loop_mode[slot] = hl;
    B->ctrl_next ^= 1;
    if (hl != 2) ctx->stage_times = crg_stage_times{};
    // sample indices of the films' next calls continue after this batch's
    for (uint32_t v = 0; v < nviews; ++v) films[v]->spp += vdev[v].set.spp;
    return wait ? batch_wait(ctx) : CRG_OK;
}

} // namespace crg
