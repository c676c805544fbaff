// adjoint.cu — path-replay adjoint of the extended estimator (sm_103a).
//
// Path replay backpropagation (Vicini, Speierer & Jakob, "Path Replay
// Backpropagation", SIGGRAPH 2021): each adjoint sample re-traces its path from
// its random-number key (pixel, sample, dimension, seed) with the forward
// shading code (render_common.cuh), so no path is stored.  With the random
// decisions fixed (Russian roulette detached, as in PRB), every contribution
// to a sample's radiance is a product of per-bounce factors, each depending on
// one material's colour, times the emitter's colour and emission.  The
// gradient of <adjoint, pixel mean> with respect to a factor's parameter is
// therefore the contribution times d log(factor) / d parameter, summed over
// the factors the contribution carries: every contribution adds
// delta_pixel * contribution * d log(factor) to the gradient of the material
// of each factor it carries (at most one factor per bounce): Lambert and glass colour (1 / colour), GGX F0 through Schlick's
// Fresnel, emitter colour (1 / colour) and emission (1 / emission).
// Instead of adding to every factor at every contribution (quadratic in the
// path length), a thread keeps the running sum Wc of its path's contribution
// weights (delta_pixel * contribution) and, per factor, the value of Wc when
// the factor was pushed: the factor's gradient is d log(factor) times the
// weight that arrived after it (Wc at path end minus that value), added once
// when the path ends.  A light sample taken at a vertex is shaded after that
// vertex's factor was pushed but does not carry it (it carries the BSDF
// evaluated towards the light instead), so its weight is also added to the
// pushed factor's start value; when both factors are the same (Lambert) the
// two cancel and nothing is done.  Emitter terms go to a one-entry per-thread
// cache keyed by the emitter's material.  Gradients accumulate in FP64: per
// warp in shared memory, then once per block into the caller's arrays.
#include "render_common.cuh"

namespace crg {
using namespace rc;
namespace {

constexpr int kMaxFactors = 32;

struct GradTape {
    uint32_t n;
    uint32_t mat[kMaxFactors];
    v3 dlog[kMaxFactors];
    double pre[kMaxFactors][3]; // Wc when the factor was pushed
    double wc[3];               // weight of the path's contributions so far
    double dx, dy, dz;          // adjoint of the pixel mean / spp, per channel
    uint32_t em_mat;            // emitter cache (0xffffffff = empty)
    double ew[3];
    const crg_material *mats;
    double *g_col, *g_em;

    __device__ __forceinline__ void add3(uint32_t m, v3 d, double wx, double wy, double wz) {
        if (wx != 0.0 && d.x != 0.0f) atomicAdd(&g_col[3 * m + 0], wx * (double)d.x);
        if (wy != 0.0 && d.y != 0.0f) atomicAdd(&g_col[3 * m + 1], wy * (double)d.y);
        if (wz != 0.0 && d.z != 0.0f) atomicAdd(&g_col[3 * m + 2], wz * (double)d.z);
    }
    __device__ __forceinline__ void flush_emitter() {
        if (em_mat == 0xffffffffu) return;
        const crg_material &em = mats[em_mat];
        add3(em_mat, inv_or_zero(mk(em.colour[0], em.colour[1], em.colour[2])), ew[0], ew[1], ew[2]);
        if (em.emission > 0.0f) atomicAdd(&g_em[em_mat], (ew[0] + ew[1] + ew[2]) / (double)em.emission);
        em_mat = 0xffffffffu;
    }
    __device__ __forceinline__ void emitter(uint32_t m, double wx, double wy, double wz) {
        if (m != em_mat) {
            flush_emitter();
            em_mat = m;
            ew[0] = ew[1] = ew[2] = 0.0;
        }
        ew[0] += wx;
        ew[1] += wy;
        ew[2] += wz;
    }
    __device__ __forceinline__ void begin() {
        n = 0;
        wc[0] = wc[1] = wc[2] = 0.0;
    }
    // Weight of contribution C, added to the running sum.
    __device__ __forceinline__ void weigh(v3 C, double &wx, double &wy, double &wz) {
        wx = dx * (double)C.x;
        wy = dy * (double)C.y;
        wz = dz * (double)C.z;
        wc[0] += wx;
        wc[1] += wy;
        wc[2] += wz;
    }
    __device__ __forceinline__ void mult(uint32_t m, v3 d) {
        if (n < kMaxFactors) {
            mat[n] = m;
            dlog[n] = d;
            pre[n][0] = wc[0];
            pre[n][1] = wc[1];
            pre[n][2] = wc[2];
            ++n;
        }
    }
    __device__ __forceinline__ void env(v3 C) {
        double wx, wy, wz;
        weigh(C, wx, wy, wz);
    }
    __device__ __forceinline__ void emit(v3 C, uint32_t m) {
        double wx, wy, wz;
        weigh(C, wx, wy, wz);
        emitter(m, wx, wy, wz);
    }
    // Light sample at the vertex whose factor (if any) has index nf.
    __device__ __forceinline__ void nee(const NeeReq &nr, uint32_t nf) {
        double wx, wy, wz;
        weigh(nr.c, wx, wy, wz);
        emitter(nr.light_mat, wx, wy, wz);
        const bool pushed = n > nf;
        if (pushed && mat[nf] == nr.bsdf_mat && __float_as_uint(dlog[nf].x) == __float_as_uint(nr.bsdf_dlog.x) &&
            __float_as_uint(dlog[nf].y) == __float_as_uint(nr.bsdf_dlog.y) &&
            __float_as_uint(dlog[nf].z) == __float_as_uint(nr.bsdf_dlog.z))
            return;
        if (pushed) {
            pre[nf][0] += wx;
            pre[nf][1] += wy;
            pre[nf][2] += wz;
        }
        add3(nr.bsdf_mat, nr.bsdf_dlog, wx, wy, wz);
    }
    // Path end: every factor gets the weight that arrived after it.
    __device__ __forceinline__ void end() {
        for (uint32_t k = 0; k < n; ++k)
            add3(mat[k], dlog[k], wc[0] - pre[k][0], wc[1] - pre[k][1], wc[2] - pre[k][2]);
    }
};

template <int W, bool INST>
__global__ void __launch_bounds__(128) k_adjoint(SceneDev S, CamDev cam, crg_settings set, const float *__restrict__ adj,
                                                 double *__restrict__ g_col, double *__restrict__ g_em, uint32_t nmat,
                                                 uint32_t copies) {
    extern __shared__ double sh[];
    double *col = g_col, *em = g_em;
    const uint32_t nacc = 4 * nmat;
    if (copies) {
        for (uint32_t k = threadIdx.x; k < copies * nacc; k += blockDim.x) sh[k] = 0.0;
        __syncthreads();
        double *mine = sh + (size_t)((threadIdx.x >> 5) % copies) * nacc;
        col = mine;
        em = mine + 3 * nmat;
    }
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t Wd = set.width, Hd = set.height;
    PathCtx C{pix, 0, set.seed, 0, 0, 0, 0ull, 0ull};
    uint32_t lanes = __ballot_sync(0xFFFFFFFFu, pix < Wd * Hd);
    if (pix < Wd * Hd) {
        const uint32_t px = pix % Wd, py = pix / Wd;
        const size_t fidx = (size_t)(Wd - 1 - px) + (size_t)(Hd - 1 - py) * Wd;
        const double inv = 1.0 / (double)set.spp;
        GradTape tape;
        tape.mats = S.mats;
        tape.g_col = col;
        tape.g_em = em;
        tape.em_mat = 0xffffffffu;
        tape.dx = (double)adj[fidx * 3] * inv;
        tape.dy = (double)adj[fidx * 3 + 1] * inv;
        tape.dz = (double)adj[fidx * 3 + 2] * inv;
        const bool live = tape.dx != 0.0 || tape.dy != 0.0 || tape.dz != 0.0;
        // one loop over segments with path regeneration, as in the forward megakernel
        PathState ps;
        Aov aov;
        uint32_t s = 0, i = 0;
        for (;;) {
            // the lanes still replaying meet before every segment (as in the forward megakernel)
            lanes = __ballot_sync(lanes, live && s < set.spp);
            if (!(live && s < set.spp)) break;
            if (i == 0) {
                C.sample = s;
                const f4 g0 = rand4(pix, s, 0, set.seed);
                const float x = ((float)px + g0.x) / (float)Wd;
                const float y = ((float)py + g0.y) / (float)Hd;
                v3 o, d;
                camera_ray(cam, x, y, set.aspect, o, d);
                path_start(ps, o, d);
                tape.begin();
            }
            if (i < set.max_bounces) {
                Hit h;
                const bool found = closest<W, false, INST>(S, ps.o, ps.d, INFINITY, h, C);
                NeeReq nr;
                const uint32_t nf = tape.n;
                const bool cont = shade_extended(S, set, C, i, ps, found, h, aov, nr, &tape);
                if (nr.kind != 0 && shadow_visible<W, false, INST>(S, nr, C)) {
                    ps.L = add(ps.L, nr.c);
                    tape.nee(nr, nf);
                }
                ++i;
                if (cont && i < set.max_bounces) continue;
            }
            tape.end();
            ++s;
            i = 0;
        }
        tape.flush_emitter();
    }
    if (C.err) atomicOr(S.err, C.err);
    if (copies) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < nacc; k += blockDim.x) {
            double v = 0.0;
            for (uint32_t c = 0; c < copies; ++c) v += sh[(size_t)c * nacc + k];
            if (v != 0.0) atomicAdd(k < 3 * nmat ? &g_col[k] : &g_em[k - 3 * nmat], v);
        }
    }
}

// Block sums of (I - T)^2 in FP64, one atomic per block; d_adjoint written alongside.
__global__ void __launch_bounds__(256) k_loss_l2(const float *__restrict__ sum, float inv_spp, const float *__restrict__ tgt,
                                                 float *__restrict__ adj, double *__restrict__ loss, uint64_t n, float scale,
                                                 double inv_n) {
    __shared__ double part[8];
    double acc = 0.0;
    for (uint64_t k = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const float d = sum[k] * inv_spp - tgt[k];
        adj[k] = d * scale;
        acc += (double)d * (double)d;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[w];
        atomicAdd(loss, t * inv_n);
    }
}

} // namespace

crg_status launch_loss_l2(crg_film *f, const float *target, float *adj, double *loss, cudaStream_t st) {
    const uint64_t n = (uint64_t)f->width * f->height * 3;
    CRG_CUDA(f->ctx, cudaMemsetAsync(loss, 0, sizeof(double), st));
    const uint32_t T = 256;
    const uint64_t want = (n + T - 1) / T;
    const uint32_t blocks = (uint32_t)(want < 4096 ? want : 4096);
    k_loss_l2<<<blocks, T, 0, st>>>((const float *)f->sum.ptr, 1.0f / (float)f->spp, target, adj, loss, n,
                                    2.0f / (float)n, 1.0 / (double)n);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(f->ctx, e, "k_loss_l2 launch");
    return CRG_OK;
}

crg_status launch_backward(crg_scene *s, const CamDev &cam, const crg_settings &set, const float *adj, double *g_col,
                           double *g_em, cudaStream_t st) {
    const SceneDev S = scene_dev(s);
    const uint32_t T = 128;
    const uint64_t npix = (uint64_t)set.width * set.height;
    const uint32_t blocks = (uint32_t)((npix + T - 1) / T);
    // one FP64 accumulator copy per warp when it fits in 48 KB, else one per block, else global atomics
    const size_t per_copy = sizeof(double) * 4 * (size_t)s->nmat;
    const uint32_t copies = per_copy * (T / 32) <= 48 * 1024 ? T / 32 : (per_copy <= 48 * 1024 ? 1 : 0);
    const size_t dyn = per_copy * copies;
    switch (s->width) {
    case 2:
        if (S.ninst > kLoopPlacements) k_adjoint<2, true><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, copies);
        else k_adjoint<2, false><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, copies);
        break;
    case 4:
        if (S.ninst > kLoopPlacements) k_adjoint<4, true><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, copies);
        else k_adjoint<4, false><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, copies);
        break;
    default:
        if (S.ninst > kLoopPlacements) k_adjoint<8, true><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, copies);
        else k_adjoint<8, false><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, copies);
        break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(s->ctx, e, "k_adjoint launch");
    return CRG_OK;
}

} // namespace crg
