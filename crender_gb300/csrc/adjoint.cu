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
// the factors the contribution carries.  A thread keeps its path's factor list
// (at most one per bounce) and, at every contribution, adds
// delta_pixel * contribution * d log(factor) to the gradient of each factor's
// material: Lambert and glass colour (1 / colour), GGX F0 through Schlick's
// Fresnel, emitter colour (1 / colour) and emission (1 / emission).
// Gradients accumulate in FP64: per block in shared memory, then once per
// block into the caller's arrays.
#include "render_common.cuh"

namespace crg {
using namespace rc;
namespace {

constexpr int kMaxFactors = 32;

struct GradTape {
    uint32_t n;
    uint32_t mat[kMaxFactors];
    v3 dlog[kMaxFactors];
    double dx, dy, dz; // adjoint of the pixel mean / spp, per channel
    const crg_material *mats;
    double *g_col, *g_em;

    __device__ __forceinline__ void add_factor(uint32_t m, v3 d, double wx, double wy, double wz) {
        if (wx != 0.0 && d.x != 0.0f) atomicAdd(&g_col[3 * m + 0], wx * (double)d.x);
        if (wy != 0.0 && d.y != 0.0f) atomicAdd(&g_col[3 * m + 1], wy * (double)d.y);
        if (wz != 0.0 && d.z != 0.0f) atomicAdd(&g_col[3 * m + 2], wz * (double)d.z);
    }
    __device__ __forceinline__ void emitter(uint32_t m, double wx, double wy, double wz) {
        const crg_material &em = mats[m];
        const v3 col = mk(em.colour[0], em.colour[1], em.colour[2]);
        add_factor(m, inv_or_zero(col), wx, wy, wz);
        if (em.emission > 0.0f) atomicAdd(&g_em[m], (wx + wy + wz) / (double)em.emission);
    }
    __device__ __forceinline__ void path(v3 C, double &wx, double &wy, double &wz) {
        wx = dx * (double)C.x;
        wy = dy * (double)C.y;
        wz = dz * (double)C.z;
        for (uint32_t k = 0; k < n; ++k) add_factor(mat[k], dlog[k], wx, wy, wz);
    }
    __device__ __forceinline__ void mult(uint32_t m, v3 d) {
        if (n < kMaxFactors) {
            mat[n] = m;
            dlog[n] = d;
            ++n;
        }
    }
    __device__ __forceinline__ void env(v3 C) {
        double wx, wy, wz;
        path(C, wx, wy, wz);
    }
    __device__ __forceinline__ void emit(v3 C, uint32_t m) {
        double wx, wy, wz;
        path(C, wx, wy, wz);
        emitter(m, wx, wy, wz);
    }
    __device__ __forceinline__ void nee(const NeeReq &nr) {
        double wx, wy, wz;
        path(nr.c, wx, wy, wz);
        add_factor(nr.bsdf_mat, nr.bsdf_dlog, wx, wy, wz);
        emitter(nr.light_mat, wx, wy, wz);
    }
};

template <int W>
__global__ void __launch_bounds__(128) k_adjoint(SceneDev S, CamDev cam, crg_settings set, const float *__restrict__ adj,
                                                 double *__restrict__ g_col, double *__restrict__ g_em, uint32_t nmat,
                                                 int use_shared) {
    extern __shared__ double sh[];
    double *col = g_col, *em = g_em;
    if (use_shared) {
        for (uint32_t k = threadIdx.x; k < 4 * nmat; k += blockDim.x) sh[k] = 0.0;
        __syncthreads();
        col = sh;
        em = sh + 3 * nmat;
    }
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t Wd = set.width, Hd = set.height;
    PathCtx C{pix, 0, set.seed, 0, 0, 0, 0ull, 0ull};
    if (pix < Wd * Hd) {
        const uint32_t px = pix % Wd, py = pix / Wd;
        const size_t fidx = (size_t)(Wd - 1 - px) + (size_t)(Hd - 1 - py) * Wd;
        const double inv = 1.0 / (double)set.spp;
        GradTape tape;
        tape.mats = S.mats;
        tape.g_col = col;
        tape.g_em = em;
        tape.dx = (double)adj[fidx * 3] * inv;
        tape.dy = (double)adj[fidx * 3 + 1] * inv;
        tape.dz = (double)adj[fidx * 3 + 2] * inv;
        const bool live = tape.dx != 0.0 || tape.dy != 0.0 || tape.dz != 0.0;
        for (uint32_t s = 0; live && s < set.spp; ++s) {
            C.sample = s;
            const f4 g0 = rand4(pix, s, 0, set.seed);
            const float x = ((float)px + g0.x) / (float)Wd;
            const float y = ((float)py + g0.y) / (float)Hd;
            v3 o, d;
            camera_ray(cam, x, y, set.aspect, o, d);
            PathState ps;
            path_start(ps, o, d);
            Aov aov;
            tape.n = 0;
            for (uint32_t i = 0; i < set.max_bounces; ++i) {
                Hit h;
                const bool found = closest<W, false>(S, ps.o, ps.d, INFINITY, h, C);
                NeeReq nr;
                const bool cont = shade_extended(S, set, C, i, ps, found, h, aov, nr, &tape);
                if (nr.kind != 0 && shadow_visible<W, false>(S, nr, C)) {
                    ps.L = add(ps.L, nr.c);
                    tape.nee(nr);
                }
                if (!cont) break;
            }
        }
    }
    if (C.err) atomicOr(S.err, C.err);
    if (use_shared) {
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < 3 * nmat; k += blockDim.x)
            if (sh[k] != 0.0) atomicAdd(&g_col[k], sh[k]);
        for (uint32_t k = threadIdx.x; k < nmat; k += blockDim.x)
            if (sh[3 * nmat + k] != 0.0) atomicAdd(&g_em[k], sh[3 * nmat + k]);
    }
}

} // namespace

crg_status launch_backward(crg_scene *s, const CamDev &cam, const crg_settings &set, const float *adj, double *g_col,
                           double *g_em, cudaStream_t st) {
    const SceneDev S = scene_dev(s);
    const uint32_t T = 128;
    const uint64_t npix = (uint64_t)set.width * set.height;
    const uint32_t blocks = (uint32_t)((npix + T - 1) / T);
    const size_t shmem = sizeof(double) * 4 * (size_t)s->nmat;
    const int use_shared = shmem <= 48 * 1024 ? 1 : 0;
    const size_t dyn = use_shared ? shmem : 0;
    switch (s->width) {
    case 2: k_adjoint<2><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, use_shared); break;
    case 4: k_adjoint<4><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, use_shared); break;
    default: k_adjoint<8><<<blocks, T, dyn, st>>>(S, cam, set, adj, g_col, g_em, s->nmat, use_shared); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(s->ctx, e, "k_adjoint launch");
    return CRG_OK;
}

} // namespace crg
