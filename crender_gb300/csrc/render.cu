// render.cu — one-thread-per-pixel path-tracing megakernel (sm_103a).
//
// The drop-in for cr::renderer's sample passes (CRender
// src/render/renderer.cpp:116-144, 240-384): each thread owns one pixel,
// draws settings.spp samples in order and adds them to the pixel's FP32 sum
// (and optional FP64 sum / sum of squares) in that order, so the film is
// bit-identical to a sequential CPU accumulation of the same samples.
//
// FAITHFUL follows process_hit / _sample_pixel (renderer.cpp:21-102,
// 258-384): Lambert = normalize(Ng + uniform sphere point), mirror metal,
// Fresnel-less glass, emission folded into the throughput, optional sun NEE
// with the reference's colour-squared weight.  EXTENDED adds emissive-
// triangle NEE with power-heuristic MIS, GGX (VNDF sampling), Fresnel
// dielectric and Russian roulette; Lambert still scatters into the geometric
// normal's hemisphere as the reference does.
//
// Random dimension groups: 0 = pixel jitter, 1 + 2i = BSDF at segment i,
// 2 + 2i = light sample at segment i (pcg4d keyed by pixel/sample/group/seed).
#include <cmath>

#include "render_common.cuh"

namespace crg {

CamDev camera_params(const crg_camera &c) {
    CamDev p;
    for (int a = 0; a < 3; ++a) p.pos[a] = c.position[a];
    const double k = 3.14159265358979323846 / 180.0;
    const double ax = c.rotation[0] * k, ay = c.rotation[1] * k, az = c.rotation[2] * k;
    const double Ry[3][3] = {{std::cos(ax), 0, std::sin(ax)}, {0, 1, 0}, {-std::sin(ax), 0, std::cos(ax)}};
    const double Rx[3][3] = {{1, 0, 0}, {0, std::cos(ay), -std::sin(ay)}, {0, std::sin(ay), std::cos(ay)}};
    const double Rz[3][3] = {{std::cos(az), -std::sin(az), 0}, {std::sin(az), std::cos(az), 0}, {0, 0, 1}};
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            T[i][j] = 0;
            for (int m = 0; m < 3; ++m) T[i][j] += Ry[i][m] * Rx[m][j];
        }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double r = 0;
            for (int m = 0; m < 3; ++m) r += T[i][m] * Rz[m][j];
            p.R[3 * i + j] = (float)r;
        }
    p.w = (float)(1.0 / std::tan(0.5 * (double)c.fov * k));
    p.mode = c.mode;
    p.scale = c.scale;
    return p;
}

using namespace rc;

namespace {

// MINB blocks of 128 threads per SM: 5 (96 registers, some spilled) when the grid fills the
// GPU at that occupancy, else 4 (no spills: a grid below one wave gains nothing from the
// extra warps and loses the spill traffic).
// INST: the scene is traced through its placements (models and instances);
// kernels for plain one-mesh scenes are compiled without that code.
template <int W, int MODE, bool CNT, int MINB, bool INST>
__global__ void __launch_bounds__(128, MINB) k_render(SceneDev S, CamDev cam, crg_settings set, FilmDev F, uint64_t spp0) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t Wd = set.width, Hd = set.height;
    PathCtx C{pix, 0, set.seed, 0, 0, 0, 0ull, 0ull};
    uint32_t lanes = __ballot_sync(0xFFFFFFFFu, pix < Wd * Hd);
    if (pix < Wd * Hd) {
        const uint32_t px = pix % Wd, py = pix / Wd;
        const size_t fidx = (size_t)(Wd - 1 - px) + (size_t)(Hd - 1 - py) * Wd;
        float acc[3] = {F.sum[fidx * 3], F.sum[fidx * 3 + 1], F.sum[fidx * 3 + 2]};
        double a64[3] = {0, 0, 0}, q64[3] = {0, 0, 0};
        if (F.sum64) {
            a64[0] = F.sum64[fidx * 3]; a64[1] = F.sum64[fidx * 3 + 1]; a64[2] = F.sum64[fidx * 3 + 2];
            q64[0] = F.sumsq64[fidx * 3]; q64[1] = F.sumsq64[fidx * 3 + 1]; q64[2] = F.sumsq64[fidx * 3 + 2];
        }
        Aov aov;
        PathState ps;
        // Path regeneration (Novak, Havran and Dachsbacher 2010): one loop over
        // segments, in which a lane whose path has ended starts its pixel's next
        // sample, so a warp runs for the largest total segment count of its lanes
        // instead of the longest path of every sample.  A pixel's samples still run
        // and accumulate in order, so the film is unchanged.
        uint32_t s = 0, i = 0;
        for (;;) {
            // the lanes still rendering meet here before every segment, so the warp
            // enters each segment's traversal together
            lanes = __ballot_sync(lanes, s < set.spp);
            if (s >= set.spp) break;
            if (i == 0) {
                C.sample = (uint32_t)(spp0 + s);
                const f4 g0 = rand4(pix, C.sample, 0, set.seed);
                const float x = ((float)px + g0.x) / (float)Wd;
                const float y = ((float)py + g0.y) / (float)Hd;
                v3 o, d;
                camera_ray(cam, x, y, set.aspect, o, d);
                aov.albedo = mk(0, 0, 0);
                aov.normal = mk(0, 0, 0);
                aov.depth = 0.0f;
                path_start(ps, o, d);
            }
            if (i < set.max_bounces) {
                Hit h;
                C.segments++;
                const bool found = closest<W, CNT, INST>(S, ps.o, ps.d, INFINITY, h, C);
                NeeReq nr;
                const bool cont = MODE == CRG_MODE_EXTENDED ? shade_extended(S, set, C, i, ps, found, h, aov, nr)
                                                            : shade_faithful(S, set, C, i, ps, found, h, aov, nr);
                if (nr.kind != 0 && shadow_visible<W, CNT, INST>(S, nr, C)) ps.L = add(ps.L, nr.c);
                ++i;
                if (cont && i < set.max_bounces) continue;
            }
            ++s;
            i = 0;
            const v3 L = ps.L;
            acc[0] += L.x;
            acc[1] += L.y;
            acc[2] += L.z;
            if (F.sum64) {
                a64[0] += (double)L.x; a64[1] += (double)L.y; a64[2] += (double)L.z;
                q64[0] += (double)L.x * (double)L.x;
                q64[1] += (double)L.y * (double)L.y;
                q64[2] += (double)L.z * (double)L.z;
            }
        }
        F.sum[fidx * 3] = acc[0];
        F.sum[fidx * 3 + 1] = acc[1];
        F.sum[fidx * 3 + 2] = acc[2];
        if (F.sum64) {
            F.sum64[fidx * 3] = a64[0]; F.sum64[fidx * 3 + 1] = a64[1]; F.sum64[fidx * 3 + 2] = a64[2];
            F.sumsq64[fidx * 3] = q64[0]; F.sumsq64[fidx * 3 + 1] = q64[1]; F.sumsq64[fidx * 3 + 2] = q64[2];
        }
        if (F.aov_albedo && set.spp > 0) {
            reinterpret_cast<float4 *>(F.aov_albedo)[fidx] = make_float4(aov.albedo.x, aov.albedo.y, aov.albedo.z, 1.0f);
            reinterpret_cast<float4 *>(F.aov_normal)[fidx] =
                make_float4(aov.normal.x * 0.5f + 0.5f, aov.normal.y * 0.5f + 0.5f, aov.normal.z * 0.5f + 0.5f, 1.0f);
            const float dv = mn(aov.depth, 200.0f) / 200.0f;
            reinterpret_cast<float4 *>(F.aov_depth)[fidx] = make_float4(dv, dv, dv, 1.0f);
        }
    }
    if (C.err) atomicOr(S.err, C.err);
    if (CNT) {
        unsigned long long seg = C.segments, sh = C.shadow, nd = C.nodes, tr = C.tris;
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            seg += __shfl_xor_sync(0xFFFFFFFFu, seg, off);
            sh += __shfl_xor_sync(0xFFFFFFFFu, sh, off);
            nd += __shfl_xor_sync(0xFFFFFFFFu, nd, off);
            tr += __shfl_xor_sync(0xFFFFFFFFu, tr, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&S.counters[1], seg);
            atomicAdd(&S.counters[2], sh);
            atomicAdd(&S.counters[3], nd);
            atomicAdd(&S.counters[4], tr);
        }
    }
}

template <int W, int MINB, bool INST>
void launch_m(const SceneDev &S, const CamDev &cam, const crg_settings &set, const FilmDev &F, uint64_t spp0,
              uint32_t blocks, cudaStream_t st) {
    const uint32_t T = 128;
    if (S.counters) {
        if (set.mode == CRG_MODE_EXTENDED) k_render<W, CRG_MODE_EXTENDED, true, MINB, INST><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
        else k_render<W, CRG_MODE_FAITHFUL, true, MINB, INST><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
    } else {
        if (set.mode == CRG_MODE_EXTENDED) k_render<W, CRG_MODE_EXTENDED, false, MINB, INST><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
        else k_render<W, CRG_MODE_FAITHFUL, false, MINB, INST><<<blocks, T, 0, st>>>(S, cam, set, F, spp0);
    }
}

template <int W>
void launch_w(const SceneDev &S, const CamDev &cam, const crg_settings &set, const FilmDev &F, uint64_t spp0,
              int sm_count, cudaStream_t st) {
    const uint64_t npix = (uint64_t)set.width * set.height;
    const uint32_t blocks = (uint32_t)((npix + 127) / 128);
    if (S.ninst > kLoopPlacements) launch_m<W, 4, true>(S, cam, set, F, spp0, blocks, st); // the top-level tree
    else if ((uint64_t)blocks >= 5ull * (uint64_t)(sm_count > 0 ? sm_count : 1)) launch_m<W, 5, false>(S, cam, set, F, spp0, blocks, st);
    else launch_m<W, 4, false>(S, cam, set, F, spp0, blocks, st);
}

} // namespace

namespace {
// Emitter records (see SceneDev::light_rec), built once per emitter table with
// the same device arithmetic the NEE sample would otherwise repeat per path.
__global__ void k_light_records(SceneDev S, float4 *__restrict__ rec) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= S.nlights) return;
    const uint32_t prim = S.light_prim[j];
    v3 a, b, c;
    prim_verts(S, prim, a, b, c);
    if (S.ninst) {
        const float4 *F = S.inst + 6 * (size_t)S.light_inst[j] + 3;
        a = xf_point(F, a);
        b = xf_point(F, b);
        c = xf_point(F, c);
    }
    const uint32_t mi = S.mat_idx[prim];
    const crg_material &m = S.mats[mi];
    float4 *r = rec + 4 * (size_t)j;
    r[0] = make_float4(a.x, a.y, a.z, S.light_pdf[j]);
    r[1] = make_float4(b.x, b.y, b.z, __uint_as_float(prim));
    r[2] = make_float4(c.x, c.y, c.z, __uint_as_float(mi));
    r[3] = make_float4(m.colour[0] * m.emission, m.colour[1] * m.emission, m.colour[2] * m.emission,
                       __uint_as_float(textured(S, m) ? 1u : 0u));
}

} // namespace

// Builds the emitter records of a scene's current emitter table (call after the
// table, the materials, the textures or the instances change).
crg_status build_light_records(crg_scene *s) {
    if (s->nlights == 0) return CRG_OK;
    crg_status rc = dev_alloc(s->ctx, s->light_rec, 64 * (size_t)s->nlights);
    if (rc != CRG_OK) return rc;
    const SceneDev S = scene_dev(s);
    k_light_records<<<(s->nlights + 127) / 128, 128>>>(S, (float4 *)s->light_rec.ptr);
    CRG_CUDA(s->ctx, cudaGetLastError());
    CRG_CUDA(s->ctx, cudaDeviceSynchronize());
    return CRG_OK;
}

namespace rc {
SceneDev scene_dev(const crg_scene *s) {
    SceneDev S{};
    S.nodes = (const uint4 *)s->wide.ptr;
    S.tris = (const float4 *)s->tris.ptr;
    S.mat_idx = (const uint32_t *)s->mat_idx.ptr;
    S.mats = (const crg_material *)s->mats.ptr;
    S.light_prim = (const uint32_t *)s->light_prim.ptr;
    S.light_alias = (const float2 *)s->light_alias.ptr;
    S.light_pdf = (const float *)s->light_pdf.ptr;
    S.mat_light_pdf = (const float *)s->mat_light_pdf.ptr;
    S.verts = (const float *)s->verts.ptr;
    S.uvs = (const float *)s->uvs.ptr;
    S.texels = (const float4 *)s->texels.ptr;
    S.tex_info = (const uint4 *)s->tex_info.ptr;
    S.ntex = s->texels.ptr ? s->ntex : 0;
    S.inst = (const float4 *)s->inst.ptr;
    S.inst_root = (const uint32_t *)s->inst_root.ptr;
    S.tlas = (const float4 *)s->tlas.ptr;
    S.tlas_root = s->tlas_root;
    S.light_inst = (const uint32_t *)s->light_inst.ptr;
    S.light_rec = (const float4 *)s->light_rec.ptr;
    S.ninst = s->inst.ptr ? s->ninst : 0;
    S.nlights = s->nlights;
    S.ntri = s->ntri;
    S.sky = (const float4 *)s->sky.ptr;
    S.sky_w = s->sky.ptr ? s->sky_w : 0;
    S.sky_h = s->sky_h;
    S.sky_rot_u = s->sky_rot_u;
    S.sky_rot_v = s->sky_rot_v;
    S.sun_on = s->sun_enabled;
    for (int k = 0; k < 9; ++k) S.sun_frame[k] = s->sun_frame[k];
    S.sun_cos = s->sun_cos;
    S.sun_pdf = s->sun_pdf;
    for (int k = 0; k < 3; ++k) {
        S.sun_neg_dir[k] = -s->sun.direction[k];
        S.sun_rad[k] = s->sun.colour[k] * s->sun.intensity;
    }
    S.err = (uint32_t *)s->err.ptr;
    S.counters = s->counting ? (unsigned long long *)s->counters.ptr : nullptr;
    return S;
}
} // namespace rc

crg_status launch_render(crg_scene *s, const CamDev &cam, const crg_settings &set, crg_film *film, cudaStream_t st) {
    const SceneDev S = scene_dev(s);
    FilmDev F{(float *)film->sum.ptr,
              (double *)film->sum64.ptr,
              (double *)film->sumsq64.ptr,
              (float *)film->aov_albedo.ptr,
              (float *)film->aov_normal.ptr,
              (float *)film->aov_depth.ptr,
              film->width,
              film->height};
    if (s->ntri == 0) return set_error(s->ctx, CRG_ERR_INVALID_ARG, "crg_render: scene has no triangles");
    switch (s->width) {
    case 2: launch_w<2>(S, cam, set, F, film->spp, s->ctx->sm_count, st); break;
    case 4: launch_w<4>(S, cam, set, F, film->spp, s->ctx->sm_count, st); break;
    default: launch_w<8>(S, cam, set, F, film->spp, s->ctx->sm_count, st); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(s->ctx, e, "k_render launch");
    return CRG_OK;
}

} // namespace crg
