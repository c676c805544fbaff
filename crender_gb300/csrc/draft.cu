// draft.cu — draft-mode preview (sm_103a).
//
// cr::draft_renderer (CRender src/render/draft/draft_renderer.cpp:150-271)
// rasterises every mesh instance with OpenGL (assets/app/shaders/
// draft_mode.vert / .frag): no lighting, each fragment the material's flat
// colour, or its texture at the fragment's texture coordinate, over the
// skybox drawn by draft_mode_background.comp.  That image is primary
// visibility: the nearest surface at each pixel centre.  Here it is computed
// by one ray per pixel centre through the scene's resident BVH (instances
// included), with the rasteriser's near and far planes (0.1 and 10000 along
// the view axis; 0.01 for orthographic cameras) as the ray's extent, so no
// second copy of the geometry is kept for drawing.  The image has the film's
// pixel layout (both axes flipped, as crg_film_display), so a viewer can show
// either.  Colours are looked up like the path tracer's (nearest texel,
// modulo wrap) rather than with GL's filtering.
#include "render_common.cuh"

namespace crg {
using namespace rc;
namespace {

template <int W>
__global__ void __launch_bounds__(128) k_draft(SceneDev S, CamDev cam, uint32_t Wd, uint32_t Hd, float aspect,
                                               float4 *__restrict__ out) {
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= Wd * Hd) return;
    const uint32_t px = pix % Wd, py = pix / Wd;
    const float x = ((float)px + 0.5f) / (float)Wd;
    const float y = ((float)py + 0.5f) / (float)Hd;
    v3 o, d;
    camera_ray(cam, x, y, aspect, o, d);
    const float cz = dot(d, mk(cam.R[2], cam.R[5], cam.R[8]));
    const float zn = cam.mode == CRG_CAMERA_ORTHOGRAPHIC ? 0.01f : 0.1f;
    PathCtx C{pix, 0, 0, 0, 0, 0, 0ull, 0ull};
    Hit h;
    const bool found = cz > 0.0f && closest_t<W, false, true>(S, o, d, zn / cz, 10000.0f / cz, h, C);
    float4 c;
    if (found) {
        const HitGeom g = hit_geom<false>(S, h, o, d);
        const crg_material &m = S.mats[__ldg(&S.mat_idx[h.prim])];
        const float4 col = hit_colour(S, m, h.prim, h.slot, g.ro, g.rd);
        c = textured(S, m) ? col : make_float4(col.x, col.y, col.z, 1.0f);
    } else {
        const v3 e = sample_sky(S, d);
        c = make_float4(e.x, e.y, e.z, 1.0f);
    }
    out[(size_t)(Wd - 1 - px) + (size_t)(Hd - 1 - py) * Wd] = c;
    if (C.err) atomicOr(S.err, C.err);
}

} // namespace

crg_status launch_draft(crg_scene *s, const CamDev &cam, uint32_t w, uint32_t h, float aspect, float *d_rgba,
                        cudaStream_t st) {
    const SceneDev S = scene_dev(s);
    const uint64_t npix = (uint64_t)w * h;
    const uint32_t blocks = (uint32_t)((npix + 127) / 128);
    switch (s->width) {
    case 2: k_draft<2><<<blocks, 128, 0, st>>>(S, cam, w, h, aspect, (float4 *)d_rgba); break;
    case 4: k_draft<4><<<blocks, 128, 0, st>>>(S, cam, w, h, aspect, (float4 *)d_rgba); break;
    default: k_draft<8><<<blocks, 128, 0, st>>>(S, cam, w, h, aspect, (float4 *)d_rgba); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(s->ctx, e, "k_draft launch");
    return CRG_OK;
}

} // namespace crg
