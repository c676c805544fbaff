"""Textured materials and per-corner texture coordinates through the C ABI
(crg_scene_create uvs + crg_scene_set_textures), against the oracle: colour from
the texture at the interpolated coordinate, alpha pass-through texels, a
textured emitter.  Bit-identical films, as for untextured scenes; the wavefront
form equals the megakernel."""
import numpy as np
import pytest

from crender_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def gpu_scene(ctx, sc):
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"], uvs=sc.get("uvs"))
    if sc.get("textures"):
        s.set_textures(sc["textures"])
    return s.build()


def render_gpu(ctx, sc, st, sun=False):
    s = gpu_scene(ctx, sc)
    if sun:
        s.set_sun(True)
    f = api.Film(ctx, st.width, st.height, f64=True, aov=True)
    api.render(s, sc["camera"], st, f)
    out = f.download(f64=True, aov=True)
    f.close()
    s.close()
    return out


@pytest.mark.parametrize("mode", [0, 1])
def test_textured_box_matches_oracle(ctx, orc, mode):
    sc = scenes.textured_box()
    st = api.make_settings(64, 48, 4, 8, 3, mode, 11, 64 / 48)
    g = render_gpu(ctx, sc, st)
    o = orc.render(sc, sc["camera"], st)
    for k in ("sum", "sum64", "sumsq64", "albedo", "normal", "depth"):
        assert np.array_equal(g[k].view(np.uint8), o[k].view(np.uint8)), k
    assert g["sum"].sum() > 0


def test_alpha_texels_let_the_sun_through(ctx, orc):
    """Faithful estimator with the sun on: shadow rays step through alpha-zero
    texels of the boxes (renderer.cpp:330-345)."""
    sc = scenes.textured_box()
    st = api.make_settings(48, 48, 4, 6, 0, 0, 2)
    g = render_gpu(ctx, sc, st, sun=True)
    o = orc.render(sc, sc["camera"], st, sun_enabled=True)
    assert np.array_equal(g["sum"].view(np.uint32), o["sum"].view(np.uint32))


def test_wavefront_equals_megakernel_with_textures(ctx):
    sc = scenes.textured_box()
    s = gpu_scene(ctx, sc)
    views = [(0, sc["camera"], api.make_settings(96, 64, 8, 8, 3, 1, 4, 1.5)),
             (0, sc["camera"], api.make_settings(40, 40, 16, 8, 3, 0, 5))]
    mega, wave = [], []
    for _, cam, st in views:
        f = api.Film(ctx, st.width, st.height)
        api.render(s, cam, st, f)
        mega.append(f.download()["sum"])
        f.close()
    films = [api.Film(ctx, st.width, st.height) for _, _, st in views]
    ctx.check(api.render_batch([s], views, films))
    wave = [f.download()["sum"] for f in films]
    for f in films:
        f.close()
    s.close()
    for a, b in zip(mega, wave):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_textures_replace_and_clear(ctx):
    sc = scenes.textured_box()
    s = gpu_scene(ctx, sc)
    st = api.make_settings(32, 32, 2, 8, 3, 1, 1)
    f = api.Film(ctx, 32, 32)
    api.render(s, sc["camera"], st, f)
    a = f.download()["sum"]
    s.set_textures([])  # materials fall back to their colours
    f.reset()
    api.render(s, sc["camera"], st, f)
    b = f.download()["sum"]
    assert not np.array_equal(a, b)
    lib = ctx.lib
    assert lib.crg_scene_set_textures(s.h, 1, None, None, None) == 1
    f.close()
    s.close()


def test_adjoint_rejects_textured_materials(ctx):
    sc = scenes.textured_box()
    s = gpu_scene(ctx, sc)
    st = api.make_settings(16, 16, 1, 4, 0, 1, 1)
    adj = api.DeviceBuffer(ctx, 16 * 16 * 12)
    gc, ge = api.DeviceBuffer(ctx, len(sc["mats"]) * 24), api.DeviceBuffer(ctx, len(sc["mats"]) * 8)
    cam = api.make_camera(sc["camera"])
    import ctypes as C

    rc = ctx.lib.crg_backward(s.h, C.byref(cam), C.byref(st), adj.ptr, gc.ptr, ge.ptr, None)
    assert rc == 6  # CRG_ERR_UNSUPPORTED
    for b in (adj, gc, ge):
        b.free()
    s.close()
