"""Scenes of several models through the C ABI (crg_scene_add_model,
crg_scene_set_model_instances): every model its own BVH and instance list,
traced through the top-level tree over the placements.  Checked bit for bit
against the oracle, which runs cr::scene::cast_ray's loop over entities
(src/render/scene.cpp:79-98) around cr::model::intersect's loop over
instances (src/objects/model.cpp:99-126) literally, with every model's own
BVH: queries (ties between models included), faithful and extended renders
with AOVs, the wavefront form, the adjoint, the draft preview, each model's
BVH layout, and a model added to a built scene."""
import numpy as np
import pytest

from crender_gb300 import _abi, api, scenes
from test_instances_cpu import random_rays

pytestmark = pytest.mark.gpu


def gpu_scene(ctx, sc, width=8, treelet=1):
    return api.Scene.from_models(ctx, sc).build(width, treelet)


@pytest.mark.parametrize("width", [2, 4, 8])
def test_queries_match_oracle(ctx, orc, width):
    sc = scenes.multi_model_box(duplicate=True)
    s = gpu_scene(ctx, sc, width)
    assert s.model_count() == 4
    rays = random_rays(20000, 19)
    rays["org"][:, 2] = -1.4
    rays["tmin"][::7] = 0.05
    g = s.intersect(rays)
    o = orc.scene_intersect(sc, rays)
    assert np.sum(o["prim"] != 0xFFFFFFFF) > 5000
    for k in ("t", "prim", "u", "v"):
        assert np.array_equal(g[k].view(np.uint32), o[k].view(np.uint32)), k
    sh = rays.copy()
    sh["tmax"] = np.where(np.isfinite(o["t"]), o["t"] * np.float32(0.999), 20.0)
    assert np.array_equal(s.intersect(sh, any_hit=True), orc.scene_intersect(sc, sh, any_hit=True))
    s.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_render_matches_oracle(ctx, orc, mode):
    sc = scenes.multi_model_box()
    s = gpu_scene(ctx, sc)
    st = api.make_settings(64, 48, 4, 8, 3, mode, 23, 64 / 48)
    f = api.Film(ctx, st.width, st.height, f64=True, aov=True)
    api.render(s, sc["camera"], st, f)
    g = f.download(f64=True, aov=True)
    o = orc.render(sc, sc["camera"], st)
    for k in ("sum", "sum64", "sumsq64", "albedo", "normal", "depth"):
        assert np.array_equal(g[k].view(np.uint8), o[k].view(np.uint8)), k
    assert g["sum"].sum() > 0
    f.close()
    s.close()


def test_faithful_sun_through_models(ctx, orc):
    sc = scenes.multi_model_box()
    s = gpu_scene(ctx, sc)
    s.set_sun(True)
    st = api.make_settings(40, 32, 2, 6, 0, 0, 5, 1.25)
    f = api.Film(ctx, st.width, st.height)
    api.render(s, sc["camera"], st, f)
    g = f.download()["sum"]
    o = orc.render(sc, sc["camera"], st, sun_enabled=True)["sum"]
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    f.close()
    s.close()


def test_wavefront_equals_megakernel_in_a_mixed_batch(ctx):
    """A batch over a multi-model scene and the plain box scene: the placements'
    split kernels and the one-mesh scene's views in one launch."""
    sc, box = scenes.multi_model_box(), scenes.box_scene()
    s = gpu_scene(ctx, sc)
    b = api.Scene(ctx, box["verts"], box["mat_idx"], box["mats"]).build(8, 1)
    views = [(0, sc["camera"], api.make_settings(72, 48, 8, 8, 3, 1, 3, 72 / 48)),
             (1, box["camera"], api.make_settings(40, 40, 4, 8, 3, 1, 4)),
             (0, sc["camera"], api.make_settings(32, 32, 4, 8, 3, 0, 5))]
    mega = []
    for si, cam, st in views:
        f = api.Film(ctx, st.width, st.height)
        api.render((s, b)[si], cam, st, f)
        mega.append(f.download()["sum"])
        f.close()
    # six placements: the top-level tree, walked per lane by the refill kernels (and the static fetch)
    for fuse, refill in ((1, 16), (1, 4), (1, 32), (1, 0xFFFFFFFF), (3, 16)):
        films = [api.Film(ctx, st.width, st.height) for _, _, st in views]
        ctx.check(api.render_batch([s, b], views, films, dict(fuse=fuse, refill=refill)))
        for f, m in zip(films, mega):
            assert np.array_equal(f.download()["sum"].view(np.uint32), m.view(np.uint32)), (fuse, refill)
            f.close()
    s.close()
    b.close()


def test_adjoint_matches_oracle(ctx, orc):
    sc = scenes.multi_model_box()
    s = gpu_scene(ctx, sc)
    W, nmat = 24, len(sc["mats"])
    st = api.make_settings(W, W, 8, 8, 3, 1, 17)
    adj = np.random.default_rng(3).uniform(-1, 1, W * W * 3).astype(np.float32)
    ab = api.DeviceBuffer.from_array(ctx, adj)
    gc = api.DeviceBuffer.from_array(ctx, np.zeros(nmat * 3))
    ge = api.DeviceBuffer.from_array(ctx, np.zeros(nmat))
    api.backward(s, sc["camera"], st, ab, gc, ge)
    g_c = gc.download(np.zeros(nmat * 3)).reshape(nmat, 3)
    g_e = ge.download(np.zeros(nmat))
    oc, oe = orc.adjoint(sc, sc["camera"], st, adj)
    assert np.abs(oc).max() > 0 and np.abs(oe).max() > 0
    assert np.allclose(g_c, oc, rtol=1e-9, atol=1e-12 * np.abs(oc).max())
    assert np.allclose(g_e, oe, rtol=1e-9, atol=1e-12 * np.abs(oe).max())
    for buf in (ab, gc, ge):
        buf.free()
    s.close()


def test_draft_matches_oracle(ctx, orc):
    sc = scenes.multi_model_box()
    s = gpu_scene(ctx, sc)
    W, H = 48, 32
    dst = api.DeviceBuffer(ctx, W * H * 16)
    api.draft_render(s, sc["camera"], W, H, dst, 1.5)
    g = dst.download(np.zeros(W * H * 4, np.float32))
    o = orc.draft_render(sc, sc["camera"], W, H, 1.5)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    dst.free()
    s.close()


def _model_layout(s, m):
    """Model m's wide nodes, triangle slots and order from the scene arrays, with
    scene-wide indices turned back into model-local ones."""
    i, mi = s.info(), s.model_info(m)
    _, order, wide, tris = s.download_bvh()
    nb = i["node_bytes"]
    w = wide[mi["node_base"] * nb:(mi["node_base"] + mi["n_wide_nodes"]) * nb].copy().view(np.uint32).reshape(-1, nb // 4)
    w[:, 4] -= np.uint32(mi["node_base"])
    w[:, 5] -= np.uint32(mi["first_prim"])
    t = tris[mi["first_prim"]:mi["first_prim"] + mi["ntri"]].copy()
    tp = t[:, 3].view(np.uint32)
    tp -= np.uint32(mi["first_prim"])
    return w.view(np.uint8).ravel(), t, order[mi["first_prim"]:mi["first_prim"] + mi["ntri"]]


def test_each_model_bvh_equals_its_own_build_and_adding_a_model_keeps_the_others(ctx, orc):
    sc = scenes.multi_model_box()
    ms = sc["models"]
    s = api.Scene(ctx, ms[0]["verts"], ms[0]["mat_idx"], ms[0]["mats"])
    s.add_model(ms[1]["verts"], ms[1]["mat_idx"], ms[1]["mats"])
    s.build(8, 1, 2)
    before = [_model_layout(s, m) for m in range(2)]
    k = s.add_model(ms[2]["verts"], ms[2]["mat_idx"], ms[2]["mats"])
    assert k == 2
    assert s.model_info(2)["built"] == 0 and s.model_info(0)["built"] == 1
    with pytest.raises(Exception):
        s.intersect(random_rays(8, 1))  # not built since the model was added
    s.build(8, 1, 2)
    for m in range(3):
        w, t, order = _model_layout(s, m)
        ob = orc.Bvh(ms[m]["verts"], 8, 1, 2)
        _, oorder, owide, otris = ob.download()
        assert np.array_equal(w, owide), m
        assert np.array_equal(t.view(np.uint32), otris.view(np.uint32)), m
        assert np.array_equal(order, oorder), m
        if m < 2:
            assert np.array_equal(w, before[m][0]) and np.array_equal(t.view(np.uint32), before[m][1].view(np.uint32))
    s.close()


def test_model_instances_validate_and_clear(ctx):
    sc = scenes.multi_model_box()
    s = gpu_scene(ctx, sc)
    with pytest.raises(Exception):
        s.set_model_instances(7, np.eye(4, dtype=np.float32)[None])  # no such model
    with pytest.raises(Exception):
        s.set_model_instances(1, np.zeros((1, 4, 4), np.float32))  # singular
    rays = random_rays(3000, 5)
    rays["org"][:, 2] = -1.4
    a = s.intersect(rays)
    s.set_model_instances(1, None)  # model 1 back to one identity instance
    b = s.intersect(rays)
    assert not np.array_equal(a["prim"], b["prim"])
    s.set_model_instances(1, sc["models"][1]["instances"])
    assert np.array_equal(s.intersect(rays).view(np.uint8), a.view(np.uint8))
    assert s.model_info(1)["ninst"] == 3
    s.close()
