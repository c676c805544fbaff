"""Instances (crg_scene_set_instances: cr::entity::instances::transforms and the
per-instance loop of cr::model::intersect, src/objects/model.cpp:99-126) through
the C ABI, against the oracle's literal restatement of that loop (every
instance traced to infinity; the GPU prunes by the best world distance):
queries, faithful / extended renders with AOVs, the wavefront form and the
adjoint."""
import numpy as np
import pytest

from crender_gb300 import api, scenes
from test_instances_cpu import random_rays

pytestmark = pytest.mark.gpu


def gpu_scene(ctx, sc, width=8):
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(width, 1)
    s.set_instances(sc["instances"])
    return s


@pytest.mark.parametrize("width", [2, 4, 8])
def test_queries_match_oracle(ctx, orc, width):
    sc = scenes.instanced_box()
    s = gpu_scene(ctx, sc, width)
    rays = random_rays(20000, 9)
    rays["tmin"][::7] = 0.05
    g = s.intersect(rays)
    o = orc.scene_intersect(sc, rays)
    for k in ("t", "prim", "u", "v"):
        assert np.array_equal(g[k].view(np.uint32), o[k].view(np.uint32)), k
    sh = rays.copy()
    sh["tmax"] = np.where(np.isfinite(o["t"]), o["t"] * np.float32(0.999), 20.0)
    assert np.array_equal(s.intersect(sh, any_hit=True), orc.scene_intersect(sc, sh, any_hit=True))
    s.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_render_matches_oracle(ctx, orc, mode):
    sc = scenes.instanced_box()
    s = gpu_scene(ctx, sc)
    st = api.make_settings(64, 40, 4, 8, 3, mode, 21, 1.6)
    f = api.Film(ctx, st.width, st.height, f64=True, aov=True)
    api.render(s, sc["camera"], st, f)
    g = f.download(f64=True, aov=True)
    o = orc.render(sc, sc["camera"], st)
    for k in ("sum", "sum64", "sumsq64", "albedo", "normal", "depth"):
        assert np.array_equal(g[k].view(np.uint8), o[k].view(np.uint8)), k
    assert g["sum"].sum() > 0
    f.close()
    s.close()


def test_faithful_sun_through_instances(ctx, orc):
    sc = scenes.instanced_box()
    s = gpu_scene(ctx, sc)
    s.set_sun(True)
    st = api.make_settings(48, 32, 2, 6, 0, 0, 5, 1.5)
    f = api.Film(ctx, st.width, st.height)
    api.render(s, sc["camera"], st, f)
    g = f.download()["sum"]
    o = orc.render(sc, sc["camera"], st, sun_enabled=True)["sum"]
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    f.close()
    s.close()


def test_wavefront_equals_megakernel(ctx):
    sc = scenes.instanced_box()
    s = gpu_scene(ctx, sc)
    views = [(0, sc["camera"], api.make_settings(80, 48, 8, 8, 3, 1, 3, 80 / 48)),
             (0, sc["camera"], api.make_settings(32, 32, 4, 8, 3, 0, 4))]
    mega = []
    for _, cam, st in views:
        f = api.Film(ctx, st.width, st.height)
        api.render(s, cam, st, f)
        mega.append(f.download()["sum"])
        f.close()
    for fuse in (1, 2, 3):
        films = [api.Film(ctx, st.width, st.height) for _, _, st in views]
        ctx.check(api.render_batch([s], views, films, dict(fuse=fuse)))
        for f, m in zip(films, mega):
            assert np.array_equal(f.download()["sum"].view(np.uint32), m.view(np.uint32)), fuse
            f.close()
    s.close()


def test_wavefront_refill_through_placements_in_a_mixed_batch(ctx):
    """A scene of three placements (the loop, with per-lane refill) beside a
    one-mesh scene in one batch: every refill threshold and fusion level gives
    the megakernel's films."""
    sc, box = scenes.instanced_box(), scenes.box_scene()
    s = gpu_scene(ctx, sc)
    b = api.Scene(ctx, box["verts"], box["mat_idx"], box["mats"]).build(8, 1)
    views = [(0, sc["camera"], api.make_settings(64, 40, 8, 8, 3, 1, 7, 64 / 40)),
             (1, box["camera"], api.make_settings(40, 40, 4, 8, 3, 1, 8)),
             (0, sc["camera"], api.make_settings(24, 24, 4, 8, 3, 0, 9))]
    mega = []
    for si, cam, st in views:
        f = api.Film(ctx, st.width, st.height)
        api.render((s, b)[si], cam, st, f)
        mega.append(f.download()["sum"])
        f.close()
    try:
        for fuse, refill in ((1, 4), (1, 16), (1, 32), (2, 8)):
            films = [api.Film(ctx, st.width, st.height) for _, _, st in views]
            ctx.check(api.render_batch([s, b], views, films, dict(fuse=fuse, refill=refill)))
            for f, m in zip(films, mega):
                assert np.array_equal(f.download()["sum"].view(np.uint32), m.view(np.uint32)), (fuse, refill)
                f.close()
    finally:
        s.close()
        b.close()


def test_adjoint_matches_oracle(ctx, orc):
    sc = scenes.instanced_box()
    s = gpu_scene(ctx, sc)
    W, nmat = 24, len(sc["mats"])
    st = api.make_settings(W, W, 8, 8, 3, 1, 13)
    adj = np.random.default_rng(2).uniform(-1, 1, W * W * 3).astype(np.float32)
    ab = api.DeviceBuffer.from_array(ctx, adj)
    gc = api.DeviceBuffer.from_array(ctx, np.zeros(nmat * 3))
    ge = api.DeviceBuffer.from_array(ctx, np.zeros(nmat))
    api.backward(s, sc["camera"], st, ab, gc, ge)
    g_c = gc.download(np.zeros(nmat * 3)).reshape(nmat, 3)
    g_e = ge.download(np.zeros(nmat))
    oc, oe = orc.adjoint(sc, sc["camera"], st, adj)
    assert np.abs(oc).max() > 0
    assert np.allclose(g_c, oc, rtol=1e-9, atol=1e-12 * np.abs(oc).max())
    assert np.allclose(g_e, oe, rtol=1e-9, atol=1e-12 * np.abs(oe).max())
    for b in (ab, gc, ge):
        b.free()
    s.close()


def test_instances_validate_and_clear(ctx):
    sc = scenes.box_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build()
    bad = np.eye(4, dtype=np.float32)[None].copy()
    bad[0, 3, 0] = 0.5  # projective row
    with pytest.raises(Exception):
        s.set_instances(bad)
    with pytest.raises(Exception):
        s.set_instances(np.zeros((1, 4, 4), np.float32))  # singular
    rays = random_rays(2000, 3)
    plain = s.intersect(rays)
    s.set_instances(np.stack([scenes.affine((0.0, 0.0, 2.0))]))
    moved = s.intersect(rays)
    assert not np.array_equal(plain["prim"], moved["prim"])
    s.set_instances(None)
    assert np.array_equal(s.intersect(rays).view(np.uint8), plain.view(np.uint8))
    s.close()
