"""Textured materials in the oracle (process_hit's colour from image::get_uv,
src/render/renderer.cpp:30-35, src/objects/image.h:104-109): invariances that pin
the lookup without a GPU."""
import numpy as np

from crender_gb300 import api, scenes


def test_constant_texture_equals_material_colour(orc):
    """A 1x1 texture holding a material's colour renders bit-identically to the
    untextured material, in both estimators and with any texture coordinates."""
    sc = scenes.box_scene()
    tx = dict(sc, mats=sc["mats"].copy())
    tx["mats"]["tex"][[0, 3]] = [0, 1]
    tx["textures"] = [sc["mats"]["colour"][0][None, None, :], sc["mats"]["colour"][3][None, None, :]]
    tx["uvs"] = np.random.default_rng(1).uniform(-3, 3, (36, 6)).astype(np.float32)
    for mode in (0, 1):
        st = api.make_settings(24, 24, 2, 8, 3, mode, 3)
        a = orc.render(sc, sc["camera"], st)["sum"]
        b = orc.render(tx, tx["camera"], st)["sum"]
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), mode


def test_alpha_texture_equals_alpha_material(orc):
    """A texture whose alpha is zero everywhere makes a pass-through surface,
    exactly like a material with colour alpha 0 (renderer.cpp:37-41)."""
    sc = scenes.box_scene()
    alpha_mat = dict(sc, mats=sc["mats"].copy())
    alpha_mat["mats"]["colour"][2] = (0.14, 0.45, 0.09, 0.0)
    alpha_tex = dict(sc, mats=sc["mats"].copy())
    alpha_tex["mats"]["tex"][2] = 0
    alpha_tex["textures"] = [np.array([[[0.9, 0.1, 0.1, 0.0]]], np.float32)]
    st = api.make_settings(24, 24, 2, 8, 3, 0, 3)
    a = orc.render(alpha_mat, sc["camera"], st)["sum"]
    b = orc.render(alpha_tex, sc["camera"], st)["sum"]
    assert np.array_equal(a, b)


def test_textured_box_differs_and_is_finite(orc):
    sc = scenes.textured_box()
    st = api.make_settings(32, 32, 4, 8, 3, 1, 3)
    tex = orc.render(sc, sc["camera"], st)["sum"]
    plain = orc.render(scenes.box_scene(), sc["camera"], st)["sum"]
    assert np.isfinite(tex).all() and tex.sum() > 0
    assert not np.array_equal(tex, plain)
