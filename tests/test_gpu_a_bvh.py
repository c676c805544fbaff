"""GPU LBVH build and wide collapse: bit-identical to the oracle's CPU run of
the same algorithm (binary tree, sorted order, wide nodes, triangle array),
and structurally valid (every index in range, every triangle once, quantized
boxes conservative)."""
import numpy as np
import pytest

import wide_bvh
from crender_gb300 import api, scenes

pytestmark = pytest.mark.gpu


def _mats():
    return scenes.material_table([{}])


CASES = {
    "box": lambda: scenes.box_scene()["verts"],
    "soup1": lambda: scenes.soup(1, 5),
    "soup2": lambda: scenes.soup(2, 5),
    "soup3": lambda: scenes.soup(3, 5),
    "soup7": lambda: scenes.soup(7, 5),
    "soup100": lambda: scenes.soup(100, 5),
    "soup4097": lambda: scenes.soup(4097, 6),
    "soup100k": lambda: scenes.soup(100_000, 7),
    "dupes": lambda: np.repeat(scenes.soup(50, 8), 40, axis=0),  # equal Morton codes, index tie-break
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("width,treelet,leaf_max", [(8, 0, 3), (8, 1, 3), (4, 0, 1), (2, 1, 2), (4, 1, 3), (8, 0, 1)])
def test_bvh_bit_exact(ctx, orc, name, width, treelet, leaf_max):
    v = np.ascontiguousarray(CASES[name]())
    n = v.shape[0]
    s = api.Scene(ctx, v, np.zeros(n, np.uint32), _mats()).build(width, treelet, leaf_max)
    try:
        gi = s.info()
        g = s.download_bvh()
    finally:
        s.close()
    o = orc.Bvh(v, width=width, treelet=treelet, leaf_max=leaf_max)
    oi = o.info()
    og = o.download()
    assert gi == oi
    for a, b, what in zip(g, og, ("bvh2", "order", "wide", "tris")):
        assert a.shape == b.shape, what
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"{what} differs from the oracle"
    assert wide_bvh.validate(g[2], g[3], width, n, v) == gi["depth"]


def test_treelets_lower_sah(ctx, orc):
    v = scenes.soup(50_000, 11)
    z = np.zeros(len(v), np.uint32)
    a = api.Scene(ctx, v, z, _mats()).build(8, 0)
    b = api.Scene(ctx, v, z, _mats()).build(8, 1)
    try:
        assert b.info()["sah_cost"] < a.info()["sah_cost"]
    finally:
        a.close()
        b.close()


def test_empty_scene_builds(ctx):
    s = api.Scene(ctx, np.zeros((0, 9), np.float32), np.zeros(0, np.uint32), _mats()).build()
    try:
        assert s.info()["n_wide_nodes"] == 0
        rays = scenes.soup_rays(100, 3)
        h = s.intersect(rays)
        assert (h["prim"] == 0xFFFFFFFF).all() and np.isinf(h["t"]).all()
        assert (s.intersect(rays, any_hit=True) == 0).all()
    finally:
        s.close()
