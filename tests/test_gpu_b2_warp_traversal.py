"""The warp-cooperative traversal (crg_intersect_closest_with / _any_with,
CRG_TRAVERSAL_WARP: W lanes per ray, nodes staged in shared memory, per-ray
group stacks in the warp's shared memory) against the oracle and against the
per-thread traversal.

Bar: hits (t, primitive, u, v) bit-identical to the oracle's and to the
per-thread kernel's, occlusion flags identical, at BVH widths 2, 4 and 8 (the
group is W lanes), on random soups, the box scene's axis-aligned and coplanar
cases, a ragged ray count and the empty batch."""
import numpy as np
import pytest

from crender_gb300 import CrgError, _abi, api, scenes

pytestmark = pytest.mark.gpu

W = api.TRAVERSAL_WARP
T = api.TRAVERSAL_THREAD


def _same_hits(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("width,treelet,leaf_max", [(8, 0, 3), (8, 1, 1), (4, 1, 2), (2, 0, 1)])
def test_warp_matches_oracle_and_thread(ctx, orc, width, treelet, leaf_max):
    v = scenes.soup(20_000, 61)
    rays = scenes.soup_rays(65_536 + 37, 62)  # not a multiple of the rays per warp
    srays = scenes.soup_rays(65_536 + 37, 63, shadow=True)
    s = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build(width, treelet, leaf_max)
    try:
        gw = s.intersect(rays, traversal=W)
        gt = s.intersect(rays, traversal=T)
        aw = s.intersect(srays, any_hit=True, traversal=W)
        at = s.intersect(srays, any_hit=True, traversal=T)
    finally:
        s.close()
    b = orc.Bvh(v, width=width, treelet=treelet, leaf_max=leaf_max)
    o = b.closest(rays)
    assert (o["prim"] != 0xFFFFFFFF).mean() > 0.3
    assert _same_hits(gw, o), f"{int((gw['prim'] != o['prim']).sum())} prim mismatches"
    assert _same_hits(gw, gt)
    assert np.array_equal(aw, b.any(srays))
    assert np.array_equal(aw, at)


@pytest.mark.parametrize("width", [8, 4, 2])
def test_warp_box_scene_ties(ctx, orc, width):
    """Axis-aligned rays in the box scene and rays onto coplanar faces: the
    closest computed t, ties to the smaller primitive, as the brute force."""
    sc = scenes.box_scene()
    r = np.random.default_rng(71)
    n = 20_000
    rays = np.zeros(n, _abi.RAY_DTYPE)
    centre = np.where(r.uniform(size=n)[:, None] < 0.5, [0.68, 0.0, 0.33], [0.32, 0.0, 0.67])
    o = centre + np.stack([r.uniform(-0.1, 0.1, n), r.uniform(0.001, 0.2, n), r.uniform(-0.1, 0.1, n)], 1)
    d = np.stack([r.uniform(-1, 1, n), r.uniform(-1, -0.05, n), r.uniform(-1, 1, n)], 1)
    d[: n // 4, [0, 2]] = 0.0  # straight down
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["org"], rays["dir"], rays["tmin"], rays["tmax"] = o, d, 1e-5, np.inf
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(width, 1)
    try:
        g = s.intersect(rays, traversal=W)
        a = s.intersect(rays, any_hit=True, traversal=W)
    finally:
        s.close()
    ref = orc.closest_brute(sc["verts"], rays)
    assert _same_hits(g, ref)
    assert np.array_equal(a.astype(bool), ref["prim"] != 0xFFFFFFFF)


def test_warp_empty_and_invalid(ctx):
    v = scenes.soup(1_000, 81)
    s = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build(8, 0, 3)
    try:
        assert len(s.intersect(np.zeros(0, _abi.RAY_DTYPE), traversal=W)) == 0
        with pytest.raises(CrgError):
            s.intersect(scenes.soup_rays(16, 82), traversal=7)
    finally:
        s.close()


def test_warp_full_size_soup(ctx, orc):
    """The traversal microbench's workload: 1,048,576 triangles, 16M closest-hit
    and 16M shadow rays through both schemes, equal everywhere; a 65,536-ray
    subset against the oracle."""
    v = scenes.soup(1 << 20, 1)
    rays = scenes.soup_rays(1 << 24, 2)
    srays = scenes.soup_rays(1 << 24, 3, shadow=True)
    s = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build(8, 0, 3)
    try:
        gw = s.intersect(rays, traversal=W)
        gt = s.intersect(rays, traversal=T)
        aw = s.intersect(srays, any_hit=True, traversal=W)
        at = s.intersect(srays, any_hit=True, traversal=T)
    finally:
        s.close()
    assert _same_hits(gw, gt)
    assert np.array_equal(aw, at)
    idx = np.random.default_rng(19).choice(len(rays), 65_536, replace=False)
    assert _same_hits(gw[idx], orc.Bvh(v).closest(np.ascontiguousarray(rays[idx])))
