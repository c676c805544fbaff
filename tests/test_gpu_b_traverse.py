"""Closest-hit and any-hit traversal through the C ABI versus the oracle.

Bar: primitive ids, t, u, v bit-identical to the oracle's CPU traversal with
the same watertight test (ties at equal t go to the smaller primitive).  At the
full soup size (1,048,576 triangles, 16,777,216 + 16,777,216 rays) a seeded
65,536-ray subset is compared exactly, and every ray is checked against
size-independent properties (hit inside [tmin, tmax), occlusion == closest hit
before tmax)."""
import numpy as np
import pytest

from crender_gb300 import _abi, api, scenes

pytestmark = pytest.mark.gpu


def _scene(ctx, v, width=8, treelet=0, leaf_max=3):
    return api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build(width, treelet, leaf_max)


def _same_hits(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("width,treelet,leaf_max", [(8, 0, 3), (8, 1, 3), (4, 1, 2), (2, 0, 1)])
def test_closest_and_any_match_oracle(ctx, orc, width, treelet, leaf_max):
    v = scenes.soup(20_000, 21)
    rays = scenes.soup_rays(65_536, 22)
    srays = scenes.soup_rays(65_536, 23, shadow=True)
    s = _scene(ctx, v, width, treelet, leaf_max)
    try:
        g = s.intersect(rays)
        ga = s.intersect(srays, any_hit=True)
    finally:
        s.close()
    b = orc.Bvh(v, width=width, treelet=treelet, leaf_max=leaf_max)
    o = b.closest(rays)
    oa = b.any(srays)
    assert (o["prim"] != 0xFFFFFFFF).mean() > 0.3
    assert _same_hits(g, o), f"{int((g['prim'] != o['prim']).sum())} prim mismatches"
    assert np.array_equal(ga, oa)
    assert 0.05 < oa.mean() < 0.95


def test_matches_brute_force(ctx, orc):
    v = scenes.soup(2_000, 31)
    rays = scenes.soup_rays(8_192, 32)
    s = _scene(ctx, v)
    try:
        g = s.intersect(rays)
    finally:
        s.close()
    assert _same_hits(g, orc.closest_brute(v, rays))


def test_fp64_classification_of_mismatches(ctx, orc):
    """FP32 watertight hits versus an FP64 brute force: any primitive that
    differs must be an edge/vertex tie (hit within 1e-5 of an edge) or a
    t-tie within 1e-5 relative."""
    v = scenes.soup(2_000, 41)
    rays = scenes.soup_rays(8_192, 42)
    s = _scene(ctx, v)
    try:
        g = s.intersect(rays)
    finally:
        s.close()
    t64, p64, ed = orc.closest_f64(v, rays)
    diff = g["prim"] != p64
    for i in np.nonzero(diff)[0]:
        if p64[i] == 0xFFFFFFFF or g["prim"][i] == 0xFFFFFFFF:
            assert ed[i] < 1e-5 or not np.isfinite(t64[i])
        else:
            assert ed[i] < 1e-5 or abs(g["t"][i] - t64[i]) <= 1e-5 * t64[i]
    hit = (~diff) & (p64 != 0xFFFFFFFF)
    rel = np.abs(g["t"][hit].astype(np.float64) - t64[hit]) / t64[hit]
    assert rel.max() < 1e-5


def test_axis_aligned_and_box_scene(ctx, orc):
    sc = scenes.box_scene()
    v = sc["verts"]
    rng = np.random.default_rng(5)
    n = 20_000
    r = np.zeros(n, _abi.RAY_DTYPE)
    r["org"] = rng.uniform(0.05, 0.95, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d[: n // 4, :2] = 0.0  # rays along z
    d[n // 4: n // 2, 1:] = 0.0  # rays along x
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r["dir"] = d.astype(np.float32)
    r["tmin"] = 1e-5
    r["tmax"] = np.inf
    s = _scene(ctx, v)
    try:
        g = s.intersect(r)
        ga = s.intersect(r, any_hit=True)
    finally:
        s.close()
    b = orc.Bvh(v)
    assert _same_hits(g, b.closest(r))
    assert np.array_equal(ga, b.any(r))


def test_counted_traversal(ctx, orc):
    v = scenes.soup(20_000, 51)
    rays = scenes.soup_rays(4_096, 52)
    s = _scene(ctx, v)
    try:
        h, nodes, tris = s.intersect(rays, counted=True)
    finally:
        s.close()
    assert _same_hits(h, orc.Bvh(v).closest(rays))
    assert (nodes >= 1).all() and tris.sum() > 0


def test_full_size_soup(ctx, orc):
    """The traversal microbench workload itself: 1,048,576 triangles, 16M
    primary and 16M shadow rays."""
    v = scenes.soup(1 << 20, 1)
    rays = scenes.soup_rays(1 << 24, 2)
    srays = scenes.soup_rays(1 << 24, 3, shadow=True)
    s = _scene(ctx, v)
    try:
        g = s.intersect(rays)
        ga = s.intersect(srays, any_hit=True)
        # closest hit with the shadow rays' tmax gives the occlusion predicate too
        gs = s.intersect(srays)
    finally:
        s.close()
    hit = g["prim"] != 0xFFFFFFFF
    assert hit.mean() > 0.5
    assert (g["t"][hit] > 1e-5).all() and np.isinf(g["t"][~hit]).all()
    assert np.array_equal(ga.astype(bool), gs["prim"] != 0xFFFFFFFF)
    assert (gs["t"][ga.astype(bool)] < srays["tmax"][ga.astype(bool)]).all()
    idx = np.random.default_rng(9).choice(len(rays), 65_536, replace=False)
    b = orc.Bvh(v)
    assert _same_hits(g[idx], b.closest(np.ascontiguousarray(rays[idx])))
    assert np.array_equal(ga[idx], b.any(np.ascontiguousarray(srays[idx])))


@pytest.mark.parametrize("width,treelet", [(8, 0), (8, 1), (4, 1), (2, 0)])
def test_coplanar_faces_match_brute_force(ctx, orc, width, treelet):
    """Rays from inside the box scene's inner boxes toward the floor their bottom
    faces lie on: the closest computed t among coplanar triangles, as the brute
    force finds it, whatever the BVH."""
    sc = scenes.box_scene()
    r = np.random.default_rng(13)
    n = 20000
    rays = np.zeros(n, _abi.RAY_DTYPE)
    centre = np.where(r.uniform(size=n)[:, None] < 0.5, [0.68, 0.0, 0.33], [0.32, 0.0, 0.67])
    o = centre + np.stack([r.uniform(-0.1, 0.1, n), r.uniform(0.001, 0.2, n), r.uniform(-0.1, 0.1, n)], 1)
    d = np.stack([r.uniform(-1, 1, n), r.uniform(-1, -0.05, n), r.uniform(-1, 1, n)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["org"], rays["dir"], rays["tmin"], rays["tmax"] = o, d, 1e-5, np.inf
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(width, treelet)
    g = s.intersect(rays)
    s.close()
    assert _same_hits(g, orc.closest_brute(sc["verts"], rays))
