"""CPU checks of the oracle: known answers, independent restatements, golden
fixtures, and estimator cross-checks.  The reference ships no tests or golden
vectors and cannot be built here, so parity with the reference itself is
unpinned; these pin the oracle's own semantics."""
import ctypes as C
import math
import os

import numpy as np
import pytest

import wide_bvh
from golden import make_golden
from crender_gb300 import _abi, api, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")


def pcg4d_py(v):
    """Independent Python restatement of pcg4d (Jarzynski & Olano 2020)."""
    M = 0xFFFFFFFF
    x, y, z, w = [(a * 1664525 + 1013904223) & M for a in v]
    x = (x + y * w) & M; y = (y + z * x) & M; z = (z + x * y) & M; w = (w + y * z) & M
    x ^= x >> 16; y ^= y >> 16; z ^= z >> 16; w ^= w >> 16
    x = (x + y * w) & M; y = (y + z * x) & M; z = (z + x * y) & M; w = (w + y * z) & M
    return [(h >> 8) / 16777216.0 for h in (x, y, z, w)]


def test_golden_fixtures_reproduce(orc):
    g = np.load(GOLDEN)
    r = np.zeros(4, np.float32)
    for row in g["rng"]:
        key = [int(k) for k in row[:4]]
        orc.lib().orc_rand4(*key, r.ctypes.data)
        assert np.array_equal(r, row[4:].astype(np.float32))
        assert pcg4d_py(key) == pytest.approx(row[4:].tolist(), abs=0)
    v = g["soup500"]
    for W, tl in ((8, 0), (8, 1), (4, 1), (2, 0)):
        bvh2, order, wide, tris = orc.Bvh(v, width=W, treelet=tl).download()
        assert np.array_equal(wide, g[f"bvh_w{W}_t{tl}_wide"])
        assert np.array_equal(order, g[f"bvh_w{W}_t{tl}_order"])
        assert np.array_equal(bvh2.view(np.uint32), g[f"bvh_w{W}_t{tl}_bvh2"].view(np.uint32))
    rays = g["rays512"].view(_abi.RAY_DTYPE)
    assert np.array_equal(orc.Bvh(v).closest(rays).view(np.uint8), g["hits512"])
    sc = scenes.box_scene()
    for mode, rr in ((0, 0), (1, 3)):
        f = orc.render(sc, sc["camera"], api.make_settings(16, 16, 4, 8, rr, mode, 42))
        assert np.array_equal(f["sum"].view(np.uint32), g[f"box16_mode{mode}_sum"].view(np.uint32))
        assert np.array_equal(f["sum64"].view(np.uint64), g[f"box16_mode{mode}_sum64"].view(np.uint64))
    tx, inst = scenes.textured_box(), scenes.instanced_box()
    for mode in (0, 1):
        st = api.make_settings(16, 12, 4, 8, 3, mode, 43, 16 / 12)
        for name, s in (("textured16", tx), ("instanced16", inst)):
            f = orc.render(s, s["camera"], st)
            assert np.array_equal(f["sum"].view(np.uint32), g[f"{name}_mode{mode}_sum"].view(np.uint32)), name
    d = orc.draft_render(tx, tx["camera"], 24, 16, 1.5)
    assert np.array_equal(d.view(np.uint32), g["draft_textured_24x16"].view(np.uint32))
    for name, kw in make_golden.POST_CASES.items():
        p = orc.post_process(g["post_input"], api.post_settings(**kw))
        assert np.array_equal(p.view(np.uint32), g[f"post_{name}"].view(np.uint32)), name


def test_sincos2pi_accuracy(orc):
    u = np.concatenate([np.linspace(0, 1, 100_001, dtype=np.float32), np.float32([0.125, 0.25, 0.375, 0.5, 0.75])])
    s, c = C.c_float(), C.c_float()
    err = 0.0
    for x in u[::7]:
        orc.lib().orc_sincos2pi(float(x), C.byref(s), C.byref(c))
        err = max(err, abs(s.value - math.sin(2 * math.pi * float(x))), abs(c.value - math.cos(2 * math.pi * float(x))))
    assert err < 3e-7
    orc.lib().orc_sincos2pi(0.25, C.byref(s), C.byref(c))
    assert s.value == 1.0 and abs(c.value) < 1e-7


def test_rng_uniform(orc):
    r = np.zeros(4, np.float32)
    vals = []
    for i in range(20_000):
        orc.lib().orc_rand4(i % 977, i // 977, 3, 1, r.ctypes.data)
        vals.append(r.copy())
    v = np.asarray(vals)
    assert abs(v.mean() - 0.5) < 0.005 and (v >= 0).all() and (v < 1).all()
    hist = np.histogram(v, bins=16, range=(0, 1))[0] / v.size
    assert np.abs(hist - 1 / 16).max() < 0.005


def test_morton_interleave(orc):
    def spread(x):
        return sum(((x >> i) & 1) << (3 * i) for i in range(10))

    for x, y, z in [(0, 0, 0), (1023, 0, 0), (0, 1023, 0), (0, 0, 1023), (5, 700, 333), (1023, 1023, 1023)]:
        assert orc.lib().orc_morton3(x, y, z) == (spread(x) << 2) | (spread(y) << 1) | spread(z)


def _ray(o, d, tmin=1e-5, tmax=np.inf):
    r = np.zeros(1, _abi.RAY_DTYPE)
    r["org"], r["dir"], r["tmin"], r["tmax"] = o, d, tmin, tmax
    return r


def test_watertight_known_answers(orc):
    tri = np.float32([[0, 0, 0, 1, 0, 0, 0, 1, 0]])
    h = orc.closest_brute(tri, _ray((0.25, 0.25, -2.0), (0, 0, 1)))
    assert h["prim"][0] == 0 and h["t"][0] == np.float32(2.0)
    assert h["u"][0] == np.float32(0.25) and h["v"][0] == np.float32(0.25)
    # back side hits too (no culling), miss outside, tmax respected
    assert orc.closest_brute(tri, _ray((0.25, 0.25, 3.0), (0, 0, -1)))["t"][0] == np.float32(3.0)
    assert orc.closest_brute(tri, _ray((0.75, 0.75, -1.0), (0, 0, 1)))["prim"][0] == 0xFFFFFFFF
    assert orc.closest_brute(tri, _ray((0.25, 0.25, -2.0), (0, 0, 1), tmax=1.5))["prim"][0] == 0xFFFFFFFF


def test_watertight_shared_edge_never_leaks(orc):
    """Rays swept across the shared diagonal of a quad always hit one of the
    two triangles (Woop et al. 2013's guarantee)."""
    q = np.float32([[0, 0, 0, 1, 0, 0, 1, 1, 0], [0, 0, 0, 1, 1, 0, 0, 1, 0]])
    n = 20_001
    r = np.zeros(n, _abi.RAY_DTYPE)
    t = np.linspace(0.0, 1.0, n)
    r["org"] = np.stack([t, t + np.float32(1e-7) * (t > 0.5), np.full(n, -1.0)], 1).astype(np.float32)
    r["org"][:, :2] = np.clip(r["org"][:, :2], 0.02, 0.97)
    d = np.stack([np.full(n, 0.013), np.full(n, -0.007), np.ones(n)], 1)
    r["dir"] = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    r["tmin"], r["tmax"] = 1e-5, np.inf
    h = orc.closest_brute(q, r)
    assert (h["prim"] != 0xFFFFFFFF).all()


@pytest.mark.parametrize("width,treelet,leaf_max", [(8, 0, 3), (8, 1, 3), (4, 1, 1), (2, 0, 2)])
def test_bvh_traversal_equals_brute_force(orc, width, treelet, leaf_max):
    v = np.concatenate([scenes.soup(3000, 61), np.repeat(scenes.soup(20, 62), 5, axis=0)])
    rays = np.concatenate([scenes.soup_rays(4096, 63), scenes.soup_rays(2048, 64, shadow=True)])
    b = orc.Bvh(v, width=width, treelet=treelet, leaf_max=leaf_max)
    assert np.array_equal(b.closest(rays).view(np.uint8), orc.closest_brute(v, rays).view(np.uint8))
    bvh2, order, wide, tris = b.download()
    assert wide_bvh.validate(wide, tris, width, len(v), v) == b.info()["depth"]
    brute = orc.closest_brute(v, rays)
    occl_expected = (brute["prim"] != 0xFFFFFFFF) & (brute["t"] < rays["tmax"])
    assert np.array_equal(b.any(rays).astype(bool), occl_expected)


def test_box_scene_ties_and_axis_rays(orc):
    sc = scenes.box_scene()
    rng = np.random.default_rng(5)
    n = 50_000
    r = np.zeros(n, _abi.RAY_DTYPE)
    r["org"] = rng.uniform(0.05, 0.95, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d[: n // 4, :2] = 0.0
    d[n // 4: n // 2, 1:] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r["dir"], r["tmin"], r["tmax"] = d.astype(np.float32), 1e-5, np.inf
    b = orc.Bvh(sc["verts"])
    assert np.array_equal(b.closest(r).view(np.uint8), orc.closest_brute(sc["verts"], r).view(np.uint8))


def test_treelets_reduce_sah(orc):
    v = scenes.soup(20_000, 71)
    assert orc.Bvh(v, treelet=1).info()["sah_cost"] < orc.Bvh(v, treelet=0).info()["sah_cost"]


def test_camera_centre_ray(orc):
    sc = scenes.box_scene()
    st = api.make_settings(512, 512, 1)
    o, d = np.zeros(3, np.float32), np.zeros(3, np.float32)
    orc.lib().orc_camera_ray(C.byref(api.make_camera(sc["camera"])), C.byref(st), 256, 256, 0.0, 0.0,
                             o.ctypes.data, d.ctypes.data)
    assert np.allclose(o, (0.5, 0.5, -1.4)) and np.allclose(d, (0, 0, 1), atol=1e-6)


def test_furnace_exact_per_sample(orc):
    """Closed box, albedo 0.5, emission 1: every faithful sample equals
    sum_{k=1..8} 0.5^k = 0.99609375 exactly (powers of two sum exactly)."""
    sc = scenes.closed_box(0.5, 1.0)
    f = orc.render(sc, sc["camera"], api.make_settings(8, 8, 16, 8, 0, 0, 3))
    assert (f["sum"] == np.float32(16 * 0.99609375)).all()
    assert (f["sumsq64"] == 16 * 0.99609375 ** 2).all()


def test_furnace_extended_mean(orc):
    sc = scenes.closed_box(0.5, 1.0)
    f = orc.render(sc, sc["camera"], api.make_settings(16, 16, 256, 8, 3, 1, 4))
    n = f["spp"]
    m = f["sum64"] / n
    se = np.sqrt((f["sumsq64"] / n - m * m).sum() / (n - 1)) / m.size
    assert abs(m.mean() - 0.99609375) < 4 * se + 1e-6


def test_faithful_vs_extended_expectation(orc):
    sc = scenes.box_scene()
    res = []
    for mode, rr, seed in ((0, 0, 1), (1, 3, 2)):
        f = orc.render(sc, sc["camera"], api.make_settings(8, 8, 16384, 8, rr, mode, seed))
        n = f["spp"]
        m = f["sum64"] / n
        res.append((m, (f["sumsq64"] / n - m * m) / (n - 1)))
    (m0, v0), (m1, v1) = res
    z = (m0 - m1) / np.sqrt(v0 + v1)
    assert np.mean(np.abs(z) > 3) <= 0.03
    assert abs(m0.mean() - m1.mean()) < 4 * np.sqrt(v0.sum() + v1.sum()) / m0.size


def test_coplanar_faces_closest_matches_brute_force(orc):
    """The box scene's inner boxes stand on the floor: their bottom faces are
    coplanar with it, and a ray from inside a box meets both at nearly the same
    t.  The BVH traversal must keep every box whose entry lies within the hit
    slack of the best t, so it returns the brute-force closest computed t
    (a floor triangle once lost to a box face here by 2.8e-6 relative)."""
    from crender_gb300 import _abi

    sc = scenes.box_scene()
    r = np.random.default_rng(12)
    n = 4000
    rays = np.zeros(n, _abi.RAY_DTYPE)
    centre = np.where(r.uniform(size=n)[:, None] < 0.5, [0.68, 0.0, 0.33], [0.32, 0.0, 0.67])
    o = centre + np.stack([r.uniform(-0.1, 0.1, n), r.uniform(0.001, 0.2, n), r.uniform(-0.1, 0.1, n)], 1)
    d = np.stack([r.uniform(-1, 1, n), r.uniform(-1, -0.05, n), r.uniform(-1, 1, n)], 1)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["org"], rays["dir"], rays["tmin"], rays["tmax"] = o, d, 1e-5, np.inf
    rays[0]["org"] = (0.354058266, 0.00953761488, 0.564555764)
    rays[0]["dir"] = (-0.718778908, -0.331720859, 0.610997558)
    got = orc.Bvh(sc["verts"], 8, 0, 3).closest(rays)
    want = orc.closest_brute(sc["verts"], rays)
    assert got[0]["prim"] == want[0]["prim"] == 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_alias_table_selects_in_proportion_to_power(orc):
    """The emitter alias table (Walker's method, Vose's construction): column j
    kept with probability prob_j, else its alias; every entry's total selection
    probability equals its weight's share."""
    from crender_gb300 import _abi

    for n, seed in ((1, 0), (2, 1), (1280, 2), (5000, 3)):
        w = np.random.default_rng(seed).gamma(0.5, 1.0, n) + 1e-9
        prob = np.zeros(n, np.float32)
        alias = np.zeros(n, np.uint32)
        orc.lib().orc_alias_table(_abi.ptr(w), n, _abi.ptr(prob), _abi.ptr(alias))
        p = prob.astype(np.float64) / n
        np.add.at(p, alias, (1.0 - prob.astype(np.float64)) / n)
        assert np.allclose(p, w / w.sum(), rtol=1e-5, atol=1e-12)
        assert np.all((prob >= 0) & (prob <= 1)) and np.all(alias < n)


def _camera_f64(cam, x, y, aspect):
    """FP64 restatement of cr::camera::get_ray and _update_cache
    (src/render/camera.cpp:14-39, 54-68): M = T(position) Ry(rot.x) Rx(rot.y)
    Rz(rot.z) (glm::rotate multiplies on the right); perspective rays leave the
    position along normalize(M (u, v, 1/tan(fov/2), 0)); orthographic rays leave
    M (s u, s v, 0, 1) along M's third column."""
    ax, ay, az = np.radians(np.asarray(cam["rotation"], np.float64))
    Ry = np.array([[np.cos(ax), 0, np.sin(ax)], [0, 1, 0], [-np.sin(ax), 0, np.cos(ax)]])
    Rx = np.array([[1, 0, 0], [0, np.cos(ay), -np.sin(ay)], [0, np.sin(ay), np.cos(ay)]])
    Rz = np.array([[np.cos(az), -np.sin(az), 0], [np.sin(az), np.cos(az), 0], [0, 0, 1]])
    M = Ry @ Rx @ Rz
    pos = np.asarray(cam["position"], np.float64)
    if cam.get("mode", 0) == 1:
        s = cam.get("scale", 1.0)
        o = pos + M @ np.array([s * (2 * x - 1), s * (2 * y - 1), 0.0])
        d = M[:, 2]
    else:
        w = 1.0 / np.tan(0.5 * np.radians(cam["fov"]))
        o = pos
        d = M @ np.array([(2 * x - 1) * aspect, 2 * y - 1, w])
    return o, d / np.linalg.norm(d)


@pytest.mark.parametrize("mode", [0, 1])
def test_camera_rays_match_restatement(orc, mode):
    """The oracle's camera (basis formed in double, rounded once) against the
    FP64 restatement, for random poses, fields of view, aspects and jitters."""
    r = np.random.default_rng(5 + mode)
    o, d = np.zeros(3, np.float32), np.zeros(3, np.float32)
    for _ in range(200):
        cam = dict(position=tuple(r.uniform(-5, 5, 3)),
                   rotation=(r.uniform(-180, 180), r.uniform(-90, 90), r.uniform(-180, 180)),
                   fov=float(r.uniform(20, 120)), mode=mode, scale=float(r.uniform(0.2, 3)))
        W, H = int(r.integers(1, 2000)), int(r.integers(1, 2000))
        aspect = float(r.uniform(0.5, 2.0))
        st = api.make_settings(W, H, 1, aspect=aspect)
        px, py = int(r.integers(0, W)), int(r.integers(0, H))
        jx, jy = np.float32(r.random()), np.float32(r.random())
        orc.lib().orc_camera_ray(C.byref(api.make_camera(cam)), C.byref(st), px, py, float(jx), float(jy),
                                 o.ctypes.data, d.ctypes.data)
        x = float(np.float32(np.float32(px) + jx) / np.float32(W))
        y = float(np.float32(np.float32(py) + jy) / np.float32(H))
        o64, d64 = _camera_f64(cam, x, y, float(np.float32(aspect)))
        pos = np.asarray(cam["position"], np.float32).astype(np.float64)
        assert np.allclose(o, o64, rtol=0, atol=4e-6 * (1 + np.abs(pos).max() + 3 * cam["scale"]))
        assert np.allclose(d, d64, rtol=0, atol=2e-6)
        assert abs(np.linalg.norm(d.astype(np.float64)) - 1) < 1e-6
