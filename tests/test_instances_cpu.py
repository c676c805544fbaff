"""Instances in the oracle (cr::model::intersect's loop over
instances::transforms, src/objects/model.cpp:99-126), pinned against an FP64
brute force over the transformed ("baked") triangles and against the plain
mesh."""
import numpy as np

from crender_gb300 import _abi, api, scenes


def baked(sc):
    """World-space triangles of every instance, in float64."""
    v = sc["verts"].reshape(-1, 3, 3).astype(np.float64)
    out = []
    for m in sc["instances"].astype(np.float64):
        out.append(v @ m[:3, :3].T + m[:3, 3])
    return np.concatenate(out)


def brute_f64(tris, o, d):
    """Moller-Trumbore in float64: (t, index) of the closest hit, t > 1e-4."""
    e1 = tris[:, 1] - tris[:, 0]
    e2 = tris[:, 2] - tris[:, 0]
    pv = np.cross(d, e2)
    det = np.einsum("ij,ij->i", e1, pv)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / det
        tv = o - tris[:, 0]
        u = np.einsum("ij,ij->i", tv, pv) * inv
        qv = np.cross(tv, e1)
        v = (qv @ d) * inv
        t = np.einsum("ij,ij->i", e2, qv) * inv
    ok = (np.abs(det) > 1e-12) & (u >= 0) & (v >= 0) & (u + v <= 1) & (t > 1e-4)
    if not ok.any():
        return np.inf, -1
    t = np.where(ok, t, np.inf)
    k = int(np.argmin(t))
    return t[k], k


def random_rays(n, seed):
    r = np.random.default_rng(seed)
    rays = np.zeros(n, _abi.RAY_DTYPE)
    o = np.stack([r.uniform(-1.5, 2.5, n), r.uniform(0.1, 1.2, n), np.full(n, -3.0)], 1)
    tgt = np.stack([r.uniform(-1.5, 2.5, n), r.uniform(0.0, 1.3, n), r.uniform(0.0, 1.4, n)], 1)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["org"], rays["dir"] = o, d
    rays["tmin"], rays["tmax"] = 1e-5, np.inf
    return rays


def test_instanced_closest_matches_baked_brute_force(orc):
    sc = scenes.instanced_box()
    rays = random_rays(600, 4)
    hits = orc.scene_intersect(sc, rays)
    tris = baked(sc)
    ntri = len(sc["verts"])
    agree = 0
    for i in range(len(rays)):
        t, k = brute_f64(tris, rays["org"][i].astype(np.float64), rays["dir"][i].astype(np.float64))
        if k < 0:
            assert hits["prim"][i] == 0xFFFFFFFF
            continue
        assert abs(hits["t"][i] - t) <= 1e-4 * t
        agree += int(hits["prim"][i] == k % ntri)
    assert agree >= 0.98 * np.sum(hits["prim"] != 0xFFFFFFFF)  # shared edges / coplanar copies may tie


def test_instanced_any_hit_agrees_with_closest(orc):
    sc = scenes.instanced_box()
    rays = random_rays(500, 5)
    hits = orc.scene_intersect(sc, rays)
    sh = rays.copy()
    sh["tmax"] = np.where(np.isfinite(hits["t"]), hits["t"] * 1.01, 50.0)
    occ = orc.scene_intersect(sc, sh, any_hit=True)
    assert np.array_equal(occ.astype(bool), np.isfinite(hits["t"]))
    sh["tmax"] = np.where(np.isfinite(hits["t"]), hits["t"] * 0.99, 50.0)
    assert not orc.scene_intersect(sc, sh, any_hit=True).any()


def test_identity_instance_renders_like_the_plain_mesh(orc):
    """One identity instance: the same image up to the rounding of the
    reference's renormalised direction and recomputed distance."""
    sc = scenes.box_scene()
    inst = dict(sc, instances=np.eye(4, dtype=np.float32)[None])
    st = api.make_settings(32, 32, 32, 8, 3, 1, 7)
    a = orc.render(sc, sc["camera"], st)["sum"]
    b = orc.render(inst, sc["camera"], st)["sum"]
    assert np.abs(a.mean() - b.mean()) < 2e-3 * a.mean()
    assert np.mean(a == b) > 0.3  # paths whose rounding never flipped a decision are bit-identical
