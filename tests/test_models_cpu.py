"""Scenes of several models, each with its own instance list, in the oracle:
cr::scene::cast_ray's loop over entities (src/render/scene.cpp:79-98) around
cr::model::intersect's loop over one entity's instances
(src/objects/model.cpp:99-126), a model without a list being one identity
instance (src/render/entities/registry.cpp:73-74).  Pinned against an FP64
brute force over every placement's world-space ("baked") triangles."""
import numpy as np

from crender_gb300 import api, scenes
from test_instances_cpu import brute_f64, random_rays


def baked_models(sc):
    """World triangles of every placement in placement order, float64, and the
    scene primitive index of each."""
    out, prim = [], []
    first = 0
    for m in sc["models"]:
        v = np.asarray(m["verts"], np.float32).reshape(-1, 3, 3).astype(np.float64)
        xs = m.get("instances")
        xs = [np.eye(4)] if xs is None or len(xs) == 0 else np.asarray(xs, np.float64)
        for x in xs:
            out.append(v @ x[:3, :3].T + x[:3, 3])
            prim.append(first + np.arange(len(v)))
        first += len(v)
    return np.concatenate(out), np.concatenate(prim)


def test_models_closest_matches_baked_brute_force(orc):
    sc = scenes.multi_model_box()
    rays = random_rays(800, 11)
    rays["org"][:, 2] = -1.4
    hits = orc.scene_intersect(sc, rays)
    tris, prim = baked_models(sc)
    agree = found = 0
    for i in range(len(rays)):
        t, k = brute_f64(tris, rays["org"][i].astype(np.float64), rays["dir"][i].astype(np.float64))
        if k < 0:
            assert hits["prim"][i] == 0xFFFFFFFF
            continue
        found += 1
        assert abs(hits["t"][i] - t) <= 1e-4 * t
        agree += int(hits["prim"][i] == prim[k])
    assert found > 300
    assert agree >= 0.98 * found  # shared edges may tie


def test_models_any_hit_agrees_with_closest(orc):
    sc = scenes.multi_model_box()
    rays = random_rays(600, 12)
    hits = orc.scene_intersect(sc, rays)
    sh = rays.copy()
    sh["tmax"] = np.where(np.isfinite(hits["t"]), hits["t"] * 1.01, 50.0)
    occ = orc.scene_intersect(sc, sh, any_hit=True)
    assert np.array_equal(occ.astype(bool), np.isfinite(hits["t"]))
    sh["tmax"] = np.where(np.isfinite(hits["t"]), hits["t"] * 0.99, 50.0)
    assert not orc.scene_intersect(sc, sh, any_hit=True).any()


def test_tie_between_models_goes_to_the_earlier_model(orc):
    """Model 3 repeats model 1's mesh under the same identity transform as
    model 1's first instance: every hit on that copy ties exactly, and the
    reference's strict `<` over entities keeps model 1's."""
    sc = scenes.multi_model_box(duplicate=True)
    first3 = sum(len(m["verts"]) for m in sc["models"][:3])
    r = np.random.default_rng(13)
    n = 400
    rays = random_rays(n, 13)
    rays["org"] = np.stack([r.uniform(-0.3, 0.3, n), r.uniform(0.05, 0.25, n), np.full(n, -2.0)], 1)
    rays["dir"] = np.tile(np.array([0.0, 0.0, 1.0], np.float32), (n, 1))
    hits = orc.scene_intersect(sc, rays)
    onbox = (hits["prim"] != 0xFFFFFFFF)
    assert onbox.sum() > 100
    assert not np.any((hits["prim"] >= first3) & onbox)  # never the later copy


def test_one_model_scene_is_the_plain_mesh(orc):
    sc = scenes.box_scene()
    one = scenes.merge_models([dict(verts=sc["verts"], mat_idx=sc["mat_idx"], mats=sc["mats"])], sc["camera"])
    st = api.make_settings(24, 24, 4, 8, 3, 1, 3)
    a = orc.render(sc, sc["camera"], st)["sum"]
    b = orc.render(one, sc["camera"], st)["sum"]
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_models_render_converges_to_the_same_image_in_both_estimators(orc):
    """The extended estimator and the faithful one estimate the same integral
    on Lambertian scenes; with per-model emitters (the ceiling light and one
    lamp per instance of model 2) the means agree within their noise."""
    sc = scenes.multi_model_box()
    lam = dict(sc)
    lam["models"] = [dict(m, mats=scenes.material_table([
        {"colour": tuple(mm["colour"]), "emission": float(mm["emission"])} for mm in m["mats"]]))
        for m in sc["models"]]
    lam = scenes.merge_models(lam["models"], sc["camera"])
    st1 = api.make_settings(16, 16, 256, 8, 0, 1, 9)
    st0 = api.make_settings(16, 16, 256, 8, 0, 0, 9)
    a = orc.render(lam, lam["camera"], st1)
    b = orc.render(lam, lam["camera"], st0)
    ma, mb = a["sum64"].mean() / 256, b["sum64"].mean() / 256
    va = a["sumsq64"].mean() / 256 - (a["sum64"] / 256).mean() ** 2
    assert ma > 0 and abs(ma - mb) < 0.05 * ma, (ma, mb, va)
