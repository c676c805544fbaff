"""The seeded synthetic workloads the benchmark and the parity tests run, pinned
to their definitions: the box scene (36 triangles, 34 non-emitters, a two-sided
light of emission 17 just under the ceiling), the 1,048,576-triangle soup and
its ray generator, the displaced icosphere (20 x 458^2 triangles plus the
ground and a tessellated sphere light; 60 / 25 / 15 % Lambert / GGX / glass
materials; a constant environment of radiance 1), the 64-view batch and the
inverse-rendering scene."""
import math

import numpy as np

from crender_gb300 import scenes


def test_box_scene():
    sc = scenes.box_scene()
    assert sc["verts"].shape == (36, 9) and sc["verts"].dtype == np.float32
    em = sc["mats"]["emission"][sc["mat_idx"]]
    assert (em == 0).sum() == 34 and (em == 17.0).sum() == 2
    light = sc["verts"][em > 0].reshape(-1, 3, 3)
    assert np.allclose(light[..., 1], np.float32(1.0 - 1e-3))
    assert np.isclose(sum(0.5 * np.linalg.norm(np.cross(t[1] - t[0], t[2] - t[0])) for t in light.astype(np.float64)),
                      0.25 * 0.25)
    v = sc["verts"].reshape(-1, 3)
    assert v.min() >= 0.0 and v.max() <= 1.0
    assert (sc["mats"]["shade_type"] == scenes.SHADE_SMOOTH).all()
    assert sc["camera"]["fov"] == 40.0 and sc["camera"]["position"][2] < 0  # outside the open face


def test_soup_and_rays():
    v = scenes.soup(1 << 20, 1)
    assert v.shape == (1 << 20, 9) and v.dtype == np.float32
    t = v.reshape(-1, 3, 3).astype(np.float64)
    cen = t.mean(axis=1)
    off = (t - cen[:, None, :]).reshape(-1)
    assert abs(cen.mean() - 0.5) < 2e-3 and abs(cen.std() - math.sqrt(1 / 12)) < 2e-3
    # vertex offsets N(0, 0.01^2) per axis, measured about the vertex mean (3 samples: 2/3 of the variance)
    assert abs(off.std() - 0.01 * math.sqrt(2 / 3)) < 2e-4
    assert np.array_equal(v, scenes.soup(1 << 20, 1))  # seeded
    for shadow in (False, True):
        r = scenes.soup_rays(1 << 16, 3 if shadow else 2, shadow=shadow)
        o = r["org"].astype(np.float64)
        d = r["dir"].astype(np.float64)
        assert np.allclose(np.linalg.norm(o - 0.5, axis=1), math.sqrt(3) / 2, atol=1e-6)
        assert np.allclose(np.linalg.norm(d, axis=1), 1, atol=1e-6)
        assert (r["tmin"] == np.float32(1e-5)).all()
        if shadow:
            assert r["tmax"].min() >= 0.1 and r["tmax"].max() <= 1.0
        else:
            assert np.isinf(r["tmax"]).all()
        # every ray points into the unit cube: its target is the origin plus t d for some t
        assert ((0.5 - o) * d).sum(axis=1).min() > 0


def test_displaced_scene():
    sc = scenes.displaced_scene()
    n = len(sc["verts"])
    sphere, ground = 20 * 458 ** 2, 2
    light = n - sphere - ground
    assert sphere == 4_195_280 and light > 0
    em = sc["mats"]["emission"][sc["mat_idx"]]
    assert (em[sphere + ground:] > 0).all() and (em[:sphere + ground] == 0).all()
    st = sc["mats"]["shade_type"][sc["mat_idx"][:sphere]]
    frac = [np.mean(st == k) for k in (scenes.SHADE_SMOOTH, scenes.SHADE_METAL, scenes.SHADE_GLASS)]
    assert np.allclose(frac, [0.60, 0.25, 0.15], atol=0.01)
    metal = sc["mats"][sc["mats"]["shade_type"] == scenes.SHADE_METAL]
    assert metal["roughness"].min() >= 0.05 and metal["roughness"].max() <= 0.5
    glass = sc["mats"][sc["mats"]["shade_type"] == scenes.SHADE_GLASS]
    assert np.allclose(glass["ior"], 1.5)
    r = np.linalg.norm(sc["verts"][:sphere].reshape(-1, 3).astype(np.float64), axis=1)
    assert r.min() > 1 - 0.05 * 1.01 and r.max() < 1 + 0.05 * 1.01  # radial fBm of amplitude 0.05
    assert sc["skybox"].shape == (1, 1, 4) and np.all(sc["skybox"][..., :3] == 1.0)
    assert (sc["width"], sc["height"], sc["spp"], sc["max_bounces"]) == (1920, 1080, 256, 16)


def test_batch_views():
    views = scenes.batch_views()
    assert len(views) == 64
    samples = {0: 0, 1: 0}
    for si, cam, st in views:
        assert (st["width"], st["height"]) in [(128, 128), (256, 256), (512, 512), (1024, 768), (1920, 1080)]
        assert st["spp"] in (16, 64, 256)
        assert st["max_bounces"] == (8 if si == 0 else 16)
        samples[si] += st["width"] * st["height"] * st["spp"]
    assert samples[0] + samples[1] == 4_728_979_456  # the batch workload's samples per step
    assert samples == {0: 1_705_197_568, 1: 3_023_781_888}


def test_inverse_box():
    true = scenes.inverse_box()
    init = scenes.inverse_box(albedo=np.full((34, 3), 0.5), light_colour=np.full(3, 10 / 17))
    assert len(true["mats"]) == 35 and (true["mat_idx"][:34] == np.arange(34)).all()
    assert np.allclose(init["mats"]["colour"][:34, :3], 0.5)
    radiance = init["mats"]["colour"][34, :3].astype(np.float64) * float(init["mats"]["emission"][34])
    assert np.allclose(radiance, 10.0, rtol=1e-6)
    box = scenes.box_scene()
    assert np.allclose(true["mats"]["colour"][:34, :3], box["mats"]["colour"][box["mat_idx"][:34], :3])
