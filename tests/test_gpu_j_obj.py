"""An OBJ model through the C++ adapter (crg::host::load_model ->
scene::add_model, whose indexed arrays go to crg_scene_create_indexed and are
de-indexed on the device) renders bit-identically to the same triangles
expanded on the host and sent through crg_scene_create."""
import subprocess

import numpy as np
import pytest

from crender_gb300 import api, scenes
from test_obj_cpu import EXE, MTL, OBJ, restate

pytestmark = pytest.mark.gpu


def test_obj_model_renders_like_host_expansion(ctx, tmp_path):
    (tmp_path / "test.mtl").write_text(MTL)
    (tmp_path / "test.obj").write_text(OBJ)
    W, H, spp = 48, 32, 4
    out = tmp_path / "out.bin"
    r = subprocess.run([EXE, "objrender", str(tmp_path / "test.obj"), str(out), str(W), str(H), str(spp)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    b = out.read_bytes()
    n = np.frombuffer(b, np.uint64, 1)[0]
    got = np.frombuffer(b, np.float32, W * H * 3, 8)
    assert n == spp

    pos, tc, vi, ti, mi, col = restate(OBJ, MTL)
    verts = pos[vi].reshape(-1, 9)
    mats = scenes.material_table([{"colour": tuple(c)} for c in col])
    s = api.Scene(ctx, verts, mi, mats).build(8, 1)
    ctx.check(ctx.lib.crg_scene_set_sun(s.h, 1, None))  # the library's default sun, as the adapter uses it
    cam = dict(position=(0.0, 0.5, -3.0), rotation=(0.0, 0.0, 0.0), fov=60.0, mode=0, scale=1.0)
    f = api.Film(ctx, W, H)
    api.render(s, cam, api.make_settings(W, H, spp, 6, 0, 0, 1, W / H), f)
    want = f.download()["sum"]
    f.close()
    s.close()
    assert want.sum() > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), int(np.sum(got != want))


def test_indexed_scene_equals_expanded_scene(ctx):
    """crg_scene_create_indexed (device expansion, texture coordinates with
    missing entries) against crg_scene_create on the host-expanded arrays."""
    sc = scenes.textured_box()
    v = sc["verts"].reshape(-1, 3)
    pos, inv = np.unique(v, axis=0, return_inverse=True)
    vi = inv.reshape(-1, 3).astype(np.uint32)
    uv = sc["uvs"].reshape(-1, 2)
    tcs, tinv = np.unique(uv, axis=0, return_inverse=True)
    ti = tinv.reshape(-1, 3).astype(np.int32)
    ti[5, 1] = -1  # a corner without a coordinate reads (0, 0)
    uvs = sc["uvs"].copy().reshape(-1, 3, 2)
    uvs[5, 1] = 0.0
    a = api.Scene.from_indexed(ctx, pos, vi, sc["mat_idx"], sc["mats"], tcs, ti)
    b = api.Scene(ctx, pos[vi].reshape(-1, 9), sc["mat_idx"], sc["mats"], uvs=uvs.reshape(-1, 6))
    st = api.make_settings(40, 40, 4, 8, 3, 1, 2)
    films = []
    for s in (a, b):
        s.set_textures(sc["textures"])
        s.build()
        f = api.Film(ctx, 40, 40)
        api.render(s, sc["camera"], st, f)
        films.append(f.download()["sum"])
        f.close()
        s.close()
    assert films[0].sum() > 0
    assert np.array_equal(films[0].view(np.uint32), films[1].view(np.uint32))
