"""The C++ host adapter (crg::host::scene / camera / renderer, the interface
of cr::scene / cr::camera / cr::renderer) driven by its self-test program: a
scene of two models (each add_model call one library model with its own BVH),
a renderer run to a target spp in one-sample passes, an update() that changes
the depth and restarts, and cast_rays, each compared with direct ABI calls."""
import os
import subprocess

import numpy as np
import pytest

from crender_gb300 import _abi, api, scenes

pytestmark = pytest.mark.gpu
EXE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "crender_gb300", "_build",
                   "crg_host_selftest")


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    r = np.zeros(n, _abi.RAY_DTYPE)
    o = np.tile(np.array([0.5, 0.5, -1.4], np.float32), (n, 1))
    tgt = rng.uniform(0.02, 0.98, (n, 3)).astype(np.float32)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r["org"], r["dir"] = o, d
    r["tmin"], r["tmax"] = 1e-5, np.inf
    return r


@pytest.mark.parametrize("mode", [0, 1])
def test_adapter_matches_abi(ctx, tmp_path, mode):
    sc = scenes.box_scene()
    W, H, spp, bounces = 64, 48, 8, 8
    rays = _rays(256, 3)
    cam = api.make_camera(sc["camera"])
    hdr = np.array([0x54475243, len(sc["mat_idx"]), len(sc["mats"]), W, H, spp, bounces, mode, len(rays), 20], np.uint32)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        for a in (hdr, sc["verts"].astype(np.float32), sc["mat_idx"].astype(np.uint32), sc["mats"]):
            f.write(np.ascontiguousarray(a).tobytes())
        f.write(bytes(cam))
        f.write(rays.tobytes())
    r = subprocess.run([EXE, str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    buf = open(out, "rb").read()
    n = W * H * 3
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(buf, dtype, count, off)
        off += a.nbytes
        return a

    spp1, s1 = take(np.uint64, 1)[0], take(np.float32, n)
    spp2, s2 = take(np.uint64, 1)[0], take(np.float32, n)
    total_rays = take(np.uint64, 1)[0]
    rec = take(np.uint8, len(rays) * 20).view(np.dtype([("prim", "<u4"), ("t", "<f4"), ("n", "<f4", 3)]))
    assert off == len(buf)
    assert spp1 == spp and spp2 == spp
    assert total_rays > 0

    # the adapter registered two models (triangles [0, 20) and [20, 36), each with
    # the whole material table): the same two models through the ABI
    scene = api.Scene(ctx, sc["verts"][:20], sc["mat_idx"][:20], sc["mats"])
    scene.add_model(sc["verts"][20:], sc["mat_idx"][20:], sc["mats"])
    scene.build(8, 1)
    film = api.Film(ctx, W, H)
    try:
        for b, got in ((bounces, s1), (bounces // 2, s2)):
            film.reset()
            api.render(scene, sc["camera"], api.make_settings(W, H, spp, b, 0, mode, 1, W / H), film)
            want = film.download()["sum"]
            assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), int(np.sum(got != want))
        hits = scene.intersect(rays)
        assert np.array_equal(rec["prim"], hits["prim"])
        hit = hits["prim"] != 0xFFFFFFFF
        assert hit.sum() > 200
        assert np.array_equal(rec["t"][hit].view(np.uint32), hits["t"][hit].view(np.uint32))
        assert np.allclose(np.linalg.norm(rec["n"][hit], axis=1), 1.0, atol=1e-5)
    finally:
        film.close()
        scene.close()


def test_adapter_draft_post_instances(ctx, tmp_path):
    """crg::host::draft_renderer, post_processor and scene::set_instances (the
    cr::draft_renderer / cr::post_processor / instances interfaces) against
    direct ABI calls."""
    sc = scenes.box_scene()
    W, H, spp, bounces = 48, 40, 4, 6
    rays = _rays(512, 5)
    cam = api.make_camera(sc["camera"])
    hdr = np.array([0x54475243, len(sc["mat_idx"]), len(sc["mats"]), W, H, spp, bounces, 1, len(rays), 36], np.uint32)
    inp, out = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        for a in (hdr, sc["verts"].astype(np.float32), sc["mat_idx"].astype(np.uint32), sc["mats"]):
            f.write(np.ascontiguousarray(a).tobytes())
        f.write(bytes(cam))
        f.write(rays.tobytes())
    r = subprocess.run([EXE, "extras", str(inp), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    buf = open(out, "rb").read()
    n4 = W * H * 4
    draft = np.frombuffer(buf, np.float32, n4, 0)
    progress = np.frombuffer(buf, np.float32, n4, n4 * 4)
    post = np.frombuffer(buf, np.float32, n4, n4 * 8)
    rec = np.frombuffer(buf, np.dtype([("prim", "<u4"), ("t", "<f4")]), len(rays), n4 * 12)

    scene = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
    img = api.DeviceBuffer(ctx, n4 * 4)
    dst = api.DeviceBuffer(ctx, n4 * 4)
    try:
        api.draft_render(scene, sc["camera"], W, H, img, W / H)
        assert np.array_equal(img.download(np.zeros(n4, np.float32)).view(np.uint32), draft.view(np.uint32))
        img.upload(np.ascontiguousarray(progress))
        ps = api.post_settings(bloom=1, bloom_threshold=0.6, bloom_strength=0.8, tonemapping=1, tonemap_type=1,
                               exposure=1.2, gamma=2.2, mode=1)
        api.post_process(ctx, img, dst, W, H, ps)
        assert np.array_equal(dst.download(np.zeros(n4, np.float32)).view(np.uint32), post.view(np.uint32))
        moved = np.eye(4, dtype=np.float32)
        moved[0, 3] = 0.25
        scene.set_instances(np.stack([np.eye(4, dtype=np.float32), moved]))
        hits = scene.intersect(rays)
        assert np.array_equal(rec["prim"], hits["prim"])
        hit = hits["prim"] != 0xFFFFFFFF
        assert hit.sum() > 200
        assert np.array_equal(rec["t"][hit].view(np.uint32), hits["t"][hit].view(np.uint32))
    finally:
        img.free()
        dst.free()
        scene.close()
