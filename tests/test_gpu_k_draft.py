"""crg_draft_render (cr::draft_renderer's preview as one ray per pixel centre)
against the oracle, bit for bit: flat and textured colours, skybox background,
instances, orthographic camera."""
import numpy as np
import pytest

from crender_gb300 import api, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["textured", "instanced", "ortho"])
def test_draft_matches_oracle(ctx, orc, kind):
    sc = scenes.instanced_box() if kind == "instanced" else scenes.textured_box()
    cam = dict(sc["camera"])
    if kind == "ortho":
        cam.update(mode=1, scale=0.7)
    sky = np.random.default_rng(3).uniform(0, 1, (16, 32, 4)).astype(np.float32)
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"], uvs=sc.get("uvs"))
    if sc.get("textures"):
        s.set_textures(sc["textures"])
    s.build()
    if kind == "instanced":
        s.set_instances(sc["instances"])
    s.set_skybox(sky)
    W, H = 160, 96
    out = api.DeviceBuffer(ctx, W * H * 16)
    api.draft_render(s, cam, W, H, out, W / H)
    g = out.download(np.zeros(W * H * 4, np.float32))
    o = orc.draft_render(sc, cam, W, H, W / H, skybox=sky)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32)), int(np.sum(g != o))
    out.free()
    s.close()
