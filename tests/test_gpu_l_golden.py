"""The library against the committed golden fixtures (tests/golden/golden.npz,
written by the oracle): BVH layouts of a 500-triangle soup, closest hits of 512
rays, box / textured / instanced renders with both estimators, the draft
preview and the post-processor.  These pin the GPU path to stored answers, so a
change that moved the oracle and the kernels together still shows here."""
import os

import numpy as np
import pytest

from crender_gb300 import _abi, api, scenes
from golden import make_golden

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")
POW_ULP = 5  # CUDA powf (<= 4 ulp) vs glibc powf (< 1 ulp), as in the post-processing parity test


@pytest.fixture(scope="module")
def g():
    return np.load(GOLDEN)


def ulp_diff(a, b):
    a = a.view(np.int32).astype(np.int64)
    b = b.view(np.int32).astype(np.int64)
    a = np.where(a < 0, -(a & 0x7FFFFFFF), a)
    b = np.where(b < 0, -(b & 0x7FFFFFFF), b)
    return int(np.abs(a - b).max())


@pytest.mark.parametrize("width,treelet", [(8, 0), (8, 1), (4, 1), (2, 0)])
def test_bvh_layouts(ctx, g, width, treelet):
    v = g["soup500"]
    s = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build(width, treelet)
    bvh2, order, wide, _ = s.download_bvh()
    s.close()
    assert np.array_equal(wide, g[f"bvh_w{width}_t{treelet}_wide"])
    assert np.array_equal(order, g[f"bvh_w{width}_t{treelet}_order"])
    assert np.array_equal(bvh2.view(np.uint32), g[f"bvh_w{width}_t{treelet}_bvh2"].view(np.uint32))


def test_closest_hits(ctx, g):
    v = g["soup500"]
    s = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}])).build()
    hits = s.intersect(g["rays512"].view(_abi.RAY_DTYPE))
    s.close()
    assert np.array_equal(hits.view(np.uint8), g["hits512"])


def render(ctx, sc, st, f64=False):
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"], uvs=sc.get("uvs"))
    if sc.get("textures"):
        s.set_textures(sc["textures"])
    s.build()
    if sc.get("instances") is not None:
        s.set_instances(sc["instances"])
    f = api.Film(ctx, st.width, st.height, f64=f64)
    api.render(s, sc["camera"], st, f)
    out = f.download(f64=f64)
    f.close()
    s.close()
    return out


@pytest.mark.parametrize("mode,rr", [(0, 0), (1, 3)])
def test_box_renders(ctx, g, mode, rr):
    out = render(ctx, scenes.box_scene(), api.make_settings(16, 16, 4, 8, rr, mode, 42), f64=True)
    assert np.array_equal(out["sum"].view(np.uint32), g[f"box16_mode{mode}_sum"].view(np.uint32))
    assert np.array_equal(out["sum64"].view(np.uint64), g[f"box16_mode{mode}_sum64"].view(np.uint64))


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", ["textured16", "instanced16"])
def test_feature_renders(ctx, g, mode, name):
    sc = scenes.textured_box() if name == "textured16" else scenes.instanced_box()
    out = render(ctx, sc, api.make_settings(16, 12, 4, 8, 3, mode, 43, 16 / 12))
    assert out["sum"].sum() > 0
    assert np.array_equal(out["sum"].view(np.uint32), g[f"{name}_mode{mode}_sum"].view(np.uint32))


def test_draft_preview(ctx, g):
    sc = scenes.textured_box()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"], uvs=sc["uvs"])
    s.set_textures(sc["textures"])
    s.build()
    W, H = 24, 16
    out = api.DeviceBuffer(ctx, W * H * 16)
    api.draft_render(s, sc["camera"], W, H, out, 1.5)
    got = out.download(np.zeros(W * H * 4, np.float32))
    out.free()
    s.close()
    assert np.array_equal(got.view(np.uint32), g["draft_textured_24x16"].reshape(-1).view(np.uint32))


@pytest.mark.parametrize("name", list(make_golden.POST_CASES))
def test_post_processing(ctx, g, name):
    img = g["post_input"]
    h, w = img.shape[:2]
    s = api.post_settings(**make_golden.POST_CASES[name])
    src = api.DeviceBuffer.from_array(ctx, img)
    dst = api.DeviceBuffer(ctx, img.nbytes)
    api.post_process(ctx, src, dst, w, h, s)
    got = dst.download(np.zeros_like(img))
    src.free()
    dst.free()
    tol = POW_ULP if (s.tonemapping and s.tonemap_type in (0, 1, 3)) else 0
    assert ulp_diff(got, g[f"post_{name}"]) <= tol
