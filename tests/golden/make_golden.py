"""Regenerates the golden fixtures in tests/golden/ from the CPU oracle.

The reference (CRender) ships no tests or golden vectors and cannot be built
here, so these fixtures pin the oracle against regressions and give the GPU
tests a committed answer to compare with.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from crender_gb300 import api, scenes  # noqa: E402
from oracle import orc  # noqa: E402


# post-processing settings pinned by the fixtures (bloom / gray / each tone curve; faithful and full coverage)
POST_CASES = {
    "bloom_faithful": dict(bloom=1, bloom_threshold=0.5),
    "bloom_full": dict(bloom=1, bloom_threshold=0.5, mode=1),
    "gray_linear": dict(gray_scale=1, tonemapping=1, tonemap_type=0),
    "reinhard": dict(tonemapping=1, tonemap_type=1, exposure=1.3),
    "jim_richard": dict(tonemapping=1, tonemap_type=2),
    "uncharted_full": dict(bloom=1, tonemapping=1, tonemap_type=3, mode=1),
}


def main():
    out = {}
    # RNG and sincos known answers
    r = np.zeros(4, np.float32)
    rng_rows = []
    for key in [(0, 0, 0, 0), (1, 2, 3, 4), (262143, 63, 15, 1), (0xFFFFFFFF, 7, 1, 0x9E3779B9)]:
        orc.lib().orc_rand4(*key, r.ctypes.data)
        rng_rows.append(list(key) + r.tolist())
    out["rng"] = np.asarray(rng_rows, np.float64)
    # BVH of a small soup (all layouts)
    v = scenes.soup(500, 77)
    for W, tl in ((8, 0), (8, 1), (4, 1), (2, 0)):
        b = orc.Bvh(v, width=W, treelet=tl)
        bvh2, order, wide, tris = b.download()
        out[f"bvh_w{W}_t{tl}_wide"] = wide
        out[f"bvh_w{W}_t{tl}_order"] = order
        out[f"bvh_w{W}_t{tl}_bvh2"] = bvh2
    out["soup500"] = v
    rays = scenes.soup_rays(512, 78)
    out["rays512"] = rays.view(np.uint8)
    out["hits512"] = orc.Bvh(v).closest(rays).view(np.uint8)
    # box renders, both estimators
    sc = scenes.box_scene()
    for mode, rr in ((0, 0), (1, 3)):
        f = orc.render(sc, sc["camera"], api.make_settings(16, 16, 4, 8, rr, mode, 42))
        out[f"box16_mode{mode}_sum"] = f["sum"]
        out[f"box16_mode{mode}_sum64"] = f["sum64"]
    # rows beyond the core path: textured and instanced box renders, the draft preview, post-processing
    tx, inst = scenes.textured_box(), scenes.instanced_box()
    for mode in (0, 1):
        st = api.make_settings(16, 12, 4, 8, 3, mode, 43, 16 / 12)
        out[f"textured16_mode{mode}_sum"] = orc.render(tx, tx["camera"], st)["sum"]
        out[f"instanced16_mode{mode}_sum"] = orc.render(inst, inst["camera"], st)["sum"]
    out["draft_textured_24x16"] = orc.draft_render(tx, tx["camera"], 24, 16, 1.5)
    img = np.random.default_rng(44).gamma(0.6, 0.8, (20, 24, 4)).astype(np.float32)
    out["post_input"] = img
    for name, kw in POST_CASES.items():
        out[f"post_{name}"] = orc.post_process(img, api.post_settings(**kw))
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print("wrote", os.path.join(HERE, "golden.npz"), sorted(out))


if __name__ == "__main__":
    main()
