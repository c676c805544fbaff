"""Draft preview oracle (cr::draft_renderer's unlit nearest-surface image,
src/render/draft/draft_renderer.cpp:150-271): known answers."""
import numpy as np

from crender_gb300 import scenes


def test_flat_colours_and_background(orc):
    sc = scenes.box_scene()
    sky = np.array([[[0.1, 0.2, 0.3, 1.0]]], np.float32)
    W, H = 40, 30
    img = orc.draft_render(sc, sc["camera"], W, H, W / H, skybox=sky).reshape(H, W, 4)
    cols = {tuple(np.round(c, 4)) for c in sc["mats"]["colour"][:, :3].astype(np.float64)}
    cols.add((0.1, 0.2, 0.3))
    seen = {tuple(np.round(p, 4)) for p in img[..., :3].reshape(-1, 3).astype(np.float64)}
    assert seen <= cols and len(seen) >= 4  # walls, boxes, light (flat colours) and the sky
    assert np.all(img[..., 3] == 1.0)


def test_near_plane_clips(orc):
    """A quad 0.05 in front of the camera is behind the 0.1 near plane and is
    not drawn; moved to 0.2 it covers the image."""
    sc = scenes.box_scene()
    cam = sc["camera"]
    z = cam["position"][2]
    for dz, covered in ((0.05, False), (0.2, True)):
        q = np.array([[-5, -5, z + dz, 5, -5, z + dz, 5, 5, z + dz], [-5, -5, z + dz, 5, 5, z + dz, -5, 5, z + dz]],
                     np.float32)
        mats = scenes.material_table([*[dict(colour=tuple(c)) for c in sc["mats"]["colour"]],
                                      {"colour": (0.0, 0.0, 1.0, 1.0)}])
        s2 = dict(sc, verts=np.concatenate([sc["verts"], q]), mat_idx=np.concatenate([sc["mat_idx"], [4, 4]]).astype(np.uint32),
                  mats=mats)
        img = orc.draft_render(s2, cam, 16, 16).reshape(16, 16, 4)
        blue = np.all(img[..., :3] == [0, 0, 1], axis=-1)
        assert blue.all() if covered else not blue.any()
