"""Python binding of the CPU oracle (oracle/_build/liborc.so).  TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check (never to stand in for) the GPU path.  Build with `make -C oracle`.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
from crender_gb300 import _abi  # noqa: E402
from crender_gb300._abi import ptr  # noqa: E402

LIB = os.path.join(HERE, "_build", "liborc.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = _abi.bind(C.CDLL(LIB), _abi.ORC_SIGNATURES)
    return _lib


class Bvh:
    def __init__(self, verts: np.ndarray, width=8, treelet=0, leaf_max=3, rounds=3):
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
        self.ntri = self.verts.shape[0]
        self.opts = _abi.BuildOpts(width, treelet, leaf_max, rounds)
        self.h = C.c_void_p()
        rc = lib().orc_bvh_build(ptr(self.verts), self.ntri, C.byref(self.opts), C.byref(self.h))
        assert rc == 0, rc

    def info(self) -> dict:
        i = _abi.BvhInfo()
        lib().orc_bvh_info(self.h, C.byref(i))
        return {k: getattr(i, k) for k, _ in i._fields_}

    def download(self):
        i = self.info()
        bvh2 = np.zeros((i["n_bvh2_nodes"], 8), np.float32)
        order = np.zeros(i["ntri"], np.uint32)
        wide = np.zeros(i["n_wide_nodes"] * i["node_bytes"], np.uint8)
        tris = np.zeros((i["n_tri_slots"], 12), np.float32)
        lib().orc_bvh_download(self.h, ptr(bvh2), ptr(order), ptr(wide), ptr(tris))
        return bvh2, order, wide, tris

    def closest(self, rays, nthreads=0):
        hits = np.zeros(len(rays), _abi.HIT_DTYPE)
        lib().orc_intersect_closest(self.h, ptr(rays), ptr(hits), len(rays), nthreads)
        return hits

    def any(self, rays, nthreads=0):
        occ = np.zeros(len(rays), np.uint32)
        lib().orc_intersect_any(self.h, ptr(rays), ptr(occ), len(rays), nthreads)
        return occ

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_bvh_free(self.h)
            self.h = None


def closest_brute(verts, rays):
    verts = np.ascontiguousarray(verts, np.float32)
    hits = np.zeros(len(rays), _abi.HIT_DTYPE)
    lib().orc_intersect_closest_brute(ptr(verts), verts.size // 9, ptr(rays), ptr(hits), len(rays))
    return hits


def closest_f64(verts, rays):
    verts = np.ascontiguousarray(verts, np.float32)
    n = len(rays)
    t = np.zeros(n, np.float64)
    prim = np.zeros(n, np.uint32)
    ed = np.zeros(n, np.float64)
    lib().orc_intersect_closest_f64(ptr(verts), verts.size // 9, ptr(rays), ptr(t), ptr(prim), ptr(ed), n)
    return t, prim, ed


def scene_desc(scene: dict, sun_enabled=False, sun=None, skybox=None, sky_rot=(0.0, 0.0), build=None):
    """orc_scene_desc of a scene dict {verts, mat_idx, mats[, uvs, textures]}; textures
    is a list of RGBA32F [h, w, 4] arrays."""
    from crender_gb300.api import make_sun

    d = _abi.OrcSceneDesc()
    keep = [np.ascontiguousarray(scene["verts"], np.float32), np.ascontiguousarray(scene["mat_idx"], np.uint32),
            np.ascontiguousarray(scene["mats"])]
    d.verts, d.mat_idx, d.mats = ptr(keep[0]), ptr(keep[1]), ptr(keep[2])
    d.ntri = keep[0].size // 9
    d.nmat = len(keep[2])
    if scene.get("uvs") is not None:
        uv = np.ascontiguousarray(scene["uvs"], np.float32)
        keep.append(uv)
        d.uvs = ptr(uv)
    texs = [np.ascontiguousarray(t, np.float32) for t in scene.get("textures") or []]
    if texs:
        arr = (C.c_void_p * len(texs))(*[ptr(t) for t in texs])
        tw = np.array([t.shape[1] for t in texs], np.uint32)
        th = np.array([t.shape[0] for t in texs], np.uint32)
        keep += [texs, arr, tw, th]
        d.ntex, d.tex_rgba, d.tex_w, d.tex_h = len(texs), C.cast(arr, C.POINTER(C.c_void_p)), ptr(tw), ptr(th)
    if scene.get("models") is not None:
        # several models (crg_scene_add_model): consecutive primitive ranges, per-model instance lists
        ms = scene["models"]
        mn = np.array([len(np.asarray(m["verts"]).reshape(-1, 9)) for m in ms], np.uint32)
        mk = np.array([0 if m.get("instances") is None else len(m["instances"]) for m in ms], np.uint32)
        xs = [np.transpose(np.asarray(m["instances"], np.float32), (0, 2, 1)) for m in ms
              if m.get("instances") is not None and len(m["instances"])]
        xf = np.ascontiguousarray(np.concatenate(xs) if xs else np.zeros((0, 4, 4), np.float32))
        keep += [mn, mk, xf]
        d.nmodels, d.model_ntri, d.model_ninst = len(ms), ptr(mn), ptr(mk)
        d.xforms, d.ninst = (ptr(xf) if len(xf) else None), len(xf)
    elif scene.get("instances") is not None and len(scene["instances"]):
        # [n, 4, 4] row-major -> column-major (glm::mat4 layout)
        xf = np.ascontiguousarray(np.transpose(np.asarray(scene["instances"], np.float32), (0, 2, 1)))
        keep.append(xf)
        d.xforms, d.ninst = ptr(xf), len(xf)
    if skybox is not None:
        sk = np.ascontiguousarray(skybox, np.float32)
        keep.append(sk)
        d.skybox, d.sky_h, d.sky_w = ptr(sk), sk.shape[0], sk.shape[1]
        d.sky_rot_u, d.sky_rot_v = sky_rot
    d.sun_enabled = int(sun_enabled)
    d.sun = make_sun(sun)
    if build is not None:
        keep.append(build)
        d.build = C.pointer(build)
    return d, keep


def render(scene: dict, camera: dict, settings: _abi.Settings, film: dict | None = None, nthreads=0, rows=None, **kw):
    """Renders into a dict film {sum, sum64, sumsq64, albedo, normal, depth, spp}."""
    from crender_gb300.api import make_camera

    W, H = settings.width, settings.height
    if film is None:
        # AOV images start at FLT_MAX, cr::image's clear value (src/objects/image.h:30-33), as the library's films do
        big = np.finfo(np.float32).max
        film = dict(sum=np.zeros(W * H * 3, np.float32), sum64=np.zeros(W * H * 3), sumsq64=np.zeros(W * H * 3),
                    albedo=np.full(W * H * 4, big, np.float32), normal=np.full(W * H * 4, big, np.float32),
                    depth=np.full(W * H * 4, big, np.float32), spp=0, segments=0, shadow_rays=0)
    d, keep = scene_desc(scene, **kw)
    f = _abi.OrcFilm()
    f.width, f.height = W, H
    f.sum_rgb = ptr(film["sum"])
    f.sum64, f.sumsq64 = ptr(film.get("sum64")), ptr(film.get("sumsq64"))
    f.aov_albedo, f.aov_normal, f.aov_depth = ptr(film.get("albedo")), ptr(film.get("normal")), ptr(film.get("depth"))
    f.spp = film["spp"]
    cam = make_camera(camera)
    if rows is None:
        rc = lib().orc_render(C.byref(d), C.byref(cam), C.byref(settings), C.byref(f), nthreads)
    else:
        rc = lib().orc_render_rows(C.byref(d), C.byref(cam), C.byref(settings), C.byref(f), rows[0], rows[1], nthreads)
    assert rc == 0, rc
    film["spp"] = f.spp
    film["segments"] = film.get("segments", 0) + f.segments
    film["shadow_rays"] = film.get("shadow_rays", 0) + f.shadow_rays
    film["render_seconds"] = f.render_seconds
    return film


def adjoint(scene: dict, camera: dict, settings: _abi.Settings, adj: np.ndarray, nthreads=0, **kw):
    """FP64 CPU gradient (colour [nmat, 3], emission [nmat]) of <adj, pixel means>."""
    from crender_gb300.api import make_camera

    d, keep = scene_desc(scene, **kw)
    nmat = d.nmat
    gc = np.zeros(3 * nmat)
    ge = np.zeros(nmat)
    adj = np.ascontiguousarray(adj, np.float32)
    cam = make_camera(camera)
    rc = lib().orc_adjoint(C.byref(d), C.byref(cam), C.byref(settings), ptr(adj), ptr(gc), ptr(ge), nthreads)
    assert rc == 0, rc
    return gc.reshape(nmat, 3), ge


def post_process(img: np.ndarray, settings: _abi.PostSettings) -> np.ndarray:
    """CPU restatement of cr::post_processor::process on an RGBA32F image [h, w, 4]."""
    img = np.ascontiguousarray(img, np.float32)
    h, w = img.shape[:2]
    out = np.zeros_like(img)
    rc = lib().orc_post_process(ptr(img), ptr(out), w, h, C.byref(settings))
    assert rc == 0, rc
    return out


def scene_intersect(scene: dict, rays: np.ndarray, any_hit=False):
    """crg_intersect_closest / _any semantics on a scene dict (instances included)."""
    d, keep = scene_desc(scene)
    rays = np.ascontiguousarray(rays)
    n = len(rays)
    if any_hit:
        out = np.zeros(n, np.uint32)
        rc = lib().orc_scene_intersect(C.byref(d), ptr(rays), None, ptr(out), n)
    else:
        out = np.zeros(n, _abi.HIT_DTYPE)
        rc = lib().orc_scene_intersect(C.byref(d), ptr(rays), ptr(out), None, n)
    assert rc == 0, rc
    return out


def draft_render(scene: dict, camera: dict, width: int, height: int, aspect=1.0, **kw):
    """crg_draft_render semantics on the CPU: RGBA32F [height * width * 4], film layout."""
    from crender_gb300.api import make_camera

    d, keep = scene_desc(scene, **kw)
    out = np.zeros(width * height * 4, np.float32)
    cam = make_camera(camera)
    rc = lib().orc_draft_render(C.byref(d), C.byref(cam), width, height, float(aspect), ptr(out))
    assert rc == 0, rc
    return out


def camera_ray(camera: dict, settings: _abi.Settings, px: int, py: int, jx: float, jy: float):
    """The oracle camera's ray through pixel (px, py) with jitter (jx, jy): (origin, direction)."""
    from crender_gb300.api import make_camera

    cam = make_camera(camera)
    o = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    lib().orc_camera_ray(C.byref(cam), C.byref(settings), px, py, float(jx), float(jy), ptr(o), ptr(d))
    return o, d
