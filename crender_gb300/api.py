"""Thin Python handles over the C ABI (include/crg.h) for tests and benchmarks.

Every method is one or two C-ABI calls; arrays cross as raw pointers.  The
names follow the reference interface they stand for: Scene ~ cr::scene
(src/render/scene.h:19-53), Film ~ the renderer's film buffers
(src/render/renderer.h:85-91), render() ~ a renderer pass.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi, check, load
from ._abi import ptr

def _default_sun_direction():
    """normalize(0.8, -1, 0) in float32 as glm (and the library) compute it: v * (1 / sqrt(dot(v, v)))."""
    d = np.array([0.8, -1.0, 0.0], np.float32)
    inv = np.float32(1.0) / np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2], dtype=np.float32)
    return tuple(float(x) for x in d * inv)


# cr::entity::sun (src/render/entities/components.h:23-29), bit-identical to crg_scene_set_sun(.., NULL)
TRAVERSAL_THREAD, TRAVERSAL_WARP = _abi.TRAVERSAL_THREAD, _abi.TRAVERSAL_WARP
DEFAULT_SUN = dict(
    size=np.float32(3.14159265359) / np.float32(48.0),
    intensity=100.0,
    direction=_default_sun_direction(),
    colour=(1.0, 0.9, 0.7),
)


def make_sun(sun=None) -> _abi.Sun:
    s = dict(DEFAULT_SUN)
    if sun:
        s.update(sun)
    return _abi.Sun(float(s["size"]), float(s["intensity"]), tuple(map(float, s["direction"])), tuple(map(float, s["colour"])))


def make_camera(cam: dict) -> _abi.Camera:
    return _abi.Camera(
        tuple(map(float, cam["position"])),
        tuple(map(float, cam.get("rotation", (0, 0, 0)))),
        float(cam.get("fov", 75.0)),
        int(cam.get("mode", 0)),
        float(cam.get("scale", 1.0)),
        0,
    )


def make_settings(width, height, spp, max_bounces=8, rr_depth=0, mode=1, seed=1, aspect=1.0) -> _abi.Settings:
    return _abi.Settings(width, height, spp, max_bounces, rr_depth, mode, seed, float(aspect))


class Context:
    def __init__(self, device: int = 0):
        self.lib = load()
        self.h = C.c_void_p()
        check(self.lib.crg_context_create(device, C.byref(self.h)))

    def check(self, status):
        check(status, self.h)

    def close(self):
        if self.h:
            self.lib.crg_context_destroy(self.h)
            self.h = C.c_void_p()

    def sync(self, stream=None):
        self.check(self.lib.crg_stream_sync(self.h, stream))


class DeviceBuffer:
    def __init__(self, ctx: Context, nbytes: int):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        self.ptr = C.c_void_p()
        ctx.check(ctx.lib.crg_device_alloc(ctx.h, self.nbytes, C.byref(self.ptr)))

    @classmethod
    def from_array(cls, ctx, a: np.ndarray, stream=None):
        b = cls(ctx, a.nbytes)
        b.upload(a, stream)
        return b

    def upload(self, a: np.ndarray, stream=None):
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        self.ctx.check(self.ctx.lib.crg_memcpy_h2d(self.ctx.h, self.ptr, ptr(a), a.nbytes, stream))

    def download(self, out: np.ndarray, stream=None):
        assert out.nbytes <= self.nbytes and out.flags["C_CONTIGUOUS"]
        self.ctx.check(self.ctx.lib.crg_memcpy_d2h(self.ctx.h, ptr(out), self.ptr, out.nbytes, stream))
        self.ctx.sync(stream)
        return out

    def free(self):
        if self.ptr:
            self.ctx.lib.crg_device_free(self.ctx.h, self.ptr)
            self.ptr = C.c_void_p()


class PinnedArray:
    """numpy view of page-locked host memory from crg_host_alloc."""

    def __init__(self, ctx: Context, shape, dtype):
        self.ctx = ctx
        dtype = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dtype.itemsize
        self.ptr = C.c_void_p()
        ctx.check(ctx.lib.crg_host_alloc(ctx.h, max(nbytes, 1), C.byref(self.ptr)))
        buf = (C.c_uint8 * max(nbytes, 1)).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, np.uint8, nbytes).view(dtype).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self.ctx.lib.crg_host_free(self.ctx.h, self.ptr)
            self.ptr = C.c_void_p()


class Scene:
    """cr::scene over the GPU path: geometry, materials, sky, sun, BVH."""

    def __init__(self, ctx: Context, verts, mat_idx, mats, uvs=None):
        self.ctx = ctx
        self.verts = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
        self.mat_idx = np.ascontiguousarray(mat_idx, np.uint32)
        self.mats = np.ascontiguousarray(mats)
        self.uvs = None if uvs is None else np.ascontiguousarray(uvs, np.float32).reshape(-1, 6)
        self.ntri = self.verts.shape[0]
        self.h = C.c_void_p()
        ctx.check(
            ctx.lib.crg_scene_create(
                ctx.h, ptr(self.verts), self.ntri, ptr(self.uvs), ptr(self.mat_idx), ptr(self.mats), len(self.mats),
                C.byref(self.h)
            )
        )

    @classmethod
    def from_indexed(cls, ctx: Context, positions, vertex_indices, mat_idx, mats, texcoords=None, tex_indices=None):
        """crg_scene_create_indexed: indexed positions / texture coordinates expanded on the device."""
        self = cls.__new__(cls)
        self.ctx = ctx
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(vertex_indices, np.uint32).reshape(-1, 3)
        self.mat_idx = np.ascontiguousarray(mat_idx, np.uint32)
        self.mats = np.ascontiguousarray(mats)
        tc = None if texcoords is None else np.ascontiguousarray(texcoords, np.float32).reshape(-1, 2)
        ti = None if tex_indices is None else np.ascontiguousarray(tex_indices, np.int32).reshape(-1, 3)
        self.ntri = len(idx)
        self.h = C.c_void_p()
        ctx.check(ctx.lib.crg_scene_create_indexed(ctx.h, ptr(pos), len(pos), ptr(idx), self.ntri, ptr(tc),
                                                   0 if tc is None else len(tc), ptr(ti), ptr(self.mat_idx),
                                                   ptr(self.mats), len(self.mats), C.byref(self.h)))
        return self

    def set_instances(self, xforms):
        """crg_scene_set_instances: [n, 4, 4] row-major matrices (numpy convention), sent
        column-major as glm stores them; None or an empty array removes the instances."""
        if xforms is None or len(xforms) == 0:
            self.ctx.check(self.ctx.lib.crg_scene_set_instances(self.h, None, 0))
            return
        x = np.ascontiguousarray(np.transpose(np.asarray(xforms, np.float32), (0, 2, 1)))
        self.ctx.check(self.ctx.lib.crg_scene_set_instances(self.h, ptr(x), len(x)))

    def add_model(self, verts, mat_idx, mats, uvs=None) -> int:
        """crg_scene_add_model: appends a model (its own BVH and instance list); mat_idx
        indexes its own mats.  Returns the model's index."""
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 9)
        mi = np.ascontiguousarray(mat_idx, np.uint32)
        mt = np.ascontiguousarray(mats)
        uv = None if uvs is None else np.ascontiguousarray(uvs, np.float32).reshape(-1, 6)
        m = C.c_uint32()
        self.ctx.check(self.ctx.lib.crg_scene_add_model(self.h, ptr(v), len(v), ptr(uv), ptr(mi), ptr(mt), len(mt),
                                                        C.byref(m)))
        self.ntri += len(v)
        return m.value

    def add_model_indexed(self, positions, vertex_indices, mat_idx, mats, texcoords=None, tex_indices=None) -> int:
        """crg_scene_add_model_indexed: as from_indexed, for an appended model."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(vertex_indices, np.uint32).reshape(-1, 3)
        mi = np.ascontiguousarray(mat_idx, np.uint32)
        mt = np.ascontiguousarray(mats)
        tc = None if texcoords is None else np.ascontiguousarray(texcoords, np.float32).reshape(-1, 2)
        ti = None if tex_indices is None else np.ascontiguousarray(tex_indices, np.int32).reshape(-1, 3)
        m = C.c_uint32()
        self.ctx.check(self.ctx.lib.crg_scene_add_model_indexed(self.h, ptr(pos), len(pos), ptr(idx), len(idx), ptr(tc),
                                                                0 if tc is None else len(tc), ptr(ti), ptr(mi), ptr(mt),
                                                                len(mt), C.byref(m)))
        self.ntri += len(idx)
        return m.value

    def set_model_instances(self, model: int, xforms):
        """crg_scene_set_model_instances: one model's [n, 4, 4] row-major transforms
        (None or empty = one identity instance)."""
        if xforms is None or len(xforms) == 0:
            self.ctx.check(self.ctx.lib.crg_scene_set_model_instances(self.h, model, None, 0))
            return
        x = np.ascontiguousarray(np.transpose(np.asarray(xforms, np.float32), (0, 2, 1)))
        self.ctx.check(self.ctx.lib.crg_scene_set_model_instances(self.h, model, ptr(x), len(x)))

    def model_count(self) -> int:
        n = C.c_uint32()
        self.ctx.check(self.ctx.lib.crg_scene_model_count(self.h, C.byref(n)))
        return n.value

    def model_info(self, model: int) -> dict:
        i = _abi.ModelInfo()
        self.ctx.check(self.ctx.lib.crg_scene_model_info(self.h, model, C.byref(i)))
        return {k: getattr(i, k) for k, _ in i._fields_}

    @classmethod
    def from_models(cls, ctx: Context, scene: dict):
        """A scene of several models from a dict made by scenes.merge_models: model 0
        by crg_scene_create, the others by crg_scene_add_model, then each model's
        instance list."""
        ms = scene["models"]
        uv0 = ms[0].get("uvs")
        self = cls(ctx, ms[0]["verts"], ms[0]["mat_idx"], ms[0]["mats"], uvs=uv0)
        for m in ms[1:]:
            self.add_model(m["verts"], m["mat_idx"], m["mats"], uvs=m.get("uvs"))
        for k, m in enumerate(ms):
            if m.get("instances") is not None and len(m["instances"]):
                self.set_model_instances(k, m["instances"])
        return self

    def set_textures(self, textures):
        """crg_scene_set_textures: a list of RGBA32F [h, w, 4] arrays (empty list removes them)."""
        texs = [np.ascontiguousarray(t, np.float32) for t in textures]
        arr = (C.c_void_p * max(len(texs), 1))(*[ptr(t) for t in texs])
        w = np.array([t.shape[1] for t in texs] or [0], np.uint32)
        h = np.array([t.shape[0] for t in texs] or [0], np.uint32)
        self.ctx.check(self.ctx.lib.crg_scene_set_textures(self.h, len(texs), arr, ptr(w), ptr(h)))

    def build(self, width=8, treelet=0, leaf_max=3, rounds=3, stream=None):
        self.opts = _abi.BuildOpts(width, treelet, leaf_max, rounds)
        self.ctx.check(self.ctx.lib.crg_scene_build(self.h, C.byref(self.opts), stream))
        return self

    def info(self) -> dict:
        i = _abi.BvhInfo()
        self.ctx.check(self.ctx.lib.crg_scene_bvh_info(self.h, C.byref(i)))
        return {k: getattr(i, k) for k, _ in i._fields_}

    def download_bvh(self):
        i = self.info()
        bvh2 = np.zeros((max(i["n_bvh2_nodes"], 0), 8), np.float32)
        order = np.zeros(i["ntri"], np.uint32)
        wide = np.zeros(i["n_wide_nodes"] * i["node_bytes"], np.uint8)
        tris = np.zeros((i["n_tri_slots"], 12), np.float32)
        self.ctx.check(self.ctx.lib.crg_scene_bvh_download(self.h, ptr(bvh2), ptr(order), ptr(wide), ptr(tris)))
        return bvh2, order, wide, tris

    def set_sun(self, enabled: bool, sun=None):
        s = make_sun(sun)
        self.ctx.check(self.ctx.lib.crg_scene_set_sun(self.h, int(enabled), C.byref(s)))

    def set_skybox(self, rgba: np.ndarray | None, rot=(0.0, 0.0)):
        if rgba is None:
            self.ctx.check(self.ctx.lib.crg_scene_set_skybox(self.h, None, 0, 0, 0.0, 0.0))
            return
        rgba = np.ascontiguousarray(rgba, np.float32)
        h, w = rgba.shape[:2]
        self.ctx.check(self.ctx.lib.crg_scene_set_skybox(self.h, ptr(rgba), w, h, float(rot[0]), float(rot[1])))

    def intersect(self, rays: np.ndarray, any_hit=False, counted=False, traversal=None):
        """Host rays in, host results out (uploads, launches, downloads).  `traversal`:
        None (the default scheme), TRAVERSAL_THREAD or TRAVERSAL_WARP."""
        n = len(rays)
        rb = DeviceBuffer.from_array(self.ctx, rays)
        ob = DeviceBuffer(self.ctx, max(n * (4 if any_hit else 16), 16))
        extra = []
        try:
            if traversal is not None and not counted:
                if any_hit:
                    self.ctx.check(self.ctx.lib.crg_intersect_any_with(self.h, rb.ptr, ob.ptr, n, traversal, None))
                    out = ob.download(np.zeros(n, np.uint32))
                else:
                    self.ctx.check(self.ctx.lib.crg_intersect_closest_with(self.h, rb.ptr, ob.ptr, n, traversal, None))
                    out = ob.download(np.zeros(n, _abi.HIT_DTYPE))
            elif any_hit:
                self.ctx.check(self.ctx.lib.crg_intersect_any(self.h, rb.ptr, ob.ptr, n, None))
                out = ob.download(np.zeros(n, np.uint32))
            elif counted:
                nb = DeviceBuffer(self.ctx, max(4 * n, 16))
                tb = DeviceBuffer(self.ctx, max(4 * n, 16))
                extra = [nb, tb]
                self.ctx.check(self.ctx.lib.crg_intersect_closest_counted(self.h, rb.ptr, ob.ptr, nb.ptr, tb.ptr, n, None))
                out = (ob.download(np.zeros(n, _abi.HIT_DTYPE)), nb.download(np.zeros(n, np.uint32)),
                       tb.download(np.zeros(n, np.uint32)))
            else:
                self.ctx.check(self.ctx.lib.crg_intersect_closest(self.h, rb.ptr, ob.ptr, n, None))
                out = ob.download(np.zeros(n, _abi.HIT_DTYPE))
            self.ctx.check(self.ctx.lib.crg_scene_poll_error(self.h))
            return out
        finally:
            rb.free()
            ob.free()
            for b in extra:
                b.free()

    def set_counting(self, on: bool):
        self.ctx.check(self.ctx.lib.crg_scene_set_counting(self.h, int(on)))

    def stats(self) -> dict:
        s = _abi.RenderStats()
        self.ctx.check(self.ctx.lib.crg_render_stats_get(self.h, C.byref(s)))
        return dict(samples=s.samples, segments=s.segments, shadow_rays=s.shadow_rays,
                    nodes_visited=s.nodes_visited, tris_tested=s.tris_tested)

    def close(self):
        if self.h:
            self.ctx.lib.crg_scene_destroy(self.h)
            self.h = C.c_void_p()


class Film:
    def __init__(self, ctx: Context, width: int, height: int, f64=False, aov=False):
        self.ctx = ctx
        self.width, self.height = width, height
        self.flags = (_abi.FILM_F64 if f64 else 0) | (_abi.FILM_AOV if aov else 0)
        self.h = C.c_void_p()
        ctx.check(ctx.lib.crg_film_create(ctx.h, width, height, self.flags, C.byref(self.h)))

    def reset(self, stream=None):
        self.ctx.check(self.ctx.lib.crg_film_reset(self.h, stream))

    @property
    def spp(self) -> int:
        v = C.c_uint64()
        self.ctx.check(self.ctx.lib.crg_film_spp(self.h, C.byref(v)))
        return v.value

    def download(self, f64=False, aov=False) -> dict:
        n = self.width * self.height
        out = {"sum": np.zeros(n * 3, np.float32)}
        if f64:
            out["sum64"] = np.zeros(n * 3, np.float64)
            out["sumsq64"] = np.zeros(n * 3, np.float64)
        if aov:
            for k in ("albedo", "normal", "depth"):
                out[k] = np.zeros(n * 4, np.float32)
        self.ctx.check(
            self.ctx.lib.crg_film_download(
                self.h, ptr(out["sum"]), ptr(out.get("sum64")), ptr(out.get("sumsq64")), ptr(out.get("albedo")),
                ptr(out.get("normal")), ptr(out.get("depth")), None
            )
        )
        return out

    def close(self):
        if self.h:
            self.ctx.lib.crg_film_destroy(self.h)
            self.h = C.c_void_p()


def render(scene: Scene, camera: dict, settings: _abi.Settings, film: Film, stream=None):
    cam = make_camera(camera)
    scene.ctx.check(scene.ctx.lib.crg_render(scene.h, C.byref(cam), C.byref(settings), film.h, stream))


def render_batch(scenes, views, films, opts=None, stream=None, wait=True):
    """crg_render_batch (wait) or crg_render_batch_async: views = [(scene_index, camera dict,
    Settings)], one film each.  Returns the status."""
    ctx = scenes[0].ctx
    sc = (C.c_void_p * len(scenes))(*[s.h.value for s in scenes])
    fl = (C.c_void_p * len(films))(*[f.h.value for f in films])
    vs = (_abi.View * len(views))()
    for i, (si, cam, st) in enumerate(views):
        vs[i].scene = si
        vs[i].camera = make_camera(cam)
        vs[i].settings = st
    o = _abi.WavefrontOpts(**(opts or {}))
    call = ctx.lib.crg_render_batch if wait else ctx.lib.crg_render_batch_async
    return call(sc, len(scenes), vs, fl, len(views), C.byref(o), stream)


def batch_wait(ctx) -> int:
    """crg_batch_wait: the first error of the batches enqueued on ctx (status)."""
    return ctx.lib.crg_batch_wait(ctx.h)


OPT_FIELDS = ("path_pool", "chunk_samples", "block_size", "fetch", "max_iterations", "count_work", "host_loop", "fuse",
              "refill")


def autotune_batch(scenes, views, sample_budget=0, widths=0, reuse=True, stream=None, leaves=0):
    """crg_autotune_batch: returns (options dict for render_batch, BVH width, trials list).
    `leaves` is a bit mask of leaf sizes to try per scene (1 << 1 | 1 << 2 | 1 << 3)."""
    ctx = scenes[0].ctx
    sc = (C.c_void_p * len(scenes))(*[s.h.value for s in scenes])
    vs = (_abi.View * len(views))()
    for i, (si, cam, st) in enumerate(views):
        vs[i].scene = si
        vs[i].camera = make_camera(cam)
        vs[i].settings = st
    o = _abi.AutotuneOpts(int(sample_budget), int(widths), int(bool(reuse)), int(leaves), 0)
    best, width, n = _abi.WavefrontOpts(), C.c_uint32(), C.c_uint32()
    cap = 64
    trials = (_abi.AutotuneTrial * cap)()
    ctx.check(ctx.lib.crg_autotune_batch(sc, len(scenes), vs, len(views), C.byref(o), C.byref(best), C.byref(width),
                                         trials, cap, C.byref(n), stream))
    opts = {k: getattr(best, k) for k in OPT_FIELDS}
    log = [dict({k: getattr(t.opts, k) for k in OPT_FIELDS}, width=t.width, ms=t.ms, msamples_per_s=t.msamples_per_s)
           for t in trials[:min(n.value, cap)]]
    return opts, width.value, log


def batch_stats(ctx) -> dict:
    s = _abi.RenderStats()
    ctx.check(ctx.lib.crg_batch_stats_get(ctx.h, C.byref(s)))
    return dict(samples=s.samples, segments=s.segments, shadow_rays=s.shadow_rays, nodes_visited=s.nodes_visited,
                tris_tested=s.tris_tested, iterations=s.iterations)


def autotune_cache_save(ctx, path: str):
    """crg_autotune_cache_save: the context's autotuner answers to a text file."""
    ctx.check(ctx.lib.crg_autotune_cache_save(ctx.h, os.fsencode(path)))


def autotune_cache_load(ctx, path: str) -> int:
    """crg_autotune_cache_load: adds a file's answers (measured on this kind of device) to
    the context's cache; returns how many were read."""
    n = C.c_uint32(0)
    ctx.check(ctx.lib.crg_autotune_cache_load(ctx.h, os.fsencode(path), C.byref(n)))
    return n.value


def stage_times(ctx) -> dict:
    """crg_batch_stage_times_get: per-stage device time (ms) of the last batch run with
    host_loop 2, and the shadow stage's share of the counted traversal work."""
    t = _abi.StageTimes()
    ctx.check(ctx.lib.crg_batch_stage_times_get(ctx.h, C.byref(t)))
    return {k: getattr(t, k) for k, _ in t._fields_}


# ---------------------------------------------------------------- differentiation
def set_materials(scene: Scene, mats: np.ndarray):
    """crg_scene_set_materials: same count, BVH kept, emitter table rebuilt."""
    mats = np.ascontiguousarray(mats)
    scene.ctx.check(scene.ctx.lib.crg_scene_set_materials(scene.h, ptr(mats), len(mats)))
    scene.mats = mats


def loss_l2(film: Film, target: DeviceBuffer, adjoint: DeviceBuffer, loss: DeviceBuffer, stream=None):
    """crg_film_loss_l2: loss = mean (I - T)^2 into `loss` (double), dLoss/dI into `adjoint` (float)."""
    film.ctx.check(film.ctx.lib.crg_film_loss_l2(film.h, target.ptr, adjoint.ptr, loss.ptr, stream))


def backward(scene: Scene, camera: dict, settings: _abi.Settings, adjoint: DeviceBuffer, grad_colour: DeviceBuffer,
             grad_emission: DeviceBuffer, stream=None):
    """crg_backward: adds d<adjoint, I>/d(colour, emission) into the two device double arrays."""
    cam = make_camera(camera)
    scene.ctx.check(scene.ctx.lib.crg_backward(scene.h, C.byref(cam), C.byref(settings), adjoint.ptr,
                                               grad_colour.ptr, grad_emission.ptr, stream))


def post_settings(**kw) -> _abi.PostSettings:
    """crg_post_settings with the reference defaults (post_processor.h:20-40), then `kw`."""
    s = _abi.PostSettings()
    check(load().crg_post_settings_default(C.byref(s)))
    for k, v in kw.items():
        setattr(s, k, v)
    return s


def post_process(ctx: Context, src: DeviceBuffer, dst: DeviceBuffer, width: int, height: int,
                 settings: _abi.PostSettings, stream=None):
    """crg_post_process on device RGBA32F images (cr::post_processor::process)."""
    assert src.nbytes >= width * height * 16 and dst.nbytes >= width * height * 16
    ctx.check(ctx.lib.crg_post_process(ctx.h, src.ptr, dst.ptr, width, height, C.byref(settings), stream))


def film_display(film: Film, dst: DeviceBuffer, stream=None):
    """crg_film_display: clamp(sum / spp, 0, 1)^(1/2.2) into a device RGBA32F image."""
    assert dst.nbytes >= film.width * film.height * 16
    film.ctx.check(film.ctx.lib.crg_film_display(film.h, dst.ptr, stream))


def draft_render(scene: Scene, camera: dict, width: int, height: int, dst: DeviceBuffer, aspect=1.0, stream=None):
    """crg_draft_render: unlit nearest-surface colour over the skybox (cr::draft_renderer)."""
    assert dst.nbytes >= width * height * 16
    cam = make_camera(camera)
    scene.ctx.check(scene.ctx.lib.crg_draft_render(scene.h, C.byref(cam), width, height, float(aspect), dst.ptr, stream))
