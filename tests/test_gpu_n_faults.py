"""Allocation failures on the GPU path, made on the host by the fault hook
(crg_debug_fail_allocation); the GPU itself is never made to fault.  For
every allocation that scene creation, a model added to a scene, the BVH
build, film creation, the batched wavefront render and the post-processor
make, the test makes exactly that allocation fail and checks that the call
returns CRG_ERR_OOM with a message, that nothing is leaked (the device's free
memory returns to its level before the call once the caller has destroyed
what it holds; measured after the call's kernels have run once, because a
kernel's first launch may enlarge the driver's local-memory reservation for
good), and that the context stays usable: the same call then
succeeds and renders the same film as on a context that never failed.
The reference has no such path (cr::exit ends the process,
src/util/exception.h:9-13)."""
import ctypes as C

import numpy as np
import pytest

from crender_gb300 import CrgError, api, scenes
from test_zz_no_alloc import _cudart, _settle

pytestmark = pytest.mark.gpu


def allocs(lib):
    a = C.c_uint64()
    lib.crg_debug_allocation_stats(C.byref(a), None, None)
    return a.value


def free_bytes(rt):
    _settle(rt)
    f, t = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(f), C.byref(t)) == 0
    return f.value


def box_film(ctx, scene, st):
    f = api.Film(ctx, st.width, st.height)
    try:
        ctx.check(api.render_batch([scene], [(0, scenes.box_scene()["camera"], st)], [f], dict(path_pool=1 << 14)))
        return f.download()["sum"]
    finally:
        f.close()


def sweep(ctx, lib, rt, op, cleanup):
    """Runs op() once to count its allocations, then once per allocation with
    that one failing.  op returns the object(s) it made; cleanup destroys them."""
    before = allocs(lib)
    made = op()
    n = allocs(lib) - before
    cleanup(made)
    assert n >= 1
    for k in range(n):
        level = free_bytes(rt)
        lib.crg_debug_fail_allocation(k)
        with pytest.raises(CrgError) as e:
            made = op()
            cleanup(made)  # not reached when the call failed
        lib.crg_debug_fail_allocation(-1)
        msg = str(e.value)
        assert msg.startswith("OOM: ") and ("alloc" in msg or "out of memory" in msg), msg
        assert free_bytes(rt) == level, (k, n)
    return n


def test_scene_create_add_model_and_build_fail_cleanly(ctx):
    rt = _cudart()
    lib = ctx.lib
    sc = scenes.box_scene()
    st = api.make_settings(24, 24, 2, 6, 3, 1, 5)

    def create():
        return api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"])

    assert sweep(ctx, lib, rt, create, lambda s: s.close()) >= 5

    def build():
        s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"])
        try:
            s.build(8, 1)
        except CrgError:
            s.close()
            raise
        return s

    base = create()
    build().close()  # the build kernels' first launches size the driver's local memory once
    base_level = free_bytes(rt)
    assert sweep(ctx, lib, rt, build, lambda s: s.close()) >= 8
    assert free_bytes(rt) == base_level

    # a failed add_model leaves the scene as it was: its model count is unchanged
    lib.crg_debug_fail_allocation(0)
    with pytest.raises(CrgError):
        base.add_model(sc["verts"][:6], sc["mat_idx"][:6], sc["mats"])
    lib.crg_debug_fail_allocation(-1)
    assert base.model_count() == 1
    base.close()

    # the context still works: build and render as on a fresh context
    s = build()
    got = box_film(ctx, s, st)
    s.close()
    ctx2 = api.Context(0)
    s2 = api.Scene(ctx2, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
    want = box_film(ctx2, s2, st)
    s2.close()
    ctx2.close()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_film_batch_and_post_fail_cleanly():
    rt = _cudart()
    ctx = api.Context(0)
    lib = ctx.lib
    sc = scenes.box_scene()
    s = api.Scene(ctx, sc["verts"], sc["mat_idx"], sc["mats"]).build(8, 1)
    st = api.make_settings(32, 24, 2, 6, 3, 1, 9)
    try:
        sweep(ctx, lib, rt, lambda: api.Film(ctx, 32, 24, f64=True, aov=True), lambda f: f.close())
        # the wavefront workspace is the context's first batch allocation
        f = api.Film(ctx, st.width, st.height)
        lib.crg_debug_fail_allocation(0)
        rc = api.render_batch([s], [(0, sc["camera"], st)], [f], dict(path_pool=1 << 14))
        lib.crg_debug_fail_allocation(-1)
        assert rc == 2 and b"injected" in lib.crg_last_error_string(ctx.h)
        ctx.check(api.render_batch([s], [(0, sc["camera"], st)], [f], dict(path_pool=1 << 14)))
        got = f.download()["sum"]
        ref = api.Film(ctx, st.width, st.height)
        api.render(s, sc["camera"], st, ref)
        assert np.array_equal(got.view(np.uint32), ref.download()["sum"].view(np.uint32))
        f.close()
        ref.close()
        # the post-processor's ping-pong images
        img = np.random.default_rng(1).uniform(0, 2, (24, 32, 4)).astype(np.float32)
        src = api.DeviceBuffer.from_array(ctx, img)
        dst = api.DeviceBuffer(ctx, img.nbytes)
        ps = api.post_settings(bloom=1, mode=1)
        lib.crg_debug_fail_allocation(0)
        with pytest.raises(CrgError):
            api.post_process(ctx, src, dst, 32, 24, ps)
        lib.crg_debug_fail_allocation(-1)
        api.post_process(ctx, src, dst, 32, 24, ps)
        assert np.isfinite(dst.download(np.zeros_like(img))).all()
        src.free()
        dst.free()
    finally:
        lib.crg_debug_fail_allocation(-1)
        s.close()
        ctx.close()
