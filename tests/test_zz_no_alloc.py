"""crg_build_bvh_noalloc: the BVH build for callers that cannot allocate device
memory (an application whose own pool owns the GPU's memory, or a loop that
must not pay cudaMalloc's device-wide synchronisation).  The caller passes the
vertices and the output buffers; the library's scratch is a fixed device array.

Checked through the C ABI against the allocating path (crg_scene_create +
crg_scene_build, then crg_scene_bvh_download): the wide nodes, the triangle
array and the primitive order must be bit-identical, on two calls in a row
with different inputs (the second must not see the first call's leftovers),
and the second call must change neither the device's free memory nor the
default stream-ordered pool's usage.  Sizes beyond the stated maximum must be
refused with a message."""
import ctypes as C

import numpy as np
import pytest

from crender_gb300 import _abi, api, scenes

pytestmark = pytest.mark.gpu


def _reference_build(ctx, v, opts):
    s = api.Scene(ctx, v, np.zeros(len(v), np.uint32), scenes.material_table([{}]))
    try:
        s.build(opts.width, opts.treelet, opts.leaf_max, opts.treelet_rounds)
        info = s.info()
        _, order, wide, tris = s.download_bvh()
    finally:
        s.close()
    return info, order, wide, tris


def _noalloc_build(ctx, v, opts, bufs):
    n = len(v)
    dv, dw, dt, do = bufs
    dv.upload(v)
    info = _abi.BvhInfo()
    ctx.check(ctx.lib.crg_build_bvh_noalloc(dv.ptr, n, C.byref(opts), dw.ptr, dw.nbytes, dt.ptr, do.ptr,
                                            C.byref(info), None))
    got = {k: getattr(info, k) for k, _ in info._fields_}
    wide = dw.download(np.zeros(got["n_wide_nodes"] * got["node_bytes"], np.uint8))
    tris = dt.download(np.zeros((n, 12), np.float32))
    order = do.download(np.zeros(n, np.uint32))
    return got, order, wide, tris


def _cudart():
    """The CUDA runtime libcrg.so itself uses (it links libcudart dynamically)."""
    import crender_gb300

    crender_gb300.load()
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            return C.CDLL(name, mode=C.RTLD_GLOBAL)
        except OSError:
            continue
    pytest.skip("libcudart not loadable by name")


def _default_pool(rt):
    dev = C.c_int()
    assert rt.cudaGetDevice(C.byref(dev)) == 0
    pool = C.c_void_p()
    assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
    return pool


def _settle(rt):
    """Waits for all work and gives the default pool's unused memory back, so that
    a later synchronisation cannot shrink it while it is being measured."""
    assert rt.cudaDeviceSynchronize() == 0
    assert rt.cudaMemPoolTrimTo(_default_pool(rt), C.c_size_t(0)) == 0


def _device_memory(rt):
    """(free bytes of the device, used and reserved bytes of its default stream-ordered pool)."""
    free, total = C.c_size_t(), C.c_size_t()
    assert rt.cudaMemGetInfo(C.byref(free), C.byref(total)) == 0
    pool = _default_pool(rt)
    used, reserved = C.c_uint64(), C.c_uint64()
    assert rt.cudaMemPoolGetAttribute(pool, 7, C.byref(used)) == 0      # cudaMemPoolAttrUsedMemCurrent
    assert rt.cudaMemPoolGetAttribute(pool, 5, C.byref(reserved)) == 0  # cudaMemPoolAttrReservedMemCurrent
    return free.value, used.value, reserved.value


def test_noalloc_build_matches_allocating_build_twice():
    ctx = api.Context(0)
    rt = _cudart()
    nmax = _abi.NOALLOC_MAX_TRIS
    bufs = [api.DeviceBuffer(ctx, nmax * 36), api.DeviceBuffer(ctx, nmax * 80), api.DeviceBuffer(ctx, nmax * 48),
            api.DeviceBuffer(ctx, nmax * 4)]
    try:
        cases = [(scenes.soup(nmax, 101), _abi.BuildOpts(8, 1, 3, 3)),
                 (scenes.soup(3001, 102), _abi.BuildOpts(8, 0, 3, 3))]
        for k, (v, opts) in enumerate(cases):  # two calls in a row, the second smaller than the first
            ref_info, ref_order, ref_wide, ref_tris = _reference_build(ctx, v, opts)
            _settle(rt)
            mem0 = _device_memory(rt)
            info, order, wide, tris = _noalloc_build(ctx, v, opts, bufs)
            assert rt.cudaDeviceSynchronize() == 0
            mem1 = _device_memory(rt)
            if k == 1:  # the module and its array are in place after the first call: nothing may allocate now
                assert mem1 == mem0, (mem0, mem1)
            assert ctx.lib.crg_noalloc_last_error() == b""
            assert info == ref_info
            assert np.array_equal(wide, ref_wide)
            assert np.array_equal(tris.view(np.uint32), ref_tris.view(np.uint32))
            assert np.array_equal(order, ref_order)
        # beyond the maximum: refused before any device work, with a message
        too_big = _abi.BvhInfo()
        rc = ctx.lib.crg_build_bvh_noalloc(bufs[0].ptr, nmax + 1, None, bufs[1].ptr, bufs[1].nbytes, bufs[2].ptr,
                                           bufs[3].ptr, C.byref(too_big), None)
        assert rc == 1  # CRG_ERR_INVALID_ARG
        assert b"CRG_NOALLOC_MAX_TRIS" in ctx.lib.crg_noalloc_last_error()
    finally:
        for b in bufs:
            b.free()
        ctx.close()
