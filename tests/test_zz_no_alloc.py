"""crg_build_bvh_noalloc: the BVH build for callers that cannot allocate device
memory (an application whose own pool owns the GPU's memory, or a loop that
must not pay cudaMalloc's device-wide synchronisation).  The caller passes the
vertices and the output buffers; the library's scratch is a fixed device array.

Checked through the C ABI against the allocating path (crg_scene_create +
crg_scene_build, then crg_scene_bvh_download): the wide nodes, the triangle
array and the primitive order must be bit-identical, on two calls in a row
with different inputs (the second must not see the first call's leftovers).
Sizes beyond the stated maximum must be refused."""
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


def test_noalloc_build_matches_allocating_build_twice():
    ctx = api.Context(0)
    nmax = _abi.NOALLOC_MAX_TRIS
    bufs = [api.DeviceBuffer(ctx, nmax * 36), api.DeviceBuffer(ctx, nmax * 80), api.DeviceBuffer(ctx, nmax * 48),
            api.DeviceBuffer(ctx, nmax * 4)]
    try:
        cases = [(scenes.soup(nmax, 101), _abi.BuildOpts(8, 1, 3, 3)),
                 (scenes.soup(3001, 102), _abi.BuildOpts(8, 0, 3, 3))]
        for v, opts in cases:  # two calls in a row, the second smaller than the first
            ref_info, ref_order, ref_wide, ref_tris = _reference_build(ctx, v, opts)
            info, order, wide, tris = _noalloc_build(ctx, v, opts, bufs)
            assert info == ref_info
            assert np.array_equal(wide, ref_wide)
            assert np.array_equal(tris.view(np.uint32), ref_tris.view(np.uint32))
            assert np.array_equal(order, ref_order)
        # beyond the maximum: refused before any device work
        too_big = _abi.BvhInfo()
        rc = ctx.lib.crg_build_bvh_noalloc(bufs[0].ptr, nmax + 1, None, bufs[1].ptr, bufs[1].nbytes, bufs[2].ptr,
                                           bufs[3].ptr, C.byref(too_big), None)
        assert rc == 1  # CRG_ERR_INVALID_ARG
    finally:
        for b in bufs:
            b.free()
        ctx.close()
