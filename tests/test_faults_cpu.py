"""Allocation fault injection (crg_debug_fail_allocation), the host-side hook
that makes the n-th next allocation of the library fail as if memory were
exhausted.  The reference has no error path here (cr::exit ends the process,
src/util/exception.h:9-13).  Without a GPU: the hook's countdown, its one-shot
disarming, and that calls refused before allocating consume no allocation."""
import ctypes as C

import pytest

from crender_gb300 import _abi


@pytest.fixture(scope="module")
def lib():
    import os

    import crender_gb300
    from crender_gb300 import build

    if not os.path.exists(crender_gb300.LIB_PATH):
        build.build()
    return crender_gb300.load()


def stats(lib):
    a, f, armed = C.c_uint64(), C.c_uint32(), C.c_int64()
    assert lib.crg_debug_allocation_stats(C.byref(a), C.byref(f), C.byref(armed)) == 0
    return a.value, f.value, armed.value


def test_arm_and_disarm(lib):
    assert lib.crg_debug_fail_allocation(5) == 0
    assert stats(lib)[2] == 5
    assert lib.crg_debug_fail_allocation(-1) == 0
    assert stats(lib)[2] == -1
    assert lib.crg_debug_fail_allocation(-7) == 0  # any negative count disarms
    assert stats(lib)[2] == -1


def test_refused_calls_consume_no_allocation(lib):
    """Argument errors are reported before anything is allocated, so an armed
    fault stays armed for the call that really allocates."""
    lib.crg_debug_fail_allocation(0)
    before = stats(lib)
    out = C.c_void_p()
    assert lib.crg_film_create(None, 4, 4, 0, C.byref(out)) == 1          # CRG_ERR_INVALID_ARG
    assert lib.crg_device_alloc(None, 64, C.byref(out)) == 1
    assert lib.crg_scene_build(None, None, None) == 1
    assert lib.crg_render_batch(None, 0, None, None, 0, None, None) == 1
    after = stats(lib)
    assert after == before and after[2] == 0
    lib.crg_debug_fail_allocation(-1)


def test_status_strings_name_oom(lib):
    assert lib.crg_status_string(2) == b"OOM"
