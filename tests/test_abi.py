"""The C-ABI library loads and exports every entry point include/crg.h
declares; the ctypes struct layouts match the C compiler's; without a GPU the
library fails loudly (a status, not a crash, and no fallback)."""
import ctypes as C
import os
import re
import subprocess
import textwrap

import pytest

from crender_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(ROOT, "include", "crg.h")


@pytest.fixture(scope="module")
def lib():
    import crender_gb300
    from crender_gb300 import build

    if not os.path.exists(crender_gb300.LIB_PATH):
        build.build()
    return C.CDLL(crender_gb300.LIB_PATH)


def header_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(crg_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(lib):
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_signatures_cover_the_header():
    bound = {n for n, _, _ in _abi.CRG_SIGNATURES}
    assert set(header_functions()) == bound


def test_struct_layouts_match_c(tmp_path):
    structs = {"crg_ray": _abi.Ray, "crg_hit": _abi.Hit, "crg_material": _abi.Material, "crg_sun": _abi.Sun,
               "crg_camera": _abi.Camera, "crg_settings": _abi.Settings, "crg_build_opts": _abi.BuildOpts,
               "crg_bvh_info": _abi.BvhInfo, "crg_render_stats": _abi.RenderStats, "crg_model_info": _abi.ModelInfo,
               "crg_stage_times": _abi.StageTimes,
               "crg_post_settings": _abi.PostSettings}
    lines = []
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    src = tmp_path / "sz.c"
    src.write_text(textwrap.dedent(f"""
        #include <stdio.h>
        #include <stddef.h>
        #include "{HDR}"
        int main(void) {{ {' '.join(lines)} return 0; }}
    """))
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-std=c99", "-o", str(exe), str(src)], check=True)
    out = dict(l.rsplit(" ", 1) for l in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n") if l)
    for cname, py in structs.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(py, f).offset, f"{cname}.{f}"


def test_status_strings(lib):
    lib.crg_status_string.restype = C.c_char_p
    assert lib.crg_status_string(0) == b"OK"
    assert lib.crg_status_string(5) == b"NOT_BUILT"
    lib.crg_abi_version.restype = C.c_uint32
    assert lib.crg_abi_version() == 1


def test_no_gpu_means_an_error_status(lib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = lib.crg_context_create(0, C.byref(h))
    assert rc != 0 and not h.value


def test_missing_library_fails_loudly(monkeypatch):
    import crender_gb300

    monkeypatch.setattr(crender_gb300, "_lib", None)
    monkeypatch.setattr(crender_gb300, "LIB_PATH", "/nonexistent/libcrg.so")
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        crender_gb300.load()


def test_null_arguments_are_rejected(lib):
    lib.crg_scene_build.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    assert lib.crg_scene_build(None, None, None) == 1
    lib.crg_intersect_closest.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
    assert lib.crg_intersect_closest(None, None, None, 0, None) == 1
    lib.crg_film_spp.argtypes = [C.c_void_p, C.c_void_p]
    assert lib.crg_film_spp(None, None) == 1


def test_host_adapter_built():
    """The C++ adapter library and its self-test program are built and link;
    the program rejects bad arguments before touching a device."""
    import subprocess

    root = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "crender_gb300", "_build")
    assert os.path.exists(os.path.join(root, "libcrg_host.so"))
    exe = os.path.join(root, "crg_host_selftest")
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([exe, "/nonexistent/in", "/nonexistent/out"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
