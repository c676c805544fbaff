"""Builds libcrg.so (the product) for sm_103a, in-tree under crender_gb300/_build/.

Translation units are compiled in parallel and linked with nvcc.  Flags:
  -fmad=false                       no FMA contraction in device code (explicit
                                    __fmaf_rn only where bit-parity is not needed)
  -Xcompiler -ffp-contract=off      the same for host code
  -gencode arch=compute_103a,code=sm_103a   GB300 only
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(ROOT, "csrc")
OUT = os.path.join(ROOT, "_build")
SOURCES = ["crg_api.cu", "bvh_build.cu", "traverse.cu", "render.cu", "wavefront.cu", "adjoint.cu", "autotune.cu", "post.cu", "draft.cu"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
         "-I", os.path.join(ROOT, "..", "include")]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


HOST = os.path.join(ROOT, "host")
CXX = os.environ.get("CXX", "g++")
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "..", "include")]


def build_host(libcrg: str) -> str:
    """libcrg_host.so (the C++ adapter: crg::host::scene / camera / renderer)
    and crg_host_selftest, linked against libcrg.so with an $ORIGIN rpath."""
    so = os.path.join(OUT, "libcrg_host.so")
    exe = os.path.join(OUT, "crg_host_selftest")
    link = ["-L", OUT, "-lcrg", "-Wl,-rpath,$ORIGIN", "-pthread"]
    log = _run([CXX, *CXXFLAGS, "-shared", os.path.join(HOST, "crg_host.cpp"), os.path.join(HOST, "obj_loader.cpp"),
                "-o", so + ".tmp", *link])
    os.replace(so + ".tmp", so)
    log += _run([CXX, *CXXFLAGS, os.path.join(HOST, "selftest.cpp"), "-o", exe + ".tmp", "-lcrg_host", *link])
    os.replace(exe + ".tmp", exe)
    return log


def build(verbose: bool = False, ptxas_v: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    extra = ["-Xptxas", "-v"] if ptxas_v else []
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(ROOT, "..", "include", "crg.h"))
    newest_hdr = max(os.path.getmtime(h) for h in hdrs)

    def compile_one(src):
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        if (not ptxas_v and os.path.exists(o) and os.path.getmtime(o) > max(os.path.getmtime(s), newest_hdr)
                and os.path.getmtime(o) > os.path.getmtime(__file__)):
            return ""
        return _run([NVCC, *ARCH, *FLAGS, *extra, "-c", s, "-o", o])

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        logs = list(ex.map(compile_one, SOURCES))
    objs = [os.path.join(OUT, s.replace(".cu", ".o")) for s in SOURCES]
    lib = os.path.join(OUT, "libcrg.so")
    tmp = lib + ".tmp"
    _run([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-Xcompiler", "-pthread"])
    os.replace(tmp, lib)
    logs.append(build_host(lib))
    log = "".join(logs)
    if verbose:
        sys.stdout.write(log)
    return log


if __name__ == "__main__":
    print(build(verbose=True, ptxas_v="-v" in sys.argv))
