"""Builds libgbdw.so (CUDA kernels + C ABI) and the C++ drivers in-tree for sm_103a.

Every translation unit is compiled in parallel with one -gencode (compute_103a/sm_103a),
then linked into gridbench_gb300/lib/libgbdw.so.  The drivers under drivers/ are plain C++
programs that include include/gbdw_dslash.h and link against that library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libgbdw.so")
DRIVERS = os.path.join(PKG, "drivers")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_UNITS = ["context.cu", "fields.cu", "dhop.cu", "dhop_f32.cu", "dhop_f64.cu", "dhop_f16.cu", "dhop_ds.cu",
              "blas.cu", "cg.cu", "batch.cu", "tune.cu", "dslash_api.cu", "gen_device.cu", "selftest.cu", "noalloc.cu",
              "eo.cu", "mobius.cu", "halo.cu"]
HOST_UNITS = ["gen.cc", "static_data.cc"]
DRIVER_SOURCES = {"bench_gb300": "bench_gb300.cc", "bench_simple_gb300": "bench_simple_gb300.cc"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libgbdw needs the CUDA toolkit to build")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _newer(src_files: list[str], target: str) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in src_files)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return hs + [os.path.join(INCLUDE, "gbdw.h")]


def build_lib(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nv = nvcc()
    headers = _headers()
    cmds = []
    objs = []
    for u in CUDA_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if _newer([src] + headers, obj):
            cmds.append([nv, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-fno-strict-aliasing", "-c", src, "-o", obj])
    for u in HOST_UNITS:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if _newer([src] + headers, obj):
            # no FP contraction: the generator must give identical bits on x86 and Arm
            cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
                         "-c", src, "-o", obj])
    jobs = jobs or min(len(cmds) or 1, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, cmds))
    if cmds or not os.path.exists(LIB):
        _run([nv, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"])
    if verbose:
        print(f"built {LIB} ({len(cmds)} units recompiled)")
    return LIB


def build_drivers() -> dict[str, str]:
    """Builds the bench.cc / bench_simple.cc flow drivers against libgbdw.so."""
    out = {}
    for name, src in DRIVER_SOURCES.items():
        path = os.path.join(DRIVERS, src)
        exe = os.path.join(LIBDIR, name)
        if _newer([path, LIB, os.path.join(INCLUDE, "gbdw.h"), os.path.join(INCLUDE, "gbdw_dslash.h")], exe):
            _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, path, "-o", exe, "-L", LIBDIR, "-lgbdw",
                  "-Wl,-rpath," + LIBDIR])
        out[name] = exe
    return out


def lib_is_stale() -> bool:
    srcs = [os.path.join(CSRC, u) for u in CUDA_UNITS + HOST_UNITS] + _headers()
    return _newer(srcs, LIB)


def build_all(verbose: bool = False) -> None:
    build_lib(verbose=verbose)
    build_drivers()


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
