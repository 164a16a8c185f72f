"""ORACLE build recipe (test infrastructure only).

  liboracle.so      the C restatement (oracle.c) and the seeded input generator (gen.c), gcc,
                    no FP contraction, OpenMP
  _ref/libref_dslash.so
                    GridBench's own dslash_simple.h compiled in place from the reference
                    tree through ref_shim.cc (only where that tree exists)
  _ref/libref_hand.so
                    GridBench's AVX-512 hand kernel (WilsonKernelsHandCpu.h) through
                    ref_hand_shim.cc (only on x86 hosts with AVX-512 and the reference tree)

Outputs stay under oracle/ (the _ref/ folder is git-ignored).  The reference tree is never
copied; the compiler reads it where it lies.
"""
from __future__ import annotations

import os
import platform
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("GRIDBENCH_REF", "/root/reference")
LIB = os.path.join(HERE, "liboracle.so")
REF_OUT = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_OUT, "libref_dslash.so")
HAND_LIB = os.path.join(REF_OUT, "libref_hand.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target, deps):
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in deps)


def build_oracle() -> str:
    deps = [os.path.join(HERE, f) for f in ("oracle.c", "gen.c", "oracle_body.h")]
    if _stale(LIB, deps):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
              deps[0], deps[1], "-o", LIB, "-lm"])
    return LIB


def _has_avx512() -> bool:
    if platform.machine() not in ("x86_64", "AMD64"):
        return False
    try:
        with open("/proc/cpuinfo") as f:
            return " avx512f" in f.read()
    except OSError:
        return False


def build_ref() -> dict:
    """Compiles the reference's own kernels when the reference tree is present."""
    out = {}
    if not os.path.isfile(os.path.join(REF_DIR, "dslash_simple.h")):
        return out
    os.makedirs(REF_OUT, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim.cc")
    if _stale(REF_LIB, [shim]):
        _run(["g++", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I", REF_DIR, shim, "-o", REF_LIB])
    out["dslash_simple"] = REF_LIB
    if _has_avx512():
        hshim = os.path.join(HERE, "ref_hand_shim.cc")
        if _stale(HAND_LIB, [hshim]):
            _run(["g++", "-O2", "-fPIC", "-shared", "-w", "-DAVX512", "-mavx512f", "-mavx512cd", "-mavx512dq",
                  "-mavx512bw", "-mavx512vl", "-I", REF_DIR, hshim, "-o", HAND_LIB])
        out["hand_avx512"] = HAND_LIB
    return out


if __name__ == "__main__":
    print(build_oracle())
    print(build_ref())
