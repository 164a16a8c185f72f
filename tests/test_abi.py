"""The C ABI: libgbdw.so loads without a GPU and exports every function include/*.h declares."""
import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

import gridbench_gb300 as gb
from gridbench_gb300 import _native
from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        # only the C ABI header(s): declarations of gbdw_* functions
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(gbdw_[a-z0-9_]+)\s*\(", text))
    return names


def test_every_declared_symbol_is_exported():
    L = gb.load()
    declared = _declared()
    assert len(declared) >= 40
    missing = [n for n in sorted(declared) if not hasattr(L, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    declared = _declared()
    assert declared <= set(_native.PROTOTYPES), sorted(declared - set(_native.PROTOTYPES))


def test_invalid_arguments_are_rejected_without_a_device():
    L = gb.load()
    h = C.c_void_p()
    bad = np.array([4, 0, 4, 4], dtype=np.int32)
    assert L.gbdw_lattice_create(C.byref(h), C.c_void_p(bad.ctypes.data), 4) == _native.ERR_INVALID
    assert L.gbdw_dslash_kernel(0, 1, 1, None, None, None, None, 0, 0, None, 0, None) == _native.ERR_INVALID
    assert L.gbdw_field_create(C.byref(h), None, 1, 1) == _native.ERR_INVALID
    assert "invalid" in L.gbdw_last_error().decode().lower()


def test_no_silent_cpu_fallback():
    if gb.device_available():
        pytest.skip("a device is visible")
    dims = np.array([2, 2, 2, 2], dtype=np.int32)
    h = C.c_void_p()
    assert gb.load().gbdw_lattice_create(C.byref(h), C.c_void_p(dims.ctypes.data), 2) == _native.ERR_NO_DEVICE
    U = np.zeros(16 * 144)
    phi = np.zeros(16 * 2 * 24)
    nbr, prm, nsite = gb.generate_table((2, 2, 2, 2), 2)
    with pytest.raises(gb.GbdwError) as e:
        gb.dslash_kernel(1, U, np.zeros_like(phi), phi, nbr, nsite, 2, prm)
    assert e.value.status == _native.ERR_NO_DEVICE


def test_cpp_shim_header_compiles():
    """include/gbdw_dslash.h (the WilsonKernelsHand.h-style seam) compiles as plain C++."""
    import subprocess
    import tempfile
    src = '#include "gbdw_dslash.h"\nint main(){ return Xp + Tm - 7; }\n'
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cc")
        open(p, "w").write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), p],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_empty_and_oversize_inputs_are_rejected_without_a_device():
    """Empty lattices, zero Ls and lattices beyond the 32-bit row indexing (nsite*Ls*12 < 2^31,
    e.g. 64^4 x Ls=16) fail with GBDW_ERR_INVALID before any device work."""
    L = gb.load()
    h = C.c_void_p()
    nbr = np.zeros(8, dtype=np.uint64)
    assert L.gbdw_lattice_from_table(C.byref(h), 0, 4, 1, nbr.ctypes.data, None) == _native.ERR_INVALID
    assert L.gbdw_lattice_from_table(C.byref(h), 1, 0, 1, nbr.ctypes.data, None) == _native.ERR_INVALID
    assert L.gbdw_lattice_from_table(C.byref(h), 1, 4, 3, nbr.ctypes.data, None) == _native.ERR_INVALID
    big = np.array([64, 64, 64, 64], dtype=np.int32)
    assert L.gbdw_lattice_create(C.byref(h), C.c_void_p(big.ctypes.data), 16) == _native.ERR_INVALID
    assert "too large" in L.gbdw_last_error().decode()
    ok = np.array([48, 48, 48, 48], dtype=np.int32)  # 85M 5D sites at Ls=16 fits
    st = L.gbdw_lattice_create(C.byref(h), C.c_void_p(ok.ctypes.data), 16)
    assert st in (_native.OK, _native.ERR_NO_DEVICE)
    if st == _native.OK:
        L.gbdw_lattice_destroy(h)
    assert L.gbdw_dslash_kernel(1, 1, 1, nbr.ctypes.data, nbr.ctypes.data, nbr.ctypes.data, nbr.ctypes.data, 1, 0,
                                None, 0, None) == _native.ERR_INVALID


def test_struct_layouts_match_the_header():
    """The ctypes mirrors of gbdw_cg_params / gbdw_cg_stats have the C structs' size and field
    offsets (compiled from include/gbdw.h with the host compiler)."""
    import subprocess
    import tempfile
    fields = {"gbdw_cg_params": _native.CGParams, "gbdw_cg_stats": _native.CGStats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbdw.h"', "int main(void) {"]
    for cname, py in fields.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["  return 0;", "}"]
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "t.c"), os.path.join(d, "t")
        open(src, "w").write("\n".join(lines) + "\n")
        r = subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), src, "-o", exe],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        out = dict(line.split() for line in subprocess.run([exe], capture_output=True, text=True).stdout.split("\n")
                   if line)
    for cname, py in fields.items():
        assert int(out[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(out[f"{cname}.{f}"]) == getattr(py, f).offset, (cname, f)


def test_allocation_failure_injection_argument_checks():
    """The host-side injection hook needs no device: negative counts are refused, and
    count = 0 switches injection off."""
    L = gb.load()
    assert L.gbdw_debug_fail_allocs(-1, 1) == _native.ERR_INVALID
    assert L.gbdw_debug_fail_allocs(0, -2) == _native.ERR_INVALID
    assert L.gbdw_debug_fail_allocs(0, 0) == _native.OK


def test_fp64_arithmetic_setting_without_a_device():
    """The FP64 arithmetic setting is host state: defaults (explicit operators native, solvers
    double-single), round trip, and rejection of unknown selectors and modes."""
    assert gb.get_fp64_arith(gb.FP64_OPERATORS) == gb.FP64_NATIVE
    assert gb.get_fp64_arith(gb.FP64_SOLVERS) == gb.FP64_DOUBLE_SINGLE
    try:
        gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_DOUBLE_SINGLE)
        assert gb.get_fp64_arith(gb.FP64_OPERATORS) == gb.FP64_DOUBLE_SINGLE
        gb.set_fp64_arith(gb.FP64_SOLVERS, gb.FP64_NATIVE)
        assert gb.get_fp64_arith(gb.FP64_SOLVERS) == gb.FP64_NATIVE
    finally:
        gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_NATIVE)
        gb.set_fp64_arith(gb.FP64_SOLVERS, gb.FP64_DOUBLE_SINGLE)
    L = gb.load()
    assert L.gbdw_set_fp64_arith(2, gb.FP64_NATIVE) == _native.ERR_INVALID
    assert L.gbdw_set_fp64_arith(gb.FP64_OPERATORS, 2) == _native.ERR_INVALID
    assert L.gbdw_get_fp64_arith(gb.FP64_OPERATORS, None) == _native.ERR_INVALID
    # the tuner queries reject null operands before touching a device
    assert L.gbdw_tune_query_ds(None, None, 0, None) == _native.ERR_INVALID
    assert L.gbdw_tune_set_ds(None, None, 0, 4, 1) == _native.ERR_INVALID
    assert L.gbdw_tune_query_m(None, None, None) == _native.ERR_INVALID
    assert L.gbdw_tune_query_cg(None, None, gb.F64, None) == _native.ERR_INVALID


def test_tune_cache_file_round_trip_without_a_device(tmp_path):
    """The tune cache file is host state: entries of every key family (hopping term, M, the
    fused CG step, even-odd, double-single with its register cap in `stages`) load and save back
    unchanged; malformed entries are skipped."""
    import json
    entries = {
        "g1_s1_L16_e0": [64, 2, 2, 2, 1, 1],
        "g1_s1_L16_e1": [64, 2, 3, 4, 1, 8],
        "g1_s1_L16_e16": [64, 2, 2, 2, 1, 1],      # CG step, FP64 residual
        "g2_s2_L16_e33": [64, 2, 3, 4, 1, 1],      # even-odd Schur epilogue (FP16)
        "g0_s0_L16_e64": [128, 1, 0, 4, 1, 4],     # double-single Dhop, 4 CTAs/SM, t-bricks of 4
        "g0_s0_L16_e65": [128, 1, 0, 3, 1, 4],     # double-single M, 3 CTAs/SM
    }
    bad = {"g1_s1_L12_e0": [100, 2, 0, 4, 1, 1], "g1_s1_L12_e1": [64, 3, 0, 4, 1, 1],
           "g1_s1_L12_e2": [64, 2, 0, 3, 1, 1]}   # threads, slices and stages out of range
    src = tmp_path / "in.json"
    src.write_text(json.dumps({**entries, **bad}))
    gb.tune_load(str(src))
    out = tmp_path / "out.json"
    gb.tune_save(str(out))
    saved = json.loads(out.read_text())
    for k, v in entries.items():
        assert saved.get(k) == v, k
    for k in bad:
        assert k not in saved, k
