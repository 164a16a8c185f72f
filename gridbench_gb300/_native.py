"""ctypes bindings of libgbdw.so (the C ABI declared in include/gbdw.h).

The library is built in-tree by gridbench_gb300.build; there is no CPU fallback: every
compute entry point returns GBDW_ERR_NO_DEVICE without a GPU, and load() raises if the
shared library itself is missing.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

OK, ERR_INVALID, ERR_CUDA, ERR_ALLOC, ERR_TABLE, ERR_NOT_CONVERGED, ERR_DIVERGED, ERR_NO_DEVICE = range(8)
F64, F32, F16, BF16 = 0, 1, 2, 3
CG_PLAIN, CG_MIXED, CG_DOUBLE = 0, 1, 2
FP64_OPERATORS, FP64_SOLVERS = 0, 1
FP64_NATIVE, FP64_DOUBLE_SINGLE = 0, 1

ERR_TIMEOUT = 8
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "ALLOC", 4: "TABLE", 5: "NOT_CONVERGED",
                6: "DIVERGED", 7: "NO_DEVICE", 8: "TIMEOUT"}


class GbdwError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gbdw status {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class CGParams(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("delta", C.c_double),
                ("sloppy_prec", C.c_int), ("sloppy_gauge", C.c_int), ("sloppy_residual", C.c_int)]


class CGStats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("reliable_updates", C.c_int), ("true_residual", C.c_double),
                ("seconds", C.c_double), ("final_rr", C.c_double)]


_vp = C.c_void_p
_i = C.c_int
_d = C.c_double
_u64 = C.c_uint64
_pp = C.POINTER(C.c_void_p)
_i64a = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)

# name -> (restype, argtypes); must list every function of include/gbdw.h
PROTOTYPES = {
    "gbdw_last_error": (C.c_char_p, []),
    "gbdw_version": (_i, []),
    "gbdw_device_available": (_i, []),
    "gbdw_synchronize": (_i, []),
    "gbdw_launch_count": (_u64, []),
    "gbdw_set_stream": (_i, [_vp]),
    "gbdw_stream_create": (_i, [_pp]),
    "gbdw_stream_destroy": (_i, [_vp]),
    "gbdw_dslash_kernel": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _u64, _u64, _vp, _i, _dp]),
    "gbdw_generate_gauge": (_i, [_vp, _i, _u64, _vp]),
    "gbdw_generate_fermion": (_i, [_vp, _i, _i, _u64, _vp]),
    "gbdw_generate_table": (_i, [_vp, _i, _i, _vp, _vp]),
    "gbdw_seed_from_ints": (_u64, [_vp, _i]),
    "gbdw_lattice_from_table": (_i, [_pp, _u64, _i, _i, _vp, _vp]),
    "gbdw_lattice_create": (_i, [_pp, _vp, _i]),
    "gbdw_lattice_destroy": (_i, [_vp]),
    "gbdw_lattice_info": (_i, [_vp, _i64a]),
    "gbdw_gauge_create": (_i, [_pp, _vp, _i, _vp, _i]),
    "gbdw_gauge_destroy": (_i, [_vp]),
    "gbdw_field_create": (_i, [_pp, _vp, _i, _i]),
    "gbdw_field_destroy": (_i, [_vp]),
    "gbdw_field_zero": (_i, [_vp]),
    "gbdw_field_import": (_i, [_vp, _i, _vp, _i]),
    "gbdw_field_export": (_i, [_vp, _i, _vp, _i]),
    "gbdw_field_export_async": (_i, [_vp, _i, _vp, _i]),
    "gbdw_field_copy": (_i, [_vp, _vp]),
    "gbdw_field_gaussian": (_i, [_vp, _i, _u64]),
    "gbdw_gauge_random": (_i, [_pp, _vp, _i, _u64]),
    "gbdw_dhop": (_i, [_vp, _vp, _vp, _i]),
    "gbdw_dwf_m": (_i, [_vp, _vp, _vp, _d, _d, _i, _dp]),
    "gbdw_dwf_mdagm": (_i, [_vp, _vp, _vp, _vp, _d, _d, _dp]),
    "gbdw_norm2": (_i, [_vp, _dp]),
    "gbdw_dot": (_i, [_vp, _vp, _dp, _dp]),
    "gbdw_axpby": (_i, [_d, _vp, _d, _vp]),
    "gbdw_cg_solve": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _i, C.POINTER(CGParams), C.POINTER(CGStats)]),
    "gbdw_lattice_checkerboard": (_i, [_vp, _pp, _pp]),
    "gbdw_gauge_checkerboard": (_i, [_pp, _vp, _vp]),
    "gbdw_field_pick": (_i, [_vp, _vp]),
    "gbdw_field_place": (_i, [_vp, _vp]),
    "gbdw_dhop_eo": (_i, [_vp, _vp, _vp, _i]),
    "gbdw_dwf_meo": (_i, [_vp, _vp, _vp, _vp, _d, _d, _i, _d]),
    "gbdw_dwf_m5inv": (_i, [_vp, _vp, _d, _d, _i]),
    "gbdw_dwf_mpc": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _i, _dp]),
    "gbdw_dwf_mpcdagmpc": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _dp]),
    "gbdw_cg_solve_eo": (_i, [_pp, _pp, _pp, _vp, _vp, _d, _d, _i, C.POINTER(CGParams), C.POINTER(CGStats)]),
    "gbdw_m5d": (_i, [_vp, _vp, _dp, _dp, _dp, _i]),
    "gbdw_m5d_inv": (_i, [_vp, _vp, _dp, _dp, _dp, _i]),
    "gbdw_mobius_mooee": (_i, [_vp, _vp, _d, _d, _d, _d, _i]),
    "gbdw_mobius_mooee_inv": (_i, [_vp, _vp, _d, _d, _d, _d, _i]),
    "gbdw_mobius_m": (_i, [_vp, _vp, _vp, _vp, _d, _d, _d, _d, _i, _dp]),
    "gbdw_mobius_meooe": (_i, [_vp, _vp, _vp, _vp, _d, _d, _d, _i]),
    "gbdw_mobius_mpc": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _d, _d, _d, _d, _i, _dp]),
    "gbdw_mobius_mdagm": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _d, _d, _dp]),
    "gbdw_cg_solve_mobius_eo": (_i, [_pp, _pp, _pp, _vp, _vp, _d, _d, _d, _d, _i, C.POINTER(CGParams),
                                     C.POINTER(CGStats)]),
    "gbdw_halo_bytes": (_i, [_vp, _i, C.POINTER(C.c_size_t)]),
    "gbdw_halo_pack": (_i, [_vp, _i, _i, _i, _vp]),
    "gbdw_halo_pack_all": (_i, [_vp, _i, C.POINTER(C.c_void_p)]),
    "gbdw_cg_solve_mobius": (_i, [_vp, _vp, _vp, _vp, _vp, _d, _d, _d, _d, _i, C.POINTER(CGParams),
                                  C.POINTER(CGStats)]),
    "gbdw_static_data_info": (_i, [C.c_char_p, C.c_char_p, C.POINTER(C.c_uint64), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), C.POINTER(C.c_uint64)]),
    "gbdw_static_data_read": (_i, [C.c_char_p, _vp, _u64, _vp, _u64, _vp, _u64, _vp, _u64, _vp, _u64]),
    "gbdw_static_data_write": (_i, [C.c_char_p, C.c_char_p, _u64, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "gbdw_batch_create": (_i, [_pp, _i, _pp, _pp, _pp, _i]),
    "gbdw_batch_run": (_i, [_vp]),
    "gbdw_batch_destroy": (_i, [_vp]),
    "gbdw_batch_info": (_i, [_vp, _i64a]),
    "gbdw_batch_shape": (_i, [_vp, C.POINTER(C.c_int)]),
    "gbdw_batch_set_shape": (_i, [_vp, C.POINTER(C.c_int)]),
    "gbdw_tune_dhop": (_i, [_vp, _vp, _vp, _i]),
    "gbdw_tune_load": (_i, [C.c_char_p]),
    "gbdw_tune_save": (_i, [C.c_char_p]),
    "gbdw_tune_query": (_i, [_vp, _vp, C.POINTER(C.c_int)]),
    "gbdw_tune_set": (_i, [_vp, _vp, _i, _i, _i, _i]),
    "gbdw_tune_split": (_i, [_vp, _vp, C.POINTER(C.c_int)]),
    "gbdw_tune_set_split": (_i, [_vp, _vp, _i]),
    "gbdw_tune_brick": (_i, [_vp, _vp, C.POINTER(C.c_int)]),
    "gbdw_tune_set_brick": (_i, [_vp, _vp, _i]),
    "gbdw_tune_query_m": (_i, [_vp, _vp, C.POINTER(C.c_int)]),
    "gbdw_set_fp64_arith": (_i, [_i, _i]),
    "gbdw_get_fp64_arith": (_i, [_i, C.POINTER(C.c_int)]),
    "gbdw_tune_query_ds": (_i, [_vp, _vp, _i, C.POINTER(C.c_int)]),
    "gbdw_tune_set_ds": (_i, [_vp, _vp, _i, _i, _i]),
    "gbdw_tune_query_cg": (_i, [_vp, _vp, _i, C.POINTER(C.c_int)]),
    "gbdw_selftest_wait_timeout": (_i, [_u64]),
    "gbdw_timer_create": (_i, [_pp]),
    "gbdw_timer_start": (_i, [_vp]),
    "gbdw_timer_stop": (_i, [_vp, _dp]),
    "gbdw_timer_destroy": (_i, [_vp]),
    "gbdw_flush_l2": (_i, [C.c_size_t]),
    "gbdw_norm2_noalloc": (_i, [_vp, _i, _u64, _dp]),
    "gbdw_debug_fail_allocs": (_i, [_i, _i]),
    "gbdw_host_alloc": (_i, [C.c_size_t, _pp]),
    "gbdw_host_free": (_i, [_vp]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads libgbdw.so (building it in-tree first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path) or _build.lib_is_stale():
        if not build_if_missing:
            raise OSError(f"libgbdw.so not built (or older than its sources) at {path}")
        _build.build_lib()
    L = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != OK:
        raise GbdwError(status, load().gbdw_last_error().decode(errors="replace"))
