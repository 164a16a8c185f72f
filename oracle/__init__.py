"""ORACLE -- test infrastructure only.

CPU restatement of GridBench's scalar hopping term (dslash_simple.h:19-150) plus DhopDag,
the SIMD-lane layout (WilsonKernelsHandGpu.h:33-41) and the Shamir domain-wall operator,
with ctypes access to the reference's own kernels when they were compiled here
(oracle/_ref/).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this package; the product library never does.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")

_lib = None
_ref = None
_hand = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        for sfx, rp in (("_d", _f64p), ("_f", _f32p)):
            f = getattr(L, "or_dslash" + sfx)
            f.argtypes = [rp, rp, rp, _u64p, C.c_uint64, C.c_uint64, _u8p, C.c_int]
            f.restype = None
            f = getattr(L, "or_dslash_sites" + sfx)
            f.argtypes = [rp, rp, rp, _u64p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int]
            f.restype = None
            f = getattr(L, "or_dslash_lanes" + sfx)
            f.argtypes = [rp, rp, rp, _u64p, C.c_uint64, C.c_uint64, _u8p, C.c_int, C.c_int]
            f.restype = None
            f = getattr(L, "or_dwf_m" + sfx)
            f.argtypes = [rp, rp, rp, _u64p, C.c_uint64, C.c_uint64, C.c_double, C.c_double, C.c_int]
            f.restype = None
        L.or_seed_from_ints.argtypes = [C.c_void_p, C.c_int]
        L.or_seed_from_ints.restype = C.c_uint64
        L.or_generate_gauge.argtypes = [C.c_void_p, C.c_int, C.c_uint64, _f64p]
        L.or_generate_fermion.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_uint64, _f64p]
        L.or_generate_table.argtypes = [C.c_void_p, C.c_int, C.c_int, _u64p, _u8p]
        for n in ("or_generate_gauge", "or_generate_fermion", "or_generate_table"):
            getattr(L, n).restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        L.or_set_threads.restype = None
        L.or_max_threads.restype = C.c_int
        _lib = L
    return _lib


def _dims(dims) -> np.ndarray:
    d = np.ascontiguousarray(dims, dtype=np.int32)
    if d.shape != (4,):
        raise ValueError("dims must have 4 entries (Lx, Ly, Lz, Lt)")
    return d


def seed_from_ints(seeds) -> int:
    a = np.ascontiguousarray(seeds, dtype=np.int32)
    return int(lib().or_seed_from_ints(C.c_void_p(a.ctypes.data), len(a)))


def generate_gauge(dims, nsimd: int = 1, seeds=(1, 2, 3, 4)) -> np.ndarray:
    """Doubled random SU(3) field in the reference layout, FP64 (the oracle's own generator,
    bit-identical to the product's; TableGenerate.cc:44,54 plays this role for GridBench)."""
    d = _dims(dims)
    U = np.empty(int(np.prod(d)) * 8 * 9 * 2, dtype=np.float64)
    if lib().or_generate_gauge(C.c_void_p(d.ctypes.data), nsimd, seed_from_ints(seeds), U):
        raise ValueError("bad dims / nsimd")
    return U


def generate_fermion(dims, Ls: int, nsimd: int = 1, seeds=(5, 6, 7, 8)) -> np.ndarray:
    """Gaussian 5D fermion in the reference layout, FP64 (TableGenerate.cc:36's role)."""
    d = _dims(dims)
    phi = np.empty(int(np.prod(d)) * Ls * 24, dtype=np.float64)
    if lib().or_generate_fermion(C.c_void_p(d.ctypes.data), Ls, nsimd, seed_from_ints(seeds), phi):
        raise ValueError("bad dims / Ls / nsimd")
    return phi


def generate_table(dims, Ls: int, nsimd: int = 1):
    """nbr/prm stencil tables (TableGenerate.cc:75-91); returns (nbr, prm, nsite)."""
    d = _dims(dims)
    nsite = int(np.prod(d)) // nsimd
    nbr = np.empty(nsite * Ls * 8, dtype=np.uint64)
    prm = np.empty(nsite * Ls * 8, dtype=np.uint8)
    if lib().or_generate_table(C.c_void_p(d.ctypes.data), Ls, nsimd, nbr, prm):
        raise ValueError("bad dims / Ls / nsimd")
    return nbr, prm, nsite


def _sfx(a):
    return "_d" if a.dtype == np.float64 else "_f"


def dslash(U, phi, nbr, prm, nsite, Ls, dag=0):
    """Hopping term (or DhopDag) on the Nsimd=1 layout; returns Psi."""
    out = np.zeros_like(phi)
    getattr(lib(), "or_dslash" + _sfx(phi))(U, out, phi, nbr, nsite, Ls, prm, int(dag))
    return out


def dslash_sites(U, phi, out, nbr, site0, site1, Ls, dag=0):
    """Hopping term over 4D sites [site0, site1) into `out` (timing samples)."""
    getattr(lib(), "or_dslash_sites" + _sfx(phi))(U, out, phi, nbr, site0, site1, Ls, int(dag))


def threads() -> int:
    """OpenMP threads the oracle uses (OMP_NUM_THREADS or every host core)."""
    n = os.environ.get("OMP_NUM_THREADS")
    return int(n) if n and n.isdigit() else (os.cpu_count() or 1)


def set_threads(n: int) -> None:
    """Threads of the oracle's parallel loops from now on (restore with set_threads(threads()))."""
    lib().or_set_threads(int(n))


def dslash_lanes(U, phi, nbr, prm, nsite, Ls, nsimd, dag=0):
    out = np.zeros_like(phi)
    getattr(lib(), "or_dslash_lanes" + _sfx(phi))(U, out, phi, nbr, nsite, Ls, prm, int(nsimd), int(dag))
    return out


def dwf_m(U, phi, nbr, nsite, Ls, M5, mf, dag=0):
    out = np.zeros_like(phi)
    getattr(lib(), "or_dwf_m" + _sfx(phi))(U, out, phi, nbr, nsite, Ls, float(M5), float(mf), int(dag))
    return out


def dwf_mdagm(U, phi, nbr, nsite, Ls, M5, mf):
    return dwf_m(U, dwf_m(U, phi, nbr, nsite, Ls, M5, mf, 0), nbr, nsite, Ls, M5, mf, 1)


# ------------------------------------------------------------------ the reference itself
def ref():
    """GridBench's own dslash_simple.h compiled here, or None where the tree is absent."""
    global _ref
    if _ref is None:
        libs = _build.build_ref() if os.path.isdir(_build.REF_DIR) else {}
        path = libs.get("dslash_simple") or (_build.REF_LIB if os.path.exists(_build.REF_LIB) else None)
        if path is None:
            return None
        L = C.CDLL(path)
        for name in ("ref_dslash_kernel", "ref_dslash_kernel_unroll"):
            f = getattr(L, name)
            f.argtypes = [_f64p, _f64p, _f64p, _u64p, C.c_uint64, C.c_uint64, _u8p]
            f.restype = None
        _ref = L
    return _ref


def hand():
    """GridBench's AVX-512 hand kernel compiled here, or None."""
    global _hand
    if _hand is None:
        libs = _build.build_ref() if os.path.isdir(_build.REF_DIR) else {}
        path = libs.get("hand_avx512")
        if path is None:
            return None
        L = C.CDLL(path)
        L.ref_hand_nsimd_d.restype = C.c_int
        L.ref_hand_nsimd_f.restype = C.c_int
        L.ref_hand_dslash_d.argtypes = [C.c_int, _f64p, _f64p, _f64p, _u64p, C.c_uint64, C.c_uint64, _u8p]
        L.ref_hand_dslash_d.restype = C.c_double
        L.ref_hand_dslash_f.argtypes = [C.c_int, _f32p, _f32p, _f32p, _u64p, C.c_uint64, C.c_uint64, _u8p]
        L.ref_hand_dslash_f.restype = C.c_double
        _hand = L
    return _hand


def aligned_copy(a: np.ndarray, align: int = 64) -> np.ndarray:
    """Copy of `a` whose data starts on an `align`-byte boundary (the reference's SIMD types
    are loaded with aligned vector loads; AlignedAllocator.h:17 aligns to 2 MiB)."""
    buf = np.empty(a.nbytes + align, dtype=np.uint8)
    off = (-buf.ctypes.data) % align
    out = buf[off:off + a.nbytes].view(a.dtype)
    out[:] = a.ravel()
    return out
