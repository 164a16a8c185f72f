"""GB300-native domain-wall Wilson hopping term (GridBench's Dhop) -- Python host mirror.

Everything here forwards to libgbdw.so through its C ABI (include/gbdw.h); numpy arrays
carry host data in GridBench's reference layout.  The names follow the reference:
dslash_kernel() is the seam of WilsonKernelsHand.h:17-29, generate_*() play the role of
TableGenerate.cc, and the objects (Lattice, Gauge, Field) expose the GB300 layout.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _native
from ._native import (BF16, CG_DOUBLE, CG_MIXED, CG_PLAIN, F16, F32, F64, FP64_DOUBLE_SINGLE, FP64_NATIVE,
                      FP64_OPERATORS, FP64_SOLVERS, CGParams, CGStats, GbdwError, check, load)

__all__ = ["F64", "F32", "F16", "BF16", "CG_PLAIN", "CG_MIXED", "CG_DOUBLE", "GbdwError", "load",
           "device_available", "launch_count", "synchronize", "seed_from_ints", "generate_gauge",
           "generate_fermion", "generate_table", "Lattice", "Gauge", "Field", "dhop", "dwf_m", "dwf_mdagm",
           "cg_solve", "Batch", "dslash_kernel", "Timer", "flush_l2", "m5d", "m5d_inv", "mobius_mooee",
           "mobius_mooee_inv", "mobius_m", "mobius_meooe", "mobius_mpc", "mobius_mdagm", "cg_solve_mobius", "cg_solve_mobius_eo"]

_DT = {F64: np.float64, F32: np.float32}


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data)


def device_available() -> bool:
    return bool(load().gbdw_device_available())


def launch_count() -> int:
    return int(load().gbdw_launch_count())


def synchronize() -> None:
    check(load().gbdw_synchronize())


def flush_l2(nbytes: int) -> None:
    check(load().gbdw_flush_l2(nbytes))


def seed_from_ints(seeds: Sequence[int]) -> int:
    a = np.ascontiguousarray(seeds, dtype=np.int32)
    return int(load().gbdw_seed_from_ints(_ptr(a), len(a)))


def _dims(dims) -> np.ndarray:
    d = np.ascontiguousarray(dims, dtype=np.int32)
    if d.shape != (4,):
        raise ValueError("dims must have 4 entries (Lx, Ly, Lz, Lt)")
    return d


def generate_gauge(dims, nsimd: int = 1, seeds=(1, 2, 3, 4)) -> np.ndarray:
    """Doubled random SU(3) field, reference layout, FP64 (TableGenerate.cc:44,54)."""
    d = _dims(dims)
    V = int(np.prod(d))
    U = np.empty(V * 8 * 9 * 2, dtype=np.float64)
    check(load().gbdw_generate_gauge(_ptr(d), nsimd, seed_from_ints(seeds), _ptr(U)))
    return U


def generate_fermion(dims, Ls: int, nsimd: int = 1, seeds=(5, 6, 7, 8)) -> np.ndarray:
    """Gaussian 5D fermion, reference layout, FP64 (TableGenerate.cc:36)."""
    d = _dims(dims)
    V = int(np.prod(d))
    phi = np.empty(V * Ls * 24, dtype=np.float64)
    check(load().gbdw_generate_fermion(_ptr(d), Ls, nsimd, seed_from_ints(seeds), _ptr(phi)))
    return phi


def generate_table(dims, Ls: int, nsimd: int = 1):
    """nbr/prm stencil tables (TableGenerate.cc:75-91); returns (nbr uint64, prm uint8, nsite)."""
    d = _dims(dims)
    nsite = int(np.prod(d)) // nsimd
    nbr = np.empty(nsite * Ls * 8, dtype=np.uint64)
    prm = np.empty(nsite * Ls * 8, dtype=np.uint8)
    check(load().gbdw_generate_table(_ptr(d), Ls, nsimd, _ptr(nbr), _ptr(prm)))
    return nbr, prm, nsite


class _Handle:
    _destroy = ""

    def __init__(self):
        self.h = C.c_void_p()

    def close(self):
        if self.h and self.h.value:
            getattr(load(), self._destroy)(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Lattice(_Handle):
    _destroy = "gbdw_lattice_destroy"

    @classmethod
    def from_table(cls, nbr: np.ndarray, prm: np.ndarray | None, nsite: int, Ls: int, nsimd: int = 1):
        self = cls()
        nbr = np.ascontiguousarray(nbr, dtype=np.uint64)
        prm_p = None
        if prm is not None:
            prm = np.ascontiguousarray(prm, dtype=np.uint8)
            prm_p = _ptr(prm)
        check(load().gbdw_lattice_from_table(C.byref(self.h), nsite, Ls, nsimd, _ptr(nbr), prm_p))
        return self

    @classmethod
    def periodic(cls, dims, Ls: int):
        self = cls()
        d = _dims(dims)
        check(load().gbdw_lattice_create(C.byref(self.h), _ptr(d), Ls))
        return self

    def info(self) -> dict:
        a = (C.c_int64 * 4)()
        check(load().gbdw_lattice_info(self.h, a))
        return {"sites": a[0], "Ls": a[1], "nsimd": a[2], "fast": bool(a[3])}

    def checkerboard(self) -> tuple:
        """(even, odd) half lattices of this periodic lattice (every extent even); half-site
        index = parent site // 2."""
        e, o = Lattice(), Lattice()
        check(load().gbdw_lattice_checkerboard(self.h, C.byref(e.h), C.byref(o.h)))
        e.parent = o.parent = self
        e.parity, o.parity = 0, 1
        return e, o


class Gauge(_Handle):
    _destroy = "gbdw_gauge_destroy"

    def __init__(self, lat: Lattice, U: np.ndarray | None, prec: int = F32, seed: int | None = None):
        """From a reference-layout doubled field U, or (U=None) a device-generated random
        SU(3) field with the given seed (periodic lattices)."""
        super().__init__()
        self.lat = lat
        self.prec = prec
        if U is None:
            check(load().gbdw_gauge_random(C.byref(self.h), lat.h, prec, int(seed or 0)))
            return
        U = np.ascontiguousarray(U)
        src = F64 if U.dtype == np.float64 else F32
        check(load().gbdw_gauge_create(C.byref(self.h), lat.h, prec, _ptr(U), src))

    def checkerboard(self, half: Lattice) -> "Gauge":
        """The links of one half lattice's sites (same precision), for the even-odd operators."""
        g = Gauge.__new__(Gauge)
        _Handle.__init__(g)
        g.lat, g.prec, g.parent = half, self.prec, self
        check(load().gbdw_gauge_checkerboard(C.byref(g.h), self.h, half.h))
        return g


class Field(_Handle):
    _destroy = "gbdw_field_destroy"

    def __init__(self, lat: Lattice, prec: int = F32, nrhs: int = 1):
        super().__init__()
        self.lat = lat
        self.prec = prec
        self.nrhs = nrhs
        check(load().gbdw_field_create(C.byref(self.h), lat.h, prec, nrhs))

    def load(self, phi: np.ndarray, rhs: int = 0) -> "Field":
        phi = np.ascontiguousarray(phi)
        src = F64 if phi.dtype == np.float64 else F32
        check(load().gbdw_field_import(self.h, rhs, _ptr(phi), src))
        return self

    def numpy(self, rhs: int = 0, dtype=np.float64) -> np.ndarray:
        info = self.lat.info()
        n = info["sites"] * info["Ls"] * 24
        out = np.empty(n, dtype=dtype)
        check(load().gbdw_field_export(self.h, rhs, _ptr(out), F64 if dtype == np.float64 else F32))
        return out

    def export_into(self, out: np.ndarray, rhs: int = 0, sync: bool = True) -> np.ndarray:
        """Writes right-hand side rhs into a preallocated float64/float32 array.  sync=False
        only queues the work on the library stream (out must be page-locked, e.g. a
        PinnedArray's array; complete with synchronize())."""
        fn = load().gbdw_field_export if sync else load().gbdw_field_export_async
        check(fn(self.h, rhs, _ptr(out), F64 if out.dtype == np.float64 else F32))
        return out

    def gaussian(self, seed: int, rhs: int = 0) -> "Field":
        check(load().gbdw_field_gaussian(self.h, rhs, int(seed)))
        return self

    def zero(self):
        check(load().gbdw_field_zero(self.h))

    def copy_from(self, other: "Field"):
        check(load().gbdw_field_copy(self.h, other.h))

    def norm2(self) -> float:
        v = C.c_double()
        check(load().gbdw_norm2(self.h, C.byref(v)))
        return v.value

    def dot(self, other: "Field") -> complex:
        re, im = C.c_double(), C.c_double()
        check(load().gbdw_dot(self.h, other.h, C.byref(re), C.byref(im)))
        return complex(re.value, im.value)

    def axpby(self, a: float, x: "Field", b: float):
        """self = a x + b self"""
        check(load().gbdw_axpby(a, x.h, b, self.h))

    def pick(self, full: "Field") -> "Field":
        """self (a half-lattice field) <- the sites of its parity from full"""
        check(load().gbdw_field_pick(self.h, full.h))
        return self

    def halo_bytes(self, mu: int) -> int:
        n = C.c_size_t()
        check(load().gbdw_halo_bytes(self.h, int(mu), C.byref(n)))
        return n.value

    def halo_pack(self, mu: int, face: int, dag: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        """The spin-projected half spinors of face 0 (x_mu = 0) or 1 (x_mu = L_mu - 1) that the
        neighbouring domain reads (the transport format of include/gbdw.h), as raw bytes."""
        if out is None:
            out = np.empty(self.halo_bytes(mu), dtype=np.uint8)
        check(load().gbdw_halo_pack(self.h, int(mu), int(face), int(dag), _ptr(out)))
        return out

    def halo_pack_all(self, dst_ptrs, dag: int = 0) -> None:
        """All eight faces in one launch into device buffers; dst_ptrs[2*mu + face] are device
        addresses (16-byte aligned) of halo_bytes(mu) bytes each."""
        arr = (C.c_void_p * 8)(*[int(q) for q in dst_ptrs])
        check(load().gbdw_halo_pack_all(self.h, int(dag), arr))

    def place_into(self, full: "Field") -> "Field":
        """full <- self on self's parity (the other parity of full is kept)"""
        check(load().gbdw_field_place(full.h, self.h))
        return full


def dhop(g: Gauge, out: Field, inp: Field, dag: int = 0) -> None:
    check(load().gbdw_dhop(g.h, out.h, inp.h, int(dag)))


def dwf_m(g: Gauge, out: Field, inp: Field, M5: float, mf: float, dag: int = 0, want_norm: bool = False):
    v = C.c_double()
    check(load().gbdw_dwf_m(g.h, out.h, inp.h, M5, mf, int(dag), C.byref(v) if want_norm else None))
    return v.value if want_norm else None


def dwf_mdagm(g: Gauge, out: Field, tmp: Field, inp: Field, M5: float, mf: float) -> float:
    v = C.c_double()
    check(load().gbdw_dwf_mdagm(g.h, out.h, tmp.h, inp.h, M5, mf, C.byref(v)))
    return v.value


def read_static_data(h_path: str, cc_path: str) -> dict:
    """A static_data.h / static_data.cc pair in the reference's format: nsite (outer sites), Ls,
    nsimd and the arrays U, Phi, Psi (the reference result), nbr, prm."""
    L = load()
    ns, ls, nsimd = C.c_uint64(), C.c_int(), C.c_int()
    cnt = (C.c_uint64 * 5)()
    check(L.gbdw_static_data_info(h_path.encode(), cc_path.encode(), C.byref(ns), C.byref(ls), C.byref(nsimd), cnt))
    U, Phi, Psi = (np.empty(cnt[k], np.float64) for k in range(3))
    nbr, prm = np.empty(cnt[3], np.uint64), np.empty(cnt[4], np.uint8)
    check(L.gbdw_static_data_read(cc_path.encode(), _ptr(U), cnt[0], _ptr(Phi), cnt[1], _ptr(Psi), cnt[2],
                                  _ptr(nbr), cnt[3], _ptr(prm), cnt[4]))
    return {"nsite": ns.value, "Ls": ls.value, "nsimd": nsimd.value, "U": U, "Phi": Phi, "Psi": Psi,
            "nbr": nbr, "prm": prm}


def write_static_data(h_path: str, cc_path: str, nsite: int, Ls: int, U, Phi, Psi, nbr, prm, nsimd: int = 1):
    """Writes arrays as a static_data.h / static_data.cc pair the reference's benchmarks compile."""
    U, Phi, Psi = (np.ascontiguousarray(a, dtype=np.float64) for a in (U, Phi, Psi))
    nbr = np.ascontiguousarray(nbr, dtype=np.uint64)
    prm = np.ascontiguousarray(prm, dtype=np.uint8)
    if (U.size != nsite * 144 * nsimd or Phi.size != nsite * Ls * 24 * nsimd or Psi.size != Phi.size
            or nbr.size != nsite * Ls * 8 or prm.size != nbr.size):
        raise ValueError("array lengths disagree with nsite, Ls and nsimd")
    check(load().gbdw_static_data_write(h_path.encode(), cc_path.encode(), nsite, Ls, nsimd, _ptr(U), _ptr(Phi),
                                        _ptr(Psi), _ptr(nbr), _ptr(prm)))


def dhop_eo(g: Gauge, out: Field, inp: Field, dag: int = 0) -> None:
    """out (g's half lattice) = Dhop from the partner half's inp"""
    check(load().gbdw_dhop_eo(g.h, out.h, inp.h, int(dag)))


def dwf_meo(g: Gauge, out: Field, inp: Field, cen: Field, M5: float, mf: float, dag: int = 0,
            khop: float = 0.5) -> None:
    """out = D5 cen - khop Dhop inp on g's half lattice (khop 1/2: M's rows of that parity)"""
    check(load().gbdw_dwf_meo(g.h, out.h, inp.h, cen.h, M5, mf, int(dag), khop))


def dwf_m5inv(out: Field, inp: Field, M5: float, mf: float, dag: int = 0) -> None:
    check(load().gbdw_dwf_m5inv(out.h, inp.h, M5, mf, int(dag)))


def dwf_mpc(gp: Gauge, gq: Gauge, out: Field, tq1: Field, tq2: Field, inp: Field, M5: float, mf: float,
            dag: int = 0, want_norm: bool = False):
    v = C.c_double()
    check(load().gbdw_dwf_mpc(gp.h, gq.h, out.h, tq1.h, tq2.h, inp.h, M5, mf, int(dag),
                              C.byref(v) if want_norm else None))
    return v.value if want_norm else None


def dwf_mpcdagmpc(gp: Gauge, gq: Gauge, out: Field, tp: Field, tq1: Field, tq2: Field, inp: Field, M5: float,
                  mf: float) -> float:
    v = C.c_double()
    check(load().gbdw_dwf_mpcdagmpc(gp.h, gq.h, out.h, tp.h, tq1.h, tq2.h, inp.h, M5, mf, C.byref(v)))
    return v.value


def cg_solve_eo(g64: Sequence[Gauge], x: Field, b: Field, M5: float, mf: float, mode: int, tol: float = 1e-10,
                max_iter: int = 20000, delta: float = 0.1, g32: Sequence[Gauge] | None = None,
                gsloppy: Sequence[Gauge] | None = None, sloppy_prec: int = F16, sloppy_residual: int = 0) -> dict:
    """M x = b by CG on the odd Schur normal system; g64/g32/gsloppy are (even, odd) gauge
    halves.  true_residual is the full system's |b - M x| / |b|."""
    def pair(gs):
        return (C.c_void_p * 2)(gs[0].h.value, gs[1].h.value) if gs is not None else None
    prm = CGParams(tol, max_iter, delta, sloppy_prec, gsloppy[0].prec if gsloppy is not None else F16,
                   int(sloppy_residual))
    st = CGStats()
    status = load().gbdw_cg_solve_eo(pair(g64), pair(g32), pair(gsloppy), x.h, b.h, M5, mf, mode, C.byref(prm),
                                     C.byref(st))
    check(status)
    return {"iterations": st.iterations, "reliable_updates": st.reliable_updates,
            "true_residual": st.true_residual, "seconds": st.seconds, "final_rr": st.final_rr}


# ------------------------------------------------------------------ Mobius / Cayley 5D operators
def _coef(a, Ls: int):
    v = np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (Ls,)))
    return v, v.ctypes.data_as(C.POINTER(C.c_double))


def m5d(out: Field, inp: Field, lower, diag, upper, dag: int = 0) -> None:
    """(A psi)(s) = diag[s] psi(s) + upper[s] P- psi(s+1) + lower[s] P+ psi(s-1), s +- 1 mod Ls;
    dag: the exact adjoint of the same A.  Coefficients: scalars or Ls values."""
    Ls = inp.lat.info()["Ls"]
    (lo, plo), (di, pdi), (up, pup) = _coef(lower, Ls), _coef(diag, Ls), _coef(upper, Ls)
    check(load().gbdw_m5d(out.h, inp.h, plo, pdi, pup, int(dag)))


def m5d_inv(out: Field, inp: Field, lower, diag, upper, dag: int = 0) -> None:
    Ls = inp.lat.info()["Ls"]
    (lo, plo), (di, pdi), (up, pup) = _coef(lower, Ls), _coef(diag, Ls), _coef(upper, Ls)
    check(load().gbdw_m5d_inv(out.h, inp.h, plo, pdi, pup, int(dag)))


def mobius_mooee(out: Field, inp: Field, b: float, c: float, M5: float, mf: float, dag: int = 0) -> None:
    check(load().gbdw_mobius_mooee(out.h, inp.h, b, c, M5, mf, int(dag)))


def mobius_mooee_inv(out: Field, inp: Field, b: float, c: float, M5: float, mf: float, dag: int = 0) -> None:
    check(load().gbdw_mobius_mooee_inv(out.h, inp.h, b, c, M5, mf, int(dag)))


def mobius_m(g: Gauge, out: Field, tmp: Field, inp: Field, b: float, c: float, M5: float, mf: float,
             dag: int = 0, want_norm: bool = False):
    """Mobius domain-wall M (M^dag for dag) on a full lattice: M = Mooee - 1/2 Dhop A(b, c)."""
    v = C.c_double()
    check(load().gbdw_mobius_m(g.h, out.h, tmp.h, inp.h, b, c, M5, mf, int(dag),
                               C.byref(v) if want_norm else None))
    return v.value if want_norm else None


def mobius_meooe(g: Gauge, out: Field, tmp: Field, inp: Field, b: float, c: float, mf: float,
                 dag: int = 0) -> None:
    """Even-odd hopping block on g's half lattice (inp on the partner half)."""
    check(load().gbdw_mobius_meooe(g.h, out.h, tmp.h, inp.h, b, c, mf, int(dag)))


def mobius_mpc(gp: Gauge, gq: Gauge, out: Field, tp: Field, tq1: Field, tq2: Field, inp: Field, b: float,
               c: float, M5: float, mf: float, dag: int = 0, want_norm: bool = False):
    """Schur operator Mpc = Mooee - Meooe_pq Mooee^-1 Meooe_qp on gp's half lattice."""
    v = C.c_double()
    check(load().gbdw_mobius_mpc(gp.h, gq.h, out.h, tp.h, tq1.h, tq2.h, inp.h, b, c, M5, mf, int(dag),
                                 C.byref(v) if want_norm else None))
    return v.value if want_norm else None


def mobius_mdagm(g: Gauge, out: Field, t: Field, tmp: Field, inp: Field, b: float, c: float, M5: float,
                 mf: float) -> float:
    v = C.c_double()
    check(load().gbdw_mobius_mdagm(g.h, out.h, t.h, tmp.h, inp.h, b, c, M5, mf, C.byref(v)))
    return v.value


def cg_solve_mobius(g64: Gauge, x: Field, b: Field, b5: float, c5: float, M5: float, mf: float, mode: int,
                    tol: float = 1e-10, max_iter: int = 20000, delta: float = 0.1, g32: Gauge | None = None,
                    gsloppy: Gauge | None = None, sloppy_prec: int = F16, sloppy_residual: int = 0) -> dict:
    """Mobius M^dag M x = b by CG with reliable updates (modes as cg_solve)."""
    prm = CGParams(tol, max_iter, delta, sloppy_prec, gsloppy.prec if gsloppy is not None else F16,
                   int(sloppy_residual))
    st = CGStats()
    status = load().gbdw_cg_solve_mobius(g64.h, g32.h if g32 is not None else None,
                                         gsloppy.h if gsloppy is not None else None, x.h, b.h, b5, c5, M5, mf,
                                         mode, C.byref(prm), C.byref(st))
    check(status)
    return {"iterations": st.iterations, "reliable_updates": st.reliable_updates,
            "true_residual": st.true_residual, "seconds": st.seconds, "final_rr": st.final_rr}


def cg_solve_mobius_eo(g64: Sequence[Gauge], x: Field, b: Field, b5: float, c5: float, M5: float, mf: float,
                       mode: int, tol: float = 1e-10, max_iter: int = 20000, delta: float = 0.1,
                       g32: Sequence[Gauge] | None = None, gsloppy: Sequence[Gauge] | None = None,
                       sloppy_prec: int = F16, sloppy_residual: int = 0) -> dict:
    """Mobius M x = b by CG on the odd Schur normal system; g64/g32/gsloppy are (even, odd)
    gauge halves.  true_residual is the full system's |b - M x| / |b|."""
    def pair(gs):
        return (C.c_void_p * 2)(gs[0].h.value, gs[1].h.value) if gs is not None else None
    prm = CGParams(tol, max_iter, delta, sloppy_prec, gsloppy[0].prec if gsloppy is not None else F16,
                   int(sloppy_residual))
    st = CGStats()
    check(load().gbdw_cg_solve_mobius_eo(pair(g64), pair(g32), pair(gsloppy), x.h, b.h, b5, c5, M5, mf, mode,
                                         C.byref(prm), C.byref(st)))
    return {"iterations": st.iterations, "reliable_updates": st.reliable_updates,
            "true_residual": st.true_residual, "seconds": st.seconds, "final_rr": st.final_rr}


def cg_solve(g64: Gauge, x: Field, b: Field, M5: float, mf: float, mode: int, tol: float = 1e-10,
             max_iter: int = 20000, delta: float = 0.1, g32: Gauge | None = None, gsloppy: Gauge | None = None,
             sloppy_prec: int = F16, sloppy_residual: int = 0) -> dict:
    """M^dag M x = b (Shamir) by CG with reliable updates.  sloppy_residual = 1 keeps the mixed
    mode's iterated residual in FP16 (FP16 spinors and links only)."""
    prm = CGParams(tol, max_iter, delta, sloppy_prec, gsloppy.prec if gsloppy is not None else F16,
                   int(sloppy_residual))
    st = CGStats()
    status = load().gbdw_cg_solve(g64.h, g32.h if g32 is not None else None,
                                  gsloppy.h if gsloppy is not None else None, x.h, b.h, M5, mf, mode,
                                  C.byref(prm), C.byref(st))
    check(status)
    return {"iterations": st.iterations, "reliable_updates": st.reliable_updates,
            "true_residual": st.true_residual, "seconds": st.seconds, "final_rr": st.final_rr}


class Batch(_Handle):
    _destroy = "gbdw_batch_destroy"

    def __init__(self, gauges: Sequence[Gauge], outs: Sequence[Field], ins: Sequence[Field], dag: int = 0):
        super().__init__()
        n = len(gauges)
        self._keep = (list(gauges), list(outs), list(ins))
        G = (C.c_void_p * n)(*[g.h.value for g in gauges])
        O = (C.c_void_p * n)(*[o.h.value for o in outs])
        I = (C.c_void_p * n)(*[i.h.value for i in ins])
        check(load().gbdw_batch_create(C.byref(self.h), n, G, O, I, int(dag)))

    def run(self):
        check(load().gbdw_batch_run(self.h))

    def set_shape(self, threads: int, spt_f32: int, spt_f16: int, split: int):
        """Pins the launch shape and the tile split (rebuilds the graph)."""
        check(load().gbdw_batch_set_shape(self.h, (C.c_int * 4)(threads, spt_f32, spt_f16, split)))

    def info(self) -> dict:
        a = (C.c_int64 * 4)()
        check(load().gbdw_batch_info(self.h, a))
        s = (C.c_int * 4)()
        check(load().gbdw_batch_shape(self.h, s))
        return {"items": a[0], "ctas": a[1], "threads": a[2], "graph": bool(a[3]), "spt_f32": s[1], "spt_f16": s[2],
                "tile_split": s[3]}


def tune_dhop(g: Gauge, out: Field, inp: Field, dag: int = 0) -> tuple:
    check(load().gbdw_tune_dhop(g.h, out.h, inp.h, int(dag)))
    return tune_query(g, inp)


def tune_query(g: Gauge, inp: Field) -> tuple:
    """(threads per CTA, slices per thread, form, stages); form 0 direct loads, 1 TMA-staged
    CTA ring, 2 TMA-staged ring per warp, 3 direct FP32/FP16 kernel specialised for Ls*nrhs = 16, 4 the same over 2x2x2x2 site blocks."""
    cfg = (C.c_int * 4)()
    check(load().gbdw_tune_query(g.h, inp.h, cfg))
    return tuple(int(v) for v in cfg)


def tune_set(g: Gauge, inp: Field, threads: int, spt: int, form: int = 0, stages: int = 4):
    check(load().gbdw_tune_set(g.h, inp.h, threads, spt, form, stages))


def tune_split(g: Gauge, inp: Field) -> int:
    """Tiles per site (Ls / RHS tiling) of the direct form chosen for fields like inp."""
    v = C.c_int()
    check(load().gbdw_tune_split(g.h, inp.h, C.byref(v)))
    return v.value


def tune_set_split(g: Gauge, inp: Field, split: int):
    check(load().gbdw_tune_set_split(g.h, inp.h, int(split)))


def tune_brick(g: Gauge, inp: Field) -> int:
    """t-brick sweep order of the direct form chosen for fields like inp (1: natural order)."""
    v = C.c_int()
    check(load().gbdw_tune_brick(g.h, inp.h, C.byref(v)))
    return v.value


def tune_set_brick(g: Gauge, inp: Field, brick: int):
    check(load().gbdw_tune_set_brick(g.h, inp.h, int(brick)))


def set_fp64_arith(where: int, mode: int) -> None:
    """FP64 operators in native FP64 (FP64_NATIVE) or on FP32 pairs (FP64_DOUBLE_SINGLE, ~1e-14
    relative), for explicit operator calls (FP64_OPERATORS) or the solvers (FP64_SOLVERS)."""
    check(load().gbdw_set_fp64_arith(int(where), int(mode)))


def tune_query_ds(g: Gauge, inp: Field, epi: int = 0) -> tuple:
    """(CTAs per SM of the register cap, t-brick) of the double-single FP64 operator, for Dhop
    (epi 0) or M (epi 1)."""
    cfg = (C.c_int * 2)()
    check(load().gbdw_tune_query_ds(g.h, inp.h, int(epi), cfg))
    return tuple(int(v) for v in cfg)


def tune_set_ds(g: Gauge, inp: Field, epi: int, minb: int, brick: int = 1) -> None:
    check(load().gbdw_tune_set_ds(g.h, inp.h, int(epi), int(minb), int(brick)))


def get_fp64_arith(where: int) -> int:
    v = C.c_int()
    check(load().gbdw_get_fp64_arith(int(where), C.byref(v)))
    return v.value


def tune_query_m(g: Gauge, inp: Field) -> tuple:
    """(threads, slices per thread, form, stages, split, brick) of the Shamir M pass and the CG
    passes built on it, for fields like inp with one right-hand side."""
    cfg = (C.c_int * 6)()
    check(load().gbdw_tune_query_m(g.h, inp.h, cfg))
    return tuple(int(v) for v in cfg)


def tune_query_cg(g: Gauge, inp: Field, rprec: int) -> tuple:
    """The same six numbers for the fused CG step (M^dag M with the residual update) with an
    iterated residual of precision rprec (F64, F32 or F16)."""
    cfg = (C.c_int * 6)()
    check(load().gbdw_tune_query_cg(g.h, inp.h, int(rprec), cfg))
    return tuple(int(v) for v in cfg)


def tune_save(path: str):
    check(load().gbdw_tune_save(path.encode()))


def tune_load(path: str):
    check(load().gbdw_tune_load(path.encode()))


class Stream:
    """A non-blocking CUDA stream of the library; `with s:` makes the library queue on it."""

    def __init__(self):
        self.h = C.c_void_p()
        check(load().gbdw_stream_create(C.byref(self.h)))

    def __enter__(self):
        check(load().gbdw_set_stream(self.h))
        return self

    def __exit__(self, *exc):
        load().gbdw_set_stream(None)

    def synchronize(self):
        with self:
            synchronize()

    def close(self):
        if self.h and self.h.value:
            load().gbdw_stream_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PinnedArray:
    """numpy view of page-locked host memory (freed with the object)."""

    def __init__(self, n: int, dtype=np.float32):
        self.ptr = C.c_void_p()
        nbytes = int(n) * np.dtype(dtype).itemsize
        check(load().gbdw_host_alloc(nbytes, C.byref(self.ptr)))
        buf = (C.c_char * nbytes).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(n))

    def close(self):
        if self.ptr and self.ptr.value:
            self.array = None
            load().gbdw_host_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Timer(_Handle):
    """CUDA-event timer on the library stream."""
    _destroy = "gbdw_timer_destroy"

    def __init__(self):
        super().__init__()
        check(load().gbdw_timer_create(C.byref(self.h)))

    def start(self):
        check(load().gbdw_timer_start(self.h))

    def stop(self) -> float:
        ms = C.c_double()
        check(load().gbdw_timer_stop(self.h, C.byref(ms)))
        return ms.value


def dslash_kernel(nrep: int, U: np.ndarray, out: np.ndarray, inp: np.ndarray, nbr: np.ndarray, nsite: int, Ls: int,
                  prm: np.ndarray | None, nsimd: int = 1, dag: int = 0) -> float:
    """The reference seam dslash_kernel(nrep, U, out, in, nbr, nsite, Ls, prm)
    (WilsonKernelsHand.h:17-29): applies the hopping term nrep times on the GPU and writes
    `out`; returns microseconds over repetitions 1..nrep-1.  Precision follows the arrays
    (float64 -> vComplexD, float32 -> vComplexF)."""
    if not (U.dtype == out.dtype == inp.dtype) or U.dtype not in (np.float64, np.float32):
        raise TypeError("U, out and in must share dtype float64 or float32")
    for a in (U, out, inp):
        if not a.flags.c_contiguous:
            raise ValueError("arrays must be C-contiguous")
    prec = F64 if U.dtype == np.float64 else F32
    nbr = np.ascontiguousarray(nbr, dtype=np.uint64)
    prm_p = None
    if prm is not None:
        prm = np.ascontiguousarray(prm, dtype=np.uint8)
        prm_p = _ptr(prm)
    usec = C.c_double()
    check(load().gbdw_dslash_kernel(nrep, prec, nsimd, _ptr(U), _ptr(out), _ptr(inp), _ptr(nbr), nsite, Ls, prm_p,
                                    int(dag), C.byref(usec)))
    return usec.value
