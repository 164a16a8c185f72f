"""ORACLE -- test infrastructure only.

Mobius (Cayley-form) domain-wall operators restated with numpy on the reference layout
(Psi[(site*Ls + s)*12 + spin*3 + colour], dslash_simple.h:3,144).  GridBench has no
5th-dimension operators; the structure is Grid's CayleyFermion5D (M5D / Mooee / MooeeInv /
Meooe around WilsonFermion5D's Dhop; Grid is the un-vendored library TableGenerate.cc:8 links
against, no version pinned) with the Mobius kernel of Brower, Neff and Orginos
(arXiv:1206.5214).  The 5th-dimension parts are written as dense Ls x Ls matrices per
chirality (P+ = spins 0,1 and P- = spins 2,3 in the chiral basis of WilsonKernelsHandCpu.h),
their adjoints as transposes and inverses by LAPACK -- a different method from the library's
recursions.  The hopping term is the oracle's restatement of dslash_simple.h.  With b = 1,
c = 0 the Mobius operator is the Shamir operator of `oracle.dwf_m`, which pins it.
"""
from __future__ import annotations

import numpy as np


def _cx(phi: np.ndarray, Ls: int) -> np.ndarray:
    return np.ascontiguousarray(phi, dtype=np.float64).view(np.complex128).reshape(-1, Ls, 12)


def _flat(x: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(x).view(np.float64).reshape(-1)


def matrices(Ls: int, lower, diag, upper):
    """(A psi)(s) = diag[s] psi(s) + upper[s] P- psi(s+1) + lower[s] P+ psi(s-1), cyclic in s:
    the P+ matrix (spins 0,1) and the P- matrix (spins 2,3)."""
    lower, diag, upper = (np.broadcast_to(np.asarray(a, dtype=np.float64), (Ls,)) for a in (lower, diag, upper))
    mp = np.diag(diag).astype(np.float64)
    mm = np.diag(diag).astype(np.float64)
    for s in range(Ls):
        mp[s, (s - 1) % Ls] += lower[s]
        mm[s, (s + 1) % Ls] += upper[s]
    return mp, mm


def _apply(mp, mm, phi, Ls):
    x = _cx(phi, Ls)
    out = np.empty_like(x)
    out[:, :, :6] = np.einsum("st,ntk->nsk", mp, x[:, :, :6])
    out[:, :, 6:] = np.einsum("st,ntk->nsk", mm, x[:, :, 6:])
    return _flat(out)


def m5d(phi, Ls, lower, diag, upper, dag=0):
    mp, mm = matrices(Ls, lower, diag, upper)
    if dag:
        mp, mm = mp.T, mm.T
    return _apply(mp, mm, phi, Ls)


def m5d_inv(phi, Ls, lower, diag, upper, dag=0):
    mp, mm = matrices(Ls, lower, diag, upper)
    if dag:
        mp, mm = mp.T, mm.T
    return _apply(np.linalg.inv(mp), np.linalg.inv(mm), phi, Ls)


def cyclic(Ls, d, e, mf, scale=1.0):
    """A(d, e): diag d, lower = upper = e, the walls (upper[Ls-1], lower[0]) e -> -mf e."""
    lower = np.full(Ls, scale * e)
    upper = np.full(Ls, scale * e)
    upper[Ls - 1] = -mf * scale * e
    lower[0] = -mf * scale * e
    return lower, np.full(Ls, scale * d), upper


def mooee_coef(Ls, b, c, M5, mf):
    return cyclic(Ls, 1.0 + b * (4.0 - M5), -(1.0 - c * (4.0 - M5)), mf)


def meo5_coef(Ls, b, c, mf):
    return cyclic(Ls, b, c, mf)


def mobius_m(U, phi, nbr, prm, nsite, Ls, b, c, M5, mf, dag=0):
    """M = Mooee - 1/2 Dhop A(b, c);  M^dag = Mooee^dag - 1/2 A(b, c)^dag DhopDag."""
    from . import dslash
    oo, eo = mooee_coef(Ls, b, c, M5, mf), meo5_coef(Ls, b, c, mf)
    if not dag:
        t = m5d(phi, Ls, *eo)
        return m5d(phi, Ls, *oo) - 0.5 * dslash(U, t, nbr, prm, nsite, Ls, 0)
    t = dslash(U, np.ascontiguousarray(phi, dtype=np.float64), nbr, prm, nsite, Ls, 1)
    return m5d(phi, Ls, *oo, dag=1) - 0.5 * m5d(t, Ls, *eo, dag=1)
