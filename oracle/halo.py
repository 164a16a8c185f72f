"""ORACLE -- test infrastructure only.

The spin projection and reconstruction of each hopping leg, restated with numpy from the
per-leg macros of GridBench's hand kernel (WilsonKernelsHandCpu.h:94-303, the projector and
reconstruct pairs used at :435-442), and the pieces a 4D domain decomposition of the hopping
term needs: the face sites of a local volume, the projected half spinors a face sends, and the
contribution such a half spinor makes at the receiving site (u = U h, then reconstruct).

Leg order Xp, Yp, Zp, Tp, Xm, Ym, Zm, Tm (WilsonKernelsHand.h:5-12).  DhopDag uses each leg's
opposite-sign partner's spin structure with the same link and neighbour.
"""
from __future__ import annotations

import numpy as np

# h0 = psi0 + a * psi[A],  h1 = psi1 + b * psi[B]
PROJ = {
    0: ((3, -1j), (2, -1j)),  # Xp
    1: ((3, 1), (2, -1)),     # Yp
    2: ((2, -1j), (3, 1j)),   # Zp
    3: ((2, -1), (3, -1)),    # Tp
    4: ((3, 1j), (2, 1j)),    # Xm
    5: ((3, -1), (2, 1)),     # Ym
    6: ((2, 1j), (3, -1j)),   # Zm
    7: ((2, 1), (3, 1)),      # Tm
}
# r0 += u0, r1 += u1;  r2 += c2 * u[k2],  r3 += c3 * u[k3]
RECON = {
    0: ((1, 1j), (0, 1j)),
    1: ((1, -1), (0, 1)),
    2: ((0, 1j), (1, -1j)),
    3: ((0, -1), (1, -1)),
    4: ((1, -1j), (0, -1j)),
    5: ((1, 1), (0, -1)),
    6: ((0, -1j), (1, 1j)),
    7: ((0, 1), (1, 1)),
}


def project(psi: np.ndarray, leg: int) -> np.ndarray:
    """psi (..., 4, 3) complex -> (..., 2, 3): the leg's half spinor."""
    (A, a), (B, b) = PROJ[leg]
    return np.stack([psi[..., 0, :] + a * psi[..., A, :], psi[..., 1, :] + b * psi[..., B, :]], axis=-2)


def reconstruct(u: np.ndarray, leg: int) -> np.ndarray:
    """u = U h (..., 2, 3) -> the leg's full-spinor contribution (..., 4, 3)."""
    (k2, c2), (k3, c3) = RECON[leg]
    return np.stack([u[..., 0, :], u[..., 1, :], c2 * u[..., k2, :], c3 * u[..., k3, :]], axis=-2)


def site_index(c, dims) -> int:
    return int(c[0] + dims[0] * (c[1] + dims[1] * (c[2] + dims[2] * c[3])))


def face_sites(dims, mu: int, xmu: int) -> np.ndarray:
    """Sites with x_mu = xmu, the three other coordinates lexicographic (lowest fastest)."""
    others = [d for d in range(4) if d != mu]
    out = []
    for k in range(dims[others[2]]):
        for j in range(dims[others[1]]):
            for i in range(dims[others[0]]):
                c = [0, 0, 0, 0]
                c[others[0]], c[others[1]], c[others[2]], c[mu] = i, j, k, xmu
                out.append(site_index(c, dims))
    return np.array(out, dtype=np.int64)


def pack(phi: np.ndarray, dims, Ls: int, mu: int, face: int, dag: int = 0) -> np.ndarray:
    """The half spinors (nface, Ls, 2, 3) a local field (reference layout) sends across face 0
    (x_mu = 0, read through the receiver's forward leg mu) or face 1 (x_mu = L_mu - 1, read
    through its backward leg mu + 4)."""
    psi = np.ascontiguousarray(phi, dtype=np.float64).view(np.complex128).reshape(-1, Ls, 4, 3)
    sites = face_sites(dims, mu, 0 if face == 0 else dims[mu] - 1)
    leg = (mu if face == 0 else mu + 4) ^ (4 if dag else 0)
    return project(psi[sites], leg)


def halo_contribution(U: np.ndarray, site: int, leg: int, h: np.ndarray, dag: int = 0) -> np.ndarray:
    """(Ls, 4, 3): leg `leg` of `site` fed by the received half spinors h (Ls, 2, 3); U is the
    reference-layout doubled gauge field of the receiving domain's sites."""
    Ux = np.ascontiguousarray(U, dtype=np.float64).view(np.complex128).reshape(-1, 8, 3, 3)[site, leg]
    u = np.einsum("rc,shc->shr", Ux, h)
    return reconstruct(u, leg ^ (4 if dag else 0))
