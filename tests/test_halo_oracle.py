"""The halo oracle: its per-leg projection/reconstruction table rebuilds the full hopping term
of the pinned Dhop oracle, and a two-domain decomposition fed only by packed half spinors
reproduces the full-lattice Dhop (CPU, numpy)."""
import numpy as np
import pytest

import oracle
from oracle import halo
from conftest import make_case, rel_err


def _dhop_from_table(c, dag):
    Ls, ns = c["Ls"], c["nsite"]
    psi = c["phi"].view(np.complex128).reshape(ns, Ls, 4, 3)
    U = c["U"].view(np.complex128).reshape(ns, 8, 3, 3)
    nb = (c["nbr"].reshape(ns, Ls, 8)[:, 0, :] // Ls).astype(np.int64)
    out = np.zeros_like(psi)
    for leg in range(8):
        sleg = leg ^ (4 if dag else 0)
        h = halo.project(psi[nb[:, leg]], sleg)
        u = np.einsum("nrc,nshc->nshr", U[:, leg], h)
        out += halo.reconstruct(u, sleg)
    return out.reshape(-1).view(np.float64)


@pytest.mark.parametrize("dag", [0, 1])
def test_leg_table_rebuilds_the_dhop_oracle(dag):
    c = make_case((4, 2, 2, 4), 3)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 3, dag)
    assert rel_err(_dhop_from_table(c, dag), ref) < 1e-14


def split(c, mu):
    """Global (4,4,4,4) case split in direction mu into A (x_mu < 2) and B (x_mu >= 2): local
    dims, the global site of each local site, and the local fields."""
    G = c["dims"]
    D = list(G)
    D[mu] = G[mu] // 2
    Ls = c["Ls"]
    psi = c["phi"].view(np.complex128).reshape(-1, Ls, 12)
    maps = []
    for off in (0, D[mu]):
        m = []
        for t in range(D[3]):
            for z in range(D[2]):
                for y in range(D[1]):
                    for x in range(D[0]):
                        g = [x, y, z, t]
                        g[mu] += off
                        m.append(halo.site_index(g, G))
        maps.append(np.array(m))
    fields = [np.ascontiguousarray(psi[m]).reshape(-1).view(np.float64) for m in maps]
    return tuple(D), maps, fields


def domain_dhop(c, mu, dag, D, maps, halos_from_A):
    """Dhop on B's sites from B's own spinors and A's packed faces: the full-lattice oracle on
    a field with A's sites zeroed gives every leg that stays inside B; each leg that crosses
    into A adds U h for the received half spinor h."""
    Ls = c["Ls"]
    phiB = c["phi"].view(np.complex128).reshape(-1, Ls, 12).copy()
    phiB[maps[0]] = 0
    inner = oracle.dslash(c["U"], phiB.reshape(-1).view(np.float64), c["nbr"], c["prm"], c["nsite"], Ls, dag)
    out = inner.view(np.complex128).reshape(-1, Ls, 4, 3)[maps[1]].copy()
    lo, hi = halos_from_A  # A's face 0 (x_mu = 0) and face 1 (x_mu = L - 1)
    faceB0 = halo.face_sites(D, mu, 0)            # B's local x_mu = 0: backward leg into A's high face
    faceB1 = halo.face_sites(D, mu, D[mu] - 1)    # B's last slab: forward leg into A's low face (wrap)
    for f, ls in enumerate(faceB0):
        out[ls] += halo.halo_contribution(c["U"], maps[1][ls], mu + 4, hi[f], dag)
    for f, ls in enumerate(faceB1):
        out[ls] += halo.halo_contribution(c["U"], maps[1][ls], mu, lo[f], dag)
    return out.reshape(-1).view(np.float64)


@pytest.mark.parametrize("mu", [0, 1, 2, 3])
@pytest.mark.parametrize("dag", [0, 1])
def test_two_domains_fed_by_packed_halos(mu, dag):
    c = make_case((4, 4, 4, 4), 4)
    D, maps, (fa, fb) = split(c, mu)
    halos = (halo.pack(fa, D, 4, mu, 0, dag), halo.pack(fa, D, 4, mu, 1, dag))
    got = domain_dhop(c, mu, dag, D, maps, halos)
    full = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 4, dag)
    ref = full.view(np.complex128).reshape(-1, 4, 12)[maps[1]].reshape(-1).view(np.float64)
    assert rel_err(got, ref) < 1e-14
