"""Input generator (TableGenerate.cc's role): SU(3) links, doubled field, tables, layouts."""
import hashlib
import glob
import os

import numpy as np
import pytest

import gridbench_gb300 as gb
from conftest import GOLDEN, make_case


def _links(U):
    return (U[0::2] + 1j * U[1::2]).reshape(-1, 8, 3, 3)


def test_su3_unitary_det_one():
    U = _links(gb.generate_gauge((4, 4, 4, 4)))
    M = U.reshape(-1, 3, 3)
    eye = np.eye(3)
    assert np.abs(M @ M.conj().transpose(0, 2, 1) - eye).max() < 1e-13
    assert np.abs(np.linalg.det(M) - 1).max() < 1e-13


def test_doubled_links_are_backward_daggers():
    dims = (4, 3, 2, 5)
    U = _links(gb.generate_gauge(dims))
    Lx, Ly, Lz, Lt = dims
    for site in range(0, Lx * Ly * Lz * Lt, 7):
        x = [site % Lx, (site // Lx) % Ly, (site // (Lx * Ly)) % Lz, site // (Lx * Ly * Lz)]
        for mu in range(4):
            y = list(x)
            y[mu] = (y[mu] - 1) % dims[mu]
            back = y[0] + Lx * (y[1] + Ly * (y[2] + Lz * y[3]))
            np.testing.assert_array_equal(U[site, mu + 4], U[back, mu].conj().T)


def test_gaussian_source_moments():
    phi = gb.generate_fermion((8, 8, 8, 8), 4)
    assert abs(phi.mean()) < 0.01
    assert abs(phi.var() - 1.0) < 0.01


def test_table_bijective_and_inverse():
    dims, Ls = (4, 6, 2, 4), 3
    nbr, prm, nsite = gb.generate_table(dims, Ls)
    t = nbr.reshape(nsite * Ls, 8)
    assert prm.sum() == 0
    for mu in range(8):
        assert len(np.unique(t[:, mu])) == nsite * Ls  # a permutation of the 5D sites
        back = t[t[:, mu], (mu + 4) % 8]
        np.testing.assert_array_equal(back, np.arange(nsite * Ls))
    # nbr5 = nbr4 * Ls + s
    s = np.arange(nsite * Ls) % Ls
    assert np.all(t % Ls == s[:, None])


@pytest.mark.parametrize("nsimd", [2, 4, 8, 16])
def test_lane_layout_is_same_field(nsimd):
    """The lane layout is a reordering of the scalar layout: same global field."""
    dims, Ls = (4, 4, 4, 4), 2
    a = make_case(dims, Ls, 1)
    b = make_case(dims, Ls, nsimd)
    np.testing.assert_array_equal(np.sort(a["U"]), np.sort(b["U"]))
    np.testing.assert_array_equal(np.sort(a["phi"]), np.sort(b["phi"]))
    assert b["prm"].sum() > 0


def test_generator_reproduces_golden_inputs():
    """Bit-identical generation (no libm transcendental, no FP contraction)."""
    files = sorted(glob.glob(os.path.join(GOLDEN, "golden_simple_*.npz")))
    assert files
    for f in files:
        g = np.load(f)
        c = make_case(tuple(g["dims"]), int(g["Ls"]))
        for k in ("U", "phi", "nbr", "prm"):
            assert hashlib.sha256(np.ascontiguousarray(c[k]).tobytes()).hexdigest() == str(g["sha_" + k]), k


def test_generator_rejects_bad_dims():
    with pytest.raises(gb.GbdwError):
        gb.generate_gauge((3, 4, 4, 4), nsimd=16)  # x not divisible by its lane split
    with pytest.raises(gb.GbdwError):
        gb.generate_table((4, 4, 4, 4), 2, nsimd=3)


def _oracle_case(dims, Ls, nsimd=1):
    import oracle
    nbr, prm, nsite = oracle.generate_table(dims, Ls, nsimd)
    return {"U": oracle.generate_gauge(dims, nsimd), "phi": oracle.generate_fermion(dims, Ls, nsimd), "nbr": nbr,
            "prm": prm, "nsite": nsite}


@pytest.mark.parametrize("dims,Ls,nsimd", [((4, 4, 4, 4), 4, 1), ((4, 6, 2, 4), 3, 1), ((8, 8, 8, 8), 8, 4),
                                           ((4, 4, 4, 8), 2, 16), ((2, 4, 4, 4), 3, 8), ((6, 2, 2, 10), 1, 2)])
def test_oracle_generator_is_bit_identical_to_product(dims, Ls, nsimd):
    """The oracle's own generator (oracle/gen.c, used by the reference-side CPU runs so they
    never load the product library) and the product's gbdw_generate_* give the same bits."""
    a = _oracle_case(dims, Ls, nsimd)
    b = make_case(dims, Ls, nsimd)
    for k in ("U", "phi", "nbr", "prm"):
        assert np.ascontiguousarray(a[k]).tobytes() == np.ascontiguousarray(b[k]).tobytes(), k
    assert a["nsite"] == b["nsite"]


def test_oracle_generator_reproduces_golden_inputs():
    import oracle
    for f in sorted(glob.glob(os.path.join(GOLDEN, "golden_*.npz"))):
        g = np.load(f)
        c = _oracle_case(tuple(g["dims"]), int(g["Ls"]), int(g["nsimd"]))
        for k in ("U", "phi", "nbr", "prm"):
            if "sha_" + k in g:
                assert hashlib.sha256(np.ascontiguousarray(c[k]).tobytes()).hexdigest() == str(g["sha_" + k]), (f, k)
    assert oracle.seed_from_ints((1, 2, 3, 4)) == gb.seed_from_ints((1, 2, 3, 4))
    with pytest.raises(ValueError):
        oracle.generate_gauge((3, 4, 4, 4), nsimd=16)
