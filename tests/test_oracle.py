"""The oracle (CPU restatement) pinned to GridBench's own kernels and golden vectors."""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, make_case, rel_err


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "golden_simple_*.npz"))))
def test_oracle_matches_dslash_simple_golden(f):
    g = np.load(f)
    c = make_case(tuple(g["dims"]), int(g["Ls"]))
    out = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], c["Ls"])
    np.testing.assert_array_equal(out, g["psi"])  # bit-exact, same operation order


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "golden_hand_*.npz"))))
def test_oracle_lanes_matches_hand_kernel_golden(f):
    g = np.load(f)
    ns = int(g["nsimd"])
    dt = np.float64 if "f64" in os.path.basename(f) else np.float32
    c = make_case(tuple(g["dims"]), int(g["Ls"]), ns)
    out = oracle.dslash_lanes(c["U"].astype(dt), c["phi"].astype(dt), c["nbr"], c["prm"], c["nsite"], c["Ls"], ns)
    tol = 1e-14 if dt == np.float64 else 2e-7
    assert rel_err(out, g["psi"]) < tol


def test_oracle_matches_reference_build_when_present():
    ref = oracle.ref()
    if ref is None:
        pytest.skip("reference tree not present on this host")
    c = make_case((4, 4, 2, 6), 5)
    psi = np.zeros_like(c["phi"])
    ref.ref_dslash_kernel(c["U"], psi, c["phi"], c["nbr"], c["nsite"], c["Ls"], c["prm"])
    out = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], c["Ls"])
    np.testing.assert_array_equal(out, psi)
    psi2 = np.zeros_like(psi)
    ref.ref_dslash_kernel_unroll(c["U"], psi2, c["phi"], c["nbr"], c["nsite"], c["Ls"], c["prm"])
    np.testing.assert_array_equal(psi2, psi)


def test_lane_and_scalar_oracles_agree():
    a = make_case((4, 4, 4, 4), 2, 1)
    b = make_case((4, 4, 4, 4), 2, 4)
    oa = oracle.dslash(a["U"], a["phi"], a["nbr"], a["prm"], a["nsite"], 2)
    ob = oracle.dslash_lanes(b["U"], b["phi"], b["nbr"], b["prm"], b["nsite"], 2, 4)
    np.testing.assert_array_equal(np.sort(oa), np.sort(ob))


def _cdot(x, y):
    xc = x[0::2] + 1j * x[1::2]
    yc = y[0::2] + 1j * y[1::2]
    return np.vdot(xc, yc)


def test_dhopdag_is_adjoint():
    c = make_case((4, 4, 2, 2), 3)
    y = c["phi"]
    x = make_case((4, 4, 2, 2), 3, fseeds=(9, 9, 9, 9))["phi"]
    Dy = oracle.dslash(c["U"], y, c["nbr"], c["prm"], c["nsite"], 3, 0)
    Ddx = oracle.dslash(c["U"], x, c["nbr"], c["prm"], c["nsite"], 3, 1)
    a, b = _cdot(x, Dy), _cdot(Ddx, y)
    assert abs(a - b) / abs(a) < 1e-13


def test_dwf_m_is_adjoint_and_mdagm_positive():
    c = make_case((2, 2, 4, 2), 6)
    y = c["phi"]
    x = make_case((2, 2, 4, 2), 6, fseeds=(3, 1, 4, 1))["phi"]
    My = oracle.dwf_m(c["U"], y, c["nbr"], c["nsite"], 6, 1.8, 0.01, 0)
    Mdx = oracle.dwf_m(c["U"], x, c["nbr"], c["nsite"], 6, 1.8, 0.01, 1)
    a, b = _cdot(x, My), _cdot(Mdx, y)
    assert abs(a - b) / abs(a) < 1e-13
    A = oracle.dwf_mdagm(c["U"], y, c["nbr"], c["nsite"], 6, 1.8, 0.01)
    assert _cdot(y, A).real > 0
    assert abs(_cdot(y, A).imag) / abs(_cdot(y, A).real) < 1e-13


def test_dwf_m_free_field_structure():
    """With Dhop switched off (unit links are not needed: compare against the explicit
    5D formula on one site) the 5D terms follow P+/P- and -mf at the wall."""
    c = make_case((2, 2, 2, 2), 4)
    U0 = np.zeros_like(c["U"])  # Dhop == 0
    phi = c["phi"]
    out = oracle.dwf_m(U0, phi, c["nbr"], c["nsite"], 4, 1.8, 0.01, 0)
    P = phi.reshape(c["nsite"], 4, 12, 2)
    O = out.reshape(c["nsite"], 4, 12, 2)
    a5 = 5 - 1.8
    for s in range(4):
        up = P[:, (s + 1) % 4] * (-0.01 if s == 3 else 1.0)
        dn = P[:, (s - 1) % 4] * (-0.01 if s == 0 else 1.0)
        exp = a5 * P[:, s].copy()
        exp[:, :6] -= dn[:, :6]
        exp[:, 6:] -= up[:, 6:]
        np.testing.assert_allclose(O[:, s], exp, rtol=0, atol=1e-14)
