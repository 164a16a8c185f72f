"""The Mobius oracle (numpy restatement) pinned to the Shamir oracle and to its own algebra."""
import numpy as np
import pytest

import oracle
from oracle import mobius as mob
from conftest import make_case, rel_err

M5, MF = 1.8, 0.01


def _cdot(a, b):
    a = a.view(np.complex128)
    b = b.view(np.complex128)
    return complex(np.vdot(a, b))


@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("Ls", [1, 2, 5, 8])
def test_mobius_b1_c0_is_the_shamir_oracle(dag, Ls):
    c = make_case((4, 2, 2, 4), Ls)
    out = mob.mobius_m(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, 1.0, 0.0, M5, MF, dag)
    ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, dag)
    assert rel_err(out, ref) < 1e-14


def test_mobius_adjoint_pair():
    c = make_case((4, 2, 2, 4), 6)
    c2 = make_case((4, 2, 2, 4), 6, fseeds=(9, 10, 11, 12))
    x, y = c["phi"], c2["phi"]
    args = (c["U"], None, c["nbr"], c["prm"], c["nsite"], 6, 1.5, 0.5, M5, MF)
    my = mob.mobius_m(args[0], y, *args[2:])
    mdx = mob.mobius_m(args[0], x, *args[2:], dag=1)
    a, b = _cdot(x, my), _cdot(mdx, y)
    assert abs(a - b) / abs(a) < 1e-13


@pytest.mark.parametrize("dag", [0, 1])
def test_m5d_inverse_and_adjoint(dag):
    Ls = 7
    rng = np.random.default_rng(3)
    lo, di, up = rng.normal(size=Ls), 3.0 + rng.random(Ls), rng.normal(size=Ls)
    c = make_case((2, 2, 2, 2), Ls)
    x = c["phi"]
    y = mob.m5d(x, Ls, lo, di, up, dag)
    assert rel_err(mob.m5d_inv(y, Ls, lo, di, up, dag), x) < 1e-13
    z = make_case((2, 2, 2, 2), Ls, fseeds=(1, 1, 2, 3))["phi"]
    a = _cdot(z, mob.m5d(x, Ls, lo, di, up, 0))
    b = _cdot(mob.m5d(z, Ls, lo, di, up, 1), x)
    assert abs(a - b) / abs(a) < 1e-13


@pytest.mark.parametrize("Ls", [1, 4, 7])
def test_mobius_split_equals_the_published_cayley_form(Ls):
    """Mooee + Meooe equals the Mobius kernel as Brower, Neff and Orginos write it,
    (b D_W + 1) psi_s + (c D_W - 1) chi_s with chi_s = P- psi_(s+1) + P+ psi_(s-1) (walls -mf) and
    D_W = (4 - M5) - 1/2 Dhop, computed here from the Dhop oracle directly."""
    b5, c5 = 1.5, 0.5
    c = make_case((4, 2, 2, 4), Ls)
    phi = c["phi"]
    psi = phi.view(np.complex128).reshape(-1, Ls, 12)
    chi = np.zeros_like(psi)
    for s in range(Ls):
        up, dn = (s + 1) % Ls, (s - 1) % Ls
        fu = -MF if s == Ls - 1 else 1.0
        fd = -MF if s == 0 else 1.0
        chi[:, s, 6:] = fu * psi[:, up, 6:]   # P- psi(s+1)
        chi[:, s, :6] = fd * psi[:, dn, :6]   # P+ psi(s-1)
    chiv = chi.reshape(-1).view(np.float64)

    def dw(v):
        return (4.0 - M5) * v - 0.5 * oracle.dslash(c["U"], np.ascontiguousarray(v), c["nbr"], c["prm"],
                                                     c["nsite"], Ls, 0)

    ref = b5 * dw(phi) + phi + c5 * dw(chiv) - chiv
    got = mob.mobius_m(c["U"], phi, c["nbr"], c["prm"], c["nsite"], Ls, b5, c5, M5, MF, 0)
    assert rel_err(got, ref) < 1e-14
