"""Shamir domain-wall operator M, M^dagger, M^dagger M and the FP16/BF16 storage forms."""
import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu

M5, MF = 1.8, 0.01


def _setup(dims, Ls, prec, gprec=None):
    c = make_case(dims, Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], gprec if gprec is not None else prec)
    x = gb.Field(lat, prec).load(c["phi"])
    return c, lat, g, x


@pytest.mark.parametrize("prec,tol", [(gb.F64, 1e-12), (gb.F32, 1e-6)])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("Ls", [4, 6, 8])
def test_dwf_m_matches_oracle(gpu, prec, tol, dag, Ls):
    c, lat, g, x = _setup((4, 4, 2, 4), Ls, prec)
    y = gb.Field(lat, prec)
    n2 = gb.dwf_m(g, y, x, M5, MF, dag, want_norm=True)
    ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, dag)
    out = y.numpy()
    assert rel_err(out, ref) < tol
    assert abs(n2 - float(np.sum(out ** 2))) / n2 < (1e-12 if prec == gb.F64 else 1e-6)


@pytest.mark.parametrize("prec,tol", [(gb.F64, 1e-12), (gb.F32, 1e-6)])
def test_mdagm_matches_oracle_and_pap(gpu, prec, tol):
    c, lat, g, x = _setup((4, 4, 4, 4), 8, prec)
    y, t = gb.Field(lat, prec), gb.Field(lat, prec)
    pap = gb.dwf_mdagm(g, y, t, x, M5, MF)
    ref = oracle.dwf_mdagm(c["U"], c["phi"], c["nbr"], c["nsite"], 8, M5, MF)
    assert rel_err(y.numpy(), ref) < tol
    m = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 8, M5, MF, 0)
    assert abs(pap - float(np.sum(m ** 2))) / pap < tol * 10


@pytest.mark.parametrize("gprec,tol", [(gb.F16, 5e-3), (gb.BF16, 3e-2)])
@pytest.mark.parametrize("dag", [0, 1])
def test_fp16_storage_dhop_and_m(gpu, gprec, tol, dag):
    """FP16 spinor + per-site FP32 norm, 12-real FP16/BF16 links, FP32 arithmetic: the
    relative error against the FP64 oracle is reported and bounded."""
    c, lat, g, x = _setup((4, 4, 4, 4), 8, gb.F16, gprec)
    y = gb.Field(lat, gb.F16)
    gb.dhop(g, y, x, dag)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 8, dag)
    e1 = rel_err(y.numpy(), ref)
    gb.dwf_m(g, y, x, M5, MF, dag)
    ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 8, M5, MF, dag)
    e2 = rel_err(y.numpy(), ref)
    print(f"FP16 storage rel err vs FP64: Dhop {e1:.2e}  M {e2:.2e}")
    assert e1 < tol and e2 < tol


@pytest.mark.parametrize("form,spt,stages", [(0, 1, 4), (0, 2, 4), (0, 4, 4), (1, 2, 2), (1, 2, 4), (1, 4, 2),
                                              (1, 4, 4), (2, 2, 2), (2, 4, 4)])
@pytest.mark.parametrize("gprec", [gb.F16, gb.BF16])
def test_fp16_every_shape(gpu, form, spt, stages, gprec):
    c, lat, g, x = _setup((4, 2, 6, 2), 12, gb.F16, gprec)
    y = gb.Field(lat, gb.F16)
    gb.tune_set(g, x, 128, spt, form, stages)
    for dag in (0, 1):
        n2 = gb.dwf_m(g, y, x, M5, MF, dag, want_norm=True)
        ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 12, M5, MF, dag)
        out = y.numpy()
        assert rel_err(out, ref) < (5e-3 if gprec == gb.F16 else 3e-2)
        assert abs(n2 - float(np.sum(out ** 2))) / n2 < 1e-5
        gb.dhop(g, y, x, dag)
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 12, dag)
        assert rel_err(y.numpy(), ref) < (5e-3 if gprec == gb.F16 else 3e-2)
    gb.synchronize()


@pytest.mark.parametrize("prec,tol", [(gb.F64, 1e-12), (gb.F32, 1e-6)])
@pytest.mark.parametrize("stages", [2, 4])
def test_staged_form_m_and_norm(gpu, prec, tol, stages):
    c, lat, g, x = _setup((4, 4, 2, 4), 8, prec)
    y = gb.Field(lat, prec)
    for form, spt in ((1, 1), (1, 2), (2, 1), (2, 2)):
        try:
            gb.tune_set(g, x, 128, spt, form, stages)
        except gb.GbdwError:
            continue  # a staged ring that does not fit in shared memory
        for dag in (0, 1):
            n2 = gb.dwf_m(g, y, x, M5, MF, dag, want_norm=True)
            ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 8, M5, MF, dag)
            out = y.numpy()
            assert rel_err(out, ref) < tol
            assert abs(n2 - float(np.sum(out ** 2))) / n2 < tol * 10
    gb.synchronize()


def test_fp16_roundtrip_precision(gpu):
    c, lat, g, x = _setup((4, 4, 4, 4), 4, gb.F16, gb.F16)
    assert rel_err(x.numpy(), c["phi"]) < 1e-3


def test_m_rejects_multi_rhs_and_inplace(gpu):
    c, lat, g, x = _setup((2, 2, 2, 2), 4, gb.F32)
    X = gb.Field(lat, gb.F32, 2)
    Y = gb.Field(lat, gb.F32, 2)
    with pytest.raises(gb.GbdwError):
        gb.dwf_m(g, Y, X, M5, MF)
    with pytest.raises(gb.GbdwError):
        gb.dhop(g, x, x)


@pytest.mark.parametrize("gprec", [gb.F16, gb.BF16])
def test_fp16_ls16_specialised_form(gpu, gprec):
    """Form 3 (row stride fixed at Ls = 16 at compile time) on FP16 spinors: Dhop, DhopDag,
    M and M^dagger with the fused norm."""
    c, lat, g, x = _setup((4, 2, 6, 2), 16, gb.F16, gprec)
    y = gb.Field(lat, gb.F16)
    gb.tune_set(g, x, 64, 2, 3, 4)
    assert tuple(gb.tune_query(g, x)) == (64, 2, 3, 4)
    tol = 5e-3 if gprec == gb.F16 else 3e-2
    for dag in (0, 1):
        n2 = gb.dwf_m(g, y, x, M5, MF, dag, want_norm=True)
        ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 16, M5, MF, dag)
        out = y.numpy()
        assert rel_err(out, ref) < tol
        assert abs(n2 - float(np.sum(out ** 2))) / n2 < 1e-5
        gb.dhop(g, y, x, dag)
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 16, dag)
        assert rel_err(y.numpy(), ref) < tol
    gb.synchronize()
