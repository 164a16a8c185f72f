"""The double-single form of the FP64 operator (FP64 fields and gauge, arithmetic on FP32 pairs)
against the FP64 oracle: Dhop and DhopDag on periodic and table lattices (each register cap and
t-brick order, several right-hand sides), M with its fused norm, the even-odd hopping term and the
Schur epilogue, at the FP64 tolerance (1e-12 relative) and the reference's own acceptance sum
(sum of squared differences <= 1e-10, bench_simple.cc:114-119).  The setting is restored after
each test; the solvers' default (double-single) is covered by the CG tests."""
import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12
M5, MF = 1.8, 0.01


@pytest.fixture
def ds_ops(gpu):
    prev = gb.get_fp64_arith(gb.FP64_OPERATORS)
    gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_DOUBLE_SINGLE)
    yield
    gb.set_fp64_arith(gb.FP64_OPERATORS, prev)


def test_setting_defaults_and_validation(gpu):
    assert gb.get_fp64_arith(gb.FP64_SOLVERS) == gb.FP64_DOUBLE_SINGLE
    with pytest.raises(gb.GbdwError):
        gb.set_fp64_arith(5, gb.FP64_NATIVE)
    with pytest.raises(gb.GbdwError):
        gb.set_fp64_arith(gb.FP64_OPERATORS, 3)


@pytest.mark.parametrize("dims,Ls", [((4, 4, 4, 4), 8), ((4, 2, 6, 2), 3), ((8, 8, 8, 8), 16)])
@pytest.mark.parametrize("dag", [0, 1])
def test_ds_dhop_matches_oracle(ds_ops, dims, Ls, dag):
    c = make_case(dims, Ls)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, dag)
    for lat in (gb.Lattice.periodic(dims, Ls), gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)):
        g = gb.Gauge(lat, c["U"], gb.F64)
        x, y = gb.Field(lat, gb.F64).load(c["phi"]), gb.Field(lat, gb.F64)
        gb.dhop(g, y, x, dag)
        out = y.numpy()
        assert rel_err(out, ref) < TOL, (dims, Ls, dag)
        assert float(np.sum((out - ref) ** 2)) <= 1e-10
        # not the native kernel's result bit for bit: the arithmetic differs at ~1e-15
        gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_NATIVE)
        gb.dhop(g, y, x, dag)
        nat = y.numpy()
        gb.set_fp64_arith(gb.FP64_OPERATORS, gb.FP64_DOUBLE_SINGLE)
        assert rel_err(out, nat) < TOL


@pytest.mark.parametrize("minb,brick", [(4, 1), (3, 1), (4, 2), (3, 4), (4, 8)])
def test_ds_register_caps_and_t_bricks(ds_ops, minb, brick):
    """Each register cap and t-brick sweep order of the double-single kernel, Dhop and M, and
    the tuner's own pick."""
    dims, Ls = (4, 4, 4, 8), 8
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x, y = gb.Field(lat, gb.F64).load(c["phi"]), gb.Field(lat, gb.F64)
    gb.tune_set_ds(g, x, 0, minb, brick)
    gb.tune_set_ds(g, x, 1, minb, brick)
    assert gb.tune_query_ds(g, x, 0) == (minb, brick)
    for dag in (0, 1):
        gb.dhop(g, y, x, dag)
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, dag)
        assert rel_err(y.numpy(), ref) < TOL, (minb, brick, dag)
        gb.dwf_m(g, y, x, M5, MF, dag)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, dag)
        assert rel_err(y.numpy(), refm) < TOL, (minb, brick, dag)
    gb.tune_dhop(g, y, x)
    m, b = gb.tune_query_ds(g, x, 1)
    assert m in (3, 4) and b in (1, 2, 4, 8)
    gb.dwf_m(g, y, x, M5, MF, 0)
    assert rel_err(y.numpy(), oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, 0)) < TOL
    with pytest.raises(gb.GbdwError):
        gb.tune_set_ds(g, x, 0, 4, 3)  # Lt = 8 is no multiple of 3
    g32, x32 = gb.Gauge(lat, c["U"], gb.F32), gb.Field(lat, gb.F32)
    with pytest.raises(gb.GbdwError):
        gb.tune_set_ds(g32, x32, 0, 4, 1)  # FP32 fields have no double-single form


def test_ds_multi_rhs(ds_ops):
    dims, Ls, k = (4, 4, 2, 4), 4, 3  # Ls * nrhs = 12 (pairs) and 3 right-hand sides
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, c["U"], gb.F64)
    X, Y = gb.Field(lat, gb.F64, k), gb.Field(lat, gb.F64, k)
    srcs = [gb.generate_fermion(dims, Ls, 1, (9 + r, 6, 7, 8)) for r in range(k)]
    for r in range(k):
        X.load(srcs[r], r)
    gb.dhop(g, Y, X)
    for r in range(k):
        ref = oracle.dslash(c["U"], srcs[r], c["nbr"], c["prm"], c["nsite"], Ls)
        assert rel_err(Y.numpy(r), ref) < TOL, r


@pytest.mark.parametrize("Ls", [5, 8])
@pytest.mark.parametrize("dag", [0, 1])
def test_ds_m_and_norm(ds_ops, Ls, dag):
    dims = (4, 4, 4, 4)
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x, y = gb.Field(lat, gb.F64).load(c["phi"]), gb.Field(lat, gb.F64)
    n2 = gb.dwf_m(g, y, x, M5, MF, dag, want_norm=True)
    ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, dag)
    out = y.numpy()
    assert rel_err(out, ref) < TOL
    assert abs(n2 - float(np.sum(ref ** 2))) / n2 < 1e-12


def test_ds_even_odd(ds_ops):
    """Dhop_eo and the Schur operator's fused epilogue on half lattices against the full oracle
    restricted to one parity."""
    dims, Ls = (4, 4, 2, 4), 8
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, c["U"], gb.F64)
    le, lo = lat.checkerboard()
    ge = g.checkerboard(le)
    x = gb.Field(lat, gb.F64).load(c["phi"])
    xo, xe = gb.Field(lo, gb.F64).pick(x), gb.Field(le, gb.F64).pick(x)
    par = _parity(dims)
    phi = np.asarray(c["phi"]).reshape(int(np.prod(dims)), Ls * 24)
    odd_only = np.where(par[:, None] == 1, phi, 0.0).reshape(-1)
    y = gb.Field(le, gb.F64)
    for dag in (0, 1):
        gb.dhop_eo(ge, y, xo, dag)
        ref = oracle.dslash(c["U"], odd_only, c["nbr"], c["prm"], c["nsite"], Ls, dag)
        ref_e = ref.reshape(-1, Ls * 24)[par == 0].reshape(-1)
        assert rel_err(y.numpy(), ref_e) < TOL
        gb.dwf_meo(ge, y, xo, xe, M5, MF, dag)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, dag)
        assert rel_err(y.numpy(), refm.reshape(-1, Ls * 24)[par == 0].reshape(-1)) < TOL


def _parity(dims):
    x, y, z, t = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    return ((x + y + z + t) % 2).transpose(3, 2, 1, 0).reshape(-1)


def test_ds_cg_double_mode_true_residual(gpu):
    """The FP64 CG with its operator in double-single arithmetic (the solvers' default) reaches
    a 1e-10 true residual recomputed by the FP64 oracle operator on the host."""
    assert gb.get_fp64_arith(gb.FP64_SOLVERS) == gb.FP64_DOUBLE_SINGLE
    dims, Ls = (4, 4, 4, 4), 8
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g64 = gb.Gauge(lat, c["U"], gb.F64)
    b = gb.Field(lat, gb.F64).load(c["phi"])
    x = gb.Field(lat, gb.F64)
    st = gb.cg_solve(g64, x, b, M5, MF, gb.CG_DOUBLE, tol=1e-10)
    assert st["true_residual"] <= 1e-10
    xs = x.numpy()
    r = c["phi"] - oracle.dwf_mdagm(c["U"], xs, c["nbr"], c["nsite"], Ls, M5, MF)
    assert np.linalg.norm(r) / np.linalg.norm(c["phi"]) <= 2e-10
