"""Even-odd (red-black) operators and the Schur-complement solver, checked against the full
lattice oracle: the half-lattice hopping term is the full Dhop restricted to one parity, D5^-1
inverts the oracle's 5th-dimension operator, and the Schur operator is M's odd rows on a
vector whose even rows of M vanish."""
import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu

M5, MF = 1.8, 0.01
TOL = {gb.F64: 1e-12, gb.F32: 1e-6, gb.F16: 5e-3}


def parity_of(dims):
    x, y, z, t = np.meshgrid(*[np.arange(d) for d in dims], indexing="ij")
    par = (x + y + z + t) % 2
    return par.transpose(3, 2, 1, 0).reshape(-1)  # lexicographic, x fastest


def halves(a, dims, Ls):
    v = np.asarray(a).reshape(int(np.prod(dims)), Ls * 24)
    par = parity_of(dims)
    return v[par == 0].reshape(-1), v[par == 1].reshape(-1)


def masked(a, dims, Ls, keep):
    v = np.asarray(a, dtype=np.float64).reshape(int(np.prod(dims)), Ls * 24).copy()
    v[parity_of(dims) != keep] = 0.0
    return v.reshape(-1)


def setup(dims, Ls, prec, gprec=None):
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, c["U"], gprec if gprec is not None else prec)
    le, lo = lat.checkerboard()
    return c, lat, g, le, lo, g.checkerboard(le), g.checkerboard(lo)


def _to64(f, lat):
    out = gb.Field(lat, gb.F64)
    out.copy_from(f)
    return out


def test_half_lattice_pick_place_round_trip(gpu):
    dims, Ls = (4, 2, 6, 4), 4
    c, lat, g, le, lo, ge, go = setup(dims, Ls, gb.F32)
    for prec in (gb.F64, gb.F32, gb.F16):
        x = gb.Field(lat, prec).load(c["phi"])
        xe, xo = gb.Field(le, prec).pick(x), gb.Field(lo, prec).pick(x)
        he, ho = halves(x.numpy(), dims, Ls)
        assert np.array_equal(xe.numpy(), he) and np.array_equal(xo.numpy(), ho)
        y = gb.Field(lat, prec)
        xe.place_into(y)
        xo.place_into(y)
        assert np.array_equal(y.numpy(), x.numpy())


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
@pytest.mark.parametrize("dag", [0, 1])
def test_dhop_eo_is_restricted_full_dhop(gpu, prec, dag):
    dims, Ls = (4, 4, 2, 6), 8
    c, lat, g, le, lo, ge, go = setup(dims, Ls, prec)
    x = gb.Field(lat, prec).load(c["phi"])
    for out_par, (gout, lout, lin) in enumerate(((ge, le, lo), (go, lo, le))):
        xin = gb.Field(lin, prec).pick(x)
        y = gb.Field(lout, prec)
        gb.dhop_eo(gout, y, xin, dag)
        ref = oracle.dslash(c["U"], masked(c["phi"], dims, Ls, 1 - out_par), c["nbr"], c["prm"], c["nsite"], Ls, dag)
        want = halves(ref, dims, Ls)[out_par]
        assert rel_err(y.numpy(), want) < TOL[prec], (out_par, dag)


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("Ls", [8, 16])
def test_m5inv_inverts_the_fifth_dimension_operator(gpu, prec, dag, Ls):
    """Ls = 16 takes the register-resident form of the kernel, other extents the general one."""
    dims = (2, 2, 2, 4)
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    x = gb.Field(lat, prec).load(c["phi"])
    y = gb.Field(lat, prec)
    gb.dwf_m5inv(y, x, M5, MF, dag)
    back = oracle.dwf_m(np.zeros_like(c["U"]), y.numpy(), c["nbr"], c["nsite"], Ls, M5, MF, dag)
    assert rel_err(back, x.numpy()) < TOL[prec]


@pytest.mark.parametrize("Ls", [1, 5, 12, 64])
def test_m5inv_odd_and_even_ls(gpu, Ls):
    dims = (2, 2, 2, 2)
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    x = gb.Field(lat, gb.F64).load(c["phi"])
    y = gb.Field(lat, gb.F64)
    for dag in (0, 1):
        gb.dwf_m5inv(y, x, M5, MF, dag)
        back = oracle.dwf_m(np.zeros_like(c["U"]), y.numpy(), c["nbr"], c["nsite"], Ls, M5, MF, dag)
        assert rel_err(back, c["phi"]) < 1e-12


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
@pytest.mark.parametrize("dag", [0, 1])
def test_schur_operator_matches_full_operator(gpu, prec, dag):
    """v = (1/2 D5^-1 Dhop_eo x_o, x_o) makes (M v)_e = 0 and (M v)_o = Mpc x_o."""
    dims, Ls = (4, 4, 2, 4), 8
    c, lat, g, le, lo, ge, go = setup(dims, Ls, prec)
    x = gb.Field(lat, prec).load(c["phi"])
    xo = gb.Field(lo, prec).pick(x)
    t1, t2 = gb.Field(le, prec), gb.Field(le, prec)
    gb.dhop_eo(ge, t1, xo, dag)
    gb.dwf_m5inv(t2, t1, M5, MF, dag)
    ve = gb.Field(le, gb.F64)
    ve.axpby(0.5, _to64(t2, le), 0.0)
    v = gb.Field(lat, gb.F64)
    ve.place_into(v)
    _to64(xo, lo).place_into(v)
    mv = oracle.dwf_m(c["U"], v.numpy(), c["nbr"], c["nsite"], Ls, M5, MF, dag)
    mve, mvo = halves(mv, dims, Ls)
    y = gb.Field(lo, prec)
    n2 = gb.dwf_mpc(go, ge, y, t1, t2, xo, M5, MF, dag, want_norm=True)
    tol = TOL[prec] * (10 if prec == gb.F16 else 1)
    assert np.linalg.norm(mve) / np.linalg.norm(mvo) < tol
    assert rel_err(y.numpy(), mvo) < tol
    assert abs(n2 - float(np.sum(y.numpy() ** 2))) / n2 < max(1e-5, TOL[prec])


def test_mpcdagmpc_is_hermitian_positive(gpu):
    dims, Ls = (4, 4, 2, 4), 8
    c, lat, g, le, lo, ge, go = setup(dims, Ls, gb.F64)
    a = gb.Field(lo, gb.F64).gaussian(3)
    b = gb.Field(lo, gb.F64).gaussian(4)
    tp, t1, t2 = gb.Field(lo, gb.F64), gb.Field(le, gb.F64), gb.Field(le, gb.F64)
    Aa, Ab = gb.Field(lo, gb.F64), gb.Field(lo, gb.F64)
    pap = gb.dwf_mpcdagmpc(go, ge, Aa, tp, t1, t2, a, M5, MF)
    gb.dwf_mpcdagmpc(go, ge, Ab, tp, t1, t2, b, M5, MF)
    assert abs(a.dot(Ab) - Aa.dot(b)) < 1e-11 * abs(a.dot(Ab))  # <a, A b> = <A a, b>
    assert abs(a.dot(Aa).real - pap) < 1e-11 * pap and pap > 0


@pytest.mark.parametrize("mode,sp", [(gb.CG_DOUBLE, gb.F64), (gb.CG_PLAIN, gb.F32), (gb.CG_MIXED, gb.F16),
                                     (gb.CG_MIXED, gb.F32)])
def test_eo_solver_solves_m(gpu, mode, sp):
    dims, Ls = (4, 4, 4, 4), 8
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    le, lo = lat.checkerboard()
    g64 = gb.Gauge(lat, c["U"], gb.F64)
    G64 = (g64.checkerboard(le), g64.checkerboard(lo))
    g32 = gb.Gauge(lat, c["U"], gb.F32)
    G32 = (g32.checkerboard(le), g32.checkerboard(lo))
    gsl = gb.Gauge(lat, c["U"], sp) if mode == gb.CG_MIXED else None
    GS = (gsl.checkerboard(le), gsl.checkerboard(lo)) if gsl is not None else None
    b = gb.Field(lat, gb.F64).load(c["phi"])
    x = gb.Field(lat, gb.F64)
    st = gb.cg_solve_eo(G64, x, b, M5, MF, mode, tol=1e-10, g32=G32, gsloppy=GS, sloppy_prec=sp)
    res = c["phi"] - oracle.dwf_m(c["U"], x.numpy(), c["nbr"], c["nsite"], Ls, M5, MF, 0)
    full = float(np.linalg.norm(res) / np.linalg.norm(c["phi"]))
    print(f"EO mode {mode} sp {sp}: {st}, oracle |b-Mx|/|b| = {full:.3e}")
    assert full < 1e-8
    assert abs(full - st["true_residual"]) <= 1e-3 * full + 1e-13


def test_eo_solution_equals_unpreconditioned_solution(gpu):
    """The Schur solve of M x = b and CG on M^dag M x = M^dag b reach the same x."""
    dims, Ls = (4, 4, 4, 4), 8
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    le, lo = lat.checkerboard()
    g64 = gb.Gauge(lat, c["U"], gb.F64)
    G64 = (g64.checkerboard(le), g64.checkerboard(lo))
    b = gb.Field(lat, gb.F64).load(c["phi"])
    x1 = gb.Field(lat, gb.F64)
    gb.cg_solve_eo(G64, x1, b, M5, MF, gb.CG_DOUBLE, tol=1e-11)
    mdb = gb.Field(lat, gb.F64)
    gb.dwf_m(g64, mdb, b, M5, MF, 1)
    x2 = gb.Field(lat, gb.F64)
    gb.cg_solve(g64, x2, mdb, M5, MF, gb.CG_DOUBLE, tol=1e-11)
    assert rel_err(x1.numpy(), x2.numpy()) < 1e-7


def test_checkerboard_needs_even_extents(gpu):
    lat = gb.Lattice.periodic((4, 3, 4, 4), 4)
    with pytest.raises(gb.GbdwError):
        lat.checkerboard()


@pytest.mark.parametrize("shape", [(128, 2, 0, 4), (64, 2, 3, 4), (128, 1, 1, 4), (64, 2, 2, 2), (128, 2, 4, 4)])
def test_eo_hopping_in_every_launch_form(gpu, shape):
    """The half-lattice hopping term through each launch form of the FP32 kernel at Ls = 16
    (the blocked form falls back to the specialised direct one on a half lattice), and the
    fused Schur step (Dhop_oe with the diagonal of another field) in the same forms."""
    dims, Ls = (4, 4, 2, 4), 16
    c, lat, g, le, lo, ge, go = setup(dims, Ls, gb.F32)
    x = gb.Field(lat, gb.F32).load(c["phi"])
    xo = gb.Field(lo, gb.F32).pick(x)
    xe = gb.Field(le, gb.F32).pick(x)
    gb.tune_set(g, x, *shape)
    # half lattices keep their own tuned shapes: pin them too (the blocked form has no half-lattice
    # variant; the specialised direct form is what a half lattice runs in its place)
    gb.tune_set(ge, xo, *(shape if shape[2] != 4 else (64, 2, 3, 4)))
    y = gb.Field(le, gb.F32)
    for dag in (0, 1):
        gb.dhop_eo(ge, y, xo, dag)
        ref = oracle.dslash(c["U"], masked(c["phi"], dims, Ls, 1), c["nbr"], c["prm"], c["nsite"], Ls, dag)
        assert rel_err(y.numpy(), halves(ref, dims, Ls)[0]) < 1e-6, (shape, dag)
        # (M x)_e = D5 x_e - 1/2 Dhop_eo x_o
        gb.dwf_meo(ge, y, xo, xe, M5, MF, dag)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, dag)
        assert rel_err(y.numpy(), halves(refm, dims, Ls)[0]) < 1e-6, (shape, dag)
        # the fused |out|^2 counts every CTA of the form actually launched (a half lattice
        # runs the blocked form's fallback)
        t1, t2, z = gb.Field(le, gb.F32), gb.Field(le, gb.F32), gb.Field(lo, gb.F32)
        n2 = gb.dwf_mpc(go, ge, z, t1, t2, xo, M5, MF, dag, want_norm=True)
        zz = z.numpy()
        assert abs(n2 - float(np.sum(zz * zz))) / n2 < 1e-5, (shape, dag)
    gb.synchronize()


@pytest.mark.parametrize("split", [0, 1, 2, 4])
def test_eo_tuned_and_tiled_shapes(gpu, split):
    """The autotuner on even-odd operands (gauge and output on one half, input on the other)
    keeps shapes of their own, which the even-odd hopping term and the Schur epilogue then run
    (split 0); Ls tiles pinned on the half lattice (splits 1, 2, 4 of the direct forms) give the
    same results."""
    dims, Ls = (4, 4, 2, 4), 16
    c, lat, g, le, lo, ge, go = setup(dims, Ls, gb.F32)
    x = gb.Field(lat, gb.F32).load(c["phi"])
    xo = gb.Field(lo, gb.F32).pick(x)
    xe = gb.Field(le, gb.F32).pick(x)
    y = gb.Field(le, gb.F32)
    if split == 0:
        gb.tune_dhop(ge, y, xo)
        shape = gb.tune_query(ge, xo)
        assert shape[2] in (0, 1, 2, 3) and gb.tune_brick(ge, xo) == 1
    else:
        gb.tune_set(ge, xo, 64, 2, 3, 4)
        gb.tune_set_split(ge, xo, split)
        assert gb.tune_split(ge, xo) == split and gb.tune_query_m(ge, xo)[4] == split
    for dag in (0, 1):
        gb.dhop_eo(ge, y, xo, dag)
        ref = oracle.dslash(c["U"], masked(c["phi"], dims, Ls, 1), c["nbr"], c["prm"], c["nsite"], Ls, dag)
        assert rel_err(y.numpy(), halves(ref, dims, Ls)[0]) < 1e-6, (split, dag)
        gb.dwf_meo(ge, y, xo, xe, M5, MF, dag)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, M5, MF, dag)
        assert rel_err(y.numpy(), halves(refm, dims, Ls)[0]) < 1e-6, (split, dag)
    gb.synchronize()


def test_eo_solver_fp16_residual(gpu):
    """Even-odd mixed FP16 solve with an FP16 iterated residual (the fused Schur adjoint pass
    with the FP16-r epilogue) reaches the target, and the full system's residual agrees with
    the oracle's."""
    dims, Ls = (4, 4, 4, 4), 8
    c, lat, g64, le, lo, ge64, go64 = setup(dims, Ls, gb.F64)
    g16 = gb.Gauge(lat, c["U"], gb.F16)
    G16 = (g16.checkerboard(le), g16.checkerboard(lo))
    b = gb.Field(lat, gb.F64).load(c["phi"])
    x = gb.Field(lat, gb.F64)
    st = gb.cg_solve_eo((ge64, go64), x, b, M5, MF, gb.CG_MIXED, tol=1e-10, max_iter=5000, delta=0.03,
                        gsloppy=G16, sloppy_prec=gb.F16, sloppy_residual=1)
    print(st)
    m = oracle.dwf_m(c["U"], x.numpy(), c["nbr"], c["nsite"], Ls, M5, MF, 0)
    res = np.linalg.norm(c["phi"] - m) / np.linalg.norm(c["phi"])
    assert res < 1e-8 and abs(res - st["true_residual"]) <= 1e-3 * res + 1e-14
