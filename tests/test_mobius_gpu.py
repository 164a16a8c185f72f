"""Mobius / Cayley 5th-dimension operators on the GPU against the numpy oracle
(oracle/mobius.py, itself pinned to the Shamir oracle)."""
import numpy as np
import pytest

import gridbench_gb300 as gb
from oracle import mobius as mob
from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu

M5, MF = 1.8, 0.01
B5, C5 = 1.5, 0.5  # Mobius scale b + c = 2 (b - c = 1)
TOL = {gb.F64: 1e-13, gb.F32: 1e-6, gb.F16: 5e-3}


def _coefs(Ls, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=Ls), 3.0 + rng.random(Ls), rng.normal(size=Ls)


def _cdot(a, b):
    return complex(np.vdot(a.view(np.complex128), b.view(np.complex128)))


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("Ls", [1, 3, 8, 16])
def test_m5d_matches_oracle(gpu, prec, dag, Ls):
    c = make_case((4, 2, 2, 4), Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    x, y = gb.Field(lat, prec).load(c["phi"]), gb.Field(lat, prec)
    lo, di, up = _coefs(Ls, Ls + 10 * dag)
    gb.m5d(y, x, lo, di, up, dag)
    ref = mob.m5d(c["phi"], Ls, lo, di, up, dag)
    assert rel_err(y.numpy(), ref) < TOL[prec]


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("Ls", [1, 2, 5, 16, 64])
def test_m5d_inv_matches_oracle(gpu, prec, dag, Ls):
    c = make_case((2, 2, 2, 4), Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    x, y, z = gb.Field(lat, prec).load(c["phi"]), gb.Field(lat, prec), gb.Field(lat, prec)
    lo, di, up = _coefs(Ls, 7 + Ls)
    gb.m5d_inv(y, x, lo, di, up, dag)
    ref = mob.m5d_inv(c["phi"], Ls, lo, di, up, dag)
    assert rel_err(y.numpy(), ref) < TOL[prec] * (4 if prec == gb.F16 else 1)
    gb.m5d(z, y, lo, di, up, dag)  # A A^-1 = 1
    assert rel_err(z.numpy(), c["phi"]) < TOL[prec] * (4 if prec == gb.F16 else 1)


def test_m5d_inv_rejects_singular(gpu):
    c = make_case((2, 2, 2, 2), 4)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4)
    x, y = gb.Field(lat, gb.F64).load(c["phi"]), gb.Field(lat, gb.F64)
    with pytest.raises(gb.GbdwError):
        gb.m5d_inv(y, x, 0.0, [1.0, 0.0, 1.0, 1.0], 0.0)  # a zero diagonal entry
    with pytest.raises(gb.GbdwError):
        gb.m5d_inv(y, x, -1.0, 1.0, 0.0)  # P+ block: 1 - S with a cyclic shift, singular
    with pytest.raises(gb.GbdwError):
        gb.m5d(x, x, 0.0, 1.0, 0.0)  # in place


@pytest.mark.parametrize("prec", [gb.F64, gb.F32])
@pytest.mark.parametrize("dag", [0, 1])
def test_mobius_b1_c0_equals_shamir(gpu, prec, dag):
    c = make_case((4, 4, 2, 4), 8)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 8)
    g = gb.Gauge(lat, c["U"], prec)
    x = gb.Field(lat, prec).load(c["phi"])
    y, t, z = gb.Field(lat, prec), gb.Field(lat, prec), gb.Field(lat, prec)
    gb.mobius_m(g, y, t, x, 1.0, 0.0, M5, MF, dag)
    gb.dwf_m(g, z, x, M5, MF, dag)
    assert rel_err(y.numpy(), z.numpy()) < (1e-14 if prec == gb.F64 else 1e-6)


@pytest.mark.parametrize("prec,gprec", [(gb.F64, gb.F64), (gb.F32, gb.F32), (gb.F16, gb.F16)])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("Ls", [6, 16])
def test_mobius_m_matches_oracle(gpu, prec, gprec, dag, Ls):
    c = make_case((4, 4, 2, 4), Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], gprec)
    x = gb.Field(lat, prec).load(c["phi"])
    y, t = gb.Field(lat, prec), gb.Field(lat, prec)
    n2 = gb.mobius_m(g, y, t, x, B5, C5, M5, MF, dag, want_norm=True)
    ref = mob.mobius_m(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, dag)
    out = y.numpy()
    assert rel_err(out, ref) < TOL[prec]
    assert abs(n2 - float(np.sum(out ** 2))) / n2 < (1e-12 if prec == gb.F64 else 1e-5)


def test_mobius_adjoint_and_mooee_inverse(gpu):
    c = make_case((4, 4, 4, 4), 8)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 8)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x = gb.Field(lat, gb.F64).load(c["phi"])
    yv = make_case((4, 4, 4, 4), 8, fseeds=(9, 10, 11, 12))["phi"]
    y = gb.Field(lat, gb.F64).load(yv)
    my, mdx, t = gb.Field(lat, gb.F64), gb.Field(lat, gb.F64), gb.Field(lat, gb.F64)
    gb.mobius_m(g, my, t, y, B5, C5, M5, MF, 0)
    gb.mobius_m(g, mdx, t, x, B5, C5, M5, MF, 1)
    a, b = _cdot(c["phi"], my.numpy()), _cdot(mdx.numpy(), yv)
    assert abs(a - b) / abs(a) < 1e-13
    for dag in (0, 1):
        gb.mobius_mooee(t, x, B5, C5, M5, MF, dag)
        gb.mobius_mooee_inv(my, t, B5, C5, M5, MF, dag)
        assert rel_err(my.numpy(), c["phi"]) < 1e-13


@pytest.mark.parametrize("prec", [gb.F64, gb.F32])
@pytest.mark.parametrize("dag", [0, 1])
def test_mobius_even_odd_blocks(gpu, prec, dag):
    """M by parity blocks: (M x)_p = Mooee x_p + Meooe_pq x_q (and the same for M^dag)."""
    Ls = 8
    c = make_case((4, 4, 4, 4), Ls)
    lat = gb.Lattice.periodic((4, 4, 4, 4), Ls)
    halves = lat.checkerboard()
    gfull = gb.Gauge(lat, c["U"], prec)
    gh = [gfull.checkerboard(h) for h in halves]
    x = gb.Field(lat, prec).load(c["phi"])
    mx, t = gb.Field(lat, prec), gb.Field(lat, prec)
    gb.mobius_m(gfull, mx, t, x, B5, C5, M5, MF, dag)
    xs = [gb.Field(h, prec).pick(x) for h in halves]
    got = gb.Field(lat, prec)
    for p in (0, 1):
        q = 1 - p
        a, h = gb.Field(halves[p], prec), gb.Field(halves[p], prec)
        tmp = gb.Field(halves[p if dag else q], prec)
        gb.mobius_mooee(a, xs[p], B5, C5, M5, MF, dag)
        gb.mobius_meooe(gh[p], h, tmp, xs[q], B5, C5, MF, dag)
        a.axpby(1.0, h, 1.0)
        a.place_into(got)
    assert rel_err(got.numpy(), mx.numpy()) < TOL[prec] * 10


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
def test_mobius_schur_operator(gpu, prec):
    """Mpc = Mooee - Meooe_oe Mooee^-1 Meooe_eo composed from the single blocks; Mpc^dag is its
    adjoint; |Mpc x|^2 is fused."""
    Ls = 8
    c = make_case((4, 4, 4, 4), Ls)
    lat = gb.Lattice.periodic((4, 4, 4, 4), Ls)
    ev, od = lat.checkerboard()
    gfull = gb.Gauge(lat, c["U"], prec)
    ge, go = gfull.checkerboard(ev), gfull.checkerboard(od)
    x = gb.Field(lat, prec).load(c["phi"])
    xo = gb.Field(od, prec).pick(x)
    tp, tq1, tq2, out = gb.Field(od, prec), gb.Field(ev, prec), gb.Field(ev, prec), gb.Field(od, prec)
    n2 = gb.mobius_mpc(go, ge, out, tp, tq1, tq2, xo, B5, C5, M5, MF, 0, want_norm=True)
    a1, a2, tmp_o = gb.Field(ev, prec), gb.Field(ev, prec), gb.Field(od, prec)
    gb.mobius_meooe(ge, a1, tmp_o, xo, B5, C5, MF, 0)
    gb.mobius_mooee_inv(a2, a1, B5, C5, M5, MF, 0)
    b1, b2, tmp_e = gb.Field(od, prec), gb.Field(od, prec), gb.Field(ev, prec)
    gb.mobius_meooe(go, b1, tmp_e, a2, B5, C5, MF, 0)
    gb.mobius_mooee(b2, xo, B5, C5, M5, MF, 0)
    ref = b2.numpy() - b1.numpy()
    got = out.numpy()
    assert rel_err(got, ref) < TOL[prec] * 10
    assert abs(n2 - float(np.sum(got ** 2))) / n2 < (1e-12 if prec == gb.F64 else 1e-5)
    if prec == gb.F64:
        yfull = gb.Field(lat, prec).load(make_case((4, 4, 4, 4), Ls, fseeds=(3, 1, 4, 1))["phi"])
        y = gb.Field(od, prec).pick(yfull)
        my, mdx = gb.Field(od, prec), gb.Field(od, prec)
        gb.mobius_mpc(go, ge, my, tp, tq1, tq2, y, B5, C5, M5, MF, 0)
        gb.mobius_mpc(go, ge, mdx, tp, tq1, tq2, xo, B5, C5, M5, MF, 1)
        a, b = xo.dot(my), mdx.dot(y)
        assert abs(a - b) / abs(a) < 1e-13


def test_mobius_mdagm_matches_oracle(gpu):
    Ls = 8
    c = make_case((4, 4, 2, 4), Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x = gb.Field(lat, gb.F64).load(c["phi"])
    out, t, tmp = gb.Field(lat, gb.F64), gb.Field(lat, gb.F64), gb.Field(lat, gb.F64)
    pap = gb.mobius_mdagm(g, out, t, tmp, x, B5, C5, M5, MF)
    m = mob.mobius_m(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, 0)
    ref = mob.mobius_m(c["U"], m, c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, 1)
    assert rel_err(out.numpy(), ref) < 1e-13
    assert abs(pap - float(np.sum(m ** 2))) / pap < 1e-12


@pytest.mark.parametrize("mode,sp", [(gb.CG_DOUBLE, gb.F16), (gb.CG_PLAIN, gb.F16), (gb.CG_MIXED, gb.F16),
                                     (gb.CG_MIXED, gb.F32)])
def test_mobius_cg_reaches_1e10(gpu, mode, sp):
    """Mobius M^dag M x = b to a 1e-10 true residual, re-checked with the numpy oracle."""
    Ls = 8
    c = make_case((4, 4, 4, 4), Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g64, g32, g16 = (gb.Gauge(lat, c["U"], p) for p in (gb.F64, gb.F32, gb.F16))
    b = gb.Field(lat, gb.F64).load(c["phi"])
    x = gb.Field(lat, gb.F64)
    st = gb.cg_solve_mobius(g64, x, b, B5, C5, M5, MF, mode, tol=1e-10, max_iter=5000, delta=0.03 if sp == gb.F16
                            else 1e-4, g32=g32, gsloppy=g16 if sp == gb.F16 else g32, sloppy_prec=sp)
    print(mode, sp, st)
    assert st["true_residual"] <= 1e-10
    xv = x.numpy()
    m = mob.mobius_m(c["U"], xv, c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, 0)
    ax = mob.mobius_m(c["U"], m, c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, 1)
    assert np.linalg.norm(c["phi"] - ax) / np.linalg.norm(c["phi"]) <= 2e-10
    if mode != gb.CG_DOUBLE:
        assert st["reliable_updates"] >= 1


@pytest.mark.parametrize("mode,sp", [(gb.CG_DOUBLE, gb.F16), (gb.CG_PLAIN, gb.F16), (gb.CG_MIXED, gb.F16),
                                     (gb.CG_MIXED, gb.F32)])
def test_mobius_eo_solver(gpu, mode, sp):
    """The Mobius M x = b through the odd Schur complement: the full system's true residual
    (reported, and re-checked with the numpy oracle) reaches 1e-10 scale, and the solution
    equals the one of CG on M^dag M x = M^dag b."""
    Ls = 8
    dims = (4, 4, 4, 4)
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    ev, od = lat.checkerboard()
    g = {p: gb.Gauge(lat, c["U"], p) for p in (gb.F64, gb.F32, gb.F16)}
    halves = {p: (g[p].checkerboard(ev), g[p].checkerboard(od)) for p in g}
    b = gb.Field(lat, gb.F64).load(c["phi"])
    x = gb.Field(lat, gb.F64)
    st = gb.cg_solve_mobius_eo(halves[gb.F64], x, b, B5, C5, M5, MF, mode, tol=1e-10, max_iter=5000,
                               delta=0.03 if sp == gb.F16 else 1e-4, g32=halves[gb.F32],
                               gsloppy=halves[gb.F16 if sp == gb.F16 else gb.F32], sloppy_prec=sp)
    print(mode, sp, st)
    xv = x.numpy()
    m = mob.mobius_m(c["U"], xv, c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, 0)
    res = np.linalg.norm(c["phi"] - m) / np.linalg.norm(c["phi"])
    assert abs(res - st["true_residual"]) <= 1e-3 * res + 1e-14
    assert res < 1e-8
    if mode == gb.CG_DOUBLE:
        # the unpreconditioned normal equations give the same solution
        mdb = mob.mobius_m(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, 1)
        rhs = gb.Field(lat, gb.F64).load(mdb)
        y = gb.Field(lat, gb.F64)
        gb.cg_solve_mobius(g[gb.F64], y, rhs, B5, C5, M5, MF, gb.CG_DOUBLE, tol=1e-12, max_iter=5000)
        assert rel_err(xv, y.numpy()) < 1e-7


FORMS_LS16 = [(128, 2, 0, 4), (64, 2, 3, 4), (128, 2, 4, 4), (64, 2, 2, 2), (128, 2, 1, 2), (64, 4, 0, 4)]


@pytest.mark.parametrize("Ls", [2, 4, 8, 16, 32])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
def test_mobius_fused_pass_every_form(gpu, Ls, dag, prec):
    """One hopping pass each for M^dag (every precision: A(b, c)^dag applied in the epilogue) and
    for M (FP32: A(b, c) applied to the neighbours' slices as they are loaded; FP64 and FP16 keep
    two passes), Ls a power of two, the neighbouring slices taken by lane shuffles; against the
    oracle in every launch form the tuner may pick, with the fused norm; a periodic lattice so
    the blocked form applies at Ls = 16."""
    dims = (4, 2, 4, 2)
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, c["U"], prec)
    x = gb.Field(lat, prec).load(c["phi"])
    y, t = gb.Field(lat, prec), gb.Field(lat, prec)
    ref = mob.mobius_m(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, dag)
    shapes = FORMS_LS16 if Ls == 16 else [(128, 2, 0, 4), (64, 2, 2, 2), (128, 1, 0, 4)]
    for shape in shapes:
        try:
            gb.tune_set(g, x, *shape)
        except gb.GbdwError:
            continue
        y.zero()
        n2 = gb.mobius_m(g, y, t, x, B5, C5, M5, MF, dag, want_norm=True)
        out = y.numpy()
        assert rel_err(out, ref) < TOL[prec], shape
        assert abs(n2 - float(np.sum(out ** 2))) / n2 < (1e-12 if prec == gb.F64 else 1e-5), shape
    gb.synchronize()


@pytest.mark.parametrize("dag", [0, 1])
def test_mobius_unfused_extents(gpu, dag):
    """Ls = 6 and 12 (not powers of two) keep the two-pass operators."""
    for Ls in (6, 12):
        c = make_case((2, 2, 4, 2), Ls)
        lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
        g = gb.Gauge(lat, c["U"], gb.F32)
        x = gb.Field(lat, gb.F32).load(c["phi"])
        y, t = gb.Field(lat, gb.F32), gb.Field(lat, gb.F32)
        gb.mobius_m(g, y, t, x, B5, C5, M5, MF, dag)
        ref = mob.mobius_m(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, B5, C5, M5, MF, dag)
        assert rel_err(y.numpy(), ref) < TOL[gb.F32], Ls
