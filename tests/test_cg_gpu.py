"""CG on M^dagger M (Shamir, M5=1.8, mf=0.01): plain FP32-kernel/FP64-residual, mixed FP16
storage with reliable updates, and all-FP64; the true residual is re-checked on the CPU with
the FP64 oracle operator."""
import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import make_case

pytestmark = pytest.mark.gpu

M5, MF = 1.8, 0.01


def _true_residual(c, x, Ls):
    Ax = oracle.dwf_mdagm(c["U"], x, c["nbr"], c["nsite"], Ls, M5, MF)
    return np.linalg.norm(c["phi"] - Ax) / np.linalg.norm(c["phi"])


@pytest.fixture(scope="module")
def setup(gpu):
    dims, Ls = (4, 4, 4, 4), 8
    c = make_case(dims, Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g64 = gb.Gauge(lat, c["U"], gb.F64)
    g32 = gb.Gauge(lat, c["U"], gb.F32)
    g16 = gb.Gauge(lat, c["U"], gb.F16)
    b = gb.Field(lat, gb.F64).load(c["phi"])
    return c, lat, g64, g32, g16, b, Ls


@pytest.mark.parametrize("mode,sp", [(gb.CG_DOUBLE, gb.F16), (gb.CG_PLAIN, gb.F16), (gb.CG_MIXED, gb.F16),
                                     (gb.CG_MIXED, gb.F32)])
def test_cg_reaches_1e10_true_residual(setup, mode, sp):
    c, lat, g64, g32, g16, b, Ls = setup
    x = gb.Field(lat, gb.F64)
    gs = g16 if sp == gb.F16 else g32
    st = gb.cg_solve(g64, x, b, M5, MF, mode, tol=1e-10, max_iter=5000, g32=g32, gsloppy=gs, sloppy_prec=sp)
    print(mode, sp, st)
    assert st["true_residual"] <= 1e-10
    assert _true_residual(c, x.numpy(), Ls) <= 2e-10
    if mode != gb.CG_DOUBLE:
        assert st["reliable_updates"] >= 1


def test_cg_iteration_limit_is_reported(setup):
    c, lat, g64, g32, g16, b, Ls = setup
    x = gb.Field(lat, gb.F64)
    with pytest.raises(gb.GbdwError) as e:
        gb.cg_solve(g64, x, b, M5, MF, gb.CG_MIXED, tol=1e-10, max_iter=3, g32=g32, gsloppy=g16)
    assert e.value.status == 5  # GBDW_ERR_NOT_CONVERGED


def test_cg_rejects_wrong_precisions(setup):
    c, lat, g64, g32, g16, b, Ls = setup
    x = gb.Field(lat, gb.F32)
    with pytest.raises(gb.GbdwError):
        gb.cg_solve(g64, x, b, M5, MF, gb.CG_PLAIN, g32=g32)
    x = gb.Field(lat, gb.F64)
    with pytest.raises(gb.GbdwError):
        gb.cg_solve(g64, x, b, M5, MF, gb.CG_MIXED, gsloppy=g32, sloppy_prec=gb.F16)


def test_cg_mixed_with_bf16_links_and_initial_guess(setup):
    """FP16 spinors with BF16 12-real links as the sloppy operator, and a non-zero initial
    guess (the first true residual is then computed, not copied from b)."""
    c, lat, g64, g32, g16, b, Ls = setup
    gbf = gb.Gauge(lat, c["U"], gb.BF16)
    x = gb.Field(lat, gb.F64).load(0.01 * c["phi"])
    st = gb.cg_solve(g64, x, b, M5, MF, gb.CG_MIXED, tol=1e-10, max_iter=5000, delta=0.1, g32=g32, gsloppy=gbf,
                     sloppy_prec=gb.F16)
    assert st["true_residual"] <= 1e-10
    assert _true_residual(c, x.numpy(), Ls) <= 2e-10


@pytest.mark.parametrize("delta", [0.3, 1e-4])
def test_cg_reliable_update_threshold_extremes(setup, delta):
    """A frequent (0.3) and a rare (1e-4) reliable-update threshold both reach the target with
    the FP32 sloppy operator; the rare one needs fewer updates."""
    c, lat, g64, g32, g16, b, Ls = setup
    x = gb.Field(lat, gb.F64)
    st = gb.cg_solve(g64, x, b, M5, MF, gb.CG_MIXED, tol=1e-10, max_iter=5000, delta=delta, g32=g32, gsloppy=g32,
                     sloppy_prec=gb.F32)
    assert st["true_residual"] <= 1e-10 and _true_residual(c, x.numpy(), Ls) <= 2e-10
    assert st["reliable_updates"] <= (4 if delta < 1e-3 else 40)


@pytest.mark.parametrize("delta", [0.03, 0.1])
def test_cg_mixed_fp16_residual(setup, delta):
    """The mixed FP16 solve with its iterated residual stored in FP16 (the fused adjoint pass
    updates r in FP16 with per-slice norms) still reaches the 1e-10 true residual."""
    c, lat, g64, g32, g16, b, Ls = setup
    x = gb.Field(lat, gb.F64)
    st = gb.cg_solve(g64, x, b, M5, MF, gb.CG_MIXED, tol=1e-10, max_iter=5000, delta=delta, g32=g32,
                     gsloppy=g16, sloppy_prec=gb.F16, sloppy_residual=1)
    print(delta, st)
    assert st["true_residual"] <= 1e-10
    assert _true_residual(c, x.numpy(), Ls) <= 2e-10
