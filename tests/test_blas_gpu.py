"""BLAS-1 with FP64 global sums across storage precisions."""
import numpy as np
import pytest

import gridbench_gb300 as gb
from conftest import make_case

pytestmark = pytest.mark.gpu


def _c(a):
    return a[0::2] + 1j * a[1::2]


@pytest.mark.parametrize("prec,tol", [(gb.F64, 1e-14), (gb.F32, 1e-6), (gb.F16, 2e-3)])
def test_norm_dot_axpby(gpu, prec, tol):
    c = make_case((4, 4, 4, 4), 4)
    d = make_case((4, 4, 4, 4), 4, fseeds=(1, 1, 2, 3))
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4)
    x = gb.Field(lat, prec).load(c["phi"])
    y = gb.Field(lat, prec).load(d["phi"])
    xa, ya = x.numpy(), y.numpy()  # values as stored
    # F64 fields sum in FP64 throughout; F32/F16 fields sum each 24-real entry in FP32 and
    # everything above the entry in FP64
    sum_tol = 1e-12 if prec == gb.F64 else 1e-7
    assert abs(x.norm2() - np.sum(xa ** 2)) / np.sum(xa ** 2) < sum_tol
    dt = x.dot(y)
    ref = np.vdot(_c(xa), _c(ya))
    assert abs(dt - ref) / abs(ref) < (1e-10 if prec == gb.F64 else 1e-5)
    y.axpby(0.5, x, -2.0)
    exp = 0.5 * xa - 2.0 * ya
    assert np.linalg.norm(y.numpy() - exp) / np.linalg.norm(exp) < tol


def test_precision_conversions(gpu):
    c = make_case((2, 2, 2, 2), 8)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 8)
    f64 = gb.Field(lat, gb.F64).load(c["phi"])
    for p, tol in ((gb.F32, 1e-7), (gb.F16, 1e-3)):
        f = gb.Field(lat, p)
        f.copy_from(f64)
        back = gb.Field(lat, gb.F64)
        back.copy_from(f)
        assert np.linalg.norm(back.numpy() - c["phi"]) / np.linalg.norm(c["phi"]) < tol
