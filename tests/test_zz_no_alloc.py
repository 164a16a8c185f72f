"""gbdw_norm2_noalloc, the entry point for callers that cannot allocate device memory (a
program whose own pool allocator owns the GPU, or a solver loop that must not pay for
cudaMalloc).  The input lives in memory the caller allocated -- here a torch tensor -- and the
result must agree with gbdw_norm2 on the same data, on two calls in a row (the calls share
one fixed scratch array, so the second call must not see the first call's leftovers)."""
import ctypes as C

import numpy as np
import pytest

import gridbench_gb300 as gb
from conftest import make_case

pytestmark = pytest.mark.gpu


def test_noalloc_norm_matches_field_norm(gpu):
    torch = pytest.importorskip("torch")
    L = gb.load()
    c = make_case((8, 8, 8, 8), 8)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 8)
    out = C.c_double()
    for prec, dt, tol in ((gb.F64, np.float64, 1e-12), (gb.F32, np.float32, 1e-7)):
        ref = gb.Field(lat, prec).load(c["phi"]).norm2()
        dev = torch.from_numpy(c["phi"].astype(dt)).cuda()
        torch.cuda.synchronize()
        n = dev.numel() // 2
        for _ in range(2):
            out.value = -1.0
            st = L.gbdw_norm2_noalloc(C.c_void_p(dev.data_ptr()), prec, n, C.byref(out))
            assert st == 0, L.gbdw_last_error().decode()
            assert abs(out.value - ref) / ref < tol
        # a shorter prefix: the scratch left by the longer call must not leak into this one
        half = torch.from_numpy(c["phi"][: 2 * (n // 3)].astype(dt)).cuda()
        torch.cuda.synchronize()
        st = L.gbdw_norm2_noalloc(C.c_void_p(half.data_ptr()), prec, n // 3, C.byref(out))
        exp = float(np.sum(c["phi"][: 2 * (n // 3)].astype(dt).astype(np.float64) ** 2))
        assert st == 0 and abs(out.value - exp) / exp < tol
    st = L.gbdw_norm2_noalloc(C.c_void_p(dev.data_ptr()), gb.F32, (1 << 24) + 1, C.byref(out))
    assert st == 1 and "exceed" in L.gbdw_last_error().decode()
