"""Failure detection without a GPU fault: a bounded device-side wait that nothing completes
expires, the kernel records a status, the host reads it, and the context stays usable."""
import time

import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


def test_expired_wait_is_reported_and_context_survives(gpu):
    gb.synchronize()
    L = gb.load()
    t0 = time.time()
    assert L.gbdw_selftest_wait_timeout(20_000_000) == 0  # 20 ms limit
    with pytest.raises(gb.GbdwError) as e:
        gb.synchronize()
    assert e.value.status == 8  # GBDW_ERR_TIMEOUT
    assert time.time() - t0 < 5.0
    gb.synchronize()  # the error word was cleared
    c = make_case((4, 4, 4, 4), 4)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4)
    g = gb.Gauge(lat, c["U"], gb.F32)
    x, y = gb.Field(lat, gb.F32).load(c["phi"]), gb.Field(lat, gb.F32)
    gb.dhop(g, y, x)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 4)
    assert rel_err(y.numpy(), ref) < 1e-6
    gb.synchronize()
