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


def test_injected_allocation_failures_are_reported_and_context_survives(gpu):
    """A device allocation made to fail on the host (gbdw_debug_fail_allocs: cudaMalloc is not
    called and reports nothing; the library sees an exhausted device) comes back as
    GBDW_ERR_ALLOC with a message, leaves nothing half-built, and the next calls work."""
    L = gb.load()
    c = make_case((4, 4, 4, 4), 4)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4)
    g = gb.Gauge(lat, c["U"], gb.F32)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 4)
    try:
        # the field's own storage
        assert L.gbdw_debug_fail_allocs(0, 1) == 0
        with pytest.raises(gb.GbdwError) as e:
            gb.Field(lat, gb.F32)
        assert e.value.status == 3 and "alloc" in str(e.value).lower()  # GBDW_ERR_ALLOC
        # the FP16 field's second allocation (its norms) after the first succeeded
        assert L.gbdw_debug_fail_allocs(1, 1) == 0
        with pytest.raises(gb.GbdwError) as e:
            gb.Field(lat, gb.F16)
        assert e.value.status == 3
        # a gauge field
        assert L.gbdw_debug_fail_allocs(0, 1) == 0
        with pytest.raises(gb.GbdwError) as e:
            gb.Gauge(lat, c["U"], gb.F64)
        assert e.value.status == 3
    finally:
        L.gbdw_debug_fail_allocs(0, 0)
    x, y = gb.Field(lat, gb.F32).load(c["phi"]), gb.Field(lat, gb.F32)
    gb.dhop(g, y, x)
    assert rel_err(y.numpy(), ref) < 1e-6
    x16 = gb.Field(lat, gb.F16).load(c["phi"])
    assert x16.norm2() > 0
    gb.synchronize()


def test_injected_failure_of_reduction_scratch(gpu):
    """The library's own scratch (the FP64 reduction of a norm on a fresh stream) failing to
    allocate is reported, and the same call succeeds once allocations work again."""
    L = gb.load()
    c = make_case((4, 4, 2, 2), 4)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4)
    x = gb.Field(lat, gb.F64).load(c["phi"])
    exp = float(np.sum(c["phi"] ** 2))
    gb.synchronize()  # the import ran on the library's own stream
    s = gb.Stream()  # a new stream has no scratch yet, so its first reduction allocates
    try:
        with s:
            assert L.gbdw_debug_fail_allocs(0, 1) == 0
            with pytest.raises(gb.GbdwError) as e:
                x.norm2()
            assert e.value.status == 3
            L.gbdw_debug_fail_allocs(0, 0)
            assert abs(x.norm2() - exp) / exp < 1e-13
    finally:
        L.gbdw_debug_fail_allocs(0, 0)
        s.close()
    gb.synchronize()
