"""Persistent batched hopping term in a CUDA graph: equals per-instance launches."""
import numpy as np
import pytest

import gridbench_gb300 as gb
from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu


def test_batch_equals_individual(gpu):
    specs = [((4, 4, 4, 4), 8, gb.F32), ((2, 2, 2, 2), 12, gb.F16), ((6, 6, 6, 6), 16, gb.F32),
             ((4, 4, 4, 4), 12, gb.F16), ((8, 8, 8, 8), 8, gb.F16), ((2, 4, 2, 4), 16, gb.F32)]
    keep, G, O, I, refs = [], [], [], [], []
    for k, (dims, Ls, prec) in enumerate(specs):
        c = make_case(dims, Ls, gseeds=(k, 1, 2, 3), fseeds=(k, 4, 5, 6))
        lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
        g = gb.Gauge(lat, c["U"], prec)
        x = gb.Field(lat, prec).load(c["phi"])
        y = gb.Field(lat, prec)
        r = gb.Field(lat, prec)
        gb.dhop(g, r, x)
        keep.append(lat)
        G.append(g)
        O.append(y)
        I.append(x)
        refs.append(r.numpy())
    b = gb.Batch(G, O, I)
    info = b.info()
    assert info["graph"] and info["items"] > 0 and info["ctas"] > 0
    b.run()
    b.run()
    for y, r, (dims, Ls, prec) in zip(O, refs, specs):
        assert rel_err(y.numpy(), r) < (1e-6 if prec == gb.F32 else 2e-3)


def test_batch_rejects_fp64(gpu):
    c = make_case((2, 2, 2, 2), 4)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x, y = gb.Field(lat, gb.F64), gb.Field(lat, gb.F64)
    with pytest.raises(gb.GbdwError):
        gb.Batch([g], [y], [x])
