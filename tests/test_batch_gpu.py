"""Persistent batched hopping term in a CUDA graph: every instance against the oracle, for the
autotuned shape and for pinned shapes covering each tile split (Ls tiles and RHS tiles), with
instances of several right-hand sides, odd Ls and every supported precision pairing."""
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import make_case, rel_err

pytestmark = pytest.mark.gpu

TOL = {gb.F32: 1e-6, gb.F16: 5e-3}

# (dims, Ls, spinor precision, gauge precision, right-hand sides)
SPECS = [((4, 4, 4, 4), 8, gb.F32, gb.F32, 1), ((2, 2, 2, 2), 12, gb.F16, gb.F16, 1),
         ((6, 6, 6, 6), 16, gb.F32, gb.F32, 1), ((4, 4, 4, 4), 12, gb.F16, gb.BF16, 1),
         ((8, 8, 8, 8), 8, gb.F16, gb.F16, 1), ((2, 4, 2, 4), 16, gb.F32, gb.F32, 1),
         ((4, 2, 4, 2), 5, gb.F32, gb.F32, 1), ((4, 4, 2, 2), 4, gb.F32, gb.F32, 3),
         ((2, 4, 4, 2), 8, gb.F16, gb.F16, 4), ((4, 4, 4, 2), 12, gb.F32, gb.F32, 12),
         ((2, 2, 4, 2), 16, gb.F32, gb.F32, 4), ((2, 2, 2, 4), 12, gb.F16, gb.F16, 2),
         ((2, 4, 2, 2), 12, gb.F16, gb.F16, 4), ((4, 2, 2, 2), 8, gb.F16, gb.BF16, 2)]


@pytest.fixture(scope="module")
def batch(gpu):
    keep, G, O, I, refs = [], [], [], [], []
    for k, (dims, Ls, sp, gp, nrhs) in enumerate(SPECS):
        c = make_case(dims, Ls, gseeds=(k, 1, 2, 3), fseeds=(k, 4, 5, 6))
        lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
        g = gb.Gauge(lat, c["U"], gp)
        x = gb.Field(lat, sp, nrhs)
        rr = []
        for r in range(nrhs):
            src = c["phi"] if r == 0 else gb.generate_fermion(dims, Ls, 1, (k, 4, 5, 6 + r))
            x.load(src, r)
            rr.append(oracle.dslash(c["U"], src, c["nbr"], c["prm"], c["nsite"], Ls))
        keep.append(lat)
        G.append(g)
        O.append(gb.Field(lat, sp, nrhs))
        I.append(x)
        refs.append(rr)
    return gb.Batch(G, O, I), O, refs, keep


def _check(O, refs, what):
    for k, (y, rr) in enumerate(zip(O, refs)):
        for r, ref in enumerate(rr):
            assert rel_err(y.numpy(r), ref) < TOL[SPECS[k][2]], (what, k, r)


def test_batch_tuned_shape_matches_oracle(batch):
    b, O, refs, _ = batch
    info = b.info()
    assert info["graph"] and info["items"] > 0 and info["ctas"] > 0
    for y in O:
        y.zero()
    b.run()
    b.run()
    _check(O, refs, info)


@pytest.mark.parametrize("threads", [64, 128])
@pytest.mark.parametrize("split", [1, 2, 4, 8, 16])
def test_batch_every_shape_and_tile_matches_oracle(batch, threads, split):
    """split 2..4 cut each site's slices into Ls tiles; 8 and 16 reach RHS tiles on the
    multi-RHS instances (one s, some right-hand sides); slices per thread 2 and 1."""
    b, O, refs, _ = batch
    for spt in (2, 1):
        b.set_shape(threads, spt, spt, split)
        info = b.info()
        assert (info["threads"], info["spt_f32"], info["tile_split"]) == (threads, spt, split)
        for y in O:
            y.zero()
        b.run()
        _check(O, refs, (threads, spt, split))


def test_batch_rejects_fp64_and_bad_shapes(batch):
    c = make_case((2, 2, 2, 2), 4)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x, y = gb.Field(lat, gb.F64), gb.Field(lat, gb.F64)
    with pytest.raises(gb.GbdwError):
        gb.Batch([g], [y], [x])
    b = batch[0]
    for bad in ((96, 2, 2, 1), (256, 2, 2, 1), (64, 3, 2, 1), (64, 2, 2, 3)):
        with pytest.raises(gb.GbdwError):
            b.set_shape(*bad)
