"""Oracle parity at the benchmarked shapes themselves: the 16^4 x Ls=16 headline lattice (FP32
and FP64, Dhop and DhopDag, every launch form the autotuner may pick), the 24^4 x Ls=12 lattice
with 12 right-hand sides in one launch, the 64-instance batch of uneven lattices, and the
32^4 x Ls=16 CG solves whose true residual is recomputed on the host with the FP64 oracle
operator.  Each compares the GPU result with the CPU restatement of dslash_simple.h (the
oracle) on the same seeded inputs, at the tolerances of the smaller parity tests."""
import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import make_case, need_host_memory, rel_err

pytestmark = pytest.mark.gpu

TOL = {gb.F64: 1e-12, gb.F32: 1e-6, gb.F16: 5e-3}  # relative to the FP64 oracle
GiB = 2.0 ** 30

# FP32 launch shapes (threads, slices per thread, form, stages) the autotuner chooses between
# at Ls = 16: direct, TMA warp rings, the specialised direct form and its 2^4 site blocks
FP32_LS16_FORMS = [(128, 2, 0, 4), (64, 2, 2, 2), (64, 2, 3, 4), (128, 2, 4, 4)]


@pytest.fixture(scope="module")
def headline(gpu):
    """16^4 x Ls=16 inputs on a periodic lattice (as the benchmark builds it) and the oracle's
    Dhop and DhopDag of them."""
    need_host_memory(4 * GiB)
    dims, Ls = (16, 16, 16, 16), 16
    c = make_case(dims, Ls)
    refs = {dag: oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, dag) for dag in (0, 1)}
    lat = gb.Lattice.periodic(dims, Ls)
    return c, lat, refs


@pytest.mark.parametrize("dag", [0, 1])
def test_fp64_16x16_matches_oracle(headline, dag):
    c, lat, refs = headline
    g = gb.Gauge(lat, c["U"], gb.F64)
    x, y = gb.Field(lat, gb.F64).load(c["phi"]), gb.Field(lat, gb.F64)
    gb.tune_dhop(g, y, x, dag)
    gb.dhop(g, y, x, dag)
    out = y.numpy()
    assert rel_err(out, refs[dag]) <= TOL[gb.F64]
    # the reference's own acceptance test: sum of squared differences <= 1e-10 (bench_simple.cc:114-119)
    assert float(np.sum((out - refs[dag]) ** 2)) <= 1e-10


@pytest.mark.parametrize("dag", [0, 1])
def test_fp32_16x16_matches_oracle_in_every_form(headline, dag):
    """The headline kernel: the tuner's pick and each candidate form, against the FP64
    oracle at the FP32 accuracy target, 1e-6 relative."""
    c, lat, refs = headline
    g = gb.Gauge(lat, c["U"], gb.F32)
    x, y = gb.Field(lat, gb.F32).load(c["phi"]), gb.Field(lat, gb.F32)
    gb.tune_dhop(g, y, x, dag)
    shapes = [tuple(gb.tune_query(g, x))] + FP32_LS16_FORMS
    for shape in shapes:
        gb.tune_set(g, x, *shape)
        y.zero()
        gb.dhop(g, y, x, dag)
        assert rel_err(y.numpy(), refs[dag]) <= TOL[gb.F32], shape


@pytest.mark.parametrize("dag", [0, 1])
def test_fp32_16x16_m_on_its_own_tuned_shape(headline, dag):
    """M (the CG's operator) runs on the shape the tuner timed for M itself, which may differ
    from the hopping term's; both match the oracle, and gbdw_tune_set pins the two together."""
    c, lat, _ = headline
    g = gb.Gauge(lat, c["U"], gb.F32)
    x, y = gb.Field(lat, gb.F32).load(c["phi"]), gb.Field(lat, gb.F32)
    gb.tune_dhop(g, y, x, dag)
    m_shape = gb.tune_query_m(g, x)
    assert len(m_shape) == 6 and m_shape[2] in range(5) and m_shape[4] >= 1 and m_shape[5] >= 1
    ref = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 16, 1.8, 0.01, dag)
    gb.dwf_m(g, y, x, 1.8, 0.01, dag)
    assert rel_err(y.numpy(), ref) <= TOL[gb.F32]
    for rp in (gb.F64, gb.F32):
        cg = gb.tune_query_cg(g, x, rp)
        assert len(cg) == 6 and cg[2] in range(5)
    gb.tune_set(g, x, 64, 2, 2, 2)
    assert gb.tune_query_m(g, x) == (64, 2, 2, 2, 1, 1)
    assert gb.tune_query_cg(g, x, gb.F64) == (64, 2, 2, 2, 1, 1)
    y.zero()
    gb.dwf_m(g, y, x, 1.8, 0.01, dag)
    assert rel_err(y.numpy(), ref) <= TOL[gb.F32]


def test_fp16_16x16_matches_oracle(headline):
    """The mixed CG's sloppy operator (FP16 spinors with per-slice norms, 12-real FP16 links)
    at the headline shape, with the tuner's pick."""
    c, lat, refs = headline
    g = gb.Gauge(lat, c["U"], gb.F16)
    x, y = gb.Field(lat, gb.F16).load(c["phi"]), gb.Field(lat, gb.F16)
    gb.tune_dhop(g, y, x)
    gb.dhop(g, y, x)
    assert rel_err(y.numpy(), refs[0]) <= TOL[gb.F16]


def test_multi_rhs_24x12_k12_matches_oracle(gpu):
    """12 Gaussian sources sharing one gauge field in a single launch (24^4 x Ls=12): every
    right-hand side equals the oracle's Dhop of its own source."""
    need_host_memory(6 * GiB)
    dims, Ls, k = (24, 24, 24, 24), 12, 12
    U = gb.generate_gauge(dims)
    nbr, prm, nsite = gb.generate_table(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, U, gb.F32)
    X, Y = gb.Field(lat, gb.F32, k), gb.Field(lat, gb.F32, k)
    seeds = [(100 + r, 6, 7, 8) for r in range(k)]
    for r in range(k):
        X.load(gb.generate_fermion(dims, Ls, 1, seeds[r]), r)
    gb.tune_dhop(g, Y, X)
    gb.dhop(g, Y, X)
    for r in range(k):
        src = gb.generate_fermion(dims, Ls, 1, seeds[r])
        ref = oracle.dslash(U, src, nbr, prm, nsite, Ls)
        assert rel_err(Y.numpy(r), ref) <= TOL[gb.F32], r


def batch_specs(n=64, seed=2024):
    """The benchmarked batch: 4D volumes uniform over {8^4, 12^4, 16^4, 20^4, 24^4}, Ls over
    {8, 12, 16}, FP32 or FP16 storage with equal odds."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        L = int(rng.choice([8, 12, 16, 20, 24]))
        Ls = int(rng.choice([8, 12, 16]))
        out.append(((L, L, L, L), Ls, gb.F32 if rng.random() < 0.5 else gb.F16))
    return out


def test_batch_64_instances_match_oracle(gpu):
    """Every instance of the 64-instance persistent batch (one graph replay) against the
    oracle's Dhop of its own inputs: FP32 within 1e-6, FP16 storage within 5e-3."""
    need_host_memory(4 * GiB)
    specs = batch_specs()
    keep, G, O, I = [], [], [], []
    for k, (dims, Ls, prec) in enumerate(specs):
        lat = gb.Lattice.periodic(dims, Ls)
        g = gb.Gauge(lat, gb.generate_gauge(dims, 1, (k, 1, 2, 3)), prec)
        x = gb.Field(lat, prec).load(gb.generate_fermion(dims, Ls, 1, (k, 4, 5, 6)))
        keep.append(lat)
        G.append(g)
        O.append(gb.Field(lat, prec))
        I.append(x)
    b = gb.Batch(G, O, I)
    b.run()
    b.run()
    gb.synchronize()
    for k, (dims, Ls, prec) in enumerate(specs):
        nbr, prm, nsite = gb.generate_table(dims, Ls)
        ref = oracle.dslash(gb.generate_gauge(dims, 1, (k, 1, 2, 3)), gb.generate_fermion(dims, Ls, 1, (k, 4, 5, 6)),
                            nbr, prm, nsite, Ls)
        assert rel_err(O[k].numpy(), ref) <= TOL[prec], (k, dims, Ls, prec)


@pytest.fixture(scope="module")
def cg32(gpu):
    need_host_memory(20 * GiB)
    dims, Ls = (32, 32, 32, 32), 16
    U = gb.generate_gauge(dims)
    phi = gb.generate_fermion(dims, Ls)
    nbr, prm, nsite = gb.generate_table(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    gs = {p: gb.Gauge(lat, U, p) for p in (gb.F64, gb.F32, gb.F16)}
    b = gb.Field(lat, gb.F64).load(phi)
    return {"U": U, "phi": phi, "nbr": nbr, "nsite": nsite, "Ls": Ls, "lat": lat, "g": gs, "b": b}


@pytest.mark.parametrize("mode", ["plain", "mixed_fp16"])
def test_cg_32x16_true_residual_recomputed_by_oracle(cg32, mode):
    """CG on M^dag M (Shamir, M5 = 1.8, mf = 0.01) at 32^4 x Ls=16 to a 1e-10 true residual,
    plain (FP32 operator, FP64 vectors) and mixed (FP16 operator and iterated residual,
    reliable updates), at the benchmark's thresholds; the solution's residual
    |b - M^dag M x| / |b| is recomputed on the host with the oracle's FP64 operator."""
    c = cg32
    g = c["g"]
    x = gb.Field(c["lat"], gb.F64)
    if mode == "plain":
        st = gb.cg_solve(g[gb.F64], x, c["b"], 1.8, 0.01, gb.CG_PLAIN, delta=1e-4, g32=g[gb.F32])
    else:
        st = gb.cg_solve(g[gb.F64], x, c["b"], 1.8, 0.01, gb.CG_MIXED, delta=0.03, g32=g[gb.F32],
                         gsloppy=g[gb.F16], sloppy_prec=gb.F16, sloppy_residual=1)
    assert st["true_residual"] <= 1e-10
    xs = x.numpy()
    del x
    Ax = oracle.dwf_mdagm(c["U"], xs, c["nbr"], c["nsite"], c["Ls"], 1.8, 0.01)
    res = float(np.linalg.norm(c["phi"] - Ax) / np.linalg.norm(c["phi"]))
    print(mode, st, "oracle residual", res)
    assert res <= 2e-10
