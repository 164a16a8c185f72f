"""GPU hopping term (FP64/FP32, Dhop/DhopDag) against the oracle, the reference's golden
vectors, the drop-in seam, lane layouts, general tables and full-size properties."""
import glob
import os

import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from conftest import GOLDEN, make_case, rel_err

pytestmark = pytest.mark.gpu

TOL = {gb.F64: 1e-12, gb.F32: 1e-6}  # relative to the FP64 oracle (1e-6: the FP32 target)


def _run(c, prec, dag=0, nrhs=1):
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], c["Ls"], c["nsimd"])
    g = gb.Gauge(lat, c["U"], prec)
    x = gb.Field(lat, prec).load(c["phi"])
    y = gb.Field(lat, prec)
    gb.dhop(g, y, x, dag)
    return y.numpy(), lat


@pytest.mark.parametrize("dims,Ls", [((2, 2, 2, 2), 4), ((4, 4, 4, 4), 4), ((4, 2, 6, 2), 3), ((8, 8, 8, 8), 8)])
@pytest.mark.parametrize("prec", [gb.F64, gb.F32])
@pytest.mark.parametrize("dag", [0, 1])
def test_dhop_matches_oracle(gpu, dims, Ls, prec, dag):
    c = make_case(dims, Ls)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, dag)
    out, lat = _run(c, prec, dag)
    assert lat.info()["fast"]
    assert rel_err(out, ref) < TOL[prec]


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "golden_simple_*.npz"))))
def test_fp64_matches_dslash_simple_golden(gpu, f):
    g = np.load(f)
    c = make_case(tuple(g["dims"]), int(g["Ls"]))
    out, _ = _run(c, gb.F64)
    assert rel_err(out, g["psi"]) < 1e-13
    # the reference's own check: sum of squared differences <= 1e-10 (bench_simple.cc:114-119)
    assert float(np.sum((out - g["psi"]) ** 2)) <= 1e-10


@pytest.mark.parametrize("f", sorted(glob.glob(os.path.join(GOLDEN, "golden_hand_*.npz"))))
def test_dropin_lane_layout_matches_hand_kernel_golden(gpu, f):
    """bench.cc's VGPU flow: Nsimd-lane data through dslash_kernel, compared with the
    reference's AVX-512 hand kernel output on the same data."""
    g = np.load(f)
    ns = int(g["nsimd"])
    dt = np.float64 if "f64" in os.path.basename(f) else np.float32
    c = make_case(tuple(g["dims"]), int(g["Ls"]), ns)
    U = c["U"].astype(dt)
    phi = c["phi"].astype(dt)
    out = np.zeros_like(phi)
    usec = gb.dslash_kernel(3, U, out, phi, c["nbr"], c["nsite"], c["Ls"], c["prm"], nsimd=ns)
    assert usec > 0
    assert rel_err(out, g["psi"]) < (1e-13 if dt == np.float64 else 1e-6)


@pytest.mark.parametrize("nsimd", [2, 4, 8, 16])
@pytest.mark.parametrize("dag", [0, 1])
def test_lane_layouts_match_oracle(gpu, nsimd, dag):
    c = make_case((4, 4, 4, 4), 4, nsimd)
    ref = oracle.dslash_lanes(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 4, nsimd, dag)
    out = np.zeros_like(c["phi"])
    # the seam has no dag argument in the reference; use the object API for dag
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 4, nsimd)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x = gb.Field(lat, gb.F64).load(c["phi"])
    y = gb.Field(lat, gb.F64)
    gb.dhop(g, y, x, dag)
    assert rel_err(y.numpy(), ref) < 1e-13
    if dag == 0:
        gb.dslash_kernel(1, c["U"].copy(), out, c["phi"], c["nbr"], c["nsite"], 4, c["prm"], nsimd=nsimd)
        assert rel_err(out, ref) < 1e-13


def test_dslash_kernel_dropin_nrep_and_timing(gpu):
    c = make_case((4, 4, 4, 4), 8)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 8)
    for dt, tol in ((np.float64, 1e-13), (np.float32, 1e-6)):
        out = np.zeros(c["phi"].shape, dtype=dt)
        usec = gb.dslash_kernel(5, c["U"].astype(dt), out, c["phi"].astype(dt), c["nbr"], c["nsite"], 8, c["prm"])
        assert usec > 0
        assert rel_err(out, ref) < tol


def test_general_table_path(gpu):
    """A table that does not factorise into nbr4*Ls + s runs on the general gather kernel
    and still follows the table exactly (the reference kernel obeys any table)."""
    c = make_case((4, 4, 2, 2), 4)
    t = c["nbr"].reshape(c["nsite"], 4, 8).copy()
    Ls = 4
    # X-forward leg also steps one slice in s
    site = t[:, :, 0] // Ls
    s = t[:, :, 0] % Ls
    t[:, :, 0] = site * Ls + (s + 1) % Ls
    nbr = t.ravel()
    ref = oracle.dslash(c["U"], c["phi"], nbr, c["prm"], c["nsite"], Ls)
    for prec in (gb.F64, gb.F32):
        lat = gb.Lattice.from_table(nbr, c["prm"], c["nsite"], Ls)
        assert not lat.info()["fast"]
        g = gb.Gauge(lat, c["U"], prec)
        x = gb.Field(lat, prec).load(c["phi"])
        y = gb.Field(lat, prec)
        gb.dhop(g, y, x)
        assert rel_err(y.numpy(), ref) < TOL[prec]


def test_table_out_of_range_is_rejected(gpu):
    c = make_case((2, 2, 2, 2), 2)
    nbr = c["nbr"].copy()
    nbr[5] = c["nsite"] * 2 + 7
    with pytest.raises(gb.GbdwError) as e:
        gb.Lattice.from_table(nbr, c["prm"], c["nsite"], 2)
    assert e.value.status == 4


SHAPES = {gb.F32: [(0, s, 4) for s in (1, 2, 4)] + [(f, s, st) for f in (1, 2) for s in (1, 2) for st in (2, 4)],
          gb.F64: [(0, s, 4) for s in (1, 2)] + [(f, s, st) for f in (1, 2) for s in (1, 2) for st in (2, 4)]}


@pytest.mark.parametrize("prec", [gb.F32, gb.F64])
@pytest.mark.parametrize("threads", [64, 128, 256])
@pytest.mark.parametrize("Ls", [8, 12])
def test_every_launch_shape(gpu, prec, threads, Ls):
    """Direct and TMA-staged forms, every compiled slice split and stage count, Dhop and
    DhopDag, including a lattice whose site count is not a multiple of the CTA's sites."""
    c = make_case((4, 6, 2, 3), Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], prec)
    x = gb.Field(lat, prec).load(c["phi"])
    y = gb.Field(lat, prec)
    for dag in (0, 1):
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, dag)
        for form, spt, stages in SHAPES[prec]:
            if Ls % spt:
                continue
            try:
                gb.tune_set(g, x, threads, spt, form, stages)
            except gb.GbdwError:
                assert form != 0  # a staged ring that does not fit (or a site wider than a warp)
                continue
            y.zero()
            gb.dhop(g, y, x, dag)
            assert rel_err(y.numpy(), ref) < TOL[prec], (form, spt, stages, dag)
    gb.synchronize()


@pytest.mark.parametrize("shape", [(128, 2, 0, 4), (64, 2, 3, 4), (128, 2, 2, 2), (64, 2, 2, 2)])
def test_fp32_ls16_specialised_kernels(gpu, shape):
    """FP32 with Ls*nrhs = 16 runs kernels whose row stride is a compile-time constant (the
    direct form, form 3 and the two-stage warp rings): Dhop, DhopDag and the fused M."""
    c = make_case((4, 6, 2, 3), 16)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 16)
    g = gb.Gauge(lat, c["U"], gb.F32)
    x = gb.Field(lat, gb.F32).load(c["phi"])
    y = gb.Field(lat, gb.F32)
    gb.tune_set(g, x, *shape)
    assert tuple(gb.tune_query(g, x)) == shape
    for dag in (0, 1):
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 16, dag)
        y.zero()
        gb.dhop(g, y, x, dag)
        assert rel_err(y.numpy(), ref) < TOL[gb.F32], (shape, dag)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 16, 1.8, 0.01, dag)
        gb.dwf_m(g, y, x, 1.8, 0.01, dag)
        assert rel_err(y.numpy(), refm) < TOL[gb.F32], (shape, dag)
    gb.synchronize()


def test_periodic_lattice_equals_table_lattice(gpu):
    c = make_case((4, 6, 2, 4), 4)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 4)
    lat = gb.Lattice.periodic((4, 6, 2, 4), 4)
    g = gb.Gauge(lat, c["U"], gb.F64)
    x = gb.Field(lat, gb.F64).load(c["phi"])
    y = gb.Field(lat, gb.F64)
    gb.dhop(g, y, x)
    assert rel_err(y.numpy(), ref) < 1e-13


def test_multi_rhs_equals_single_rhs(gpu):
    dims, Ls, k = (4, 4, 4, 4), 4, 3
    c = make_case(dims, Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], gb.F32)
    X = gb.Field(lat, gb.F32, k)
    Y = gb.Field(lat, gb.F32, k)
    srcs = [gb.generate_fermion(dims, Ls, 1, (5 + r, 6, 7, 8)) for r in range(k)]
    for r in range(k):
        X.load(srcs[r], r)
    gb.dhop(g, Y, X)
    for r in range(k):
        ref = oracle.dslash(c["U"], srcs[r], c["nbr"], c["prm"], c["nsite"], Ls)
        assert rel_err(Y.numpy(r), ref) < 1e-6


def test_full_size_properties_16x16(gpu):
    """16^4 x 16 (the roofline workload): FP32 within 1e-6 of the GPU FP64 result, DhopDag
    adjoint to Dhop, linearity -- properties that do not need the CPU oracle at full size."""
    dims, Ls = (16, 16, 16, 16), 16
    lat = gb.Lattice.periodic(dims, Ls)
    U = gb.generate_gauge(dims)
    g64 = gb.Gauge(lat, U, gb.F64)
    g32 = gb.Gauge(lat, U, gb.F32)
    a = gb.generate_fermion(dims, Ls)
    b = gb.generate_fermion(dims, Ls, 1, (9, 10, 11, 12))
    x64 = gb.Field(lat, gb.F64).load(a)
    y64 = gb.Field(lat, gb.F64)
    x32 = gb.Field(lat, gb.F32).load(a)
    y32 = gb.Field(lat, gb.F32)
    for dag in (0, 1):
        gb.dhop(g64, y64, x64, dag)
        gb.dhop(g32, y32, x32, dag)
        d = gb.Field(lat, gb.F64)
        d.copy_from(y32)
        d.axpby(-1.0, y64, 1.0)
        assert np.sqrt(d.norm2() / y64.norm2()) < 1e-6
    # <b, D a> == <Ddag b, a>
    bf = gb.Field(lat, gb.F64).load(b)
    Da = gb.Field(lat, gb.F64)
    Ddb = gb.Field(lat, gb.F64)
    gb.dhop(g64, Da, x64, 0)
    gb.dhop(g64, Ddb, bf, 1)
    lhs = bf.dot(Da)
    rhs = Ddb.dot(x64)
    assert abs(lhs - rhs) / abs(lhs) < 1e-12
    # linearity: D(2a + b) = 2 Da + Db
    s = gb.Field(lat, gb.F64)
    s.copy_from(bf)
    s.axpby(2.0, x64, 1.0)
    Ds = gb.Field(lat, gb.F64)
    gb.dhop(g64, Ds, s, 0)
    Db = gb.Field(lat, gb.F64)
    gb.dhop(g64, Db, bf, 0)
    Ds.axpby(-2.0, Da, 1.0)
    Ds.axpby(-1.0, Db, 1.0)
    assert np.sqrt(Ds.norm2() / Db.norm2()) < 1e-13


@pytest.mark.parametrize("prec,tol", [(gb.F32, 1e-6), (gb.F16, 5e-3)])
def test_blocked_site_order_form(gpu, prec, tol):
    """Form 4: the Ls = 16 kernel with each CTA on a 2x2x2x2 block of sites (periodic lattice,
    even extents): Dhop, DhopDag and M, against the oracle."""
    dims = (4, 6, 2, 4)
    c = make_case(dims, 16)
    lat = gb.Lattice.periodic(dims, 16)
    g = gb.Gauge(lat, c["U"], prec)
    x = gb.Field(lat, prec).load(c["phi"])
    y = gb.Field(lat, prec)
    gb.tune_set(g, x, 128, 2, 4, 4)
    assert tuple(gb.tune_query(g, x)) == (128, 2, 4, 4)
    for dag in (0, 1):
        gb.dhop(g, y, x, dag)
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 16, dag)
        assert rel_err(y.numpy(), ref) < tol, dag
        n2 = gb.dwf_m(g, y, x, 1.8, 0.01, dag, want_norm=True)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 16, 1.8, 0.01, dag)
        out = y.numpy()
        assert rel_err(out, refm) < tol, dag
        assert abs(n2 - float(np.sum(out ** 2))) / n2 < 1e-5
    # a table lattice has no extents: the form is refused
    lt = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 16)
    gt = gb.Gauge(lt, c["U"], prec)
    xt = gb.Field(lt, prec).load(c["phi"])
    with pytest.raises(gb.GbdwError):
        gb.tune_set(gt, xt, 128, 2, 4, 4)
    gb.synchronize()


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
def test_pinned_host_import_export_and_queued_export(gpu, prec):
    """Page-locked host buffers through the synchronous and the queued export on a library
    stream give the same result as pageable memory; a queued export into pageable memory is
    refused."""
    dims, Ls = (4, 4, 2, 6), 8
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    n = c["phi"].size
    hin = gb.PinnedArray(n, np.float64)
    hin.array[:] = c["phi"]
    x_pinned = gb.Field(lat, prec).load(hin.array)
    x_paged = gb.Field(lat, prec).load(np.array(c["phi"]))
    ref = x_paged.numpy()
    assert np.array_equal(x_pinned.numpy(), ref)
    hout = gb.PinnedArray(n, np.float64)
    x_pinned.export_into(hout.array)
    assert np.array_equal(hout.array, ref)
    hout.array[:] = 0.0
    with gb.Stream() as s:
        x_pinned.export_into(hout.array, sync=False)
        gb.synchronize()
    assert np.array_equal(hout.array, ref)
    with pytest.raises(gb.GbdwError):
        x_pinned.export_into(np.zeros(n), sync=False)


@pytest.mark.parametrize("form", [0, 3])
def test_fp32_ls12_and_12_rhs_specialised_kernels(gpu, form):
    """FP32 at Ls = 12 with one right-hand side (Ls*nrhs = 12) and with 12 (144): the direct form
    and form 3 with compile-time row strides give the oracle's Dhop / DhopDag for every rhs,
    and M at Ls = 12."""
    dims, Ls, k = (4, 2, 4, 2), 12, 12
    c = make_case(dims, Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], gb.F32)
    x1, y1 = gb.Field(lat, gb.F32).load(c["phi"]), gb.Field(lat, gb.F32)
    X, Y = gb.Field(lat, gb.F32, k), gb.Field(lat, gb.F32, k)
    srcs = [gb.generate_fermion(dims, Ls, 1, (5 + r, 6, 7, 8)) for r in range(k)]
    for r in range(k):
        X.load(srcs[r], r)
    gb.tune_set(g, x1, 64, 2, form, 4)
    gb.tune_set(g, X, 64, 2, form, 4)
    assert tuple(gb.tune_query(g, X)) == (64, 2, form, 4)
    for dag in (0, 1):
        gb.dhop(g, y1, x1, dag)
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], Ls, dag)
        assert rel_err(y1.numpy(), ref) < TOL[gb.F32], dag
        gb.dwf_m(g, y1, x1, 1.8, 0.01, dag)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], Ls, 1.8, 0.01, dag)
        assert rel_err(y1.numpy(), refm) < TOL[gb.F32], dag
        gb.dhop(g, Y, X, dag)
        for r in range(k):
            ref = oracle.dslash(c["U"], srcs[r], c["nbr"], c["prm"], c["nsite"], Ls, dag)
            assert rel_err(Y.numpy(r), ref) < TOL[gb.F32], (dag, r)
    gb.synchronize()


@pytest.mark.parametrize("form,threads", [(0, 128), (0, 64), (3, 64)])
@pytest.mark.parametrize("split", [1, 2, 4])
def test_direct_forms_with_ls_and_rhs_tiles(gpu, form, threads, split):
    """Ls / RHS tiles of the direct forms (each site's slices cut into `split` tiles, threads
    ordered tile, site, group): Dhop, DhopDag and M at Ls = 16 with one right-hand side, and Dhop
    with 12 right-hand sides at Ls = 12 (form 3 exists there for FP32 Dhop), every rhs against
    the oracle."""
    c = make_case((4, 6, 2, 3), 16)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], 16)
    g = gb.Gauge(lat, c["U"], gb.F32)
    x, y = gb.Field(lat, gb.F32).load(c["phi"]), gb.Field(lat, gb.F32)
    gb.tune_set(g, x, threads, 2, form, 4)
    gb.tune_set_split(g, x, split)
    assert gb.tune_split(g, x) == split
    for dag in (0, 1):
        y.zero()
        gb.dhop(g, y, x, dag)
        ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 16, dag)
        assert rel_err(y.numpy(), ref) < TOL[gb.F32], (form, split, dag)
        n2 = gb.dwf_m(g, y, x, 1.8, 0.01, dag, want_norm=True)
        refm = oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 16, 1.8, 0.01, dag)
        out = y.numpy()
        assert rel_err(out, refm) < TOL[gb.F32], (form, split, dag)
        assert abs(n2 - float(np.sum(out ** 2))) / n2 < 1e-5
    # 12 right-hand sides: tiles of 72 / 36 slices (6 / 3 values of s with all 12 rhs)
    dims, Ls, k = (4, 2, 4, 2), 12, 12
    c = make_case(dims, Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], gb.F32)
    X, Y = gb.Field(lat, gb.F32, k), gb.Field(lat, gb.F32, k)
    srcs = [gb.generate_fermion(dims, Ls, 1, (5 + r, 6, 7, 8)) for r in range(k)]
    for r in range(k):
        X.load(srcs[r], r)
    gb.tune_set(g, X, threads, 2, form, 4)
    gb.tune_set_split(g, X, split)
    gb.dhop(g, Y, X)
    for r in range(k):
        ref = oracle.dslash(c["U"], srcs[r], c["nbr"], c["prm"], c["nsite"], Ls)
        assert rel_err(Y.numpy(r), ref) < TOL[gb.F32], (form, split, r)
    with pytest.raises(gb.GbdwError):
        gb.tune_set_split(g, X, 5)  # 144 slices do not cut into 5 tiles
    gb.synchronize()


@pytest.mark.parametrize("form,threads", [(0, 128), (3, 64)])
@pytest.mark.parametrize("split", [3, 6, 12, 36])
def test_multi_rhs_tile_sweeps(gpu, form, threads, split):
    """12 right-hand sides at Ls = 12 (144 slices per site) in 3 to 36 tile sweeps: tiles of
    whole values of s (48, 24, 12 slices) and of some right-hand sides at one s (4 slices); every
    rhs against the oracle, Dhop and DhopDag."""
    dims, Ls, k = (4, 2, 4, 2), 12, 12
    c = make_case(dims, Ls)
    lat = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)
    g = gb.Gauge(lat, c["U"], gb.F32)
    X, Y = gb.Field(lat, gb.F32, k), gb.Field(lat, gb.F32, k)
    srcs = [gb.generate_fermion(dims, Ls, 1, (5 + r, 6, 7, 8)) for r in range(k)]
    for r in range(k):
        X.load(srcs[r], r)
    gb.tune_set(g, X, threads, 2, form, 4)
    gb.tune_set_split(g, X, split)
    for dag in (0, 1):
        Y.zero()
        gb.dhop(g, Y, X, dag)
        for r in range(k):
            ref = oracle.dslash(c["U"], srcs[r], c["nbr"], c["prm"], c["nsite"], Ls, dag)
            assert rel_err(Y.numpy(r), ref) < TOL[gb.F32], (form, split, dag, r)
    gb.synchronize()


@pytest.mark.parametrize("form,threads", [(0, 128), (3, 64)])
@pytest.mark.parametrize("brick", [2, 4, 8])
def test_t_brick_sweep_orders(gpu, form, threads, brick):
    """t-brick sweep orders of the direct forms on a periodic lattice (Lt = 8): Dhop, DhopDag and
    M at Ls = 16, 12 right-hand sides at Ls = 12 (form 3 at Ls*nrhs = 144), the Mobius adjoint's
    single pass, and a brick combined with a tile split — all against the oracle."""
    from oracle import mobius as mob
    dims = (4, 2, 4, 8)
    c = make_case(dims, 16)
    lat = gb.Lattice.periodic(dims, 16)
    g = gb.Gauge(lat, c["U"], gb.F32)
    x, y, t = gb.Field(lat, gb.F32).load(c["phi"]), gb.Field(lat, gb.F32), gb.Field(lat, gb.F32)
    gb.tune_set(g, x, threads, 2, form, 4)
    gb.tune_set_brick(g, x, brick)
    assert gb.tune_brick(g, x) == brick
    for dag in (0, 1):
        y.zero()
        gb.dhop(g, y, x, dag)
        assert rel_err(y.numpy(), oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 16, dag)) < 1e-6
        n2 = gb.dwf_m(g, y, x, 1.8, 0.01, dag, want_norm=True)
        out = y.numpy()
        assert rel_err(out, oracle.dwf_m(c["U"], c["phi"], c["nbr"], c["nsite"], 16, 1.8, 0.01, dag)) < 1e-6
        assert abs(n2 - float(np.sum(out ** 2))) / n2 < 1e-5
        gb.mobius_m(g, y, t, x, 1.5, 0.5, 1.8, 0.01, dag)
        ref = mob.mobius_m(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 16, 1.5, 0.5, 1.8, 0.01, dag)
        assert rel_err(y.numpy(), ref) < 1e-6, dag
    if form == 0:
        gb.tune_set_split(g, x, 2)  # a brick and a tile split together
        gb.dhop(g, y, x)
        assert rel_err(y.numpy(), oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 16)) < 1e-6
    Ls, k = 12, 12
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    g = gb.Gauge(lat, c["U"], gb.F32)
    X, Y = gb.Field(lat, gb.F32, k), gb.Field(lat, gb.F32, k)
    srcs = [gb.generate_fermion(dims, Ls, 1, (5 + r, 6, 7, 8)) for r in range(k)]
    for r in range(k):
        X.load(srcs[r], r)
    gb.tune_set(g, X, threads, 2, form, 4)
    gb.tune_set_brick(g, X, brick)
    gb.dhop(g, Y, X)
    for r in range(k):
        ref = oracle.dslash(c["U"], srcs[r], c["nbr"], c["prm"], c["nsite"], Ls)
        assert rel_err(Y.numpy(r), ref) < 1e-6, r
    with pytest.raises(gb.GbdwError):
        gb.tune_set_brick(g, X, 3)  # Lt = 8 is not a multiple of 3
    lt = gb.Lattice.from_table(c["nbr"], c["prm"], c["nsite"], Ls)  # no extents: no bricks
    gt = gb.Gauge(lt, c["U"], gb.F32)
    xt = gb.Field(lt, gb.F32, k)
    gb.tune_set(gt, xt, threads, 2, form, 4)
    with pytest.raises(gb.GbdwError):
        gb.tune_set_brick(gt, xt, 2)
    gb.synchronize()
