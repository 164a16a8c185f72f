"""Halo packing on the GPU: every face, both projector sets, F64/F32/F16, against the numpy
restatement; and a two-domain decomposition fed by the GPU-packed halos reproduces the
full-lattice Dhop oracle."""
import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle
from oracle import halo
from conftest import make_case, rel_err
from test_halo_oracle import domain_dhop, split

pytestmark = pytest.mark.gpu

TOL = {gb.F64: 1e-15, gb.F32: 1e-7, gb.F16: 2e-3}


def parse(buf, prec, nface, LsE):
    """The transport format of include/gbdw.h -> (nface, LsE, 2, 3) complex."""
    LsP = LsE if prec == gb.F64 else LsE + (LsE & 1)
    if prec == gb.F64:
        a = buf.view(np.float64).reshape(nface, 6, LsP, 2)
        z = a[..., 0] + 1j * a[..., 1]
    else:
        dt, es = (np.float32, 8) if prec == gb.F32 else (np.float16, 4)  # bytes per complex slot
        nv = nface * 6 * LsP * es
        a = buf[:nv].view(dt).astype(np.float64).reshape(nface, 6, LsP // 2, 4)
        re = a[..., 0:2].reshape(nface, 6, LsP)
        im = a[..., 2:4].reshape(nface, 6, LsP)
        z = re + 1j * im
        if prec == gb.F16:
            nrm = buf[nv:].view(np.float32).reshape(nface, LsE)
            z[:, :, :LsE] *= nrm[:, None, :]
    return z[:, :, :LsE].transpose(0, 2, 1).reshape(nface, LsE, 2, 3)


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("Ls", [3, 8])
def test_pack_every_face(gpu, prec, dag, Ls):
    dims = (4, 2, 6, 4)
    c = make_case(dims, Ls)
    lat = gb.Lattice.periodic(dims, Ls)
    f = gb.Field(lat, prec).load(c["phi"])
    for mu in range(4):
        nface = int(np.prod(dims)) // dims[mu]
        for face in (0, 1):
            got = parse(f.halo_pack(mu, face, dag), prec, nface, Ls)
            ref = halo.pack(c["phi"], dims, Ls, mu, face, dag)
            assert got.shape == ref.shape
            assert rel_err(got.reshape(-1).view(np.float64), ref.reshape(-1).view(np.float64)) < TOL[prec], (mu, face)


def test_pack_sizes_and_rejections(gpu):
    lat = gb.Lattice.periodic((4, 4, 2, 6), 5)
    f32, f16 = gb.Field(lat, gb.F32), gb.Field(lat, gb.F16)
    assert f32.halo_bytes(2) == 4 * 4 * 6 * 6 * 6 * 8        # face sites x 6 rows x LsP 6 x 8 B
    assert f16.halo_bytes(3) == 4 * 4 * 2 * 6 * 6 * 4 + 4 * 4 * 2 * 5 * 4
    with pytest.raises(gb.GbdwError):
        f32.halo_pack(4, 0)
    with pytest.raises(gb.GbdwError):
        f32.halo_pack(0, 2)
    ev, od = lat.checkerboard()
    with pytest.raises(gb.GbdwError):
        gb.Field(ev, gb.F32).halo_bytes(0)


@pytest.mark.parametrize("prec,tol", [(gb.F64, 1e-14), (gb.F32, 1e-6), (gb.F16, 5e-3)])
@pytest.mark.parametrize("dag", [0, 1])
def test_two_domains_fed_by_gpu_halos(gpu, prec, tol, dag):
    c = make_case((4, 4, 4, 4), 4)
    for mu in range(4):
        D, maps, (fa, fb) = split(c, mu)
        la = gb.Lattice.periodic(D, 4)
        A = gb.Field(la, prec).load(fa)
        nface = int(np.prod(D)) // D[mu]
        halos = tuple(parse(A.halo_pack(mu, face, dag), prec, nface, 4) for face in (0, 1))
        got = domain_dhop(c, mu, dag, D, maps, halos)
        full = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 4, dag)
        ref = full.view(np.complex128).reshape(-1, 4, 12)[maps[1]].reshape(-1).view(np.float64)
        assert rel_err(got, ref) < tol, mu


def test_pack_into_device_memory(gpu):
    """A device destination (here a CUDA allocation made by torch, used only as memory) gets the
    same bytes as the host path."""
    torch = pytest.importorskip("torch")
    dims, Ls = (4, 4, 4, 4), 8
    c = make_case(dims, Ls)
    f = gb.Field(gb.Lattice.periodic(dims, Ls), gb.F32).load(c["phi"])
    host = f.halo_pack(1, 1, 0)
    dev = torch.empty(host.size, dtype=torch.uint8, device="cuda")
    gb.check(gb.load().gbdw_halo_pack(f.h, 1, 1, 0, gb.C.c_void_p(dev.data_ptr())))
    gb.synchronize()
    assert np.array_equal(dev.cpu().numpy(), host)


@pytest.mark.parametrize("prec", [gb.F64, gb.F32, gb.F16])
@pytest.mark.parametrize("Ls", [5, 8])
def test_pack_all_faces_one_launch(gpu, prec, Ls):
    """The eight faces of one launch equal the single-face packs byte for byte."""
    torch = pytest.importorskip("torch")
    dims = (4, 2, 6, 4)
    c = make_case(dims, Ls)
    f = gb.Field(gb.Lattice.periodic(dims, Ls), prec).load(c["phi"])
    for dag in (0, 1):
        bufs = [torch.zeros(f.halo_bytes(k // 2), dtype=torch.uint8, device="cuda") for k in range(8)]
        n0 = gb.launch_count()
        f.halo_pack_all([b.data_ptr() for b in bufs], dag)
        assert gb.launch_count() - n0 == 1
        gb.synchronize()
        for k in range(8):
            one = f.halo_pack(k // 2, k % 2, dag)
            got = bufs[k].cpu().numpy()
            LsP = Ls if prec == gb.F64 else Ls + (Ls & 1)
            if LsP == Ls:
                assert np.array_equal(got, one), k
            else:  # the padded slot of odd extents is not written
                nface = int(np.prod(dims)) // dims[k // 2]
                assert rel_err(parse(got, prec, nface, Ls).reshape(-1).view(np.float64),
                               parse(one, prec, nface, Ls).reshape(-1).view(np.float64)) == 0.0


@pytest.mark.parametrize("prec", [gb.F32, gb.F16])
def test_pack_multi_rhs_field(gpu, prec):
    """A field with several right-hand sides (slices rhs-innermost, e = s * nrhs + r) packs every
    rhs's half spinors in its own slice positions."""
    dims, Ls, k = (4, 2, 2, 4), 4, 3
    lat = gb.Lattice.periodic(dims, Ls)
    srcs = [gb.generate_fermion(dims, Ls, 1, (3 + r, 4, 5, 6)) for r in range(k)]
    f = gb.Field(lat, prec, k)
    for r in range(k):
        f.load(srcs[r], r)
    for mu in range(4):
        nface = int(np.prod(dims)) // dims[mu]
        for face in (0, 1):
            got = parse(f.halo_pack(mu, face, 0), prec, nface, Ls * k).reshape(nface, Ls, k, 2, 3)
            for r in range(k):
                ref = halo.pack(srcs[r], dims, Ls, mu, face, 0)
                assert rel_err(np.ascontiguousarray(got[:, :, r]).reshape(-1).view(np.float64),
                               ref.reshape(-1).view(np.float64)) < TOL[prec], (mu, face, r)
