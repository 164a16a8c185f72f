"""The C++ drivers that keep bench.cc / bench_simple.cc's flow, linked to libgbdw.so through
include/gbdw_dslash.h, checked against the oracle's result."""
import os
import re
import subprocess

import numpy as np
import pytest

from gridbench_gb300 import build
import oracle
from conftest import make_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def exes(gpu):
    build.build_lib()
    return build.build_drivers()


def test_bench_flow_driver(exes, tmp_path):
    for nsimd, flag in ((1, []), (4, []), (8, ["--float"])):
        c = make_case((4, 4, 4, 4), 8, nsimd)
        if nsimd == 1:
            ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 8)
        else:
            ref = oracle.dslash_lanes(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 8, nsimd)
        p = tmp_path / f"ref{nsimd}.bin"
        ref.astype(np.float64).tofile(p)
        r = subprocess.run([exes["bench_gb300"], "--dims", "4", "4", "4", "4", "--Ls", "8", "--nsimd", str(nsimd),
                            "--nrep", "20", "--ref", str(p)] + flag, capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "Gflop/s" in r.stdout
        rel = float(re.search(r"reldiff ([0-9.eE+-]+)", r.stdout).group(1))
        assert rel < (1e-6 if flag else 1e-13), r.stdout


def test_bench_simple_flow_driver(exes, tmp_path):
    c = make_case((4, 4, 4, 4), 4)
    ref = oracle.dslash(c["U"], c["phi"], c["nbr"], c["prm"], c["nsite"], 4)
    p = tmp_path / "ref.bin"
    ref.tofile(p)
    r = subprocess.run([exes["bench_simple_gb300"], "--dims", "4", "4", "4", "4", "--Ls", "4", "--nrep", "10",
                        "--ref", str(p)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "normdiff" in r.stdout


def test_dropin_kernel_on_a_static_data_file(gpu, tmp_path):
    """The flow of bench_simple.cc on data read from a static_data.h / .cc pair: the drop-in
    seam reproduces the file's reference result to the 9 digits the format keeps."""
    import gridbench_gb300 as gb
    from conftest import rel_err
    dims, Ls = (4, 4, 2, 2), 8
    U = gb.generate_gauge(dims)
    phi = gb.generate_fermion(dims, Ls)
    nbr, prm, nsite = gb.generate_table(dims, Ls)
    psi = oracle.dslash(U, phi, nbr, prm, nsite, Ls)
    h, cc = str(tmp_path / "static_data.h"), str(tmp_path / "static_data.cc")
    gb.write_static_data(h, cc, nsite, Ls, U, phi, psi, nbr, prm)
    d = gb.read_static_data(h, cc)
    out = np.zeros_like(d["Phi"])
    gb.dslash_kernel(1, d["U"], out, d["Phi"], d["nbr"], d["nsite"], d["Ls"], d["prm"])
    assert rel_err(out, d["Psi"]) < 1e-7
