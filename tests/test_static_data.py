"""The reference's static-data files (TableGenerate.cc:93-138): the writer's layout, and a
write -> read round trip that keeps tables exact and doubles to the format's 9 digits.
Host-only (no device)."""
import os
import re

import numpy as np
import pytest

import gridbench_gb300 as gb
import oracle


@pytest.mark.parametrize("nsimd", [1, 4])
def test_static_data_round_trip(tmp_path, nsimd):
    dims, Ls = (4, 2, 2, 4), 4
    U = gb.generate_gauge(dims, nsimd)
    phi = gb.generate_fermion(dims, Ls, nsimd)
    nbr, prm, nsite = gb.generate_table(dims, Ls, nsimd)
    psi = oracle.dslash_lanes(U, phi, nbr, prm, nsite, Ls, nsimd) if nsimd > 1 else \
        oracle.dslash(U, phi, nbr, prm, nsite, Ls)
    h, cc = str(tmp_path / "static_data.h"), str(tmp_path / "static_data.cc")
    gb.write_static_data(h, cc, nsite, Ls, U, phi, psi, nbr, prm, nsimd)
    d = gb.read_static_data(h, cc)
    assert (d["nsite"], d["Ls"], d["nsimd"]) == (nsite, Ls, nsimd)
    assert np.array_equal(d["nbr"], np.asarray(nbr, np.uint64))
    assert np.array_equal(d["prm"], np.asarray(prm, np.uint8))
    for k, ref in (("U", U), ("Phi", phi), ("Psi", psi)):
        ref = np.asarray(ref, np.float64).ravel()
        assert d[k].shape == ref.shape
        assert np.max(np.abs(d[k] - ref) / np.maximum(np.abs(ref), 1e-300)) <= 5.1e-9, k


def test_static_data_layout(tmp_path):
    """Line layout of the files the reference's benchmarks compile in: one entry per line, the
    arrays closed by a sentinel 0, the header's two constants and five extern declarations."""
    dims, Ls = (2, 2, 2, 2), 2
    U = gb.generate_gauge(dims)
    phi = gb.generate_fermion(dims, Ls)
    nbr, prm, nsite = gb.generate_table(dims, Ls)
    h, cc = str(tmp_path / "static_data.h"), str(tmp_path / "static_data.cc")
    gb.write_static_data(h, cc, nsite, Ls, U, phi, phi, nbr, prm)
    head = open(h).read().splitlines()
    assert head[0] == "#include <stdint.h>"
    assert re.fullmatch(r"const uint64_t nsite = 16 ; ", head[1])
    assert re.fullmatch(r"const int Ls = 2 ; ", head[2])
    assert [ln.split()[-2] for ln in head[3:]] == ["U_static[]", "Phi_static[]", "Psi_cpp_static[]",
                                                   "nbr_static[]", "prm_static[]"]
    text = open(cc).read()
    for name, n in (("U_static", nsite * 144), ("Phi_static", nsite * Ls * 24), ("nbr_static", nsite * Ls * 8)):
        body = text[text.index(name + "[] = {"):]
        body = body[:body.index("}")]
        entries = [e.strip() for e in body.split("{", 1)[1].split(",")]
        assert len(entries) == n + 1 and entries[-1] == "0"
    first = text.split("double U_static[] = { \n ", 1)[1].split("\n", 1)[0]
    # "%16.8le": a 16-wide field after four spaces, 8 digits after the point
    assert re.fullmatch(r"    [ -]*\d\.\d{8}e[+-]\d\d, ", first) and len(first) == 4 + 16 + 2, first
    assert re.search(r"\n    0x[0-9a-f]+, \n", text)


def test_static_data_rejects_inconsistent_files(tmp_path):
    h, cc = tmp_path / "static_data.h", tmp_path / "static_data.cc"
    h.write_text("#include <stdint.h>\nconst uint64_t nsite = 2 ; \nconst int Ls = 1 ; \n")
    cc.write_text("double U_static[] = { 1.0, 0}; double Phi_static[] = { 0}; double Psi_cpp_static[] = { 0};"
                  "uint64_t nbr_static[] = { 0}; uint8_t prm_static[] = { 0};")
    with pytest.raises(gb.GbdwError):
        gb.read_static_data(str(h), str(cc))
    with pytest.raises(gb.GbdwError):
        gb.read_static_data(str(h), str(tmp_path / "missing.cc"))
