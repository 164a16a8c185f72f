"""Writes the golden vectors under tests/golden/ from GridBench's OWN kernels.

GridBench's golden arrays (static_data.cc, made by Grid through TableGenerate.cc) are not in
the reference tree (.MISSING_LARGE_BLOBS), so the inputs come from this project's seeded
generator and the outputs from the reference code compiled where it lies (oracle/build.py):
  - dslash_simple.h  (scalar, Nsimd = 1, FP64)          -> golden_simple_*.npz
  - WilsonKernelsHandCpu.h on AVX-512 (Nsimd = 4 FP64,  -> golden_hand_*.npz
    Nsimd = 8 FP32, with lane permutes)
Each file stores the reference output and SHA-256 digests of the generated inputs, so a test
can also check that the generator reproduces the same bits.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import gridbench_gb300 as gb  # noqa: E402
import oracle  # noqa: E402

CASES_SIMPLE = [((2, 2, 2, 2), 4), ((4, 4, 4, 4), 4), ((4, 2, 6, 2), 3)]
CASES_HAND = [((4, 4, 4, 4), 4, 4, np.float64), ((4, 4, 4, 4), 2, 8, np.float32)]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("the reference tree is not available here; golden vectors need it")
    for dims, Ls in CASES_SIMPLE:
        U = gb.generate_gauge(dims)
        phi = gb.generate_fermion(dims, Ls)
        nbr, prm, nsite = gb.generate_table(dims, Ls)
        psi = np.zeros_like(phi)
        ref.ref_dslash_kernel(U, psi, phi, nbr, nsite, Ls, prm)
        name = "golden_simple_%s_Ls%d.npz" % ("x".join(map(str, dims)), Ls)
        np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), Ls=Ls, nsimd=1, psi=psi,
                            sha_U=digest(U), sha_phi=digest(phi), sha_nbr=digest(nbr), sha_prm=digest(prm))
        print("wrote", name)
    hand = oracle.hand()
    if hand is None:
        print("AVX-512 reference kernel not available here; skipping lane-layout goldens")
        return
    for dims, Ls, ns, dt in CASES_HAND:
        U = oracle.aligned_copy(gb.generate_gauge(dims, ns).astype(dt))
        phi = oracle.aligned_copy(gb.generate_fermion(dims, Ls, ns).astype(dt))
        nbr, prm, nsite = gb.generate_table(dims, Ls, ns)
        out = oracle.aligned_copy(np.zeros_like(phi))
        fn = hand.ref_hand_dslash_d if dt == np.float64 else hand.ref_hand_dslash_f
        assert (hand.ref_hand_nsimd_d() if dt == np.float64 else hand.ref_hand_nsimd_f()) == ns
        fn(2, U, out, phi, nbr, nsite, Ls, prm)
        name = "golden_hand_n%d_%s_%s_Ls%d.npz" % (ns, "f64" if dt == np.float64 else "f32",
                                                   "x".join(map(str, dims)), Ls)
        np.savez_compressed(os.path.join(HERE, name), dims=np.array(dims), Ls=Ls, nsimd=ns, psi=np.array(out),
                            sha_nbr=digest(nbr), sha_prm=digest(prm))
        print("wrote", name)


if __name__ == "__main__":
    main()
