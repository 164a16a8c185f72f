// ORACLE support (test infrastructure only): builds GridBench's hand-unrolled CPU kernel
// (WilsonKernelsHandCpu.h through the WilsonKernelsHand.h seam) for AVX-512 from the
// reference tree where it lies.  Its vComplexD has 4 lanes and vComplexF 8, so running it on
// the generator's lane layouts checks the lane / permute convention against the reference.
#include <stdint.h>
#include <stdio.h>

#include <cassert>
#include <chrono>
#include <iostream>
#include <vector>

#include "Simd.h"
#include "WilsonKernelsHand.h"

extern "C" int ref_hand_nsimd_d(void) { return vComplexD::Nsimd(); }
extern "C" int ref_hand_nsimd_f(void) { return vComplexF::Nsimd(); }

extern "C" double ref_hand_dslash_d(int nrep, double* U, double* out, double* in, uint64_t* nbr, uint64_t nsite,
                                    uint64_t Ls, uint8_t* prm) {
  return dslash_kernel<vComplexD>(nrep, (vComplexD*)U, (vComplexD*)out, (vComplexD*)in, nbr, nsite, Ls, prm);
}

extern "C" double ref_hand_dslash_f(int nrep, float* U, float* out, float* in, uint64_t* nbr, uint64_t nsite,
                                    uint64_t Ls, uint8_t* prm) {
  return dslash_kernel<vComplexF>(nrep, (vComplexF*)U, (vComplexF*)out, (vComplexF*)in, nbr, nsite, Ls, prm);
}
