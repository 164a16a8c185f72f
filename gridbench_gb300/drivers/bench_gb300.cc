// The bench.cc driver flow (bench.cc:59-202) on the GB300: build the inputs (here from the
// seeded generator, standing in for the missing static_data.cc), lay them out with Nsimd
// lanes, call dslash_kernel<vComplex>(nrep, ...), report Gflop/s and compare with a
// reference result if one is given.
//
//   bench_gb300 [--dims Lx Ly Lz Lt] [--Ls n] [--nsimd n] [--float] [--nrep n]
//               [--ref file] [--out file]
// --ref reads the reference result as raw doubles in the same layout; --out writes ours.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <iostream>
#include <vector>

#include "gbdw_dslash.h"

int main(int argc, char** argv) {
  int dims[4] = {8, 8, 8, 8};
  int Ls = 8, nsimd = 1, nrep = 1000;
  bool single = false;
  const char* ref_path = nullptr;
  const char* out_path = nullptr;
  for (int i = 1; i < argc; ++i) {
    if (!strcmp(argv[i], "--dims") && i + 4 < argc) {
      for (int d = 0; d < 4; ++d) dims[d] = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "--Ls") && i + 1 < argc) {
      Ls = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "--nsimd") && i + 1 < argc) {
      nsimd = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "--nrep") && i + 1 < argc) {
      nrep = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "--float")) {
      single = true;
    } else if (!strcmp(argv[i], "--ref") && i + 1 < argc) {
      ref_path = argv[++i];
    } else if (!strcmp(argv[i], "--out") && i + 1 < argc) {
      out_path = argv[++i];
    } else {
      fprintf(stderr, "unknown argument %s\n", argv[i]);
      return 2;
    }
  }
  const uint64_t V = uint64_t(dims[0]) * dims[1] * dims[2] * dims[3];
  const uint64_t nsite = V / uint64_t(nsimd);
  const uint64_t umax = nsite * 18 * 8 * nsimd;
  const uint64_t fmax = nsite * 24 * Ls * nsimd;
  const uint64_t vol = nsite * Ls * nsimd;
  printf("Nsimd %d\n", nsimd);

  std::vector<double> U(umax), Phi(fmax), Psi(fmax, 0.0);
  std::vector<uint64_t> nbr(nsite * Ls * 8);
  std::vector<uint8_t> prm(nsite * Ls * 8);
  const int gseeds[4] = {1, 2, 3, 4}, fseeds[4] = {5, 6, 7, 8};
  gbdw_cxx::check(gbdw_generate_gauge(dims, nsimd, gbdw_seed_from_ints(gseeds, 4), U.data()), "generate gauge");
  gbdw_cxx::check(gbdw_generate_fermion(dims, Ls, nsimd, gbdw_seed_from_ints(fseeds, 4), Phi.data()), "generate fermion");
  gbdw_cxx::check(gbdw_generate_table(dims, Ls, nsimd, nbr.data(), prm.data()), "generate table");

  std::cout << std::endl << "Calling dslash_kernel " << std::endl;
  const double flops = 1320.0 * double(vol);
  double usec = 0.0;
  try {
    if (!single) {
#define GBDW_RUN_D(N)                                                                                   \
  case N: {                                                                                             \
    typedef gbdw_cxx::vcomplex<double, N> vComplexD;                                                    \
    usec = dslash_kernel<vComplexD>(nrep, (vComplexD*)U.data(), (vComplexD*)Psi.data(), (vComplexD*)Phi.data(), \
                                    nbr.data(), nsite, Ls, prm.data());                                 \
  } break;
      switch (nsimd) {
        GBDW_RUN_D(1) GBDW_RUN_D(2) GBDW_RUN_D(4) GBDW_RUN_D(8) GBDW_RUN_D(16)
        default: fprintf(stderr, "nsimd must be 1,2,4,8,16\n"); return 2;
      }
    } else {
      std::vector<float> fU(U.begin(), U.end()), fPhi(Phi.begin(), Phi.end()), fPsi(fmax, 0.f);
#define GBDW_RUN_F(N)                                                                                    \
  case N: {                                                                                              \
    typedef gbdw_cxx::vcomplex<float, N> vComplexF;                                                      \
    usec = dslash_kernel<vComplexF>(nrep, (vComplexF*)fU.data(), (vComplexF*)fPsi.data(), (vComplexF*)fPhi.data(), \
                                    nbr.data(), nsite, Ls, prm.data());                                  \
  } break;
      switch (nsimd) {
        GBDW_RUN_F(1) GBDW_RUN_F(2) GBDW_RUN_F(4) GBDW_RUN_F(8) GBDW_RUN_F(16)
        default: fprintf(stderr, "nsimd must be 1,2,4,8,16\n"); return 2;
      }
      for (uint64_t i = 0; i < fmax; ++i) Psi[i] = fPsi[i];  // copy back to double (bench.cc:166-169)
    }
  } catch (const std::exception& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  const int timed = nrep > 1 ? nrep - 1 : 1;
  std::cout << std::endl
            << "\t" << timed * flops / usec / 1000. << " Gflop/s in " << (single ? "single" : "double")
            << " precision; kernel call " << usec / timed << " microseconds " << std::endl
            << std::endl;
  if (out_path) {
    FILE* f = fopen(out_path, "wb");
    if (!f || fwrite(Psi.data(), sizeof(double), fmax, f) != fmax) {
      fprintf(stderr, "cannot write %s\n", out_path);
      return 1;
    }
    fclose(f);
  }
  if (ref_path) {
    std::vector<double> Psi_cpp(fmax);
    FILE* f = fopen(ref_path, "rb");
    if (!f || fread(Psi_cpp.data(), sizeof(double), fmax, f) != fmax) {
      fprintf(stderr, "cannot read %s\n", ref_path);
      return 1;
    }
    fclose(f);
    double err = 0, nref = 0, nres = 0;
    for (uint64_t i = 0; i < fmax; ++i) {
      err += (Psi_cpp[i] - Psi[i]) * (Psi_cpp[i] - Psi[i]);
      nres += Psi[i] * Psi[i];
      nref += Psi_cpp[i] * Psi_cpp[i];
    }
    std::cout << "normdiff " << err << " ref " << nref << " result " << nres << std::endl;
    for (int ii = 0; ii < 8; ++ii) std::cout << ii << " ref " << Psi_cpp[ii] << " result " << Psi[ii] << std::endl;
    std::cout << "reldiff " << std::sqrt(err / nref) << std::endl;
  }
  return 0;
}
