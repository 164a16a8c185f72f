// The bench_simple.cc driver flow (bench_simple.cc:69-149) on the GB300: the scalar
// dslash_kernel<ComplexD>(U, Psi, Phi, nbr, nsite, Ls, prm) is called nrep times, timed, and
// checked against a reference result with sum (Psi_cpp - Psi)^2 <= 1e-10.
//
//   bench_simple_gb300 [--dims Lx Ly Lz Lt] [--Ls n] [--nrep n] --ref file
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <cmath>
#include <iostream>
#include <vector>

#include "gbdw_dslash.h"

struct ComplexD {
  double re, im;
};

int main(int argc, char** argv) {
  int dims[4] = {8, 8, 8, 8};
  int Ls = 8, nrep = 300;
  const char* ref_path = nullptr;
  for (int i = 1; i < argc; ++i) {
    if (!strcmp(argv[i], "--dims") && i + 4 < argc) {
      for (int d = 0; d < 4; ++d) dims[d] = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "--Ls") && i + 1 < argc) {
      Ls = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "--nrep") && i + 1 < argc) {
      nrep = atoi(argv[++i]);
    } else if (!strcmp(argv[i], "--ref") && i + 1 < argc) {
      ref_path = argv[++i];
    } else {
      fprintf(stderr, "unknown argument %s\n", argv[i]);
      return 2;
    }
  }
  const uint64_t nsite = uint64_t(dims[0]) * dims[1] * dims[2] * dims[3];
  const uint64_t umax = nsite * 18 * 8, fmax = nsite * 24 * Ls, vol = nsite * Ls;
  std::vector<double> U(umax), Psi(fmax, 0.0), Phi(fmax), Psi_cpp(fmax);
  std::vector<uint64_t> nbr(nsite * Ls * 8);
  std::vector<uint8_t> prm(nsite * Ls * 8);
  const int gseeds[4] = {1, 2, 3, 4}, fseeds[4] = {5, 6, 7, 8};
  gbdw_cxx::check(gbdw_generate_gauge(dims, 1, gbdw_seed_from_ints(gseeds, 4), U.data()), "generate gauge");
  gbdw_cxx::check(gbdw_generate_fermion(dims, Ls, 1, gbdw_seed_from_ints(fseeds, 4), Phi.data()), "generate fermion");
  gbdw_cxx::check(gbdw_generate_table(dims, Ls, 1, nbr.data(), prm.data()), "generate table");
  if (!ref_path) {
    fprintf(stderr, "--ref file is required (reference result, raw doubles)\n");
    return 2;
  }
  FILE* f = fopen(ref_path, "rb");
  if (!f || fread(Psi_cpp.data(), sizeof(double), fmax, f) != fmax) {
    fprintf(stderr, "cannot read %s\n", ref_path);
    return 1;
  }
  fclose(f);

  std::cout << std::endl << "Calling dslash_kernel " << std::endl;
  const double flops = 1320.0 * double(vol);
  const auto start = std::chrono::steady_clock::now();
  try {
    for (int i = 0; i < nrep; ++i)
      dslash_kernel<ComplexD>((ComplexD*)U.data(), (ComplexD*)Psi.data(), (ComplexD*)Phi.data(), nbr.data(), nsite, Ls,
                              prm.data());
  } catch (const std::exception& e) {
    fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  const double usec =
      std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - start).count();
  std::cout << std::endl
            << "\t" << nrep * flops / usec / 1000. << " Gflop/s in double precision; kernel call " << usec / nrep
            << " microseconds (host buffers: upload, run and download per call)" << std::endl
            << std::endl;
  double err = 0;
  for (uint64_t i = 0; i < fmax; ++i) err += std::pow(Psi_cpp[i] - Psi[i], 2);
  std::cout << "normdiff " << err << std::endl;
  if (!(err <= 1.0e-10)) {
    std::cout << "FAILED: normdiff above 1e-10" << std::endl;
    return 1;
  }
  return 0;
}
