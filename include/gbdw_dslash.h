/*
 * gbdw_dslash.h -- C++ seam with the shape of GridBench's WilsonKernelsHand.h.
 *
 * A driver written against the reference (bench.cc:148-164, bench_simple.cc:100-106)
 * includes this header instead of WilsonKernelsHand.h and links libgbdw.so: the same
 * dslash_kernel calls then run on the GB300.
 *
 *   template<class Simd> double dslash_kernel(int nrep, Simd* U, Simd* out, Simd* in,
 *                                             uint64_t* nbr, uint64_t nsite, uint64_t Ls,
 *                                             uint8_t* prm);            WilsonKernelsHand.h:17-29
 *   template<class Complex> void dslash_kernel(Complex* U, Complex* Psi, Complex* Phi,
 *                                              uint64_t* nbr, uint64_t nsite, uint64_t Ls,
 *                                              uint8_t* prm);           dslash_simple.h:19-20
 *
 * Simd may be any type with a static Nsimd() (the reference's vComplexD/vComplexF, or
 * gbdw_cxx::vcomplex below) or a plain complex (Nsimd = 1); the real width is taken from
 * sizeof(Simd) / (2 Nsimd).  The reference reports CUDA errors and exits with status 0
 * (Macros.h:47-51); here a failure throws std::runtime_error carrying gbdw_last_error().
 */
#ifndef GBDW_DSLASH_H
#define GBDW_DSLASH_H

#include <stddef.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

#include "gbdw.h"

/* Direction ids of the doubled gauge field and the tables (WilsonKernelsHand.h:5-12). */
#ifndef Xp
#define Xp (0)
#define Yp (1)
#define Zp (2)
#define Tp (3)
#define Xm (4)
#define Ym (5)
#define Zm (6)
#define Tm (7)
#endif

namespace gbdw_cxx {

/* Nsimd complex numbers of real type R, lane-minor, as the reference's vector types. */
template <class R, int N>
struct vcomplex {
  R v[2 * N];
  static constexpr int Nsimd() { return N; }
};

template <class S>
auto nsimd_impl(int) -> decltype(S::Nsimd(), int()) {
  return int(S::Nsimd());
}
template <class S>
int nsimd_impl(long) {
  return 1;
}
template <class S>
int nsimd_of() {
  return nsimd_impl<S>(0);
}

template <class S>
int prec_of() {
  const size_t real_bytes = sizeof(S) / (2 * size_t(nsimd_of<S>()));
  if (real_bytes == 8) return GBDW_F64;
  if (real_bytes == 4) return GBDW_F32;
  throw std::runtime_error("dslash_kernel: element type is neither double nor float complex");
}

inline void check(int status, const char* what) {
  if (status != GBDW_OK) throw std::runtime_error(std::string(what) + ": " + gbdw_last_error());
}

}  // namespace gbdw_cxx

template <class Simd>
double dslash_kernel(int nrep, Simd* Up, Simd* outp, Simd* inp, uint64_t* nbr, uint64_t nsite, uint64_t Ls,
                     uint8_t* prm) {
  double usec = 0.0;
  gbdw_cxx::check(gbdw_dslash_kernel(nrep, gbdw_cxx::prec_of<Simd>(), gbdw_cxx::nsimd_of<Simd>(), Up, outp, inp, nbr,
                                     nsite, Ls, prm, 0, &usec),
                  "dslash_kernel");
  return usec;
}

template <class Complex>
void dslash_kernel(Complex* U, Complex* Psi, Complex* Phi, uint64_t* nbr, uint64_t nsite, uint64_t Ls, uint8_t* prm) {
  (void)dslash_kernel<Complex>(1, U, Psi, Phi, nbr, nsite, Ls, prm);
}

#endif /* GBDW_DSLASH_H */
