// ORACLE support (test infrastructure only): builds GridBench's own scalar hopping term,
// dslash_simple.h, from the reference tree where it lies, and exposes it with C linkage.
// The complex type below provides exactly the operations dslash_simple.h uses (the role
// bench_simple.cc:20-64 gives its myComplex); it is written here, not taken from there.
#include <stdint.h>

#define RESTRICT

template <class R>
struct RefComplex {
  R re, im;
  RefComplex() {}
  template <class F>
  RefComplex(F a, F b) : re(R(a)), im(R(b)) {}
  RefComplex operator-() const { return RefComplex(-re, -im); }
  RefComplex& operator+=(const RefComplex& o) {
    re += o.re;
    im += o.im;
    return *this;
  }
  RefComplex& operator-=(const RefComplex& o) {
    re -= o.re;
    im -= o.im;
    return *this;
  }
};
template <class R>
RefComplex<R> operator*(const RefComplex<R>& a, const RefComplex<R>& b) {
  return RefComplex<R>(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <class R>
RefComplex<R> operator+(const RefComplex<R>& a, const RefComplex<R>& b) {
  return RefComplex<R>(a.re + b.re, a.im + b.im);
}
template <class R>
RefComplex<R> operator-(const RefComplex<R>& a, const RefComplex<R>& b) {
  return RefComplex<R>(a.re - b.re, a.im - b.im);
}

#include "dslash_simple.h"

typedef RefComplex<double> CD;

extern "C" void ref_dslash_kernel(double* U, double* Psi, double* Phi, uint64_t* nbr, uint64_t nsite, uint64_t Ls,
                                  uint8_t* prm) {
  dslash_kernel<CD>((CD*)U, (CD*)Psi, (CD*)Phi, nbr, nsite, Ls, prm);
}

extern "C" void ref_dslash_kernel_unroll(double* U, double* Psi, double* Phi, uint64_t* nbr, uint64_t nsite,
                                         uint64_t Ls, uint8_t* prm) {
  dslash_kernel_unroll<CD>((CD*)U, (CD*)Psi, (CD*)Phi, nbr, nsite, Ls, prm);
}
