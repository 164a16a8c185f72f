// Double-word ("double-single") arithmetic on pairs of FP32 numbers: a value is h + l with
// |l| <= ulp(h) / 2, about 48 significant bits (relative rounding ~2^-47), computed on the FP32
// pipe.  GB300 executes FP64 at 1/64 of its FP32 rate, so the FP64-accurate hopping operator
// (the solvers' true residuals and the FP64 CG) runs its arithmetic in this form instead of in
// FP64: FP64 fields are split into pairs as they are loaded and joined back to FP64 as they are
// stored.
//
// The building blocks are the published error-free transformations and double-word
// algorithms:
//   two_sum       Knuth, TAOCP vol. 2, sec. 4.2.2 (Moller 1965): s + e = a + b exactly;
//   fast_two_sum  Dekker 1971: the same for |a| >= |b| in three operations;
//   two_prod      p + e = a * b exactly with one FMA;
//   add / mul     Joldes, Muller, Popescu, "Tight and rigorous error bounds for basic
//                 building blocks of double-word arithmetic", ACM TOMS 44 (2017):
//                 SloppyDWPlusDW (Alg. 5; error <= 2^-47 (|a| + |b|), the bound of a sum
//                 of terms that FP64 accumulation of the same terms also has) and
//                 DWTimesDW (Alg. 12 without its l*l term; relative error below 2^-45).
// The split of an FP64 value uses integer operations only (no FP64 instruction): h takes the
// sign, exponent and leading 24 mantissa bits, l the remaining 29 bits rounded to 24, then the
// pair is renormalised.  Magnitudes below 2^-126 are flushed to zero and l is dropped below
// 2^-74 (relative precision 2^-24 there), and products below about 2^-100 lose trailing bits to
// FP32 subnormals; the operator's links and spinors stay far inside that range.
#pragma once
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#include <cmath>
#define GBDW_HD inline
#else
#define GBDW_HD __host__ __device__ __forceinline__
#endif

namespace gbdw {

struct dsf {
  float h, l;
  dsf() = default;
  GBDW_HD constexpr dsf(float a, float b) : h(a), l(b) {}
  // from an FP64 value (see ds_split) or an integer / exact constant
  GBDW_HD explicit dsf(double d);
  GBDW_HD explicit dsf(int v) : dsf(double(v)) {}
  // to FP64: exact sum of the pair rounded once
  GBDW_HD explicit operator double() const { return double(h) + double(l); }
  GBDW_HD explicit operator float() const { return h + l; }
};

namespace ds_detail {
GBDW_HD uint64_t bits(double d) {
#ifdef __CUDA_ARCH__
  return uint64_t(__double_as_longlong(d));
#else
  uint64_t b;
  std::memcpy(&b, &d, 8);
  return b;
#endif
}
GBDW_HD float from_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(b);
#else
  float f;
  std::memcpy(&f, &b, 4);
  return f;
#endif
}
GBDW_HD uint32_t fbits(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(f);
#else
  uint32_t b;
  std::memcpy(&b, &f, 4);
  return b;
#endif
}
GBDW_HD float fma_(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fma(a, b, c);
#endif
}
GBDW_HD float mul_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
GBDW_HD float add_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
GBDW_HD float sub_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
}  // namespace ds_detail

// s + e = a + b exactly (Knuth)
GBDW_HD dsf ds_two_sum(float a, float b) {
  using namespace ds_detail;
  const float s = add_(a, b);
  const float bb = sub_(s, a);
  const float e = add_(sub_(a, sub_(s, bb)), sub_(b, bb));
  return {s, e};
}
// s + e = a + b exactly when |a| >= |b| or a == 0 (Dekker)
GBDW_HD dsf ds_fast_two_sum(float a, float b) {
  using namespace ds_detail;
  const float s = add_(a, b);
  return {s, sub_(b, sub_(s, a))};
}

// The split of an FP64 value into a normalised pair, with integer operations only.
GBDW_HD dsf ds_split(double d) {
  using namespace ds_detail;
  const uint64_t b = bits(d);
  const uint32_t hi = uint32_t(b >> 32), lo = uint32_t(b);
  const uint32_t sgn = hi & 0x80000000u;
  const int e = int((hi >> 20) & 0x7ffu);  // biased FP64 exponent
  const int ef = e - 896;                   // the same exponent biased for FP32 (1023 - 127)
  if (ef <= 0) return {from_bits(sgn), 0.f};                 // zero, subnormal or below 2^-126
  if (ef >= 255) return {from_bits(sgn | 0x7f800000u), 0.f};  // beyond FP32 range, inf, nan
  const float h = from_bits(sgn | (uint32_t(ef) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
  // remaining 29 mantissa bits, worth rem * 2^(e - 1075)
  const uint32_t rem = lo & 0x1fffffffu;
  const int pe = e - 948;  // FP32-biased exponent of 2^(e - 1075)
  float l = 0.f;
  if (pe > 0 && rem != 0) {
    l = mul_(float(rem), from_bits(uint32_t(pe) << 23));
    l = from_bits(fbits(l) | sgn);
  }
  return ds_fast_two_sum(h, l);
}

GBDW_HD dsf::dsf(double d) : dsf(ds_split(d)) {}

// SloppyDWPlusDW
GBDW_HD dsf operator+(dsf a, dsf b) {
  using namespace ds_detail;
  const dsf s = ds_two_sum(a.h, b.h);
  return ds_fast_two_sum(s.h, add_(s.l, add_(a.l, b.l)));
}
GBDW_HD dsf operator-(dsf a) { return {-a.h, -a.l}; }
GBDW_HD dsf operator-(dsf a, dsf b) { return a + (-b); }
GBDW_HD dsf& operator+=(dsf& a, dsf b) { return a = a + b; }
GBDW_HD dsf& operator-=(dsf& a, dsf b) { return a = a - b; }
// DWTimesDW without the l*l term
GBDW_HD dsf operator*(dsf a, dsf b) {
  using namespace ds_detail;
  const float p = mul_(a.h, b.h);
  float e = fma_(a.h, b.h, -p);
  e = fma_(a.h, b.l, e);
  e = fma_(a.l, b.h, e);
  return ds_fast_two_sum(p, e);
}
// a * b + c with one renormalisation: the exact product's leading part is summed with c by
// two_sum, its trailing part and c's joined in FP32
GBDW_HD dsf fma(dsf a, dsf b, dsf c) {
  using namespace ds_detail;
  const float p = mul_(a.h, b.h);
  float pe = fma_(a.h, b.h, -p);
  pe = fma_(a.h, b.l, pe);
  pe = fma_(a.l, b.h, pe);
  const dsf s = ds_two_sum(p, c.h);
  return ds_fast_two_sum(s.h, add_(s.l, add_(pe, c.l)));
}

}  // namespace gbdw
