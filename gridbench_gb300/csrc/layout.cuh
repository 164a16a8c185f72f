// Spinor storage of the GB300 layout and its element access.
//
// A row is one spin-colour component of one 4D site: row = site*12 + sc, holding the
// LsE = Ls*nrhs fifth-dimension slices (rhs innermost).
//   F64     : double2 per slice; slice e at double2 index row*LsP + e (LsP = LsE).
//   F32/F16 : slices grouped in pairs, each pair stored as (Re s, Re s+1, Im s, Im s+1);
//             rows padded to an even slice count LsP.  Re of slice e sits at real index
//             row*2*LsP + 4*(e>>1) + (e&1) and Im two reals further.
// A 128-bit (F32) or 64-bit (F16) load of a slice pair therefore lands {Re, Re} and {Im, Im}
// in adjacent registers, which is the operand form of Blackwell's packed FFMA2 / FADD2 /
// FMUL2: two slices run through one instruction.  F16 values are stored divided by a
// per-slice FP32 norm held in norm[site*LsE + e].
#pragma once
#include "common.cuh"
#include "dsfloat.cuh"

namespace gbdw {

// Internal precision tag of the double-single operator: FP64 storage (the F64 layout), arithmetic
// on FP32 pairs (dsfloat.cuh), links from the gauge field's split copy.
constexpr int GBDW_DS = 7;

__host__ __device__ inline int padded_slices(int prec, int LsE) {
  return prec == GBDW_F64 ? LsE : LsE + (LsE & 1);
}
__host__ __device__ inline int64_t re_index(int64_t row, int e, int LsP) {
  return row * 2 * int64_t(LsP) + 4 * (e >> 1) + (e & 1);
}

// One complex component for two adjacent slices.
struct cp2 {
  float2 r, i;
};

template <bool SMEM, class V>
__device__ __forceinline__ V ldv(const V* p) {
  if constexpr (SMEM) return *p;
  else return __ldg(p);
}

__device__ __forceinline__ float2 h2f(unsigned w) {
  __half2 h = *reinterpret_cast<__half2*>(&w);
  return __half22float2(h);
}
__device__ __forceinline__ unsigned f2h(float a, float b) {
  __half2 h = __floats2half2_rn(a, b);
  return *reinterpret_cast<unsigned*>(&h);
}

// ------------------------------------------------------------------ single slices
template <int P>
struct Elem;
template <>
struct Elem<GBDW_F64> {
  template <bool SMEM = false>
  __device__ static cpx<double> ld(const void* b, int64_t row, int e, int LsP) {
    const double2 a = ldv<SMEM>((const double2*)b + row * LsP + e);
    return {a.x, a.y};
  }
  __device__ static void st(void* b, int64_t row, int e, int LsP, double re, double im) {
    ((double2*)b)[row * LsP + e] = make_double2(re, im);
  }
};
template <>
struct Elem<GBDW_F32> {
  template <bool SMEM = false>
  __device__ static cpx<float> ld(const void* b, int64_t row, int e, int LsP) {
    const float* f = (const float*)b + re_index(row, e, LsP);
    return {ldv<SMEM>(f), ldv<SMEM>(f + 2)};
  }
  __device__ static void st(void* b, int64_t row, int e, int LsP, float re, float im) {
    float* f = (float*)b + re_index(row, e, LsP);
    f[0] = re;
    f[2] = im;
  }
};
// DS: FP64 storage, split into pairs on load and joined on store.
template <>
struct Elem<GBDW_DS> {
  template <bool SMEM = false>
  __device__ static cpx<dsf> ld(const void* b, int64_t row, int e, int LsP) {
    const double2 a = ldv<SMEM>((const double2*)b + row * LsP + e);
    return {ds_split(a.x), ds_split(a.y)};
  }
  __device__ static void st(void* b, int64_t row, int e, int LsP, dsf re, dsf im) {
    ((double2*)b)[row * LsP + e] = make_double2(double(re), double(im));
  }
};
// F16: returns / takes the stored (norm-scaled) values.
template <>
struct Elem<GBDW_F16> {
  template <bool SMEM = false>
  __device__ static cpx<float> ld(const void* b, int64_t row, int e, int LsP) {
    const unsigned short* h = (const unsigned short*)b + re_index(row, e, LsP);
    const unsigned short a = ldv<SMEM>(h), c = ldv<SMEM>(h + 2);
    return {__half2float(__ushort_as_half(a)), __half2float(__ushort_as_half(c))};
  }
  __device__ static void st(void* b, int64_t row, int e, int LsP, float re, float im) {
    unsigned short* h = (unsigned short*)b + re_index(row, e, LsP);
    h[0] = __half_as_ushort(__float2half_rn(re));
    h[2] = __half_as_ushort(__float2half_rn(im));
  }
};

// ------------------------------------------------------------------ N consecutive slices
// e0 % N == 0; for N >= 2 the slices come in whole pairs (e0 even).
template <int P, int N, bool SMEM = false>
struct Vec {
  using T = typename std::conditional<P == GBDW_F64, double, typename std::conditional<P == GBDW_DS, dsf, float>::type>::type;

  __device__ static void load(const void* b, int64_t row, int e0, int LsP, cpx<T> (&v)[N]) {
    if constexpr (P == GBDW_F64 || P == GBDW_DS || N == 1) {
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = Elem<P>::template ld<SMEM>(b, row, e0 + j, LsP);
    } else {
      cp2 q[N / 2];
      load_pairs(b, row, e0, LsP, q);
#pragma unroll
      for (int k = 0; k < N / 2; ++k) {
        v[2 * k] = {q[k].r.x, q[k].i.x};
        v[2 * k + 1] = {q[k].r.y, q[k].i.y};
      }
    }
  }
  // F32/F16, N even: the pairs themselves
  __device__ static void load_pairs(const void* b, int64_t row, int e0, int LsP, cp2 (&q)[N / 2]) {
    if constexpr (P == GBDW_F32) {
      const float4* f = reinterpret_cast<const float4*>((const float*)b + row * 2 * int64_t(LsP) + 2 * e0);
#pragma unroll
      for (int k = 0; k < N / 2; ++k) {
        const float4 a = ldv<SMEM>(f + k);
        q[k] = {make_float2(a.x, a.y), make_float2(a.z, a.w)};
      }
    } else if constexpr (P == GBDW_F16) {
      const uint2* h = reinterpret_cast<const uint2*>((const unsigned short*)b + row * 2 * int64_t(LsP) + 2 * e0);
#pragma unroll
      for (int k = 0; k < N / 2; ++k) {
        const uint2 a = ldv<SMEM>(h + k);
        q[k] = {h2f(a.x), h2f(a.y)};
      }
    }
  }
  // F16, N even: the stored half2 pairs {Re,Re}, {Im,Im} without conversion
  __device__ static void load_pairs_raw(const void* b, int64_t row, int e0, int LsP, uint2 (&q)[N / 2]) {
    const uint2* h = reinterpret_cast<const uint2*>((const unsigned short*)b + row * 2 * int64_t(LsP) + 2 * e0);
#pragma unroll
    for (int k = 0; k < N / 2; ++k) q[k] = ldv<SMEM>(h + k);
  }
  // F64 / F32 stores
  __device__ static void store(void* b, int64_t row, int e0, int LsP, const cpx<T> (&v)[N]) {
    if constexpr (P == GBDW_F64 || P == GBDW_DS || N == 1) {
#pragma unroll
      for (int j = 0; j < N; ++j) Elem<P>::st(b, row, e0 + j, LsP, v[j].r, v[j].i);
    } else {
      float4* f = reinterpret_cast<float4*>((float*)b + row * 2 * int64_t(LsP) + 2 * e0);
#pragma unroll
      for (int k = 0; k < N / 2; ++k) f[k] = make_float4(v[2 * k].r, v[2 * k + 1].r, v[2 * k].i, v[2 * k + 1].i);
    }
  }
  // F16 store of already-scaled values
  __device__ static void store_scaled(void* b, int64_t row, int e0, int LsP, const cpx<float> (&v)[N]) {
    if constexpr (N == 1) {
      Elem<GBDW_F16>::st(b, row, e0, LsP, v[0].r, v[0].i);
    } else {
      uint2* h = reinterpret_cast<uint2*>((unsigned short*)b + row * 2 * int64_t(LsP) + 2 * e0);
#pragma unroll
      for (int k = 0; k < N / 2; ++k)
        h[k] = make_uint2(f2h(v[2 * k].r, v[2 * k + 1].r), f2h(v[2 * k].i, v[2 * k + 1].i));
    }
  }
};

}  // namespace gbdw
