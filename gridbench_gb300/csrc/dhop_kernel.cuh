// The domain-wall Wilson hopping kernel (Dhop / DhopDag, optionally fused into the Shamir
// operator M) for the GB300 layout of layout.cuh.
//
// Maths per 5D site (WilsonKernelsHandCpu.h:94-303, applied per leg at :435-442, scalar form
// dslash_simple.h:39-145): for each of the 8 legs, project the neighbour spinor to two
// half-spinor colour vectors h0 = psi0 + c0 psi_a, h1 = psi1 + c1 psi_b, multiply both by the
// doubled link U[site][leg], and accumulate r0 += u0, r1 += u1, r_a += conj(c0) u0,
// r_b += conj(c1) u1.  (a, b) = (3, 2) for X/Y legs and (2, 3) for Z/T legs; the unit
// coefficients per leg are
//     Xp: -i,-i   Yp: +1,-1   Zp: -i,+i   Tp: -1,-1   and the m-legs have the opposite signs.
// DhopDag = gamma5 Dhop gamma5 swaps every leg's spin structure with its opposite-sign
// partner while keeping the leg's neighbour and link.
//
// Work decomposition: one thread per (4D site, N consecutive slices).  The 4D neighbour and
// the link of a leg are loaded once per thread and reused over its N slices; threads of one
// site read the same link (one broadcast transaction) and consecutive threads read
// consecutive slices, so each spinor component load of a warp is a run of whole sectors.
// FP32/FP16 with an even N run the arithmetic on slice pairs with packed FFMA2/FADD2/FMUL2.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "layout.cuh"

namespace gbdw {

template <int P>
struct Arith {
  using T = float;
};
template <>
struct Arith<GBDW_F64> {
  using T = double;
};
template <>
struct Arith<GBDW_DS> {
  using T = dsf;
};

template <int N>
__device__ __forceinline__ void load_norms(const float* nrm, int64_t e, float (&v)[N]) {
  if constexpr (N == 1) {
    v[0] = __ldg(nrm + e);
  } else if constexpr (N == 2) {
    const float2 a = __ldg((const float2*)nrm + (e >> 1));
    v[0] = a.x;
    v[1] = a.y;
  } else {
#pragma unroll
    for (int k = 0; k < N / 4; ++k) {
      const float4 a = __ldg((const float4*)nrm + (e >> 2) + k);
      v[4 * k] = a.x;
      v[4 * k + 1] = a.y;
      v[4 * k + 2] = a.z;
      v[4 * k + 3] = a.w;
    }
  }
}
template <int N>
__device__ __forceinline__ void store_norms(float* nrm, int64_t e, const float (&v)[N]) {
  if constexpr (N == 1) {
    nrm[e] = v[0];
  } else if constexpr (N == 2) {
    ((float2*)nrm)[e >> 1] = make_float2(v[0], v[1]);
  } else {
#pragma unroll
    for (int k = 0; k < N / 4; ++k) ((float4*)nrm)[(e >> 2) + k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  }
}

// ------------------------------------------------------------------ links
// Full 3x3 (F64/F32) or two rows with the third rebuilt as conj(r0 x r1) (exact for SU(3)).
__device__ __forceinline__ cpx<float> h2c(unsigned w) {
  const float2 f = h2f(w);
  return {f.x, f.y};
}
__device__ __forceinline__ cpx<float> b2c(unsigned w) {
  __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&w);
  const float2 f = __bfloat1622float2(h);
  return {f.x, f.y};
}
// conj(a b - c d) with each complex product as two packed FMAs on (re, im):
// a b = a.r (b.r, b.i) + a.i (-b.i, b.r).
__device__ __forceinline__ cpx<float> cross_conj(cpx<float> a, cpx<float> b, cpx<float> c, cpx<float> d) {
  float2 t = __fmul2_rn(make_float2(a.r, a.r), make_float2(b.r, b.i));
  t = __ffma2_rn(make_float2(a.i, a.i), make_float2(-b.i, b.r), t);
  t = __ffma2_rn(make_float2(-c.r, -c.r), make_float2(d.r, d.i), t);
  t = __ffma2_rn(make_float2(-c.i, -c.i), make_float2(-d.i, d.r), t);
  return {t.x, -t.y};
}
__device__ __forceinline__ void third_row(cpx<float> (&u)[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    u[2][c] = cross_conj(u[0][c1], u[1][c2], u[0][c2], u[1][c1]);
  }
}

template <int GP>
struct LinkIO;
template <>
struct LinkIO<GBDW_F32> {
  static constexpr unsigned bytes = 72;
  template <bool SMEM = false>
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<float> (&u)[3][3]) {
    const float2* p = (const float2*)U + link * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float2 a = ldv<SMEM>(p + k);
      u[k / 3][k % 3] = {a.x, a.y};
    }
  }
};
template <>
struct LinkIO<GBDW_F64> {
  static constexpr unsigned bytes = 144;
  template <bool SMEM = false>
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<double> (&u)[3][3]) {
    const double2* p = (const double2*)U + link * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double2 a = ldv<SMEM>(p + k);
      u[k / 3][k % 3] = {a.x, a.y};
    }
  }
};
// the F64 gauge field's split copy: one float4 (re h, re l, im h, im l) per entry
template <>
struct LinkIO<GBDW_DS> {
  static constexpr unsigned bytes = 144;
  template <bool SMEM = false>
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<dsf> (&u)[3][3]) {
    const float4* p = (const float4*)U + link * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float4 a = ldv<SMEM>(p + k);
      u[k / 3][k % 3] = {dsf(a.x, a.y), dsf(a.z, a.w)};
    }
  }
};
template <>
struct LinkIO<GBDW_F16> {
  static constexpr unsigned bytes = 24;
  template <bool SMEM = false>
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<float> (&u)[3][3]) {
    const uint2* p = (const uint2*)U + link * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint2 a = ldv<SMEM>(p + k);
      u[(2 * k) / 3][(2 * k) % 3] = h2c(a.x);
      u[(2 * k + 1) / 3][(2 * k + 1) % 3] = h2c(a.y);
    }
    third_row(u);
  }
};
template <>
struct LinkIO<GBDW_BF16> {
  static constexpr unsigned bytes = 24;
  template <bool SMEM = false>
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<float> (&u)[3][3]) {
    const uint2* p = (const uint2*)U + link * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint2 a = ldv<SMEM>(p + k);
      u[(2 * k) / 3][(2 * k) % 3] = b2c(a.x);
      u[(2 * k + 1) / 3][(2 * k + 1) % 3] = b2c(a.y);
    }
    third_row(u);
  }
};

// ------------------------------------------------------------------ leg spin structure
// unit codes: 0:+1 1:-1 2:+i 3:-i
template <int LT>
struct LegSpin {
  static constexpr int d = LT & 3;
  static constexpr int A = d < 2 ? 3 : 2;
  static constexpr int B = d < 2 ? 2 : 3;
  static constexpr int c0p = d == 0 ? 3 : d == 1 ? 0 : d == 2 ? 3 : 1;
  static constexpr int c1p = d == 0 ? 3 : d == 1 ? 1 : d == 2 ? 2 : 1;
  static constexpr int C0 = LT < 4 ? c0p : (c0p ^ 1);
  static constexpr int C1 = LT < 4 ? c1p : (c1p ^ 1);
};

// ------------------------------------------------------------------ packed pair arithmetic
__device__ __forceinline__ float2 bc(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ cp2 cadd2(cp2 a, cp2 b) { return {__fadd2_rn(a.r, b.r), __fadd2_rn(a.i, b.i)}; }
template <int C>
__device__ __forceinline__ cp2 cunit2(cp2 a) {
  if constexpr (C == 0) return a;
  else if constexpr (C == 1) return {neg2(a.r), neg2(a.i)};
  else if constexpr (C == 2) return {neg2(a.i), a.r};
  else return {a.i, neg2(a.r)};
}
// acc += (c a) * n for a unit c (codes of LegSpin) and a per-slice factor n (nn = -n).
template <int C>
__device__ __forceinline__ void cacc2(cp2& acc, cp2 a, float2 n, float2 nn) {
  if constexpr (C == 0) {
    acc.r = __ffma2_rn(a.r, n, acc.r);
    acc.i = __ffma2_rn(a.i, n, acc.i);
  } else if constexpr (C == 1) {
    acc.r = __ffma2_rn(a.r, nn, acc.r);
    acc.i = __ffma2_rn(a.i, nn, acc.i);
  } else if constexpr (C == 2) {  // i a = (-a.i, a.r)
    acc.r = __ffma2_rn(a.i, nn, acc.r);
    acc.i = __ffma2_rn(a.r, n, acc.i);
  } else {  // -i a = (a.i, -a.r)
    acc.r = __ffma2_rn(a.i, n, acc.r);
    acc.i = __ffma2_rn(a.r, nn, acc.i);
  }
}
// Row r of the link (one complex per colour, the same for both slices) times h.
__device__ __forceinline__ cp2 su3_row2(const cpx<float> (&u)[3], const cp2 (&h)[3]) {
  cp2 o;
  o.r = __fmul2_rn(bc(u[0].r), h[0].r);
  o.i = __fmul2_rn(bc(u[0].r), h[0].i);
  o.r = __ffma2_rn(bc(-u[0].i), h[0].i, o.r);
  o.i = __ffma2_rn(bc(u[0].i), h[0].r, o.i);
#pragma unroll
  for (int c = 1; c < 3; ++c) {
    o.r = __ffma2_rn(bc(u[c].r), h[c].r, o.r);
    o.i = __ffma2_rn(bc(u[c].r), h[c].i, o.i);
    o.r = __ffma2_rn(bc(-u[c].i), h[c].i, o.r);
    o.i = __ffma2_rn(bc(u[c].i), h[c].r, o.i);
  }
  return o;
}

// One leg on NP slice pairs: the neighbour's rows start at row0 of `in` (global or smem);
// nrm points at the F16 norms of its first slice.
// x + c*y on stored FP16 pairs (Re pair in .x, Im pair in .y), c a unit; both operands share
// the site norm, so the sum is formed before the conversion to FP32.
template <int C>
__device__ __forceinline__ cp2 hproj(uint2 x, uint2 y) {
  const __half2 xr = *reinterpret_cast<__half2*>(&x.x), xi = *reinterpret_cast<__half2*>(&x.y);
  const __half2 yr = *reinterpret_cast<__half2*>(&y.x), yi = *reinterpret_cast<__half2*>(&y.y);
  __half2 r, i;
  if constexpr (C == 0) { r = __hadd2(xr, yr); i = __hadd2(xi, yi); }
  else if constexpr (C == 1) { r = __hsub2(xr, yr); i = __hsub2(xi, yi); }
  else if constexpr (C == 2) { r = __hsub2(xr, yi); i = __hadd2(xi, yr); }   // + i y
  else { r = __hadd2(xr, yi); i = __hsub2(xi, yr); }                         // - i y
  return {__half22float2(r), __half22float2(i)};
}

// Mobius A(b, c) applied to a neighbour's slice pair (s0, s0+1) as it is loaded (the forward
// Mobius M: the hopping term acts on A(b, c) psi):
//   (A psi)(s) = b psi(s) + c [w_hi(s) P- psi(s+1) + w_lo(s) P+ psi(s-1)],
// w_lo(0) = w_hi(Ls-1) = -mf.  The site's Ls/2 lanes load the same neighbour's pairs in order,
// so psi(s0-1) is the second slice of the lane below and psi(s0+2) the first slice of the lane
// above (shuffles inside the site's group of lanes, which wraps around the 5th dimension).
struct MobLeg {
  float b, c, clo, chi;  // clo: coefficient of slice s0's s-1 term, chi: of slice s0+1's s+1 term
  int G, from_lo, from_hi;
};
__device__ __forceinline__ MobLeg make_mobleg(int Ls, double b, double c, double mf, int s0) {
  MobLeg m;
  m.G = Ls >> 1;
  const int lg = int(threadIdx.x) & (m.G - 1);
  m.from_lo = (lg + m.G - 1) & (m.G - 1);
  m.from_hi = (lg + 1) & (m.G - 1);
  m.b = float(b);
  m.c = float(c);
  m.clo = s0 == 0 ? float(-mf * c) : float(c);
  m.chi = s0 + 2 == Ls ? float(-mf * c) : float(c);
  return m;
}
// spins 0, 1 (P+): slice s0 takes psi(s0-1) from the lane below, slice s0+1 takes psi(s0)
__device__ __forceinline__ void mob_lower(cp2& a, const MobLeg& m) {
  const unsigned mask = __activemask();
  const float mr = __shfl_sync(mask, a.r.y, m.from_lo, m.G), mi = __shfl_sync(mask, a.i.y, m.from_lo, m.G);
  a.r = __ffma2_rn(make_float2(m.b, m.b), a.r, make_float2(m.clo * mr, m.c * a.r.x));
  a.i = __ffma2_rn(make_float2(m.b, m.b), a.i, make_float2(m.clo * mi, m.c * a.i.x));
}
// spins 2, 3 (P-): slice s0 takes psi(s0+1), slice s0+1 takes psi(s0+2) from the lane above
__device__ __forceinline__ void mob_upper(cp2& a, const MobLeg& m) {
  const unsigned mask = __activemask();
  const float qr = __shfl_sync(mask, a.r.x, m.from_hi, m.G), qi = __shfl_sync(mask, a.i.x, m.from_hi, m.G);
  a.r = __ffma2_rn(make_float2(m.b, m.b), a.r, make_float2(m.c * a.r.y, m.chi * qr));
  a.i = __ffma2_rn(make_float2(m.b, m.b), a.i, make_float2(m.c * a.i.y, m.chi * qi));
}

template <int PIN, int DAG, int NP, int L, bool SMEM, bool MOB = false>
__device__ __forceinline__ void hop_leg_pairs(const cpx<float> (&u)[3][3], const void* in, int64_t row0, int e0,
                                              int LsP, const float* nrm, cp2 (&acc)[NP][12],
                                              const MobLeg* ml = nullptr) {
  using S = LegSpin<DAG ? (L ^ 4) : L>;
  cp2 h0[NP][3], h1[NP][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if constexpr (PIN == GBDW_F16) {
      uint2 x[NP], y[NP], z[NP], w[NP];
      Vec<PIN, 2 * NP, SMEM>::load_pairs_raw(in, row0 + 0 * 3 + c, e0, LsP, x);
      Vec<PIN, 2 * NP, SMEM>::load_pairs_raw(in, row0 + S::A * 3 + c, e0, LsP, y);
      Vec<PIN, 2 * NP, SMEM>::load_pairs_raw(in, row0 + 1 * 3 + c, e0, LsP, z);
      Vec<PIN, 2 * NP, SMEM>::load_pairs_raw(in, row0 + S::B * 3 + c, e0, LsP, w);
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        h0[q][c] = hproj<S::C0>(x[q], y[q]);
        h1[q][c] = hproj<S::C1>(z[q], w[q]);
      }
    } else {
      cp2 x[NP], y[NP], z[NP], w[NP];
      Vec<PIN, 2 * NP, SMEM>::load_pairs(in, row0 + 0 * 3 + c, e0, LsP, x);
      Vec<PIN, 2 * NP, SMEM>::load_pairs(in, row0 + S::A * 3 + c, e0, LsP, y);
      Vec<PIN, 2 * NP, SMEM>::load_pairs(in, row0 + 1 * 3 + c, e0, LsP, z);
      Vec<PIN, 2 * NP, SMEM>::load_pairs(in, row0 + S::B * 3 + c, e0, LsP, w);
      if constexpr (MOB && NP == 1) {
        mob_lower(x[0], *ml);  // spin 0
        mob_lower(z[0], *ml);  // spin 1
        mob_upper(y[0], *ml);  // spin A (2 or 3)
        mob_upper(w[0], *ml);  // spin B (3 or 2)
      }
#pragma unroll
      for (int q = 0; q < NP; ++q) {
        h0[q][c] = cadd2(x[q], cunit2<S::C0>(y[q]));
        h1[q][c] = cadd2(z[q], cunit2<S::C1>(w[q]));
      }
    }
  }
  if constexpr (PIN == GBDW_F16) {
    // U h is linear in h: the neighbour's per-slice norm scales the products as they are
    // accumulated (FFMA2 in place of FADD2) instead of every projected component
#pragma unroll
    for (int q = 0; q < NP; ++q) {
      const float2 nr = ldv<SMEM>(reinterpret_cast<const float2*>(nrm) + q);
      const float2 nn = neg2(nr);
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const cp2 u0 = su3_row2(u[r], h0[q]);
        const cp2 u1 = su3_row2(u[r], h1[q]);
        cacc2<0>(acc[q][0 * 3 + r], u0, nr, nn);
        cacc2<0>(acc[q][1 * 3 + r], u1, nr, nn);
        cacc2<conj_unit<S::C0>::v>(acc[q][S::A * 3 + r], u0, nr, nn);
        cacc2<conj_unit<S::C1>::v>(acc[q][S::B * 3 + r], u1, nr, nn);
      }
    }
  } else {
#pragma unroll
    for (int q = 0; q < NP; ++q)
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const cp2 u0 = su3_row2(u[r], h0[q]);
        const cp2 u1 = su3_row2(u[r], h1[q]);
        acc[q][0 * 3 + r] = cadd2(acc[q][0 * 3 + r], u0);
        acc[q][1 * 3 + r] = cadd2(acc[q][1 * 3 + r], u1);
        acc[q][S::A * 3 + r] = cadd2(acc[q][S::A * 3 + r], cunit2<conj_unit<S::C0>::v>(u0));
        acc[q][S::B * 3 + r] = cadd2(acc[q][S::B * 3 + r], cunit2<conj_unit<S::C1>::v>(u1));
      }
  }
}

// One leg on N single slices (FP64, or N == 1).
template <int PIN, int DAG, int N, int L, bool SMEM, class T>
__device__ __forceinline__ void hop_leg_scalar(const cpx<T> (&u)[3][3], const void* in, int64_t row0, int e0, int LsP,
                                               const float* nrm, cpx<T> (&acc)[N][12]) {
  using S = LegSpin<DAG ? (L ^ 4) : L>;
  cpx<T> h0[N][3], h1[N][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cpx<T> x[N], y[N], z[N], w[N];
    Vec<PIN, N, SMEM>::load(in, row0 + 0 * 3 + c, e0, LsP, x);
    Vec<PIN, N, SMEM>::load(in, row0 + S::A * 3 + c, e0, LsP, y);
    Vec<PIN, N, SMEM>::load(in, row0 + 1 * 3 + c, e0, LsP, z);
    Vec<PIN, N, SMEM>::load(in, row0 + S::B * 3 + c, e0, LsP, w);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const cpx<T> ya = cunit<S::C0>(y[j]);
      const cpx<T> wb = cunit<S::C1>(w[j]);
      h0[j][c] = {x[j].r + ya.r, x[j].i + ya.i};
      h1[j][c] = {z[j].r + wb.r, z[j].i + wb.i};
    }
  }
  if constexpr (PIN == GBDW_F16) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const float nr = ldv<SMEM>(nrm + j);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        h0[j][c].r *= nr;
        h0[j][c].i *= nr;
        h1[j][c].r *= nr;
        h1[j][c].i *= nr;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < N; ++j) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      cpx<T> u0 = {T(0), T(0)}, u1 = {T(0), T(0)};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        cmac(u0, u[r][c], h0[j][c]);
        cmac(u1, u[r][c], h1[j][c]);
      }
      const cpx<T> ra = cunit<conj_unit<S::C0>::v>(u0);
      const cpx<T> rb = cunit<conj_unit<S::C1>::v>(u1);
      acc[j][0 * 3 + r].r += u0.r;
      acc[j][0 * 3 + r].i += u0.i;
      acc[j][1 * 3 + r].r += u1.r;
      acc[j][1 * 3 + r].i += u1.i;
      acc[j][S::A * 3 + r].r += ra.r;
      acc[j][S::A * 3 + r].i += ra.i;
      acc[j][S::B * 3 + r].r += rb.r;
      acc[j][S::B * 3 + r].i += rb.i;
    }
  }
}

// Accumulator of one thread: slice pairs for FP32/FP16 with even N, single slices otherwise.
template <int PIN, int N>
struct Acc {
  static constexpr bool paired = (PIN == GBDW_F32 || PIN == GBDW_F16) && N % 2 == 0;
  using T = typename Arith<PIN>::T;
  using Pair = cp2[N / 2 > 0 ? N / 2 : 1][12];
  using Single = cpx<T>[N][12];
  typename std::conditional<paired, Pair, Single>::type v;
  __device__ __forceinline__ void zero() {
    if constexpr (paired) {
#pragma unroll
      for (int q = 0; q < N / 2; ++q)
#pragma unroll
        for (int k = 0; k < 12; ++k) v[q][k] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    } else {
#pragma unroll
      for (int j = 0; j < N; ++j)
#pragma unroll
        for (int k = 0; k < 12; ++k) v[j][k] = {T(0), T(0)};
    }
  }
  __device__ __forceinline__ void unpack(cpx<T> (&a)[N][12]) const {
    if constexpr (paired) {
#pragma unroll
      for (int q = 0; q < N / 2; ++q)
#pragma unroll
        for (int k = 0; k < 12; ++k) {
          a[2 * q][k] = {v[q][k].r.x, v[q][k].i.x};
          a[2 * q + 1][k] = {v[q][k].r.y, v[q][k].i.y};
        }
    } else {
#pragma unroll
      for (int j = 0; j < N; ++j)
#pragma unroll
        for (int k = 0; k < 12; ++k) a[j][k] = v[j][k];
    }
  }
};

template <int PIN, int DAG, int N, int L, bool SMEM, bool MOB = false>
__device__ __forceinline__ void hop_leg(const cpx<typename Arith<PIN>::T> (&u)[3][3], const void* in, int64_t row0,
                                        int e0, int LsP, const float* nrm, Acc<PIN, N>& acc,
                                        const MobLeg* ml = nullptr) {
  if constexpr (Acc<PIN, N>::paired) hop_leg_pairs<PIN, DAG, N / 2, L, SMEM, MOB>(u, in, row0, e0, LsP, nrm, acc.v, ml);
  else hop_leg_scalar<PIN, DAG, N, L, SMEM>(u, in, row0, e0, LsP, nrm, acc.v);
}

// ------------------------------------------------------------------ kernel parameters
struct DhopParams {
  const void* U;
  const void* in;
  const float* in_norm;
  void* out;
  float* out_norm;
  const uint32_t* nbr4;  // fast path
  const uint32_t* nbr5;  // general path
  int64_t nsite;
  int LsE;               // slices per row (Ls * nrhs)
  int LsP;               // stored slots per row (LsE rounded up to even for F32/F16)
  int Ls;
  double a5;             // 5 - M5   (M epilogue)
  double mf;             // domain-wall mass (M epilogue)
  double* partials;      // fused |out|^2 when non-null
  unsigned* counter;
  double* result;
  unsigned* err;         // device error word (bounded waits that expired)
  // M epilogue: the field of the diagonal (5th-dimension) part, when it is not `in` (the
  // even-odd Schur operator), and the coefficient of the hopping term (1/2 for M).
  const void* cen = nullptr;
  const float* cen_norm = nullptr;
  double khop = 0.5;
  // coefficient of the 5th-dimension hopping part of the epilogue (1 for Shamir; the Mobius
  // operator's diagonal block carries 1 - c (4 - M5) there)
  double c5 = 1.0;
  int dims[4] = {0, 0, 0, 0};  // periodic lattice extents (the blocked site order needs them)
  // CG residual epilogues (EPI 2: FP32 r, EPI 3: FP64 r): r -= alpha * M(in) in place of
  // storing M(in), |r|^2 into the partials; alpha is read from device memory.
  void* r = nullptr;
  float* r_norm = nullptr;  // EPI 4: FP16 r with per-slice norms
  int rLsP = 0;
  const double* alpha = nullptr;
  // Mobius operator in one pass (one right-hand side, Ls a power of two <= 64, two slices per
  // thread): with EPI 1 and DhopDag the hopping result v is replaced by A(mb, mc)^dag v before the
  // M epilogue (Mooee^dag in - khop A(b, c)^dag DhopDag in); with EPI 6 (FP32) A(mb, mc) is
  // applied to the neighbours as they are loaded (Mooee in - khop Dhop A(b, c) in)
  int mob = 0;
  double mb = 1.0, mc = 0.0;
  // direct forms: slices per tile when each site's slices are cut into tiles (0: one tile)
  int TE = 0;
  // direct forms on periodic lattices: sweep in t-bricks of this many t-slices (0/1: natural order)
  int brick = 0;
};

// Writes N slices of v[N][12] (slices e0.., norms for F16); returns the sum of squares of
// what was stored.
template <int POUT, int N, class T>
__device__ __forceinline__ float store_spinor(void* out, float* out_norm, int64_t site, int e0, int LsE, int LsP,
                                              const cpx<T> (&v)[N][12]) {
  float nrm2 = 0.f;
  const int64_t row0 = site * 12;
  if constexpr (POUT == GBDW_F16) {
    float scale[N], nm[N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
      float m = 0.f;
#pragma unroll
      for (int k = 0; k < 12; ++k) m = fmaxf(m, fmaxf(fabsf(float(v[j][k].r)), fabsf(float(v[j][k].i))));
      nm[j] = m;
      scale[j] = m > 0.f ? 1.0f / m : 0.f;
    }
    store_norms<N>(out_norm, site * LsE + e0, nm);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      cpx<float> w[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        w[j] = {float(v[j][k].r) * scale[j], float(v[j][k].i) * scale[j]};
        // norm of the value as stored
        const float2 b = __half22float2(__floats2half2_rn(w[j].r, w[j].i));
        nrm2 = fmaf(b.x * nm[j], b.x * nm[j], nrm2);
        nrm2 = fmaf(b.y * nm[j], b.y * nm[j], nrm2);
      }
      Vec<GBDW_F16, N>::store_scaled(out, row0 + k, e0, LsP, w);
    }
  } else {
    using TO = typename Arith<POUT>::T;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      cpx<TO> w[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        w[j] = {TO(v[j][k].r), TO(v[j][k].i)};
        nrm2 = fmaf(float(w[j].r), float(w[j].r), nrm2);
        nrm2 = fmaf(float(w[j].i), float(w[j].i), nrm2);
      }
      Vec<POUT, N>::store(out, row0 + k, e0, LsP, w);
    }
  }
  return nrm2;
}

template <int N>
__device__ __forceinline__ double sumsq(const cpx<double> (&v)[N][12]) {
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int k = 0; k < 12; ++k) s += v[j][k].r * v[j][k].r + v[j][k].i * v[j][k].i;
  return s;
}
template <int N>
__device__ __forceinline__ double sumsq(const cpx<float> (&)[N][12]) {
  return 0.0;
}
template <int N>
__device__ __forceinline__ double sumsq(const cpx<dsf> (&v)[N][12]) {
  dsf s(0.f, 0.f);
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int k = 0; k < 12; ++k) s = fma(v[j][k].i, v[j][k].i, fma(v[j][k].r, v[j][k].r, s));
  return double(s);
}

// ------------------------------------------------------------------ Shamir 5D terms
// out(s) = a5 psi(s) - k D(s) - [P- psi(s+1) + P+ psi(s-1)]       (dag = 0)
// out(s) = a5 psi(s) - k D(s) - [P+ psi(s+1) + P- psi(s-1)]       (dag = 1)
// P+ keeps spins 0,1 and P- spins 2,3 (gamma5 = diag(1,1,-1,-1)); a step across the
// s boundary picks up -mf.  k = p.khop (1/2 for M) and psi is p.cen when set, else the
// hopping input.  Requires nrhs == 1 (LsE == Ls).
template <int PIN, int DAG, int N, class T>
__device__ __forceinline__ void dwf_epilogue(const DhopParams& p, int64_t site, int s0, cpx<T> (&acc)[N][12]) {
  const int Ls = p.Ls;
  const int LsP = p.LsP;
  const int64_t row0 = site * 12;
  const void* cin = p.cen ? p.cen : p.in;
  const float* cnorm = p.cen ? p.cen_norm : p.in_norm;
  cpx<T> cen[N][12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    cpx<T> x[N];
    Vec<PIN, N>::load(cin, row0 + k, s0, LsP, x);
#pragma unroll
    for (int j = 0; j < N; ++j) cen[j][k] = x[j];
  }
  const int slo = (s0 == 0) ? Ls - 1 : s0 - 1;
  const int shi = (s0 + N == Ls) ? 0 : s0 + N;
  const T flo = (s0 == 0) ? T(-p.mf) : T(1);
  const T fhi = (s0 + N == Ls) ? T(-p.mf) : T(1);
  constexpr int LO0 = DAG ? 2 : 0;  // first spin fed by psi(s-1)
  constexpr int HI0 = DAG ? 0 : 2;  // first spin fed by psi(s+1)
  cpx<T> lo[6], hi[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    lo[k] = Elem<PIN>::ld(cin, row0 + LO0 * 3 + k, slo, LsP);
    hi[k] = Elem<PIN>::ld(cin, row0 + HI0 * 3 + k, shi, LsP);
  }
  T nlo = flo, nhi = fhi;
  if constexpr (PIN == GBDW_F16) {
    float nc[N];
    load_norms<N>(cnorm, site * Ls + s0, nc);
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        cen[j][k].r *= nc[j];
        cen[j][k].i *= nc[j];
      }
    nlo *= __ldg(cnorm + site * Ls + slo);
    nhi *= __ldg(cnorm + site * Ls + shi);
  }
  const T a5 = T(p.a5), kh = T(p.khop), c5 = T(p.c5);
#pragma unroll
  for (int j = 0; j < N; ++j) {
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      acc[j][k].r = a5 * cen[j][k].r - kh * acc[j][k].r;
      acc[j][k].i = a5 * cen[j][k].i - kh * acc[j][k].i;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const cpx<T> m = (j == 0) ? cpx<T>{lo[k].r * nlo, lo[k].i * nlo} : cen[j - 1 < 0 ? 0 : j - 1][LO0 * 3 + k];
      acc[j][LO0 * 3 + k].r -= c5 * m.r;
      acc[j][LO0 * 3 + k].i -= c5 * m.i;
      const cpx<T> q = (j == N - 1) ? cpx<T>{hi[k].r * nhi, hi[k].i * nhi} : cen[j + 1 >= N ? N - 1 : j + 1][HI0 * 3 + k];
      acc[j][HI0 * 3 + k].r -= c5 * q.r;
      acc[j][HI0 * 3 + k].i -= c5 * q.i;
    }
  }
}

// ------------------------------------------------------------------ Mobius 5th-dimension adjoint
// v <- A(b, c)^dag v on one thread's slice pair (s0, s0+1):
//   (A^dag v)(s) = b v(s) + c [w_lo(s) P- v(s-1) + w_hi(s) P+ v(s+1)],
// w_lo(0) = w_hi(Ls-1) = -mf, 1 elsewhere.  The Ls/2 threads of a site hold its slices in
// consecutive lanes (pairs in order), so P- v(s0-1) is the second slice of the lane below and
// P+ v(s0+2) the first slice of the lane above, both taken with shuffles inside the site's
// group of lanes (which wraps around the 5th dimension).  Every site's lanes are active or
// inactive together.
template <class T>
__device__ __forceinline__ void mobius_adj_hop(const DhopParams& p, int s0, cpx<T> (&v)[2][12]) {
  const int G = p.Ls >> 1;  // lanes per site: a power of two <= 32
  const unsigned mask = __activemask();
  const int lg = int(threadIdx.x) & (G - 1);
  const int from_lo = (lg + G - 1) & (G - 1);
  const int from_hi = (lg + 1) & (G - 1);
  cpx<T> vm[6], vp[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    vm[k] = {__shfl_sync(mask, v[1][6 + k].r, from_lo, G), __shfl_sync(mask, v[1][6 + k].i, from_lo, G)};
    vp[k] = {__shfl_sync(mask, v[0][k].r, from_hi, G), __shfl_sync(mask, v[0][k].i, from_hi, G)};
  }
  const T b = T(p.mb), c = T(p.mc);
  const T clo = s0 == 0 ? T(-p.mf) * c : c;           // slice s0: its s-1 wraps at the wall
  const T chi = s0 + 2 == p.Ls ? T(-p.mf) * c : c;    // slice s0+1: its s+1 wraps at the wall
  cpx<T> h[2][12];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    // P+ (spins 0, 1) from s+1
    h[0][k] = {b * v[0][k].r + c * v[1][k].r, b * v[0][k].i + c * v[1][k].i};
    h[1][k] = {b * v[1][k].r + chi * vp[k].r, b * v[1][k].i + chi * vp[k].i};
    // P- (spins 2, 3) from s-1
    h[0][6 + k] = {b * v[0][6 + k].r + clo * vm[k].r, b * v[0][6 + k].i + clo * vm[k].i};
    h[1][6 + k] = {b * v[1][6 + k].r + c * v[0][6 + k].r, b * v[1][6 + k].i + c * v[0][6 + k].i};
  }
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int k = 0; k < 12; ++k) v[j][k] = h[j][k];
}

// ------------------------------------------------------------------ per-site finish
// EPI 0: store Dhop(in); EPI 1: store M(in); EPI 2 / 3 / 4: r -= alpha M(in) with r FP32 / FP64 /
// FP16 (the CG residual update fused into the operator's second pass; M(in) is not stored);
// EPI 6: store the Mobius M(in), A(b, c) applied to the neighbours as they are loaded.
// Returns |what was stored|^2 in part (FP32 outputs) or dpart (FP64 outputs and EPI 2-4).
template <int PIN, int POUT, int DAG, int N, int EPI, class T>
__device__ __forceinline__ void finish_site(const DhopParams& p, int64_t site, int s0, int LsE, int LsP,
                                            cpx<T> (&v)[N][12], float& part, double& dpart) {
  if constexpr (EPI == 1 && DAG == 1 && N == 2 && PIN != GBDW_DS) {
    if (p.mob) mobius_adj_hop(p, s0, v);
  }
  if constexpr (EPI >= 1) dwf_epilogue<PIN, DAG, N>(p, site, s0, v);
  if constexpr (EPI == 4) {
    // FP16 r: dequantise with its per-slice norms, update in FP32, store with new norms
    const float al = float(*p.alpha);
    float nr[N];
    load_norms<N>(p.r_norm, site * LsE + s0, nr);
    cpx<float> rv[N][12];
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      cpx<float> x[N];
      Vec<GBDW_F16, N>::load(p.r, site * 12 + k, s0, p.rLsP, x);
#pragma unroll
      for (int j = 0; j < N; ++j)
        rv[j][k] = {fmaf(-al, float(v[j][k].r), x[j].r * nr[j]), fmaf(-al, float(v[j][k].i), x[j].i * nr[j])};
    }
    dpart = double(store_spinor<GBDW_F16, N>(p.r, p.r_norm, site, s0, LsE, p.rLsP, rv));
  } else if constexpr (EPI == 2 || EPI == 3) {
    constexpr int RP = EPI == 2 ? GBDW_F32 : GBDW_F64;
    using TR = typename Arith<RP>::T;
    const TR al = TR(*p.alpha);
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      cpx<TR> rv[N];
      Vec<RP, N>::load(p.r, site * 12 + k, s0, p.rLsP, rv);
      TR ks = TR(0);
#pragma unroll
      for (int j = 0; j < N; ++j) {
        rv[j].r -= al * TR(v[j][k].r);
        rv[j].i -= al * TR(v[j][k].i);
        ks += rv[j].r * rv[j].r + rv[j].i * rv[j].i;
      }
      s += double(ks);
      Vec<RP, N>::store(p.r, site * 12 + k, s0, p.rLsP, rv);
    }
    dpart = s;
  } else {
    part = store_spinor<POUT, N>(p.out, p.out_norm, site, s0, LsE, LsP, v);
    if constexpr (POUT == GBDW_F64 || POUT == GBDW_DS) dpart = sumsq<N>(v);
  }
}

// ------------------------------------------------------------------ kernels
// Hopping sum for one thread: site and first slice s0 of N consecutive slices.
template <int PIN, int GP, int DAG, int N, bool MOB = false>
__device__ __forceinline__ void dhop_thread(const DhopParams& p, unsigned site, int s0,
                                            cpx<typename Arith<PIN>::T> (&out)[N][12]) {
  using T = typename Arith<PIN>::T;
  Acc<PIN, N> acc;
  acc.zero();
  const uint32_t* nb = p.nbr4 + size_t(site) * 8;
  MobLeg ml;
  if constexpr (MOB) ml = make_mobleg(p.Ls, p.mb, p.mc, p.mf, s0);
#define GBDW_LEG(L)                                                                                    \
  {                                                                                                    \
    const int64_t n = __ldg(nb + L);                                                                   \
    cpx<T> u[3][3];                                                                                    \
    LinkIO<GP>::load(p.U, size_t(site) * 8 + L, u);                                                    \
    hop_leg<PIN, DAG, N, L, false, MOB>(u, p.in, n * 12, s0, p.LsP, p.in_norm + n * p.LsE + s0, acc, &ml); \
  }
  // each forward leg next to its backward partner: the x-neighbours of a CTA's sites are the
  // CTA's own sites, and a spinor one thread reads for X+ is read again for X- by the thread
  // of the site two steps along x while its lines are still in L1
  GBDW_LEG(0) GBDW_LEG(4) GBDW_LEG(1) GBDW_LEG(5) GBDW_LEG(2) GBDW_LEG(6) GBDW_LEG(3) GBDW_LEG(7)
#undef GBDW_LEG
  acc.unpack(out);
}

// EPI 0: out = Dhop(in) ; EPI 1: out = M(in) (Shamir).  |out|^2 fused when p.partials != 0.
// MINB > 0 caps registers so that MINB CTAs of up to MAXT threads fit on an SM (more warps,
// more loads in flight); MINB = 0 leaves the compiler free up to 256 threads.
// LSPC > 0: the launch guarantees LsE == LsP == LSPC, so every row offset is a compile-time
// constant.  BLK: a CTA of 16*G threads takes a 2x2x2x2 block of 4D sites instead of 16
// consecutive ones, so half of every site's neighbours are the CTA's own sites and their
// loads can hit L1 (needs a periodic lattice with even extents, p.dims).
template <int PIN, int POUT, int GP, int DAG, int N, int EPI, int MINB = 0, int LSPC = 0, int MAXT = 128,
          int BLK = 0>
__global__ void __launch_bounds__(MINB > 0 ? MAXT : 256, MINB > 0 ? MINB : 1) k_dhop(const DhopParams p_) {
  using T = typename Arith<PIN>::T;
  DhopParams p = p_;
  if constexpr (LSPC > 0) {
    p.LsE = LSPC;
    p.LsP = LSPC;
  }
  const unsigned G = unsigned(p.LsE) / N;
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = tid < unsigned(p.nsite) * G;
  float part = 0.f;
  double dpart = 0.0;
  if (active) {
    unsigned site = tid / G;
    int s0 = int(tid - site * G) * N;
    if constexpr (!BLK) {
      if (p.TE > 0 && p.TE < p.LsE) {
        // Ls / RHS tiles: threads ordered (tile, site, slice group), TE slices per tile, so a
        // CTA holds more sites with fewer slices each (the link is reused over one tile)
        const unsigned GT = unsigned(p.TE) / N;
        const unsigned per_tile = unsigned(p.nsite) * GT;
        const unsigned tile = tid / per_tile;
        const unsigned r = tid - tile * per_tile;
        site = r / GT;
        s0 = int(tile) * p.TE + int(r - site * GT) * N;
      }
      if (p.brick > 1) {
        // t-bricks: the sweep visits sites (t brick, z, y, x, t inside the brick), so a site's
        // neighbours along t are read within a few sites of each other instead of a whole 3D
        // volume apart (periodic lattice, Lt a multiple of the brick)
        unsigned j = site;
        const unsigned B = unsigned(p.brick);
        const unsigned tin = j % B;
        j /= B;
        const unsigned Lx = unsigned(p.dims[0]), Ly = unsigned(p.dims[1]), Lz = unsigned(p.dims[2]);
        const unsigned x = j % Lx;
        j /= Lx;
        const unsigned y = j % Ly;
        j /= Ly;
        const unsigned z = j % Lz;
        const unsigned tb = j / Lz;
        site = x + Lx * (y + Ly * (z + Lz * (tb * B + tin)));
      }
    }
    if constexpr (BLK) {
      const unsigned l = threadIdx.x / G;  // 0..15 inside the block
      const unsigned hx = unsigned(p.dims[0]) >> 1, hy = unsigned(p.dims[1]) >> 1, hz = unsigned(p.dims[2]) >> 1;
      unsigned b = blockIdx.x;
      const unsigned bx = b % hx;
      b /= hx;
      const unsigned by = b % hy;
      b /= hy;
      const unsigned bz = b % hz;
      const unsigned bt = b / hz;
      const unsigned x = 2 * bx + (l & 1), y = 2 * by + ((l >> 1) & 1), z = 2 * bz + ((l >> 2) & 1),
                     t = 2 * bt + (l >> 3);
      site = x + unsigned(p.dims[0]) * (y + unsigned(p.dims[1]) * (z + unsigned(p.dims[2]) * t));
    }
    cpx<T> acc[N][12];
    dhop_thread<PIN, GP, DAG, N, EPI == 6>(p, site, s0, acc);
    finish_site<PIN, POUT, DAG, N, EPI>(p, site, s0, p.LsE, p.LsP, acc, part, dpart);
  }
  if (p.partials) {
    double v[1] = {(POUT == GBDW_F64 || POUT == GBDW_DS || (EPI >= 2 && EPI <= 4)) ? dpart : double(part)};
    block_partial<1>(v, p.partials);
  }
}

// General 5D table (no 4D factorisation): one thread per 5D site, neighbour read per leg.
template <int PIN, int GP, int DAG>
__global__ void __launch_bounds__(256) k_dhop_general(const DhopParams p) {
  using T = typename Arith<PIN>::T;
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= unsigned(p.nsite) * unsigned(p.Ls)) return;
  const unsigned site = tid / unsigned(p.Ls);
  const int s = int(tid - site * unsigned(p.Ls));
  Acc<PIN, 1> acc;
  acc.zero();
  const uint32_t* nb = p.nbr5 + size_t(tid) * 8;
  const int64_t Ls = p.Ls;
#define GBDW_LEG(L)                                                                            \
  {                                                                                            \
    const int64_t n5 = __ldg(nb + L);                                                          \
    const int64_t ns = n5 / Ls;                                                                \
    const int sn = int(n5 - ns * Ls);                                                          \
    cpx<T> u[3][3];                                                                            \
    LinkIO<GP>::load(p.U, size_t(site) * 8 + L, u);                                            \
    hop_leg<PIN, DAG, 1, L, false>(u, p.in, ns * 12, sn, p.LsP, p.in_norm + n5, acc);         \
  }
  GBDW_LEG(0) GBDW_LEG(1) GBDW_LEG(2) GBDW_LEG(3) GBDW_LEG(4) GBDW_LEG(5) GBDW_LEG(6) GBDW_LEG(7)
#undef GBDW_LEG
  cpx<T> out[1][12];
  acc.unpack(out);
  store_spinor<PIN, 1>(p.out, p.out_norm, site, s, p.Ls, p.LsP, out);
}

// ------------------------------------------------------------------ launch dispatch
struct DhopLaunch {
  int threads;     // per CTA (target; the staged kernels round to whole sites)
  int spt;         // slices per thread
  int mode = 0;    // 0: direct loads, 1: TMA-staged (CTA ring), 2: TMA-staged (one ring per warp),
                   // 3: direct, FP32/FP16 Ls = 16 at compile time, registers balanced for 6 CTAs/SM
                   // 4: form 3 on 2x2x2x2 site blocks per 128-thread CTA (periodic, even extents)
  int stages = 4;  // staged kernels: depth of the leg ring
  int split = 1;   // forms 0 and 3: each site's Ls*nrhs slices cut into this many tiles
  int brick = 1;   // forms 0 and 3 on periodic lattices: t-brick sweep order (1: natural order)
};

// Implemented per precision family in dhop_f64.cu / dhop_f32.cu / dhop_f16.cu.
int launch_dhop_f64(const DhopParams& p, int dag, int epi, DhopLaunch L);
int launch_dhop_f32(const DhopParams& p, int dag, int epi, DhopLaunch L);
int launch_dhop_f16(const DhopParams& p, int gprec, int dag, int epi, DhopLaunch L);
int launch_dhop_general(const DhopParams& p, int prec, int dag);
// The double-single form of the FP64 operator (dhop_ds.cu): direct loads, one slice per thread in
// CTAs of DS_THREADS with registers capped for minb (3 or 4) CTAs per SM, Dhop and M; p.U must be
// the gauge field's split links (ds_links).  Its tuned shapes sit in the tune cache under the
// epilogue keys offset by DS_KEY, with `stages` holding minb and `brick` the t-brick order.
constexpr int DS_THREADS = 128;
constexpr int DS_KEY = 64;
int launch_dhop_ds(const DhopParams& p, int dag, int epi, int minb);
int ds_links(const gbdw_gauge* g, const void** out);
// whether FP64 operators run in double-single arithmetic here: the setting for solvers inside a
// SolverScope (the solvers open one), the setting for operator calls outside
bool fp64_double_single();
struct SolverScope {
  SolverScope();
  ~SolverScope();
};
// forces one FP64 arithmetic (GBDW_FP64_NATIVE / _DOUBLE_SINGLE) on this thread while alive
struct Fp64ArithOverride {
  explicit Fp64ArithOverride(int mode);
  ~Fp64ArithOverride();
  int prev;
};
// Sites per CTA, threads and dynamic shared memory of a staged form (L.mode 1 or 2), or false
// if that form cannot run for this precision and extent.
bool tma_shape(int prec, int LsE, DhopLaunch L, int* NS, int* threads, size_t* smem);

}  // namespace gbdw
