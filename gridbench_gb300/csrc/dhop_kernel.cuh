// The domain-wall Wilson hopping kernel (Dhop / DhopDag, optionally fused into the Shamir
// operator M) for the GB300 layout described in common.cuh.
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
// Work decomposition: one thread per (4D site, SPT consecutive innermost slices).  The 4D
// neighbour and the link of a leg are loaded once per thread and reused over its SPT slices;
// threads of one site read the same link (one broadcast transaction) and consecutive threads
// read consecutive slices, so each spinor component load of a warp is a run of whole sectors.
#pragma once
#include "common.cuh"

namespace gbdw {

// ------------------------------------------------------------------ storage traits
template <int P>
struct Arith {
  using T = float;
};
template <>
struct Arith<GBDW_F64> {
  using T = double;
};

// Load / store N consecutive complex entries starting at element e (e % N == 0).
template <int P, int N>
struct SpinIO;

template <int N>
struct SpinIO<GBDW_F32, N> {
  static __device__ __forceinline__ void load(const void* base, int64_t e, cpx<float> (&v)[N]) {
    if (N == 1) {
      const float2 a = __ldg((const float2*)base + e);
      v[0] = {a.x, a.y};
    } else {
#pragma unroll
      for (int k = 0; k < N / 2; ++k) {
        const float4 a = __ldg((const float4*)base + (e >> 1) + k);
        v[2 * k] = {a.x, a.y};
        v[2 * k + 1] = {a.z, a.w};
      }
    }
  }
  static __device__ __forceinline__ void store(void* base, int64_t e, const cpx<float> (&v)[N]) {
    if (N == 1) {
      ((float2*)base)[e] = make_float2(v[0].r, v[0].i);
    } else {
#pragma unroll
      for (int k = 0; k < N / 2; ++k)
        ((float4*)base)[(e >> 1) + k] = make_float4(v[2 * k].r, v[2 * k].i, v[2 * k + 1].r, v[2 * k + 1].i);
    }
  }
};

template <int N>
struct SpinIO<GBDW_F64, N> {
  static __device__ __forceinline__ void load(const void* base, int64_t e, cpx<double> (&v)[N]) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const double2 a = __ldg((const double2*)base + e + k);
      v[k] = {a.x, a.y};
    }
  }
  static __device__ __forceinline__ void store(void* base, int64_t e, const cpx<double> (&v)[N]) {
#pragma unroll
    for (int k = 0; k < N; ++k) ((double2*)base)[e + k] = make_double2(v[k].r, v[k].i);
  }
};

__device__ __forceinline__ cpx<float> h2c(unsigned w) {
  __half2 h = *reinterpret_cast<__half2*>(&w);
  const float2 f = __half22float2(h);
  return {f.x, f.y};
}
__device__ __forceinline__ unsigned c2h(float r, float i) {
  __half2 h = __floats2half2_rn(r, i);
  return *reinterpret_cast<unsigned*>(&h);
}

// F16 entries are stored divided by the site norm; load returns the stored values, the
// caller multiplies by the norm (after projection, which is linear).
template <int N>
struct SpinIO<GBDW_F16, N> {
  static __device__ __forceinline__ void load(const void* base, int64_t e, cpx<float> (&v)[N]) {
    if (N == 1) {
      v[0] = h2c(__ldg((const unsigned*)base + e));
    } else if (N == 2) {
      const uint2 a = __ldg((const uint2*)base + (e >> 1));
      v[0] = h2c(a.x);
      v[1] = h2c(a.y);
    } else {
#pragma unroll
      for (int k = 0; k < N / 4; ++k) {
        const uint4 a = __ldg((const uint4*)base + (e >> 2) + k);
        v[4 * k] = h2c(a.x);
        v[4 * k + 1] = h2c(a.y);
        v[4 * k + 2] = h2c(a.z);
        v[4 * k + 3] = h2c(a.w);
      }
    }
  }
  static __device__ __forceinline__ void store_raw(void* base, int64_t e, const unsigned (&w)[N]) {
    if (N == 1) {
      ((unsigned*)base)[e] = w[0];
    } else if (N == 2) {
      ((uint2*)base)[e >> 1] = make_uint2(w[0], w[1]);
    } else {
#pragma unroll
      for (int k = 0; k < N / 4; ++k)
        ((uint4*)base)[(e >> 2) + k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    }
  }
};

template <int N>
__device__ __forceinline__ void load_norms(const float* nrm, int64_t e, float (&v)[N]) {
  if (N == 1) {
    v[0] = __ldg(nrm + e);
  } else if (N == 2) {
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
  if (N == 1) {
    nrm[e] = v[0];
  } else if (N == 2) {
    ((float2*)nrm)[e >> 1] = make_float2(v[0], v[1]);
  } else {
#pragma unroll
    for (int k = 0; k < N / 4; ++k) ((float4*)nrm)[(e >> 2) + k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  }
}

// Link loads: full 3x3 (F64/F32) or two rows with the third rebuilt as conj(r0 x r1).
template <int GP>
struct LinkIO;

template <>
struct LinkIO<GBDW_F32> {
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<float> (&u)[3][3]) {
    const float2* p = (const float2*)U + link * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const float2 a = __ldg(p + k);
      u[k / 3][k % 3] = {a.x, a.y};
    }
  }
};
template <>
struct LinkIO<GBDW_F64> {
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<double> (&u)[3][3]) {
    const double2* p = (const double2*)U + link * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      const double2 a = __ldg(p + k);
      u[k / 3][k % 3] = {a.x, a.y};
    }
  }
};

__device__ __forceinline__ void third_row(cpx<float> (&u)[3][3]) {
  // r2 = conj(r0 x r1)
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
    cpx<float> t = cmul(u[0][c1], u[1][c2]);
    const cpx<float> q = cmul(u[0][c2], u[1][c1]);
    t.r -= q.r;
    t.i -= q.i;
    u[2][c] = {t.r, -t.i};
  }
}

template <>
struct LinkIO<GBDW_F16> {
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<float> (&u)[3][3]) {
    const uint2* p = (const uint2*)U + link * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint2 a = __ldg(p + k);
      u[(2 * k) / 3][(2 * k) % 3] = h2c(a.x);
      u[(2 * k + 1) / 3][(2 * k + 1) % 3] = h2c(a.y);
    }
    third_row(u);
  }
};

__device__ __forceinline__ cpx<float> b2c(unsigned w) {
  __nv_bfloat162 h = *reinterpret_cast<__nv_bfloat162*>(&w);
  const float2 f = __bfloat1622float2(h);
  return {f.x, f.y};
}
template <>
struct LinkIO<GBDW_BF16> {
  static __device__ __forceinline__ void load(const void* U, size_t link, cpx<float> (&u)[3][3]) {
    const uint2* p = (const uint2*)U + link * 3;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const uint2 a = __ldg(p + k);
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

// One leg for N slices: neighbour entries start at element eb (component stride LsE),
// F16 norms at nidx.
template <int PIN, int GP, int DAG, int N, int L, class T>
__device__ __forceinline__ void hop_leg(const void* __restrict__ U, size_t link, const void* __restrict__ in,
                                        const float* __restrict__ in_norm, int64_t eb, int64_t nidx,
                                        int LsE, cpx<T> (&acc)[N][12]) {
  using S = LegSpin<DAG ? (L ^ 4) : L>;
  cpx<T> h0[N][3], h1[N][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cpx<T> x[N], y[N], z[N], w[N];
    SpinIO<PIN, N>::load(in, eb + int64_t(0 * 3 + c) * LsE, x);
    SpinIO<PIN, N>::load(in, eb + int64_t(S::A * 3 + c) * LsE, y);
    SpinIO<PIN, N>::load(in, eb + int64_t(1 * 3 + c) * LsE, z);
    SpinIO<PIN, N>::load(in, eb + int64_t(S::B * 3 + c) * LsE, w);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const cpx<T> ya = cunit<S::C0>(y[j]);
      const cpx<T> wb = cunit<S::C1>(w[j]);
      h0[j][c] = {x[j].r + ya.r, x[j].i + ya.i};
      h1[j][c] = {z[j].r + wb.r, z[j].i + wb.i};
    }
  }
  if constexpr (PIN == GBDW_F16) {
    float nr[N];
    load_norms<N>(in_norm, nidx, nr);
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        h0[j][c].r *= nr[j];
        h0[j][c].i *= nr[j];
        h1[j][c].r *= nr[j];
        h1[j][c].i *= nr[j];
      }
  }
  cpx<T> u[3][3];
  LinkIO<GP>::load(U, link, u);
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
  int LsE;               // innermost extent (Ls * nrhs)
  int Ls;
  double a5;             // 5 - M5   (M epilogue)
  double mf;             // domain-wall mass (M epilogue)
  double* partials;      // fused |out|^2 when non-null
  unsigned* counter;
  double* result;
  unsigned* err;         // device error word (bounded waits that expired)
};

// Writes N slices of result spinor v[N][12] at element eo (and norms at no for F16);
// returns the sum of squares of what was stored (as read back in arithmetic precision).
template <int POUT, int N, class T>
__device__ __forceinline__ float store_spinor(void* out, float* out_norm, int64_t eo, int64_t no, int LsE,
                                              const cpx<T> (&v)[N][12]) {
  float nrm2 = 0.f;
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
    store_norms<N>(out_norm, no, nm);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      unsigned w[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        w[j] = c2h(float(v[j][k].r) * scale[j], float(v[j][k].i) * scale[j]);
        const cpx<float> b = h2c(w[j]);
        nrm2 = fmaf(b.r * nm[j], b.r * nm[j], nrm2);
        nrm2 = fmaf(b.i * nm[j], b.i * nm[j], nrm2);
      }
      SpinIO<GBDW_F16, N>::store_raw(out, eo + int64_t(k) * LsE, w);
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
      SpinIO<POUT, N>::store(out, eo + int64_t(k) * LsE, w);
    }
  }
  return nrm2;
}

// Double-precision sum of squares for FP64 outputs (exact accumulation of the stored values).
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
__device__ __forceinline__ double sumsq(const cpx<float> (&v)[N][12]) {
  return 0.0;
}

// ------------------------------------------------------------------ Shamir 5D terms
// out(s) = a5 psi(s) - 1/2 D(s) - [P- psi(s+1) + P+ psi(s-1)]       (dag = 0)
// out(s) = a5 psi(s) - 1/2 D(s) - [P+ psi(s+1) + P- psi(s-1)]       (dag = 1)
// P+ keeps spins 0,1 and P- spins 2,3 (gamma5 = diag(1,1,-1,-1)); a step across the
// s boundary picks up -mf.  Requires nrhs == 1 (LsE == Ls).
template <int PIN, int DAG, int N, class T>
__device__ __forceinline__ void dwf_epilogue(const DhopParams& p, int64_t site, int s0, cpx<T> (&acc)[N][12]) {
  const int Ls = p.Ls;
  const int64_t base = site * 12 * int64_t(Ls);
  cpx<T> cen[N][12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    cpx<T> x[N];
    SpinIO<PIN, N>::load(p.in, base + int64_t(k) * Ls + s0, x);
#pragma unroll
    for (int j = 0; j < N; ++j) cen[j][k] = x[j];
  }
  const int slo = (s0 == 0) ? Ls - 1 : s0 - 1;
  const int shi = (s0 + N == Ls) ? 0 : s0 + N;
  const T flo = (s0 == 0) ? T(-p.mf) : T(1);
  const T fhi = (s0 + N == Ls) ? T(-p.mf) : T(1);
  // spins taken from s-1 and from s+1
  constexpr int LO0 = DAG ? 2 : 0;  // first spin fed by psi(s-1)
  constexpr int HI0 = DAG ? 0 : 2;  // first spin fed by psi(s+1)
  cpx<T> lo[6], hi[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    cpx<T> x[1], y[1];
    SpinIO<PIN, 1>::load(p.in, base + int64_t(LO0 * 3 + k) * Ls + slo, x);
    SpinIO<PIN, 1>::load(p.in, base + int64_t(HI0 * 3 + k) * Ls + shi, y);
    lo[k] = x[0];
    hi[k] = y[0];
  }
  T nlo = flo, nhi = fhi;
  if constexpr (PIN == GBDW_F16) {
    float nc[N];
    load_norms<N>(p.in_norm, site * Ls + s0, nc);
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        cen[j][k].r *= nc[j];
        cen[j][k].i *= nc[j];
      }
    nlo *= __ldg(p.in_norm + site * Ls + slo);
    nhi *= __ldg(p.in_norm + site * Ls + shi);
  }
  const T a5 = T(p.a5);
#pragma unroll
  for (int j = 0; j < N; ++j) {
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      acc[j][k].r = a5 * cen[j][k].r - T(0.5) * acc[j][k].r;
      acc[j][k].i = a5 * cen[j][k].i - T(0.5) * acc[j][k].i;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      // psi(s-1) feeds spins LO0, LO0+1
      const cpx<T> m = (j == 0) ? cpx<T>{lo[k].r * nlo, lo[k].i * nlo} : cen[j - 1 < 0 ? 0 : j - 1][LO0 * 3 + k];
      acc[j][LO0 * 3 + k].r -= m.r;
      acc[j][LO0 * 3 + k].i -= m.i;
      const cpx<T> q = (j == N - 1) ? cpx<T>{hi[k].r * nhi, hi[k].i * nhi} : cen[j + 1 >= N ? N - 1 : j + 1][HI0 * 3 + k];
      acc[j][HI0 * 3 + k].r -= q.r;
      acc[j][HI0 * 3 + k].i -= q.i;
    }
  }
}

// ------------------------------------------------------------------ kernels
// Hopping sum for one thread: site and first slice s0 of N consecutive slices.
template <int PIN, int GP, int DAG, int N, class T>
__device__ __forceinline__ void dhop_thread(const DhopParams& p, unsigned site, int s0, cpx<T> (&acc)[N][12]) {
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[j][k] = {T(0), T(0)};
  const uint32_t* nb = p.nbr4 + size_t(site) * 8;
  const int64_t LsE = p.LsE;
#define GBDW_LEG(L)                                                                                  \
  {                                                                                                  \
    const int64_t n = __ldg(nb + L);                                                                 \
    hop_leg<PIN, GP, DAG, N, L>(p.U, size_t(site) * 8 + L, p.in, p.in_norm, n * 12 * LsE + s0,       \
                                n * LsE + s0, p.LsE, acc);                                           \
  }
  GBDW_LEG(0) GBDW_LEG(1) GBDW_LEG(2) GBDW_LEG(3) GBDW_LEG(4) GBDW_LEG(5) GBDW_LEG(6) GBDW_LEG(7)
#undef GBDW_LEG
}

// EPI 0: out = Dhop(in) ; EPI 1: out = M(in) (Shamir).  |out|^2 fused when p.partials != 0.
template <int PIN, int POUT, int GP, int DAG, int N, int EPI>
__global__ void __launch_bounds__(256) k_dhop(const DhopParams p) {
  using T = typename Arith<PIN>::T;
  const unsigned G = unsigned(p.LsE) / N;
  const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = tid < unsigned(p.nsite) * G;
  float part = 0.f;
  double dpart = 0.0;
  if (active) {
    const unsigned site = tid / G;
    const int s0 = int(tid - site * G) * N;
    cpx<T> acc[N][12];
    dhop_thread<PIN, GP, DAG, N>(p, site, s0, acc);
    if constexpr (EPI == 1) dwf_epilogue<PIN, DAG, N>(p, site, s0, acc);
    part = store_spinor<POUT, N>(p.out, p.out_norm, int64_t(site) * 12 * p.LsE + s0, int64_t(site) * p.LsE + s0,
                                 p.LsE, acc);
    if (POUT == GBDW_F64) dpart = sumsq<N>(acc);
  }
  if (p.partials) {
    double v[1] = {POUT == GBDW_F64 ? dpart : double(part)};
    grid_sum<1>(v, p.partials, p.counter, p.result);
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
  cpx<T> acc[1][12];
#pragma unroll
  for (int k = 0; k < 12; ++k) acc[0][k] = {T(0), T(0)};
  const uint32_t* nb = p.nbr5 + size_t(tid) * 8;
  const int64_t Ls = p.Ls;
#define GBDW_LEG(L)                                                                                   \
  {                                                                                                   \
    const int64_t n5 = __ldg(nb + L);                                                                 \
    const int64_t ns = n5 / Ls, sn = n5 - ns * Ls;                                                    \
    hop_leg<PIN, GP, DAG, 1, L>(p.U, size_t(site) * 8 + L, p.in, p.in_norm, ns * 12 * Ls + sn, n5, p.Ls, acc); \
  }
  GBDW_LEG(0) GBDW_LEG(1) GBDW_LEG(2) GBDW_LEG(3) GBDW_LEG(4) GBDW_LEG(5) GBDW_LEG(6) GBDW_LEG(7)
#undef GBDW_LEG
  store_spinor<PIN, 1>(p.out, p.out_norm, int64_t(site) * 12 * Ls + s, int64_t(site) * Ls + s, p.Ls, acc);
}

// ------------------------------------------------------------------ launch dispatch
struct DhopLaunch {
  int threads;     // per CTA (target; the staged kernel rounds to whole sites)
  int spt;         // slices per thread
  int mode = 0;    // 0: direct loads, 1: TMA-staged neighbour blocks
  int stages = 4;  // staged kernel: depth of the leg ring
};

// Implemented per precision family in dhop_f64.cu / dhop_f32.cu / dhop_f16.cu.
int launch_dhop_f64(const DhopParams& p, int dag, int epi, DhopLaunch L);
int launch_dhop_f32(const DhopParams& p, int dag, int epi, DhopLaunch L);
int launch_dhop_f16(const DhopParams& p, int gprec, int dag, int epi, DhopLaunch L);
int launch_dhop_general(const DhopParams& p, int prec, int dag);
// Sites per CTA and dynamic shared memory of the staged kernel, or false if it cannot run.
bool tma_shape(int prec, int LsE, DhopLaunch L, int* NS, int* threads, size_t* smem);

}  // namespace gbdw
