// BLAS-1 on spinor fields with FP64 global sums, and the fused vector updates of the
// conjugate-gradient solvers.  Each thread handles whole 5D entries (12 complex numbers of
// one (site, slice)), so F16 fields keep one norm per entry; consecutive threads take
// consecutive slices, so every component access of a warp is contiguous.  Sums accumulate
// each entry in the arithmetic precision and everything above an entry in FP64, followed by
// the fixed-order grid reduction of common.cuh.
#include "blas.h"
#include "common.cuh"
#include "dhop_kernel.cuh"
#include "layout.cuh"

#include <type_traits>

namespace gbdw {

namespace {

template <int P>
struct Calc {
  using T = float;
};
template <>
struct Calc<GBDW_F64> {
  using T = double;
};

template <int P, class T>
__device__ __forceinline__ void ld24(const void* d, const float* nrm, int64_t site, int e, int LsE, int LsP, T (&v)[24]) {
  const float n = (P == GBDW_F16) ? __ldg(nrm + site * LsE + e) : 1.f;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    const auto a = Elem<P>::ld(d, site * 12 + k, e, LsP);
    v[2 * k] = (P == GBDW_F16) ? T(float(a.r) * n) : T(a.r);
    v[2 * k + 1] = (P == GBDW_F16) ? T(float(a.i) * n) : T(a.i);
  }
}

// Stores v and returns the entry's |.|^2 as stored.
template <int P, class T>
__device__ __forceinline__ T st24(void* d, float* nrm, int64_t site, int e, int LsE, int LsP, const T (&v)[24]) {
  T s = T(0);
  if constexpr (P == GBDW_F16) {
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 24; ++k) m = fmaxf(m, fabsf(float(v[k])));
    const float sc = m > 0.f ? 1.f / m : 0.f;
    nrm[site * LsE + e] = m;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      const float2 f = __half22float2(__floats2half2_rn(float(v[2 * k]) * sc, float(v[2 * k + 1]) * sc));
      Elem<GBDW_F16>::st(d, site * 12 + k, e, LsP, f.x, f.y);
      s += T((f.x * f.x + f.y * f.y) * m * m);
    }
  } else {
    using S = typename std::conditional<P == GBDW_F64, double, float>::type;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      const S re = S(v[2 * k]), im = S(v[2 * k + 1]);
      Elem<P>::st(d, site * 12 + k, e, LsP, re, im);
      s += T(re) * T(re) + T(im) * T(im);
    }
  }
  return s;
}

struct FieldRef {
  const void* d;
  const float* n;
  int LsP;
};
struct FieldOut {
  void* d;
  float* n;
  int LsP;
};

template <int P>
__global__ void k_norm2(FieldRef x, int64_t nsite, int LsE, Reduce red) {
  using T = typename Calc<P>::T;
  double acc[1] = {0.0};
  const int64_t n = nsite * LsE;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / LsE;
    const int e = int(i - site * LsE);
    T v[24];
    ld24<P>(x.d, x.n, site, e, LsE, x.LsP, v);
    T s = T(0);
#pragma unroll
    for (int k = 0; k < 24; ++k) s += v[k] * v[k];
    acc[0] += double(s);
  }
  grid_sum<1>(acc, red.partials, red.counter, red.result);
}

template <int PX, int PY>
__global__ void k_dot(FieldRef x, FieldRef y, int64_t nsite, int LsE, Reduce red) {
  using T = typename Calc<(PX == GBDW_F64 || PY == GBDW_F64) ? GBDW_F64 : GBDW_F32>::T;
  double acc[2] = {0.0, 0.0};
  const int64_t n = nsite * LsE;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / LsE;
    const int e = int(i - site * LsE);
    T a[24], b[24];
    ld24<PX>(x.d, x.n, site, e, LsE, x.LsP, a);
    ld24<PY>(y.d, y.n, site, e, LsE, y.LsP, b);
    T re = T(0), im = T(0);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      re += a[2 * k] * b[2 * k] + a[2 * k + 1] * b[2 * k + 1];
      im += a[2 * k] * b[2 * k + 1] - a[2 * k + 1] * b[2 * k];
    }
    acc[0] += double(re);
    acc[1] += double(im);
  }
  grid_sum<2>(acc, red.partials, red.counter, red.result);
}

// y = a x + b y
template <int PX, int PY>
__global__ void k_axpby(double a, FieldRef x, double b, FieldOut y, int64_t nsite, int LsE) {
  using T = typename Calc<(PX == GBDW_F64 || PY == GBDW_F64) ? GBDW_F64 : GBDW_F32>::T;
  const int64_t n = nsite * LsE;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / LsE;
    const int e = int(i - site * LsE);
    T u[24], v[24];
    ld24<PX>(x.d, x.n, site, e, LsE, x.LsP, u);
    ld24<PY>(y.d, y.n, site, e, LsE, y.LsP, v);
#pragma unroll
    for (int k = 0; k < 24; ++k) v[k] = T(a) * u[k] + T(b) * v[k];
    st24<PY>(y.d, y.n, site, e, LsE, y.LsP, v);
  }
}

// r = b - t, |r|^2
template <int PB, int PT, int PR>
__global__ void k_xmy_norm(FieldRef b, FieldRef t, FieldOut r, int64_t nsite, int LsE, Reduce red) {
  using T = typename Calc<(PB == GBDW_F64 || PT == GBDW_F64 || PR == GBDW_F64) ? GBDW_F64 : GBDW_F32>::T;
  double acc[1] = {0.0};
  const int64_t n = nsite * LsE;
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / LsE;
    const int e = int(i - site * LsE);
    T u[24], v[24];
    ld24<PB>(b.d, b.n, site, e, LsE, b.LsP, u);
    ld24<PT>(t.d, t.n, site, e, LsE, t.LsP, v);
#pragma unroll
    for (int k = 0; k < 24; ++k) u[k] -= v[k];
    acc[0] += double(st24<PR>(r.d, r.n, site, e, LsE, r.LsP, u));
  }
  grid_sum<1>(acc, red.partials, red.counter, red.result);
}

// r -= alpha Ap ; |r|^2
template <int PR, int PA>
__global__ void k_cg_r(double alpha, FieldOut r, FieldRef ap, int64_t nsite, int LsE, Reduce red) {
  using T = typename Calc<PR>::T;
  double acc[1] = {0.0};
  const int64_t n = nsite * LsE;
  const T al = T(alpha);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / LsE;
    const int e = int(i - site * LsE);
    T u[24], v[24];
    ld24<PR>(r.d, r.n, site, e, LsE, r.LsP, u);
    ld24<PA>(ap.d, ap.n, site, e, LsE, ap.LsP, v);
#pragma unroll
    for (int k = 0; k < 24; ++k) u[k] -= al * v[k];
    acc[0] += double(st24<PR>(r.d, r.n, site, e, LsE, r.LsP, u));
  }
  grid_sum<1>(acc, red.partials, red.counter, red.result);
}

// x += alpha p ; p = r + beta p (both with the old p) ; optionally q = p
template <int PX, int PP, int PR, int PQ>
__global__ void k_cg_xp(double alpha, double beta, FieldOut x, FieldOut p, FieldRef r, FieldOut q, int64_t nsite,
                        int LsE) {
  using T = typename Calc<(PX == GBDW_F64 || PR == GBDW_F64) ? GBDW_F64 : GBDW_F32>::T;
  const int64_t n = nsite * LsE;
  const T al = T(alpha), be = T(beta);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / LsE;
    const int e = int(i - site * LsE);
    T u[24], v[24];
    ld24<PP>(p.d, p.n, site, e, LsE, p.LsP, v);
    ld24<PX>(x.d, x.n, site, e, LsE, x.LsP, u);
#pragma unroll
    for (int k = 0; k < 24; ++k) u[k] += al * v[k];
    st24<PX>(x.d, x.n, site, e, LsE, x.LsP, u);
    ld24<PR>(r.d, r.n, site, e, LsE, r.LsP, u);
#pragma unroll
    for (int k = 0; k < 24; ++k) v[k] = u[k] + be * v[k];
    st24<PP>(p.d, p.n, site, e, LsE, p.LsP, v);
    if (PQ >= 0) st24<PQ < 0 ? GBDW_F32 : PQ>(q.d, q.n, site, e, LsE, q.LsP, v);
  }
}

// p = r + beta p ; optionally q = p (a lower-precision copy that feeds the operator)
template <int PR, int PP, int PQ>
__global__ void k_cg_p(double beta, FieldRef r, FieldOut p, FieldOut q, int64_t nsite, int LsE) {
  using T = typename Calc<(PR == GBDW_F64 || PP == GBDW_F64) ? GBDW_F64 : GBDW_F32>::T;
  const int64_t n = nsite * LsE;
  const T be = T(beta);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / LsE;
    const int e = int(i - site * LsE);
    T u[24], v[24];
    ld24<PR>(r.d, r.n, site, e, LsE, r.LsP, u);
    ld24<PP>(p.d, p.n, site, e, LsE, p.LsP, v);
#pragma unroll
    for (int k = 0; k < 24; ++k) v[k] = u[k] + be * v[k];
    st24<PP>(p.d, p.n, site, e, LsE, p.LsP, v);
    if (PQ >= 0) st24<PQ < 0 ? GBDW_F32 : PQ>(q.d, q.n, site, e, LsE, q.LsP, v);
  }
}

FieldRef ref(const gbdw_field* f) { return FieldRef{f->d, f->norm, f->LsP}; }
FieldOut out(gbdw_field* f) { return FieldOut{f->d, f->norm, f->LsP}; }

constexpr int kThreads = 256;
int64_t grid_for(const gbdw_field* f) {
  const int64_t n = f->lat->nsite * f->LsE;
  int64_t g = (n + kThreads - 1) / kThreads;
  const int64_t cap = int64_t(num_sms()) * 8;
  return g < cap ? (g > 0 ? g : 1) : cap;
}

bool same_shape(const gbdw_field* a, const gbdw_field* b) { return a && b && a->lat == b->lat && a->nrhs == b->nrhs; }

// ------------------------------------------------------------------ slice-pair forms
// The hot CG updates on FP32/FP16 fields with an even slice count: one thread per (site, slice
// pair), 128-bit (FP32) / 64-bit (FP16) loads and stores of the paired layout, one norm pair per
// FP16 access; FP32 arithmetic as in the element-wise forms.
template <int P>
__device__ __forceinline__ void ld_pair(const void* d, const float* nrm, int64_t site, int e0, int LsE, int LsP,
                                        cpx<float> (&v)[2][12]) {
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    cpx<float> x[2];
    Vec<P, 2>::load(d, site * 12 + k, e0, LsP, x);
    v[0][k] = x[0];
    v[1][k] = x[1];
  }
  if constexpr (P == GBDW_F16) {
    float n[2];
    load_norms<2>(nrm, site * LsE + e0, n);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 12; ++k) v[j][k] = {v[j][k].r * n[j], v[j][k].i * n[j]};
  }
}

template <int PX, int PP, int PR>
__global__ void k_cg_xp_pairs(double alpha, double beta, FieldOut x, FieldOut p, FieldRef r, int64_t nsite, int LsE) {
  const int G = LsE / 2;
  const int64_t n = nsite * G;
  const float al = float(alpha), be = float(beta);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / G;
    const int e0 = int(i - site * G) * 2;
    cpx<float> u[2][12], v[2][12];
    ld_pair<PP>(p.d, p.n, site, e0, LsE, p.LsP, v);
    ld_pair<PX>(x.d, x.n, site, e0, LsE, x.LsP, u);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 12; ++k) u[j][k] = {fmaf(al, v[j][k].r, u[j][k].r), fmaf(al, v[j][k].i, u[j][k].i)};
    store_spinor<PX, 2>(x.d, x.n, site, e0, LsE, x.LsP, u);
    ld_pair<PR>(r.d, r.n, site, e0, LsE, r.LsP, u);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 12; ++k) v[j][k] = {fmaf(be, v[j][k].r, u[j][k].r), fmaf(be, v[j][k].i, u[j][k].i)};
    store_spinor<PP, 2>(p.d, p.n, site, e0, LsE, p.LsP, v);
  }
}

template <int PR, int PA>
__global__ void k_cg_r_pairs(double alpha, FieldOut r, FieldRef ap, int64_t nsite, int LsE, Reduce red) {
  double acc[1] = {0.0};
  const int G = LsE / 2;
  const int64_t n = nsite * G;
  const float al = float(alpha);
  for (int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
    const int64_t site = i / G;
    const int e0 = int(i - site * G) * 2;
    cpx<float> u[2][12], v[2][12];
    ld_pair<PR>(r.d, r.n, site, e0, LsE, r.LsP, u);
    ld_pair<PA>(ap.d, ap.n, site, e0, LsE, ap.LsP, v);
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int k = 0; k < 12; ++k) u[j][k] = {fmaf(-al, v[j][k].r, u[j][k].r), fmaf(-al, v[j][k].i, u[j][k].i)};
    acc[0] += double(store_spinor<PR, 2>(r.d, r.n, site, e0, LsE, r.LsP, u));
  }
  grid_sum<1>(acc, red.partials, red.counter, red.result);
}

bool pairs_ok(const gbdw_field* f) { return f->prec != GBDW_F64 && f->LsE % 2 == 0 && f->LsP == f->LsE; }

int64_t grid_pairs(const gbdw_field* f) {
  const int64_t n = f->lat->nsite * (f->LsE / 2);
  int64_t g = (n + kThreads - 1) / kThreads;
  const int64_t cap = int64_t(num_sms()) * 8;
  return g < cap ? (g > 0 ? g : 1) : cap;
}

}  // namespace

// ------------------------------------------------------------------ internal entry points

int blas_norm2(const gbdw_field* x, double* out, bool fetch) {
  const int64_t g = grid_for(x);
  Reduce red;
  if (int st = reduce_scratch(g, 1, &red)) return st;
  const int64_t ns = x->lat->nsite;
  const int L = x->LsE;
  switch (x->prec) {
    case GBDW_F64: k_norm2<GBDW_F64><<<unsigned(g), kThreads, 0, stream()>>>(ref(x), ns, L, red); break;
    case GBDW_F32: k_norm2<GBDW_F32><<<unsigned(g), kThreads, 0, stream()>>>(ref(x), ns, L, red); break;
    default: k_norm2<GBDW_F16><<<unsigned(g), kThreads, 0, stream()>>>(ref(x), ns, L, red); break;
  }
  GBDW_LAUNCHED();
  return fetch ? reduce_fetch(red, 1, out) : GBDW_OK;
}

int blas_xmy_norm(const gbdw_field* b, const gbdw_field* t, gbdw_field* r, double* rr) {
  if (b->prec != GBDW_F64 || r->prec != GBDW_F64 || (t->prec != GBDW_F64 && t->prec != GBDW_F32)) {
    set_error("blas_xmy_norm: b and r must be F64, t F64 or F32");
    return GBDW_ERR_INVALID;
  }
  const int64_t g = grid_for(r);
  Reduce red;
  if (int st = reduce_scratch(g, 1, &red)) return st;
  const int64_t ns = r->lat->nsite;
  const int L = r->LsE;
  if (t->prec == GBDW_F64)
    k_xmy_norm<GBDW_F64, GBDW_F64, GBDW_F64><<<unsigned(g), kThreads, 0, stream()>>>(ref(b), ref(t), out(r), ns, L, red);
  else
    k_xmy_norm<GBDW_F64, GBDW_F32, GBDW_F64><<<unsigned(g), kThreads, 0, stream()>>>(ref(b), ref(t), out(r), ns, L, red);
  GBDW_LAUNCHED();
  return reduce_fetch(red, 1, rr);
}

int blas_cg_r(double alpha, gbdw_field* r, const gbdw_field* ap, double* rr) {
  const int64_t ns = r->lat->nsite;
  const int L = r->LsE;
  if (pairs_ok(r) && pairs_ok(ap)) {
    const int64_t g = grid_pairs(r);
    Reduce red;
    if (int st = reduce_scratch(g, 1, &red)) return st;
    const int key = r->prec * 4 + ap->prec;
    if (key == GBDW_F32 * 4 + GBDW_F32)
      k_cg_r_pairs<GBDW_F32, GBDW_F32><<<unsigned(g), kThreads, 0, stream()>>>(alpha, out(r), ref(ap), ns, L, red);
    else if (key == GBDW_F32 * 4 + GBDW_F16)
      k_cg_r_pairs<GBDW_F32, GBDW_F16><<<unsigned(g), kThreads, 0, stream()>>>(alpha, out(r), ref(ap), ns, L, red);
    else if (key == GBDW_F16 * 4 + GBDW_F16)
      k_cg_r_pairs<GBDW_F16, GBDW_F16><<<unsigned(g), kThreads, 0, stream()>>>(alpha, out(r), ref(ap), ns, L, red);
    else {
      set_error("blas_cg_r: unsupported precision combination");
      return GBDW_ERR_INVALID;
    }
    GBDW_LAUNCHED();
    return reduce_fetch(red, 1, rr);
  }
  const int64_t g = grid_for(r);
  Reduce red;
  if (int st = reduce_scratch(g, 1, &red)) return st;
  const int key = r->prec * 4 + ap->prec;
#define GBDW_R(PR, PA)                                                                                  \
  case PR * 4 + PA:                                                                                     \
    k_cg_r<PR, PA><<<unsigned(g), kThreads, 0, stream()>>>(alpha, out(r), ref(ap), ns, L, red);         \
    break;
  switch (key) {
    GBDW_R(GBDW_F64, GBDW_F64)  // FP64 solve
    GBDW_R(GBDW_F64, GBDW_F32)  // plain: FP64 vectors, FP32 operator
    GBDW_R(GBDW_F32, GBDW_F16)  // mixed, FP16 sloppy
    GBDW_R(GBDW_F32, GBDW_F32)  // mixed, FP32 sloppy
    GBDW_R(GBDW_F16, GBDW_F16)  // mixed, FP16 sloppy with an FP16 iterated residual
    default:
      set_error("blas_cg_r: unsupported precision combination");
      return GBDW_ERR_INVALID;
  }
#undef GBDW_R
  GBDW_LAUNCHED();
  return reduce_fetch(red, 1, rr);
}

int blas_cg_xp(double alpha, double beta, gbdw_field* x, gbdw_field* p, const gbdw_field* r, gbdw_field* q) {
  const int64_t ns = r->lat->nsite;
  const int L = r->LsE;
  if (!q && pairs_ok(x) && pairs_ok(p) && pairs_ok(r) && x->prec == GBDW_F32) {
    const unsigned g = unsigned(grid_pairs(r));
    if (p->prec == GBDW_F16 && r->prec == GBDW_F16)
      k_cg_xp_pairs<GBDW_F32, GBDW_F16, GBDW_F16><<<g, kThreads, 0, stream()>>>(alpha, beta, out(x), out(p), ref(r), ns, L);
    else if (p->prec == GBDW_F16 && r->prec == GBDW_F32)
      k_cg_xp_pairs<GBDW_F32, GBDW_F16, GBDW_F32><<<g, kThreads, 0, stream()>>>(alpha, beta, out(x), out(p), ref(r), ns, L);
    else if (p->prec == GBDW_F32 && r->prec == GBDW_F32)
      k_cg_xp_pairs<GBDW_F32, GBDW_F32, GBDW_F32><<<g, kThreads, 0, stream()>>>(alpha, beta, out(x), out(p), ref(r), ns, L);
    else {
      set_error("blas_cg_xp: unsupported precision combination");
      return GBDW_ERR_INVALID;
    }
    GBDW_LAUNCHED();
    return GBDW_OK;
  }
  const int64_t g = grid_for(r);
  const int qp = q ? q->prec : -1;
  FieldOut qo = q ? out(q) : FieldOut{nullptr, nullptr, 0};
  const int key = ((x->prec * 4 + p->prec) * 4 + r->prec) * 8 + (qp + 1);
#define GBDW_XP(PX, PP, PR, PQ)                                                                              \
  case ((PX * 4 + PP) * 4 + PR) * 8 + (PQ + 1):                                                              \
    k_cg_xp<PX, PP, PR, PQ><<<unsigned(g), kThreads, 0, stream()>>>(alpha, beta, out(x), out(p), ref(r), qo, ns, L); \
    break;
  switch (key) {
    GBDW_XP(GBDW_F64, GBDW_F64, GBDW_F64, -1)
    GBDW_XP(GBDW_F64, GBDW_F64, GBDW_F64, GBDW_F32)
    GBDW_XP(GBDW_F32, GBDW_F16, GBDW_F32, -1)
    GBDW_XP(GBDW_F32, GBDW_F32, GBDW_F32, -1)
    GBDW_XP(GBDW_F32, GBDW_F16, GBDW_F16, -1)
    default:
      set_error("blas_cg_xp: unsupported precision combination");
      return GBDW_ERR_INVALID;
  }
#undef GBDW_XP
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int blas_cg_p(double beta, const gbdw_field* r, gbdw_field* p, gbdw_field* q) {
  const int64_t g = grid_for(r);
  const int64_t ns = r->lat->nsite;
  const int L = r->LsE;
  const int qp = q ? q->prec : -1;
  FieldOut qo = q ? out(q) : FieldOut{nullptr, nullptr, 0};
  const int key = (r->prec * 4 + p->prec) * 8 + (qp + 1);
#define GBDW_P(PR, PP, PQ)                                                                             \
  case (PR * 4 + PP) * 8 + (PQ + 1):                                                                   \
    k_cg_p<PR, PP, PQ><<<unsigned(g), kThreads, 0, stream()>>>(beta, ref(r), out(p), qo, ns, L);      \
    break;
  switch (key) {
    GBDW_P(GBDW_F64, GBDW_F64, -1)
    GBDW_P(GBDW_F64, GBDW_F64, GBDW_F32)
    GBDW_P(GBDW_F32, GBDW_F16, -1)
    GBDW_P(GBDW_F32, GBDW_F32, -1)
    GBDW_P(GBDW_F16, GBDW_F16, -1)
    default:
      set_error("blas_cg_p: unsupported precision combination");
      return GBDW_ERR_INVALID;
  }
#undef GBDW_P
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int blas_axpby(double a, const gbdw_field* x, double b, gbdw_field* y) {
  const int64_t g = grid_for(y);
  const int64_t ns = y->lat->nsite;
  const int L = y->LsE;
  const int key = x->prec * 4 + y->prec;
#define GBDW_AX(PX, PY) \
  case PX * 4 + PY: k_axpby<PX, PY><<<unsigned(g), kThreads, 0, stream()>>>(a, ref(x), b, out(y), ns, L); break;
  switch (key) {
    GBDW_AX(GBDW_F64, GBDW_F64)
    GBDW_AX(GBDW_F32, GBDW_F64)
    GBDW_AX(GBDW_F16, GBDW_F64)
    GBDW_AX(GBDW_F64, GBDW_F32)
    GBDW_AX(GBDW_F32, GBDW_F32)
    GBDW_AX(GBDW_F16, GBDW_F32)
    GBDW_AX(GBDW_F32, GBDW_F16)
    GBDW_AX(GBDW_F16, GBDW_F16)
    default:
      set_error("axpby: unsupported precision combination");
      return GBDW_ERR_INVALID;
  }
#undef GBDW_AX
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int blas_dot(const gbdw_field* x, const gbdw_field* y, double* re, double* im) {
  const int64_t g = grid_for(x);
  Reduce red;
  if (int st = reduce_scratch(g, 2, &red)) return st;
  const int64_t ns = x->lat->nsite;
  const int L = x->LsE;
  const int key = x->prec * 4 + y->prec;
#define GBDW_DOT(PX, PY) \
  case PX * 4 + PY: k_dot<PX, PY><<<unsigned(g), kThreads, 0, stream()>>>(ref(x), ref(y), ns, L, red); break;
  switch (key) {
    GBDW_DOT(GBDW_F64, GBDW_F64)
    GBDW_DOT(GBDW_F32, GBDW_F32)
    GBDW_DOT(GBDW_F16, GBDW_F16)
    GBDW_DOT(GBDW_F64, GBDW_F32)
    GBDW_DOT(GBDW_F32, GBDW_F64)
    default:
      set_error("dot: unsupported precision combination");
      return GBDW_ERR_INVALID;
  }
#undef GBDW_DOT
  GBDW_LAUNCHED();
  double v[2];
  if (int st = reduce_fetch(red, 2, v)) return st;
  if (re) *re = v[0];
  if (im) *im = v[1];
  return GBDW_OK;
}

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_norm2(const gbdw_field* x, double* out) {
  if (!x || !out) return GBDW_ERR_INVALID;
  if (int st = ensure_device()) return st;
  return blas_norm2(x, out, true);
}

int gbdw_dot(const gbdw_field* x, const gbdw_field* y, double* re, double* im) {
  if (!same_shape(x, y)) {
    set_error("gbdw_dot: fields must share lattice and nrhs");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  return blas_dot(x, y, re, im);
}

int gbdw_axpby(double a, const gbdw_field* x, double b, gbdw_field* y) {
  if (!same_shape(x, y)) {
    set_error("gbdw_axpby: fields must share lattice and nrhs");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  return blas_axpby(a, x, b, y);
}

}  // extern "C"
