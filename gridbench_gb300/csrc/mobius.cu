// Mobius (Cayley-form) domain-wall fermions around the hopping term: the generic 5th-dimension
// operator M5D, its adjoint and inverse, and the Mobius operator built from them.  GridBench
// has no 5th-dimension operators; these follow Grid's CayleyFermion5D structure (M5D /
// M5Ddag / Mooee / MooeeInv / Meooe around WilsonFermion5D's Dhop, the library GridBench's
// TableGenerate.cc:8 links against; un-vendored, no version pinned) and the Mobius kernel of
// Brower, Neff and Orginos (arXiv:1206.5214), restated here in this library's conventions.
//
// A cyclic 5th-dimension operator with per-slice real coefficients (lower, diag, upper):
//     (A psi)(s) = diag[s] psi(s) + upper[s] P- psi(s+1) + lower[s] P+ psi(s-1),
// s+1 and s-1 taken mod Ls (the wall factors live in upper[Ls-1] and lower[0]);
// P+- = (1 +- gamma5)/2 with gamma5 = diag(1,1,-1,-1) in GridBench's chiral basis, so P+ keeps
// spins 0,1 and P- spins 2,3.  Its adjoint with the same arrays is
//     (A^dag psi)(s) = diag[s] psi(s) + upper[s-1] P- psi(s-1) + lower[s+1] P+ psi(s+1).
// (Grid's M5Ddag takes pre-shifted arrays; here dag = 1 always means the exact adjoint.)
//
// The Mobius operator with parameters (b, c, M5, mf):
//     M = Mooee + Meooe,   Mooee = A(bee, -cee),   Meooe = -1/2 Dhop . A(b, c),
//     bee = 1 + b (4 - M5),   cee = 1 - c (4 - M5),
// where A(d, e) has diag d, lower = upper = e and the walls e -> -mf e.  b = 1, c = 0 gives
// bee = 5 - M5, cee = 1, A(b, c) = 1: the Shamir operator of dhop.cu.
//   M^dag = Mooee^dag - 1/2 A(b, c)^dag DhopDag.
//
// Kernels: k_m5d (out = A x [+ B y], one thread per 4D site and N slices, every operand read
// once: HBM bound, 2 spinors per 5D site per operand) and k_m5d_inv (A^-1 as two cyclic
// bidiagonal solves per chirality, O(Ls) per row, the same two-phase shared-memory tile as the
// Shamir D5^-1 in eo.cu).  With one right-hand side and Ls a power of two, M^dag is a single
// hopping pass in every precision (A(b, c)^dag applied to the hopping result in the epilogue),
// and so is M for FP32 fields (A(b, c) applied to the neighbours' slices as they are loaded);
// the neighbouring slices are taken by shuffles from the lanes of the same site (dhop_kernel.cuh).
#include <cmath>
#include <string>

#include "blas.h"
#include "common.cuh"
#include "dhop_kernel.cuh"
#include "eo.h"
#include "layout.cuh"
#include "tune.h"

namespace gbdw {

namespace {

inline unsigned nblk(int64_t n, int t) { return unsigned((n + t - 1) / t); }

constexpr int kMaxLs5 = 64;

struct Coef5 {
  double lower[kMaxLs5];  // on P+ psi(s-1)
  double diag[kMaxLs5];
  double upper[kMaxLs5];  // on P- psi(s+1)
};

struct M5DParams {
  const void* x;
  const float* x_norm;
  const void* y;  // second operand (two-operand launches only)
  const float* y_norm;
  void* out;
  float* out_norm;
  int64_t nsite;
  int Ls;
  int LsP;
  Coef5 a, b;
};

// acc (+)= A v for the N slices s0.. of one 4D site.  Rows 0-5 are spins 0,1 (P+), rows 6-11
// spins 2,3 (P-).  dag = 0: P+ rows take psi(s-1) x lower[s], P- rows psi(s+1) x upper[s];
// dag = 1: P- rows take psi(s-1) x upper[s-1], P+ rows psi(s+1) x lower[s+1].
template <int P, int DAG, int N, bool ADD>
__device__ __forceinline__ void apply5(const Coef5& c, const void* v, const float* vn, int64_t site, int s0, int Ls,
                                       int LsP, cpx<typename Arith<P>::T> (&acc)[N][12]) {
  using T = typename Arith<P>::T;
  const int64_t row0 = site * 12;
  cpx<T> cen[N][12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    cpx<T> x[N];
    Vec<P, N>::load(v, row0 + k, s0, LsP, x);
#pragma unroll
    for (int j = 0; j < N; ++j) cen[j][k] = x[j];
  }
  const int slo = (s0 == 0) ? Ls - 1 : s0 - 1;
  const int shi = (s0 + N == Ls) ? 0 : s0 + N;
  constexpr int LO0 = DAG ? 6 : 0;  // first row fed by psi(s-1)
  constexpr int HI0 = DAG ? 0 : 6;  // first row fed by psi(s+1)
  cpx<T> lo[6], hi[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    lo[k] = Elem<P>::ld(v, row0 + LO0 + k, slo, LsP);
    hi[k] = Elem<P>::ld(v, row0 + HI0 + k, shi, LsP);
  }
  if constexpr (P == GBDW_F16) {
    float nc[N];
    load_norms<N>(vn, site * Ls + s0, nc);
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int k = 0; k < 12; ++k) cen[j][k] = {cen[j][k].r * nc[j], cen[j][k].i * nc[j]};
    const float nl = __ldg(vn + site * Ls + slo), nh = __ldg(vn + site * Ls + shi);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      lo[k] = {lo[k].r * nl, lo[k].i * nl};
      hi[k] = {hi[k].r * nh, hi[k].i * nh};
    }
  }
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const int s = s0 + j;
    const int sm = (s == 0) ? Ls - 1 : s - 1, sp = (s + 1 == Ls) ? 0 : s + 1;
    const T d = T(c.diag[s]);
    const T el = DAG ? T(c.upper[sm]) : T(c.lower[s]);  // on the row fed by psi(s-1)
    const T eh = DAG ? T(c.lower[sp]) : T(c.upper[s]);  // on the row fed by psi(s+1)
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      cpx<T> w = {d * cen[j][k].r, d * cen[j][k].i};
      if (k >= LO0 && k < LO0 + 6) {
        const cpx<T> m = (j == 0) ? lo[k - LO0] : cen[j == 0 ? 0 : j - 1][k];
        w.r += el * m.r;
        w.i += el * m.i;
      } else {
        const cpx<T> q = (j == N - 1) ? hi[k - HI0] : cen[j + 1 >= N ? N - 1 : j + 1][k];
        w.r += eh * q.r;
        w.i += eh * q.i;
      }
      if constexpr (ADD) {
        acc[j][k].r += w.r;
        acc[j][k].i += w.i;
      } else {
        acc[j][k] = w;
      }
    }
  }
}

template <int P, int DAG, int N, bool TWO>
__global__ void __launch_bounds__(128) k_m5d(const __grid_constant__ M5DParams p) {
  using T = typename Arith<P>::T;
  const int G = p.Ls / N;
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= p.nsite * G) return;
  const int64_t site = i / G;
  const int s0 = int(i - site * G) * N;
  cpx<T> acc[N][12];
  apply5<P, DAG, N, false>(p.a, p.x, p.x_norm, site, s0, p.Ls, p.LsP, acc);
  if constexpr (TWO) apply5<P, DAG, N, true>(p.b, p.y, p.y_norm, site, s0, p.Ls, p.LsP, acc);
  store_spinor<P, N>(p.out, p.out_norm, site, s0, p.Ls, p.LsP, acc);
}

// One chirality's cyclic bidiagonal system  d[s] y(s) + e[s] y(s -+ 1) = x(s).  With the
// wrap unknown w (y(Ls-1) for the down sweep, y(0) for the up sweep) every y(s) = a(s) +
// B[s] w, a(s) = x(s)/d[s] - (e[s]/d[s]) a(s -+ 1) from the open end, B[s] = -(e[s]/d[s])
// B[s -+ 1] from B = -e/d there; then w = a(end) / (1 - B[end]).
struct Inv5 {
  double id[kMaxLs5];  // 1 / d[s]
  double ed[kMaxLs5];  // e[s] / d[s]
  double B[kMaxLs5];
  double w;            // 1 / (1 - B[end])
};

struct M5DInvParams {
  const void* in;
  const float* in_norm;
  void* out;
  float* out_norm;
  int64_t nsite;
  int Ls;
  int LsP;
  int nsb;  // sites per CTA
  Inv5 down, up;
};

template <int P, int DAG, int N>
__global__ void __launch_bounds__(192) k_m5d_inv(const __grid_constant__ M5DInvParams p) {
  using T = typename Arith<P>::T;
  extern __shared__ __align__(16) unsigned char m5d_smem[];
  cpx<T>* tile = reinterpret_cast<cpx<T>*>(m5d_smem);  // [nsb][12][Ls + 1]
  const int Ls = p.Ls, LsT = Ls + 1;
  const int64_t site0 = int64_t(blockIdx.x) * p.nsb;
  if (threadIdx.x < 12 * p.nsb) {
    const int ls = threadIdx.x / 12, row = threadIdx.x - 12 * (threadIdx.x / 12);
    const int64_t site = site0 + ls;
    if (site < p.nsite) {
      const int64_t r = site * 12 + row;
      cpx<T>* y = tile + (ls * 12 + row) * LsT;
      auto x = [&](int t) -> cpx<T> {
        cpx<T> e = Elem<P>::ld(p.in, r, t, p.LsP);
        if constexpr (P == GBDW_F16) {
          const float n = __ldg(p.in_norm + site * Ls + t);
          e = {e.r * n, e.i * n};
        }
        return e;
      };
      const bool down = (row < 6) != (DAG != 0);  // psi(s-1) feeds s
      if (down) {
        const Inv5& c = p.down;
        cpx<T> a = x(0);
        a = {a.r * T(c.id[0]), a.i * T(c.id[0])};
        y[0] = a;
        for (int t = 1; t < Ls; ++t) {
          const cpx<T> v = x(t);
          const T id = T(c.id[t]), ed = T(c.ed[t]);
          a = {v.r * id - ed * a.r, v.i * id - ed * a.i};
          y[t] = a;
        }
        const cpx<T> w = {a.r * T(c.w), a.i * T(c.w)};
        for (int t = 0; t < Ls; ++t) {
          const T B = T(c.B[t]);
          y[t] = {y[t].r + B * w.r, y[t].i + B * w.i};
        }
      } else {
        const Inv5& c = p.up;
        cpx<T> a = x(Ls - 1);
        a = {a.r * T(c.id[Ls - 1]), a.i * T(c.id[Ls - 1])};
        y[Ls - 1] = a;
        for (int t = Ls - 2; t >= 0; --t) {
          const cpx<T> v = x(t);
          const T id = T(c.id[t]), ed = T(c.ed[t]);
          a = {v.r * id - ed * a.r, v.i * id - ed * a.i};
          y[t] = a;
        }
        const cpx<T> w = {a.r * T(c.w), a.i * T(c.w)};
        for (int t = 0; t < Ls; ++t) {
          const T B = T(c.B[t]);
          y[t] = {y[t].r + B * w.r, y[t].i + B * w.i};
        }
      }
    }
  }
  __syncthreads();
  const int G = Ls / N;
  for (int it = threadIdx.x; it < p.nsb * G; it += blockDim.x) {
    const int ls = it / G;
    const int64_t site = site0 + ls;
    if (site >= p.nsite) break;
    const int s0 = (it - ls * G) * N;
    cpx<T> v[N][12];
#pragma unroll
    for (int k = 0; k < 12; ++k)
#pragma unroll
      for (int j = 0; j < N; ++j) v[j][k] = tile[(ls * 12 + k) * LsT + s0 + j];
    store_spinor<P, N>(p.out, p.out_norm, site, s0, Ls, p.LsP, v);
  }
}

bool same_shape(const gbdw_field* a, const gbdw_field* b) {
  return a && b && a->lat == b->lat && a->prec == b->prec && a->nrhs == 1 && b->nrhs == 1;
}

// Builds the down / up solves of A (dag = 0) or A^dag (dag = 1); false when singular.
bool inv_tables(const Coef5& c, int Ls, int dag, Inv5* down, Inv5* up) {
  double ed_[kMaxLs5], eu_[kMaxLs5];
  for (int s = 0; s < Ls; ++s) {
    const int sm = (s + Ls - 1) % Ls, sp = (s + 1) % Ls;
    ed_[s] = dag ? c.upper[sm] : c.lower[s];  // row fed by y(s-1)
    eu_[s] = dag ? c.lower[sp] : c.upper[s];  // row fed by y(s+1)
  }
  for (int s = 0; s < Ls; ++s) {
    if (!(std::fabs(c.diag[s]) > 0.0) || !std::isfinite(c.diag[s])) return false;
    down->id[s] = up->id[s] = 1.0 / c.diag[s];
    down->ed[s] = ed_[s] / c.diag[s];
    up->ed[s] = eu_[s] / c.diag[s];
  }
  down->B[0] = -down->ed[0];
  for (int s = 1; s < Ls; ++s) down->B[s] = -down->ed[s] * down->B[s - 1];
  up->B[Ls - 1] = -up->ed[Ls - 1];
  for (int s = Ls - 2; s >= 0; --s) up->B[s] = -up->ed[s] * up->B[s + 1];
  const double dd = 1.0 - down->B[Ls - 1], du = 1.0 - up->B[0];
  if (!(std::fabs(dd) > 1e-300) || !(std::fabs(du) > 1e-300) || !std::isfinite(dd) || !std::isfinite(du)) return false;
  down->w = 1.0 / dd;
  up->w = 1.0 / du;
  return true;
}

}  // namespace

// out = A x (+ B y when y is non-null), dag: the adjoints.
int m5d(gbdw_field* out, const gbdw_field* x, const Coef5& a, const gbdw_field* y, const Coef5* b, int dag) {
  if (!same_shape(out, x) || out == x || (y && (!same_shape(out, y) || out == y || !b))) {
    set_error("5th-dimension operator: distinct single-rhs fields of one lattice and precision");
    return GBDW_ERR_INVALID;
  }
  const int Ls = x->lat->Ls;
  if (Ls < 1 || Ls > kMaxLs5) {
    set_error("5th-dimension operator: needs 1 <= Ls <= 64");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  M5DParams p;
  p.x = x->d;
  p.x_norm = x->norm;
  p.y = y ? y->d : nullptr;
  p.y_norm = y ? y->norm : nullptr;
  p.out = out->d;
  p.out_norm = out->norm;
  p.nsite = x->lat->nsite;
  p.Ls = Ls;
  p.LsP = x->LsP;
  p.a = a;
  if (b) p.b = *b;
  const bool pair = Ls % 2 == 0;
  const int64_t n = p.nsite * (pair ? Ls / 2 : Ls);
  const unsigned g = nblk(n, 128);
#define GBDW_M5D_N(P, N)                                                          \
  if (y) {                                                                        \
    if (dag) k_m5d<P, 1, N, true><<<g, 128, 0, stream()>>>(p);                    \
    else k_m5d<P, 0, N, true><<<g, 128, 0, stream()>>>(p);                        \
  } else {                                                                        \
    if (dag) k_m5d<P, 1, N, false><<<g, 128, 0, stream()>>>(p);                   \
    else k_m5d<P, 0, N, false><<<g, 128, 0, stream()>>>(p);                       \
  }
#define GBDW_M5D(P)      \
  if (pair) {            \
    GBDW_M5D_N(P, 2)     \
  } else {               \
    GBDW_M5D_N(P, 1)     \
  }
  if (x->prec == GBDW_F64) {
    GBDW_M5D(GBDW_F64)
  } else if (x->prec == GBDW_F32) {
    GBDW_M5D(GBDW_F32)
  } else {
    GBDW_M5D(GBDW_F16)
  }
#undef GBDW_M5D
#undef GBDW_M5D_N
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int m5d_inv(gbdw_field* out, const gbdw_field* in, const Coef5& a, int dag) {
  if (!same_shape(out, in) || out == in) {
    set_error("5th-dimension inverse: distinct single-rhs fields of one lattice and precision");
    return GBDW_ERR_INVALID;
  }
  const int Ls = in->lat->Ls;
  if (Ls < 1 || Ls > kMaxLs5) {
    set_error("5th-dimension inverse: needs 1 <= Ls <= 64");
    return GBDW_ERR_INVALID;
  }
  M5DInvParams p;
  if (!inv_tables(a, Ls, dag, &p.down, &p.up)) {
    set_error("5th-dimension inverse: the operator is singular for these coefficients");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  p.in = in->d;
  p.in_norm = in->norm;
  p.out = out->d;
  p.out_norm = out->norm;
  p.nsite = in->lat->nsite;
  p.Ls = Ls;
  p.LsP = in->LsP;
  const size_t per_site = 12 * size_t(Ls + 1) * (in->prec == GBDW_F64 ? 16 : 8);
  p.nsb = int(std::min<size_t>(16, 49152 / per_site));
  const size_t smem = size_t(p.nsb) * per_site;
  const unsigned g = nblk(p.nsite, p.nsb);
  const int threads = 12 * p.nsb;
  const bool pair = Ls % 2 == 0;
#define GBDW_M5I(P)                                                              \
  if (pair) {                                                                    \
    if (dag) k_m5d_inv<P, 1, 2><<<g, threads, smem, stream()>>>(p);             \
    else k_m5d_inv<P, 0, 2><<<g, threads, smem, stream()>>>(p);                 \
  } else {                                                                       \
    if (dag) k_m5d_inv<P, 1, 1><<<g, threads, smem, stream()>>>(p);             \
    else k_m5d_inv<P, 0, 1><<<g, threads, smem, stream()>>>(p);                 \
  }
  if (in->prec == GBDW_F64) {
    GBDW_M5I(GBDW_F64)
  } else if (in->prec == GBDW_F32) {
    GBDW_M5I(GBDW_F32)
  } else {
    GBDW_M5I(GBDW_F16)
  }
#undef GBDW_M5I
  GBDW_LAUNCHED();
  return GBDW_OK;
}

namespace {

struct Mobius {
  double b, c, M5, mf;
  double bee() const { return 1.0 + b * (4.0 - M5); }
  double cee() const { return 1.0 - c * (4.0 - M5); }
};

bool read_coef(Coef5* c, int Ls, const double* lower, const double* diag, const double* upper) {
  if (!lower || !diag || !upper || Ls < 1 || Ls > kMaxLs5) return false;
  for (int s = 0; s < Ls; ++s) {
    c->lower[s] = lower[s];
    c->diag[s] = diag[s];
    c->upper[s] = upper[s];
    if (!std::isfinite(lower[s]) || !std::isfinite(diag[s]) || !std::isfinite(upper[s])) return false;
  }
  return true;
}

// A(d, e) with the walls e -> -mf e, times `scale`
Coef5 cyclic(int Ls, double d, double e, double mf, double scale) {
  Coef5 c;
  for (int s = 0; s < Ls; ++s) {
    c.diag[s] = scale * d;
    c.lower[s] = scale * e;
    c.upper[s] = scale * e;
  }
  c.upper[Ls - 1] = -mf * scale * e;
  c.lower[0] = -mf * scale * e;
  return c;
}

Coef5 mooee(int Ls, const Mobius& m) { return cyclic(Ls, m.bee(), -m.cee(), m.mf, 1.0); }
Coef5 meo5(int Ls, const Mobius& m, double scale) { return cyclic(Ls, m.b, m.c, m.mf, scale); }

bool check_mobius(const Mobius& m) {
  if (!std::isfinite(m.b) || !std::isfinite(m.c) || !std::isfinite(m.M5) || !std::isfinite(m.mf)) {
    set_error("Mobius operator: non-finite parameter");
    return false;
  }
  return true;
}

int check_ls(const gbdw_field* f) {
  if (!f || f->lat->Ls < 1 || f->lat->Ls > kMaxLs5) {
    set_error("Mobius operator: needs 1 <= Ls <= 64");
    return GBDW_ERR_INVALID;
  }
  return GBDW_OK;
}

// Full lattice: out = M in (dag 0) or M^dag in (dag 1); tmp a field like in.
int mobius_m(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, const Mobius& m, int dag,
             double* norm2) {
  if (int st = check_operands(g, out, in, true)) return st;
  if (int st = check_operands(g, tmp, in, true)) return st;
  if (tmp == out) {
    set_error("Mobius operator: tmp must differ from out");
    return GBDW_ERR_INVALID;
  }
  if (!check_mobius(m)) return GBDW_ERR_INVALID;
  if (int st = check_ls(in)) return st;
  const int Ls = in->lat->Ls;
  if (mobius_fusable(g, in, dag)) {
    // one pass: M in = Mooee in - 1/2 Dhop A(b, c) in with A applied to each neighbour's slices
    // as they are loaded (dag 0), or M^dag in = Mooee^dag in - 1/2 A(b, c)^dag DhopDag in with
    // A^dag applied in the epilogue (dag 1)
    DhopExtra ex;
    ex.c5 = m.cee();
    ex.mobius = true;
    ex.mb = m.b;
    ex.mc = m.c;
    return run_dhop(g, out, in, dag, 1, m.bee(), m.mf, norm2, true, nullptr, 0.5, &ex);
  }
  if (!dag) {
    // tmp = A(b, c) in;  out = Mooee in - 1/2 Dhop tmp  (the hopping epilogue with a5 = bee, c5 = cee)
    if (int st = m5d(tmp, in, meo5(Ls, m, 1.0), nullptr, nullptr, 0)) return st;
    DhopExtra ex;
    ex.c5 = m.cee();
    return run_dhop(g, out, tmp, 0, 1, m.bee(), m.mf, norm2, true, in, 0.5, &ex);
  }
  // tmp = DhopDag in;  out = Mooee^dag in + (-1/2 A(b, c))^dag tmp
  if (int st = run_dhop(g, tmp, in, 1, 0, 0.0, 0.0, nullptr)) return st;
  const Coef5 b5 = meo5(Ls, m, -0.5);
  if (int st = m5d(out, in, mooee(Ls, m), tmp, &b5, 1)) return st;
  if (norm2) return blas_norm2(out, norm2, true);
  return GBDW_OK;
}

// Even-odd hopping block on half p: out = -1/2 Dhop_pq A(b, c) in (dag 0, in on half q, tmp on
// half q) or out = -1/2 A(b, c)^dag DhopDag_pq in (dag 1, tmp on half p).
int mobius_meooe(const gbdw_gauge* gp, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, const Mobius& m,
                 int dag) {
  if (!gp || !out || !tmp || !in || tmp == out || tmp == in) {
    set_error("Mobius Meooe: null or aliased operands");
    return GBDW_ERR_INVALID;
  }
  if (!check_mobius(m)) return GBDW_ERR_INVALID;
  if (int st = check_ls(in)) return st;
  const int Ls = in->lat->Ls;
  if (!dag) {
    if (int st = m5d(tmp, in, meo5(Ls, m, -0.5), nullptr, nullptr, 0)) return st;
    return hop_eo(gp, out, tmp, 0, nullptr, 0.0, 0.0, 0.5, nullptr, true);
  }
  if (int st = hop_eo(gp, tmp, in, 1, nullptr, 0.0, 0.0, 0.5, nullptr, true)) return st;
  return m5d(out, tmp, meo5(Ls, m, -0.5), nullptr, nullptr, 1);
}

// Schur operator on half p:  Mpc = Mooee - Meooe_pq Mooee^-1 Meooe_qp  (dag: its adjoint).
// tp on half p; tq1, tq2 on half q.
int mobius_mpc_impl(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tp, gbdw_field* tq1,
                    gbdw_field* tq2, const gbdw_field* in, const Mobius& m, int dag, double* norm2, bool fetch) {
  if (!gp || !gq || gq->lat != gp->lat->partner) {
    set_error("Mobius Schur operator: gauge halves must be partners");
    return GBDW_ERR_INVALID;
  }
  if (!check_mobius(m)) return GBDW_ERR_INVALID;
  if (!out || !in || !tp || !tq1 || !tq2 || out == in || tp == in || tp == out || tq1 == tq2 ||
      tp->lat != gp->lat || tq1->lat != gq->lat || tq2->lat != gq->lat || in->lat != gp->lat) {
    set_error("Mobius Schur operator: distinct temporaries (one on this half, two on the other)");
    return GBDW_ERR_INVALID;
  }
  if (int st = check_ls(in)) return st;
  const int Ls = in->lat->Ls;
  const Coef5 oo = mooee(Ls, m), eo = meo5(Ls, m, -0.5);
  if (!dag) {
    // tp = -1/2 A(b,c) in;  tq1 = Dhop_qp tp;  tq2 = Mooee^-1 tq1;  tq1 = -1/2 A(b,c) tq2;
    // out = Mooee in - Dhop_pq tq1   (epilogue: a5 = bee, c5 = cee, khop = 1)
    if (int st = m5d(tp, in, eo, nullptr, nullptr, 0)) return st;
    if (int st = hop_eo(gq, tq1, tp, 0, nullptr, 0.0, 0.0, 0.5, nullptr, true)) return st;
    if (int st = m5d_inv(tq2, tq1, oo, 0)) return st;
    if (int st = m5d(tq1, tq2, eo, nullptr, nullptr, 0)) return st;
    DhopExtra ex;
    ex.c5 = m.cee();
    // hop_eo takes M5 and uses 5 - M5 as the diagonal coefficient
    return hop_eo(gp, out, tq1, 0, in, 5.0 - m.bee(), m.mf, 1.0, norm2, fetch, &ex);
  }
  // Mpc^dag = Mooee^dag - (-1/2 A^dag DhopDag_pq) Mooee^-dag (-1/2 A^dag DhopDag_qp):
  // tq1 = DhopDag_qp in;  tq2 = -1/2 A^dag tq1;  tq1 = Mooee^-dag tq2;  tp = DhopDag_pq tq1;
  // out = Mooee^dag in - (-1/2 A^dag) tp
  if (int st = hop_eo(gq, tq1, in, 1, nullptr, 0.0, 0.0, 0.5, nullptr, true)) return st;
  if (int st = m5d(tq2, tq1, eo, nullptr, nullptr, 1)) return st;
  if (int st = m5d_inv(tq1, tq2, oo, 1)) return st;
  if (int st = hop_eo(gp, tp, tq1, 1, nullptr, 0.0, 0.0, 0.5, nullptr, true)) return st;
  const Coef5 neg = meo5(Ls, m, 0.5);
  if (int st = m5d(out, in, oo, tp, &neg, 1)) return st;
  if (norm2) return blas_norm2(out, norm2, fetch);
  return GBDW_OK;
}

}  // namespace

int mobius_mooee_op(gbdw_field* out, const gbdw_field* in, double b, double c, double M5, double mf, int dag,
                    bool inverse) {
  const Mobius m{b, c, M5, mf};
  if (!check_mobius(m)) return GBDW_ERR_INVALID;
  if (int st = check_ls(in)) return st;
  return inverse ? m5d_inv(out, in, mooee(in->lat->Ls, m), dag) : m5d(out, in, mooee(in->lat->Ls, m), nullptr, nullptr, dag);
}

int mobius_meooe_op(const gbdw_gauge* gp, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double b, double c,
                    double mf, int dag) {
  return mobius_meooe(gp, out, tmp, in, Mobius{b, c, 0.0, mf}, dag);
}

int mobius_mpcdagmpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tpa, gbdw_field* tp,
                     gbdw_field* tq1, gbdw_field* tq2, const gbdw_field* in, double b, double c, double M5, double mf,
                     double* pap) {
  if (!tpa || tpa == in || tpa == out || tpa == tp) {
    set_error("Mobius Schur normal operator: a distinct temporary for Mpc in");
    return GBDW_ERR_INVALID;
  }
  const Mobius m{b, c, M5, mf};
  // |Mpc in|^2 stays in the reduction result: nothing between the two Schur passes reduces
  double dummy = 0.0;
  if (int st = mobius_mpc_impl(gp, gq, tpa, tp, tq1, tq2, in, m, 0, pap ? &dummy : nullptr, false)) return st;
  if (int st = mobius_mpc_impl(gp, gq, out, tp, tq1, tq2, tpa, m, 1, nullptr, true)) return st;
  if (pap) {
    Reduce red;
    if (int st = reduce_scratch(1, 1, &red)) return st;
    return reduce_fetch(red, 1, pap);
  }
  return GBDW_OK;
}

int mobius_mdagm(const gbdw_gauge* g, gbdw_field* out, gbdw_field* t, gbdw_field* tmp, const gbdw_field* in,
                 double b, double c, double M5, double mf, double* pap) {
  const Mobius m{b, c, M5, mf};
  if (int st = check_operands(g, t, in, true)) return st;
  if (int st = check_operands(g, tmp, in, true)) return st;
  if (int st = check_operands(g, out, in, true)) return st;
  if (t == tmp || out == t || out == tmp) {
    set_error("Mobius M^dag M: out, t and tmp must be distinct");
    return GBDW_ERR_INVALID;
  }
  if (!check_mobius(m)) return GBDW_ERR_INVALID;
  if (int st = check_ls(in)) return st;
  const int Ls = in->lat->Ls;
  // t = M in with |t|^2 reduced in the hopping pass and read after the adjoint passes (which
  // reduce nothing)
  DhopExtra ex;
  ex.c5 = m.cee();
  double dummy = 0.0;
  DhopExtra fx = ex;
  fx.mobius = true;
  fx.mb = m.b;
  fx.mc = m.c;
  if (mobius_fusable(g, in, 0)) {
    if (int st = run_dhop(g, t, in, 0, 1, m.bee(), m.mf, pap ? &dummy : nullptr, false, nullptr, 0.5, &fx)) return st;
  } else {
    if (int st = m5d(tmp, in, meo5(Ls, m, 1.0), nullptr, nullptr, 0)) return st;
    if (int st = run_dhop(g, t, tmp, 0, 1, m.bee(), m.mf, pap ? &dummy : nullptr, false, in, 0.5, &ex)) return st;
  }
  if (mobius_fusable(g, t, 1)) {
    if (int st = run_dhop(g, out, t, 1, 1, m.bee(), m.mf, nullptr, false, nullptr, 0.5, &fx)) return st;
  } else {
    if (int st = run_dhop(g, tmp, t, 1, 0, 0.0, 0.0, nullptr)) return st;
    const Coef5 b5 = meo5(Ls, m, -0.5);
    if (int st = m5d(out, t, mooee(Ls, m), tmp, &b5, 1)) return st;
  }
  if (pap) {
    Reduce red;
    if (int st = reduce_scratch(1, 1, &red)) return st;
    return reduce_fetch(red, 1, pap);
  }
  return GBDW_OK;
}

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_m5d(gbdw_field* out, const gbdw_field* in, const double* lower, const double* diag, const double* upper,
             int dag) {
  Coef5 c;
  if (!in || !read_coef(&c, in->lat->Ls, lower, diag, upper)) {
    set_error("gbdw_m5d: Ls finite coefficients per array, 1 <= Ls <= 64");
    return GBDW_ERR_INVALID;
  }
  return m5d(out, in, c, nullptr, nullptr, dag ? 1 : 0);
}

int gbdw_m5d_inv(gbdw_field* out, const gbdw_field* in, const double* lower, const double* diag, const double* upper,
                 int dag) {
  Coef5 c;
  if (!in || !read_coef(&c, in->lat->Ls, lower, diag, upper)) {
    set_error("gbdw_m5d_inv: Ls finite coefficients per array, 1 <= Ls <= 64");
    return GBDW_ERR_INVALID;
  }
  return m5d_inv(out, in, c, dag ? 1 : 0);
}

int gbdw_mobius_mooee(gbdw_field* out, const gbdw_field* in, double b, double c, double M5, double mf, int dag) {
  const Mobius m{b, c, M5, mf};
  if (!check_mobius(m)) return GBDW_ERR_INVALID;
  if (int st = check_ls(in)) return st;
  return m5d(out, in, mooee(in->lat->Ls, m), nullptr, nullptr, dag ? 1 : 0);
}

int gbdw_mobius_mooee_inv(gbdw_field* out, const gbdw_field* in, double b, double c, double M5, double mf, int dag) {
  const Mobius m{b, c, M5, mf};
  if (!check_mobius(m)) return GBDW_ERR_INVALID;
  if (int st = check_ls(in)) return st;
  return m5d_inv(out, in, mooee(in->lat->Ls, m), dag ? 1 : 0);
}

int gbdw_mobius_m(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double b, double c,
                  double M5, double mf, int dag, double* norm2) {
  if (int st = ensure_device()) return st;
  return mobius_m(g, out, tmp, in, Mobius{b, c, M5, mf}, dag ? 1 : 0, norm2);
}

int gbdw_mobius_meooe(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double b, double c,
                      double mf, int dag) {
  if (int st = ensure_device()) return st;
  return mobius_meooe(g, out, tmp, in, Mobius{b, c, 0.0, mf}, dag ? 1 : 0);
}

int gbdw_mobius_mdagm(const gbdw_gauge* g, gbdw_field* out, gbdw_field* t, gbdw_field* tmp, const gbdw_field* in,
                      double b, double c, double M5, double mf, double* pap) {
  if (int st = ensure_device()) return st;
  return mobius_mdagm(g, out, t, tmp, in, b, c, M5, mf, pap);
}

int gbdw_mobius_mpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tp, gbdw_field* tq1,
                    gbdw_field* tq2, const gbdw_field* in, double b, double c, double M5, double mf, int dag,
                    double* norm2) {
  if (int st = ensure_device()) return st;
  return mobius_mpc_impl(gp, gq, out, tp, tq1, tq2, in, Mobius{b, c, M5, mf}, dag ? 1 : 0, norm2, true);
}

}  // extern "C"
