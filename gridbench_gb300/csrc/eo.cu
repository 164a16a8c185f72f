// Even-odd (4D red-black) decomposition of the Shamir domain-wall operator.  The grids are
// the ones Grid builds beside the full ones (makeFourDimRedBlackGrid /
// makeFiveDimRedBlackGrid, TableGenerate.cc:26-28): a 4D checkerboard, every slice s of a
// 4D site on the site's parity.  The hopping term only connects opposite parities, the
// 5th-dimension part D5 = M - (-1/2 Dhop) is local to a 4D site, so
//     M = [[D5, -1/2 Dhop_eo], [-1/2 Dhop_oe, D5]]
// and the Schur complement on one parity p (q the other) is
//     Mpc = D5 - 1/4 Dhop_pq D5^-1 Dhop_qp,      Mpc^dag = D5^dag - 1/4 DhopDag_pq D5^-dag DhopDag_qp.
//
// Half lattices number their sites parent_site / 2 (the x extent is even), so a half field
// is a plain GB300-layout field over V/2 sites and the hopping kernels run on it unchanged:
// a half lattice's neighbour table points into the partner half, and the links of a half
// gauge field are the parent's links of that parity's sites, in half-site order.
//
// D5^-1 in closed form.  On spins 0,1 (dag = 0) D5 = a5 - S with (S psi)(s) = psi(s-1) and
// (S psi)(0) = -mf psi(Ls-1); on spins 2,3 the shift runs the other way (s+1, wrap at Ls-1);
// dag swaps the two.  S^Ls = -mf, so (a5 - S) sum_{j<Ls} S^j a5^-(j+1) = (1 + mf a5^-Ls),
// i.e.  D5^-1 = g sum_{j<Ls} a5^-j S^j  with  g = 1 / (a5 (1 + mf a5^-Ls)):  a dense Ls x Ls
// matrix per chirality whose entries are g a5^-j (no wrap) or -mf g a5^-j (one wrap), applied
// in O(Ls) per row as a first-order recursion (k_m5inv).
#include <algorithm>
#include <cmath>

#include "blas.h"
#include "common.cuh"
#include "eo.h"
#include "layout.cuh"
#include "tune.h"

namespace gbdw {

namespace {

inline unsigned nb(int64_t n, int t) { return unsigned((n + t - 1) / t); }

__global__ void k_cb_table(int4 L, int parity, int64_t nhalf, uint32_t* nbr4, uint32_t* cbsite) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nhalf) return;
  const int hx = L.x / 2;
  const int64_t rest = i / hx;
  const int xh = int(i - rest * hx);
  int c[4];
  c[1] = int(rest % L.y);
  c[2] = int((rest / L.y) % L.z);
  c[3] = int(rest / (int64_t(L.y) * L.z));
  c[0] = 2 * xh + ((parity + c[1] + c[2] + c[3]) & 1);
  const int Ld[4] = {L.x, L.y, L.z, L.w};
  cbsite[i] = uint32_t(c[0] + int64_t(L.x) * rest);
  for (int mu = 0; mu < 8; ++mu) {
    const int d = mu & 3;
    int y[4] = {c[0], c[1], c[2], c[3]};
    y[d] = mu < 4 ? (y[d] + 1) % Ld[d] : (y[d] + Ld[d] - 1) % Ld[d];
    const int64_t f = y[0] + int64_t(Ld[0]) * (y[1] + int64_t(Ld[1]) * (y[2] + int64_t(Ld[2]) * y[3]));
    nbr4[i * 8 + mu] = uint32_t(f / 2);
  }
}

// dst row i = src row map[i] (GATHER) or dst row map[i] = src row i; rows of `row` elements.
template <class E, bool GATHER>
__global__ void k_rows(const E* __restrict__ src, E* __restrict__ dst, const uint32_t* __restrict__ map, int64_t n,
                       int row) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= n * row) return;
  const int64_t h = i / row;
  const int k = int(i - h * row);
  const int64_t f = map[h];
  if (GATHER) dst[i] = src[f * row + k];
  else dst[f * row + k] = src[i];
}

template <class E, bool GATHER>
int copy_rows(const void* src, void* dst, const uint32_t* map, int64_t n, size_t row_bytes) {
  const int row = int(row_bytes / sizeof(E));
  k_rows<E, GATHER><<<nb(n * row, 256), 256, 0, stream()>>>((const E*)src, (E*)dst, map, n, row);
  GBDW_LAUNCHED();
  return GBDW_OK;
}

constexpr int kMaxLsInv = 64;
struct M5InvParams {
  const void* in;
  const float* in_norm;
  void* out;
  float* out_norm;
  int64_t nsite;
  int Ls;
  int LsP;
  int nsb;        // sites per CTA
  double ia5;     // 1 / a5
  double g;       // 1 / (a5 (1 + mf a5^-Ls))
  double mf;
};

// The recursion form of D5^-1 on one chirality, per spin-colour row (x, y of length Ls):
//   shift s-1 -> s:  y(0) = g [x(0) - mf sum_{t>=1} a5^-(Ls-t) x(t)],  y(s) = (x(s) + y(s-1)) / a5
//   shift s+1 -> s:  y(Ls-1) = g [x(Ls-1) - mf sum_{t<=Ls-2} a5^-(t+1) x(t)],  y(s) = (x(s) + y(s+1)) / a5
// which is the dense form above row by row (the wrap coefficient folds into g).  Phase 1:
// one thread per (site, row) runs both sweeps into a shared-memory tile; phase 2: one thread
// per (site, N slices) writes the tile in the field's storage format (norms for F16).
// Both sweeps of one row over values v[0..Ls) (registers when LSC > 0), results into y.
template <class T, bool DOWN, class V>
__device__ __forceinline__ void m5_sweeps(const V& v, int Ls, T ia5, T g, T mf, cpx<T>* y) {
  cpx<T> w = {T(0), T(0)};
  if constexpr (DOWN) {
    for (int t = 1; t < Ls; ++t) w = {(w.r + v(t).r) * ia5, (w.i + v(t).i) * ia5};
    cpx<T> prev = {g * (v(0).r - mf * w.r), g * (v(0).i - mf * w.i)};
    y[0] = prev;
    for (int t = 1; t < Ls; ++t) {
      prev = {(v(t).r + prev.r) * ia5, (v(t).i + prev.i) * ia5};
      y[t] = prev;
    }
  } else {
    for (int t = Ls - 2; t >= 0; --t) w = {(w.r + v(t).r) * ia5, (w.i + v(t).i) * ia5};
    cpx<T> prev = {g * (v(Ls - 1).r - mf * w.r), g * (v(Ls - 1).i - mf * w.i)};
    y[Ls - 1] = prev;
    for (int t = Ls - 2; t >= 0; --t) {
      prev = {(v(t).r + prev.r) * ia5, (v(t).i + prev.i) * ia5};
      y[t] = prev;
    }
  }
}

// LSC > 0: the launch guarantees Ls == LSC (even), and a row is loaded into registers with
// slice-pair vector loads before the sweeps; LSC == 0 reads the row slice by slice.
template <int P, int DAG, int N, int LSC>
__global__ void __launch_bounds__(192) k_m5inv(const M5InvParams p) {
  using T = typename Arith<P>::T;
  extern __shared__ __align__(16) unsigned char m5_smem[];
  cpx<T>* tile = reinterpret_cast<cpx<T>*>(m5_smem);  // [nsb][12][Ls + 1] (padded rows)
  const int Ls = LSC > 0 ? LSC : p.Ls, LsT = Ls + 1;
  const int64_t site0 = int64_t(blockIdx.x) * p.nsb;
  const T ia5 = T(p.ia5), g = T(p.g), mf = T(p.mf);
  if (threadIdx.x < 12 * p.nsb) {
    const int ls = threadIdx.x / 12, row = threadIdx.x - 12 * (threadIdx.x / 12);
    const int64_t site = site0 + ls;
    if (site < p.nsite) {
      const int64_t r = site * 12 + row;
      cpx<T>* y = tile + (ls * 12 + row) * LsT;
      const bool down = (row < 6) != (DAG != 0);  // psi(s-1) feeds s
      if constexpr (LSC > 0) {
        cpx<T> xv[LSC];
#pragma unroll
        for (int q = 0; q < LSC / 2; ++q) {
          cpx<T> v2[2];
          Vec<P, 2>::load(p.in, r, 2 * q, p.LsP, v2);
          xv[2 * q] = v2[0];
          xv[2 * q + 1] = v2[1];
        }
        if constexpr (P == GBDW_F16) {
          float nr[LSC];
          load_norms<LSC>(p.in_norm, site * LSC, nr);
#pragma unroll
          for (int t = 0; t < LSC; ++t) xv[t] = {xv[t].r * nr[t], xv[t].i * nr[t]};
        }
        auto v = [&](int t) -> const cpx<T>& { return xv[t]; };
        if (down) m5_sweeps<T, true>(v, LSC, ia5, g, mf, y);
        else m5_sweeps<T, false>(v, LSC, ia5, g, mf, y);
      } else {
        auto v = [&](int t) -> cpx<T> {
          cpx<T> e = Elem<P>::ld(p.in, r, t, p.LsP);
          if constexpr (P == GBDW_F16) {
            const float n = __ldg(p.in_norm + site * Ls + t);
            e = {e.r * n, e.i * n};
          }
          return e;
        };
        if (down) m5_sweeps<T, true>(v, Ls, ia5, g, mf, y);
        else m5_sweeps<T, false>(v, Ls, ia5, g, mf, y);
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

bool is_half(const gbdw_lattice* l) { return l && l->parity >= 0 && l->cbsite; }

}  // namespace

int m5inv(gbdw_field* out, const gbdw_field* in, double M5, double mf, int dag) {
  if (!out || !in || out == in || out->lat != in->lat || out->prec != in->prec || in->nrhs != 1 || out->nrhs != 1) {
    set_error("D5^-1: distinct single-rhs fields of one lattice and precision");
    return GBDW_ERR_INVALID;
  }
  const int Ls = in->lat->Ls;
  const double a5 = 5.0 - M5;
  if (Ls > kMaxLsInv || !(std::fabs(a5) > 1e-6)) {
    set_error("D5^-1: needs Ls <= 64 and M5 != 5");
    return GBDW_ERR_INVALID;
  }
  M5InvParams p;
  p.in = in->d;
  p.in_norm = in->norm;
  p.out = out->d;
  p.out_norm = out->norm;
  p.nsite = in->lat->nsite;
  p.Ls = Ls;
  p.LsP = in->LsP;
  p.mf = mf;
  p.ia5 = 1.0 / a5;
  const double den = a5 * (1.0 + mf * std::pow(a5, -double(Ls)));
  if (!(std::fabs(den) > 0.0) || !std::isfinite(den)) {
    set_error("D5^-1: singular 5th-dimension operator for these M5, mf");
    return GBDW_ERR_INVALID;
  }
  p.g = 1.0 / den;
  if (int st = ensure_device()) return st;
  const size_t per_site = 12 * size_t(Ls + 1) * (in->prec == GBDW_F64 ? 16 : 8);
  p.nsb = int(std::min<size_t>(16, 49152 / per_site));
  const size_t smem = size_t(p.nsb) * per_site;
  const unsigned g = nb(p.nsite, p.nsb);
  const int threads = 12 * p.nsb;
  const bool pair = Ls % 2 == 0;
#define GBDW_M5(P)                                                                               \
  if (Ls == 16) {                                                                                \
    if (dag) k_m5inv<P, 1, 2, 16><<<g, threads, smem, stream()>>>(p);                            \
    else k_m5inv<P, 0, 2, 16><<<g, threads, smem, stream()>>>(p);                                \
  } else if (pair) {                                                                             \
    if (dag) k_m5inv<P, 1, 2, 0><<<g, threads, smem, stream()>>>(p);                             \
    else k_m5inv<P, 0, 2, 0><<<g, threads, smem, stream()>>>(p);                                 \
  } else {                                                                                       \
    if (dag) k_m5inv<P, 1, 1, 0><<<g, threads, smem, stream()>>>(p);                             \
    else k_m5inv<P, 0, 1, 0><<<g, threads, smem, stream()>>>(p);                                 \
  }
  if (in->prec == GBDW_F64) {
    GBDW_M5(GBDW_F64)
  } else if (in->prec == GBDW_F32) {
    GBDW_M5(GBDW_F32)
  } else {
    GBDW_M5(GBDW_F16)
  }
#undef GBDW_M5
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int check_eo(const gbdw_gauge* g, const gbdw_field* out, const gbdw_field* in) {
  if (!g || !out || !in || out == in) {
    set_error("even-odd hopping term: null or aliased operands");
    return GBDW_ERR_INVALID;
  }
  if (!is_half(g->lat) || out->lat != g->lat || in->lat != g->lat->partner || in->prec != out->prec ||
      in->nrhs != out->nrhs) {
    set_error("even-odd hopping term: gauge and output on one half lattice, input on its partner, same precision");
    return GBDW_ERR_INVALID;
  }
  if (!((g->prec == in->prec) || (in->prec == GBDW_F16 && g->prec == GBDW_BF16))) {
    set_error("unsupported spinor/gauge precision pair (F64/F64, F32/F32, F16/F16, F16/BF16)");
    return GBDW_ERR_INVALID;
  }
  return GBDW_OK;
}

int hop_eo(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag, const gbdw_field* cen, double M5,
           double mf, double khop, double* norm2, bool fetch, const DhopExtra* ex) {
  if (int st = check_eo(g, out, in)) return st;
  if (cen && (cen->lat != out->lat || cen->prec != in->prec || cen->nrhs != 1 || in->nrhs != 1 || cen == out)) {
    set_error("even-odd operator: the diagonal field lives on the output half, same precision, single rhs");
    return GBDW_ERR_INVALID;
  }
  return run_dhop(g, out, in, dag ? 1 : 0, cen ? 1 : 0, 5.0 - M5, mf, norm2, fetch, cen, khop, ex);
}

int mpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tq1, gbdw_field* tq2,
        const gbdw_field* in, double M5, double mf, int dag, double* norm2, bool fetch) {
  if (!gp || !gq || gq->lat != gp->lat->partner) {
    set_error("Schur operator: gauge halves must be partners");
    return GBDW_ERR_INVALID;
  }
  if (!tq1 || !tq2 || tq1 == tq2 || tq1->lat != gq->lat || tq2->lat != gq->lat || !out || out == in) {
    set_error("Schur operator: two distinct temporaries on the other half, out != in");
    return GBDW_ERR_INVALID;
  }
  if (int st = hop_eo(gq, tq1, in, dag, nullptr, M5, mf, 0.5, nullptr, true)) return st;
  if (int st = m5inv(tq2, tq1, M5, mf, dag)) return st;
  return hop_eo(gp, out, tq2, dag, in, M5, mf, 0.25, norm2, fetch);
}

int mpcdagmpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tp, gbdw_field* tq1,
              gbdw_field* tq2, const gbdw_field* in, double M5, double mf, double* pap) {
  if (!tp || tp == in || tp == out) {
    set_error("Schur normal operator: the temporary on this half must differ from in and out");
    return GBDW_ERR_INVALID;
  }
  if (int st = mpc(gp, gq, tp, tq1, tq2, in, M5, mf, 0, pap, false)) return st;
  if (int st = mpc(gp, gq, out, tq1, tq2, tp, M5, mf, 1, nullptr, true)) return st;
  if (pap) {
    Reduce red;
    if (int st = reduce_scratch(1, 1, &red)) return st;
    return reduce_fetch(red, 1, pap);
  }
  return GBDW_OK;
}

int mpcdagmpc_residual(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* sink, gbdw_field* tp, gbdw_field* tq1,
                       gbdw_field* tq2, gbdw_field* r, const gbdw_field* in, double M5, double mf, double rr,
                       double out[3]) {
  if (!gp || !gq || gq->lat != gp->lat->partner || !tp || !tq1 || !tq2 || !sink || tp == in || sink == tp ||
      sink == in) {
    set_error("fused Schur step: partner gauge halves, distinct temporaries");
    return GBDW_ERR_INVALID;
  }
  double* s = cg_scalars();
  if (!s) {
    set_error("CG scalar scratch allocation failed");
    return GBDW_ERR_ALLOC;
  }
  DhopExtra e1;
  e1.sum_to = s;
  e1.num = rr;
  e1.alpha_to = s + 1;
  if (int st = hop_eo(gq, tq1, in, 0, nullptr, M5, mf, 0.5, nullptr, true)) return st;
  if (int st = m5inv(tq2, tq1, M5, mf, 0)) return st;
  if (int st = hop_eo(gp, tp, tq2, 0, in, M5, mf, 0.25, nullptr, false, &e1)) return st;
  DhopExtra e2;
  e2.r = r;
  e2.alpha = s + 1;
  e2.sum_to = s + 2;
  if (int st = hop_eo(gq, tq1, tp, 1, nullptr, M5, mf, 0.5, nullptr, true)) return st;
  if (int st = m5inv(tq2, tq1, M5, mf, 1)) return st;
  if (int st = hop_eo(gp, sink, tq2, 1, tp, M5, mf, 0.25, nullptr, false, &e2)) return st;
  return fetch_doubles(s, 3, out);
}

int field_pick(gbdw_field* half, const gbdw_field* full) {
  if (!half || !full || !is_half(half->lat) || half->lat->parent != full->lat || half->prec != full->prec ||
      half->nrhs != full->nrhs) {
    set_error("gbdw_field_pick: a half-lattice field of the full field's lattice, precision and nrhs");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const int64_t n = half->lat->nsite;
  const size_t row = 12 * size_t(half->LsP) * spinor_elem_bytes(half->prec);
  if (int st = copy_rows<uint4, true>(full->d, half->d, half->lat->cbsite, n, row)) return st;
  if (half->prec == GBDW_F16)
    return copy_rows<float, true>(full->norm, half->norm, half->lat->cbsite, n, size_t(half->LsE) * 4);
  return GBDW_OK;
}

int field_place(gbdw_field* full, const gbdw_field* half) {
  if (!half || !full || !is_half(half->lat) || half->lat->parent != full->lat || half->prec != full->prec ||
      half->nrhs != full->nrhs) {
    set_error("gbdw_field_place: a half-lattice field of the full field's lattice, precision and nrhs");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const int64_t n = half->lat->nsite;
  const size_t row = 12 * size_t(half->LsP) * spinor_elem_bytes(half->prec);
  if (int st = copy_rows<uint4, false>(half->d, full->d, half->lat->cbsite, n, row)) return st;
  if (half->prec == GBDW_F16)
    return copy_rows<float, false>(half->norm, full->norm, half->lat->cbsite, n, size_t(half->LsE) * 4);
  return GBDW_OK;
}

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_lattice_checkerboard(const gbdw_lattice* full, gbdw_lattice** even, gbdw_lattice** odd) {
  if (!full || !even || !odd || !full->fast || full->nsimd != 1 || full->parity >= 0 || full->dims[0] == 0) {
    set_error("gbdw_lattice_checkerboard: needs a periodic lattice made by gbdw_lattice_create");
    return GBDW_ERR_INVALID;
  }
  for (int d = 0; d < 4; ++d)
    if (full->dims[d] % 2) {
      set_error("gbdw_lattice_checkerboard: every extent must be even");
      return GBDW_ERR_INVALID;
    }
  if (int st = ensure_device()) return st;
  const int64_t nh = full->nsite / 2;
  gbdw_lattice* H[2] = {nullptr, nullptr};
  for (int par = 0; par < 2; ++par) {
    gbdw_lattice* L = new gbdw_lattice();
    L->nsite = nh;
    L->Ls = full->Ls;
    L->nsimd = 1;
    L->fast = true;
    L->parity = par;
    L->parent = full;
    cudaError_t e = dev_alloc((void**)&L->nbr4, size_t(nh) * 8 * sizeof(uint32_t));
    if (e == cudaSuccess) e = dev_alloc((void**)&L->cbsite, size_t(nh) * sizeof(uint32_t));
    if (e != cudaSuccess) {
      gbdw_lattice_destroy(L);
      if (H[0]) gbdw_lattice_destroy(H[0]);
      return cuda_fail(e, "cudaMalloc(checkerboard tables)");
    }
    k_cb_table<<<nb(nh, 256), 256, 0, stream()>>>(make_int4(full->dims[0], full->dims[1], full->dims[2], full->dims[3]),
                                                  par, nh, L->nbr4, L->cbsite);
    if ((e = cudaGetLastError()) != cudaSuccess) {
      gbdw_lattice_destroy(L);
      if (H[0]) gbdw_lattice_destroy(H[0]);
      return cuda_fail(e, "k_cb_table");
    }
    count_launch();
    H[par] = L;
  }
  H[0]->partner = H[1];
  H[1]->partner = H[0];
  *even = H[0];
  *odd = H[1];
  return GBDW_OK;
}

int gbdw_gauge_checkerboard(gbdw_gauge** out, const gbdw_gauge* full, const gbdw_lattice* half) {
  if (!out || !full || !is_half(half) || half->parent != full->lat) {
    set_error("gbdw_gauge_checkerboard: a half lattice of the gauge field's lattice");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  gbdw_gauge* G = new gbdw_gauge();
  G->lat = half;
  G->prec = full->prec;
  G->bytes = size_t(half->nsite) * 8 * link_bytes(full->prec);
  cudaError_t e = dev_alloc((void**)&G->d, G->bytes);
  if (e != cudaSuccess) {
    delete G;
    return cuda_fail(e, "cudaMalloc(half gauge)");
  }
  if (int st = copy_rows<uint4, true>(full->d, G->d, half->cbsite, half->nsite, 8 * link_bytes(full->prec))) {
    cudaFree(G->d);
    delete G;
    return st;
  }
  *out = G;
  return GBDW_OK;
}

int gbdw_field_pick(gbdw_field* half, const gbdw_field* full) { return field_pick(half, full); }
int gbdw_field_place(gbdw_field* full, const gbdw_field* half) { return field_place(full, half); }

int gbdw_dhop_eo(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag) {
  if (int st = ensure_device()) return st;
  return hop_eo(g, out, in, dag, nullptr, 0.0, 0.0, 0.5, nullptr, true);
}

int gbdw_dwf_meo(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, const gbdw_field* cen, double M5,
                 double mf, int dag, double khop) {
  if (!cen) {
    set_error("gbdw_dwf_meo: the diagonal field is required");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  return hop_eo(g, out, in, dag, cen, M5, mf, khop, nullptr, true);
}

int gbdw_dwf_m5inv(gbdw_field* out, const gbdw_field* in, double M5, double mf, int dag) {
  return m5inv(out, in, M5, mf, dag ? 1 : 0);
}

int gbdw_dwf_mpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tq1, gbdw_field* tq2,
                 const gbdw_field* in, double M5, double mf, int dag, double* norm2) {
  if (int st = ensure_device()) return st;
  return mpc(gp, gq, out, tq1, tq2, in, M5, mf, dag ? 1 : 0, norm2, true);
}

int gbdw_dwf_mpcdagmpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tp, gbdw_field* tq1,
                       gbdw_field* tq2, const gbdw_field* in, double M5, double mf, double* pap) {
  if (int st = ensure_device()) return st;
  return mpcdagmpc(gp, gq, out, tp, tq1, tq2, in, M5, mf, pap);
}

}  // extern "C"
