// Conjugate gradient on M^dagger M for the Shamir domain-wall operator (no counterpart in
// the reference), with reliable updates after Sleijpen and van der Vorst as used for mixed
// precision lattice solvers by Clark et al. (Comput. Phys. Commun. 181 (2010) 1517):
// the iterated residual lives in a cheap precision, and whenever it has dropped by a factor
// delta since the last update the solution is folded into the FP64 accumulator and the
// true residual r = b - A x is recomputed with the FP64 operator.  Every global sum is
// FP64; the exit test is always on the true residual.
#include <chrono>
#include <cmath>
#include <vector>

#include "blas.h"
#include "common.cuh"
#include "tune.h"

using namespace gbdw;

namespace {

struct Fields {
  std::vector<gbdw_field*> owned;
  ~Fields() {
    for (auto* f : owned) gbdw_field_destroy(f);
  }
  int make(const gbdw_lattice* lat, int prec, gbdw_field** f) {
    int st = gbdw_field_create(f, lat, prec, 1);
    if (!st) owned.push_back(*f);
    return st;
  }
};

int mdagm(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double M5, double mf,
          double* pap) {
  return gbdw_dwf_mdagm(g, out, tmp, in, M5, mf, pap);
}

}  // namespace

extern "C" int gbdw_cg_solve(const gbdw_gauge* g64, const gbdw_gauge* g32, const gbdw_gauge* gs, gbdw_field* x,
                             const gbdw_field* b, double M5, double mf, int mode, const gbdw_cg_params* prm,
                             gbdw_cg_stats* stats) {
  if (!g64 || !x || !b || !prm || g64->prec != GBDW_F64 || x->prec != GBDW_F64 || b->prec != GBDW_F64 ||
      x->lat != g64->lat || b->lat != g64->lat || x->nrhs != 1 || b->nrhs != 1 || prm->tol <= 0 || prm->max_iter < 1) {
    set_error("gbdw_cg_solve: need an F64 gauge field, F64 single-rhs x and b on its lattice, tol > 0");
    return GBDW_ERR_INVALID;
  }
  if (mode == GBDW_CG_PLAIN && (!g32 || g32->prec != GBDW_F32 || g32->lat != g64->lat)) {
    set_error("gbdw_cg_solve: plain mode needs an F32 gauge field");
    return GBDW_ERR_INVALID;
  }
  int sp = prm->sloppy_prec;
  if (mode == GBDW_CG_MIXED) {
    if (!gs || gs->lat != g64->lat || !(sp == GBDW_F16 || sp == GBDW_F32) ||
        (sp == GBDW_F16 && gs->prec != GBDW_F16 && gs->prec != GBDW_BF16) || (sp == GBDW_F32 && gs->prec != GBDW_F32)) {
      set_error("gbdw_cg_solve: mixed mode needs a sloppy gauge field matching sloppy_prec (F16 with F16/BF16, F32 with F32)");
      return GBDW_ERR_INVALID;
    }
  }
  if (mode != GBDW_CG_PLAIN && mode != GBDW_CG_MIXED && mode != GBDW_CG_DOUBLE) {
    set_error("gbdw_cg_solve: unknown mode");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const double delta = (prm->delta > 0 && prm->delta < 1) ? prm->delta : 0.1;
  const gbdw_lattice* lat = g64->lat;
  Fields F;
  gbdw_field *r = nullptr, *t64 = nullptr, *tmp64 = nullptr;
  gbdw_field *xs = nullptr, *rs = nullptr, *p = nullptr, *pq = nullptr, *ap = nullptr, *tmp = nullptr;
  const gbdw_gauge* gop = g64;  // operator of the inner iteration
  int st;
#define TRY(e)            \
  do {                    \
    if ((st = (e)) != 0) return st; \
  } while (0)
  TRY(F.make(lat, GBDW_F64, &r));
  TRY(F.make(lat, GBDW_F64, &t64));
  TRY(F.make(lat, GBDW_F64, &tmp64));
  if (mode == GBDW_CG_DOUBLE) {
    xs = x;
    rs = r;
    TRY(F.make(lat, GBDW_F64, &p));
    ap = t64;
    tmp = tmp64;
  } else if (mode == GBDW_CG_PLAIN) {
    xs = x;
    rs = r;
    gop = g32;
    TRY(F.make(lat, GBDW_F64, &p));
    TRY(F.make(lat, GBDW_F32, &pq));
    TRY(F.make(lat, GBDW_F32, &ap));
    TRY(F.make(lat, GBDW_F32, &tmp));
  } else {
    gop = gs;
    TRY(F.make(lat, GBDW_F32, &xs));
    TRY(F.make(lat, GBDW_F32, &rs));
    TRY(F.make(lat, sp, &p));
    TRY(F.make(lat, sp, &ap));
    TRY(F.make(lat, sp, &tmp));
  }

  TRY(gbdw_synchronize());
  const auto t0 = std::chrono::steady_clock::now();
  gbdw_cg_stats S{};
  double bb = 0.0;
  TRY(blas_norm2(b, &bb, true));
  if (!(bb > 0.0) || !std::isfinite(bb)) {
    set_error("gbdw_cg_solve: |b| must be finite and non-zero");
    return GBDW_ERR_INVALID;
  }
  const double stop = prm->tol * prm->tol * bb;

  // true residual r = b - A x (skipped when x is zero)
  double xx = 0.0, rr = 0.0;
  TRY(blas_norm2(x, &xx, true));
  auto true_residual = [&](double* rrt) -> int {
    int s2 = mdagm(g64, t64, tmp64, x, M5, mf, nullptr);
    if (s2) return s2;
    return blas_xmy_norm(b, t64, r, rrt);
  };
  if (xx > 0.0) {
    TRY(true_residual(&rr));
  } else {
    TRY(gbdw_field_copy(r, b));
    rr = bb;
  }
  if (mode == GBDW_CG_MIXED) {
    TRY(gbdw_field_zero(xs));
    TRY(gbdw_field_copy(rs, r));
  }
  TRY(gbdw_field_copy(p, rs));
  if (pq) TRY(gbdw_field_copy(pq, rs));
  double maxrr = rr;
  bool converged = rr <= stop;
  int it = 0;
  int err = GBDW_OK;
  double rr_true = rr;
  while (!converged && it < prm->max_iter) {
    double pap = 0.0;
    TRY(mdagm(gop, ap, tmp, pq ? pq : p, M5, mf, &pap));
    if (!(pap > 0.0) || !std::isfinite(pap)) {
      set_error("gbdw_cg_solve: <p, A p> is not positive (operator or precision breakdown)");
      err = GBDW_ERR_DIVERGED;
      break;
    }
    const double alpha = rr / pap;
    double rr_new = 0.0;
    TRY(blas_cg_r(alpha, rs, ap, &rr_new));
    ++it;
    if (!std::isfinite(rr_new)) {
      TRY(blas_axpby(alpha, p, 1.0, xs));
      set_error("gbdw_cg_solve: residual became non-finite");
      err = GBDW_ERR_DIVERGED;
      break;
    }
    if (!(rr_new < delta * delta * maxrr || rr_new <= stop)) {
      // the common iteration: x and p updated in one pass over the vectors
      const double beta = rr_new / rr;
      TRY(blas_cg_xp(alpha, beta, xs, p, rs, pq));
      rr = rr_new;
      if (rr > maxrr) maxrr = rr;
      continue;
    }
    TRY(blas_axpby(alpha, p, 1.0, xs));
    {
      // reliable update
      if (mode == GBDW_CG_MIXED) {
        TRY(blas_axpby(1.0, xs, 1.0, x));
        TRY(gbdw_field_zero(xs));
      }
      TRY(true_residual(&rr_true));
      if (mode == GBDW_CG_MIXED) TRY(gbdw_field_copy(rs, r));
      ++S.reliable_updates;
      if (rr_true <= stop) {
        converged = true;
        rr = rr_new;
        break;
      }
      rr_new = rr_true;
      maxrr = rr_true;
    }
    const double beta = rr_new / rr;
    TRY(blas_cg_p(beta, rs, p, pq));
    rr = rr_new;
    if (rr > maxrr) maxrr = rr;
  }
  if (!converged && err == 0 && mode == GBDW_CG_MIXED) {
    // fold in the last partial solution before reporting
    TRY(blas_axpby(1.0, xs, 1.0, x));
    TRY(gbdw_field_zero(xs));
  }
  if (err == 0 && !converged) TRY(true_residual(&rr_true));
  TRY(gbdw_synchronize());
  const auto t1 = std::chrono::steady_clock::now();
  S.iterations = it;
  S.true_residual = std::sqrt(rr_true / bb);
  S.final_rr = rr / bb;
  S.seconds = std::chrono::duration<double>(t1 - t0).count();
  if (stats) *stats = S;
#undef TRY
  if (err) return err;
  if (!converged) {
    set_error("gbdw_cg_solve: iteration limit reached before the target residual");
    return GBDW_ERR_NOT_CONVERGED;
  }
  return GBDW_OK;
}
