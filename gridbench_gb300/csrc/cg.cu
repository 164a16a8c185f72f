// Conjugate gradient on M^dagger M for the Shamir domain-wall operator (no counterpart in
// the reference), with reliable updates after Sleijpen and van der Vorst as used for mixed
// precision lattice solvers by Clark et al. (Comput. Phys. Commun. 181 (2010) 1517):
// the iterated residual lives in a cheap precision, and whenever it has dropped by a factor
// delta since the last update the solution is folded into the FP64 accumulator and the
// true residual r = b - A x is recomputed with the FP64 operator.  Every global sum is
// FP64; the exit test is always on the true residual.
//
// One solver core serves two operators: the full M^dagger M (gbdw_cg_solve) and the
// even-odd Schur operator Mpc^dagger Mpc on one half lattice (gbdw_cg_solve_eo, which wraps
// the Schur solve in its source preparation and solution reconstruction).
#include <chrono>
#include <cmath>
#include <functional>
#include <string>
#include <vector>

#include "blas.h"
#include "common.cuh"
#include "eo.h"
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

// out = A in, and |M in|^2 (= <in, A in>) into pap when non-null.
using Op = std::function<int(gbdw_field* out, const gbdw_field* in, double* pap)>;
// One CG step's operator with the residual update fused into its last pass:
//   r -= alpha A p with alpha = rr / <p, A p>; out = {<p, A p>, alpha, |r|^2}.  sink: a field of
//   p's lattice and precision the passes may name as their output.
using FusedOp = std::function<int(const gbdw_field* p, gbdw_field* sink, gbdw_field* r, double rr, double out[3])>;

struct Problem {
  const gbdw_lattice* lat;  // lattice of x and b
  Op exact;                 // A on FP64 fields
  Op sloppy;                // A on fields of precision `op_prec`
  FusedOp fused;            // when set (PLAIN and MIXED): A and the r update in one pass pair
  int op_prec;              // F64 (DOUBLE), F32 (PLAIN) or the sloppy precision (MIXED)
  bool half_residual_ok = false;  // the operator's passes accept an FP16 iterated residual
};

#define TRY(e)                      \
  do {                              \
    if ((st = (e)) != 0) return st; \
  } while (0)

// Solves A x = b from the initial guess in x.  x and b are FP64 on P.lat.
int cg_core(const Problem& P, int mode, gbdw_field* x, const gbdw_field* b, const gbdw_cg_params* prm,
            gbdw_cg_stats* stats, const char* who) {
  const double delta = (prm->delta > 0 && prm->delta < 1) ? prm->delta : 0.1;
  const gbdw_lattice* lat = P.lat;
  Fields F;
  gbdw_field *r = nullptr, *t64 = nullptr;
  gbdw_field *xs = nullptr, *rs = nullptr, *p = nullptr, *pq = nullptr, *ap = nullptr;
  int st;
  TRY(F.make(lat, GBDW_F64, &r));
  TRY(F.make(lat, GBDW_F64, &t64));
  if (mode == GBDW_CG_DOUBLE) {
    xs = x;
    rs = r;
    TRY(F.make(lat, GBDW_F64, &p));
    ap = t64;
  } else if (mode == GBDW_CG_PLAIN) {
    xs = x;
    rs = r;
    TRY(F.make(lat, GBDW_F64, &p));
    TRY(F.make(lat, GBDW_F32, &pq));
    TRY(F.make(lat, GBDW_F32, &ap));
  } else {
    // the iterated residual: FP32, or FP16 on request when the whole sloppy operator is FP16
    const int rprec = (prm->sloppy_residual == 1 && P.op_prec == GBDW_F16 && P.half_residual_ok) ? GBDW_F16 : GBDW_F32;
    // the solution's increment since the last reliable update stays FP32: summing hundreds of
    // small increments into an FP16 accumulator loses them (measured: no convergence)
    TRY(F.make(lat, GBDW_F32, &xs));
    TRY(F.make(lat, rprec, &rs));
    TRY(F.make(lat, P.op_prec, &p));
    TRY(F.make(lat, P.op_prec, &ap));
  }

  TRY(gbdw_synchronize());
  const auto t0 = std::chrono::steady_clock::now();
  gbdw_cg_stats S{};
  double bb = 0.0;
  TRY(blas_norm2(b, &bb, true));
  if (!(bb > 0.0) || !std::isfinite(bb)) {
    set_error(std::string(who) + ": |b| must be finite and non-zero");
    return GBDW_ERR_INVALID;
  }
  const double stop = prm->tol * prm->tol * bb;

  // true residual r = b - A x (skipped when x is zero)
  double xx = 0.0, rr = 0.0;
  TRY(blas_norm2(x, &xx, true));
  auto true_residual = [&](double* rrt) -> int {
    int s2 = P.exact(t64, x, nullptr);
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
  const bool fused = P.fused && mode != GBDW_CG_DOUBLE;
  while (!converged && it < prm->max_iter) {
    double pap = 0.0, alpha = 0.0, rr_new = 0.0;
    if (fused) {
      // A p, alpha = rr / <p, A p> on the device, and r -= alpha A p in the last pass
      double s[3];
      TRY(P.fused(pq ? pq : p, ap, rs, rr, s));
      pap = s[0];
      alpha = s[1];
      rr_new = s[2];
    } else {
      TRY(P.sloppy(ap, pq ? pq : p, &pap));
    }
    if (!(pap > 0.0) || !std::isfinite(pap)) {
      set_error(std::string(who) + ": <p, A p> is not positive (operator or precision breakdown)");
      err = GBDW_ERR_DIVERGED;
      break;
    }
    if (!fused) {
      alpha = rr / pap;
      TRY(blas_cg_r(alpha, rs, ap, &rr_new));
    }
    ++it;
    if (!std::isfinite(rr_new)) {
      TRY(blas_axpby(alpha, p, 1.0, xs));
      set_error(std::string(who) + ": residual became non-finite");
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
    // reliable update
    TRY(blas_axpby(alpha, p, 1.0, xs));
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
    const double beta = rr_new / rr;
    TRY(blas_cg_p(beta, rs, p, pq));
    rr = rr_new;
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
  if (err) return err;
  if (!converged) {
    set_error(std::string(who) + ": iteration limit reached before the target residual");
    return GBDW_ERR_NOT_CONVERGED;
  }
  return GBDW_OK;
}

// Mode, gauge and precision checks shared by both entry points; returns the precision of
// the fields the inner operator runs on.
int check_mode(int mode, const gbdw_gauge* g64, const gbdw_gauge* g32, const gbdw_gauge* gs,
               const gbdw_cg_params* prm, const char* who, int* op_prec) {
  if (!g64 || g64->prec != GBDW_F64 || !prm || prm->tol <= 0 || prm->max_iter < 1) {
    set_error(std::string(who) + ": need F64 gauge fields, tol > 0, max_iter >= 1");
    return GBDW_ERR_INVALID;
  }
  if (mode == GBDW_CG_DOUBLE) {
    *op_prec = GBDW_F64;
    return GBDW_OK;
  }
  if (mode == GBDW_CG_PLAIN) {
    if (!g32 || g32->prec != GBDW_F32 || g32->lat != g64->lat) {
      set_error(std::string(who) + ": plain mode needs F32 gauge fields");
      return GBDW_ERR_INVALID;
    }
    *op_prec = GBDW_F32;
    return GBDW_OK;
  }
  if (mode == GBDW_CG_MIXED) {
    const int sp = prm->sloppy_prec;
    if (!gs || gs->lat != g64->lat || !(sp == GBDW_F16 || sp == GBDW_F32) ||
        (sp == GBDW_F16 && gs->prec != GBDW_F16 && gs->prec != GBDW_BF16) || (sp == GBDW_F32 && gs->prec != GBDW_F32)) {
      set_error(std::string(who) +
                ": mixed mode needs sloppy gauge fields matching sloppy_prec (F16 with F16/BF16, F32 with F32)");
      return GBDW_ERR_INVALID;
    }
    *op_prec = sp;
    return GBDW_OK;
  }
  set_error(std::string(who) + ": unknown mode");
  return GBDW_ERR_INVALID;
}

}  // namespace

extern "C" int gbdw_cg_solve(const gbdw_gauge* g64, const gbdw_gauge* g32, const gbdw_gauge* gs, gbdw_field* x,
                             const gbdw_field* b, double M5, double mf, int mode, const gbdw_cg_params* prm,
                             gbdw_cg_stats* stats) {
  const char* who = "gbdw_cg_solve";
  int op_prec = GBDW_F64;
  int st;
  TRY(check_mode(mode, g64, g32, gs, prm, who, &op_prec));
  if (!x || !b || x->prec != GBDW_F64 || b->prec != GBDW_F64 || x->lat != g64->lat || b->lat != g64->lat ||
      x->nrhs != 1 || b->nrhs != 1) {
    set_error("gbdw_cg_solve: need F64 single-rhs x and b on the gauge field's lattice");
    return GBDW_ERR_INVALID;
  }
  TRY(ensure_device());
  SolverScope fp64_scope;  // the solvers' FP64 arithmetic setting applies from here
  const gbdw_lattice* lat = g64->lat;
  Fields F;
  gbdw_field *tmp64 = nullptr, *tmps = nullptr;
  TRY(F.make(lat, GBDW_F64, &tmp64));
  if (op_prec != GBDW_F64) TRY(F.make(lat, op_prec, &tmps));
  const gbdw_gauge* gop = mode == GBDW_CG_DOUBLE ? g64 : mode == GBDW_CG_PLAIN ? g32 : gs;
  Problem P;
  P.lat = lat;
  P.op_prec = op_prec;
  P.half_residual_ok = gop && gop->prec == GBDW_F16;  // the fused adjoint pass has an FP16-r form
  P.exact = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    return gbdw_dwf_mdagm(g64, out, tmp64, in, M5, mf, pap);
  };
  P.sloppy = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    return gbdw_dwf_mdagm(gop, out, tmps ? tmps : tmp64, in, M5, mf, pap);
  };
  if (tmps)
    P.fused = [&](const gbdw_field* in, gbdw_field*, gbdw_field* r, double rr, double out[3]) {
      return mdagm_residual(gop, tmps, r, in, M5, mf, rr, out);
    };
  return cg_core(P, mode, x, b, prm, stats, who);
}

// Mobius M^dag M x = b on the full lattice (the operator of mobius.cu), the same modes and
// reliable updates as gbdw_cg_solve; the adjoint pass ends in a 5th-dimension kernel, so the
// residual update runs as its own vector pass.
extern "C" int gbdw_cg_solve_mobius(const gbdw_gauge* g64, const gbdw_gauge* g32, const gbdw_gauge* gs,
                                    gbdw_field* x, const gbdw_field* b, double b5, double c5, double M5, double mf,
                                    int mode, const gbdw_cg_params* prm, gbdw_cg_stats* stats) {
  const char* who = "gbdw_cg_solve_mobius";
  int op_prec = GBDW_F64;
  int st;
  TRY(check_mode(mode, g64, g32, gs, prm, who, &op_prec));
  if (!x || !b || x->prec != GBDW_F64 || b->prec != GBDW_F64 || x->lat != g64->lat || b->lat != g64->lat ||
      x->nrhs != 1 || b->nrhs != 1) {
    set_error("gbdw_cg_solve_mobius: need F64 single-rhs x and b on the gauge field's lattice");
    return GBDW_ERR_INVALID;
  }
  TRY(ensure_device());
  SolverScope fp64_scope;  // the solvers' FP64 arithmetic setting applies from here
  const gbdw_lattice* lat = g64->lat;
  Fields F;
  gbdw_field *t64 = nullptr, *u64 = nullptr, *ts = nullptr, *us = nullptr;
  TRY(F.make(lat, GBDW_F64, &t64));
  TRY(F.make(lat, GBDW_F64, &u64));
  if (op_prec != GBDW_F64) {
    TRY(F.make(lat, op_prec, &ts));
    TRY(F.make(lat, op_prec, &us));
  }
  const gbdw_gauge* gop = mode == GBDW_CG_DOUBLE ? g64 : mode == GBDW_CG_PLAIN ? g32 : gs;
  Problem P;
  P.lat = lat;
  P.op_prec = op_prec;
  P.half_residual_ok = true;  // separate residual pass
  P.exact = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    return mobius_mdagm(g64, out, t64, u64, in, b5, c5, M5, mf, pap);
  };
  P.sloppy = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    if (op_prec == GBDW_F64) return mobius_mdagm(gop, out, t64, u64, in, b5, c5, M5, mf, pap);
    return mobius_mdagm(gop, out, ts, us, in, b5, c5, M5, mf, pap);
  };
  return cg_core(P, mode, x, b, prm, stats, who);
}

// Solves the Mobius M x = b by the Schur complement on the odd half (the same scheme as
// gbdw_cg_solve_eo with Mooee in place of D5 and Meooe = -1/2 Dhop A(b, c)):
//   b'_o = b_o - Meooe_oe Mooee^-1 b_e,   Mpc^dag Mpc x_o = Mpc^dag b'_o,
//   x_e  = Mooee^-1 (b_e - Meooe_eo x_o).
extern "C" int gbdw_cg_solve_mobius_eo(const gbdw_gauge* const g64[2], const gbdw_gauge* const g32[2],
                                       const gbdw_gauge* const gs[2], gbdw_field* x, const gbdw_field* b, double b5,
                                       double c5, double M5, double mf, int mode, const gbdw_cg_params* prm,
                                       gbdw_cg_stats* stats) {
  const char* who = "gbdw_cg_solve_mobius_eo";
  if (!g64 || !g64[0] || !g64[1]) {
    set_error("gbdw_cg_solve_mobius_eo: need the two F64 gauge halves");
    return GBDW_ERR_INVALID;
  }
  int op_prec = GBDW_F64, op1 = GBDW_F64;
  int st;
  const gbdw_gauge* e32 = g32 ? g32[0] : nullptr;
  const gbdw_gauge* o32 = g32 ? g32[1] : nullptr;
  const gbdw_gauge* es = gs ? gs[0] : nullptr;
  const gbdw_gauge* os = gs ? gs[1] : nullptr;
  TRY(check_mode(mode, g64[0], e32, es, prm, who, &op_prec));
  TRY(check_mode(mode, g64[1], o32, os, prm, who, &op1));
  const gbdw_lattice* le = g64[0]->lat;
  const gbdw_lattice* lo = g64[1]->lat;
  if (le->parity != 0 || lo->parity != 1 || le->partner != lo || !x || !b || x->prec != GBDW_F64 ||
      b->prec != GBDW_F64 || x->lat != le->parent || b->lat != le->parent || x->nrhs != 1 || b->nrhs != 1) {
    set_error("gbdw_cg_solve_mobius_eo: gauge halves [even, odd] of the lattice of x and b (F64, single rhs)");
    return GBDW_ERR_INVALID;
  }
  TRY(ensure_device());
  SolverScope fp64_scope;  // the solvers' FP64 arithmetic setting applies from here
  Fields F;
  gbdw_field *be = nullptr, *bo = nullptr, *te = nullptr, *ue = nullptr, *xo = nullptr, *co = nullptr;
  gbdw_field *to = nullptr, *po = nullptr, *pa = nullptr;
  TRY(F.make(le, GBDW_F64, &be));
  TRY(F.make(lo, GBDW_F64, &bo));
  TRY(F.make(le, GBDW_F64, &te));
  TRY(F.make(le, GBDW_F64, &ue));
  TRY(F.make(lo, GBDW_F64, &xo));
  TRY(F.make(lo, GBDW_F64, &co));
  TRY(F.make(lo, GBDW_F64, &to));
  TRY(F.make(lo, GBDW_F64, &po));
  TRY(F.make(lo, GBDW_F64, &pa));
  gbdw_field *ps = nullptr, *pas = nullptr, *q1s = nullptr, *q2s = nullptr;
  if (op_prec != GBDW_F64) {
    TRY(F.make(lo, op_prec, &ps));
    TRY(F.make(lo, op_prec, &pas));
    TRY(F.make(le, op_prec, &q1s));
    TRY(F.make(le, op_prec, &q2s));
  }
  TRY(gbdw_synchronize());
  const auto t0 = std::chrono::steady_clock::now();
  // b'_o = b_o - Meooe_oe Mooee^-1 b_e;  c_o = Mpc^dag b'_o
  TRY(field_pick(be, b));
  TRY(field_pick(bo, b));
  TRY(mobius_mooee_op(te, be, b5, c5, M5, mf, 0, true));
  TRY(mobius_meooe_op(g64[1], to, ue, te, b5, c5, mf, 0));
  TRY(blas_axpby(-1.0, to, 1.0, bo));
  TRY(gbdw_mobius_mpc(g64[1], g64[0], co, to, te, ue, bo, b5, c5, M5, mf, 1, nullptr));
  TRY(field_pick(xo, x));

  const gbdw_gauge* gpo = mode == GBDW_CG_DOUBLE ? g64[1] : mode == GBDW_CG_PLAIN ? o32 : os;
  const gbdw_gauge* gqe = mode == GBDW_CG_DOUBLE ? g64[0] : mode == GBDW_CG_PLAIN ? e32 : es;
  Problem P;
  P.lat = lo;
  P.op_prec = op_prec;
  P.half_residual_ok = true;  // separate residual pass
  P.exact = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    return mobius_mpcdagmpc(g64[1], g64[0], out, pa, po, te, ue, in, b5, c5, M5, mf, pap);
  };
  P.sloppy = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    if (op_prec == GBDW_F64) return mobius_mpcdagmpc(gpo, gqe, out, pa, po, te, ue, in, b5, c5, M5, mf, pap);
    return mobius_mpcdagmpc(gpo, gqe, out, pas, ps, q1s, q2s, in, b5, c5, M5, mf, pap);
  };
  gbdw_cg_stats S{};
  const int cst = cg_core(P, mode, xo, co, prm, &S, who);
  if (cst != GBDW_OK && cst != GBDW_ERR_NOT_CONVERGED && cst != GBDW_ERR_DIVERGED) return cst;

  // x_e = Mooee^-1 (b_e - Meooe_eo x_o)
  TRY(mobius_meooe_op(g64[0], te, to, xo, b5, c5, mf, 0));
  TRY(blas_axpby(1.0, be, -1.0, te));
  TRY(mobius_mooee_op(ue, te, b5, c5, M5, mf, 0, true));
  TRY(field_place(x, ue));
  TRY(field_place(x, xo));
  // full-system residual: (M x)_e = Mooee x_e + Meooe_eo x_o, (M x)_o = Mooee x_o + Meooe_oe x_e
  double bb = 0.0, re2 = 0.0, ro2 = 0.0;
  TRY(mobius_meooe_op(g64[0], te, to, xo, b5, c5, mf, 0));
  TRY(mobius_mooee_op(be, ue, b5, c5, M5, mf, 0, false));
  TRY(blas_axpby(1.0, be, 1.0, te));  // te = (M x)_e
  TRY(field_pick(be, b));
  TRY(blas_xmy_norm(be, te, ue, &re2));
  TRY(field_pick(ue, x));  // x_e again (ue held the even residual)
  TRY(mobius_meooe_op(g64[1], to, te, ue, b5, c5, mf, 0));
  TRY(mobius_mooee_op(po, xo, b5, c5, M5, mf, 0, false));
  TRY(blas_axpby(1.0, po, 1.0, to));  // to = (M x)_o
  TRY(field_pick(bo, b));
  TRY(blas_xmy_norm(bo, to, co, &ro2));
  TRY(blas_norm2(b, &bb, true));
  TRY(gbdw_synchronize());
  S.true_residual = std::sqrt((re2 + ro2) / bb);
  S.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = S;
  return cst;
}

// Solves M x = b (x, b FP64 on the full lattice) by the Schur complement on the odd half:
//   b'_o = b_o + 1/2 Dhop_oe D5^-1 b_e,   Mpc^dag Mpc x_o = Mpc^dag b'_o (CG, reliable updates),
//   x_e  = D5^-1 (b_e + 1/2 Dhop_eo x_o).
// tol applies to the true residual of the Schur normal system; stats->true_residual reports
// the full system's |b - M x| / |b| after reconstruction.
extern "C" int gbdw_cg_solve_eo(const gbdw_gauge* const g64[2], const gbdw_gauge* const g32[2],
                                const gbdw_gauge* const gs[2], gbdw_field* x, const gbdw_field* b, double M5,
                                double mf, int mode, const gbdw_cg_params* prm, gbdw_cg_stats* stats) {
  const char* who = "gbdw_cg_solve_eo";
  if (!g64 || !g64[0] || !g64[1]) {
    set_error("gbdw_cg_solve_eo: need the two F64 gauge halves");
    return GBDW_ERR_INVALID;
  }
  int op_prec = GBDW_F64, op1 = GBDW_F64;
  int st;
  const gbdw_gauge* e32 = g32 ? g32[0] : nullptr;
  const gbdw_gauge* o32 = g32 ? g32[1] : nullptr;
  const gbdw_gauge* es = gs ? gs[0] : nullptr;
  const gbdw_gauge* os = gs ? gs[1] : nullptr;
  TRY(check_mode(mode, g64[0], e32, es, prm, who, &op_prec));
  TRY(check_mode(mode, g64[1], o32, os, prm, who, &op1));
  const gbdw_lattice* le = g64[0]->lat;
  const gbdw_lattice* lo = g64[1]->lat;
  if (le->parity != 0 || lo->parity != 1 || le->partner != lo || !x || !b || x->prec != GBDW_F64 ||
      b->prec != GBDW_F64 || x->lat != le->parent || b->lat != le->parent || x->nrhs != 1 || b->nrhs != 1) {
    set_error("gbdw_cg_solve_eo: gauge halves [even, odd] of the lattice of x and b (F64, single rhs)");
    return GBDW_ERR_INVALID;
  }
  TRY(ensure_device());
  SolverScope fp64_scope;  // the solvers' FP64 arithmetic setting applies from here
  Fields F;
  gbdw_field *be = nullptr, *bo = nullptr, *te = nullptr, *ue = nullptr, *xo = nullptr, *co = nullptr;
  gbdw_field *tp64 = nullptr, *tq64 = nullptr;
  TRY(F.make(le, GBDW_F64, &be));
  TRY(F.make(lo, GBDW_F64, &bo));
  TRY(F.make(le, GBDW_F64, &te));
  TRY(F.make(le, GBDW_F64, &ue));
  TRY(F.make(lo, GBDW_F64, &xo));
  TRY(F.make(lo, GBDW_F64, &co));
  TRY(F.make(lo, GBDW_F64, &tp64));
  TRY(F.make(le, GBDW_F64, &tq64));
  gbdw_field *tps = nullptr, *tq1s = nullptr, *tq2s = nullptr;
  if (op_prec != GBDW_F64) {
    TRY(F.make(lo, op_prec, &tps));
    TRY(F.make(le, op_prec, &tq1s));
    TRY(F.make(le, op_prec, &tq2s));
  }
  TRY(gbdw_synchronize());
  const auto t0 = std::chrono::steady_clock::now();
  // source: b'_o = b_o + 1/2 Dhop_oe D5^-1 b_e ; rhs of the normal system c_o = Mpc^dag b'_o
  TRY(field_pick(be, b));
  TRY(field_pick(bo, b));
  TRY(m5inv(te, be, M5, mf, 0));
  TRY(hop_eo(g64[1], tp64, te, 0, nullptr, M5, mf, 0.5, nullptr, true));
  TRY(blas_axpby(0.5, tp64, 1.0, bo));
  TRY(mpc(g64[1], g64[0], co, te, ue, bo, M5, mf, 1, nullptr, true));
  TRY(field_pick(xo, x));

  const gbdw_gauge* gpo = mode == GBDW_CG_DOUBLE ? g64[1] : mode == GBDW_CG_PLAIN ? o32 : os;
  const gbdw_gauge* gqe = mode == GBDW_CG_DOUBLE ? g64[0] : mode == GBDW_CG_PLAIN ? e32 : es;
  Problem P;
  P.lat = lo;
  P.op_prec = op_prec;
  P.half_residual_ok = gpo && gqe && gpo->prec == GBDW_F16 && gqe->prec == GBDW_F16;
  P.exact = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    return mpcdagmpc(g64[1], g64[0], out, tp64, te, ue, in, M5, mf, pap);
  };
  P.sloppy = [&](gbdw_field* out, const gbdw_field* in, double* pap) {
    if (op_prec == GBDW_F64) return mpcdagmpc(gpo, gqe, out, tp64, te, ue, in, M5, mf, pap);
    return mpcdagmpc(gpo, gqe, out, tps, tq1s, tq2s, in, M5, mf, pap);
  };
  if (op_prec != GBDW_F64)
    P.fused = [&](const gbdw_field* in, gbdw_field* sink, gbdw_field* r, double rr, double out[3]) {
      return mpcdagmpc_residual(gpo, gqe, sink, tps, tq1s, tq2s, r, in, M5, mf, rr, out);
    };
  gbdw_cg_stats S{};
  const int cst = cg_core(P, mode, xo, co, prm, &S, who);
  if (cst != GBDW_OK && cst != GBDW_ERR_NOT_CONVERGED && cst != GBDW_ERR_DIVERGED) return cst;

  // x_e = D5^-1 (b_e + 1/2 Dhop_eo x_o)
  TRY(hop_eo(g64[0], te, xo, 0, nullptr, M5, mf, 0.5, nullptr, true));
  TRY(blas_axpby(1.0, be, 0.5, te));
  TRY(m5inv(ue, te, M5, mf, 0));
  TRY(field_place(x, ue));
  TRY(field_place(x, xo));
  // full-system residual: (M x)_e = D5 x_e - 1/2 Dhop_eo x_o, (M x)_o = D5 x_o - 1/2 Dhop_oe x_e
  double bb = 0.0, re2 = 0.0, ro2 = 0.0;
  TRY(hop_eo(g64[0], te, xo, 0, ue, M5, mf, 0.5, nullptr, true));
  TRY(blas_xmy_norm(be, te, tq64, &re2));
  TRY(hop_eo(g64[1], tp64, ue, 0, xo, M5, mf, 0.5, nullptr, true));
  TRY(field_pick(bo, b));
  TRY(blas_xmy_norm(bo, tp64, co, &ro2));
  TRY(blas_norm2(b, &bb, true));
  TRY(gbdw_synchronize());
  S.true_residual = std::sqrt((re2 + ro2) / bb);
  S.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = S;
  return cst;
}
#undef TRY
