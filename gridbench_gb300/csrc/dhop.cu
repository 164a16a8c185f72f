// Operator entry points: Dhop / DhopDag, the Shamir operator M / M^dagger and M^dagger M.
#include "common.cuh"
#include "dhop_kernel.cuh"
#include "layout.cuh"
#include "tune.h"

namespace gbdw {

namespace {

bool combo_ok(const gbdw_gauge* g, const gbdw_field* f) {
  if (f->prec == GBDW_F64) return g->prec == GBDW_F64;
  if (f->prec == GBDW_F32) return g->prec == GBDW_F32;
  return g->prec == GBDW_F16 || g->prec == GBDW_BF16;
}

}  // namespace

int check_operands(const gbdw_gauge* g, const gbdw_field* out, const gbdw_field* in, bool need_single_rhs) {
  if (!g || !out || !in) {
    set_error("null gauge or field");
    return GBDW_ERR_INVALID;
  }
  if (out == in) {
    set_error("hopping kernels cannot run in place (out == in)");
    return GBDW_ERR_INVALID;
  }
  if (in->lat != g->lat || out->lat != g->lat || in->nrhs != out->nrhs || in->prec != out->prec) {
    set_error("gauge and fields must share lattice, nrhs and precision");
    return GBDW_ERR_INVALID;
  }
  if (!combo_ok(g, in)) {
    set_error("unsupported spinor/gauge precision pair (F64/F64, F32/F32, F16/F16, F16/BF16)");
    return GBDW_ERR_INVALID;
  }
  if (need_single_rhs && in->nrhs != 1) {
    set_error("the domain-wall operator takes single-right-hand-side fields");
    return GBDW_ERR_INVALID;
  }
  return GBDW_OK;
}

bool form3_ok(const gbdw_field* in, int epi, int spt) {
  if (in->prec == GBDW_F64 || spt != 2 || in->LsE != in->LsP) return false;
  if (in->LsE == 16) return true;
  return in->prec == GBDW_F32 && epi <= 1 && (in->LsE == 12 || in->LsE == 144);
}

bool blocked_ok(const gbdw_lattice* lat, const gbdw_field* in) {
  if (in->prec == GBDW_F64 || in->LsE != 16 || in->LsP != 16 || lat->parity >= 0 || !lat->fast) return false;
  for (int d = 0; d < 4; ++d)
    if (lat->dims[d] <= 0 || lat->dims[d] % 2) return false;
  return true;
}

int tile_extent(int LsE, const DhopLaunch& L, bool whole_sites) {
  if (L.split <= 1 || whole_sites || (L.mode != 0 && L.mode != 3) || LsE % L.split) return 0;
  const int TE = LsE / L.split;
  return TE % L.spt == 0 ? TE : 0;
}

int brick_extent(const gbdw_lattice* lat, const DhopLaunch& L) {
  if (L.brick <= 1 || (L.mode != 0 && L.mode != 3) || lat->parity >= 0 || !lat->fast) return 0;
  for (int d = 0; d < 4; ++d)
    if (lat->dims[d] <= 0) return 0;
  return lat->dims[3] % L.brick == 0 ? L.brick : 0;
}

bool mobius_fusable(const gbdw_gauge* g, const gbdw_field* in, int dag) {
  const int Ls = g->lat->Ls;
  // the adjoint (A^dag in the epilogue) in every precision; the forward operator (A on the loaded
  // neighbours) on FP32 slice pairs
  return g->lat->fast && (dag || in->prec == GBDW_F32) && in->nrhs == 1 && in->LsE == in->LsP && Ls >= 2 &&
         Ls <= 64 && (Ls & (Ls - 1)) == 0;
}

DhopParams make_params(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in) {
  DhopParams p;
  p.U = g->d;
  p.in = in->d;
  p.in_norm = in->norm;
  p.out = out->d;
  p.out_norm = out->norm;
  p.nbr4 = g->lat->nbr4;
  p.nbr5 = g->lat->nbr5;
  p.nsite = g->lat->nsite;
  p.LsE = in->LsE;
  p.LsP = in->LsP;
  p.Ls = g->lat->Ls;
  p.a5 = 0.0;
  p.mf = 0.0;
  p.partials = nullptr;
  p.counter = nullptr;
  p.result = nullptr;
  p.err = device_error_word();
  for (int d = 0; d < 4; ++d) p.dims[d] = g->lat->parity < 0 ? g->lat->dims[d] : 0;
  return p;
}

int run_dhop(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag, int epi, double a5, double mf,
             double* norm2, bool fetch, const gbdw_field* cen, double khop, const DhopExtra* ex) {
  if (int st = ensure_device()) return st;
  const int tune_epi = epi;
  if (ex && ex->r) {
    // residual epilogue: the M pass's launch shape, r in place of the output
    if (epi != 1 || !dag || ex->r->lat != out->lat || ex->r->nrhs != 1 || !ex->alpha || in->prec == GBDW_F64 ||
        (ex->r->prec == GBDW_F64 && in->prec != GBDW_F32) ||
        (ex->r->prec == GBDW_F16 && (in->prec != GBDW_F16 || g->prec != GBDW_F16))) {
      set_error("fused CG update: adjoint M pass, FP32/FP16 operator, FP32, FP64 (FP32 operator) or FP16 (FP16 "
                "operator and links) residual on its lattice");
      return GBDW_ERR_INVALID;
    }
    epi = ex->r->prec == GBDW_F64 ? 3 : ex->r->prec == GBDW_F16 ? 4 : 2;
  }
  DhopParams p = make_params(g, out, in);
  if (ex && ex->r) {
    p.r_norm = ex->r->norm;
    p.r = ex->r->d;
    p.rLsP = ex->r->LsP;
    p.alpha = ex->alpha;
  }
  p.a5 = a5;
  p.mf = mf;
  p.khop = khop;
  if (ex) p.c5 = ex->c5;
  if (ex && ex->mobius) {
    if (epi != 1 || ex->r || !mobius_fusable(g, in, dag)) {
      set_error("fused Mobius operator: the M epilogue, one right-hand side, Ls a power of two <= 64, FP32 for "
                "the forward operator");
      return GBDW_ERR_INVALID;
    }
    p.mob = 1;
    p.mb = ex->mb;
    p.mc = ex->mc;
    if (!dag) epi = 6;  // A(b, c) on the neighbours as they are loaded; the adjoint's is in the epilogue
  }
  if (cen) {
    p.cen = cen->d;
    p.cen_norm = cen->norm;
  }
  if (!g->lat->fast) {
    if (epi || norm2 || in->nrhs != 1) {
      set_error("general (non-factorisable) tables support the plain hopping term only");
      return GBDW_ERR_INVALID;
    }
    return launch_dhop_general(p, in->prec, dag);
  }
  if (!p.err) {
    set_error("device error word allocation failed");
    return GBDW_ERR_ALLOC;
  }
  // the forward Mobius M (A(b, c) on the loaded neighbours) has the hopping term's access pattern
  // and no Shamir epilogue: it runs on the hopping term's shape
  const int key_epi = (p.mob && epi == 6) ? 0 : tune_epi;
  DhopLaunch L = tuned_launch(g->prec, in->prec, in->LsE, key_epi);
  if (g->lat->parity >= 0) find_tuned_launch(g->prec, in->prec, in->LsE, key_epi + EO_KEY, &L);
  if (ex && ex->tune_key >= 0) find_tuned_launch(g->prec, in->prec, in->LsE, ex->tune_key, &L);
  if (in->LsE % L.spt != 0) L.spt = 1;
  if (p.mob) L.spt = 2;  // the fused adjoint works on slice pairs, one site's pairs in consecutive lanes
  int NS = 0, tthreads = 0;
  size_t smem = 0;
  const bool staged = L.mode == 1 || L.mode == 2;
  if (staged && !tma_shape(in->prec, in->LsE, L, &NS, &tthreads, &smem)) L.mode = 0;
  // fall back before fixing the CTA size: the block count below must match the launch
  if (L.mode == 4 && !blocked_ok(g->lat, in)) L.mode = 3;
  if (L.mode == 3 && !form3_ok(in, epi, L.spt)) L.mode = 0;
  if (L.mode == 3) L.threads = 64;
  if (L.mode == 4) L.threads = 128;
  p.TE = tile_extent(in->LsE, L, p.mob != 0);
  p.brick = brick_extent(g->lat, L);
  const int64_t nthreads = p.nsite * (p.LsE / L.spt);
  const int64_t blocks = staged ? (p.nsite + NS - 1) / NS : (nthreads + L.threads - 1) / L.threads;
  Reduce red;
  const bool reduce = norm2 || (ex && ex->sum_to);
  if (reduce) {
    if (int st = reduce_scratch(blocks, 1, &red)) return st;
    p.partials = red.partials;
    p.counter = red.counter;
    p.result = red.result;
  }
  int st;
  if (in->prec == GBDW_F64 && g->prec == GBDW_F64 && epi <= 1 && !p.mob && fp64_double_single()) {
    // double-single arithmetic on the FP64 fields: direct form, one slice per thread, with its own
    // tuned register cap and t-brick order
    if (int s2 = ds_links(g, &p.U)) return s2;
    DhopLaunch D{DS_THREADS, 1, 0, 4};  // stages: register cap as CTAs per SM
    find_tuned_launch(g->prec, in->prec, in->LsE, tune_epi + DS_KEY, &D);
    p.TE = 0;
    p.brick = brick_extent(g->lat, DhopLaunch{DS_THREADS, 1, 0, 4, 1, D.brick});
    const int64_t blocks_ds = (p.nsite * p.LsE + DS_THREADS - 1) / DS_THREADS;
    if (reduce && blocks_ds != blocks) {
      if (int s3 = reduce_scratch(blocks_ds, 1, &red)) return s3;
      p.partials = red.partials;
      p.counter = red.counter;
      p.result = red.result;
    }
    st = launch_dhop_ds(p, dag, epi, D.stages == 3 ? 3 : 4);
    if (st) return st;
    if (reduce) {
      double* to = (ex && ex->sum_to) ? ex->sum_to : red.result;
      if (int s2 = sum_partials(red.partials, blocks_ds, to, ex ? ex->num : 0.0, ex ? ex->alpha_to : nullptr)) return s2;
      if (norm2 && fetch) return ex && ex->sum_to ? fetch_doubles(to, 1, norm2) : reduce_fetch(red, 1, norm2);
    }
    return GBDW_OK;
  }
  if (in->prec == GBDW_F64) st = launch_dhop_f64(p, dag, epi, L);
  else if (in->prec == GBDW_F32) st = launch_dhop_f32(p, dag, epi, L);
  else st = launch_dhop_f16(p, g->prec, dag, epi, L);
  if (st) return st;
  if (reduce) {
    // the kernel leaves one partial per CTA; one CTA sums them in a fixed order
    double* to = (ex && ex->sum_to) ? ex->sum_to : red.result;
    if (int s2 = sum_partials(red.partials, blocks, to, ex ? ex->num : 0.0, ex ? ex->alpha_to : nullptr)) return s2;
    if (norm2 && fetch) return ex && ex->sum_to ? fetch_doubles(to, 1, norm2) : reduce_fetch(red, 1, norm2);
  }
  return GBDW_OK;
}

bool tma_shape(int prec, int LsE, DhopLaunch L, int* NS, int* threads, size_t* smem) {
  if (L.spt < 1 || LsE % L.spt != 0) return false;
  if (prec == GBDW_F16 && LsE % 4 != 0) return false;  // the norm block must be a 16-byte multiple
  const int Tps = LsE / L.spt;
  const size_t esz = spinor_elem_bytes(prec);
  const size_t blk = 12 * size_t(padded_slices(prec, LsE)) * esz + (prec == GBDW_F16 ? 4 * size_t(LsE) : 0);
  const size_t lb = 8 * link_bytes(prec);
  if (L.mode == 3 || L.mode == 4) return false;  // direct forms: no staging shape
  if (L.mode == 2) {
    // one ring per warp: a warp owns 32/Tps whole sites
    if (Tps > 32 || L.threads % 32 != 0 || L.threads > 256) return false;
    const int nsw = 32 / Tps, W = L.threads / 32;
    const size_t per_warp = size_t(L.stages) * nsw * blk + nsw * lb + ((size_t(L.stages + 1) * 8 + 15) & ~size_t(15));
    if (W * per_warp > max_dynamic_smem()) return false;
    *NS = W * nsw;
    *threads = L.threads;
    *smem = W * per_warp;
    return true;
  }
  if (Tps > 256) return false;
  int ns = L.threads / Tps > 1 ? L.threads / Tps : 1;
  auto round32 = [](int t) { return (t + 31) / 32 * 32; };  // whole warps (grid_sum shuffles)
  while (ns > 1 && round32(ns * Tps) > 256) --ns;
  if (round32(ns * Tps) > 256) return false;
  const size_t sm = size_t(L.stages) * ns * blk + size_t(ns) * lb + size_t(L.stages + 1) * 8;
  if (sm > max_dynamic_smem()) return false;
  *NS = ns;
  *threads = round32(ns * Tps);
  *smem = sm;
  return true;
}

int mdagm_residual(const gbdw_gauge* g, gbdw_field* t, gbdw_field* r, const gbdw_field* p, double M5, double mf,
                   double rr, double out[3]) {
  if (int st = check_operands(g, t, p, true)) return st;
  double* s = cg_scalars();
  if (!s) {
    set_error("CG scalar scratch allocation failed");
    return GBDW_ERR_ALLOC;
  }
  DhopExtra e1;
  e1.sum_to = s;
  e1.num = rr;
  e1.alpha_to = s + 1;
  e1.tune_key = cg_step_key(r->prec);
  if (int st = run_dhop(g, t, p, 0, 1, 5.0 - M5, mf, nullptr, false, nullptr, 0.5, &e1)) return st;
  DhopExtra e2;
  e2.r = r;
  e2.alpha = s + 1;
  e2.sum_to = s + 2;
  e2.tune_key = e1.tune_key;
  if (int st = run_dhop(g, t, t, 1, 1, 5.0 - M5, mf, nullptr, false, nullptr, 0.5, &e2)) return st;
  return fetch_doubles(s, 3, out);
}

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_dhop(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag) {
  if (int st = check_operands(g, out, in, false)) return st;
  return run_dhop(g, out, in, dag ? 1 : 0, 0, 0.0, 0.0, nullptr);
}

int gbdw_dwf_m(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, double M5, double mf, int dag,
               double* norm2) {
  if (int st = check_operands(g, out, in, true)) return st;
  return run_dhop(g, out, in, dag ? 1 : 0, 1, 5.0 - M5, mf, norm2);
}

int gbdw_dwf_mdagm(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double M5, double mf,
                   double* pap) {
  if (int st = check_operands(g, tmp, in, true)) return st;
  if (int st = check_operands(g, out, tmp, true)) return st;
  if (out == in) {
    set_error("gbdw_dwf_mdagm: out must differ from in");
    return GBDW_ERR_INVALID;
  }
  // |M in|^2 is reduced by the first launch and read after the second, so the pair runs
  // without a host round trip in between.
  if (int st = run_dhop(g, tmp, in, 0, 1, 5.0 - M5, mf, pap, false)) return st;
  if (int st = run_dhop(g, out, tmp, 1, 1, 5.0 - M5, mf, nullptr)) return st;
  if (pap) {
    Reduce red;
    if (int st = reduce_scratch(1, 1, &red)) return st;
    return reduce_fetch(red, 1, pap);
  }
  return GBDW_OK;
}

}  // extern "C"
