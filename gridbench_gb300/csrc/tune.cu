// Autotuner for the hopping kernel: times every admissible launch shape (threads per CTA,
// slices per thread, form, ring stages, and for the direct forms the Ls / RHS tile split and the
// t-brick sweep order) on the caller's own fields with CUDA events and keeps the fastest, keyed by
// (gauge precision, spinor precision, innermost extent Ls*nrhs, epilogue).  The cache can be
// written to and read back from a small JSON object {"key": [threads, slices, form, stages,
// split, brick], ...}.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "eo.h"
#include "tune.h"

namespace gbdw {

namespace {
std::map<std::string, DhopLaunch> g_tuned;
std::mutex g_tune_mu;

std::string key_of(int gprec, int sprec, int LsE, int epi) {
  char buf[96];
  snprintf(buf, sizeof buf, "g%d_s%d_L%d_e%d", gprec, sprec, LsE, epi);
  return buf;
}
}  // namespace

DhopLaunch default_launch(int gprec, int sprec, int LsE, int epi) {
  (void)gprec;
  (void)epi;
  DhopLaunch L{128, 1};
  if (sprec == GBDW_F32) L.spt = (LsE % 2 == 0) ? 2 : 1;
  else if (sprec == GBDW_F16) L.spt = (LsE % 4 == 0) ? 4 : (LsE % 2 == 0) ? 2 : 1;
  return L;
}

DhopLaunch tuned_launch(int gprec, int sprec, int LsE, int epi) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(key_of(gprec, sprec, LsE, epi));
  if (it != g_tuned.end()) return it->second;
  return default_launch(gprec, sprec, LsE, epi);
}

bool find_tuned_launch(int gprec, int sprec, int LsE, int epi, DhopLaunch* L) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tuned.find(key_of(gprec, sprec, LsE, epi));
  if (it == g_tuned.end()) return false;
  *L = it->second;
  return true;
}

void set_tuned_launch(int gprec, int sprec, int LsE, int epi, DhopLaunch L) {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[key_of(gprec, sprec, LsE, epi)] = L;
}

// residual precisions of the fused CG step for an operator on spinors of precision sprec
// (mdagm_residual: FP64 or FP32 r with an FP32 operator, FP32 or, with FP16 links, FP16 r with FP16)
std::vector<int> cg_residual_precs(int gprec, int sprec) {
  if (sprec == GBDW_F32) return {GBDW_F64, GBDW_F32};
  if (sprec == GBDW_F16) return gprec == GBDW_F16 ? std::vector<int>{GBDW_F32, GBDW_F16} : std::vector<int>{GBDW_F32};
  return {};
}

// the shape run_dhop takes for epilogue key epi with this gauge field (half lattices: their own
// entry if one exists)
DhopLaunch lookup(const gbdw_gauge* g, const gbdw_field* in, int epi) {
  DhopLaunch L = tuned_launch(g->prec, in->prec, in->LsE, epi);
  if (g->lat->parity >= 0) find_tuned_launch(g->prec, in->prec, in->LsE, epi + EO_KEY, &L);
  return L;
}

// a pinned shape applies to the hopping term and, with one right-hand side, to M and the CG steps
// (on a half-lattice gauge field: to the even-odd hopping term and its Schur epilogue)
void pin_launch(const gbdw_gauge* g, const gbdw_field* in, const DhopLaunch& L) {
  const int ko = g->lat->parity >= 0 ? EO_KEY : 0;
  set_tuned_launch(g->prec, in->prec, in->LsE, ko, L);
  if (in->nrhs != 1) return;
  set_tuned_launch(g->prec, in->prec, in->LsE, 1 + ko, L);
  if (ko) return;
  for (int rp : cg_residual_precs(g->prec, in->prec)) set_tuned_launch(g->prec, in->prec, in->LsE, cg_step_key(rp), L);
}

bool same_launch(const DhopLaunch& a, const DhopLaunch& b) {
  return a.threads == b.threads && a.spt == b.spt && a.mode == b.mode && a.stages == b.stages && a.split == b.split &&
         a.brick == b.brick;
}

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_tune_dhop(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag) {
  // even-odd operands (gauge and out on one half lattice, in on the other) tune the even-odd
  // hopping term and its Schur-complement epilogue under their own keys
  const bool eo = g && in && g->lat && g->lat->parity >= 0 && in->lat == g->lat->partner;
  if (int st = eo ? check_eo(g, out, in) : check_operands(g, out, in, false)) return st;
  if (!g->lat->fast) return GBDW_OK;  // the general-table kernel has a single shape
  if (int st = ensure_device()) return st;
  const int ko = eo ? EO_KEY : 0;
  // candidate shapes: direct loads with 1/2/4 slices per thread, and the TMA-staged form
  // with the slice splits compiled for this precision and 2 or 4 stages
  std::vector<DhopLaunch> cands;
  const int threads_c[] = {64, 128, 256};
  const int s1 = in->prec == GBDW_F16 ? 2 : 1, s2 = in->prec == GBDW_F16 ? 4 : 2;
  for (int th : threads_c) {
    for (int spt : {1, 2, 4}) {
      if (in->LsE % spt != 0 || (in->prec == GBDW_F64 && spt > 2)) continue;
      // Ls / RHS tiles of the direct form where they cut whole groups: with many right-hand sides
      // a site's slices are many KB and the reuse distance of its spinor (one 3D volume of sites
      // along t) can exceed L2; a tile sweep over all sites shortens it by the split factor
      for (int split : {1, 2, 3, 4, 6, 8, 12, 16}) {
        DhopLaunch L{th, spt, 0, 4, split};
        if (split == 1 || tile_extent(in->LsE, L, false) > 0) cands.push_back(L);
      }
      // t-brick sweep orders (periodic lattices): the other way to shorten the reuse distance,
      // without re-reading links
      for (int brick : {2, 4, 8}) {
        DhopLaunch L{th, spt, 0, 4, 1, brick};
        if (brick_extent(g->lat, L) > 0) cands.push_back(L);
      }
    }
    for (int mode : {1, 2})
      for (int spt : {s1, s2})
        for (int stages : {2, 4}) {
          DhopLaunch L{th, spt, mode, stages};
          int ns, tt;
          size_t sm;
          if (tma_shape(in->prec, in->LsE, L, &ns, &tt, &sm)) cands.push_back(L);
        }
  }
  if (form3_ok(in, 0, 2)) {
    for (int split : {1, 2, 3, 4, 6, 8, 12, 16}) {
      const DhopLaunch L{64, 2, 3, 4, split};
      if (split == 1 || tile_extent(in->LsE, L, false) > 0) cands.push_back(L);
    }
    // t-bricks alone and with tile splits (measured at 24^4 x 12 with 12 right-hand sides: bricks
    // of 4 t-slices swept in 3 tiles beat either alone)
    for (int brick : {2, 4, 8})
      for (int split : {1, 2, 3, 4, 6}) {
        const DhopLaunch L{64, 2, 3, 4, split, brick};
        if (brick_extent(g->lat, L) > 0 && (split == 1 || tile_extent(in->LsE, L, false) > 0)) cands.push_back(L);
      }
  }
  if (blocked_ok(g->lat, in)) cands.push_back(DhopLaunch{128, 2, 4, 4});
  // FP64 fields whose operator calls run the double-single form (gbdw_set_fp64_arith): only that
  // form's shapes are timed
  const bool ds_only = in->prec == GBDW_F64 && g->prec == GBDW_F64 && !eo && fp64_double_single();
  if (ds_only) cands.clear();
  cudaEvent_t a, b;
  GBDW_CUDA(cudaEventCreate(&a));
  GBDW_CUDA(cudaEventCreate(&b));
  gbdw_field* cen = nullptr;  // the even-odd M epilogue's diagonal field (on out's half)
  if (eo && in->nrhs == 1) {
    if (int st = gbdw_field_create(&cen, out->lat, in->prec, 1)) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return st;
    }
  }
  DhopLaunch saved = tuned_launch(g->prec, in->prec, in->LsE, 0);
  if (eo) find_tuned_launch(g->prec, in->prec, in->LsE, ko, &saved);
  DhopLaunch best = saved, best_m = saved;
  float best_ms = 1e30f, best_m_ms = 1e30f;
  int status = GBDW_OK;
  // time reps launches of the hopping term (epi 0) or of M (epi 1) with shape L
  auto apply = [&](int epi) -> int {
    if (!eo) return run_dhop(g, out, in, dag, epi, 1.2, 0.01, nullptr);
    return hop_eo(g, out, in, dag, epi ? cen : nullptr, 1.8, 0.01, epi ? 0.25 : 0.5, nullptr, true);
  };
  auto time_shape = [&](const DhopLaunch& L, int epi, float* ms) -> int {
    set_tuned_launch(g->prec, in->prec, in->LsE, epi + ko, L);
    int st = GBDW_OK;
    for (int w = 0; w < 3 && !st; ++w) st = apply(epi);
    if (st) return st;
    const int reps = 10;
    cudaEventRecord(a, stream());
    for (int r = 0; r < reps && !st; ++r) st = apply(epi);
    cudaEventRecord(b, stream());
    cudaEventSynchronize(b);
    if (st) return st;
    cudaEventElapsedTime(ms, a, b);
    return GBDW_OK;
  };
  // M (one right-hand side) is timed over the same shapes on its own: its epilogue reads the
  // centre site and its 5th-dimension neighbours besides the hopping term's gather.
  DhopLaunch saved_m = tuned_launch(g->prec, in->prec, in->LsE, 1);
  if (eo) find_tuned_launch(g->prec, in->prec, in->LsE, 1 + ko, &saved_m);
  std::vector<std::pair<float, DhopLaunch>> m_times;
  for (const DhopLaunch& L : cands) {
    float ms = 0.f;
    if ((status = time_shape(L, 0, &ms))) break;
    if (ms < best_ms) {
      best_ms = ms;
      best = L;
    }
    if (in->nrhs != 1) continue;
    if ((status = time_shape(L, 1, &ms))) break;
    m_times.push_back({ms, L});
    if (ms < best_m_ms) {
      best_m_ms = ms;
      best_m = L;
    }
  }
  if (!ds_only) {
    set_tuned_launch(g->prec, in->prec, in->LsE, ko, status ? saved : best);
    if (in->nrhs == 1) set_tuned_launch(g->prec, in->prec, in->LsE, 1 + ko, status ? saved_m : best_m);
  }
  // FP64 fields: the double-single form's register cap (three or four CTAs per SM) and t-brick
  // order, for Dhop and M, timed with that form forced
  if (!status && ds_only) {
    Fp64ArithOverride force(GBDW_FP64_DOUBLE_SINGLE);
    for (int epi = 0; epi <= (in->nrhs == 1 ? 1 : 0) && !status; ++epi) {
      DhopLaunch best_ds{DS_THREADS, 1, 0, 4};
      float best_ds_ms = 1e30f;
      for (int minb : {4, 3})
        for (int brick : {1, 2, 4, 8}) {
          const DhopLaunch L{DS_THREADS, 1, 0, minb, 1, brick};
          if (brick > 1 && brick_extent(g->lat, L) == 0) continue;
          set_tuned_launch(g->prec, in->prec, in->LsE, epi + DS_KEY, L);
          for (int w = 0; w < 2 && !status; ++w) status = apply(epi);
          if (status) break;
          cudaEventRecord(a, stream());
          for (int r = 0; r < 5 && !status; ++r) status = apply(epi);
          cudaEventRecord(b, stream());
          cudaEventSynchronize(b);
          if (status) break;
          float ms = 0.f;
          cudaEventElapsedTime(&ms, a, b);
          if (ms < best_ds_ms) {
            best_ds_ms = ms;
            best_ds = L;
          }
        }
      set_tuned_launch(g->prec, in->prec, in->LsE, epi + DS_KEY, best_ds);
    }
  }
  if (cen) gbdw_field_destroy(cen);
  // The fused CG step (mdagm_residual: M with |Mp|^2 and alpha reduced, then M^dag with r updated
  // and |r|^2 reduced) reads and writes r besides M's traffic, so its best shape can differ from
  // M's (measured at 32^4 x 16 with an FP64 r: M alone fastest in t-bricks of 8 on form 3, the CG
  // step 7 % faster on the staged form).  It is timed on the real pass over a shortlist: M's four
  // fastest shapes and the fastest natural-order shape of each form.
  if (!status && !eo && in->nrhs == 1 && !m_times.empty()) {
    std::stable_sort(m_times.begin(), m_times.end(),
                     [](const std::pair<float, DhopLaunch>& x, const std::pair<float, DhopLaunch>& y) {
                       return x.first < y.first;
                     });
    std::vector<DhopLaunch> shortlist;
    auto add = [&](const DhopLaunch& L) {
      for (const DhopLaunch& q : shortlist)
        if (same_launch(q, L)) return;
      shortlist.push_back(L);
    };
    for (size_t i = 0; i < m_times.size() && i < 4; ++i) add(m_times[i].second);
    for (int form = 0; form <= 4; ++form)
      for (const auto& mt : m_times)
        if (mt.second.mode == form && mt.second.split == 1 && mt.second.brick == 1) {
          add(mt.second);
          break;
        }
    for (int rp : cg_residual_precs(g->prec, in->prec)) {
      gbdw_field* r = nullptr;
      if ((status = gbdw_field_create(&r, in->lat, rp, 1))) break;
      const int key = cg_step_key(rp);
      DhopLaunch best_cg = best_m;
      float best_cg_ms = 1e30f;
      for (const DhopLaunch& L : shortlist) {
        set_tuned_launch(g->prec, in->prec, in->LsE, key, L);
        double o3[3];
        for (int w = 0; w < 2 && !status; ++w) status = mdagm_residual(g, out, r, in, 1.8, 0.01, 1.0, o3);
        if (status) break;
        const int reps = 6;
        cudaEventRecord(a, stream());
        for (int k = 0; k < reps && !status; ++k) status = mdagm_residual(g, out, r, in, 1.8, 0.01, 1.0, o3);
        cudaEventRecord(b, stream());
        cudaEventSynchronize(b);
        if (status) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best_cg_ms) {
          best_cg_ms = ms;
          best_cg = L;
        }
      }
      set_tuned_launch(g->prec, in->prec, in->LsE, key, status ? best_m : best_cg);
      gbdw_field_destroy(r);
      if (status) break;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return status;
}

int gbdw_tune_query(const gbdw_gauge* g, const gbdw_field* in, int cfg[4]) {
  if (!g || !in || !cfg) return GBDW_ERR_INVALID;
  const DhopLaunch L = lookup(g, in, 0);
  cfg[0] = L.threads;
  cfg[1] = L.spt;
  cfg[2] = L.mode;
  cfg[3] = L.stages;
  return GBDW_OK;
}

int gbdw_tune_query_m(const gbdw_gauge* g, const gbdw_field* in, int cfg[6]) {
  if (!g || !in || !cfg) return GBDW_ERR_INVALID;
  const DhopLaunch L = lookup(g, in, 1);
  const int v[6] = {L.threads, L.spt, L.mode, L.stages, L.split, L.brick};
  for (int i = 0; i < 6; ++i) cfg[i] = v[i];
  return GBDW_OK;
}

int gbdw_tune_query_cg(const gbdw_gauge* g, const gbdw_field* in, int rprec, int cfg[6]) {
  if (!g || !in || !cfg || rprec < GBDW_F64 || rprec > GBDW_F16) return GBDW_ERR_INVALID;
  DhopLaunch L = lookup(g, in, 1);
  if (g->lat->parity < 0) find_tuned_launch(g->prec, in->prec, in->LsE, cg_step_key(rprec), &L);
  const int v[6] = {L.threads, L.spt, L.mode, L.stages, L.split, L.brick};
  for (int i = 0; i < 6; ++i) cfg[i] = v[i];
  return GBDW_OK;
}

int gbdw_tune_query_ds(const gbdw_gauge* g, const gbdw_field* in, int epi, int cfg[2]) {
  if (!g || !in || !cfg || epi < 0 || epi > 1) return GBDW_ERR_INVALID;
  DhopLaunch L{DS_THREADS, 1, 0, 4};
  find_tuned_launch(g->prec, in->prec, in->LsE, epi + DS_KEY, &L);
  cfg[0] = L.stages;
  cfg[1] = L.brick;
  return GBDW_OK;
}

int gbdw_tune_set_ds(const gbdw_gauge* g, const gbdw_field* in, int epi, int minb, int brick) {
  if (!g || !in || epi < 0 || epi > 1 || (minb != 3 && minb != 4) || brick < 1) return GBDW_ERR_INVALID;
  if (g->prec != GBDW_F64 || in->prec != GBDW_F64) {
    set_error("gbdw_tune_set_ds: the double-single form runs on F64 gauge and spinor fields");
    return GBDW_ERR_INVALID;
  }
  const DhopLaunch L{DS_THREADS, 1, 0, minb, 1, brick};
  if (brick > 1 && brick_extent(g->lat, L) == 0) {
    set_error("gbdw_tune_set_ds: a t-brick needs a periodic lattice whose Lt it divides");
    return GBDW_ERR_INVALID;
  }
  set_tuned_launch(g->prec, in->prec, in->LsE, epi + DS_KEY, L);
  return GBDW_OK;
}

int gbdw_tune_set(const gbdw_gauge* g, const gbdw_field* in, int threads, int spt, int form, int stages) {
  if (!g || !in || threads < 32 || threads > 256 || threads % 32 != 0 || !(spt == 1 || spt == 2 || spt == 4) ||
      in->LsE % spt != 0 || (in->prec == GBDW_F64 && spt > 2) || form < 0 || form > 4 ||
      (stages != 2 && stages != 4)) {
    set_error("gbdw_tune_set: threads 32..256 in steps of 32, spt 1/2/4 dividing Ls*nrhs (<= 2 for F64), "
              "form 0..4, stages 2/4");
    return GBDW_ERR_INVALID;
  }
  const DhopLaunch L{threads, spt, form, stages};
  if (form == 3 && !form3_ok(in, 0, spt)) {
    set_error("gbdw_tune_set: form 3 is the kernel with 2 slices per thread for Ls*nrhs = 16 (FP32/FP16) or "
              "12 / 144 (FP32)");
    return GBDW_ERR_INVALID;
  }
  if (form == 4 && (spt != 2 || !blocked_ok(g->lat, in))) {
    set_error("gbdw_tune_set: form 4 needs FP32/FP16, Ls*nrhs = 16, 2 slices per thread and a periodic lattice "
              "with even extents");
    return GBDW_ERR_INVALID;
  }
  if (form == 1 || form == 2) {
    const int s1 = in->prec == GBDW_F16 ? 2 : 1, s2 = in->prec == GBDW_F16 ? 4 : 2;
    int ns, tt;
    size_t sm;
    if ((spt != s1 && spt != s2) || !tma_shape(in->prec, in->LsE, L, &ns, &tt, &sm)) {
      set_error("gbdw_tune_set: the staged form is not available for this shape");
      return GBDW_ERR_INVALID;
    }
  }
  pin_launch(g, in, L);
  return GBDW_OK;
}

int gbdw_tune_split(const gbdw_gauge* g, const gbdw_field* in, int* split) {
  if (!g || !in || !split) return GBDW_ERR_INVALID;
  *split = lookup(g, in, 0).split;
  return GBDW_OK;
}

int gbdw_tune_set_split(const gbdw_gauge* g, const gbdw_field* in, int split) {
  if (!g || !in) return GBDW_ERR_INVALID;
  DhopLaunch L = lookup(g, in, 0);
  L.split = split;
  if (split < 1 || (split > 1 && tile_extent(in->LsE, L, false) == 0)) {
    set_error("gbdw_tune_set_split: the chosen form must be direct (0 or 3) and Ls*nrhs must split into whole "
              "slice groups");
    return GBDW_ERR_INVALID;
  }
  pin_launch(g, in, L);
  return GBDW_OK;
}

int gbdw_tune_brick(const gbdw_gauge* g, const gbdw_field* in, int* brick) {
  if (!g || !in || !brick) return GBDW_ERR_INVALID;
  *brick = lookup(g, in, 0).brick;
  return GBDW_OK;
}

int gbdw_tune_set_brick(const gbdw_gauge* g, const gbdw_field* in, int brick) {
  if (!g || !in) return GBDW_ERR_INVALID;
  DhopLaunch L = lookup(g, in, 0);
  L.brick = brick;
  if (brick < 1 || (brick > 1 && brick_extent(g->lat, L) == 0)) {
    set_error("gbdw_tune_set_brick: the chosen form must be direct (0 or 3) on a periodic lattice whose Lt the "
              "brick divides");
    return GBDW_ERR_INVALID;
  }
  pin_launch(g, in, L);
  return GBDW_OK;
}

int gbdw_tune_save(const char* path) {
  if (!path) return GBDW_ERR_INVALID;
  FILE* f = fopen(path, "w");
  if (!f) {
    set_error(std::string("cannot write tune cache ") + path);
    return GBDW_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_tune_mu);
  fprintf(f, "{");
  bool first = true;
  for (auto& kv : g_tuned) {
    fprintf(f, "%s\n  \"%s\": [%d, %d, %d, %d, %d, %d]", first ? "" : ",", kv.first.c_str(), kv.second.threads,
            kv.second.spt, kv.second.mode, kv.second.stages, kv.second.split, kv.second.brick);
    first = false;
  }
  fprintf(f, "\n}\n");
  fclose(f);
  return GBDW_OK;
}

int gbdw_tune_load(const char* path) {
  if (!path) return GBDW_ERR_INVALID;
  FILE* f = fopen(path, "r");
  if (!f) {
    set_error(std::string("cannot read tune cache ") + path);
    return GBDW_ERR_INVALID;
  }
  std::string text;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
  fclose(f);
  // Entries look like "g1_s1_L16_e0": [128, 2, 0, 4, 1, 1] (threads, slices per thread, form,
  // stages, tile split, t-brick; shorter entries keep the defaults of the missing numbers)
  size_t pos = 0;
  int loaded = 0;
  while ((pos = text.find('"', pos)) != std::string::npos) {
    const size_t end = text.find('"', pos + 1);
    if (end == std::string::npos) break;
    const std::string key = text.substr(pos + 1, end - pos - 1);
    int gp, sp, LsE, epi, th, spt, mode = 0, stages = 4, split = 1, brick = 1;
    const size_t lb = text.find('[', end);
    if (lb == std::string::npos) break;
    if (sscanf(key.c_str(), "g%d_s%d_L%d_e%d", &gp, &sp, &LsE, &epi) == 4 &&
        sscanf(text.c_str() + lb, "[%d , %d , %d , %d , %d , %d]", &th, &spt, &mode, &stages, &split, &brick) >= 2 &&
        th > 0 && th <= 256 && th % 32 == 0 && (spt == 1 || spt == 2 || spt == 4) && mode >= 0 && mode <= 4 &&
        // the double-single keys hold their register cap (CTAs per SM, 3 or 4) in `stages`
        (stages == 2 || stages == 4 || (epi >= DS_KEY && stages == 3)) && split >= 1 && split <= 64 && brick >= 1 &&
        brick <= 64) {
      set_tuned_launch(gp, sp, LsE, epi, DhopLaunch{th, spt, mode, stages, split, brick});
      ++loaded;
    }
    pos = text.find(']', lb);
    if (pos == std::string::npos) break;
  }
  (void)loaded;
  return GBDW_OK;
}

}  // extern "C"
