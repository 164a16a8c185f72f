// Launch-shape selection for the hopping kernel (threads per CTA, slices per thread).
#pragma once
#include "dhop_kernel.cuh"

namespace gbdw {
// Tuned entry if present, otherwise the built-in default for this precision and extent.
DhopLaunch tuned_launch(int gprec, int sprec, int LsE, int epi);
DhopLaunch default_launch(int gprec, int sprec, int LsE, int epi);
void set_tuned_launch(int gprec, int sprec, int LsE, int epi, DhopLaunch L);
// Optional parts of a hopping launch used by the fused CG step.
struct DhopExtra {
  gbdw_field* r = nullptr;          // with epi 1: r -= (*alpha) M(in) instead of storing M(in)
  const double* alpha = nullptr;    // device
  double* sum_to = nullptr;         // device: where the fused |.|^2 goes (default: the reduce result)
  double num = 0.0;                 // with alpha_to: alpha_to = num / sum
  double* alpha_to = nullptr;       // device
  double c5 = 1.0;                  // the epilogue's 5th-dimension hopping coefficient
  // Mobius operator in one pass: A(mb, mc) on the loaded neighbours (dag 0, FP32) or A(mb, mc)^dag
  // on DhopDag in before the epilogue (dag 1); epi 1, one right-hand side, Ls a power of two <= 64
  bool mobius = false;
  double mb = 1.0, mc = 0.0;
  // a tune-cache key to take the launch shape from when it holds one (else the epilogue's own)
  int tune_key = -1;
};
// tune-cache epilogue keys of the even-odd hopping term (half lattices) are offset by this; a half
// lattice without its own entry takes the full lattice's
constexpr int EO_KEY = 32;
// tune-cache key of the fused CG step (both passes of mdagm_residual) with a residual of precision rprec
inline int cg_step_key(int rprec) { return 16 + rprec; }
// the cached shape for the key, if one was tuned or pinned
bool find_tuned_launch(int gprec, int sprec, int LsE, int epi, DhopLaunch* L);
// cen / khop: the M epilogue's diagonal field (default: in) and hopping coefficient (1/2)
int run_dhop(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag, int epi, double a5, double mf,
             double* norm2, bool fetch = true, const gbdw_field* cen = nullptr, double khop = 0.5,
             const DhopExtra* ex = nullptr);
// The two passes of M^dag M with the CG update of the second fused in:
//   t = M p, s[0] = |t|^2, s[1] = alpha = rr / s[0], r -= alpha M^dag t, s[2] = |r|^2
// (s = cg_scalars(), fetched into out[3] with one synchronisation).
int mdagm_residual(const gbdw_gauge* g, gbdw_field* t, gbdw_field* r, const gbdw_field* p, double M5, double mf,
                   double rr, double out[3]);
int check_operands(const gbdw_gauge* g, const gbdw_field* out, const gbdw_field* in, bool need_single_rhs);
DhopParams make_params(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in);
// form 3 (specialised direct) applies: slice pairs, Ls*nrhs = 16 (FP32/FP16) or 12 / 144 (FP32
// Dhop and M)
bool form3_ok(const gbdw_field* in, int epi, int spt);
// form 4 (blocked site order) applies: FP32/FP16, Ls*nrhs = 16, periodic lattice, even extents
bool blocked_ok(const gbdw_lattice* lat, const gbdw_field* in);
// slices per tile of a direct launch with L.split tiles per site, or 0 (one tile: the split does
// not divide the extent into whole slice groups, a staged or blocked form, or whole_sites)
int tile_extent(int LsE, const DhopLaunch& L, bool whole_sites);
// t-brick of a direct launch on a periodic lattice whose Lt it divides, or 0 (natural order)
int brick_extent(const gbdw_lattice* lat, const DhopLaunch& L);
// the Mobius operator (dag 0) or its adjoint (dag 1) can be fused into the hopping pass for these
// operands (DhopExtra::mobius)
bool mobius_fusable(const gbdw_gauge* g, const gbdw_field* in, int dag);
}  // namespace gbdw
