// Launch-shape selection for the hopping kernel (threads per CTA, slices per thread).
#pragma once
#include "dhop_kernel.cuh"

namespace gbdw {
// Tuned entry if present, otherwise the built-in default for this precision and extent.
DhopLaunch tuned_launch(int gprec, int sprec, int LsE, int epi);
DhopLaunch default_launch(int gprec, int sprec, int LsE, int epi);
void set_tuned_launch(int gprec, int sprec, int LsE, int epi, DhopLaunch L);
// cen / khop: the M epilogue's diagonal field (default: in) and hopping coefficient (1/2)
int run_dhop(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag, int epi, double a5, double mf,
             double* norm2, bool fetch = true, const gbdw_field* cen = nullptr, double khop = 0.5);
int check_operands(const gbdw_gauge* g, const gbdw_field* out, const gbdw_field* in, bool need_single_rhs);
DhopParams make_params(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in);
// form 4 (blocked site order) applies: FP32/FP16, Ls*nrhs = 16, periodic lattice, even extents
bool blocked_ok(const gbdw_lattice* lat, const gbdw_field* in);
}  // namespace gbdw
