// FP16-storage instantiations of the hopping kernel: half2 spinor with a per-5D-site FP32
// norm, 12-real FP16 or BF16 links, FP32 arithmetic; staged form with 2/4 slices per thread.
#include "dhop_launch.cuh"

namespace gbdw {
int launch_dhop_f16(const DhopParams& p, int gprec, int dag, int epi, DhopLaunch L) {
  if (gprec == GBDW_F16) return dispatch<GBDW_F16, GBDW_F16, GBDW_F16, 2, 4>(p, dag, epi, L);
  if (gprec == GBDW_BF16) return dispatch<GBDW_F16, GBDW_F16, GBDW_BF16, 2, 4>(p, dag, epi, L);
  set_error("FP16 spinors pair with F16 or BF16 12-real links");
  return GBDW_ERR_INVALID;
}
}  // namespace gbdw
