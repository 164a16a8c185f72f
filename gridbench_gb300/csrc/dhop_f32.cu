// FP32 instantiations of the hopping kernel (FP32 spinor, FP32 9-complex links): direct
// form with 1/2/4 slices per thread, staged form with 1/2 slices and 2/4 stages.
#include "dhop_launch.cuh"

namespace gbdw {
int launch_dhop_f32(const DhopParams& p, int dag, int epi, DhopLaunch L) {
  return dispatch<GBDW_F32, GBDW_F32, GBDW_F32, 1, 2>(p, dag, epi, L);
}
}  // namespace gbdw
