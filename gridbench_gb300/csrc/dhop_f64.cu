// FP64 instantiations of the hopping kernel (FP64 spinor, FP64 9-complex links; direct form
// with 1/2 slices per thread, staged form with 1/2 slices), plus the
// general-table kernel used when a reference table does not factorise into a 4D table.
#include "dhop_launch.cuh"

namespace gbdw {
int launch_dhop_f64(const DhopParams& p, int dag, int epi, DhopLaunch L) {
  return dispatch<GBDW_F64, GBDW_F64, GBDW_F64, 1, 2>(p, dag, epi, L);
}

int launch_dhop_general(const DhopParams& p, int prec, int dag) {
  const int64_t nthreads = p.nsite * p.Ls;
  const int threads = 128;
  const unsigned blocks = unsigned((nthreads + threads - 1) / threads);
  if (prec == GBDW_F64) {
    if (dag) k_dhop_general<GBDW_F64, GBDW_F64, 1><<<blocks, threads, 0, stream()>>>(p);
    else k_dhop_general<GBDW_F64, GBDW_F64, 0><<<blocks, threads, 0, stream()>>>(p);
  } else if (prec == GBDW_F32) {
    if (dag) k_dhop_general<GBDW_F32, GBDW_F32, 1><<<blocks, threads, 0, stream()>>>(p);
    else k_dhop_general<GBDW_F32, GBDW_F32, 0><<<blocks, threads, 0, stream()>>>(p);
  } else {
    set_error("general-table hopping kernel supports F64 and F32 fields");
    return GBDW_ERR_INVALID;
  }
  GBDW_LAUNCHED();
  return GBDW_OK;
}
}  // namespace gbdw
