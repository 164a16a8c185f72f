// FP64 instantiations of the hopping kernel (FP64 spinor, FP64 9-complex links), plus the
// general-table kernel used when a reference table does not factorise into a 4D table.
#include "dhop_kernel.cuh"

namespace gbdw {
namespace {
template <int DAG, int N, int EPI>
int go(const DhopParams& p, DhopLaunch L) {
  const int64_t nthreads = p.nsite * (p.LsE / N);
  const unsigned blocks = unsigned((nthreads + L.threads - 1) / L.threads);
  k_dhop<GBDW_F64, GBDW_F64, GBDW_F64, DAG, N, EPI><<<blocks, L.threads, 0, stream()>>>(p);
  GBDW_LAUNCHED();
  return GBDW_OK;
}
template <int DAG, int EPI>
int by_n(const DhopParams& p, DhopLaunch L) {
  switch (L.spt) {
    case 1: return go<DAG, 1, EPI>(p, L);
    case 2: return go<DAG, 2, EPI>(p, L);
  }
  set_error("FP64 hopping kernel: slices per thread must be 1 or 2");
  return GBDW_ERR_INVALID;
}
}  // namespace

int launch_dhop_f64(const DhopParams& p, int dag, int epi, DhopLaunch L) {
  if (dag) return epi ? by_n<1, 1>(p, L) : by_n<1, 0>(p, L);
  return epi ? by_n<0, 1>(p, L) : by_n<0, 0>(p, L);
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
