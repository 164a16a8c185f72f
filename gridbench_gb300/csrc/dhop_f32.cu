// FP32 instantiations of the hopping kernel (FP32 spinor, FP32 9-complex links).
#include "dhop_kernel.cuh"

namespace gbdw {
namespace {
template <int DAG, int N, int EPI>
int go(const DhopParams& p, DhopLaunch L) {
  const int64_t nthreads = p.nsite * (p.LsE / N);
  const unsigned blocks = unsigned((nthreads + L.threads - 1) / L.threads);
  k_dhop<GBDW_F32, GBDW_F32, GBDW_F32, DAG, N, EPI><<<blocks, L.threads, 0, stream()>>>(p);
  GBDW_LAUNCHED();
  return GBDW_OK;
}
template <int DAG, int EPI>
int by_n(const DhopParams& p, DhopLaunch L) {
  switch (L.spt) {
    case 1: return go<DAG, 1, EPI>(p, L);
    case 2: return go<DAG, 2, EPI>(p, L);
    case 4: return go<DAG, 4, EPI>(p, L);
  }
  set_error("FP32 hopping kernel: slices per thread must be 1, 2 or 4");
  return GBDW_ERR_INVALID;
}
}  // namespace

int launch_dhop_f32(const DhopParams& p, int dag, int epi, DhopLaunch L) {
  if (dag) return epi ? by_n<1, 1>(p, L) : by_n<1, 0>(p, L);
  return epi ? by_n<0, 1>(p, L) : by_n<0, 0>(p, L);
}
}  // namespace gbdw
