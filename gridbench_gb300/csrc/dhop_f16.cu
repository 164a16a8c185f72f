// FP16-storage instantiations of the hopping kernel: half2 spinor with a per-5D-site FP32
// norm, 12-real FP16 or BF16 links, FP32 arithmetic.
#include "dhop_kernel.cuh"

namespace gbdw {
namespace {
template <int GP, int DAG, int N, int EPI>
int go(const DhopParams& p, DhopLaunch L) {
  const int64_t nthreads = p.nsite * (p.LsE / N);
  const unsigned blocks = unsigned((nthreads + L.threads - 1) / L.threads);
  k_dhop<GBDW_F16, GBDW_F16, GP, DAG, N, EPI><<<blocks, L.threads, 0, stream()>>>(p);
  GBDW_LAUNCHED();
  return GBDW_OK;
}
template <int GP, int DAG, int EPI>
int by_n(const DhopParams& p, DhopLaunch L) {
  switch (L.spt) {
    case 1: return go<GP, DAG, 1, EPI>(p, L);
    case 2: return go<GP, DAG, 2, EPI>(p, L);
    case 4: return go<GP, DAG, 4, EPI>(p, L);
  }
  set_error("FP16 hopping kernel: slices per thread must be 1, 2 or 4");
  return GBDW_ERR_INVALID;
}
template <int GP>
int by_g(const DhopParams& p, int dag, int epi, DhopLaunch L) {
  if (dag) return epi ? by_n<GP, 1, 1>(p, L) : by_n<GP, 1, 0>(p, L);
  return epi ? by_n<GP, 0, 1>(p, L) : by_n<GP, 0, 0>(p, L);
}
}  // namespace

int launch_dhop_f16(const DhopParams& p, int gprec, int dag, int epi, DhopLaunch L) {
  if (gprec == GBDW_F16) return by_g<GBDW_F16>(p, dag, epi, L);
  if (gprec == GBDW_BF16) return by_g<GBDW_BF16>(p, dag, epi, L);
  set_error("FP16 spinors pair with F16 or BF16 12-real links");
  return GBDW_ERR_INVALID;
}
}  // namespace gbdw
