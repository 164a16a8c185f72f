// Self-test of the bounded-wait machinery used by the staged kernels: one CTA arms an
// mbarrier for 16 bytes that no copy will ever deliver and waits with a short limit.  The
// wait expires, the kernel records GBDW_ERR_TIMEOUT in the device error word and returns;
// the context stays usable and gbdw_synchronize() reports the status.
#include "dhop_tma.cuh"

namespace gbdw {
namespace {
__global__ void k_wait_expires(unsigned* err, uint64_t limit_ns) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, 16);
  const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(err, unsigned(GBDW_ERR_TIMEOUT));
}
}  // namespace
}  // namespace gbdw

using namespace gbdw;

extern "C" int gbdw_selftest_wait_timeout(uint64_t limit_ns) {
  if (int st = ensure_device()) return st;
  unsigned* err = device_error_word();
  if (!err) return GBDW_ERR_ALLOC;
  if (limit_ns > 100000000ull) limit_ns = 100000000ull;
  k_wait_expires<<<1, 32, 0, stream()>>>(err, limit_ns);
  GBDW_LAUNCHED();
  return GBDW_OK;
}
