// gbdw_norm2_noalloc: the FP64-accumulated squared norm of a device array of complex numbers,
// for callers that cannot allocate device memory.
//
// Who cannot allocate: a host program that hands the GPU's memory to its own pool allocator
// at start-up (a lattice code's memory manager, a framework's caching allocator) and forbids
// other libraries from calling cudaMalloc, or a solver loop that must not pay cudaMalloc's
// latency and implicit synchronisation.  Such a caller owns the input buffer and only needs
// the reduction.  gbdw_norm2 (which works on a gbdw_field and keeps its partial sums in
// library-allocated scratch) cannot serve it; this variant keeps its partial sums, its
// completion counter and its result in the file-scope array below instead, and allocates
// nothing: no cudaMalloc, cudaFree or cudaMallocHost, and no other allocating routine.
//
// Limits and sharing:
//  - at most kNoAllocMaxEntries = 2^24 complex entries per call (one block per 16384
//    entries, 1024 blocks); larger inputs are rejected with GBDW_ERR_INVALID;
//  - every GPU that loads the library holds the array (8.3 KB) until the process exits;
//  - all calls share it: calls whose kernels overlap on the GPU (different streams, or
//    host threads racing) race on it and give wrong sums; calls in one stream are safe.
//    The counter is cleared at the start of every call, so a call never depends on what an
//    earlier call left behind.
//  - the first call on a device looks up the array's device address with
//    cudaGetSymbolAddress (once per device, with that device current);
//  - every call is synchronous: it ends with a copy of the result into host memory and a
//    synchronisation of the library's stream, so no call may be made while a stream is being
//    captured into a CUDA graph;
//  - the kernel runs on the library's stream (gbdw_set_stream selects it), so x must be
//    complete with respect to that stream: a caller that wrote x on another stream
//    synchronises that stream first or hands it to gbdw_set_stream;
//  - like the rest of the library it works on one device, the one current when the library
//    first ran (its stream lives there); once the library has run, a call made with another
//    device current is rejected.
#include <mutex>

#include "common.cuh"

namespace gbdw {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 1024;
constexpr uint64_t kNoAllocChunk = 16384;  // complex entries per block
constexpr uint64_t kNoAllocMaxEntries = uint64_t(kNoAllocMaxBlocks) * kNoAllocChunk;
constexpr int kMaxDevices = 64;

// [0, 1024): per-block partial sums; [1024]: result; [1025]: completion counter (as unsigned)
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocMaxBlocks + 8];

double* g_scratch_addr[kMaxDevices];  // device address of g_noalloc_scratch, per device
std::mutex g_setup_mu;

template <class R>
__global__ void __launch_bounds__(kNoAllocThreads) k_norm2_noalloc(const R* __restrict__ x, uint64_t n,
                                                                  double* scratch) {
  const uint64_t begin = uint64_t(blockIdx.x) * kNoAllocChunk;
  const uint64_t end = begin + kNoAllocChunk < n ? begin + kNoAllocChunk : n;
  double acc[1] = {0.0};
  for (uint64_t i = begin + threadIdx.x; i < end; i += kNoAllocThreads) {
    const double re = double(x[2 * i]), im = double(x[2 * i + 1]);
    acc[0] += re * re + im * im;
  }
  unsigned* counter = reinterpret_cast<unsigned*>(scratch + kNoAllocMaxBlocks + 1);
  grid_sum_flat<1>(acc, scratch, counter, scratch + kNoAllocMaxBlocks);
}

// Device address of the scratch array for the current device (looked up once per device).
int scratch_address(double** out) {
  int dev = 0;
  GBDW_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    set_error("gbdw_norm2_noalloc: device index beyond the supported range");
    return GBDW_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    GBDW_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_addr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_addr[dev];
  return GBDW_OK;
}

}  // namespace
}  // namespace gbdw

using namespace gbdw;

extern "C" int gbdw_norm2_noalloc(const void* x, int prec, uint64_t n, double* result) {
  if (!x || !result || (prec != GBDW_F64 && prec != GBDW_F32)) {
    set_error("gbdw_norm2_noalloc: need a device array x of F64 or F32 complex numbers and a host result pointer");
    return GBDW_ERR_INVALID;
  }
  if (n > kNoAllocMaxEntries) {
    set_error("gbdw_norm2_noalloc: " + std::to_string(n) + " complex entries exceed the maximum of " +
              std::to_string(kNoAllocMaxEntries) + " (the fixed scratch holds 1024 block partials)");
    return GBDW_ERR_INVALID;
  }
  if (n == 0) {
    *result = 0.0;
    return GBDW_OK;
  }
  // no ensure_device() here: its first run allocates (the library's stream and pinned
  // staging); before any other library call the work goes to the legacy default stream
  int dev = 0;
  GBDW_CUDA(cudaGetDevice(&dev));
  if (library_device() >= 0 && dev != library_device()) {
    set_error("gbdw_norm2_noalloc: device " + std::to_string(dev) + " is current, but the library runs on device " +
              std::to_string(library_device()) + " (its stream lives there)");
    return GBDW_ERR_INVALID;
  }
  double* scratch = nullptr;
  if (int st = scratch_address(&scratch)) return st;
  cudaStream_t s = stream();
  // the completion counter must start at zero
  GBDW_CUDA(cudaMemsetAsync(scratch + kNoAllocMaxBlocks + 1, 0, sizeof(double), s));
  const unsigned blocks = unsigned((n + kNoAllocChunk - 1) / kNoAllocChunk);
  if (prec == GBDW_F64)
    k_norm2_noalloc<double><<<blocks, kNoAllocThreads, 0, s>>>(static_cast<const double*>(x), n, scratch);
  else
    k_norm2_noalloc<float><<<blocks, kNoAllocThreads, 0, s>>>(static_cast<const float*>(x), n, scratch);
  GBDW_LAUNCHED();
  GBDW_CUDA(cudaMemcpyAsync(result, scratch + kNoAllocMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, s));
  GBDW_CUDA(cudaStreamSynchronize(s));
  return GBDW_OK;
}
