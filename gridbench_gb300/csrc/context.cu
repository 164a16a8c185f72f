// Process-wide state of libgbdw: last error, the library stream, launch counter, device
// scratch, timers and the L2 flush.  One host thread drives the library at a time, as the
// reference's drivers do (bench.cc:59-202); every call is ordered on one CUDA stream.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <atomic>
#include <map>

#include "common.cuh"

namespace gbdw {

namespace {
thread_local std::string g_error;
std::atomic<uint64_t> g_launches{0};
cudaStream_t g_user_stream = nullptr;
cudaStream_t g_own_stream = nullptr;
bool g_have_user_stream = false;
int g_device_checked = 0;  // 0 unknown, 1 ok, -1 none
int g_device = -1;         // the device current when the library first ran (its stream lives there)
int g_num_sms = 0;
// Host-side allocation-failure injection (gbdw_debug_fail_allocs): skip this many more
// device allocations, then fail this many.
std::atomic<long> g_alloc_skip{0};
std::atomic<long> g_alloc_fail{0};

struct ScratchSlot {
  void* p = nullptr;
  size_t bytes = 0;
};
// One table of scratch slots per stream the library queues on (its own stream, or each stream
// given to gbdw_set_stream), so work queued on different streams never shares a buffer.
struct SlotTable {
  ScratchSlot s[12];
};
SlotTable g_scratch_own;
std::map<cudaStream_t, SlotTable> g_scratch_user;
SlotTable& slot_table() { return g_have_user_stream ? g_scratch_user[g_user_stream] : g_scratch_own; }
double* g_pinned = nullptr;
}  // namespace

void set_error(const std::string& msg) { g_error = msg; }

int cuda_fail(cudaError_t e, const char* what) {
  // clear the runtime's record of a non-sticky error so the next launch check does not
  // report it again
  cudaGetLastError();
  char buf[512];
  snprintf(buf, sizeof buf, "CUDA error in %s: %s", what, cudaGetErrorString(e));
  g_error = buf;
  if (e == cudaErrorMemoryAllocation) return GBDW_ERR_ALLOC;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return GBDW_ERR_NO_DEVICE;
  return GBDW_ERR_CUDA;
}

int ensure_device() {
  if (g_device_checked == 1) return GBDW_OK;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    g_device_checked = -1;
    set_error("no CUDA device available: libgbdw has no CPU fallback");
    return GBDW_ERR_NO_DEVICE;
  }
  int dev = 0;
  GBDW_CUDA(cudaGetDevice(&dev));
  GBDW_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
  g_device = dev;
  if (!g_own_stream) GBDW_CUDA(cudaStreamCreateWithFlags(&g_own_stream, cudaStreamNonBlocking));
  if (!g_pinned) GBDW_CUDA(cudaMallocHost((void**)&g_pinned, 64 * sizeof(double)));
  g_device_checked = 1;
  return GBDW_OK;
}

int num_sms() { return g_num_sms > 0 ? g_num_sms : 152; }

int library_device() { return g_device; }

cudaError_t dev_alloc(void** p, size_t bytes) {
  if (g_alloc_fail.load() > 0) {
    if (g_alloc_skip.load() > 0) {
      --g_alloc_skip;
    } else {
      --g_alloc_fail;
      *p = nullptr;
      return cudaErrorMemoryAllocation;  // as cudaMalloc reports an exhausted device
    }
  }
  return cudaMalloc(p, bytes);
}

size_t max_dynamic_smem() {
  static size_t v = 0;
  if (!v) {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) == cudaSuccess && optin > 0)
      v = size_t(optin);
    else
      v = 227 * 1024;
    cudaGetLastError();
  }
  // keep 1 KB for the kernels' static shared memory (reduction scratch, barriers)
  return v - 1024;
}

cudaStream_t stream() { return g_have_user_stream ? g_user_stream : g_own_stream; }

void count_launch(uint64_t n) { g_launches += n; }

void* scratch(size_t bytes, int slot) {
  ScratchSlot& s = slot_table().s[slot];
  if (s.bytes >= bytes && s.p) return s.p;
  if (s.p) {
    cudaStreamSynchronize(stream());
    cudaFree(s.p);
    s.p = nullptr;
    s.bytes = 0;
  }
  size_t want = bytes < (1u << 20) ? (1u << 20) : bytes;
  if (dev_alloc(&s.p, want) != cudaSuccess) {
    cudaGetLastError();
    s.p = nullptr;
    return nullptr;
  }
  // zeroed in stream order: the library's stream does not synchronise with the legacy stream
  if (cudaMemsetAsync(s.p, 0, want, stream()) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(s.p);
    s.p = nullptr;
    return nullptr;
  }
  s.bytes = want;
  return s.p;
}

int reduce_scratch(int64_t nblocks, int width, Reduce* r) {
  void* part = scratch(size_t(nblocks) * size_t(width) * sizeof(double), 0);
  // slot 1: result doubles at +64 (the device error word lives at +2048)
  void* ctl = scratch(4096, 1);
  // slot 8: the two-level reduction's counters, 1 + one per group of kReduceGroup blocks
  void* cnt = scratch((size_t(1) + size_t((nblocks + kReduceGroup - 1) / kReduceGroup)) * sizeof(unsigned), 8);
  if (!part || !ctl || !cnt) {
    set_error("reduction scratch allocation failed");
    return GBDW_ERR_ALLOC;
  }
  r->partials = (double*)part;
  r->counter = (unsigned*)cnt;
  r->result = (double*)((char*)ctl + 64);
  return GBDW_OK;
}

namespace {
__global__ void __launch_bounds__(1024) k_sum_partials(const double* __restrict__ partials, int64_t n,
                                                       double* result, double num, double* alpha_out) {
  double v[1] = {0.0};
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) v[0] += partials[k];
  __shared__ double sh[32][1];
  block_sum_to_thread0<1>(v, sh);
  if (threadIdx.x == 0) {
    result[0] = v[0];
    if (alpha_out) alpha_out[0] = num / v[0];
  }
}
}  // namespace

int sum_partials(const double* partials, int64_t n, double* result, double num, double* alpha_out) {
  k_sum_partials<<<1, 1024, 0, stream()>>>(partials, n, result, num, alpha_out);
  GBDW_LAUNCHED();
  return GBDW_OK;
}

double* cg_scalars() { return (double*)scratch(64, 9); }

int fetch_doubles(const double* dev, int n, double* host) {
  GBDW_CUDA(cudaMemcpyAsync(g_pinned, dev, size_t(n) * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  GBDW_CUDA(cudaStreamSynchronize(stream()));
  for (int k = 0; k < n; ++k) host[k] = g_pinned[k];
  return GBDW_OK;
}

unsigned* device_error_word() {
  void* ctl = scratch(4096, 1);
  return ctl ? (unsigned*)((char*)ctl + 2048) : nullptr;
}

int reduce_fetch(const Reduce& r, int width, double* host) {
  GBDW_CUDA(cudaMemcpyAsync(g_pinned, r.result, size_t(width) * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  GBDW_CUDA(cudaStreamSynchronize(stream()));
  for (int w = 0; w < width; ++w) host[w] = g_pinned[w];
  return GBDW_OK;
}

namespace {
__global__ void k_flush(uint4* p, size_t n, unsigned salt) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    p[i] = make_uint4(unsigned(i) ^ salt, salt, unsigned(i >> 32), 0u);
}
}  // namespace

}  // namespace gbdw

using namespace gbdw;

struct gbdw_timer {
  cudaEvent_t a, b;
};

extern "C" {

const char* gbdw_last_error(void) { return g_error.c_str(); }
int gbdw_version(void) { return 100; }

int gbdw_device_available(void) { return ensure_device() == GBDW_OK ? 1 : 0; }

int gbdw_synchronize(void) {
  if (int st = ensure_device()) return st;
  GBDW_CUDA(cudaStreamSynchronize(stream()));
  unsigned* w = device_error_word();
  if (!w) return GBDW_ERR_ALLOC;
  unsigned h = 0;
  GBDW_CUDA(cudaMemcpy(&h, w, sizeof h, cudaMemcpyDeviceToHost));
  if (h) {
    GBDW_CUDA(cudaMemset(w, 0, sizeof h));
    set_error("a kernel's bounded wait expired (device error word " + std::to_string(h) + ")");
    return GBDW_ERR_TIMEOUT;
  }
  return GBDW_OK;
}

uint64_t gbdw_launch_count(void) { return g_launches.load(); }

int gbdw_set_stream(void* s) {
  g_user_stream = (cudaStream_t)s;
  g_have_user_stream = (s != nullptr);
  return GBDW_OK;
}

int gbdw_stream_create(void** s) {
  if (!s) return GBDW_ERR_INVALID;
  if (int st = ensure_device()) return st;
  cudaStream_t x;
  GBDW_CUDA(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
  *s = (void*)x;
  return GBDW_OK;
}

int gbdw_stream_destroy(void* s) {
  if (!s) return GBDW_OK;
  if (g_have_user_stream && g_user_stream == (cudaStream_t)s) {
    g_have_user_stream = false;
    g_user_stream = nullptr;
  }
  GBDW_CUDA(cudaStreamSynchronize((cudaStream_t)s));
  auto it = g_scratch_user.find((cudaStream_t)s);
  if (it != g_scratch_user.end()) {
    for (ScratchSlot& q : it->second.s)
      if (q.p) cudaFree(q.p);
    g_scratch_user.erase(it);
  }
  GBDW_CUDA(cudaStreamDestroy((cudaStream_t)s));
  return GBDW_OK;
}

int gbdw_timer_create(gbdw_timer** t) {
  if (!t) return GBDW_ERR_INVALID;
  if (int st = ensure_device()) return st;
  gbdw_timer* x = new gbdw_timer;
  if (cudaEventCreate(&x->a) != cudaSuccess || cudaEventCreate(&x->b) != cudaSuccess) {
    delete x;
    return cuda_fail(cudaGetLastError(), "cudaEventCreate");
  }
  *t = x;
  return GBDW_OK;
}
int gbdw_timer_start(gbdw_timer* t) {
  if (!t) return GBDW_ERR_INVALID;
  GBDW_CUDA(cudaEventRecord(t->a, stream()));
  return GBDW_OK;
}
int gbdw_timer_stop(gbdw_timer* t, double* ms) {
  if (!t) return GBDW_ERR_INVALID;
  GBDW_CUDA(cudaEventRecord(t->b, stream()));
  GBDW_CUDA(cudaEventSynchronize(t->b));
  float f = 0.f;
  GBDW_CUDA(cudaEventElapsedTime(&f, t->a, t->b));
  if (ms) *ms = double(f);
  return GBDW_OK;
}
int gbdw_timer_destroy(gbdw_timer* t) {
  if (!t) return GBDW_OK;
  cudaEventDestroy(t->a);
  cudaEventDestroy(t->b);
  delete t;
  return GBDW_OK;
}

int gbdw_flush_l2(size_t nbytes) {
  if (nbytes == 0) return GBDW_OK;
  if (int st = ensure_device()) return st;
  void* p = scratch(nbytes, 7);
  if (!p) {
    set_error("flush buffer allocation failed");
    return GBDW_ERR_ALLOC;
  }
  static unsigned salt = 1;
  k_flush<<<num_sms() * 4, 512, 0, stream()>>>((uint4*)p, nbytes / 16, salt++);
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int gbdw_host_alloc(size_t nbytes, void** ptr) {
  if (!ptr || nbytes == 0) return GBDW_ERR_INVALID;
  if (int st = ensure_device()) return st;
  GBDW_CUDA(cudaMallocHost(ptr, nbytes));
  return GBDW_OK;
}

int gbdw_debug_fail_allocs(int skip, int count) {
  if (skip < 0 || count < 0) {
    set_error("gbdw_debug_fail_allocs: skip and count must be >= 0");
    return GBDW_ERR_INVALID;
  }
  g_alloc_fail = 0;
  g_alloc_skip = skip;
  g_alloc_fail = count;
  return GBDW_OK;
}

int gbdw_host_free(void* ptr) {
  if (!ptr) return GBDW_OK;
  GBDW_CUDA(cudaFreeHost(ptr));
  return GBDW_OK;
}

}  // extern "C"
