// Internal types shared by the libgbdw translation units.
//
// Device layout ("GB300 layout"), chosen so that consecutive threads read consecutive
// addresses and one 4D link serves every fifth-dimension slice of its site:
//   spinor  [site][sc = spin*3+colour][e = s*nrhs + rhs]   complex (F64 16 B, F32 8 B, F16 4 B);
//           F32/F16 store slice pairs as (Re, Re, Im, Im) -- layout.cuh has the addressing --
//           and F16 adds norm[site][e] (FP32, max |re|,|im| over the 24 reals of that 5D site)
//   gauge   [site][mu][row][col] complex, 9 entries (F64/F32) or rows 0-1 only (F16/BF16)
//   nbr4    [site][mu] uint32 neighbour 4D site (fast path)
// "site" runs over 4D sites with SIMD lanes unrolled: site = outer_site*nsimd + lane, so a
// reference table with lane permutes maps onto a plain 4D table.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gbdw.h"

namespace gbdw {

void set_error(const std::string& msg);
int cuda_fail(cudaError_t e, const char* what);
cudaStream_t stream();
void count_launch(uint64_t n = 1);
// Device scratch owned by the library (grown on demand, kept until exit).
void* scratch(size_t bytes, int slot);
int ensure_device();
int num_sms();
// Device the library's stream belongs to (-1 before the first ensure_device()).
int library_device();
// cudaMalloc through the library's one allocation point (honours gbdw_debug_fail_allocs).
cudaError_t dev_alloc(void** p, size_t bytes);
unsigned* device_error_word();  // set by kernels whose bounded waits expired
size_t max_dynamic_smem();      // opt-in dynamic shared memory per CTA, minus room for static

#define GBDW_CUDA(call)                                       \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::gbdw::cuda_fail(e_, #call); \
  } while (0)

#define GBDW_LAUNCHED()                                                  \
  do {                                                                   \
    cudaError_t e_ = cudaGetLastError();                                 \
    if (e_ != cudaSuccess) return ::gbdw::cuda_fail(e_, "kernel launch"); \
    ::gbdw::count_launch();                                              \
  } while (0)

}  // namespace gbdw

struct gbdw_lattice {
  int64_t nsite;     // 4D sites, lanes unrolled
  int Ls;
  int nsimd;
  int dims[4];       // 0 when built from a table
  bool fast;         // 4D factorised table available
  uint32_t* nbr4;    // [nsite][8] (fast)
  uint32_t* nbr5;    // [nsite][Ls][8] neighbour (site*Ls+s) in device numbering (general)
  // Checkerboarded half lattice (even-odd): the sites of one 4D parity of a periodic parent,
  // numbered site = parent_site / 2.  nbr4 then holds neighbour indices into the partner
  // half (the other parity), and cbsite[site] the parent site.
  int parity = -1;                         // -1: not a half lattice
  const gbdw_lattice* parent = nullptr;
  const gbdw_lattice* partner = nullptr;   // the other parity of the same parent
  uint32_t* cbsite = nullptr;              // [nsite] parent site index
};

struct gbdw_gauge {
  const gbdw_lattice* lat;
  int prec;
  void* d;           // device storage
  size_t bytes;
  // F64 gauge: the links split into FP32 pairs (re h, re l, im h, im l per entry) for the
  // double-single operator, built on first use and freed with the gauge
  mutable void* d_ds = nullptr;
};

struct gbdw_field {
  const gbdw_lattice* lat;
  int prec;
  int nrhs;
  int LsE;           // Ls * nrhs, the innermost extent
  int LsP;           // stored slots per row: LsE, rounded up to even for F32/F16
  void* d;           // complex data
  float* norm;       // F16 only
  size_t bytes;
  int64_t elems() const { return lat->nsite * 12 * int64_t(LsP); }  // stored complex slots
};

namespace gbdw {

inline size_t spinor_elem_bytes(int prec) { return prec == GBDW_F64 ? 16 : prec == GBDW_F32 ? 8 : 4; }
inline size_t link_bytes(int prec) {
  return prec == GBDW_F64 ? 144 : prec == GBDW_F32 ? 72 : 24;
}

// ------------------------------------------------------------------ small complex helpers
template <class T>
struct cpx {
  T r, i;
};

template <class T>
__device__ __forceinline__ cpx<T> cmul(cpx<T> a, cpx<T> b) {
  return {a.r * b.r - a.i * b.i, a.r * b.i + a.i * b.r};
}
// acc += a*b
template <class T>
__device__ __forceinline__ void cmac(cpx<T>& acc, cpx<T> a, cpx<T> b) {
  acc.r = fma(a.r, b.r, acc.r);
  acc.r = fma(-a.i, b.i, acc.r);
  acc.i = fma(a.r, b.i, acc.i);
  acc.i = fma(a.i, b.r, acc.i);
}
// Multiply by a compile-time unit c in {+1, -1, +i, -i}: code 0:+1 1:-1 2:+i 3:-i
template <int C, class T>
__device__ __forceinline__ cpx<T> cunit(cpx<T> a) {
  if (C == 0) return a;
  if (C == 1) return {-a.r, -a.i};
  if (C == 2) return {-a.i, a.r};
  return {a.i, -a.r};
}
template <int C>
struct conj_unit {
  static constexpr int v = (C == 2) ? 3 : (C == 3) ? 2 : C;
};

// ------------------------------------------------------------------ device reductions
// Block-wide sums, then "last block finishes" passes over the per-block partials, so the sum
// order is fixed (deterministic) and no second launch is needed.
//
// grid_sum_flat: the last block sums all gridDim partials.  partials holds gridDim.x * W
// doubles, counter one unsigned that must be zero on entry and is left zero.
//
// grid_sum: two levels, so no single block walks thousands of partials after everyone else
// has finished: the last block of each group of kReduceGroup blocks sums its group (the sum
// replaces the group's first partial), and the last group to finish sums the group sums.
// counter holds 1 + ceil(gridDim.x / kReduceGroup) unsigned, zero on entry, left zero.
constexpr unsigned kReduceGroup = 128;

template <int W>
__device__ __forceinline__ void block_sum_to_thread0(double (&v)[W], double (&sh)[32][W]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int w = 0; w < W; ++w) {
    double x = v[w];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if (lane == 0) sh[warp][w] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      double x = 0.0;
      for (int k = 0; k < nw; ++k) x += sh[k][w];
      v[w] = x;
    }
  }
}

// Sum of partials[(first + k*stride)*W + w] for k < n, by the whole block, into thread 0's v.
template <int W>
__device__ __forceinline__ void block_sum_of(const double* partials, unsigned first, unsigned stride, unsigned n,
                                             double (&v)[W], double (&sh)[32][W]) {
#pragma unroll
  for (int w = 0; w < W; ++w) {
    double x = 0.0;
    for (unsigned k = threadIdx.x; k < n; k += blockDim.x)
      x += __ldcg(&partials[size_t(first + k * stride) * W + w]);
    v[w] = x;
  }
  block_sum_to_thread0<W>(v, sh);
}

// Block partials only: thread 0 of every block writes the block's sum to partials[blockIdx];
// a separate one-CTA kernel (sum_partials) adds them up in a fixed order.  For grids of many
// short blocks, where a fence and an atomic per block would hold every block until its
// stores have landed.
template <int W>
__device__ __forceinline__ void block_partial(double (&v)[W], double* partials) {
  __shared__ double sh[32][W];
  block_sum_to_thread0<W>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < W; ++w) partials[size_t(blockIdx.x) * W + w] = v[w];
  }
}

template <int W>
__device__ __forceinline__ void grid_sum_flat(double (&v)[W], double* partials, unsigned* counter,
                                              double* result) {
  __shared__ double sh[32][W];
  __shared__ bool last;
  block_sum_to_thread0<W>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < W; ++w) partials[size_t(blockIdx.x) * W + w] = v[w];
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  block_sum_of<W>(partials, 0, 1, gridDim.x, v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < W; ++w) result[w] = v[w];
    *counter = 0u;
  }
}

template <int W>
__device__ __forceinline__ void grid_sum(double (&v)[W], double* partials, unsigned* counter,
                                         double* result) {
  __shared__ double sh[32][W];
  __shared__ bool last;
  const unsigned g = blockIdx.x / kReduceGroup, g0 = g * kReduceGroup;
  const unsigned ng = (gridDim.x + kReduceGroup - 1) / kReduceGroup;
  const unsigned gsize = min(kReduceGroup, gridDim.x - g0);
  block_sum_to_thread0<W>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < W; ++w) partials[size_t(blockIdx.x) * W + w] = v[w];
    __threadfence();
    const unsigned prev = atomicAdd(&counter[1 + g], 1u);
    last = (prev == gsize - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  block_sum_of<W>(partials, g0, 1, gsize, v, sh);  // this group, fixed order
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < W; ++w) partials[size_t(g0) * W + w] = v[w];
    counter[1 + g] = 0u;
    __threadfence();
    const unsigned prev = atomicAdd(&counter[0], 1u);
    last = (prev == ng - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  block_sum_of<W>(partials, 0, kReduceGroup, ng, v, sh);  // the group sums, fixed order
  if (threadIdx.x == 0) {
#pragma unroll
    for (int w = 0; w < W; ++w) result[w] = v[w];
    counter[0] = 0u;
  }
}

// Scratch slots used for reductions: partial sums and a counter/result block.
struct Reduce {
  double* partials;
  unsigned* counter;
  double* result;
};
int reduce_scratch(int64_t nblocks, int width, Reduce* r);
// result[0] = sum of partials[0..n) in a fixed order (one CTA, on the library stream); with
// alpha_out, also alpha_out[0] = num / result[0] (the CG step length, computed on the device)
int sum_partials(const double* partials, int64_t n, double* result, double num = 0.0, double* alpha_out = nullptr);
// three device doubles for one fused CG step: <p, A p>, alpha, |r|^2 after the update
double* cg_scalars();
// copies n <= 8 device doubles to the host (synchronising the library stream)
int fetch_doubles(const double* dev, int n, double* host);
int reduce_fetch(const Reduce& r, int width, double* host);

}  // namespace gbdw
