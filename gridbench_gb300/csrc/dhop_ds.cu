// The FP64-accurate hopping operator in double-single arithmetic: FP64 fields and gauge, the
// spin/colour algebra on FP32 pairs (dsfloat.cuh).  GB300 runs FP64 at 1/64 of its FP32 rate, so
// the FP64 kernel is bound by the FP64 pipe, far from its memory roofline; this form moves the
// same bytes and computes on the FP32 pipe, at ~1e-14 relative accuracy.  It serves the solvers'
// FP64 operator (true residuals of the reliable updates, the FP64 CG) by default and any FP64
// operator call on request (gbdw_set_fp64_arith).
#include "dhop_launch.cuh"

namespace gbdw {

namespace {
int g_mode[2] = {GBDW_FP64_NATIVE, GBDW_FP64_DOUBLE_SINGLE};  // operators, solvers
thread_local int g_solver_depth = 0;
thread_local int g_forced = -1;  // Fp64ArithOverride

// one thread per link entry: FP64 complex -> (re h, re l, im h, im l)
__global__ void k_split_links(const double2* __restrict__ U, float4* __restrict__ out, int64_t n) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 a = U[i];
  const dsf r = ds_split(a.x), m = ds_split(a.y);
  out[i] = make_float4(r.h, r.l, m.h, m.l);
}
}  // namespace

SolverScope::SolverScope() { ++g_solver_depth; }
SolverScope::~SolverScope() { --g_solver_depth; }

Fp64ArithOverride::Fp64ArithOverride(int mode) : prev(g_forced) { g_forced = mode; }
Fp64ArithOverride::~Fp64ArithOverride() { g_forced = prev; }

bool fp64_double_single() {
  if (g_forced >= 0) return g_forced == GBDW_FP64_DOUBLE_SINGLE;
  return g_mode[g_solver_depth > 0 ? 1 : 0] == GBDW_FP64_DOUBLE_SINGLE;
}

int ds_links(const gbdw_gauge* g, const void** out) {
  if (g->prec != GBDW_F64) {
    set_error("double-single operator: needs an F64 gauge field");
    return GBDW_ERR_INVALID;
  }
  if (!g->d_ds) {
    const int64_t n = g->lat->nsite * 8 * 9;
    void* d = nullptr;
    cudaError_t e = dev_alloc(&d, size_t(n) * sizeof(float4));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(double-single links)");
    const int t = 256;
    k_split_links<<<unsigned((n + t - 1) / t), t, 0, stream()>>>((const double2*)g->d, (float4*)d, n);
    if ((e = cudaGetLastError()) != cudaSuccess) {
      cudaFree(d);
      return cuda_fail(e, "k_split_links");
    }
    count_launch();
    g->d_ds = d;
  }
  *out = g->d_ds;
  return GBDW_OK;
}

// Direct form, one slice per thread, 128-thread CTAs with registers capped for four CTAs per SM
// (16 warps): the arithmetic is the bound, and warps hide its dependency chains.  Measured at
// 16^4 x Ls=16 (Dhop, ms): 1.075 at this cap, 1.24 at three CTAs (170 registers), 1.79 uncapped
// (254 registers, 8 warps); two slices per thread 1.80-2.56; native FP64 1.635.
// minb: the register cap, as CTAs per SM (4: 128 registers; 3: 170, which spills less in the M
// epilogue); the t-brick order comes in p.brick.
int launch_dhop_ds(const DhopParams& p, int dag, int epi, int minb) {
  if (epi > 1 || (minb != 3 && minb != 4)) {
    set_error("double-single operator: Dhop and M, three or four CTAs per SM");
    return GBDW_ERR_INVALID;
  }
  const int64_t nthreads = p.nsite * p.LsE;
  const unsigned blocks = unsigned((nthreads + DS_THREADS - 1) / DS_THREADS);
#define GBDW_DSK(D, E, MB) k_dhop<GBDW_DS, GBDW_DS, GBDW_DS, D, 1, E, MB, 0, DS_THREADS><<<blocks, DS_THREADS, 0, stream()>>>(p)
  if (minb == 4) {
    if (dag) epi ? GBDW_DSK(1, 1, 4) : GBDW_DSK(1, 0, 4);
    else epi ? GBDW_DSK(0, 1, 4) : GBDW_DSK(0, 0, 4);
  } else {
    if (dag) epi ? GBDW_DSK(1, 1, 3) : GBDW_DSK(1, 0, 3);
    else epi ? GBDW_DSK(0, 1, 3) : GBDW_DSK(0, 0, 3);
  }
#undef GBDW_DSK
  GBDW_LAUNCHED();
  return GBDW_OK;
}

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_set_fp64_arith(int where, int mode) {
  if ((where != GBDW_FP64_OPERATORS && where != GBDW_FP64_SOLVERS) ||
      (mode != GBDW_FP64_NATIVE && mode != GBDW_FP64_DOUBLE_SINGLE)) {
    set_error("gbdw_set_fp64_arith: where GBDW_FP64_OPERATORS / GBDW_FP64_SOLVERS, mode GBDW_FP64_NATIVE / "
              "GBDW_FP64_DOUBLE_SINGLE");
    return GBDW_ERR_INVALID;
  }
  g_mode[where] = mode;
  return GBDW_OK;
}

int gbdw_get_fp64_arith(int where, int* mode) {
  if (!mode || (where != GBDW_FP64_OPERATORS && where != GBDW_FP64_SOLVERS)) return GBDW_ERR_INVALID;
  *mode = g_mode[where];
  return GBDW_OK;
}

}  // extern "C"
