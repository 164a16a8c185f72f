// Launch dispatch shared by the per-precision units: maps a runtime (dag, epilogue, slices
// per thread, form, stages) choice onto the compiled kernel instances.
#pragma once
#include "dhop_kernel.cuh"
#include "dhop_tma.cuh"

namespace gbdw {

template <int PIN, int POUT, int GP, int DAG, int N, int EPI>
int go_direct(const DhopParams& p, DhopLaunch L) {
  const int64_t nthreads = p.nsite * (p.LsE / N);
  const unsigned blocks = unsigned((nthreads + L.threads - 1) / L.threads);
  if constexpr (PIN == GBDW_F32 && N == 2) {
    // compile-time row strides for the extents of the benchmarked shapes: Ls = 16, and Ls = 12
    // with one or 12 right-hand sides
    if (p.LsE == p.LsP && (p.LsE == 16 || p.LsE == 12 || p.LsE == 144)) {
      if (p.LsE == 16) k_dhop<PIN, POUT, GP, DAG, N, EPI, 0, 16><<<blocks, L.threads, 0, stream()>>>(p);
      else if (p.LsE == 12) k_dhop<PIN, POUT, GP, DAG, N, EPI, 0, 12><<<blocks, L.threads, 0, stream()>>>(p);
      else k_dhop<PIN, POUT, GP, DAG, N, EPI, 0, 144><<<blocks, L.threads, 0, stream()>>>(p);
      GBDW_LAUNCHED();
      return GBDW_OK;
    }
  }
  k_dhop<PIN, POUT, GP, DAG, N, EPI><<<blocks, L.threads, 0, stream()>>>(p);
  GBDW_LAUNCHED();
  return GBDW_OK;
}

template <int PIN, int POUT, int GP, int DAG, int N, int EPI, int STAGES>
int go_tma(const DhopParams& p, DhopLaunch L) {
  int NS = 0, threads = 0;
  size_t smem = 0;
  if (!tma_shape(PIN, p.LsE, L, &NS, &threads, &smem)) {
    set_error("staged hopping kernel: no admissible shape for this extent");
    return GBDW_ERR_INVALID;
  }
  auto kern = k_dhop_tma<PIN, POUT, GP, DAG, N, EPI, STAGES>;
  static bool opted_in = false;  // one attribute call per instance
  if (!opted_in) {
    cudaFuncAttributes fa;
    GBDW_CUDA(cudaFuncGetAttributes(&fa, kern));
    const size_t limit = max_dynamic_smem() + 1024 - fa.sharedSizeBytes;
    GBDW_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(limit)));
    opted_in = true;
  }
  const unsigned blocks = unsigned((p.nsite + NS - 1) / NS);
  kern<<<blocks, threads, smem, stream()>>>(p, NS);
  GBDW_LAUNCHED();
  return GBDW_OK;
}

template <int PIN, int POUT, int GP, int DAG, int N, int EPI, int STAGES>
int go_tmaw(const DhopParams& p, DhopLaunch L) {
  int NS = 0, threads = 0;
  size_t smem = 0;
  if (!tma_shape(PIN, p.LsE, L, &NS, &threads, &smem)) {
    set_error("warp-staged hopping kernel: no admissible shape for this extent");
    return GBDW_ERR_INVALID;
  }
  auto kern = (PIN == GBDW_F32 && N == 2 && STAGES == 2 && p.LsE == 16 && p.LsP == 16)
                  ? k_dhop_tmaw<PIN, POUT, GP, DAG, N, EPI, STAGES, (PIN == GBDW_F32 && N == 2 && STAGES == 2) ? 16 : 0>
                  : k_dhop_tmaw<PIN, POUT, GP, DAG, N, EPI, STAGES>;
  static const void* opted_in[2] = {nullptr, nullptr};  // one attribute call per instance
  if (opted_in[0] != (const void*)kern && opted_in[1] != (const void*)kern) {
    cudaFuncAttributes fa;
    GBDW_CUDA(cudaFuncGetAttributes(&fa, kern));
    const size_t limit = max_dynamic_smem() + 1024 - fa.sharedSizeBytes;
    GBDW_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(limit)));
    opted_in[opted_in[0] ? 1 : 0] = (const void*)kern;
  }
  const unsigned blocks = unsigned((p.nsite + NS - 1) / NS);
  kern<<<blocks, threads, smem, stream()>>>(p);
  GBDW_LAUNCHED();
  return GBDW_OK;
}

// Slice splits compiled per precision: S1 and S2 for the staged forms.
template <int PIN, int POUT, int GP, int DAG, int EPI, int S1, int S2>
int by_shape(const DhopParams& p, DhopLaunch L) {
  if (L.mode == 1) {
    if (L.spt == S1) return L.stages == 2 ? go_tma<PIN, POUT, GP, DAG, S1, EPI, 2>(p, L) : go_tma<PIN, POUT, GP, DAG, S1, EPI, 4>(p, L);
    if (L.spt == S2) return L.stages == 2 ? go_tma<PIN, POUT, GP, DAG, S2, EPI, 2>(p, L) : go_tma<PIN, POUT, GP, DAG, S2, EPI, 4>(p, L);
  } else if (L.mode == 3) {
    // direct form, Ls*nrhs rows at compile time, 64-thread CTAs, registers balanced for six
    // CTAs per SM (the hoisted loads of the specialised kernel otherwise take ~250 registers)
    if constexpr (PIN == GBDW_F32 || PIN == GBDW_F16) {
      if (L.spt == 2 && p.LsE == 16 && p.LsP == 16) {
        // FP16: 128 registers at eight CTAs per SM (16 warps), no spills, 3 % faster than six;
        // FP32 also fits 128 registers but runs 4 % slower there (64.2 vs 61.5 us at 16^4 x 16:
        // fewer loads in flight per thread), so it keeps the cap of six
        constexpr int MB = PIN == GBDW_F16 ? 8 : 6;
        const unsigned blocks = unsigned((p.nsite * 8 + 63) / 64);
        k_dhop<PIN, POUT, GP, DAG, 2, EPI, MB, 16, 64><<<blocks, 64, 0, stream()>>>(p);
        GBDW_LAUNCHED();
        return GBDW_OK;
      }
    }
    // FP32 Dhop / M at Ls*nrhs = 12 (one rhs at Ls = 12) and 144 (12 rhs at Ls = 12)
    if constexpr (PIN == GBDW_F32 && EPI <= 1) {
      if (L.spt == 2 && p.LsE == p.LsP && (p.LsE == 12 || p.LsE == 144)) {
        const unsigned blocks = unsigned((p.nsite * (p.LsE / 2) + 63) / 64);
        if (p.LsE == 12) k_dhop<PIN, POUT, GP, DAG, 2, EPI, 6, 12, 64><<<blocks, 64, 0, stream()>>>(p);
        else k_dhop<PIN, POUT, GP, DAG, 2, EPI, 6, 144, 64><<<blocks, 64, 0, stream()>>>(p);
        GBDW_LAUNCHED();
        return GBDW_OK;
      }
    }
  } else if (L.mode == 4) {
    if constexpr (PIN == GBDW_F32 || PIN == GBDW_F16) {
      if (L.spt == 2 && p.LsE == 16 && p.LsP == 16 && p.nsite % 16 == 0) {
        k_dhop<PIN, POUT, GP, DAG, 2, EPI, 3, 16, 128, 1><<<unsigned(p.nsite / 16), 128, 0, stream()>>>(p);
        GBDW_LAUNCHED();
        return GBDW_OK;
      }
    }
  } else if (L.mode == 2) {
    if (L.spt == S1) return L.stages == 2 ? go_tmaw<PIN, POUT, GP, DAG, S1, EPI, 2>(p, L) : go_tmaw<PIN, POUT, GP, DAG, S1, EPI, 4>(p, L);
    if (L.spt == S2) return L.stages == 2 ? go_tmaw<PIN, POUT, GP, DAG, S2, EPI, 2>(p, L) : go_tmaw<PIN, POUT, GP, DAG, S2, EPI, 4>(p, L);
  } else {
    if (L.spt == 1) return go_direct<PIN, POUT, GP, DAG, 1, EPI>(p, L);
    if (L.spt == 2) return go_direct<PIN, POUT, GP, DAG, 2, EPI>(p, L);
    if (L.spt == 4 && PIN != GBDW_F64) return go_direct<PIN, POUT, GP, DAG, (PIN == GBDW_F64 ? 2 : 4), EPI>(p, L);
  }
  set_error("hopping kernel: slices per thread not compiled for this precision and form");
  return GBDW_ERR_INVALID;
}

// epi 0 Dhop, 1 M; the CG residual epilogues exist for the adjoint pass only: 2 (FP32 r, FP32
// and FP16 spinors), 3 (FP64 r, FP32 spinors) and 4 (FP16 r, FP16 spinors with FP16 links);
// 6 the forward Mobius M (FP32).
template <int PIN, int POUT, int GP, int S1, int S2>
int dispatch(const DhopParams& p, int dag, int epi, DhopLaunch L) {
  if (epi == 6) {
    // the forward Mobius M (A(b, c) on the loaded neighbours): FP32 slice pairs only
    if constexpr (PIN == GBDW_F32) {
      if (!dag && L.spt == 2) return by_shape<PIN, POUT, GP, 0, 6, S1, S2>(p, L);
    }
    set_error("hopping kernel: the fused Mobius M needs FP32 slice pairs and the forward operator");
    return GBDW_ERR_INVALID;
  }
  if (epi >= 2) {
    if constexpr (PIN == GBDW_F32 || PIN == GBDW_F16) {
      if (dag && epi == 2) return by_shape<PIN, POUT, GP, 1, 2, S1, S2>(p, L);
    }
    if constexpr (PIN == GBDW_F16 && GP == GBDW_F16) {
      if (dag && epi == 4) return by_shape<PIN, POUT, GP, 1, 4, S1, S2>(p, L);
    }
    if constexpr (PIN == GBDW_F32) {
      if (dag && epi == 3) return by_shape<PIN, POUT, GP, 1, 3, S1, S2>(p, L);
    }
    set_error("hopping kernel: residual epilogue not compiled for this precision / direction");
    return GBDW_ERR_INVALID;
  }
  if (dag) return epi ? by_shape<PIN, POUT, GP, 1, 1, S1, S2>(p, L) : by_shape<PIN, POUT, GP, 1, 0, S1, S2>(p, L);
  return epi ? by_shape<PIN, POUT, GP, 0, 1, S1, S2>(p, L) : by_shape<PIN, POUT, GP, 0, 0, S1, S2>(p, L);
}

}  // namespace gbdw
