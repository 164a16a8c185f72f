// TMA-staged hopping kernel.
//
// A CTA owns NS consecutive 4D sites and all their Ls*nrhs slices.  For every leg, the
// neighbour of each of those sites contributes one contiguous block of 12*LsE entries (the
// GB300 layout keeps a site's spinor together), so one cp.async.bulk per (site, leg) moves
// it into shared memory, with completion counted on an mbarrier.  The 8 legs run through a
// STAGES-deep ring of such buffers: while the threads work on leg L out of shared memory,
// the copies for legs L+1..L+STAGES-1 are in flight.  Memory-level parallelism then no longer
// depends on how many registers a thread can spend on outstanding loads.
//
// Every wait on an mbarrier is bounded (wall-clock limit from %globaltimer); on expiry the
// CTA records GBDW_ERR_TIMEOUT in the device error word, waits (bounded again) for the
// copies it issued, and returns without writing its output.
#pragma once
#include "dhop_kernel.cuh"

namespace gbdw {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bulk global -> shared copy (16-byte aligned addresses, size a multiple of 16).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the phase with the given parity to complete; false after limit_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    if (mbar_try(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

constexpr uint64_t kWaitLimitNs = 1000000000ull;  // 1 s: a copy that has not landed by then never will

template <int P>
struct ESz {
  static constexpr unsigned v = P == GBDW_F64 ? 16 : P == GBDW_F32 ? 8 : 4;
};

// Shared-memory loads of N consecutive complex entries (no __ldg: the data is in smem).
template <int P, int N>
__device__ __forceinline__ void lds(const unsigned char* base, int e, cpx<typename Arith<P>::T> (&v)[N]) {
  if constexpr (P == GBDW_F64) {
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const double2 a = reinterpret_cast<const double2*>(base)[e + k];
      v[k] = {a.x, a.y};
    }
  } else if constexpr (P == GBDW_F32) {
    if constexpr (N == 1) {
      const float2 a = reinterpret_cast<const float2*>(base)[e];
      v[0] = {a.x, a.y};
    } else {
#pragma unroll
      for (int k = 0; k < N / 2; ++k) {
        const float4 a = reinterpret_cast<const float4*>(base)[(e >> 1) + k];
        v[2 * k] = {a.x, a.y};
        v[2 * k + 1] = {a.z, a.w};
      }
    }
  } else {
    if constexpr (N == 1) {
      v[0] = h2c(reinterpret_cast<const unsigned*>(base)[e]);
    } else if constexpr (N == 2) {
      const uint2 a = reinterpret_cast<const uint2*>(base)[e >> 1];
      v[0] = h2c(a.x);
      v[1] = h2c(a.y);
    } else {
#pragma unroll
      for (int k = 0; k < N / 4; ++k) {
        const uint4 a = reinterpret_cast<const uint4*>(base)[(e >> 2) + k];
        v[4 * k] = h2c(a.x);
        v[4 * k + 1] = h2c(a.y);
        v[4 * k + 2] = h2c(a.z);
        v[4 * k + 3] = h2c(a.w);
      }
    }
  }
}

// A site's 8 doubled links in shared memory (staged as one block per site).
template <int GP>
struct LinkSmem;
template <>
struct LinkSmem<GBDW_F32> {
  static constexpr unsigned bytes = 8 * 72;
  static __device__ __forceinline__ void load(const unsigned char* site_links, int L, cpx<float> (&u)[3][3]) {
    const float2* p = reinterpret_cast<const float2*>(site_links) + L * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) u[k / 3][k % 3] = {p[k].x, p[k].y};
  }
};
template <>
struct LinkSmem<GBDW_F64> {
  static constexpr unsigned bytes = 8 * 144;
  static __device__ __forceinline__ void load(const unsigned char* site_links, int L, cpx<double> (&u)[3][3]) {
    const double2* p = reinterpret_cast<const double2*>(site_links) + L * 9;
#pragma unroll
    for (int k = 0; k < 9; ++k) u[k / 3][k % 3] = {p[k].x, p[k].y};
  }
};
template <>
struct LinkSmem<GBDW_F16> {
  static constexpr unsigned bytes = 8 * 24;
  static __device__ __forceinline__ void load(const unsigned char* site_links, int L, cpx<float> (&u)[3][3]) {
    const unsigned* p = reinterpret_cast<const unsigned*>(site_links) + L * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) u[k / 3][k % 3] = h2c(p[k]);
    third_row(u);
  }
};
template <>
struct LinkSmem<GBDW_BF16> {
  static constexpr unsigned bytes = 8 * 24;
  static __device__ __forceinline__ void load(const unsigned char* site_links, int L, cpx<float> (&u)[3][3]) {
    const unsigned* p = reinterpret_cast<const unsigned*>(site_links) + L * 6;
#pragma unroll
    for (int k = 0; k < 6; ++k) u[k / 3][k % 3] = b2c(p[k]);
    third_row(u);
  }
};

// One leg from a staged neighbour block (blk: the 12*LsE entries, nrm: its norms for F16)
// with the site's staged links.
template <int PIN, int GP, int DAG, int N, int L, class T>
__device__ __forceinline__ void hop_leg_smem(const unsigned char* site_links, const unsigned char* blk,
                                             const float* nrm, int s0, int LsE, cpx<T> (&acc)[N][12]) {
  using S = LegSpin<DAG ? (L ^ 4) : L>;
  cpx<T> u[3][3];
  LinkSmem<GP>::load(site_links, L, u);
  cpx<T> h0[N][3], h1[N][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    cpx<T> x[N], y[N], z[N], w[N];
    lds<PIN, N>(blk, (0 * 3 + c) * LsE + s0, x);
    lds<PIN, N>(blk, (S::A * 3 + c) * LsE + s0, y);
    lds<PIN, N>(blk, (1 * 3 + c) * LsE + s0, z);
    lds<PIN, N>(blk, (S::B * 3 + c) * LsE + s0, w);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const cpx<T> ya = cunit<S::C0>(y[j]);
      const cpx<T> wb = cunit<S::C1>(w[j]);
      h0[j][c] = {x[j].r + ya.r, x[j].i + ya.i};
      h1[j][c] = {z[j].r + wb.r, z[j].i + wb.i};
    }
  }
  if constexpr (PIN == GBDW_F16) {
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const float nr = nrm[s0 + j];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        h0[j][c].r *= nr;
        h0[j][c].i *= nr;
        h1[j][c].r *= nr;
        h1[j][c].i *= nr;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < N; ++j) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      cpx<T> u0 = {T(0), T(0)}, u1 = {T(0), T(0)};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        cmac(u0, u[r][c], h0[j][c]);
        cmac(u1, u[r][c], h1[j][c]);
      }
      const cpx<T> ra = cunit<conj_unit<S::C0>::v>(u0);
      const cpx<T> rb = cunit<conj_unit<S::C1>::v>(u1);
      acc[j][0 * 3 + r].r += u0.r;
      acc[j][0 * 3 + r].i += u0.i;
      acc[j][1 * 3 + r].r += u1.r;
      acc[j][1 * 3 + r].i += u1.i;
      acc[j][S::A * 3 + r].r += ra.r;
      acc[j][S::A * 3 + r].i += ra.i;
      acc[j][S::B * 3 + r].r += rb.r;
      acc[j][S::B * 3 + r].i += rb.i;
    }
  }
}


// Shared memory: STAGES rings of NS neighbour blocks (+ norms), then the NS sites' links,
// then STAGES+1 mbarriers (the last one for the links).
template <int PIN, int POUT, int GP, int DAG, int N, int EPI, int STAGES>
__global__ void __launch_bounds__(256) k_dhop_tma(const DhopParams p, int NS) {
  using T = typename Arith<PIN>::T;
  extern __shared__ __align__(128) unsigned char smem[];
  const int LsE = p.LsE;
  const int Tps = LsE / N;
  const unsigned blk = 12u * unsigned(LsE) * ESz<PIN>::v;
  const unsigned nblk = (PIN == GBDW_F16) ? 4u * unsigned(LsE) : 0u;
  const unsigned stage = unsigned(NS) * (blk + nblk);
  unsigned char* links = smem + STAGES * stage;
  uint64_t* bars = reinterpret_cast<uint64_t*>(links + NS * LinkSmem<GP>::bytes);
  const int tid = threadIdx.x;
  const int64_t site0 = int64_t(blockIdx.x) * NS;
  const int nvalid = int(min(int64_t(NS), p.nsite - site0));
  const int sl = tid / Tps;
  const int s0 = (tid - sl * Tps) * N;
  const bool active = sl < nvalid;
  const unsigned expect = unsigned(nvalid) * (blk + nblk);

  if (tid == 0) {
#pragma unroll
    for (int s = 0; s <= STAGES; ++s) mbar_init(&bars[s], 1);
    fence_mbar_init();
  }
  // the issuing threads keep their site's 8 neighbours in registers
  uint32_t nb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (tid < nvalid) {
    const uint4* q = reinterpret_cast<const uint4*>(p.nbr4 + (site0 + tid) * 8);
    const uint4 a = __ldg(q), b = __ldg(q + 1);
    nb[0] = a.x; nb[1] = a.y; nb[2] = a.z; nb[3] = a.w;
    nb[4] = b.x; nb[5] = b.y; nb[6] = b.z; nb[7] = b.w;
  }
  __syncthreads();

  auto issue = [&](int L, int st) {
    unsigned char* base = smem + st * stage;
    if (tid < nvalid) {
      const int64_t n = nb[L];
      bulk_g2s(base + tid * blk, (const unsigned char*)p.in + n * blk, blk, &bars[st]);
      if constexpr (PIN == GBDW_F16)
        bulk_g2s(base + NS * blk + tid * nblk, (const unsigned char*)p.in_norm + n * nblk, nblk, &bars[st]);
    }
    if (tid == 0) mbar_arrive_expect_tx(&bars[st], expect);
  };

  // links of the CTA's sites: one block of 8 links per site
  if (tid < nvalid)
    bulk_g2s(links + tid * LinkSmem<GP>::bytes,
             (const unsigned char*)p.U + (site0 + tid) * int64_t(LinkSmem<GP>::bytes), LinkSmem<GP>::bytes,
             &bars[STAGES]);
  if (tid == 0) mbar_arrive_expect_tx(&bars[STAGES], unsigned(nvalid) * LinkSmem<GP>::bytes);

#pragma unroll
  for (int L = 0; L < STAGES && L < 8; ++L) issue(L, L);

  cpx<T> acc[N][12];
#pragma unroll
  for (int j = 0; j < N; ++j)
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[j][k] = {T(0), T(0)};

  int consumed = 0;  // legs whose stage has been waited for
  bool failed = __syncthreads_or(!mbar_wait_bounded(&bars[STAGES], 0, kWaitLimitNs));
  const unsigned char* my_links = links + (active ? sl : 0) * LinkSmem<GP>::bytes;
#define GBDW_TMA_LEG(L)                                                                                     \
  if (!failed) {                                                                                            \
    const int st = (L) % STAGES;                                                                            \
    const bool ok = mbar_wait_bounded(&bars[st], ((L) / STAGES) & 1, kWaitLimitNs);                         \
    failed = __syncthreads_or(!ok);                                                                         \
    if (!failed) {                                                                                          \
      consumed = (L) + 1;                                                                                   \
      const unsigned char* base = smem + st * stage;                                                        \
      if (active)                                                                                           \
        hop_leg_smem<PIN, GP, DAG, N, L>(my_links, base + sl * blk,                                          \
                                         reinterpret_cast<const float*>(base + NS * blk + sl * nblk), s0,   \
                                         LsE, acc);                                                         \
      if ((L) + STAGES < 8) {                                                                               \
        __syncthreads();                                                                                    \
        fence_proxy_async_smem();                                                                           \
        issue((L) + STAGES, st);                                                                            \
      }                                                                                                     \
    }                                                                                                       \
  }
  GBDW_TMA_LEG(0) GBDW_TMA_LEG(1) GBDW_TMA_LEG(2) GBDW_TMA_LEG(3)
  GBDW_TMA_LEG(4) GBDW_TMA_LEG(5) GBDW_TMA_LEG(6) GBDW_TMA_LEG(7)
#undef GBDW_TMA_LEG
  if (failed && tid == 0) {
    atomicOr(p.err, unsigned(GBDW_ERR_TIMEOUT));
    // drain every stage that still has copies in flight before the CTA's smem is released
    const int issued = min(8, consumed + STAGES);
    for (int L = consumed; L < issued; ++L) mbar_wait_bounded(&bars[L % STAGES], (L / STAGES) & 1, kWaitLimitNs);
    mbar_wait_bounded(&bars[STAGES], 0, kWaitLimitNs);  // the link copies
  }
  float part = 0.f;
  double dpart = 0.0;
  if (active && !failed) {
    const int64_t site = site0 + sl;
    if constexpr (EPI == 1) dwf_epilogue<PIN, DAG, N>(p, site, s0, acc);
    part = store_spinor<POUT, N>(p.out, p.out_norm, site * 12 * LsE + s0, site * LsE + s0, LsE, acc);
    if constexpr (POUT == GBDW_F64) dpart = sumsq<N>(acc);
  }
  if (p.partials) {
    // also reached after a timeout, so the grid reduction stays consistent
    double v[1] = {POUT == GBDW_F64 ? dpart : double(part)};
    grid_sum<1>(v, p.partials, p.counter, p.result);
  }
}

}  // namespace gbdw
