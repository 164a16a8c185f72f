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
// try_wait with a suspend-time hint: a waiting thread sleeps (up to 20 us) until the phase
// completes instead of spinning through issue slots the computing warps need.
__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\tselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(20000u)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the phase with the given parity to complete; false after limit_ns.  Between
// polls the warp sleeps briefly, so a waiting warp stops taking issue slots from the warps
// that have data to work on.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, uint64_t limit_ns) {
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (;;) {
    __nanosleep(64);
    if (mbar_try(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

constexpr uint64_t kWaitLimitNs = 1000000000ull;  // 1 s: a copy that has not landed by then never will

template <int P>
struct ESz {
  static constexpr unsigned v = P == GBDW_F64 ? 16 : P == GBDW_F32 ? 8 : 4;
};

// Shared memory: STAGES rings of NS neighbour blocks (+ norms), then the NS sites' links,
// then STAGES+1 mbarriers (the last one for the links).
template <int PIN, int POUT, int GP, int DAG, int N, int EPI, int STAGES>
__global__ void __launch_bounds__(256) k_dhop_tma(const DhopParams p, int NS) {
  using T = typename Arith<PIN>::T;
  extern __shared__ __align__(128) unsigned char smem[];
  const int LsE = p.LsE, LsP = p.LsP;
  const int Tps = LsE / N;
  const unsigned blk = 12u * unsigned(LsP) * ESz<PIN>::v;
  const unsigned nblk = (PIN == GBDW_F16) ? 4u * unsigned(LsE) : 0u;
  const unsigned stage = unsigned(NS) * (blk + nblk);
  constexpr unsigned LB = 8 * LinkIO<GP>::bytes;  // a site's 8 links
  unsigned char* links = smem + STAGES * stage;
  uint64_t* bars = reinterpret_cast<uint64_t*>(links + NS * LB);
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
    bulk_g2s(links + tid * LB, (const unsigned char*)p.U + (site0 + tid) * int64_t(LB), LB, &bars[STAGES]);
  if (tid == 0) mbar_arrive_expect_tx(&bars[STAGES], unsigned(nvalid) * LB);

#pragma unroll
  for (int L = 0; L < STAGES && L < 8; ++L) issue(L, L);

  Acc<PIN, N> acc;
  acc.zero();
  MobLeg ml;
  if constexpr (EPI == 6) ml = make_mobleg(p.Ls, p.mb, p.mc, p.mf, s0);

  int consumed = 0;  // legs whose stage has been waited for
  bool failed = __syncthreads_or(!mbar_wait_bounded(&bars[STAGES], 0, kWaitLimitNs));
  const unsigned char* my_links = links + (active ? sl : 0) * LB;
#define GBDW_TMA_LEG(L)                                                                                     \
  if (!failed) {                                                                                            \
    const int st = (L) % STAGES;                                                                            \
    const bool ok = mbar_wait_bounded(&bars[st], ((L) / STAGES) & 1, kWaitLimitNs);                         \
    failed = __syncthreads_or(!ok);                                                                         \
    if (!failed) {                                                                                          \
      consumed = (L) + 1;                                                                                   \
      const unsigned char* base = smem + st * stage;                                                        \
      if (active) {                                                                                         \
        cpx<T> u[3][3];                                                                                     \
        LinkIO<GP>::template load<true>(my_links, (L), u);                                                  \
        hop_leg<PIN, DAG, N, L, true, EPI == 6>(u, base + sl * blk, 0, s0, LsP,                             \
                                      reinterpret_cast<const float*>(base + NS * blk + sl * nblk) + s0, acc, &ml); \
      }                                                                                                     \
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
    cpx<T> out[N][12];
    acc.unpack(out);
    finish_site<PIN, POUT, DAG, N, EPI>(p, site, s0, LsE, LsP, out, part, dpart);
  }
  if (p.partials) {
    // also reached after a timeout, so every block's partial is written
    double v[1] = {(POUT == GBDW_F64 || (EPI >= 2 && EPI <= 4)) ? dpart : double(part)};
    block_partial<1>(v, p.partials);
  }
}

// ------------------------------------------------------------------ warp-autonomous staged kernel
// Same staging as k_dhop_tma, but every warp runs its own ring: a warp owns NSW = 32/Tps
// sites (Tps = LsE/N threads per site, at most 32), its own STAGES buffers, its own links
// block and its own mbarriers, and synchronises only with __syncwarp.  No CTA-wide barrier
// sits between the legs, so a warp that finished its leg refills its buffer at once.
// Shared memory per warp: STAGES*NSW*(blk+nblk) + NSW*links + (STAGES+1)*8 bytes.
template <int PIN, int GP>
__host__ __device__ inline unsigned tmaw_warp_bytes(int NSW, int LsE, int LsP, int STAGES) {
  const unsigned esz = PIN == GBDW_F64 ? 16u : PIN == GBDW_F32 ? 8u : 4u;
  const unsigned blk = 12u * unsigned(LsP) * esz + (PIN == GBDW_F16 ? 4u * unsigned(LsE) : 0u);
  const unsigned lb = GP == GBDW_F64 ? 8u * 144u : GP == GBDW_F32 ? 8u * 72u : 8u * 24u;
  // barrier area padded to 16 bytes so every warp's buffers stay 16-byte aligned for TMA
  return unsigned(STAGES) * unsigned(NSW) * blk + unsigned(NSW) * lb + ((unsigned(STAGES + 1) * 8u + 15u) & ~15u);
}

template <int PIN, int POUT, int GP, int DAG, int N, int EPI, int STAGES, int LSPC = 0>
__global__ void __launch_bounds__(256) k_dhop_tmaw(const DhopParams p_) {
  using T = typename Arith<PIN>::T;
  extern __shared__ __align__(128) unsigned char smem[];
  DhopParams p = p_;
  if constexpr (LSPC > 0) {
    p.LsE = LSPC;
    p.LsP = LSPC;
  }
  const int LsE = p.LsE, LsP = p.LsP;
  const int Tps = LsE / N;
  const int NSW = 32 / Tps;
  const unsigned blk = 12u * unsigned(LsP) * ESz<PIN>::v;
  const unsigned nblk = (PIN == GBDW_F16) ? 4u * unsigned(LsE) : 0u;
  const unsigned stage = unsigned(NSW) * (blk + nblk);
  constexpr unsigned LB = 8 * LinkIO<GP>::bytes;  // a site's 8 links
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned char* wbase = smem + warp * tmaw_warp_bytes<PIN, GP>(NSW, LsE, LsP, STAGES);
  unsigned char* links = wbase + STAGES * stage;
  uint64_t* bars = reinterpret_cast<uint64_t*>(links + NSW * LB);
  const int64_t site0 = (int64_t(blockIdx.x) * (blockDim.x >> 5) + warp) * NSW;
  const int nvalid = int(max(int64_t(0), min(int64_t(NSW), p.nsite - site0)));
  const int sl = lane / Tps;
  const int s0 = (lane - sl * Tps) * N;
  const bool active = sl < nvalid;
  const unsigned expect = unsigned(nvalid) * (blk + nblk);

  Acc<PIN, N> acc;
  acc.zero();
  MobLeg ml;
  if constexpr (EPI == 6) ml = make_mobleg(p.Ls, p.mb, p.mc, p.mf, s0);
  bool failed = false;
  int consumed = 0;

  if (nvalid > 0) {
    if (lane == 0) {
#pragma unroll
      for (int s = 0; s <= STAGES; ++s) mbar_init(&bars[s], 1);
      fence_mbar_init();
    }
    uint32_t nb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (lane < nvalid) {
      const uint4* q = reinterpret_cast<const uint4*>(p.nbr4 + (site0 + lane) * 8);
      const uint4 a = __ldg(q), b = __ldg(q + 1);
      nb[0] = a.x; nb[1] = a.y; nb[2] = a.z; nb[3] = a.w;
      nb[4] = b.x; nb[5] = b.y; nb[6] = b.z; nb[7] = b.w;
    }
    __syncwarp();
    auto issue = [&](int L, int st) {
      unsigned char* base = wbase + st * stage;
      if (lane < nvalid) {
        const int64_t n = nb[L];
        bulk_g2s(base + lane * blk, (const unsigned char*)p.in + n * blk, blk, &bars[st]);
        if constexpr (PIN == GBDW_F16)
          bulk_g2s(base + NSW * blk + lane * nblk, (const unsigned char*)p.in_norm + n * nblk, nblk, &bars[st]);
      }
      if (lane == 0) mbar_arrive_expect_tx(&bars[st], expect);
    };
    if (lane < nvalid)
      bulk_g2s(links + lane * LB, (const unsigned char*)p.U + (site0 + lane) * int64_t(LB), LB, &bars[STAGES]);
    if (lane == 0) mbar_arrive_expect_tx(&bars[STAGES], unsigned(nvalid) * LB);
#pragma unroll
    for (int L = 0; L < STAGES && L < 8; ++L) issue(L, L);

    failed = __any_sync(0xffffffffu, !mbar_wait_bounded(&bars[STAGES], 0, kWaitLimitNs));
    const unsigned char* my_links = links + (active ? sl : 0) * LB;
#define GBDW_TMAW_LEG(L)                                                                                   \
  if (!failed) {                                                                                           \
    const int st = (L) % STAGES;                                                                           \
    failed = __any_sync(0xffffffffu, !mbar_wait_bounded(&bars[st], ((L) / STAGES) & 1, kWaitLimitNs));    \
    if (!failed) {                                                                                         \
      consumed = (L) + 1;                                                                                  \
      const unsigned char* base = wbase + st * stage;                                                      \
      if (active) {                                                                                        \
        cpx<T> u[3][3];                                                                                    \
        LinkIO<GP>::template load<true>(my_links, (L), u);                                                 \
        hop_leg<PIN, DAG, N, L, true, EPI == 6>(u, base + sl * blk, 0, s0, LsP,                            \
                                      reinterpret_cast<const float*>(base + NSW * blk + sl * nblk) + s0, acc, &ml); \
      }                                                                                                    \
      if ((L) + STAGES < 8) {                                                                              \
        __syncwarp();                                                                                      \
        fence_proxy_async_smem();                                                                          \
        issue((L) + STAGES, st);                                                                           \
      }                                                                                                    \
    }                                                                                                      \
  }
    GBDW_TMAW_LEG(0) GBDW_TMAW_LEG(1) GBDW_TMAW_LEG(2) GBDW_TMAW_LEG(3)
    GBDW_TMAW_LEG(4) GBDW_TMAW_LEG(5) GBDW_TMAW_LEG(6) GBDW_TMAW_LEG(7)
#undef GBDW_TMAW_LEG
    if (failed && lane == 0) {
      atomicOr(p.err, unsigned(GBDW_ERR_TIMEOUT));
      const int issued = min(8, consumed + STAGES);
      for (int L = consumed; L < issued; ++L) mbar_wait_bounded(&bars[L % STAGES], (L / STAGES) & 1, kWaitLimitNs);
      mbar_wait_bounded(&bars[STAGES], 0, kWaitLimitNs);
    }
    __syncwarp();
  }
  float part = 0.f;
  double dpart = 0.0;
  if (active && !failed) {
    const int64_t site = site0 + sl;
    cpx<T> out[N][12];
    acc.unpack(out);
    finish_site<PIN, POUT, DAG, N, EPI>(p, site, s0, LsE, LsP, out, part, dpart);
  }
  if (p.partials) {
    double v[1] = {(POUT == GBDW_F64 || (EPI >= 2 && EPI <= 4)) ? dpart : double(part)};
    block_partial<1>(v, p.partials);
  }
}

}  // namespace gbdw
