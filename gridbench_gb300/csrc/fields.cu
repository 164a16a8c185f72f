// Lattices, gauge fields and spinor fields on the device, and the conversions between the
// reference layout (dslash_simple.h:3-5, Nsimd lanes per bench.cc:105-139) and the GB300
// layout of common.cuh.
#include <cstring>
#include <vector>

#include "common.cuh"
#include "dhop_kernel.cuh"
#include "layout.cuh"

namespace gbdw {

bool is_device_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool is_pinned_host(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Makes `bytes` of src available on the device: returns src itself for device memory,
// otherwise a copy in scratch slot `slot` (a staging buffer of the current stream).
int stage_in(const void* src, size_t bytes, int slot, const void** dev) {
  if (is_device_ptr(src)) {
    *dev = src;
    return GBDW_OK;
  }
  void* s = scratch(bytes, slot);
  if (!s) {
    set_error("staging buffer allocation failed");
    return GBDW_ERR_ALLOC;
  }
  GBDW_CUDA(cudaMemcpyAsync(s, src, bytes, cudaMemcpyHostToDevice, stream()));
  *dev = s;
  return GBDW_OK;
}

namespace {

__device__ __forceinline__ int lane_mask(int mu, int nsimd) { return nsimd >> (3 - (mu & 3) + 1); }

// Checks a reference table and derives the 4D table.  flags: bit0 out of range,
// bit1 not 4D-factorisable.
__global__ void k_table_check(const uint64_t* nbr, const uint8_t* prm, int64_t nouter, int Ls, int nsimd,
                              uint32_t* nbr4, unsigned* flags) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;  // (o, s, mu)
  if (i >= nouter * Ls * 8) return;
  const int mu = int(i & 7);
  const int64_t os = i >> 3;
  const int64_t o = os / Ls;
  const int s = int(os - o * Ls);
  const uint64_t n = nbr[i];
  const uint64_t n0 = nbr[(o * Ls) * 8 + mu];
  const unsigned p = prm ? prm[i] : 0u;
  const unsigned p0 = prm ? prm[(o * Ls) * 8 + mu] : 0u;
  if (n >= uint64_t(nouter) * uint64_t(Ls)) {
    atomicOr(flags, 1u);
    return;
  }
  if (n0 % uint64_t(Ls) != 0 || n != n0 + uint64_t(s) || p != p0) atomicOr(flags, 2u);
  if (s == 0 && nbr4) {
    const uint64_t no = n0 / uint64_t(Ls);
    for (int lane = 0; lane < nsimd; ++lane) {
      const int nl = p0 ? (lane ^ lane_mask(mu, nsimd)) : lane;
      nbr4[(o * nsimd + lane) * 8 + mu] = uint32_t(no * nsimd + nl);
    }
  }
}

__global__ void k_table_general(const uint64_t* nbr, const uint8_t* prm, int64_t nouter, int Ls, int nsimd,
                                uint32_t* nbr5) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nouter * Ls * 8) return;
  const int mu = int(i & 7);
  const int64_t os = i >> 3;
  const int64_t o = os / Ls;
  const int s = int(os - o * Ls);
  const uint64_t n = nbr[i];
  const unsigned p = prm ? prm[i] : 0u;
  const uint64_t no = n / uint64_t(Ls), sn = n % uint64_t(Ls);
  for (int lane = 0; lane < nsimd; ++lane) {
    const int nl = p ? (lane ^ lane_mask(mu, nsimd)) : lane;
    nbr5[((o * nsimd + lane) * Ls + s) * 8 + mu] = uint32_t((no * nsimd + nl) * Ls + sn);
  }
}

__global__ void k_table_periodic(int4 L, uint32_t* nbr4) {
  const int64_t site = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  const int64_t V = int64_t(L.x) * L.y * L.z * L.w;
  if (site >= V) return;
  int x[4];
  int64_t r = site;
  const int Ld[4] = {L.x, L.y, L.z, L.w};
  for (int d = 0; d < 4; ++d) {
    x[d] = int(r % Ld[d]);
    r /= Ld[d];
  }
  for (int mu = 0; mu < 8; ++mu) {
    const int d = mu & 3;
    int y[4] = {x[0], x[1], x[2], x[3]};
    y[d] = mu < 4 ? (y[d] + 1) % Ld[d] : (y[d] + Ld[d] - 1) % Ld[d];
    nbr4[site * 8 + mu] = uint32_t(y[0] + int64_t(Ld[0]) * (y[1] + int64_t(Ld[1]) * (y[2] + int64_t(Ld[2]) * y[3])));
  }
}

// Reference gauge (complex SRC, nsimd lanes) -> device storage P.
template <class SRC, int P>
__global__ void k_gauge_import(const SRC* src, int64_t nsite, int nsimd, void* dst) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;  // (site, mu)
  if (i >= nsite * 8) return;
  const int64_t site = i >> 3;
  const int mu = int(i & 7);
  const int64_t o = site / nsimd;
  const int lane = int(site - o * nsimd);
  const int nrows = (P == GBDW_F16 || P == GBDW_BF16) ? 2 : 3;
  for (int k = 0; k < nrows * 3; ++k) {
    const int64_t j = ((o * 8 + mu) * 9 + k) * nsimd + lane;
    const double re = double(src[2 * j]), im = double(src[2 * j + 1]);
    if (P == GBDW_F64) {
      ((double2*)dst)[i * 9 + k] = make_double2(re, im);
    } else if (P == GBDW_F32) {
      ((float2*)dst)[i * 9 + k] = make_float2(float(re), float(im));
    } else if (P == GBDW_F16) {
      ((__half2*)dst)[i * 6 + k] = __floats2half2_rn(float(re), float(im));
    } else {
      ((__nv_bfloat162*)dst)[i * 6 + k] = __floats2bfloat162_rn(float(re), float(im));
    }
  }
}

// Reference spinor (complex SRC, nsimd lanes, Ls slices) -> right-hand side `rhs` of a field.
template <class SRC, int P>
__global__ void k_spinor_import(const SRC* src, int64_t nsite, int Ls, int nsimd, int nrhs, int rhs, void* dst,
                                float* norm, int LsP) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;  // (site, s)
  if (i >= nsite * Ls) return;
  const int64_t site = i / Ls;
  const int s = int(i - site * Ls);
  const int64_t o = site / nsimd;
  const int lane = int(site - o * nsimd);
  const int LsE = Ls * nrhs;
  const int e = s * nrhs + rhs;
  double v[24];
  for (int k = 0; k < 12; ++k) {
    const int64_t j = ((o * Ls + s) * 12 + k) * nsimd + lane;
    v[2 * k] = double(src[2 * j]);
    v[2 * k + 1] = double(src[2 * j + 1]);
  }
  if (P == GBDW_F16) {
    float m = 0.f;
    for (int k = 0; k < 24; ++k) m = fmaxf(m, fabsf(float(v[k])));
    const float sc = m > 0.f ? 1.f / m : 0.f;
    norm[site * LsE + e] = m;
    for (int k = 0; k < 12; ++k) Elem<GBDW_F16>::st(dst, site * 12 + k, e, LsP, float(v[2 * k]) * sc, float(v[2 * k + 1]) * sc);
  } else {
    for (int k = 0; k < 12; ++k) Elem<P>::st(dst, site * 12 + k, e, LsP, v[2 * k], v[2 * k + 1]);
  }
}

template <int P>
__device__ __forceinline__ void read_entry(const void* d, const float* norm, int64_t row, int e, int LsP, int64_t nidx,
                                           double& re, double& im) {
  const auto a = Elem<P>::ld(d, row, e, LsP);
  if (P == GBDW_F16) {
    const float n = norm[nidx];
    re = double(float(a.r) * n);
    im = double(float(a.i) * n);
  } else {
    re = double(a.r);
    im = double(a.i);
  }
}

template <class DST, int P>
__global__ void k_spinor_export(const void* srcd, const float* norm, int64_t nsite, int Ls, int nsimd, int nrhs,
                                int rhs, DST* dst, int LsP) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nsite * Ls) return;
  const int64_t site = i / Ls;
  const int s = int(i - site * Ls);
  const int64_t o = site / nsimd;
  const int lane = int(site - o * nsimd);
  const int LsE = Ls * nrhs;
  const int e = s * nrhs + rhs;
  for (int k = 0; k < 12; ++k) {
    double re, im;
    read_entry<P>(srcd, norm, site * 12 + k, e, LsP, site * LsE + e, re, im);
    const int64_t j = ((o * Ls + s) * 12 + k) * nsimd + lane;
    dst[2 * j] = DST(re);
    dst[2 * j + 1] = DST(im);
  }
}

// Site-block conversions for the common case Nsimd = 1, one right-hand side: a site's spinor
// is one contiguous run of 12*Ls entries in both layouts, so one warp per site moves it with
// coalesced 16-byte accesses through shared memory and permutes it there.
template <class SRC, int P>
__global__ void k_import_blocks(const SRC* __restrict__ src, int64_t nsite, int Ls, void* dst, float* norm, int LsP) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t site = int64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
  if (site >= nsite) return;
  const int nreal = 24 * Ls;  // reals of the site block
  SRC* buf = reinterpret_cast<SRC*>(sm) + size_t(warp) * nreal;
  const SRC* s = src + site * nreal;
  constexpr int V = 16 / sizeof(SRC);  // reals per 16-byte vector
  for (int i = lane; i < nreal / V; i += 32) reinterpret_cast<uint4*>(buf)[i] = __ldg(reinterpret_cast<const uint4*>(s) + i);
  __syncwarp();
  for (int e = lane; e < Ls; e += 32) {
    const SRC* v = buf + e * 24;
    if (P == GBDW_F16) {
      float m = 0.f;
      for (int k = 0; k < 24; ++k) m = fmaxf(m, fabsf(float(v[k])));
      const float sc = m > 0.f ? 1.f / m : 0.f;
      norm[site * Ls + e] = m;
      for (int k = 0; k < 12; ++k) Elem<GBDW_F16>::st(dst, site * 12 + k, e, LsP, float(v[2 * k]) * sc, float(v[2 * k + 1]) * sc);
    } else {
      for (int k = 0; k < 12; ++k) Elem<P>::st(dst, site * 12 + k, e, LsP, v[2 * k], v[2 * k + 1]);
    }
  }
}

template <class DST, int P>
__global__ void k_export_blocks(const void* __restrict__ srcd, const float* __restrict__ norm, int64_t nsite, int Ls,
                                DST* __restrict__ dst, int LsP) {
  extern __shared__ __align__(16) unsigned char sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t site = int64_t(blockIdx.x) * (blockDim.x >> 5) + warp;
  if (site >= nsite) return;
  const int nreal = 24 * Ls;
  DST* buf = reinterpret_cast<DST*>(sm) + size_t(warp) * nreal;
  for (int e = lane; e < Ls; e += 32) {
    const float n = (P == GBDW_F16) ? __ldg(norm + site * Ls + e) : 1.f;
    for (int k = 0; k < 12; ++k) {
      const auto a = Elem<P>::ld(srcd, site * 12 + k, e, LsP);
      buf[e * 24 + 2 * k] = (P == GBDW_F16) ? DST(float(a.r) * n) : DST(a.r);
      buf[e * 24 + 2 * k + 1] = (P == GBDW_F16) ? DST(float(a.i) * n) : DST(a.i);
    }
  }
  __syncwarp();
  constexpr int V = 16 / sizeof(DST);
  uint4* d = reinterpret_cast<uint4*>(dst + site * nreal);
  for (int i = lane; i < nreal / V; i += 32) d[i] = reinterpret_cast<const uint4*>(buf)[i];
}

// Field-to-field precision conversion, one thread per 5D entry (site, e).
template <int PS, int PD>
__global__ void k_field_convert(const void* src, const float* snorm, void* dst, float* dnorm, int64_t nsite, int LsE,
                                int LsPs, int LsPd) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= nsite * LsE) return;
  const int64_t site = i / LsE;
  const int e = int(i - site * LsE);
  double v[24];
  for (int k = 0; k < 12; ++k) read_entry<PS>(src, snorm, site * 12 + k, e, LsPs, i, v[2 * k], v[2 * k + 1]);
  if (PD == GBDW_F16) {
    float m = 0.f;
    for (int k = 0; k < 24; ++k) m = fmaxf(m, fabsf(float(v[k])));
    const float sc = m > 0.f ? 1.f / m : 0.f;
    dnorm[i] = m;
    for (int k = 0; k < 12; ++k) Elem<GBDW_F16>::st(dst, site * 12 + k, e, LsPd, float(v[2 * k]) * sc, float(v[2 * k + 1]) * sc);
  } else {
    for (int k = 0; k < 12; ++k) Elem<PD>::st(dst, site * 12 + k, e, LsPd, v[2 * k], v[2 * k + 1]);
  }
}

inline unsigned nblk(int64_t n, int t) { return unsigned((n + t - 1) / t); }

}  // namespace

int field_convert(gbdw_field* dst, const gbdw_field* src) {
  const int64_t n = src->lat->nsite * src->LsE;
  if (n == 0) return GBDW_OK;
  const int t = 256;
#define GBDW_CONV(PS, PD) \
  k_field_convert<PS, PD><<<nblk(n, t), t, 0, stream()>>>(src->d, src->norm, dst->d, dst->norm, src->lat->nsite, src->LsE, \
                                                          src->LsP, dst->LsP)
  const int key = src->prec * 4 + dst->prec;
  switch (key) {
    case GBDW_F64 * 4 + GBDW_F32: GBDW_CONV(GBDW_F64, GBDW_F32); break;
    case GBDW_F64 * 4 + GBDW_F16: GBDW_CONV(GBDW_F64, GBDW_F16); break;
    case GBDW_F32 * 4 + GBDW_F64: GBDW_CONV(GBDW_F32, GBDW_F64); break;
    case GBDW_F32 * 4 + GBDW_F16: GBDW_CONV(GBDW_F32, GBDW_F16); break;
    case GBDW_F16 * 4 + GBDW_F64: GBDW_CONV(GBDW_F16, GBDW_F64); break;
    case GBDW_F16 * 4 + GBDW_F32: GBDW_CONV(GBDW_F16, GBDW_F32); break;
    case GBDW_F64 * 4 + GBDW_F64:
    case GBDW_F32 * 4 + GBDW_F32:
      GBDW_CUDA(cudaMemcpyAsync(dst->d, src->d, src->bytes, cudaMemcpyDeviceToDevice, stream()));
      return GBDW_OK;
    case GBDW_F16 * 4 + GBDW_F16:
      GBDW_CUDA(cudaMemcpyAsync(dst->d, src->d, src->bytes, cudaMemcpyDeviceToDevice, stream()));
      GBDW_CUDA(cudaMemcpyAsync(dst->norm, src->norm, size_t(n) * sizeof(float), cudaMemcpyDeviceToDevice, stream()));
      return GBDW_OK;
    default:
      set_error("unsupported field conversion");
      return GBDW_ERR_INVALID;
  }
#undef GBDW_CONV
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int lattice_from_table_impl(gbdw_lattice** out, uint64_t nouter, int Ls, int nsimd, const uint64_t* nbr,
                            const uint8_t* prm, bool force_general) {
  if (!out || !nbr || nouter == 0 || Ls < 1 || !(nsimd == 1 || nsimd == 2 || nsimd == 4 || nsimd == 8 || nsimd == 16)) {
    set_error("gbdw_lattice_from_table: invalid arguments");
    return GBDW_ERR_INVALID;
  }
  if (double(nouter) * nsimd * Ls * 12 >= 2147483647.0) {
    set_error("gbdw_lattice_from_table: lattice too large for 32-bit site indexing");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const int64_t nent = int64_t(nouter) * Ls * 8;
  const void* dnbr = nullptr;
  const void* dprm = nullptr;
  if (int st = stage_in(nbr, size_t(nent) * 8, 2, &dnbr)) return st;
  if (prm)
    if (int st = stage_in(prm, size_t(nent), 3, &dprm)) return st;
  gbdw_lattice* L = new gbdw_lattice();
  L->nsite = int64_t(nouter) * nsimd;
  L->Ls = Ls;
  L->nsimd = nsimd;
  L->nbr4 = nullptr;
  L->nbr5 = nullptr;
  unsigned* dflags = (unsigned*)scratch(64, 4);
  if (!dflags) {
    delete L;
    set_error("flag allocation failed");
    return GBDW_ERR_ALLOC;
  }
  auto fail = [&](int st) {
    if (L->nbr4) cudaFree(L->nbr4);
    if (L->nbr5) cudaFree(L->nbr5);
    delete L;
    return st;
  };
  cudaError_t e = dev_alloc((void**)&L->nbr4, size_t(L->nsite) * 8 * sizeof(uint32_t));
  if (e != cudaSuccess) return fail(cuda_fail(e, "cudaMalloc(nbr4)"));
  if ((e = cudaMemsetAsync(dflags, 0, sizeof(unsigned), stream())) != cudaSuccess) return fail(cuda_fail(e, "memset"));
  k_table_check<<<nblk(nent, 256), 256, 0, stream()>>>((const uint64_t*)dnbr, (const uint8_t*)dprm, int64_t(nouter), Ls,
                                                        nsimd, L->nbr4, dflags);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(cuda_fail(e, "k_table_check"));
  count_launch();
  unsigned flags = 0;
  if ((e = cudaMemcpyAsync(&flags, dflags, sizeof(unsigned), cudaMemcpyDeviceToHost, stream())) != cudaSuccess)
    return fail(cuda_fail(e, "flags"));
  if ((e = cudaStreamSynchronize(stream())) != cudaSuccess) return fail(cuda_fail(e, "sync"));
  if (flags & 1u) {
    set_error("neighbour table entry out of range (>= nsite*Ls)");
    return fail(GBDW_ERR_TABLE);
  }
  L->fast = !(flags & 2u) && !force_general;
  if (!L->fast) {
    e = dev_alloc((void**)&L->nbr5, size_t(L->nsite) * Ls * 8 * sizeof(uint32_t));
    if (e != cudaSuccess) return fail(cuda_fail(e, "cudaMalloc(nbr5)"));
    k_table_general<<<nblk(nent, 256), 256, 0, stream()>>>((const uint64_t*)dnbr, (const uint8_t*)dprm, int64_t(nouter),
                                                            Ls, nsimd, L->nbr5);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(cuda_fail(e, "k_table_general"));
    count_launch();
  }
  for (int d = 0; d < 4; ++d) L->dims[d] = 0;
  *out = L;
  return GBDW_OK;
}

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_lattice_from_table(gbdw_lattice** lat, uint64_t nsite, int Ls, int nsimd, const uint64_t* nbr,
                            const uint8_t* prm) {
  return lattice_from_table_impl(lat, nsite, Ls, nsimd, nbr, prm, false);
}

int gbdw_lattice_create(gbdw_lattice** lat, const int dims[4], int Ls) {
  if (!lat || !dims || Ls < 1) {
    set_error("gbdw_lattice_create: invalid arguments");
    return GBDW_ERR_INVALID;
  }
  int64_t V = 1;
  for (int d = 0; d < 4; ++d) {
    if (dims[d] < 1) {
      set_error("gbdw_lattice_create: dims must be >= 1");
      return GBDW_ERR_INVALID;
    }
    V *= dims[d];
  }
  if (double(V) * Ls * 12 >= 2147483647.0) {
    set_error("gbdw_lattice_create: lattice too large for 32-bit site indexing");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  gbdw_lattice* L = new gbdw_lattice();
  L->nsite = V;
  L->Ls = Ls;
  L->nsimd = 1;
  L->fast = true;
  L->nbr5 = nullptr;
  for (int d = 0; d < 4; ++d) L->dims[d] = dims[d];
  cudaError_t e = dev_alloc((void**)&L->nbr4, size_t(V) * 8 * sizeof(uint32_t));
  if (e != cudaSuccess) {
    delete L;
    return cuda_fail(e, "cudaMalloc(nbr4)");
  }
  k_table_periodic<<<nblk(V, 256), 256, 0, stream()>>>(make_int4(dims[0], dims[1], dims[2], dims[3]), L->nbr4);
  if ((e = cudaGetLastError()) != cudaSuccess) {
    cudaFree(L->nbr4);
    delete L;
    return cuda_fail(e, "k_table_periodic");
  }
  count_launch();
  *lat = L;
  return GBDW_OK;
}

int gbdw_lattice_destroy(gbdw_lattice* lat) {
  if (!lat) return GBDW_OK;
  cudaStreamSynchronize(stream());
  if (lat->nbr4) cudaFree(lat->nbr4);
  if (lat->nbr5) cudaFree(lat->nbr5);
  if (lat->cbsite) cudaFree(lat->cbsite);
  delete lat;
  return GBDW_OK;
}

int gbdw_lattice_info(const gbdw_lattice* lat, int64_t info[4]) {
  if (!lat || !info) return GBDW_ERR_INVALID;
  info[0] = lat->nsite;
  info[1] = lat->Ls;
  info[2] = lat->nsimd;
  info[3] = lat->fast ? 1 : 0;
  return GBDW_OK;
}

int gbdw_gauge_create(gbdw_gauge** g, const gbdw_lattice* lat, int prec, const void* src, int src_prec) {
  if (!g || !lat || !src || prec < GBDW_F64 || prec > GBDW_BF16 || (src_prec != GBDW_F64 && src_prec != GBDW_F32)) {
    set_error("gbdw_gauge_create: invalid arguments");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const int64_t nlink = lat->nsite * 8;
  const size_t src_bytes = size_t(nlink) * 9 * (src_prec == GBDW_F64 ? 16 : 8);
  const void* dsrc = nullptr;
  if (int st = stage_in(src, src_bytes, 2, &dsrc)) return st;
  gbdw_gauge* G = new gbdw_gauge();
  G->lat = lat;
  G->prec = prec;
  G->bytes = size_t(nlink) * link_bytes(prec);
  cudaError_t e = dev_alloc((void**)&G->d, G->bytes);
  if (e != cudaSuccess) {
    delete G;
    return cuda_fail(e, "cudaMalloc(gauge)");
  }
  const int t = 256;
  const int64_t nsite = lat->nsite;
  const int ns = lat->nsimd;
#define GBDW_GI(SRC, P) k_gauge_import<SRC, P><<<nblk(nlink, t), t, 0, stream()>>>((const SRC*)dsrc, nsite, ns, G->d)
  if (src_prec == GBDW_F64) {
    switch (prec) {
      case GBDW_F64: GBDW_GI(double, GBDW_F64); break;
      case GBDW_F32: GBDW_GI(double, GBDW_F32); break;
      case GBDW_F16: GBDW_GI(double, GBDW_F16); break;
      default: GBDW_GI(double, GBDW_BF16); break;
    }
  } else {
    switch (prec) {
      case GBDW_F64: GBDW_GI(float, GBDW_F64); break;
      case GBDW_F32: GBDW_GI(float, GBDW_F32); break;
      case GBDW_F16: GBDW_GI(float, GBDW_F16); break;
      default: GBDW_GI(float, GBDW_BF16); break;
    }
  }
#undef GBDW_GI
  if ((e = cudaGetLastError()) != cudaSuccess) {
    cudaFree(G->d);
    delete G;
    return cuda_fail(e, "k_gauge_import");
  }
  count_launch();
  *g = G;
  return GBDW_OK;
}

int gbdw_gauge_destroy(gbdw_gauge* g) {
  if (!g) return GBDW_OK;
  cudaStreamSynchronize(stream());
  cudaFree(g->d);
  if (g->d_ds) cudaFree(g->d_ds);
  delete g;
  return GBDW_OK;
}

int gbdw_field_create(gbdw_field** f, const gbdw_lattice* lat, int prec, int nrhs) {
  if (!f || !lat || prec < GBDW_F64 || prec > GBDW_F16 || nrhs < 1) {
    set_error("gbdw_field_create: invalid arguments");
    return GBDW_ERR_INVALID;
  }
  if (double(lat->nsite) * lat->Ls * nrhs * 12 >= 2147483647.0) {
    set_error("gbdw_field_create: field too large for 32-bit indexing");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  gbdw_field* F = new gbdw_field();
  F->lat = lat;
  F->prec = prec;
  F->nrhs = nrhs;
  F->LsE = lat->Ls * nrhs;
  F->LsP = padded_slices(prec, F->LsE);
  F->norm = nullptr;
  F->bytes = size_t(F->elems()) * spinor_elem_bytes(prec);
  cudaError_t e = dev_alloc((void**)&F->d, F->bytes);
  if (e != cudaSuccess) {
    delete F;
    return cuda_fail(e, "cudaMalloc(field)");
  }
  if (prec == GBDW_F16) {
    e = dev_alloc((void**)&F->norm, size_t(lat->nsite) * F->LsE * sizeof(float));
    if (e != cudaSuccess) {
      cudaFree(F->d);
      delete F;
      return cuda_fail(e, "cudaMalloc(norm)");
    }
  }
  *f = F;
  return gbdw_field_zero(F);
}

int gbdw_field_destroy(gbdw_field* f) {
  if (!f) return GBDW_OK;
  cudaStreamSynchronize(stream());
  cudaFree(f->d);
  if (f->norm) cudaFree(f->norm);
  delete f;
  return GBDW_OK;
}

int gbdw_field_zero(gbdw_field* f) {
  if (!f) return GBDW_ERR_INVALID;
  GBDW_CUDA(cudaMemsetAsync(f->d, 0, f->bytes, stream()));
  if (f->norm) GBDW_CUDA(cudaMemsetAsync(f->norm, 0, size_t(f->lat->nsite) * f->LsE * sizeof(float), stream()));
  return GBDW_OK;
}

int gbdw_field_import(gbdw_field* f, int rhs, const void* src, int src_prec) {
  if (!f || !src || rhs < 0 || rhs >= f->nrhs || (src_prec != GBDW_F64 && src_prec != GBDW_F32)) {
    set_error("gbdw_field_import: invalid arguments");
    return GBDW_ERR_INVALID;
  }
  const gbdw_lattice* L = f->lat;
  const int64_t n5 = L->nsite * L->Ls;
  const size_t bytes = size_t(n5) * 12 * (src_prec == GBDW_F64 ? 16 : 8);
  const int t = 256;
  // site blocks: 4 warps per CTA, 24*Ls reals of shared memory per warp
  const size_t blk_smem = 4 * size_t(24) * L->Ls * (src_prec == GBDW_F64 ? 8 : 4);
  const bool blocks = L->nsimd == 1 && f->nrhs == 1 && blk_smem <= 48 * 1024;
  // host memory goes through a copy engine into the stream's staging buffer: the copy needs
  // no SMs, so copies of work queued on other streams overlap with it
  const void* dsrc = nullptr;
  if (int st = stage_in(src, bytes, 5, &dsrc)) return st;
  if (blocks && (uintptr_t(dsrc) & 15) == 0) {
    const unsigned nb = unsigned((L->nsite + 3) / 4);
#define GBDW_IB(SRC, P) \
  k_import_blocks<SRC, P><<<nb, 128, blk_smem, stream()>>>((const SRC*)dsrc, L->nsite, L->Ls, f->d, f->norm, f->LsP)
    if (src_prec == GBDW_F64) {
      if (f->prec == GBDW_F64) GBDW_IB(double, GBDW_F64);
      else if (f->prec == GBDW_F32) GBDW_IB(double, GBDW_F32);
      else GBDW_IB(double, GBDW_F16);
    } else {
      if (f->prec == GBDW_F64) GBDW_IB(float, GBDW_F64);
      else if (f->prec == GBDW_F32) GBDW_IB(float, GBDW_F32);
      else GBDW_IB(float, GBDW_F16);
    }
#undef GBDW_IB
    GBDW_LAUNCHED();
    return GBDW_OK;
  }
#define GBDW_SI(SRC, P)                                                                                      \
  k_spinor_import<SRC, P><<<nblk(n5, t), t, 0, stream()>>>((const SRC*)dsrc, L->nsite, L->Ls, L->nsimd, f->nrhs, rhs, \
                                                          f->d, f->norm, f->LsP)
  if (src_prec == GBDW_F64) {
    if (f->prec == GBDW_F64) GBDW_SI(double, GBDW_F64);
    else if (f->prec == GBDW_F32) GBDW_SI(double, GBDW_F32);
    else GBDW_SI(double, GBDW_F16);
  } else {
    if (f->prec == GBDW_F64) GBDW_SI(float, GBDW_F64);
    else if (f->prec == GBDW_F32) GBDW_SI(float, GBDW_F32);
    else GBDW_SI(float, GBDW_F16);
  }
#undef GBDW_SI
  GBDW_LAUNCHED();
  return GBDW_OK;
}

static int field_export(const gbdw_field* f, int rhs, void* dst, int dst_prec, bool sync) {
  if (!f || !dst || rhs < 0 || rhs >= f->nrhs || (dst_prec != GBDW_F64 && dst_prec != GBDW_F32)) {
    set_error("gbdw_field_export: invalid arguments");
    return GBDW_ERR_INVALID;
  }
  const gbdw_lattice* L = f->lat;
  const int64_t n5 = L->nsite * L->Ls;
  const size_t bytes = size_t(n5) * 12 * (dst_prec == GBDW_F64 ? 16 : 8);
  const int t = 256;
  const size_t blk_smem = 4 * size_t(24) * L->Ls * (dst_prec == GBDW_F64 ? 8 : 4);
  const bool blocks = L->nsimd == 1 && f->nrhs == 1 && blk_smem <= 48 * 1024;
  const bool dev = is_device_ptr(dst);
  void* ddst = dst;
  if (!dev) {
    if (!sync && !is_pinned_host(dst)) {
      set_error("gbdw_field_export_async: the destination must be device or page-locked host memory");
      return GBDW_ERR_INVALID;
    }
    ddst = scratch(bytes, 6);
    if (!ddst) {
      set_error("staging buffer allocation failed");
      return GBDW_ERR_ALLOC;
    }
  }
  if (blocks && (uintptr_t(ddst) & 15) == 0) {
    const unsigned nb = unsigned((L->nsite + 3) / 4);
#define GBDW_EB(DST, P) \
  k_export_blocks<DST, P><<<nb, 128, blk_smem, stream()>>>(f->d, f->norm, L->nsite, L->Ls, (DST*)ddst, f->LsP)
    if (dst_prec == GBDW_F64) {
      if (f->prec == GBDW_F64) GBDW_EB(double, GBDW_F64);
      else if (f->prec == GBDW_F32) GBDW_EB(double, GBDW_F32);
      else GBDW_EB(double, GBDW_F16);
    } else {
      if (f->prec == GBDW_F64) GBDW_EB(float, GBDW_F64);
      else if (f->prec == GBDW_F32) GBDW_EB(float, GBDW_F32);
      else GBDW_EB(float, GBDW_F16);
    }
#undef GBDW_EB
  } else {
#define GBDW_SE(DST, P) \
  k_spinor_export<DST, P><<<nblk(n5, t), t, 0, stream()>>>(f->d, f->norm, L->nsite, L->Ls, L->nsimd, f->nrhs, rhs, \
                                                           (DST*)ddst, f->LsP)
  if (dst_prec == GBDW_F64) {
    if (f->prec == GBDW_F64) GBDW_SE(double, GBDW_F64);
    else if (f->prec == GBDW_F32) GBDW_SE(double, GBDW_F32);
    else GBDW_SE(double, GBDW_F16);
  } else {
    if (f->prec == GBDW_F64) GBDW_SE(float, GBDW_F64);
    else if (f->prec == GBDW_F32) GBDW_SE(float, GBDW_F32);
    else GBDW_SE(float, GBDW_F16);
  }
#undef GBDW_SE
  }
  GBDW_LAUNCHED();
  if (!dev) GBDW_CUDA(cudaMemcpyAsync(dst, ddst, bytes, cudaMemcpyDeviceToHost, stream()));
  if (sync) GBDW_CUDA(cudaStreamSynchronize(stream()));
  return GBDW_OK;
}

int gbdw_field_export(const gbdw_field* f, int rhs, void* dst, int dst_prec) {
  return field_export(f, rhs, dst, dst_prec, true);
}

int gbdw_field_export_async(const gbdw_field* f, int rhs, void* dst, int dst_prec) {
  return field_export(f, rhs, dst, dst_prec, false);
}

int gbdw_field_copy(gbdw_field* dst, const gbdw_field* src) {
  if (!dst || !src || dst->lat != src->lat || dst->nrhs != src->nrhs) {
    set_error("gbdw_field_copy: fields must share lattice and nrhs");
    return GBDW_ERR_INVALID;
  }
  return field_convert(dst, src);
}

}  // extern "C"
