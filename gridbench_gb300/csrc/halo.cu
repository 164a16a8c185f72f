// Halo packing for a 4D domain decomposition of the hopping term.  GridBench runs on one node
// and exchanges no halos; Grid, which it wraps, sends spin-projected half spinors between
// ranks (its Wilson "compressor"), and this is that step's GB300 form for one GPU's local
// volume, ready for a multi-GPU split.
//
// Across the face of its local volume in direction mu a domain needs its neighbour domain's
// spinors at the adjacent face, and only through the spin projection of the leg that reads them:
// h0 = psi0 + c0 psi_A, h1 = psi1 + c1 psi_B (the per-leg table of WilsonKernelsHandCpu.h:94-303),
// half the bytes of the full spinor.  No link is needed: the doubled gauge field holds
// U[mu+4](x) = U[mu](x - mu)^dagger at the receiving site, so the receiver multiplies.
//   face 0 (x_mu = 0) is read by the domain at -mu through its forward leg mu;
//   face 1 (x_mu = L_mu - 1) is read by the domain at +mu through its backward leg mu + 4;
// dag = 1 packs for DhopDag (each leg with its opposite-sign partner's projector).
//
// Buffer (the transport format): face site f (the three other coordinates lexicographic, the
// lowest dimension fastest) x row k (h0 colours 0..2, then h1 colours 0..2) x the field's LsE
// slices in its own storage format (F64: double2 per slice; F32/F16: slice pairs stored as
// (Re s, Re s+1, Im s, Im s+1) over LsP slots); for F16 a block of nface * LsE FP32 norms (the
// largest |component| of each slice's packed half spinor) follows the values.
// One thread per (face site, slice): every face spinor is read once, 6 of its 12 complex
// components are written -- HBM bound, 1.5 spinors of traffic per packed 5D site.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "dhop_kernel.cuh"
#include "layout.cuh"

namespace gbdw {

bool is_device_ptr(const void* p);  // fields.cu

namespace {

template <class T, int C>
__device__ __forceinline__ cpx<T> unit_times(cpx<T> a) {
  if constexpr (C == 0) return a;
  else if constexpr (C == 1) return {-a.r, -a.i};
  else if constexpr (C == 2) return {-a.i, a.r};  // i a
  else return {a.i, -a.r};                          // -i a
}

struct HaloParams {
  const void* in;
  const float* in_norm;
  void* out;
  float* out_norm;
  int dims[4];
  int mu;
  int xmu;  // the face's coordinate in direction mu
  int64_t nface;
  int LsE;
  int LsP;
};

template <int P, int LT>
__global__ void __launch_bounds__(256) k_halo_pack(const HaloParams p) {
  using T = typename Arith<P>::T;
  using S = LegSpin<LT>;
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= p.nface * p.LsE) return;
  const int64_t f = i / p.LsE;
  const int e = int(i - f * p.LsE);
  int c[4];
  int64_t r = f;
#pragma unroll
  for (int d = 0; d < 4; ++d) {
    if (d == p.mu) {
      c[d] = p.xmu;
    } else {
      c[d] = int(r % p.dims[d]);
      r /= p.dims[d];
    }
  }
  const int64_t site = c[0] + int64_t(p.dims[0]) * (c[1] + int64_t(p.dims[1]) * (c[2] + int64_t(p.dims[2]) * c[3]));
  const int64_t row0 = site * 12;
  cpx<T> h[6];
#pragma unroll
  for (int col = 0; col < 3; ++col) {
    const cpx<T> x = Elem<P>::ld(p.in, row0 + 0 * 3 + col, e, p.LsP);
    const cpx<T> y = Elem<P>::ld(p.in, row0 + S::A * 3 + col, e, p.LsP);
    const cpx<T> z = Elem<P>::ld(p.in, row0 + 1 * 3 + col, e, p.LsP);
    const cpx<T> w = Elem<P>::ld(p.in, row0 + S::B * 3 + col, e, p.LsP);
    const cpx<T> ya = unit_times<T, S::C0>(y), wb = unit_times<T, S::C1>(w);
    h[col] = {x.r + ya.r, x.i + ya.i};
    h[3 + col] = {z.r + wb.r, z.i + wb.i};
  }
  const int64_t orow = f * 6;
  if constexpr (P == GBDW_F16) {
    // dequantise with the source slice's norm, renormalise the half spinor
    const float n = __ldg(p.in_norm + site * p.LsE + e);
    float m = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      h[k] = {h[k].r * n, h[k].i * n};
      m = fmaxf(m, fmaxf(fabsf(h[k].r), fabsf(h[k].i)));
    }
    const float s = m > 0.f ? 1.0f / m : 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) Elem<P>::st(p.out, orow + k, e, p.LsP, h[k].r * s, h[k].i * s);
    p.out_norm[f * p.LsE + e] = m;
  } else {
#pragma unroll
    for (int k = 0; k < 6; ++k) Elem<P>::st(p.out, orow + k, e, p.LsP, h[k].r, h[k].i);
  }
}

int64_t face_sites(const gbdw_lattice* L, int mu) {
  int64_t n = 1;
  for (int d = 0; d < 4; ++d)
    if (d != mu) n *= L->dims[d];
  return n;
}

size_t halo_value_bytes(const gbdw_field* f, int mu) {
  return size_t(face_sites(f->lat, mu)) * 6 * size_t(f->LsP) * spinor_elem_bytes(f->prec);
}

size_t halo_bytes(const gbdw_field* f, int mu) {
  size_t b = halo_value_bytes(f, mu);
  if (f->prec == GBDW_F16) b += size_t(face_sites(f->lat, mu)) * size_t(f->LsE) * sizeof(float);
  return b;
}

int check_halo(const gbdw_field* f, int mu) {
  if (!f || mu < 0 || mu > 3) {
    set_error("halo: a field and a direction 0..3");
    return GBDW_ERR_INVALID;
  }
  const gbdw_lattice* L = f->lat;
  if (L->parity >= 0 || L->nsimd != 1 || L->dims[0] <= 0) {
    set_error("halo: needs a field on a periodic full lattice made by gbdw_lattice_create (nsimd 1)");
    return GBDW_ERR_INVALID;
  }
  return GBDW_OK;
}

template <int P>
void launch_pack(const HaloParams& p, int leg) {
  const unsigned g = unsigned((p.nface * p.LsE + 255) / 256);
  switch (leg) {
    case 0: k_halo_pack<P, 0><<<g, 256, 0, stream()>>>(p); break;
    case 1: k_halo_pack<P, 1><<<g, 256, 0, stream()>>>(p); break;
    case 2: k_halo_pack<P, 2><<<g, 256, 0, stream()>>>(p); break;
    case 3: k_halo_pack<P, 3><<<g, 256, 0, stream()>>>(p); break;
    case 4: k_halo_pack<P, 4><<<g, 256, 0, stream()>>>(p); break;
    case 5: k_halo_pack<P, 5><<<g, 256, 0, stream()>>>(p); break;
    case 6: k_halo_pack<P, 6><<<g, 256, 0, stream()>>>(p); break;
    default: k_halo_pack<P, 7><<<g, 256, 0, stream()>>>(p); break;
  }
}

}  // namespace

}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_halo_bytes(const gbdw_field* f, int mu, size_t* bytes) {
  if (int st = check_halo(f, mu)) return st;
  if (!bytes) {
    set_error("gbdw_halo_bytes: null output");
    return GBDW_ERR_INVALID;
  }
  *bytes = halo_bytes(f, mu);
  return GBDW_OK;
}

int gbdw_halo_pack(const gbdw_field* f, int mu, int face, int dag, void* dst) {
  if (int st = check_halo(f, mu)) return st;
  if (!dst || (face != 0 && face != 1)) {
    set_error("gbdw_halo_pack: face 0 (low) or 1 (high) and a destination");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const size_t bytes = halo_bytes(f, mu);
  const bool dev = is_device_ptr(dst);
  void* d = dst;
  if (!dev) {
    d = scratch(bytes, 11);
    if (!d) {
      set_error("halo staging buffer allocation failed");
      return GBDW_ERR_ALLOC;
    }
  } else if ((uintptr_t(dst) & 15) != 0) {
    set_error("gbdw_halo_pack: a device destination must be 16-byte aligned");
    return GBDW_ERR_INVALID;
  }
  HaloParams p;
  p.in = f->d;
  p.in_norm = f->norm;
  p.out = d;
  p.out_norm = f->prec == GBDW_F16 ? (float*)((char*)d + halo_value_bytes(f, mu)) : nullptr;
  for (int k = 0; k < 4; ++k) p.dims[k] = f->lat->dims[k];
  p.mu = mu;
  p.xmu = face == 0 ? 0 : f->lat->dims[mu] - 1;
  p.nface = face_sites(f->lat, mu);
  p.LsE = f->LsE;
  p.LsP = f->LsP;
  // the receiving leg: forward mu for the low face, backward mu + 4 for the high face
  const int leg = (face == 0 ? mu : mu + 4) ^ (dag ? 4 : 0);
  if (f->prec == GBDW_F64) launch_pack<GBDW_F64>(p, leg);
  else if (f->prec == GBDW_F32) launch_pack<GBDW_F32>(p, leg);
  else launch_pack<GBDW_F16>(p, leg);
  GBDW_LAUNCHED();
  if (!dev) {
    GBDW_CUDA(cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, stream()));
    GBDW_CUDA(cudaStreamSynchronize(stream()));
  }
  return GBDW_OK;
}

}  // extern "C"
