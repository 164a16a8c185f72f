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
// One thread per (face site, slice pair) over all requested faces in one launch: every face
// spinor is read once, 6 of its 12 complex components are written -- HBM bound, 1.5 spinors of
// traffic per packed 5D site.
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

// One launch packs up to 8 faces: thread -> (face k, face site f, first slice e0 of N).
struct HaloFace {
  void* out;
  float* out_norm;
  int64_t nface;
  int64_t first;  // first thread of this face
  int mu;
  int xmu;  // the face's coordinate in direction mu
  int leg;  // the receiving leg whose projector applies (after dag)
};

struct HaloParams {
  const void* in;
  const float* in_norm;
  int dims[4];
  int LsE;
  int LsP;
  int nfaces;
  int64_t total;  // threads over all faces
  HaloFace face[8];
};

template <int P, int LT, int N>
__device__ __forceinline__ void pack_face(const HaloParams& p, const HaloFace& F, int64_t f, int e0) {
  using T = typename Arith<P>::T;
  using S = LegSpin<LT>;
  int c[4];
  int64_t r = f;
#pragma unroll
  for (int d = 0; d < 4; ++d) {
    if (d == F.mu) {
      c[d] = F.xmu;
    } else {
      c[d] = int(r % p.dims[d]);
      r /= p.dims[d];
    }
  }
  const int64_t site = c[0] + int64_t(p.dims[0]) * (c[1] + int64_t(p.dims[1]) * (c[2] + int64_t(p.dims[2]) * c[3]));
  const int64_t row0 = site * 12;
  cpx<T> h[6][N];
#pragma unroll
  for (int col = 0; col < 3; ++col) {
    cpx<T> x[N], y[N], z[N], w[N];
    Vec<P, N>::load(p.in, row0 + 0 * 3 + col, e0, p.LsP, x);
    Vec<P, N>::load(p.in, row0 + S::A * 3 + col, e0, p.LsP, y);
    Vec<P, N>::load(p.in, row0 + 1 * 3 + col, e0, p.LsP, z);
    Vec<P, N>::load(p.in, row0 + S::B * 3 + col, e0, p.LsP, w);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const cpx<T> ya = unit_times<T, S::C0>(y[j]), wb = unit_times<T, S::C1>(w[j]);
      h[col][j] = {x[j].r + ya.r, x[j].i + ya.i};
      h[3 + col][j] = {z[j].r + wb.r, z[j].i + wb.i};
    }
  }
  const int64_t orow = f * 6;
  if constexpr (P == GBDW_F16) {
    // dequantise with the source slices' norms, renormalise each slice's half spinor
    float n[N], m[N], sc[N];
    load_norms<N>(p.in_norm, site * p.LsE + e0, n);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      m[j] = 0.f;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        h[k][j] = {h[k][j].r * n[j], h[k][j].i * n[j]};
        m[j] = fmaxf(m[j], fmaxf(fabsf(h[k][j].r), fabsf(h[k][j].i)));
      }
      sc[j] = m[j] > 0.f ? 1.0f / m[j] : 0.f;
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      cpx<float> v[N];
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = {h[k][j].r * sc[j], h[k][j].i * sc[j]};
      Vec<P, N>::store_scaled(F.out, orow + k, e0, p.LsP, v);
    }
#pragma unroll
    for (int j = 0; j < N; ++j) F.out_norm[f * p.LsE + e0 + j] = m[j];
  } else {
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      cpx<T> v[N];
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = h[k][j];
      Vec<P, N>::store(F.out, orow + k, e0, p.LsP, v);
    }
  }
}

template <int P, int N>
__global__ void __launch_bounds__(256) k_halo_pack(const __grid_constant__ HaloParams p) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;
  if (i >= p.total) return;
  int k = 0;
  while (k + 1 < p.nfaces && i >= p.face[k + 1].first) ++k;
  const HaloFace& F = p.face[k];
  const int G = p.LsE / N;
  const int64_t t = i - F.first;
  const int64_t f = t / G;
  const int e0 = int(t - f * G) * N;
  switch (F.leg) {
    case 0: pack_face<P, 0, N>(p, F, f, e0); break;
    case 1: pack_face<P, 1, N>(p, F, f, e0); break;
    case 2: pack_face<P, 2, N>(p, F, f, e0); break;
    case 3: pack_face<P, 3, N>(p, F, f, e0); break;
    case 4: pack_face<P, 4, N>(p, F, f, e0); break;
    case 5: pack_face<P, 5, N>(p, F, f, e0); break;
    case 6: pack_face<P, 6, N>(p, F, f, e0); break;
    default: pack_face<P, 7, N>(p, F, f, e0); break;
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
void launch_pack(const HaloParams& p, int N) {
  const unsigned g = unsigned((p.total + 255) / 256);
  if (N == 2) k_halo_pack<P, 2><<<g, 256, 0, stream()>>>(p);
  else k_halo_pack<P, 1><<<g, 256, 0, stream()>>>(p);
}

// Packs the faces (mu[k], face[k]) into device buffers dst[k] in one launch.
int pack_faces(const gbdw_field* f, int n, const int* mu, const int* face, int dag, void* const* dst) {
  HaloParams p;
  p.in = f->d;
  p.in_norm = f->norm;
  for (int k = 0; k < 4; ++k) p.dims[k] = f->lat->dims[k];
  p.LsE = f->LsE;
  p.LsP = f->LsP;
  p.nfaces = n;
  const int N = (f->prec != GBDW_F64 && f->LsE % 2 == 0) ? 2 : 1;
  int64_t first = 0;
  for (int k = 0; k < n; ++k) {
    HaloFace& F = p.face[k];
    F.out = dst[k];
    F.out_norm = f->prec == GBDW_F16 ? (float*)((char*)dst[k] + halo_value_bytes(f, mu[k])) : nullptr;
    F.nface = face_sites(f->lat, mu[k]);
    F.first = first;
    F.mu = mu[k];
    F.xmu = face[k] == 0 ? 0 : f->lat->dims[mu[k]] - 1;
    // the receiving leg: forward mu for the low face, backward mu + 4 for the high face
    F.leg = (face[k] == 0 ? mu[k] : mu[k] + 4) ^ (dag ? 4 : 0);
    first += F.nface * (f->LsE / N);
  }
  p.total = first;
  if (f->prec == GBDW_F64) launch_pack<GBDW_F64>(p, N);
  else if (f->prec == GBDW_F32) launch_pack<GBDW_F32>(p, N);
  else launch_pack<GBDW_F16>(p, N);
  GBDW_LAUNCHED();
  return GBDW_OK;
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
  if (int st = pack_faces(f, 1, &mu, &face, dag, &d)) return st;
  if (!dev) {
    GBDW_CUDA(cudaMemcpyAsync(dst, d, bytes, cudaMemcpyDeviceToHost, stream()));
    GBDW_CUDA(cudaStreamSynchronize(stream()));
  }
  return GBDW_OK;
}

int gbdw_halo_pack_all(const gbdw_field* f, int dag, void* const dst[8]) {
  if (int st = check_halo(f, 0)) return st;
  if (!dst) {
    set_error("gbdw_halo_pack_all: eight destinations");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  for (int k = 0; k < 8; ++k)
    if (!dst[k] || !is_device_ptr(dst[k]) || (uintptr_t(dst[k]) & 15) != 0) {
      set_error("gbdw_halo_pack_all: eight 16-byte aligned device destinations");
      return GBDW_ERR_INVALID;
    }
  const int mu[8] = {0, 0, 1, 1, 2, 2, 3, 3}, face[8] = {0, 1, 0, 1, 0, 1, 0, 1};
  return pack_faces(f, 8, mu, face, dag, dst);
}

}  // extern "C"
