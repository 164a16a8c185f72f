// Device-side random inputs for large benchmark workloads: Gaussian spinors and random SU(3)
// doubled gauge fields on periodic lattices.  Same recipe as the host generator (counter-based
// splitmix64 streams keyed by the global site, Gaussian -> Gram-Schmidt -> det = 1 for links,
// i.i.d. N(0,1) real and imaginary parts for spinors) but with CUDA's log/sincos, so the bits
// differ from gbdw_generate_*; parity tests use the host generator.
#include "common.cuh"
#include "layout.cuh"

namespace gbdw {
namespace {

__device__ __forceinline__ uint64_t sm_next(uint64_t& st) {
  uint64_t z = (st += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Box-Muller pair from two uniforms in (0, 1].
__device__ __forceinline__ double2 gauss2(uint64_t& st) {
  const double u1 = (double((sm_next(st) >> 11)) + 1.0) * 0x1.0p-53;
  const double u2 = double(sm_next(st) >> 11) * 0x1.0p-53;
  const double r = sqrt(-2.0 * log(u1));
  double s, c;
  sincospi(2.0 * u2, &s, &c);
  return make_double2(r * c, r * s);
}

__global__ void k_field_gaussian(void* d, float* norm, int prec, int64_t nsite, int Ls, int nrhs, int rhs,
                                 uint64_t seed, int LsP) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;  // (site, s)
  if (i >= nsite * Ls) return;
  const int64_t site = i / Ls;
  const int s = int(i - site * Ls);
  const int LsE = Ls * nrhs;
  const int e = s * nrhs + rhs;
  uint64_t st = seed ^ (uint64_t(i) * 0xD1B54A32D192ED03ull);
  sm_next(st);
  double2 v[12];
  float m = 0.f;
  for (int k = 0; k < 12; ++k) {
    v[k] = gauss2(st);
    m = fmaxf(m, fmaxf(fabsf(float(v[k].x)), fabsf(float(v[k].y))));
  }
  const float sc = m > 0.f ? 1.f / m : 0.f;
  if (prec == GBDW_F16) norm[site * LsE + e] = m;
  for (int k = 0; k < 12; ++k) {
    if (prec == GBDW_F64) Elem<GBDW_F64>::st(d, site * 12 + k, e, LsP, v[k].x, v[k].y);
    else if (prec == GBDW_F32) Elem<GBDW_F32>::st(d, site * 12 + k, e, LsP, float(v[k].x), float(v[k].y));
    else Elem<GBDW_F16>::st(d, site * 12 + k, e, LsP, float(v[k].x) * sc, float(v[k].y) * sc);
  }
}

// Forward links U_mu(x), FP64, [site][4][9] complex.
__global__ void k_su3_forward(double2* out, int64_t nsite, uint64_t seed) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;  // (site, mu)
  if (i >= nsite * 4) return;
  uint64_t st = seed ^ (uint64_t(i) * 0xD1B54A32D192ED03ull);
  sm_next(st);
  double2 m[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) m[r][c] = gauss2(st);
  for (int r = 0; r < 3; ++r) {
    for (int q = 0; q < r; ++q) {
      double dr = 0, di = 0;  // <m_q, m_r>
      for (int c = 0; c < 3; ++c) {
        dr += m[q][c].x * m[r][c].x + m[q][c].y * m[r][c].y;
        di += m[q][c].x * m[r][c].y - m[q][c].y * m[r][c].x;
      }
      for (int c = 0; c < 3; ++c) {
        m[r][c].x -= dr * m[q][c].x - di * m[q][c].y;
        m[r][c].y -= dr * m[q][c].y + di * m[q][c].x;
      }
    }
    double n = 0;
    for (int c = 0; c < 3; ++c) n += m[r][c].x * m[r][c].x + m[r][c].y * m[r][c].y;
    n = rsqrt(n);
    for (int c = 0; c < 3; ++c) {
      m[r][c].x *= n;
      m[r][c].y *= n;
    }
  }
  auto mul = [](double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
  auto sub = [](double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); };
  const double2 a0 = mul(m[0][0], sub(mul(m[1][1], m[2][2]), mul(m[1][2], m[2][1])));
  const double2 a1 = mul(m[0][1], sub(mul(m[1][0], m[2][2]), mul(m[1][2], m[2][0])));
  const double2 a2 = mul(m[0][2], sub(mul(m[1][0], m[2][1]), mul(m[1][1], m[2][0])));
  const double2 det = make_double2(a0.x - a1.x + a2.x, a0.y - a1.y + a2.y);
  const double dn = rsqrt(det.x * det.x + det.y * det.y);
  const double2 ph = make_double2(det.x * dn, -det.y * dn);
  for (int c = 0; c < 3; ++c) m[2][c] = mul(m[2][c], ph);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) out[i * 9 + r * 3 + c] = m[r][c];
}

// Doubled field in storage precision P: U[mu] = fwd(x, mu), U[mu+4] = fwd(x - mu, mu)^dagger.
template <int P>
__global__ void k_su3_double(const double2* fwd, const uint32_t* nbr4, int64_t nsite, void* dst) {
  const int64_t i = blockIdx.x * int64_t(blockDim.x) + threadIdx.x;  // (site, mu 0..7)
  if (i >= nsite * 8) return;
  const int64_t site = i >> 3;
  const int mu = int(i & 7);
  double2 u[9];
  if (mu < 4) {
    for (int k = 0; k < 9; ++k) u[k] = fwd[(site * 4 + mu) * 9 + k];
  } else {
    const int64_t back = nbr4[site * 8 + mu];  // x - mu
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        const double2 a = fwd[(back * 4 + (mu - 4)) * 9 + c * 3 + r];
        u[r * 3 + c] = make_double2(a.x, -a.y);
      }
  }
  if (P == GBDW_F64) {
    for (int k = 0; k < 9; ++k) ((double2*)dst)[i * 9 + k] = u[k];
  } else if (P == GBDW_F32) {
    for (int k = 0; k < 9; ++k) ((float2*)dst)[i * 9 + k] = make_float2(float(u[k].x), float(u[k].y));
  } else if (P == GBDW_F16) {
    for (int k = 0; k < 6; ++k) ((__half2*)dst)[i * 6 + k] = __floats2half2_rn(float(u[k].x), float(u[k].y));
  } else {
    for (int k = 0; k < 6; ++k)
      ((__nv_bfloat162*)dst)[i * 6 + k] = __floats2bfloat162_rn(float(u[k].x), float(u[k].y));
  }
}

inline unsigned nb(int64_t n, int t) { return unsigned((n + t - 1) / t); }

}  // namespace
}  // namespace gbdw

using namespace gbdw;

extern "C" {

int gbdw_field_gaussian(gbdw_field* f, int rhs, uint64_t seed) {
  if (!f || rhs < 0 || rhs >= f->nrhs) {
    set_error("gbdw_field_gaussian: invalid arguments");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const int64_t n = f->lat->nsite * f->lat->Ls;
  k_field_gaussian<<<nb(n, 256), 256, 0, stream()>>>(f->d, f->norm, f->prec, f->lat->nsite, f->lat->Ls, f->nrhs, rhs,
                                                     seed * 0x9E3779B97F4A7C15ull + uint64_t(rhs), f->LsP);
  GBDW_LAUNCHED();
  return GBDW_OK;
}

int gbdw_gauge_random(gbdw_gauge** g, const gbdw_lattice* lat, int prec, uint64_t seed) {
  if (!g || !lat || prec < GBDW_F64 || prec > GBDW_BF16 || !lat->fast || lat->nsimd != 1) {
    set_error("gbdw_gauge_random: needs a 4D-factorised single-lane lattice and a valid precision");
    return GBDW_ERR_INVALID;
  }
  if (int st = ensure_device()) return st;
  const int64_t nsite = lat->nsite;
  double2* fwd = (double2*)scratch(size_t(nsite) * 4 * 9 * sizeof(double2), 2);
  if (!fwd) {
    set_error("gbdw_gauge_random: scratch allocation failed");
    return GBDW_ERR_ALLOC;
  }
  gbdw_gauge* G = new gbdw_gauge();
  G->lat = lat;
  G->prec = prec;
  G->bytes = size_t(nsite) * 8 * link_bytes(prec);
  cudaError_t e = dev_alloc((void**)&G->d, G->bytes);
  if (e != cudaSuccess) {
    delete G;
    return cuda_fail(e, "cudaMalloc(gauge)");
  }
  k_su3_forward<<<nb(nsite * 4, 128), 128, 0, stream()>>>(fwd, nsite, seed);
  count_launch();
  const unsigned blocks = nb(nsite * 8, 256);
  switch (prec) {
    case GBDW_F64: k_su3_double<GBDW_F64><<<blocks, 256, 0, stream()>>>(fwd, lat->nbr4, nsite, G->d); break;
    case GBDW_F32: k_su3_double<GBDW_F32><<<blocks, 256, 0, stream()>>>(fwd, lat->nbr4, nsite, G->d); break;
    case GBDW_F16: k_su3_double<GBDW_F16><<<blocks, 256, 0, stream()>>>(fwd, lat->nbr4, nsite, G->d); break;
    default: k_su3_double<GBDW_BF16><<<blocks, 256, 0, stream()>>>(fwd, lat->nbr4, nsite, G->d); break;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    cudaFree(G->d);
    delete G;
    return cuda_fail(e, "k_su3_double");
  }
  count_launch();
  *g = G;
  return GBDW_OK;
}

}  // extern "C"
