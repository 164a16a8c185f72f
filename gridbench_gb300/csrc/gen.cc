// Seeded input generator: the role TableGenerate.cc:19-91 plays for GridBench, without Grid.
//
// Produces, in GridBench's reference layout (FP64, re/im interleaved):
//   - a random SU(3) gauge field (Gaussian complex 3x3 -> Gram-Schmidt -> det fixed to 1),
//     stored doubled: U[mu+4](x) = U[mu](x - mu)^dagger (what Grid's DoubleStore writes and
//     TableGenerate.cc:54 dumps as Uds);
//   - a 5D fermion with i.i.d. N(0,1) real and imaginary parts (TableGenerate.cc:36);
//   - the nbr/prm stencil table (TableGenerate.cc:75-91): nbr[(site*Ls+s)*8+mu] is the 5D
//     index of the neighbour in direction mu (Xp,Yp,Zp,Tp,Xm,Ym,Zm,Tm), prm the SIMD
//     permute flag set when the step wraps an outer dimension that is split over lanes.
//
// SIMD layout with nsimd lanes (Grid's default): dimensions are halved from T downwards
// (nsimd=4 splits Z and T), global coordinate x_d = o_d + O_d * i_d with O_d = L_d / split_d,
// outer site o lexicographic (x fastest), lane = sum_d i_d * stride_d (x fastest).
//
// Random numbers are keyed by the GLOBAL site index, so the same field comes out in every
// SIMD layout.  Gaussians use Marsaglia's polar method with a logarithm evaluated here from
// the atanh series (frexp, +, *, / only) and this file is compiled without FP contraction,
// so the generated data is bit-identical on every IEEE-754 host.
#include "../../include/gbdw.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>

namespace gbdw {
void set_error(const std::string& msg);
}

namespace {

inline uint64_t splitmix_next(uint64_t& st) {
  uint64_t z = (st += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Stream {
  uint64_t st;
  Stream(uint64_t seed, uint64_t key) {
    st = seed ^ (key * 0xD1B54A32D192ED03ull);
    splitmix_next(st);
  }
  double uniform() { return double(splitmix_next(st) >> 11) * 0x1.0p-53; }  // [0,1)
};

// Natural log for x > 0 (normal numbers), from ln x = e ln2 + 2 atanh((m-1)/(m+1)).
double portable_log(double x) {
  int e = 0;
  double m = std::frexp(x, &e);  // exact: x = m 2^e, m in [0.5, 1)
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e -= 1;
  }
  const double z = (m - 1.0) / (m + 1.0);  // |z| <= 0.1716
  const double z2 = z * z;
  double term = z, sum = z;
  for (int k = 3; k <= 31; k += 2) {
    term = term * z2;
    sum = sum + term / double(k);
  }
  return 2.0 * sum + double(e) * 0.69314718055994530942;
}

// One complex number with independent N(0,1) real and imaginary parts (polar method).
void gaussian_pair(Stream& rng, double& re, double& im) {
  for (;;) {
    const double u = 2.0 * rng.uniform() - 1.0;
    const double v = 2.0 * rng.uniform() - 1.0;
    const double s = u * u + v * v;
    if (s > 0.0 && s < 1.0) {
      const double f = std::sqrt(-2.0 * portable_log(s) / s);
      re = u * f;
      im = v * f;
      return;
    }
  }
}

struct Cplx {
  double re, im;
};
inline Cplx cmul(Cplx a, Cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
inline Cplx cconjmul(Cplx a, Cplx b) {  // conj(a) * b
  return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re};
}

// Random SU(3) matrix m[row][col] for (global site, direction).
void random_su3(uint64_t seed, uint64_t gsite, int mu, Cplx m[3][3]) {
  Stream rng(seed, gsite * 4 + uint64_t(mu));
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) gaussian_pair(rng, m[r][c].re, m[r][c].im);
  // Gram-Schmidt over the rows.
  for (int r = 0; r < 3; ++r) {
    for (int q = 0; q < r; ++q) {
      Cplx d{0.0, 0.0};
      for (int c = 0; c < 3; ++c) {
        const Cplx t = cconjmul(m[q][c], m[r][c]);
        d.re += t.re;
        d.im += t.im;
      }
      for (int c = 0; c < 3; ++c) {
        const Cplx t = cmul(d, m[q][c]);
        m[r][c].re -= t.re;
        m[r][c].im -= t.im;
      }
    }
    double n = 0.0;
    for (int c = 0; c < 3; ++c) n += m[r][c].re * m[r][c].re + m[r][c].im * m[r][c].im;
    n = 1.0 / std::sqrt(n);
    for (int c = 0; c < 3; ++c) {
      m[r][c].re *= n;
      m[r][c].im *= n;
    }
  }
  // The determinant of a unitary matrix has modulus one; multiply the last row by its
  // conjugate so that det = 1.
  const Cplx c0 = cmul(m[1][1], m[2][2]), c1 = cmul(m[1][2], m[2][1]);
  const Cplx c2 = cmul(m[1][0], m[2][2]), c3 = cmul(m[1][2], m[2][0]);
  const Cplx c4 = cmul(m[1][0], m[2][1]), c5 = cmul(m[1][1], m[2][0]);
  const Cplx a0 = cmul(m[0][0], Cplx{c0.re - c1.re, c0.im - c1.im});
  const Cplx a1 = cmul(m[0][1], Cplx{c2.re - c3.re, c2.im - c3.im});
  const Cplx a2 = cmul(m[0][2], Cplx{c4.re - c5.re, c4.im - c5.im});
  Cplx det{a0.re - a1.re + a2.re, a0.im - a1.im + a2.im};
  const double dn = 1.0 / std::sqrt(det.re * det.re + det.im * det.im);
  const Cplx phase{det.re * dn, -det.im * dn};
  for (int c = 0; c < 3; ++c) m[2][c] = cmul(m[2][c], phase);
}

struct Layout {
  int L[4], split[4], O[4], stride[4];
  int nsimd;
  uint64_t V, nouter;
  bool init(const int dims[4], int ns) {
    nsimd = ns;
    if (ns != 1 && ns != 2 && ns != 4 && ns != 8 && ns != 16) return false;
    int nn = ns;
    for (int d = 3; d >= 0; --d) {
      split[d] = 1;
      if (nn >= 2) {
        split[d] = 2;
        nn /= 2;
      }
    }
    V = 1;
    for (int d = 0; d < 4; ++d) {
      L[d] = dims[d];
      if (L[d] < 1 || L[d] % split[d] != 0) return false;
      O[d] = L[d] / split[d];
      V *= uint64_t(L[d]);
    }
    int st = 1;
    for (int d = 0; d < 4; ++d) {
      stride[d] = st;
      st *= split[d];
    }
    nouter = V / uint64_t(ns);
    return true;
  }
  uint64_t global_index(const int x[4]) const {
    return uint64_t(x[0]) + uint64_t(L[0]) * (uint64_t(x[1]) + uint64_t(L[1]) * (uint64_t(x[2]) + uint64_t(L[2]) * uint64_t(x[3])));
  }
  // (outer site, lane) -> global coordinates
  void coords(uint64_t o, int lane, int x[4]) const {
    uint64_t r = o;
    for (int d = 0; d < 4; ++d) {
      const int od = int(r % uint64_t(O[d]));
      r /= uint64_t(O[d]);
      const int id = (lane / stride[d]) % split[d];
      x[d] = od + O[d] * id;
    }
  }
};

bool check_dims(const int dims[4]) {
  if (!dims) return false;
  for (int d = 0; d < 4; ++d)
    if (dims[d] < 1 || dims[d] > 4096) return false;
  return true;
}

}  // namespace

extern "C" uint64_t gbdw_seed_from_ints(const int* seeds, int n) {
  uint64_t st = 0x6A09E667F3BCC909ull;
  uint64_t h = 0;
  for (int i = 0; i < n; ++i) {
    st ^= uint64_t(uint32_t(seeds[i])) + 0x100000000ull * uint64_t(i + 1);
    h ^= splitmix_next(st);
  }
  return h;
}

extern "C" int gbdw_generate_gauge(const int dims[4], int nsimd, uint64_t seed, double* U) {
  Layout lay;
  if (!check_dims(dims) || !lay.init(dims, nsimd)) {
    gbdw::set_error("gbdw_generate_gauge: bad dims/nsimd (each dim >= 1 and divisible by its lane split)");
    return GBDW_ERR_INVALID;
  }
  if (!U) return GBDW_OK;
  const int64_t nout = int64_t(lay.nouter);
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < nout; ++o) {
    for (int lane = 0; lane < nsimd; ++lane) {
      int x[4];
      lay.coords(uint64_t(o), lane, x);
      const uint64_t g = lay.global_index(x);
      for (int mu = 0; mu < 4; ++mu) {
        Cplx m[3][3];
        // forward link U_mu(x)
        random_su3(seed, g, mu, m);
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) {
            const uint64_t idx = ((uint64_t(o) * 8 + uint64_t(mu)) * 9 + uint64_t(r * 3 + c)) * uint64_t(nsimd) + uint64_t(lane);
            U[2 * idx] = m[r][c].re;
            U[2 * idx + 1] = m[r][c].im;
          }
        // backward link U_mu(x - mu)^dagger
        int xm[4] = {x[0], x[1], x[2], x[3]};
        xm[mu] = (xm[mu] + lay.L[mu] - 1) % lay.L[mu];
        random_su3(seed, lay.global_index(xm), mu, m);
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) {
            const uint64_t idx = ((uint64_t(o) * 8 + uint64_t(mu + 4)) * 9 + uint64_t(r * 3 + c)) * uint64_t(nsimd) + uint64_t(lane);
            U[2 * idx] = m[c][r].re;
            U[2 * idx + 1] = -m[c][r].im;
          }
      }
    }
  }
  return GBDW_OK;
}

extern "C" int gbdw_generate_fermion(const int dims[4], int Ls, int nsimd, uint64_t seed, double* phi) {
  Layout lay;
  if (!check_dims(dims) || !lay.init(dims, nsimd) || Ls < 1) {
    gbdw::set_error("gbdw_generate_fermion: bad dims/Ls/nsimd");
    return GBDW_ERR_INVALID;
  }
  if (!phi) return GBDW_OK;
  const int64_t nout = int64_t(lay.nouter);
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < nout; ++o) {
    for (int lane = 0; lane < nsimd; ++lane) {
      int x[4];
      lay.coords(uint64_t(o), lane, x);
      const uint64_t g = lay.global_index(x);
      for (int s = 0; s < Ls; ++s) {
        Stream rng(seed, g * uint64_t(Ls) + uint64_t(s));
        for (int sc = 0; sc < 12; ++sc) {
          double re, im;
          gaussian_pair(rng, re, im);
          const uint64_t idx = ((uint64_t(o) * uint64_t(Ls) + uint64_t(s)) * 12 + uint64_t(sc)) * uint64_t(nsimd) + uint64_t(lane);
          phi[2 * idx] = re;
          phi[2 * idx + 1] = im;
        }
      }
    }
  }
  return GBDW_OK;
}

extern "C" int gbdw_generate_table(const int dims[4], int Ls, int nsimd, uint64_t* nbr, uint8_t* prm) {
  Layout lay;
  if (!check_dims(dims) || !lay.init(dims, nsimd) || Ls < 1) {
    gbdw::set_error("gbdw_generate_table: bad dims/Ls/nsimd");
    return GBDW_ERR_INVALID;
  }
  const int64_t nout = int64_t(lay.nouter);
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < nout; ++o) {
    int oc[4];
    uint64_t r = uint64_t(o);
    for (int d = 0; d < 4; ++d) {
      oc[d] = int(r % uint64_t(lay.O[d]));
      r /= uint64_t(lay.O[d]);
    }
    for (int mu = 0; mu < 8; ++mu) {
      const int d = mu & 3;
      int on[4] = {oc[0], oc[1], oc[2], oc[3]};
      bool wrap;
      if (mu < 4) {
        wrap = (on[d] + 1 == lay.O[d]);
        on[d] = wrap ? 0 : on[d] + 1;
      } else {
        wrap = (on[d] == 0);
        on[d] = wrap ? lay.O[d] - 1 : on[d] - 1;
      }
      const uint64_t onb = uint64_t(on[0]) + uint64_t(lay.O[0]) * (uint64_t(on[1]) + uint64_t(lay.O[1]) * (uint64_t(on[2]) + uint64_t(lay.O[2]) * uint64_t(on[3])));
      const uint8_t p = (wrap && lay.split[d] == 2) ? 1 : 0;
      for (int s = 0; s < Ls; ++s) {
        const uint64_t j = (uint64_t(o) * uint64_t(Ls) + uint64_t(s)) * 8 + uint64_t(mu);
        if (nbr) nbr[j] = onb * uint64_t(Ls) + uint64_t(s);
        if (prm) prm[j] = p;
      }
    }
  }
  return GBDW_OK;
}
