/*
 * ORACLE input generator -- test infrastructure only.
 *
 * The inputs of every parity test and of the CPU baseline: a seeded random SU(3) gauge field
 * stored doubled, a Gaussian 5D fermion and the nbr/prm stencil tables, in GridBench's
 * reference layout (TableGenerate.cc:19-91 produces the same three things with Grid; its
 * array layout is the one dslash_simple.h:3-5,40 and WilsonKernelsHandGpu.h:33-41 read).
 *
 * This is a second, independent implementation of the seeded generator the product library
 * carries for its users (libgbdw's gbdw_generate_*): the reference-side CPU runs (bench.py
 * --impl reference, the CPU baseline) take their inputs from here and never load the product
 * library.  tests/test_generator.py checks both bit for bit against each other and against
 * the SHA-256 digests in tests/golden/.
 *
 * The definition it follows (and with it every host reproduces the same bits):
 *   - random stream per (seed, key): state = seed ^ key * 0xD1B54A32D192ED03, advanced once;
 *     SplitMix64 steps (Steele, Lea, Flood, OOPSLA 2014); uniform = (next >> 11) * 2^-53;
 *   - Gaussian pairs by Marsaglia's polar method, with ln evaluated from the series
 *     ln x = e ln 2 + 2 atanh((m - 1)/(m + 1)) (terms up to z^31) on frexp's mantissa m,
 *     moved to [sqrt(1/2), sqrt(2));
 *   - SU(3) link of (global site g, direction mu): key 4 g + mu, nine Gaussian complex
 *     entries row-major, Gram-Schmidt over the rows, the last row multiplied by the conjugate
 *     phase of the determinant;
 *   - doubled field: U[mu+4](x) = U[mu](x - mu)^dagger;
 *   - fermion entry (g, s, sc): key g Ls + s, twelve Gaussian complex numbers in sc order;
 *   - SIMD layout with nsimd lanes: dimensions halved from T downwards, x_d = o_d + O_d i_d,
 *     outer site o lexicographic (x fastest), lane = sum_d i_d stride_d (x fastest);
 *   - table: nbr[(o Ls + s) 8 + mu] = outer neighbour * Ls + s, prm set where the step wraps a
 *     dimension split over lanes (TableGenerate.cc:75-91).
 * Compiled without FP contraction (oracle/build.py).
 */
#include <math.h>
#include <stdint.h>

static uint64_t gen_next(uint64_t* st) {
  uint64_t z = (*st += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t gen_stream(uint64_t seed, uint64_t key) {
  uint64_t st = seed ^ (key * 0xD1B54A32D192ED03ull);
  (void)gen_next(&st);
  return st;
}

static double gen_uniform(uint64_t* st) { return (double)(gen_next(st) >> 11) * 0x1.0p-53; }

static double gen_log(double x) {
  int e = 0;
  double m = frexp(x, &e);
  if (m < 0.70710678118654752440) {
    m = m * 2.0;
    e -= 1;
  }
  const double z = (m - 1.0) / (m + 1.0);
  const double z2 = z * z;
  double term = z, sum = z;
  for (int k = 3; k <= 31; k += 2) {
    term = term * z2;
    sum = sum + term / (double)k;
  }
  return 2.0 * sum + (double)e * 0.69314718055994530942;
}

/* (re, im) with independent N(0,1) parts */
static void gen_gauss(uint64_t* st, double* re, double* im) {
  for (;;) {
    const double u = 2.0 * gen_uniform(st) - 1.0;
    const double v = 2.0 * gen_uniform(st) - 1.0;
    const double s = u * u + v * v;
    if (s > 0.0 && s < 1.0) {
      const double f = sqrt(-2.0 * gen_log(s) / s);
      *re = u * f;
      *im = v * f;
      return;
    }
  }
}

/* complex helpers on (re, im) pairs stored in double[2] */
static void gen_mul(const double* a, const double* b, double* o) {
  const double re = a[0] * b[0] - a[1] * b[1];
  const double im = a[0] * b[1] + a[1] * b[0];
  o[0] = re;
  o[1] = im;
}

/* m[row][col][re/im] */
static void gen_su3(uint64_t seed, uint64_t g, int mu, double m[3][3][2]) {
  uint64_t st = gen_stream(seed, g * 4 + (uint64_t)mu);
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) gen_gauss(&st, &m[r][c][0], &m[r][c][1]);
  for (int r = 0; r < 3; ++r) {
    for (int q = 0; q < r; ++q) {
      /* d = <row q, row r> = sum_c conj(m[q][c]) m[r][c] */
      double d[2] = {0.0, 0.0};
      for (int c = 0; c < 3; ++c) {
        d[0] += m[q][c][0] * m[r][c][0] + m[q][c][1] * m[r][c][1];
        d[1] += m[q][c][0] * m[r][c][1] - m[q][c][1] * m[r][c][0];
      }
      for (int c = 0; c < 3; ++c) {
        double t[2];
        gen_mul(d, m[q][c], t);
        m[r][c][0] -= t[0];
        m[r][c][1] -= t[1];
      }
    }
    double n = 0.0;
    for (int c = 0; c < 3; ++c) n += m[r][c][0] * m[r][c][0] + m[r][c][1] * m[r][c][1];
    n = 1.0 / sqrt(n);
    for (int c = 0; c < 3; ++c) {
      m[r][c][0] *= n;
      m[r][c][1] *= n;
    }
  }
  /* det by the first row's cofactors */
  double p[6][2], cof[3][2], a[3][2];
  gen_mul(m[1][1], m[2][2], p[0]);
  gen_mul(m[1][2], m[2][1], p[1]);
  gen_mul(m[1][0], m[2][2], p[2]);
  gen_mul(m[1][2], m[2][0], p[3]);
  gen_mul(m[1][0], m[2][1], p[4]);
  gen_mul(m[1][1], m[2][0], p[5]);
  for (int k = 0; k < 3; ++k) {
    cof[k][0] = p[2 * k][0] - p[2 * k + 1][0];
    cof[k][1] = p[2 * k][1] - p[2 * k + 1][1];
    gen_mul(m[0][k], cof[k], a[k]);
  }
  const double dre = a[0][0] - a[1][0] + a[2][0];
  const double dim = a[0][1] - a[1][1] + a[2][1];
  const double dn = 1.0 / sqrt(dre * dre + dim * dim);
  const double ph[2] = {dre * dn, -dim * dn};
  for (int c = 0; c < 3; ++c) {
    double t[2];
    gen_mul(m[2][c], ph, t);
    m[2][c][0] = t[0];
    m[2][c][1] = t[1];
  }
}

typedef struct {
  int L[4], split[4], O[4], stride[4];
  int nsimd;
  uint64_t nouter;
} GenLayout;

static int gen_layout(GenLayout* g, const int* dims, int nsimd) {
  if (!dims || (nsimd != 1 && nsimd != 2 && nsimd != 4 && nsimd != 8 && nsimd != 16)) return 0;
  int left = nsimd;
  for (int d = 3; d >= 0; --d) {
    g->split[d] = left >= 2 ? 2 : 1;
    if (left >= 2) left /= 2;
  }
  uint64_t V = 1;
  int st = 1;
  for (int d = 0; d < 4; ++d) {
    g->L[d] = dims[d];
    if (dims[d] < 1 || dims[d] > 4096 || dims[d] % g->split[d]) return 0;
    g->O[d] = dims[d] / g->split[d];
    g->stride[d] = st;
    st *= g->split[d];
    V *= (uint64_t)dims[d];
  }
  g->nsimd = nsimd;
  g->nouter = V / (uint64_t)nsimd;
  return 1;
}

static uint64_t gen_global(const GenLayout* g, const int x[4]) {
  return (uint64_t)x[0] +
         (uint64_t)g->L[0] * ((uint64_t)x[1] + (uint64_t)g->L[1] * ((uint64_t)x[2] + (uint64_t)g->L[2] * (uint64_t)x[3]));
}

static void gen_coords(const GenLayout* g, uint64_t o, int lane, int x[4]) {
  for (int d = 0; d < 4; ++d) {
    x[d] = (int)(o % (uint64_t)g->O[d]) + g->O[d] * ((lane / g->stride[d]) % g->split[d]);
    o /= (uint64_t)g->O[d];
  }
}

uint64_t or_seed_from_ints(const int* seeds, int n) {
  uint64_t st = 0x6A09E667F3BCC909ull, h = 0;
  for (int i = 0; i < n; ++i) {
    st ^= (uint64_t)(uint32_t)seeds[i] + 0x100000000ull * (uint64_t)(i + 1);
    h ^= gen_next(&st);
  }
  return h;
}

int or_generate_gauge(const int* dims, int nsimd, uint64_t seed, double* U) {
  GenLayout g;
  if (!gen_layout(&g, dims, nsimd) || !U) return 1;
  const int64_t nout = (int64_t)g.nouter;
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < nout; ++o) {
    for (int lane = 0; lane < nsimd; ++lane) {
      int x[4];
      gen_coords(&g, (uint64_t)o, lane, x);
      for (int mu = 0; mu < 4; ++mu) {
        double m[3][3][2];
        int xb[4] = {x[0], x[1], x[2], x[3]};
        xb[mu] = (xb[mu] + g.L[mu] - 1) % g.L[mu];
        for (int half = 0; half < 2; ++half) {
          gen_su3(seed, gen_global(&g, half ? xb : x), mu, m);
          const uint64_t link = (uint64_t)o * 8 + (uint64_t)(mu + 4 * half);
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
              /* forward: m[r][c]; backward: conj(m[c][r]) */
              const double re = half ? m[c][r][0] : m[r][c][0];
              const double im = half ? -m[c][r][1] : m[r][c][1];
              const uint64_t k = ((link * 9 + (uint64_t)(r * 3 + c)) * (uint64_t)nsimd + (uint64_t)lane) * 2;
              U[k] = re;
              U[k + 1] = im;
            }
        }
      }
    }
  }
  return 0;
}

int or_generate_fermion(const int* dims, int Ls, int nsimd, uint64_t seed, double* phi) {
  GenLayout g;
  if (!gen_layout(&g, dims, nsimd) || Ls < 1 || !phi) return 1;
  const int64_t nout = (int64_t)g.nouter;
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < nout; ++o) {
    for (int lane = 0; lane < nsimd; ++lane) {
      int x[4];
      gen_coords(&g, (uint64_t)o, lane, x);
      const uint64_t gs = gen_global(&g, x);
      for (int s = 0; s < Ls; ++s) {
        uint64_t st = gen_stream(seed, gs * (uint64_t)Ls + (uint64_t)s);
        for (int sc = 0; sc < 12; ++sc) {
          const uint64_t k = ((((uint64_t)o * (uint64_t)Ls + (uint64_t)s) * 12 + (uint64_t)sc) * (uint64_t)nsimd +
                              (uint64_t)lane) * 2;
          gen_gauss(&st, &phi[k], &phi[k + 1]);
        }
      }
    }
  }
  return 0;
}

int or_generate_table(const int* dims, int Ls, int nsimd, uint64_t* nbr, uint8_t* prm) {
  GenLayout g;
  if (!gen_layout(&g, dims, nsimd) || Ls < 1) return 1;
  const int64_t nout = (int64_t)g.nouter;
#pragma omp parallel for schedule(static)
  for (int64_t o = 0; o < nout; ++o) {
    int oc[4];
    uint64_t r = (uint64_t)o;
    for (int d = 0; d < 4; ++d) {
      oc[d] = (int)(r % (uint64_t)g.O[d]);
      r /= (uint64_t)g.O[d];
    }
    for (int mu = 0; mu < 8; ++mu) {
      const int d = mu & 3;
      int on[4] = {oc[0], oc[1], oc[2], oc[3]};
      const int wrap = mu < 4 ? (on[d] == g.O[d] - 1) : (on[d] == 0);
      on[d] = mu < 4 ? (wrap ? 0 : on[d] + 1) : (wrap ? g.O[d] - 1 : on[d] - 1);
      const uint64_t nb = (uint64_t)on[0] +
                          (uint64_t)g.O[0] * ((uint64_t)on[1] + (uint64_t)g.O[1] * ((uint64_t)on[2] + (uint64_t)g.O[2] * (uint64_t)on[3]));
      const uint8_t p = (uint8_t)(wrap && g.split[d] == 2);
      for (int s = 0; s < Ls; ++s) {
        const uint64_t j = ((uint64_t)o * (uint64_t)Ls + (uint64_t)s) * 8 + (uint64_t)mu;
        if (nbr) nbr[j] = nb * (uint64_t)Ls + (uint64_t)s;
        if (prm) prm[j] = p;
      }
    }
  }
  return 0;
}
