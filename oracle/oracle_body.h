/*
 * ORACLE body (test infrastructure only), included by oracle.c once per REAL type.
 */

typedef struct {
  REAL re, im;
} OR_CAT(cx, SFX);
#define CX OR_CAT(cx, SFX)

static inline CX OR_CAT(cadd, SFX)(CX a, CX b) { CX r = {a.re + b.re, a.im + b.im}; return r; }
static inline CX OR_CAT(csub, SFX)(CX a, CX b) { CX r = {a.re - b.re, a.im - b.im}; return r; }
static inline CX OR_CAT(cmul, SFX)(CX a, CX b) {
  CX r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return r;
}
/* i*a and -i*a */
static inline CX OR_CAT(ci, SFX)(CX a) { CX r = {-a.im, a.re}; return r; }
static inline CX OR_CAT(cmi, SFX)(CX a) { CX r = {a.im, -a.re}; return r; }

#define CADD OR_CAT(cadd, SFX)
#define CSUB OR_CAT(csub, SFX)
#define CMUL OR_CAT(cmul, SFX)
#define CI OR_CAT(ci, SFX)
#define CMI OR_CAT(cmi, SFX)

/* Two-spin projection for leg mu (dslash_simple.h:42-83).  dag applies the leg's
 * opposite-sign partner (gamma5 Dhop gamma5), which is the projection of leg mu^4. */
static void OR_CAT(project, SFX)(int mu, const CX* p /* [4][3] */, CX chi[2][3]) {
  for (int c = 0; c < 3; ++c) {
    const CX p0 = p[0 * 3 + c], p1 = p[1 * 3 + c], p2 = p[2 * 3 + c], p3 = p[3 * 3 + c];
    switch (mu) {
      case 0: chi[0][c] = CSUB(p0, CI(p3)); chi[1][c] = CSUB(p1, CI(p2)); break;  /* Xp */
      case 1: chi[0][c] = CADD(p0, p3);     chi[1][c] = CSUB(p1, p2);     break;  /* Yp */
      case 2: chi[0][c] = CSUB(p0, CI(p2)); chi[1][c] = CADD(p1, CI(p3)); break;  /* Zp */
      case 3: chi[0][c] = CSUB(p0, p2);     chi[1][c] = CSUB(p1, p3);     break;  /* Tp */
      case 4: chi[0][c] = CADD(p0, CI(p3)); chi[1][c] = CADD(p1, CI(p2)); break;  /* Xm */
      case 5: chi[0][c] = CSUB(p0, p3);     chi[1][c] = CADD(p1, p2);     break;  /* Ym */
      case 6: chi[0][c] = CADD(p0, CI(p2)); chi[1][c] = CSUB(p1, CI(p3)); break;  /* Zm */
      default: chi[0][c] = CADD(p0, p2);    chi[1][c] = CADD(p1, p3);     break;  /* Tm */
    }
  }
}

/* Four-spin reconstruction and accumulation for leg mu (dslash_simple.h:88-141). */
static void OR_CAT(reconstruct, SFX)(int mu, CX uchi[2][3], CX* r /* [4][3] */) {
  for (int c = 0; c < 3; ++c) {
    const CX u0 = uchi[0][c], u1 = uchi[1][c];
    r[0 * 3 + c] = CADD(r[0 * 3 + c], u0);
    r[1 * 3 + c] = CADD(r[1 * 3 + c], u1);
    CX* r2 = &r[2 * 3 + c];
    CX* r3 = &r[3 * 3 + c];
    switch (mu) {
      case 0: *r2 = CADD(*r2, CI(u1)); *r3 = CADD(*r3, CI(u0)); break;
      case 1: *r2 = CSUB(*r2, u1);     *r3 = CADD(*r3, u0);     break;
      case 2: *r2 = CADD(*r2, CI(u0)); *r3 = CSUB(*r3, CI(u1)); break;
      case 3: *r2 = CSUB(*r2, u0);     *r3 = CSUB(*r3, u1);     break;
      case 4: *r2 = CSUB(*r2, CI(u1)); *r3 = CSUB(*r3, CI(u0)); break;
      case 5: *r2 = CADD(*r2, u1);     *r3 = CSUB(*r3, u0);     break;
      case 6: *r2 = CSUB(*r2, CI(u0)); *r3 = CADD(*r3, CI(u1)); break;
      default: *r2 = CADD(*r2, u0);    *r3 = CADD(*r3, u1);     break;
    }
  }
}

/* SU(3) times two colour vectors: uchi[h][r] = sum_c U[r][c] chi[h][c] (dslash_simple.h:7-17). */
static void OR_CAT(su3_mult, SFX)(const CX* u /* [3][3] */, CX chi[2][3], CX uchi[2][3]) {
  for (int h = 0; h < 2; ++h)
    for (int r = 0; r < 3; ++r) {
      CX a = CMUL(u[r * 3 + 0], chi[h][0]);
      a = CADD(a, CMUL(u[r * 3 + 1], chi[h][1]));
      a = CADD(a, CMUL(u[r * 3 + 2], chi[h][2]));
      uchi[h][r] = a;
    }
}

/* One 5D site of the hopping term: out[12] = sum over 8 legs (dslash_simple.h:30-149).
 * nbr_of(mu) gives the 5D neighbour index. */
static void OR_CAT(dhop_site, SFX)(const CX* U, const CX* in, const uint64_t* nb, uint64_t site, int dag, CX* out) {
  CX res[12];
  memset(res, 0, sizeof res);
  for (int mu = 0; mu < 8; ++mu) {
    const CX* p = in + nb[mu] * 12;
    CX chi[2][3], uchi[2][3];
    const int spin_leg = dag ? (mu ^ 4) : mu;
    OR_CAT(project, SFX)(spin_leg, p, chi);
    OR_CAT(su3_mult, SFX)(U + (site * 8 + (uint64_t)mu) * 9, chi, uchi);
    OR_CAT(reconstruct, SFX)(spin_leg, uchi, res);
  }
  memcpy(out, res, sizeof res);
}

/* Hopping term over the whole lattice, Nsimd = 1 layout.  prm is ignored as in
 * dslash_simple.h (it is all zero for Nsimd = 1).  OpenMP over 4D sites like the reference's
 * CPU kernel (WilsonKernelsHandCpu.h:423-426). */
void OR_CAT(or_dslash, SFX)(const REAL* Up, REAL* Psip, const REAL* Phip, const uint64_t* nbr, uint64_t nsite,
                            uint64_t Ls, const uint8_t* prm, int dag) {
  (void)prm;
  const CX* U = (const CX*)Up;
  const CX* Phi = (const CX*)Phip;
  CX* Psi = (CX*)Psip;
  const int64_t ns = (int64_t)nsite;
#pragma omp parallel for schedule(static)
  for (int64_t site = 0; site < ns; ++site)
    for (uint64_t s = 0; s < Ls; ++s) {
      const uint64_t s5 = (uint64_t)site * Ls + s;
      OR_CAT(dhop_site, SFX)(U, Phi, nbr + s5 * 8, (uint64_t)site, dag, Psi + s5 * 12);
    }
}

/* The same over 4D sites [site0, site1) only: a bounded sample of the full lattice for the
 * CPU baseline timing. */
void OR_CAT(or_dslash_sites, SFX)(const REAL* Up, REAL* Psip, const REAL* Phip, const uint64_t* nbr,
                                  uint64_t site0, uint64_t site1, uint64_t Ls, int dag) {
  const CX* U = (const CX*)Up;
  const CX* Phi = (const CX*)Phip;
  CX* Psi = (CX*)Psip;
#pragma omp parallel for schedule(static)
  for (int64_t site = (int64_t)site0; site < (int64_t)site1; ++site)
    for (uint64_t s = 0; s < Ls; ++s) {
      const uint64_t s5 = (uint64_t)site * Ls + s;
      OR_CAT(dhop_site, SFX)(U, Phi, nbr + s5 * 8, (uint64_t)site, dag, Psi + s5 * 12);
    }
}

/* Hopping term on the SIMD-lane layout: every complex of the Nsimd=1 layout becomes nsimd
 * complexes, lane-minor.  A leg with prm set reads lane ^ (nsimd >> (P+1)), P = 3,2,1,0 for
 * X,Y,Z,T (WilsonKernelsHandGpu.h:33-41, permute semantics Simd.h:105-116). */
void OR_CAT(or_dslash_lanes, SFX)(const REAL* Up, REAL* Psip, const REAL* Phip, const uint64_t* nbr,
                                  uint64_t nsite, uint64_t Ls, const uint8_t* prm, int nsimd, int dag) {
  const CX* U = (const CX*)Up;
  const CX* Phi = (const CX*)Phip;
  CX* Psi = (CX*)Psip;
  const int64_t ns = (int64_t)nsite;
#pragma omp parallel for schedule(static)
  for (int64_t site = 0; site < ns; ++site)
    for (uint64_t s = 0; s < Ls; ++s)
      for (int lane = 0; lane < nsimd; ++lane) {
        const uint64_t s5 = (uint64_t)site * Ls + s;
        CX res[12];
        memset(res, 0, sizeof res);
        for (int mu = 0; mu < 8; ++mu) {
          const int P = 3 - (mu & 3);
          const int pl = prm[s5 * 8 + mu] ? (lane ^ (nsimd >> (P + 1))) : lane;
          CX p[12], u[9];
          for (int k = 0; k < 12; ++k) p[k] = Phi[(nbr[s5 * 8 + mu] * 12 + (uint64_t)k) * nsimd + pl];
          for (int k = 0; k < 9; ++k) u[k] = U[(((uint64_t)site * 8 + mu) * 9 + (uint64_t)k) * nsimd + lane];
          CX chi[2][3], uchi[2][3];
          const int spin_leg = dag ? (mu ^ 4) : mu;
          OR_CAT(project, SFX)(spin_leg, p, chi);
          OR_CAT(su3_mult, SFX)(u, chi, uchi);
          OR_CAT(reconstruct, SFX)(spin_leg, uchi, res);
        }
        for (int k = 0; k < 12; ++k) Psi[(s5 * 12 + (uint64_t)k) * nsimd + lane] = res[k];
      }
}

/* Shamir domain-wall operator on the Nsimd = 1 layout (no counterpart in the reference):
 *   (M psi)(s) = (5-M5) psi(s) - 1/2 Dhop psi(s) - P- psi(s+1) - P+ psi(s-1)
 * with P+ keeping spins 0,1, P- spins 2,3, and -mf on the steps that wrap in s.
 * dag = 1: M^dagger = (5-M5) - 1/2 DhopDag - P+ psi(s+1) - P- psi(s-1). */
void OR_CAT(or_dwf_m, SFX)(const REAL* Up, REAL* outp, const REAL* inp, const uint64_t* nbr, uint64_t nsite,
                           uint64_t Ls, double M5, double mf, int dag) {
  const CX* U = (const CX*)Up;
  const CX* in = (const CX*)inp;
  CX* out = (CX*)outp;
  const int64_t ns = (int64_t)nsite;
  const REAL a5 = (REAL)(5.0 - M5);
#pragma omp parallel for schedule(static)
  for (int64_t site = 0; site < ns; ++site)
    for (uint64_t s = 0; s < Ls; ++s) {
      const uint64_t s5 = (uint64_t)site * Ls + s;
      CX d[12];
      OR_CAT(dhop_site, SFX)(U, in, nbr + s5 * 8, (uint64_t)site, dag, d);
      const uint64_t sp = (s + 1 == Ls) ? 0 : s + 1;
      const uint64_t sm = (s == 0) ? Ls - 1 : s - 1;
      const REAL fp = (s + 1 == Ls) ? (REAL)(-mf) : (REAL)1;
      const REAL fm = (s == 0) ? (REAL)(-mf) : (REAL)1;
      const CX* cen = in + s5 * 12;
      const CX* up = in + ((uint64_t)site * Ls + sp) * 12;
      const CX* dn = in + ((uint64_t)site * Ls + sm) * 12;
      for (int k = 0; k < 12; ++k) {
        const int spin = k / 3;
        /* which neighbour slice feeds this spin */
        const int from_up = dag ? (spin < 2) : (spin >= 2);
        const CX nb = from_up ? up[k] : dn[k];
        const REAL f = from_up ? fp : fm;
        CX v;
        v.re = a5 * cen[k].re - (REAL)0.5 * d[k].re - f * nb.re;
        v.im = a5 * cen[k].im - (REAL)0.5 * d[k].im - f * nb.im;
        out[s5 * 12 + k] = v;
      }
    }
}

#undef CX
#undef CADD
#undef CSUB
#undef CMUL
#undef CI
#undef CMI
