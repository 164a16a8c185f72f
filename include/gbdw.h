/*
 * gbdw.h -- C ABI of the GB300 domain-wall Wilson hopping-term library (libgbdw.so).
 *
 * Plain C: opaque handles, plain pointers and sizes, integer status codes.  No CUDA or
 * torch types appear in any signature, so the library can be bound from C, C++ (see
 * gbdw_dslash.h), ctypes, cgo or JNI alike.
 *
 * Conventions shared with GridBench (reference file:line in brackets):
 *   - spinor  Psi[(site*Ls + s)*12 + spin*3 + colour], complex, re/im interleaved
 *     [dslash_simple.h:3,144]; with Nsimd SIMD lanes every complex becomes Nsimd complexes,
 *     lane-minor [Simd_gpu_vec.h:110-128, bench.cc:105-139].
 *   - doubled gauge field U[(site*8 + mu)*9 + row*3 + col], mu = Xp,Yp,Zp,Tp,Xm,Ym,Zm,Tm
 *     [dslash_simple.h:5, WilsonKernelsHand.h:5-12]; U[mu+4](x) = U[mu](x - mu)^dagger.
 *   - neighbour table nbr[(site*Ls + s)*8 + mu] = 5D spinor index, prm[...] = lane-permute
 *     flag [TableGenerate.cc:75-91]; leg mu with prm set reads lane ^ (Nsimd >> (P+1)),
 *     P = 3,2,1,0 for X,Y,Z,T [WilsonKernelsHandGpu.h:33-41].
 *   - the output is the unscaled hopping sum, no -1/2 and no mass term [TableGenerate.cc:52].
 *
 * Every entry point returns GBDW_OK (0) or a positive gbdw_status; gbdw_last_error() gives
 * the message.  Nothing in the library exits the process.
 */
#ifndef GBDW_H
#define GBDW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status / precision */

typedef enum {
  GBDW_OK = 0,
  GBDW_ERR_INVALID = 1,       /* bad argument (null pointer, size, unsupported combination) */
  GBDW_ERR_CUDA = 2,          /* a CUDA runtime call failed */
  GBDW_ERR_ALLOC = 3,         /* device or pinned allocation failed */
  GBDW_ERR_TABLE = 4,         /* neighbour table out of range */
  GBDW_ERR_NOT_CONVERGED = 5, /* solver hit its iteration limit */
  GBDW_ERR_DIVERGED = 6,      /* solver produced a non-finite or non-positive quantity */
  GBDW_ERR_NO_DEVICE = 7,     /* no CUDA device visible */
  GBDW_ERR_TIMEOUT = 8        /* a bounded device-side wait expired (reported by gbdw_synchronize) */
} gbdw_status;

/* Storage precision of a field.  Arithmetic is FP64 for GBDW_F64 and FP32 otherwise. */
typedef enum {
  GBDW_F64 = 0,  /* complex double */
  GBDW_F32 = 1,  /* complex float */
  GBDW_F16 = 2,  /* spinor: half2 per complex + one FP32 norm per 5D site;
                    gauge : 12-real (two rows) half2, third row rebuilt as conj(r0 x r1) */
  GBDW_BF16 = 3  /* gauge only: 12-real bf16 */
} gbdw_prec;

const char* gbdw_last_error(void);
int gbdw_version(void);                 /* 100*major + minor */
int gbdw_device_available(void);        /* 1 if a CUDA device can be used, else 0 */
int gbdw_synchronize(void);             /* waits for the library stream */
uint64_t gbdw_launch_count(void);       /* kernels this process launched through the library */
int gbdw_set_stream(void* cuda_stream); /* NULL = the library's own non-blocking stream */
/* a non-blocking CUDA stream owned by the caller (for gbdw_set_stream).  Each stream the
 * library queues on gets its own scratch and staging buffers (freed by gbdw_stream_destroy for
 * streams made here, held until exit for others). */
int gbdw_stream_create(void** cuda_stream);
int gbdw_stream_destroy(void* cuda_stream);

/* ------------------------------------------------------------------ drop-in seam
 * Replaces template<class Simd> double dslash_kernel(int nrep, Simd* Up, Simd* outp,
 *   Simd* inp, uint64_t* nbr, uint64_t nsite, uint64_t Ls, uint8_t* prm)
 *   [WilsonKernelsHand.h:17-18,25-26], called from bench.cc:148-164.
 * prec is GBDW_F64 (vComplexD) or GBDW_F32 (vComplexF); nsimd is the lane count of the
 * Simd type (1 for the dslash_simple layout).  nsite counts outer (SIMD) sites, as in the
 * reference.  Pointers may be host (pageable or pinned) or device/managed memory: host
 * buffers are copied in once per call and out once after the last repetition.  The
 * hopping term is applied nrep times; *usec receives the device time of repetitions
 * 1..nrep-1 (all of them when nrep == 1), mirroring WilsonKernelsHandCpu.h:407-450.
 * dag = 1 applies DhopDag = gamma5 Dhop gamma5 (no counterpart in the reference). */
int gbdw_dslash_kernel(int nrep, int prec, int nsimd, const void* U, void* out, const void* in,
                       const uint64_t* nbr, uint64_t nsite, uint64_t Ls, const uint8_t* prm,
                       int dag, double* usec);

/* ------------------------------------------------------------------ generator
 * Seeded equivalent of TableGenerate.cc:19-91 without Grid: random SU(3) links (Gaussian
 * complex 3x3, Gram-Schmidt, det fixed to 1), the doubled field, i.i.d. N(0,1) source,
 * and nbr/prm for a periodic lattice dims[4] = {Lx,Ly,Lz,Lt} laid out with nsimd lanes
 * (1, 2, 4, 8 or 16; lanes split T first, then Z, Y, X, each split dimension halved).
 * Outputs are in the reference layout, FP64.  Any output pointer may be NULL.
 * Sizes (nsite = Lx*Ly*Lz*Lt / nsimd): U 144*nsite*nsimd doubles, phi 24*nsite*Ls*nsimd
 * doubles, nbr and prm nsite*Ls*8 entries.  Deterministic across machines. */
int gbdw_generate_gauge(const int dims[4], int nsimd, uint64_t seed, double* U);
int gbdw_generate_fermion(const int dims[4], int Ls, int nsimd, uint64_t seed, double* phi);
int gbdw_generate_table(const int dims[4], int Ls, int nsimd, uint64_t* nbr, uint8_t* prm);
uint64_t gbdw_seed_from_ints(const int* seeds, int n);  /* e.g. {1,2,3,4} as in TableGenerate */

/* ------------------------------------------------------------------ lattices and fields */

/* Device-side random inputs for large workloads (same recipe as the generator above, but
 * with CUDA's log/sincos, so the bits differ from gbdw_generate_*):
 * gbdw_field_gaussian fills right-hand side rhs with i.i.d. N(0,1) re/im;
 * gbdw_gauge_random creates a random SU(3) doubled gauge field (periodic lattices made by
 * gbdw_lattice_create); equal seeds give the same field in every precision. */

typedef struct gbdw_lattice gbdw_lattice;
typedef struct gbdw_gauge gbdw_gauge;
typedef struct gbdw_field gbdw_field;

/* Lattice from a reference neighbour table (host or device pointers).  The table is
 * range-checked; if every entry has the form nbr = nbr4(site,mu)*Ls + s with a permute
 * flag independent of s, the 4D fast path is used, otherwise the general 5D gather. */
int gbdw_lattice_from_table(gbdw_lattice** lat, uint64_t nsite, int Ls, int nsimd,
                            const uint64_t* nbr, const uint8_t* prm);
/* Periodic lattice built on the device (no table upload). */
int gbdw_lattice_create(gbdw_lattice** lat, const int dims[4], int Ls);
int gbdw_lattice_destroy(gbdw_lattice* lat);
/* info[0]=sites (4D, lanes unrolled) info[1]=Ls info[2]=nsimd info[3]=fast path (1/0) */
int gbdw_lattice_info(const gbdw_lattice* lat, int64_t info[4]);

/* Gauge field stored at prec (F64, F32, F16 or BF16) from a reference-layout doubled
 * field src (src_prec F64 or F32, host or device pointer). */
int gbdw_gauge_create(gbdw_gauge** g, const gbdw_lattice* lat, int prec, const void* src,
                      int src_prec);
int gbdw_gauge_destroy(gbdw_gauge* g);

/* Spinor field with nrhs right-hand sides (stored rhs-innermost so one gauge load serves
 * Ls*nrhs slices). */
int gbdw_field_create(gbdw_field** f, const gbdw_lattice* lat, int prec, int nrhs);
int gbdw_field_destroy(gbdw_field* f);
int gbdw_field_zero(gbdw_field* f);
/* Copy one right-hand side in from / out to the reference layout (src/dst prec F64 or F32,
 * host or device pointer). */
int gbdw_field_import(gbdw_field* f, int rhs, const void* src, int src_prec);
int gbdw_field_export(const gbdw_field* f, int rhs, void* dst, int dst_prec);
/* As gbdw_field_export, but returns once the work is queued on the library stream (dst must be
 * device or page-locked host memory; complete with gbdw_synchronize).  Host transfers run on a
 * copy engine through a staging buffer of the current stream, so imports and exports queued on
 * two streams overlap (the host link is full duplex). */
int gbdw_field_export_async(const gbdw_field* f, int rhs, void* dst, int dst_prec);
/* dst = src with precision conversion (same lattice and nrhs). */
int gbdw_field_copy(gbdw_field* dst, const gbdw_field* src);
int gbdw_field_gaussian(gbdw_field* f, int rhs, uint64_t seed);
int gbdw_gauge_random(gbdw_gauge** g, const gbdw_lattice* lat, int prec, uint64_t seed);

/* ------------------------------------------------------------------ operators
 * out = Dhop(in) (dag=0) or DhopDag(in) (dag=1) over all right-hand sides. */
int gbdw_dhop(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag);

/* Shamir domain-wall operator (no counterpart in the reference):
 *   (M psi)(s) = (5 - M5) psi(s) - 1/2 Dhop psi(s) - P- psi(s+1) - P+ psi(s-1),
 * P+- = (1 +- gamma5)/2, gamma5 = diag(1,1,-1,-1), and the s-wrap terms carry -mf.
 * dag = 1 applies M^dagger.  If norm2 is non-NULL it receives |out|^2 (FP64 sum). */
int gbdw_dwf_m(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, double M5, double mf,
               int dag, double* norm2);
/* out = M^dagger M in, tmp holds M in.  If pap is non-NULL it receives <in, out> = |M in|^2. */
int gbdw_dwf_mdagm(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in,
                   double M5, double mf, double* pap);

/* ------------------------------------------------------------------ BLAS-1 (FP64 sums) */
int gbdw_norm2(const gbdw_field* x, double* out);
int gbdw_dot(const gbdw_field* x, const gbdw_field* y, double* re, double* im); /* <x,y> */
int gbdw_axpby(double a, const gbdw_field* x, double b, gbdw_field* y);          /* y=ax+by */

/* ------------------------------------------------------------------ solvers
 * Solve M^dagger M x = b for the Shamir operator.  mode:
 *   GBDW_CG_PLAIN : FP32 operator, FP64 x/r/p vectors and sums, reliable updates with the
 *                   FP64 operator (the plain FP32-kernel / FP64-residual solve);
 *   GBDW_CG_MIXED : sloppy operator at sloppy_prec (F16 spinor + 12-real F16 gauge, or F32),
 *                   low-precision inner vectors, reliable updates that recompute the true
 *                   residual r = b - A x, the sums and the solution in FP64;
 *   GBDW_CG_DOUBLE: everything FP64 (accuracy reference).
 * b and x are FP64 fields.  Stops when the true relative residual |b-Ax|/|b| <= tol. */
enum { GBDW_CG_PLAIN = 0, GBDW_CG_MIXED = 1, GBDW_CG_DOUBLE = 2 };
typedef struct {
  double tol;           /* target true relative residual, e.g. 1e-10 */
  int max_iter;         /* iteration limit (GBDW_ERR_NOT_CONVERGED beyond it) */
  double delta;         /* reliable-update threshold on |r|/max|r| (e.g. 0.1) */
  int sloppy_prec;      /* GBDW_F16 or GBDW_F32 for GBDW_CG_MIXED */
  int sloppy_gauge;     /* GBDW_F16, GBDW_BF16 or GBDW_F32 */
  int sloppy_residual;  /* GBDW_CG_MIXED with FP16 spinors and FP16 links: 1 keeps the iterated
                           residual in FP16 (per-slice norms) instead of FP32; 0 otherwise */
} gbdw_cg_params;
typedef struct {
  int iterations;
  int reliable_updates;
  double true_residual;  /* |b - A x| / |b| in FP64 at exit */
  double seconds;        /* wall time of the solve (device-synchronised) */
  double final_rr;       /* last iterated |r|^2 / |b|^2 */
} gbdw_cg_stats;
int gbdw_cg_solve(const gbdw_gauge* g_double, const gbdw_gauge* g_single,
                  const gbdw_gauge* g_sloppy, gbdw_field* x, const gbdw_field* b, double M5,
                  double mf, int mode, const gbdw_cg_params* prm, gbdw_cg_stats* stats);

/* ------------------------------------------------------------------ even-odd (red-black)
 * The 4D checkerboard of the reference's red-black grids (TableGenerate.cc:26-28,
 * makeFourDimRedBlackGrid / makeFiveDimRedBlackGrid).  No counterpart kernels exist in the
 * reference; everything here follows from the full operator by restriction:
 *   M = [[D5, -1/2 Dhop_eo], [-1/2 Dhop_oe, D5]],   D5 = the 5th-dimension (site-local) part,
 *   Mpc = D5 - 1/4 Dhop_pq D5^-1 Dhop_qp on half p.
 * Half lattices hold the sites of one parity of a periodic lattice with even extents,
 * numbered parent_site / 2; half fields and half gauge fields live on them. */
/* even (parity 0) and odd half of a lattice made by gbdw_lattice_create; destroy each half
 * with gbdw_lattice_destroy */
int gbdw_lattice_checkerboard(const gbdw_lattice* full, gbdw_lattice** even, gbdw_lattice** odd);
/* the links of the half's sites, in half-site order (a copy; precision of `full`) */
int gbdw_gauge_checkerboard(gbdw_gauge** out, const gbdw_gauge* full, const gbdw_lattice* half);
/* half <- the half's parity of full ; full <- half on the half's parity (other sites kept) */
int gbdw_field_pick(gbdw_field* half, const gbdw_field* full);
int gbdw_field_place(gbdw_field* full, const gbdw_field* half);
/* out (half p, on g's lattice) = Dhop_pq in (half q); dag: DhopDag_pq */
int gbdw_dhop_eo(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag);
/* out (half p) = D5 cen - khop Dhop_pq in (D5^dag, DhopDag for dag); khop 1/2 gives M's
 * rows of parity p */
int gbdw_dwf_meo(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, const gbdw_field* cen,
                 double M5, double mf, int dag, double khop);
/* out = D5^-1 in (D5^-dag for dag) in closed form; any lattice, single rhs, Ls <= 64 */
int gbdw_dwf_m5inv(gbdw_field* out, const gbdw_field* in, double M5, double mf, int dag);
/* out = Mpc in (Mpc^dag for dag) on half p = gp's lattice; tq1, tq2 temporaries on half q;
 * |out|^2 into norm2 when non-null */
int gbdw_dwf_mpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tq1,
                 gbdw_field* tq2, const gbdw_field* in, double M5, double mf, int dag, double* norm2);
/* out = Mpc^dag Mpc in; tp on half p, tq1/tq2 on half q; pap = |Mpc in|^2 */
int gbdw_dwf_mpcdagmpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tp,
                       gbdw_field* tq1, gbdw_field* tq2, const gbdw_field* in, double M5, double mf,
                       double* pap);
/* Solves M x = b (x, b F64 on the full lattice; x holds the initial guess) by CG on the odd
 * Schur normal system with the modes and reliable updates of gbdw_cg_solve.  g_*[0] / [1]
 * are the even / odd gauge halves (g_single for PLAIN, g_sloppy for MIXED).  tol is the
 * target of the Schur normal system's true residual; stats->true_residual reports the full
 * system's |b - M x| / |b|. */
int gbdw_cg_solve_eo(const gbdw_gauge* const g_double[2], const gbdw_gauge* const g_single[2],
                     const gbdw_gauge* const g_sloppy[2], gbdw_field* x, const gbdw_field* b,
                     double M5, double mf, int mode, const gbdw_cg_params* prm, gbdw_cg_stats* stats);

/* ------------------------------------------------------------------ Mobius / Cayley 5D operators
 * No counterpart in GridBench: the 5th-dimension operators Grid's CayleyFermion5D builds
 * around the hopping term (M5D, M5Ddag, Mooee, MooeeInv, Meooe), for Mobius domain-wall
 * fermions (Brower, Neff, Orginos, arXiv:1206.5214).  A cyclic 5th-dimension operator with
 * per-slice real coefficients (arrays of Ls entries):
 *   (A psi)(s) = diag[s] psi(s) + upper[s] P- psi(s+1) + lower[s] P+ psi(s-1),  s +- 1 mod Ls,
 * P+ keeping spins 0,1 and P- spins 2,3; dag = 1 applies the exact adjoint of the same A (Grid's
 * M5Ddag instead takes pre-shifted arrays).  Any lattice (full or half), single rhs, F64/F32/F16
 * fields, 1 <= Ls <= 64, out != in.
 * The Mobius operator (b, c, M5, mf): M = Mooee - 1/2 Dhop A(b, c) with
 *   Mooee = A(diag 1 + b (4 - M5), off-diagonal -(1 - c (4 - M5))),
 * A(d, e): diag d, lower = upper = e, the walls (upper[Ls-1], lower[0]) e -> -mf e.
 * b = 1, c = 0 is the Shamir operator of gbdw_dwf_m. */
int gbdw_m5d(gbdw_field* out, const gbdw_field* in, const double* lower, const double* diag,
             const double* upper, int dag);
/* out = A^-1 in (A^-dag for dag): two cyclic bidiagonal solves per chirality;
 * GBDW_ERR_INVALID when A is singular */
int gbdw_m5d_inv(gbdw_field* out, const gbdw_field* in, const double* lower, const double* diag,
                 const double* upper, int dag);
int gbdw_mobius_mooee(gbdw_field* out, const gbdw_field* in, double b, double c, double M5, double mf,
                      int dag);
int gbdw_mobius_mooee_inv(gbdw_field* out, const gbdw_field* in, double b, double c, double M5,
                          double mf, int dag);
/* out = M in (M^dag in for dag) on a full lattice; tmp: a field like in (distinct from out and in);
 * |out|^2 into norm2 when non-null */
int gbdw_mobius_m(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double b,
                  double c, double M5, double mf, int dag, double* norm2);
/* even-odd hopping block on half p = g's lattice, in on half q:
 * dag 0: out = -1/2 Dhop_pq A(b, c) in, tmp on half q;  dag 1: out = -1/2 A(b, c)^dag DhopDag_pq in,
 * tmp on half p */
int gbdw_mobius_meooe(const gbdw_gauge* g, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double b,
                      double c, double mf, int dag);
/* Schur operator on half p: Mpc = Mooee - Meooe_pq Mooee^-1 Meooe_qp (its adjoint for dag);
 * tp on half p, tq1 / tq2 on half q; |out|^2 into norm2 when non-null */
int gbdw_mobius_mpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tp,
                    gbdw_field* tq1, gbdw_field* tq2, const gbdw_field* in, double b, double c, double M5,
                    double mf, int dag, double* norm2);
/* out = M^dag M in (full lattice); t, tmp temporaries like in (out, t, tmp distinct);
 * pap = |M in|^2 when non-null */
int gbdw_mobius_mdagm(const gbdw_gauge* g, gbdw_field* out, gbdw_field* t, gbdw_field* tmp,
                      const gbdw_field* in, double b, double c, double M5, double mf, double* pap);
/* Solves M^dag M x = b for the Mobius operator (x, b F64 on the full lattice; x holds the initial
 * guess) with the modes, gauge fields and reliable updates of gbdw_cg_solve. */
int gbdw_cg_solve_mobius(const gbdw_gauge* g_double, const gbdw_gauge* g_single,
                         const gbdw_gauge* g_sloppy, gbdw_field* x, const gbdw_field* b, double b5,
                         double c5, double M5, double mf, int mode, const gbdw_cg_params* prm,
                         gbdw_cg_stats* stats);

/* Solves the Mobius M x = b (x, b F64 on the full lattice) by CG on the odd Schur normal system
 * Mpc^dag Mpc (Mpc = Mooee - Meooe_oe Mooee^-1 Meooe_eo), with the modes, gauge halves and
 * reliable updates of gbdw_cg_solve_eo; stats->true_residual is the full system's |b - M x| / |b|. */
int gbdw_cg_solve_mobius_eo(const gbdw_gauge* const g_double[2], const gbdw_gauge* const g_single[2],
                            const gbdw_gauge* const g_sloppy[2], gbdw_field* x, const gbdw_field* b,
                            double b5, double c5, double M5, double mf, int mode,
                            const gbdw_cg_params* prm, gbdw_cg_stats* stats);

/* ------------------------------------------------------------------ halo packing
 * No counterpart in GridBench (one node, no halo exchange): the spin-projected half spinors a
 * neighbouring domain of a 4D decomposition reads across one face of this field's local volume,
 * as Grid's Wilson compressor sends them.  face 0 (x_mu = 0) feeds the domain at -mu through
 * its forward leg mu, face 1 (x_mu = L_mu - 1) the domain at +mu through its backward leg mu+4;
 * dag = 1 packs for DhopDag.  Layout: face site (other coordinates lexicographic, lowest
 * dimension fastest) x 6 rows (h0 colours 0..2, h1 colours 0..2) x the field's slices in its
 * storage format (F64 double2 per slice; F32/F16 slice pairs (Re s, Re s+1, Im s, Im s+1) over the
 * field's padded slot count); F16 appends one FP32 norm per (face site, slice).  Fields on a
 * periodic lattice from gbdw_lattice_create; dst is device memory (16-byte aligned) or host
 * memory (copied back before returning). */
int gbdw_halo_bytes(const gbdw_field* f, int mu, size_t* bytes);
int gbdw_halo_pack(const gbdw_field* f, int mu, int face, int dag, void* dst);
/* all eight faces in one launch: dst[2*mu + face], each a 16-byte aligned device buffer of
 * gbdw_halo_bytes(f, mu) bytes */
int gbdw_halo_pack_all(const gbdw_field* f, int dag, void* const dst[8]);

/* ------------------------------------------------------------------ static-data files
 * The reference's exchange format for Grid-generated test data (TableGenerate.cc:93-138,
 * read by bench.cc:55-88 and bench_simple.cc:72-84 as compiled-in arrays): static_data.h holds
 * `nsite` (outer sites) and `Ls`, static_data.cc the arrays U_static (nsite*144*Nsimd doubles,
 * the doubled gauge field), Phi_static and Psi_cpp_static (nsite*Ls*24*Nsimd doubles, source
 * and reference Dhop result), nbr_static (uint64) and prm_static (uint8), nsite*Ls*8 each,
 * every array closed by a sentinel 0.  Host-only; no device needed. */
/* sizes of a file pair: counts = entries of U, Phi, Psi_cpp, nbr, prm (sentinels excluded) */
int gbdw_static_data_info(const char* h_path, const char* cc_path, uint64_t* nsite, int* Ls,
                          int* nsimd, uint64_t counts[5]);
/* reads the five arrays into caller buffers whose lengths must equal the counts above */
int gbdw_static_data_read(const char* cc_path, double* U, uint64_t nU, double* Phi, uint64_t nPhi,
                          double* Psi, uint64_t nPsi, uint64_t* nbr, uint64_t nnbr, uint8_t* prm,
                          uint64_t nprm);
/* writes a file pair in the reference's layout (doubles as %16.8le: 9 significant digits) */
int gbdw_static_data_write(const char* h_path, const char* cc_path, uint64_t nsite, int Ls, int nsimd,
                           const double* U, const double* Phi, const double* Psi,
                           const uint64_t* nbr, const uint8_t* prm);

/* ------------------------------------------------------------------ batched persistent Dhop
 * Many independent instances (own lattice, gauge field, Ls, right-hand sides and precision) in
 * one persistent launch, replayed through a CUDA graph; the launch shape and the Ls / RHS
 * tiling are chosen by timing the caller's own batch at creation. */
typedef struct gbdw_batch gbdw_batch;
int gbdw_batch_create(gbdw_batch** b, int n, const gbdw_gauge* const* gauges,
                      gbdw_field* const* outs, const gbdw_field* const* ins, int dag);
int gbdw_batch_run(gbdw_batch* b);        /* one graph replay */
int gbdw_batch_destroy(gbdw_batch* b);
/* info[0]=work items info[1]=persistent CTAs info[2]=threads per CTA info[3]=graph (1/0) */
int gbdw_batch_info(const gbdw_batch* b, int64_t info[4]);
/* The autotuned shape: shape[0] threads per CTA, shape[1] / shape[2] slices per thread of the
 * FP32 / FP16 instances, shape[3] tile split (each site's Ls*nrhs slices are cut into up to
 * this many contiguous tiles: an Ls tile of some values of s with every right-hand side, or an
 * RHS tile of some right-hand sides at one s). */
int gbdw_batch_shape(const gbdw_batch* b, int shape[4]);
/* Pins a shape (same meaning; threads 64/128, slices per thread 1 or 2, split a power of two)
 * and rebuilds the graph. */
int gbdw_batch_set_shape(gbdw_batch* b, const int shape[4]);

/* ------------------------------------------------------------------ autotuner
 * Times the launch shapes of the hopping kernel for (g, field) and stores the fastest in
 * the process cache and, if path is non-NULL, in a JSON file read back by gbdw_tune_load.
 * Untuned shapes use built-in defaults.  Even-odd operands (g and out on one half lattice, in on
 * its partner, as gbdw_dhop_eo takes them) tune the even-odd hopping term and its Schur epilogue
 * under keys of their own; a half lattice without them runs the full lattice's shapes.  The
 * gbdw_tune_query / _set / _split / _brick calls on a half-lattice gauge field read and pin those. */
int gbdw_tune_dhop(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag);
int gbdw_tune_load(const char* path);
int gbdw_tune_save(const char* path);
/* Writes the chosen shape for a field into cfg[4]: threads per CTA, slices per thread,
 * form (0 direct loads, 1 TMA-staged neighbour blocks with one ring per CTA, 2 the same with
 * one ring per warp, 3 the direct form specialised for FP32/FP16 with Ls*nrhs = 16, 4 form 3 over 2x2x2x2
 * site blocks on periodic lattices with even extents) and stages of
 * the staged forms. */
int gbdw_tune_query(const gbdw_gauge* g, const gbdw_field* in, int cfg[4]);
/* Pins the shape for fields like `in` (threads a multiple of 32 up to 256; slices per thread
 * 1, 2 or 4 dividing Ls*nrhs, at most 2 for F64; form 0..4; stages 2/4). */
int gbdw_tune_set(const gbdw_gauge* g, const gbdw_field* in, int threads, int spt, int form, int stages);
/* Ls / RHS tiles of the direct forms (0 and 3): each site's Ls*nrhs slices are cut into `split`
 * contiguous tiles, threads ordered (tile, site, slice group), so each tile is one sweep over all
 * sites: a CTA holds more sites with fewer slices each (one link load per site and tile), and a
 * site's spinor is reused by its neighbours within a shorter stretch of the sweep.  The tuner
 * chooses among the splits 1, 2, 3, 4, 6, 8, 12, 16 that cut whole slice groups;
 * gbdw_tune_split reads the choice for fields like `in`, gbdw_tune_set_split pins it (1 = whole
 * sites; gbdw_tune_set resets it to 1). */
int gbdw_tune_split(const gbdw_gauge* g, const gbdw_field* in, int* split);
int gbdw_tune_set_split(const gbdw_gauge* g, const gbdw_field* in, int split);
/* t-brick sweep order of the direct forms on periodic lattices: sites are visited as (t brick,
 * z, y, x, t inside the brick), so neighbours along t are read close together in the sweep instead
 * of a whole 3D volume apart (what lets a site's spinor leave L2 before its next reader when a
 * site holds many slices, e.g. many right-hand sides).  The tuner chooses among 1 (natural order),
 * 2, 4, 8; gbdw_tune_brick reads the choice, gbdw_tune_set_brick pins it (Lt must be a multiple). */
int gbdw_tune_brick(const gbdw_gauge* g, const gbdw_field* in, int* brick);
int gbdw_tune_set_brick(const gbdw_gauge* g, const gbdw_field* in, int brick);
/* The shape of the Shamir M pass (and of the CG passes built on it) for fields like `in` with one
 * right-hand side: cfg[6] = threads, slices per thread, form, stages, split, brick.  gbdw_tune_dhop
 * times M over the same candidates as the hopping term and keeps its own fastest; the gbdw_tune_set*
 * calls pin the hopping term, M and the CG steps together. */
int gbdw_tune_query_m(const gbdw_gauge* g, const gbdw_field* in, int cfg[6]);
/* The shape of the fused CG step (M with |M p|^2 reduced, then M^dag with r -= alpha M^dag M p and
 * |r|^2 reduced) for an iterated residual of precision rprec (GBDW_F64/F32/F16), same cfg[6]
 * layout.  gbdw_tune_dhop times that step on a shortlist of M's fastest shapes; untuned, it is M's. */
int gbdw_tune_query_cg(const gbdw_gauge* g, const gbdw_field* in, int rprec, int cfg[6]);

/* ------------------------------------------------------------------ FP64 arithmetic
 * GB300 executes FP64 at 1/64 of its FP32 rate, which leaves the FP64 hopping operator bound by
 * its arithmetic, far from its memory roofline.  Its double-single form keeps the FP64 fields
 * and gauge in memory and computes on FP32 pairs (~48 significant bits, ~1e-14 relative against
 * FP64).  `where` selects the explicit FP64 operator calls (gbdw_dhop, gbdw_dwf_m, ... on F64
 * fields; default GBDW_FP64_NATIVE) or the solvers' FP64 operator (true residuals, the FP64 CG;
 * default GBDW_FP64_DOUBLE_SINGLE).  The setting is process-wide. */
enum { GBDW_FP64_OPERATORS = 0, GBDW_FP64_SOLVERS = 1 };
enum { GBDW_FP64_NATIVE = 0, GBDW_FP64_DOUBLE_SINGLE = 1 };
int gbdw_set_fp64_arith(int where, int mode);
int gbdw_get_fp64_arith(int where, int* mode);
/* gbdw_tune_dhop on F64 fields while explicit operators run double-single tunes that form's
 * shapes (used by the solvers as well): cfg[2] = CTAs per SM the registers are capped for (3 or
 * 4) and the t-brick sweep order, for Dhop (epi 0) or M (epi 1). */
int gbdw_tune_query_ds(const gbdw_gauge* g, const gbdw_field* in, int epi, int cfg[2]);
int gbdw_tune_set_ds(const gbdw_gauge* g, const gbdw_field* in, int epi, int minb, int brick);

/* ------------------------------------------------------------------ timing on the library stream */
typedef struct gbdw_timer gbdw_timer;
int gbdw_timer_create(gbdw_timer** t);
int gbdw_timer_start(gbdw_timer* t);
int gbdw_timer_stop(gbdw_timer* t, double* ms); /* synchronises, returns elapsed ms */
int gbdw_timer_destroy(gbdw_timer* t);
/* Writes nbytes of junk through a scratch buffer to evict L2 (no-op if nbytes == 0). */
int gbdw_flush_l2(size_t nbytes);

/* Runs one CTA whose bounded mbarrier wait cannot complete (nothing is copied), so it expires
 * after limit_ns (at most 0.1 s); the next gbdw_synchronize() then reports GBDW_ERR_TIMEOUT.
 * Exercises the timeout path of the staged kernels without any fault. */
int gbdw_selftest_wait_timeout(uint64_t limit_ns);

/* Sum of |x_i|^2 in FP64 over n complex numbers (re, im interleaved; prec GBDW_F64 or
 * GBDW_F32) in device memory the caller owns, written to *result (host).  For callers that
 * cannot allocate device memory -- programs whose own pool allocator owns the GPU, solver
 * loops that must not pay cudaMalloc's latency -- it allocates nothing: its partial sums live
 * in a fixed 8 KB device array that every GPU loading the library keeps until exit.  No
 * counterpart in the reference.  Limit: n <= 2^24 (larger n returns GBDW_ERR_INVALID).  All
 * calls share that array, so calls that overlap on the GPU race; calls in one stream do not.
 * The first call on each device looks the array up (cudaGetSymbolAddress).  The call is
 * synchronous (it copies the result to the host and waits for the library's stream), so it
 * must not be made while any stream is being captured into a CUDA graph.  It reads x on the
 * library's stream: x must be complete with respect to that stream (synchronise the stream
 * that wrote x first, or make it the library's stream with gbdw_set_stream).  Single device,
 * like the rest of the library: once the library has run, a call made with a device current
 * other than the one it first ran on returns GBDW_ERR_INVALID. */
int gbdw_norm2_noalloc(const void* x, int prec, uint64_t n, double* result);

/* Host-side fault injection for tests (no counterpart in the reference; GridBench exits on
 * any CUDA error, Macros.h:47-51): after `skip` more device allocations made by the library,
 * the next `count` fail exactly as an exhausted device makes cudaMalloc fail, so the caller
 * sees GBDW_ERR_ALLOC; later allocations succeed again.  count = 0 switches injection off.
 * No kernel is involved: the GPU never faults. */
int gbdw_debug_fail_allocs(int skip, int count);

/* Page-locked host memory for fast host<->device copies of reference-layout buffers. */
int gbdw_host_alloc(size_t nbytes, void** ptr);
int gbdw_host_free(void* ptr);

#ifdef __cplusplus
}
#endif
#endif /* GBDW_H */
