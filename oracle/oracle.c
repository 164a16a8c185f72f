/*
 * ORACLE -- test infrastructure only.  CPU restatement of GridBench's scalar hopping term,
 * used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to check and to
 * time against.  Nothing in the product library links or calls this file.
 *
 * Parity pin: tests compare this restatement with the reference's own dslash_simple.h
 * compiled in place (oracle/build.py -> oracle/_ref/) and with golden vectors made by that
 * build (tests/golden/).
 *
 * Layout (Nsimd = 1): Psi/Phi[(site*Ls+s)*12 + spin*3 + colour] complex, U[(site*8+mu)*9 +
 * row*3 + col] complex, nbr[(site*Ls+s)*8+mu] a 5D index (dslash_simple.h:3-5,40).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

/* Threads of the parallel loops below (the CPU baseline is timed at one thread and at all). */
void or_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int or_max_threads(void) { return omp_get_max_threads(); }

#define OR_CAT2(a, b) a##b
#define OR_CAT(a, b) OR_CAT2(a, b)

/* ------------------------------------------------------------------------------------------
 * The kernel body is written once over REAL (double or float) and instantiated twice.
 * Complex numbers are (re, im) pairs of REAL.
 * ------------------------------------------------------------------------------------------ */

#define REAL double
#define SFX _d
#include "oracle_body.h"
#undef REAL
#undef SFX

#define REAL float
#define SFX _f
#include "oracle_body.h"
#undef REAL
#undef SFX
