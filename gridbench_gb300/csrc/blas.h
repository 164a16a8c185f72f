// Internal BLAS-1 entry points (no argument checking beyond precision support).
#pragma once
#include "common.cuh"

namespace gbdw {
int blas_norm2(const gbdw_field* x, double* out, bool fetch);
int blas_dot(const gbdw_field* x, const gbdw_field* y, double* re, double* im);
int blas_axpby(double a, const gbdw_field* x, double b, gbdw_field* y);
// r = b - t and rr = |r|^2 (b, r F64; t F64 or F32)
int blas_xmy_norm(const gbdw_field* b, const gbdw_field* t, gbdw_field* r, double* rr);
// r -= alpha ap ; rr = |r|^2
int blas_cg_r(double alpha, gbdw_field* r, const gbdw_field* ap, double* rr);
// x += alpha p ; p = r + beta p (both with the old p) ; q = p when q != NULL
int blas_cg_xp(double alpha, double beta, gbdw_field* x, gbdw_field* p, const gbdw_field* r, gbdw_field* q);
// p = r + beta p ; q = p when q != NULL
int blas_cg_p(double beta, const gbdw_field* r, gbdw_field* p, gbdw_field* q);
int field_convert(gbdw_field* dst, const gbdw_field* src);
}  // namespace gbdw
