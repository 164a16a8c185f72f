// Internal even-odd building blocks (eo.cu), used by the solvers.
#pragma once
#include "common.cuh"

namespace gbdw {
// out = D5^-1 in (D5^-dag for dag), site-local, any lattice
int m5inv(gbdw_field* out, const gbdw_field* in, double M5, double mf, int dag);
// operands of the even-odd hopping term: gauge and out on one half lattice, in on its partner
int check_eo(const gbdw_gauge* g, const gbdw_field* out, const gbdw_field* in);
// out (half p) = Dhop_pq in (half q); with cen (half p): out = D5 cen - khop Dhop_pq in
struct DhopExtra;
int hop_eo(const gbdw_gauge* g, gbdw_field* out, const gbdw_field* in, int dag, const gbdw_field* cen, double M5,
           double mf, double khop, double* norm2, bool fetch, const DhopExtra* ex = nullptr);
// Schur operator on half p (or its adjoint); tq1, tq2 temporaries on half q
int mpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tq1, gbdw_field* tq2,
        const gbdw_field* in, double M5, double mf, int dag, double* norm2, bool fetch);
// out = Mpc^dag Mpc in, pap = |Mpc in|^2
int mpcdagmpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tp, gbdw_field* tq1,
              gbdw_field* tq2, const gbdw_field* in, double M5, double mf, double* pap);
// Mpc^dag Mpc with the CG update of its last pass fused in (see mdagm_residual): tp = Mpc in,
// s[0] = |tp|^2, s[1] = alpha = rr / s[0], r -= alpha Mpc^dag tp, s[2] = |r|^2 -> out[3].
// sink: any field of in's lattice and precision (written by nothing, named as the output).
int mpcdagmpc_residual(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* sink, gbdw_field* tp, gbdw_field* tq1,
                       gbdw_field* tq2, gbdw_field* r, const gbdw_field* in, double M5, double mf, double rr,
                       double out[3]);
// Mobius M^dag M on a full lattice (mobius.cu); t, tmp temporaries like in; pap = |M in|^2
int mobius_mdagm(const gbdw_gauge* g, gbdw_field* out, gbdw_field* t, gbdw_field* tmp, const gbdw_field* in,
                 double b, double c, double M5, double mf, double* pap);
// Mobius blocks (mobius.cu): Mooee / Mooee^-1 (inverse) on any lattice; the even-odd hopping
// block on half p; Mpc^dag Mpc on half p (tpa, tp on p; tq1, tq2 on q; pap = |Mpc in|^2)
int mobius_mooee_op(gbdw_field* out, const gbdw_field* in, double b, double c, double M5, double mf, int dag,
                    bool inverse);
int mobius_meooe_op(const gbdw_gauge* gp, gbdw_field* out, gbdw_field* tmp, const gbdw_field* in, double b, double c,
                    double mf, int dag);
int mobius_mpcdagmpc(const gbdw_gauge* gp, const gbdw_gauge* gq, gbdw_field* out, gbdw_field* tpa, gbdw_field* tp,
                     gbdw_field* tq1, gbdw_field* tq2, const gbdw_field* in, double b, double c, double M5, double mf,
                     double* pap);
int field_pick(gbdw_field* half, const gbdw_field* full);
int field_place(gbdw_field* full, const gbdw_field* half);
}  // namespace gbdw
