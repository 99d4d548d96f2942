/* capc.h -- cylinder-plane geometry at T = 0, GPU-batched: the C form of the
 * reference's CasimirCP class (src/capc.cpp:20-154).  A cylinder of radius R at
 * separation d from a plane, both perfect reflectors; the scalar Dirichlet ('D') and
 * Neumann ('N') modes are computed separately (E_EM = E_D + E_N, capc.cpp:311-314).
 * Lengths in any unit (the reference uses metres); q in inverse units of R and d.
 * A DN or p that is not 'D'/'d' means Neumann, as in capc.cpp:51-53 and :131-133.
 * Contract violations (R <= 0, d <= 0, q <= 0, epsrel <= 0) abort with a message. */
#ifndef CAPS_GB300_CAPC_H
#define CAPS_GB300_CAPC_H

#include "libcaps.h"

#ifdef __cplusplus
extern "C" {
#endif

/* lmax = max(25, ceil(eta R/d)), the value capc's main() sets (capc.cpp:281-284) */
int caps_capc_lmax(double R, double d, double eta);

/* PFA energy per length of one scalar mode in units of hbar c, -pi^3/1920 sqrt(R/2d)/d^2
 * (capc.cpp:271); the electromagnetic PFA is twice this */
double caps_capc_pfa(double R, double d);

/* CasimirCP::logdet (capc.cpp:47-127): log(1 - M_00) + log det(1 - (U - V))
 * + log det(1 - (U + V + alpha v v^T)) at wave number q; dimension lmax
 * (lmax <= 0: the constructor's default max(25, (int)(5R/d)), capc.cpp:28).
 * detalg as kernel_logdet (matrix.c:57-149): DETALG_HODLR keeps the HODLR rules
 * (trace shortcut, |tr| > |logdet| check) with an exact dense factorisation; the
 * others the dense rules (trace and Mercator shortcuts). */
double caps_capc_logdet(double R, double d, int lmax, double q, char DN, detalg_t detalg);

/* the same for nq wave numbers in one GPU batch; returns the number of NaN results
 * (numerical failures) */
int caps_capc_logdet_batch(double R, double d, int lmax, const double *q, int nq, char DN, detalg_t detalg, double *out);

/* CasimirCP::energy at T = 0 (capc.cpp:129-153): E/(hbar c L_cyl) =
 * 1/(8 pi d) int_0^inf dx q logdet(q), q = x/(2d), by QUADPACK qagi with relative
 * tolerance epsrel; every node of a qagi step is one GPU batch.  neval and ier
 * (may be NULL) receive qagi's counters. */
double caps_capc_energy_T0(double R, double d, int lmax, char p, double epsrel, detalg_t detalg, int *neval, int *ier);

#ifdef __cplusplus
}
#endif

#endif
