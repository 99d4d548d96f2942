/* bessel.h -- modified Bessel functions of integer order, the subset of the
 * reference's bessel.h (src/include/bessel.h) that the cylinder-plane geometry uses.
 * Same names and arguments as the reference (bessel.c:283-633): the logs of I_n(x) and
 * K_n(x) for x > 0, a negative order replaced by its modulus.  Edge values: log I_0(0) = 0
 * and log I_n(0) = -inf for n >= 2, as the reference; NaN for log I_1(x <= 0), for any
 * log I_n at x < 0 and for log K_n(x <= 0) (the reference's asymptotic branch, n >= 100,
 * gives +inf at x = 0).  Host functions (no GPU needed), own algorithms: trapezoidal
 * rules on integral representations and recurrences (caps_gb300/csrc/capc.cu). */
#ifndef CAPS_GB300_BESSEL_H
#define CAPS_GB300_BESSEL_H

#ifdef __cplusplus
extern "C" {
#endif

double bessel_logI0(double x);        /* bessel.c:283 */
double bessel_logI1(double x);        /* bessel.c:388 */
double bessel_logK0(double x);        /* bessel.c:336 */
double bessel_logK1(double x);        /* bessel.c:436 */
double bessel_logIn(int n, double x); /* bessel.c:583 */
double bessel_logKn(int n, double x); /* bessel.c:546 */

#ifdef __cplusplus
}
#endif

#endif
