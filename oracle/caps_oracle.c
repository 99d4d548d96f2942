/*
 * caps_oracle.c -- CPU restatement of the CaPS v0.5 round-trip-matrix log-det path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GPU library
 * and the timed CPU baseline ("port") of bench.py.  Nothing in the product path
 * links, loads or calls it.
 *
 * Every function follows the reference algorithm cited beside it (paths are
 * relative to the CaPS source tree).  The one deliberate difference is the
 * quadrature rule: the reference calls QUADPACK (dqags/dqage/dqagi, adaptive
 * Gauss-Kronrod with Wynn extrapolation) on the three intervals [1,a], [a,b],
 * [b,inf) chosen by K_estimate; here the same three intervals are integrated by
 * an adaptive Gauss-Legendre bisection to a tighter tolerance.  The reference
 * result is insensitive to the integration tolerance (logdetD moves by <=3e-16
 * relative when epsrel goes from 1e-8 to 1e-12), so this does not limit parity.
 *
 * Determinants follow the dense LU path of src/matrix.c (trace shortcut,
 * Mercator shortcut, LU with partial pivoting, Kahan sum of log|U_ii|).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "caps_oracle.h"

#define O_LOG2   0.69314718055994530942
#define O_C      299792458.0 /* speed of light, constants.h */
#define O_LOGPI  1.14472988584940017414
#define O_HALF_LOG_2PI 0.91893853320467274178
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static inline double sq(double x) { return x * x; }
static inline int sgn(double x) { return (x > 0) - (x < 0); }

static void die(const char *msg)
{
    fprintf(stderr, "caps_oracle: %s\n", msg);
    abort();
}

/* ------------------------------------------------------------------------- */
/* log n and log n!  (src/logfac.c:66597-66651)                               */
/* ------------------------------------------------------------------------- */
static double lfac_table[1024];
static pthread_once_t tables_once = PTHREAD_ONCE_INIT;

static void tables_init(void)
{
    for (int n = 0; n < 1024; n++)
        lfac_table[n] = lgamma(n + 1.0);
}

double oracle_logi(unsigned n) { return log((double)n); }

/* table below 1024, first-order Stirling above (src/logfac.c:66615-66628) */
double oracle_lfac(unsigned n)
{
    pthread_once(&tables_once, tables_init);
    if (n < 1024)
        return lfac_table[n];
    const double dn = (double)n;
    return (dn + 0.5) * log(dn) - dn + O_HALF_LOG_2PI + (1. / 12) / dn;
}

/* ------------------------------------------------------------------------- */
/* helpers (src/misc.c)                                                       */
/* ------------------------------------------------------------------------- */
static double sqrtpm1(double x) { return x / (sqrt(1 + x) + 1); } /* misc.c:56 */

static double logadd(double a, double b) /* misc.c:70 */
{
    if (isinf(a) && a < 0) return b;
    if (isinf(b) && b < 0) return a;
    if (a > b) return a + log1p(exp(b - a));
    return b + log1p(exp(a - b));
}

static double kahan(const double *v, size_t n) /* misc.c:26 */
{
    double s = 0, c = 0;
    for (size_t i = 0; i < n; i++) {
        double y = v[i] - c;
        double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    return s;
}

typedef struct { double v; int s; } lv_t; /* log|x| and sign of x */

static double logadd_signed(const lv_t *t, int n, int *sign) /* misc.c:95 */
{
    double mx = t[0].v;
    for (int i = 1; i < n; i++) if (t[i].v > mx) mx = t[i].v;
    double s = 0;
    for (int i = 0; i < n; i++) s += t[i].s * exp(t[i].v - mx);
    *sign = sgn(s);
    return mx + log(fabs(s));
}

/* ------------------------------------------------------------------------- */
/* modified Bessel functions (src/bessel.c:635-833)                           */
/* ------------------------------------------------------------------------- */

/* I_nu(x)/I_{nu+1}(x) from the continued fraction DLMF 10.33.1,
 * 2(nu+1)/x + 1/(2(nu+2)/x + 1/(2(nu+3)/x + ...)), modified Lentz evaluation.
 * Follows bessel_ratioI (bessel.c:635). */
double oracle_ratioI(double nu, double x)
{
    const double tiny = 1e-300;
    const double t = 2 / x;
    double f = (nu + 1) * t, C = f, D = 0;
    for (int k = 2; k < 100000; k++) {
        const double b = (nu + k) * t;
        D = b + D; D = (D == 0) ? tiny : D; D = 1 / D;
        C = b + 1 / C; C = (C == 0) ? tiny : C;
        const double delta = C * D;
        f *= delta;
        if (fabs(delta - 1) < 1e-17) break;
    }
    return f;
}

/* Debye polynomials U_k(p) of the uniform expansion DLMF 10.41.10, written as
 * polynomials in p^2 after taking out p^k. */
static void debye_u(double p2, double U[6])
{
    U[0] = 1;
    U[1] = (3 - 5 * p2) / 24;
    U[2] = (81 + p2 * (-462 + 385 * p2)) / 1152;
    U[3] = (30375 + p2 * (-369603 + p2 * (765765 - 425425 * p2))) / 414720;
    U[4] = (4465125 + p2 * (-94121676 + p2 * (349922430 + p2 * (-446185740 + 185910725 * p2)))) / 39813120;
    U[5] = (1519035525. + p2 * (-49286948607. + p2 * (284499769554. + p2 * (-614135872350. + p2 * (566098157625. - 188699385875. * p2))))) / 6688604160.;
}

/* log I_nu(x), uniform asymptotic expansion DLMF 10.41.3 (bessel.c:673) */
double oracle_logI_asymp(double nu, double x)
{
    const double z = x / nu, a = sqrt(1 + z * z), p2 = 1 / (1 + z * z);
    double U[6]; debye_u(p2, U);
    const double y = 1 / (nu * a);
    const double s = log1p(y * (U[1] + y * (U[2] + y * (U[3] + y * (U[4] + y * U[5])))));
    const double eta = a + log(z / (1 + a));
    return nu * eta - 0.5 * log(2 * M_PI * nu * a) + s;
}

/* log K_nu(x), uniform asymptotic expansion DLMF 10.41.4 (bessel.c:706) */
double oracle_logK_asymp(double nu, double x)
{
    const double z = x / nu, a = sqrt(1 + z * z), p2 = 1 / (1 + z * z);
    double U[6]; debye_u(p2, U);
    const double y = -1 / (nu * a);
    const double s = log1p(y * (U[1] + y * (U[2] + y * (U[3] + y * (U[4] + y * U[5])))));
    const double eta = a + log(z / (1 + a));
    return -nu * eta - 0.5 * log(a) + 0.5 * log(0.5 * M_PI / nu) + s;
}

/* log I_{n+1/2}(x), log K_{n+1/2}(x) (bessel.c:781): K by upward recurrence
 * K_{l+1/2} = (2l-1)/x K_{l-1/2} + K_{l-3/2} with 1e100 rescaling for n<100,
 * uniform asymptotics for n>=100; I from the Wronskian with the ratio I. */
void oracle_logIK_half(int n, double x, double *logI, double *logK)
{
    const double logx = log(x), invx = 1 / x;
    double lk, lkp;
    if (n >= 100) {
        lkp = oracle_logK_asymp(n + 1.5, x);
        lk  = oracle_logK_asymp(n + 0.5, x);
    } else {
        double k0 = 1, k1 = 1 + invx;
        double pre = -x + 0.5 * (log(M_PI / 2) - logx);
        for (int l = 2; l <= n + 1; l++) {
            double kn = (2 * l - 1) * k1 * invx + k0;
            k0 = k1; k1 = kn;
            if (k0 > 1e100) { k0 *= 1e-100; k1 *= 1e-100; pre += log(1e100); }
        }
        lk = pre + log(k0);
        lkp = pre + log(k1);
    }
    if (logK) *logK = lk;
    if (logI) {
        if (n >= 100) *logI = oracle_logI_asymp(n + 0.5, x);
        else *logI = -logx - lkp - log1p(exp(lk - lkp - log(oracle_ratioI(n + 0.5, x))));
    }
}

/* log I_n(x) for integer 0<=n<=12 and moderate x by its power series
 * (used only by the small-argument Legendre expansion below). */
static double bessel_In_series(int n, double x)
{
    const double y = 0.25 * x * x;
    double term = 1, sum = 1;
    for (int k = 1; k < 400; k++) {
        term *= y / (k * (double)(k + n));
        sum += term;
        if (term < 1e-17 * sum) break;
    }
    return exp(n * log(0.5 * x) - lgamma(n + 1.0)) * sum;
}

/* ------------------------------------------------------------------------- */
/* Mie coefficients (src/libcaps.c:485-602)                                   */
/* ------------------------------------------------------------------------- */
void oracle_mie(double LbyR, double xi_, int l, double epsm1, double *lna, double *lnb)
{
    const double chi = xi_ / (1 + LbyR);
    const double ln_chi = log(xi_) - log1p(LbyR);
    double lIp, lKp, lIm, lKm;
    oracle_logIK_half(l, chi, &lIp, &lKp);
    oracle_logIK_half(l - 1, chi, &lIm, &lKm);
    const double ratio = oracle_ratioI(l - 0.5, chi);

    if (isinf(epsm1)) { /* perfect reflector, libcaps.c:485 */
        *lnb = O_LOGPI - O_LOG2 + lIp - lKp;
        const double num = O_LOGPI - O_LOG2 + lIp + log(chi * ratio - l);
        const double den = logadd(log((double)l) + lKp, ln_chi + lKm);
        *lna = num - den;
        return;
    }
    /* Drude-type metal, libcaps.c:557 */
    const double ln_n = log1p(epsm1) / 2, n = exp(ln_n), ln_l = log((double)l);
    double lIp_n, lKp_n, lIm_n, lKm_n;
    oracle_logIK_half(l, n * chi, &lIp_n, &lKp_n);
    oracle_logIK_half(l - 1, n * chi, &lIm_n, &lKm_n);
    const double ratio_n = oracle_ratioI(l - 0.5, n * chi);

    const double ln_gB = lIp_n + lIp + ln_chi + log(n * ratio_n - ratio);
    const double ln_gC = log(epsm1) + lIp_n + logadd(ln_chi + lKm, ln_l + lKp);
    const double ln_gD = ln_chi + logadd(lIp_n + lKm, ln_n + lKp + lIm_n);
    const double num = lIp_n + lIp + log(-l * epsm1 + n * chi * (n * ratio - ratio_n));
    *lnb = O_LOGPI - O_LOG2 + ln_gB - ln_gD;
    *lna = O_LOGPI - O_LOG2 + num - logadd(ln_gC, ln_gD);
}

/* Fresnel coefficients (src/libcaps.c:616) */
static void fresnel(double epsm1, double xi_, double k_, double *rTE, double *rTM)
{
    if (isinf(epsm1)) { *rTM = 1; *rTE = -1; return; }
    const double x = sq(xi_) / (sq(xi_) + sq(k_)) * epsm1;
    const double bm1 = sqrtpm1(x);
    *rTE = -bm1 / (2 + bm1);
    *rTM = (epsm1 - bm1) / (epsm1 + 2 + bm1);
}

/* log Lambda_{l1 l2}^{(m)} (src/libcaps.c:45) */
double oracle_lnLambda(int l1, int l2, int m)
{
    return (log(2. * l1 + 1) + log(2. * l2 + 1) - log((double)l1) - log(l1 + 1.) - log((double)l2) - log(l2 + 1.)
            + oracle_lfac(l1 - m) + oracle_lfac(l2 - m) - oracle_lfac(l1 + m) - oracle_lfac(l2 + m)) / 2;
}

/* lmin for given m (src/libcaps.c:63) */
int oracle_lmin(double LbyR, int ldim, int m)
{
    if (m == 0) return 1;
    const int l = (int)round(m / sqrt(2 * LbyR));
    int lmin = l - ldim / 2;
    return lmin < m ? m : lmin;
}

/* ------------------------------------------------------------------------- */
/* Legendre functions for x > 1 (src/plm.c)                                   */
/* ------------------------------------------------------------------------- */

/* log P_l(x), recurrence (plm.c:252) */
static double lnPl_rec(int l, double x)
{
    if (l == 0) return 0;
    if (l == 1) return log(x);
    double pre = 0, v0 = 1, v1 = x;
    for (int n = 1; n < l; n++) {
        double v = ((2 * n + 1) * x * v1 - n * v0) / (n + 1);
        v0 = v1; v1 = v;
        if (v > 1e100) { pre += log(1e100); v0 *= 1e-100; v1 *= 1e-100; }
    }
    return pre + log(v1);
}

/* log P_l(x), large-argument expansion of Bogaert, Michiels & Fostier,
 * SIAM J. Sci. Comput. 34 (2012), sec. 3.2 (plm.c:133).  The prefactor
 * Gamma(l+1)/Gamma(l+3/2) uses its asymptotic series in 1/l. */
static double lnPl_large(int l, double x, double sh)
{
    const int M = 17;
    const double xi = acosh(x), ex = x + sh;
    const double k = 1. / l;
    double C = (1 + k * (-3. / 8 + k * (25. / 128 + k * (-105. / 1024 + k * (1659. / 32768 + k * (-6237. / 262144 + k * 50765. / 4194304)))))) / sqrt((double)l);
    double sum = 0, shm = 1, exm = 1;
    for (int m = 0; m < M; m++) {
        sum += C * (exm + exp(-(m + 2 * l + 1) * xi)) / shm;
        shm *= sh; exm *= ex;
        C *= sq(m + 0.5) / ((2 * m + 2) * (l + 1.5 + m));
    }
    return -(O_LOG2 + O_LOGPI) / 2 - log(sh) / 2 + log(sum) + (l + 0.5) * xi;
}

/* log P_l(x), small-argument Bessel expansion of the same paper, sec. 3.3,
 * coefficient functions f_n of eqs. (3.27)-(3.31) (plm.c:169-235). */
static double lnPl_small(int l, double x)
{
    const double v = l + 0.5, xi = acosh(x), y = xi * v;
    double h[13], yn = 1;
    for (int n = 0; n < 13; n++) { h[n] = yn * bessel_In_series(n, y); yn *= -y; }
    const double f0 = h[0];
    const double f2 = 1. / 8 * h[1] - 1. / 12 * h[2];
    const double f4 = 11. / 384 * h[2] - 7. / 160 * h[3] + 1. / 160 * h[4];
    const double f6 = 173. / 15360 * h[3] - 101. / 3584 * h[4] + 671. / 80640 * h[5] - 61. / 120960 * h[6];
    const double f8 = 22931. / 3440640 * h[4] - 90497. / 3870720 * h[5] + 217. / 20480 * h[6] - 1261. / 967680 * h[7] + 1261. / 29030400 * h[8];
    const double f10 = 1319183. / 247726080 * h[5] - 10918993. / 454164480 * h[6] + 1676287. / 113541120 * h[7] - 7034857. / 2554675200 * h[8] + 1501. / 8110080 * h[9] - 79. / 20275200 * h[10];
    const double f12 = 233526463. / 43599790080 * h[6] - 1396004969. / 47233105920 * h[7] + 2323237523. / 101213798400 * h[8] - 72836747. / 12651724800 * h[9] + 3135577. / 5367398400 * h[10] - 1532789. / 61993451520 * h[11] + 66643. / 185980354560 * h[12];
    const double v2 = v * v;
    const double s = f0 + (f2 + (f4 + (f6 + (f8 + (f10 + f12 / v2) / v2) / v2) / v2) / v2) / v2;
    return log(s);
}

/* log P_l(x) (plm.c:299) */
double oracle_lnPl(int l, double x)
{
    if (l < 100) return lnPl_rec(l, x);
    const double sh = sqrt((x + 1) * (x - 1));
    return ((l + 1) * sh > 25) ? lnPl_large(l, x, sh) : lnPl_small(l, x);
}

/* log P_l^m(x), upward recurrence in l from P_m^m (plm.c:72) */
static double lnPlm_up(int l, int m, double x)
{
    double pre = oracle_lfac(2 * m) - m * O_LOG2 - oracle_lfac(m) + m / 2. * log((x + 1) * (x - 1));
    if (l == m) return pre;
    double a0 = 1, a1 = x * (2 * m + 1);
    if (a1 == 0) return -INFINITY;
    for (int ll = 2; ll < l + 1 - m; ll++) {
        const double k = (2. * m - 1.) / ll;
        double a2 = (2 + k) * x * a1 - (1 + k) * a0;
        a0 = a1; a1 = a2;
        const double e = fabs(a1);
        if (e < 1e-100) { pre -= log(1e100); a1 *= 1e100; a0 *= 1e100; }
        else if (e > 1e100) { pre += log(1e100); a1 *= 1e-100; a0 *= 1e-100; }
    }
    return pre + log(fabs(a1));
}

/* P_l^{m-1}(x)/P_l^m(x) from the continued fraction DLMF 14.14.1; the fraction
 * terminates at j=l+1.  Modified Lentz evaluation (plm.c:328). */
double oracle_Plm_cf(long l, long m, double x)
{
    const double tiny = 1e-300;
    const double al = (1 - 1 / (x * x)) / 4;
    const double a0 = x * (l - m + 1) * (double)(l + m) * al;
    double f = (double)m; if (f == 0) f = tiny;
    double C = f, D = 0;
    for (long j = m + 1; j <= l + 1; j++) {
        const double aj = (double)(l + 1 - j) * (double)(l + j) * al;
        if (aj == 0) break;
        D = j + aj * D; if (D == 0) D = tiny; D = 1 / D;
        C = j + aj / C; if (C == 0) C = tiny;
        const double d = C * D;
        f *= d;
        if (fabs(d - 1) < 1e-17) break;
    }
    return x * sqrt(1 - 1 / (x * x)) * f / (2 * a0);
}

/* log P_l^m(x), continued fraction + downward recurrence in m (plm.c:391) */
static double lnPlm_down(int l, int m, double x)
{
    double pre = oracle_lnPl(l, x);
    if (m == 0) return pre;
    const double c = 2 * x / sqrt((x - 1) * (x + 1));
    double vp = 1, vm = oracle_Plm_cf(l, m, x);
    for (int mm = m - 2; mm >= 0; mm--) {
        double v = (vp + (mm + 1) * vm * c) / ((l + 1. + mm) * (l - mm));
        vp = vm; vm = v;
        if (vm < 1e-100) { vm *= 1e100; vp *= 1e100; pre += log(1e100); }
    }
    return pre - log(fabs(vm));
}

/* log P_l^m(x) for x>1, no Condon-Shortley phase (plm.c:47) */
double oracle_lnPlm(int l, int m, double x)
{
    if (m == 0) return oracle_lnPl(l, x);
    if (l - m <= 200) return lnPlm_up(l, m, x);
    return lnPlm_down(l, m, x);
}

/* first and second logarithmic derivative of P_l^m (plm.c:436) */
static double dlnPlm(int l, int m, double x, double *d2)
{
    double p = 0, q = 0;
    const double c2 = (x + 1) * (x - 1), c = sqrt(c2);
    if (m + 1 <= l) p = 1 / oracle_Plm_cf(l, m + 1, x);
    const double df = p / c + m * x / c2;
    if (d2) {
        if (m + 2 <= l) q = p / oracle_Plm_cf(l, m + 2, x);
        *d2 = (q - p * p - m * (x * x + 1) / c2) / c2;
    }
    return df;
}

/* ------------------------------------------------------------------------- */
/* K integrals (src/integration.c:42-489)                                     */
/* ------------------------------------------------------------------------- */
typedef struct {
    int nu, m, p; /* p: 0 TE, 1 TM */
    double alpha, factor, lognorm, epsm1;
} kargs_t;

/* -log of the integrand peak shape used by K_estimate (integration.c:42) */
static double k_f(double x, int nu, int m, double alpha)
{
    if (x <= 1) die("k_f: x<=1");
    if (m == 0) return alpha * x - oracle_lnPlm(nu, 2, x);
    return alpha * x - oracle_lnPlm(nu, 2 * m, x) + log(x * x - 1);
}

/* peak position, Laplace estimate and borders a,b (integration.c:104) */
static double k_estimate(int nu, int m, double alpha, double eps, double *a, double *b, double *approx)
{
    const int maxiter = 75, mpos = m > 0, m_ = m > 1 ? m : 1;
    double fxmax, fp = 0, fpp = 0, xmax;
    int i;

    if (m == 1) {
        const double thr = (nu - 2.) * (nu + 3.) / (6 * alpha);
        if (thr < 2) {
            *a = 1;
            *b = 1 - log(eps) / alpha;
            double lk;
            oracle_logIK_half(nu, alpha, NULL, &lk);
            const double lt1 = 1.5 * log(alpha) + log(2 / M_PI) / 2 + lk;
            const double lt2 = -alpha + log(alpha + nu * (nu + 1) / 2.);
            const double arg = -exp(lt2 - lt1);
            fxmax = alpha - log((nu - 1.) * nu * (nu + 1.) * (nu + 2) / 8.);
            xmax = 1;
            *approx = (fabs(arg) < 1) ? lt1 + log1p(arg) : -fxmax;
            goto bordercheck;
        }
    }

    if (nu == 2 * m) {
        const double r = (nu / 2 - 1) / alpha;
        xmax = r + sqrt(1 + r * r);
    } else
        xmax = sqrt(1 + sq((nu + 0.5) / alpha));

    for (i = 0; i < maxiter; i++) {
        const double xold = xmax, x2m1 = xmax * xmax - 1;
        double d2, d = dlnPlm(nu, 2 * m_, xmax, &d2);
        fp = alpha - d + mpos * 2 * xmax / x2m1;
        fpp = -d2 - mpos * 2 * (xmax * xmax + 1) / sq(x2m1);
        xmax = xmax - fp / fpp;
        if (xmax <= 1) xmax = 1 + (xold - 1) / 2;
        const double delta = fabs(xmax - xold);
        if (delta < 1e-13 || (xmax > 1.001 && delta < 1e-6)) break;
    }
    if (!isfinite(xmax)) die("k_estimate: xmax");
    fxmax = k_f(xmax, nu, m, alpha);
    if (!isfinite(fxmax) || !isfinite(fpp) || fpp < 0) die("k_estimate: fxmax/fpp");
    *approx = log(2 * M_PI / fpp) / 2 - fxmax;
    {
        const double width = -log(eps) / sqrt(fpp);
        *a = fmax(1, xmax - width);
        *b = xmax + width;
    }

bordercheck:
    if (*a > 1) {
        for (i = 0; i < maxiter; i++) {
            if (exp(fxmax - k_f(*a, nu, m, alpha)) < eps) break;
            *a = 1 + 0.5 * (*a - 1);
        }
        if (i == maxiter) die("k_estimate: left border");
    }
    for (i = 0; i < maxiter; i++) {
        if (exp(fxmax - k_f(*b, nu, m, alpha)) < eps) break;
        *b = 1 + 2 * (*b - 1);
    }
    if (i == maxiter) die("k_estimate: right border");
    return xmax;
}

/* integrand r_p e^{-alpha x} P_nu^{2m}(x)/(x^2-1) (or P_nu^2 e^{-alpha x} for m=0),
 * scaled by exp(-lognorm) (integration.c:257) */
static double k_integrand(double x, const kargs_t *g)
{
    x *= g->factor;
    const double x2m1 = (x + 1) * (x - 1);
    double v;
    if (g->m) v = exp(-g->lognorm + oracle_lnPlm(g->nu, 2 * g->m, x) - g->alpha * x - log(x2m1));
    else      v = exp(-g->lognorm + oracle_lnPlm(g->nu, 2, x) - g->alpha * x);
    const double xt = g->alpha / 2;
    double rTE, rTM;
    fresnel(g->epsm1, xt, xt * sqrt(x2m1), &rTE, &rTM);
    if (!isfinite(v)) die("k_integrand: non-finite");
    return g->p ? rTM * v : rTE * v;
}

/* Gauss-Legendre nodes/weights on [-1,1] by Newton iteration on P_n */
#define GLN 15
static double gl_x[GLN], gl_w[GLN];
static pthread_once_t gl_once = PTHREAD_ONCE_INIT;
static void gl_init(void)
{
    const int n = GLN;
    for (int i = 0; i < n; i++) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; j++) { double p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
            pp = n * (z * p1 - p2) / (z * z - 1);
            double z1 = z; z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-16) break;
        }
        gl_x[i] = z; gl_w[i] = 2 / ((1 - z * z) * pp * pp);
    }
}

static double gl_panel(const kargs_t *g, double a, double b, long *nev)
{
    const double h = (b - a) / 2, c = (a + b) / 2;
    double s = 0;
    for (int i = 0; i < GLN; i++) s += gl_w[i] * k_integrand(c + h * gl_x[i], g);
    *nev += GLN;
    return s * h;
}

static double gl_adapt(const kargs_t *g, double a, double b, double whole, double tol, int depth, long *nev)
{
    const double mid = (a + b) / 2;
    const double l = gl_panel(g, a, mid, nev), r = gl_panel(g, mid, b, nev);
    if (fabs(l + r - whole) <= tol || depth >= 40) return l + r;
    return gl_adapt(g, a, mid, l, tol / 1.4142135623730951, depth + 1, nev)
         + gl_adapt(g, mid, b, r, tol / 1.4142135623730951, depth + 1, nev);
}

static double gl_integrate(const kargs_t *g, double a, double b, double tol_rel, double tol_abs, long *nev)
{
    pthread_once(&gl_once, gl_init);
    const double w = gl_panel(g, a, b, nev);
    const double tol = fmax(tol_abs, tol_rel * fabs(w));
    return gl_adapt(g, a, b, w, tol, 0, nev);
}

#define K_EPSREL 1e-13

/* log|K_{nu,p}^{(m)}(alpha)| and its sign (integration.c:288) */
static double integrate_K(int nu, int m, int p, double alpha, double epsm1, int *sign, long *nev)
{
    double a, b, lognorm;
    k_estimate(nu, m, alpha, 1e-6, &a, &b, &lognorm);
    if (a < 1.0001) a = 1;
    kargs_t g = { nu, m, p, alpha, 1.0, lognorm, epsm1 };

    const double I2 = gl_integrate(&g, a, b, K_EPSREL, 0, nev);
    double I1 = 0, I3 = 0;
    if (a > 1) {
        const double fa = k_integrand(a, &g);
        if ((a - 1) * fa > I2 * K_EPSREL) /* same neglect test as the reference with our tolerance */
            I1 = gl_integrate(&g, 1, a, K_EPSREL, 1e-3 * K_EPSREL * fabs(I2), nev);
    }
    /* [b, inf): geometric panels until the remainder is negligible */
    {
        double lo = b, w = fmax(b - a, 1 / alpha);
        for (int k = 0; k < 200; k++) {
            const double piece = gl_integrate(&g, lo, lo + w, K_EPSREL, 1e-3 * K_EPSREL * fabs(I2), nev);
            I3 += piece;
            if (fabs(piece) < 1e-20 * fabs(I2 + I3)) break;
            lo += w; w *= 2;
        }
    }
    const double sum = I1 + I2 + I3;
    if (!(sum != 0) || !isfinite(sum)) die("integrate_K: bad sum");
    *sign = sgn(sum);
    return log(fabs(sum)) + lognorm;
}

/* ------------------------------------------------------------------------- */
/* per-(xi,m) evaluation context with K and I caches                          */
/* ------------------------------------------------------------------------- */
typedef struct {
    double LbyR, xi_, alpha, epsm1_plate, epsm1_sphere;
    int m, ldim, lmin, is_pr;
    int nK; double *K[2]; /* log|K| by nu-2m_ ... indexed nu */
    int nI; double *I[2]; int8_t *Is[2]; /* log|I| table over (l1,l2), l in [0, lmax+2] */
    int lmaxI;
    double *al, *bl;
    long nev;
} ctx_t;

static double ctx_K(ctx_t *c, int nu, int p, int *sign)
{
    if (nu >= c->nK) die("ctx_K: nu out of range");
    *sign = p ? 1 : -1;
    if (isnan(c->K[p][nu])) {
        int s;
        c->K[p][nu] = integrate_K(nu, c->m, p, c->alpha, c->epsm1_plate, &s, &c->nev);
        if (s != *sign) die("ctx_K: unexpected sign");
    }
    return c->K[p][nu];
}

static double falpha(double p, double n, double nu) /* integration.c:492 */
{
    return ((sq(p) - sq(n + nu + 1)) * (sq(p) - sq(n - nu))) / (4 * sq(p) - 1);
}

/* log|I_{l1 l2,p}^{(m)}| via the q-sum of K integrals (integration.c:497) */
static double integrate_I_raw(ctx_t *c, int l1, int l2, int pp, int *sign)
{
    const int m_ = c->m > 0 ? c->m : 1;
    const double n = l1, nu = l2, m = m_;
    const double n4 = l1 + l2 - 2 * m_;
    const int l12 = l1 + l2;
    const int qmax = (int)fmin(fmin(n, nu), (l12 - 2 * m_) / 2);
    if (qmax < 0) die("integrate_I: qmax<0");
    const double Ap = -2 * m * (n - nu) * (n + nu + 1);
    const double log_a0 = oracle_lfac(2 * l1) - oracle_lfac(l1) + oracle_lfac(2 * l2) - oracle_lfac(l2) + oracle_lfac(l1 + l2)
                        - oracle_lfac(2 * l12) + oracle_lfac(l12 - 2 * m_) - oracle_lfac(l1 - m_) - oracle_lfac(l2 - m_);
    double *aq = malloc((qmax + 1) * sizeof(double));
    lv_t *t = malloc((qmax + 1) * sizeof(lv_t));
    int s, q = 0;
    aq[0] = 1;
    t[0].v = ctx_K(c, l12, pp, &s); t[0].s = s;
    if (qmax == 0) goto done;
    q = 1;
    aq[1] = (n + nu - 1.5) * (1 - (2 * n + 2 * nu - 1) / (n4 * (n4 - 1)) * ((m - n) * (m - n + 1) / (2 * n - 1) + (m - nu) * (m - nu + 1) / (2 * nu - 1)));
    t[1].v = ctx_K(c, l12 - 2, pp, &s) + log(fabs(aq[1])); t[1].s = sgn(aq[1]) * s;
    if (qmax == 1) goto done;
    q = 2;
    aq[2] = (2 * n + 2 * nu - 1) * (2 * n + 2 * nu - 7) / 4 * ((2 * n + 2 * nu - 3) / (n4 * (n4 - 1)) * ((2 * n + 2 * nu - 5) / (2 * (n4 - 2) * (n4 - 3))
              * ((m - n) * (m - n + 1) * (m - n + 2) * (m - n + 3) / (2 * n - 1) / (2 * n - 3)
              + 2 * (m - n) * (m - n + 1) * (m - nu) * (m - nu + 1) / ((2 * n - 1) * (2 * nu - 1))
              + (m - nu) * (m - nu + 1) * (m - nu + 2) * (m - nu + 3) / (2 * nu - 1) / (2 * nu - 3)) - (m - n) * (m - n + 1) / (2 * n - 1)
              - (m - nu) * (m - nu + 1) / (2 * nu - 1)) + 0.5);
    t[2].v = ctx_K(c, l12 - 4, pp, &s) + log(fabs(aq[2])); t[2].s = sgn(aq[2]) * s;
    if (qmax == 2) goto done;
    {
        double lscale = 0; int count = 0;
        for (q = 3; q <= qmax; q++) {
            const double p = n + nu - 2 * q, p1 = p - 2 * m, p2 = p + 2 * m;
            if (Ap != 0) {
                const double c0 = (p + 2) * (p + 3) * (p1 + 1) * (p1 + 2) * Ap * falpha(p + 1, n, nu);
                const double c1 = Ap * (Ap * Ap + (p + 1) * (p + 3) * (p1 + 2) * (p2 + 2) * falpha(p + 2, n, nu)
                                             + (p + 2) * (p + 4) * (p1 + 3) * (p2 + 3) * falpha(p + 3, n, nu));
                const double c2 = -(p + 2) * (p + 3) * (p2 + 3) * (p2 + 4) * Ap * falpha(p + 4, n, nu);
                aq[q] = (c1 * aq[q - 1] + c2 * aq[q - 2]) / c0;
            } else
                aq[q] = (p + 1) * (p2 + 2) * falpha(p + 2, n, nu) * aq[q - 1] / ((p + 2) * (p1 + 1) * falpha(p + 1, n, nu));
            if (fabs(aq[q]) > 1e100) {
                lscale += log(fabs(aq[q])); aq[q - 1] /= fabs(aq[q]); aq[q] = sgn(aq[q]);
            } else if (fabs(aq[q]) < 1e-100 && fabs(aq[q]) > 0) {
                lscale -= log(fabs(aq[q])); aq[q - 1] *= fabs(aq[q]); aq[q] = sgn(aq[q]);
            }
            t[q].v = lscale + ctx_K(c, l12 - 2 * q, pp, &s) + log(fabs(aq[q]));
            t[q].s = sgn(aq[q]) * s;
            if (t[q].v - t[0].v < -60) { if (++count >= 3) break; }
            else count = 0;
        }
    }
done:;
    const int nt = (q < qmax ? q : qmax) + 1;
    double r = log_a0 + logadd_signed(t, nt, sign);
    free(aq); free(t);
    if (!isfinite(r)) die("integrate_I: non-finite");
    return r;
}

/* I with the symmetry, PR and l<m rules (integration.c:627) */
static double ctx_I(ctx_t *c, int l1, int l2, int p, int *sign)
{
    if (l1 < c->m || l2 < c->m) { *sign = 0; return -INFINITY; }
    if (c->is_pr && p == 0) { double v = ctx_I(c, l1, l2, 1, sign); *sign = -1; return v; }
    if (l1 < l2) { int tmp = l1; l1 = l2; l2 = tmp; }
    if (l1 > c->lmaxI) die("ctx_I: l out of range");
    const size_t idx = (size_t)l1 * (c->lmaxI + 1) + l2;
    if (isnan(c->I[p][idx])) {
        int s;
        c->I[p][idx] = integrate_I_raw(c, l1, l2, p, &s);
        c->Is[p][idx] = (int8_t)s;
    }
    *sign = c->Is[p][idx];
    return c->I[p][idx];
}

static double int_A(ctx_t *c, int l1, int l2, int p, int *sign) /* integration.c:762 */
{
    if (c->m == 0) { *sign = 0; return -INFINITY; }
    return 2 * log((double)c->m) + ctx_I(c, l1, l2, p, sign);
}

static double int_B(ctx_t *c, int l1, int l2, int p, int *sign) /* integration.c:794 */
{
    const int m = c->m;
    if (m == 0) return ctx_I(c, l1, l2, p, sign);
    int s1, s2, s3, s4;
    const double I1 = ctx_I(c, l1 - 1, l2 - 1, p, &s1), I2 = ctx_I(c, l1 + 1, l2 - 1, p, &s2);
    const double I3 = ctx_I(c, l1 - 1, l2 + 1, p, &s3), I4 = ctx_I(c, l1 + 1, l2 + 1, p, &s4);
    const double den = (2 * l1 + 1.) * (2 * l2 + 1.);
    const double mx = fmax(fmax(I1, I2), fmax(I3, I4));
    double I = (l1 + 1.) * (l1 + m) * (l2 + 1.) * (l2 + m) / den * s1 * exp(I1 - mx);
    I -= l1 * (l1 - m + 1.) * (l2 + 1.) * (l2 + m) / den * s2 * exp(I2 - mx);
    I -= (l1 + 1.) * (l1 + m) * l2 * (l2 - m + 1.) / den * s3 * exp(I3 - mx);
    I += l1 * (l1 - m + 1.) * l2 * (l2 - m + 1.) / den * s4 * exp(I4 - mx);
    *sign = sgn(I);
    return mx + log(fabs(I));
}

static double int_C(ctx_t *c, int l1, int l2, int p, int *sign) /* integration.c:842 */
{
    const int m = c->m;
    if (m == 0) { *sign = 0; return -INFINITY; }
    int s1, s2;
    const double I1 = ctx_I(c, l1, l2 - 1, p, &s1), I2 = ctx_I(c, l1, l2 + 1, p, &s2);
    const double den = 2 * l2 + 1;
    double I = -(l2 + 1.) * (l2 + m) / den * s1 * exp(I1 - I2);
    I += l2 * (l2 - m + 1.) / den * s2;
    *sign = sgn(I);
    return log((double)m) + I2 + log(fabs(I));
}

static double int_D(ctx_t *c, int l1, int l2, int p, int *sign) { return int_C(c, l2, l1, p, sign); }

static void ctx_init(ctx_t *c, const oracle_geom_t *g, double xi_, int m)
{
    memset(c, 0, sizeof(*c));
    c->LbyR = g->L / g->R;
    c->xi_ = xi_; c->alpha = 2 * xi_; c->m = m; c->ldim = g->ldim;
    c->lmin = oracle_lmin(c->LbyR, g->ldim, m);
    const double xi = xi_ * 299792458. / (g->L + g->R);
    c->epsm1_plate = oracle_epsm1(&g->plate, xi);
    c->epsm1_sphere = oracle_epsm1(&g->sphere, xi);
    c->is_pr = g->plate.kind == ORACLE_PERFECT;
    c->lmaxI = c->lmin + g->ldim + 1;
    c->nK = 2 * (c->lmaxI + 2) + 4;
    for (int p = 0; p < 2; p++) {
        c->K[p] = malloc(c->nK * sizeof(double));
        for (int i = 0; i < c->nK; i++) c->K[p][i] = NAN;
        const size_t ni = (size_t)(c->lmaxI + 1) * (c->lmaxI + 1);
        c->I[p] = malloc(ni * sizeof(double));
        c->Is[p] = calloc(ni, 1);
        for (size_t i = 0; i < ni; i++) c->I[p][i] = NAN;
    }
    c->al = malloc(g->ldim * sizeof(double));
    c->bl = malloc(g->ldim * sizeof(double));
    for (int j = 0; j < g->ldim; j++) c->al[j] = c->bl[j] = NAN;
}

static void ctx_free(ctx_t *c)
{
    for (int p = 0; p < 2; p++) { free(c->K[p]); free(c->I[p]); free(c->Is[p]); }
    free(c->al); free(c->bl);
}

/* matrix element M_{l1 l2}^{(m)}(p1,p2) (libcaps.c:761) */
static double M_elem(ctx_t *c, int l1, int l2, char p1, char p2)
{
    const int lmin = c->lmin;
    if (isnan(c->al[l1 - lmin])) oracle_mie(c->LbyR, c->xi_, l1, c->epsm1_sphere, &c->al[l1 - lmin], &c->bl[l1 - lmin]);
    if (isnan(c->al[l2 - lmin])) oracle_mie(c->LbyR, c->xi_, l2, c->epsm1_sphere, &c->al[l2 - lmin], &c->bl[l2 - lmin]);
    const double lL = oracle_lnLambda(l1, l2, c->m);
    const double al1 = c->al[l1 - lmin], bl1 = c->bl[l1 - lmin], al2 = c->al[l2 - lmin], bl2 = c->bl[l2 - lmin];
    int sA, sB, sC, sD;
    if (p1 == p2) {
        if (p1 == 'E') {
            const double lA = int_A(c, l1, l2, 0, &sA), lB = int_B(c, l1, l2, 1, &sB);
            const double mie = (al1 + al2) / 2;
            return exp(lB + mie + lL) * sB - exp(lA + mie + lL) * sA;
        }
        const double lA = int_A(c, l1, l2, 1, &sA), lB = int_B(c, l1, l2, 0, &sB);
        const double mie = (bl1 + bl2) / 2;
        return exp(lA + mie + lL) * sA - exp(lB + mie + lL) * sB;
    }
    if (c->m == 0) return 0;
    if (p1 == 'E') {
        const double lC = int_C(c, l1, l2, 0, &sC), lD = int_D(c, l1, l2, 1, &sD);
        const double mie = (al1 + bl2) / 2;
        return exp(lD + mie + lL) * sD - exp(lC + mie + lL) * sC;
    }
    const double lC = int_C(c, l1, l2, 1, &sC), lD = int_D(c, l1, l2, 0, &sD);
    const double mie = (bl1 + al2) / 2;
    return exp(lC + mie + lL) * sC - exp(lD + mie + lL) * sD;
}

/* element (i,j) of the 2*ldim interleaved matrix (libcaps.c:717) */
static double kernel_M(ctx_t *c, int i, int j)
{
    static const char pol[2] = { 'E', 'M' };
    return M_elem(c, c->lmin + i / 2, c->lmin + j / 2, pol[i % 2], pol[j % 2]);
}

double oracle_epsm1(const oracle_material_t *mat, double xi)
{
    if (mat->kind == ORACLE_PERFECT) return INFINITY;
    return sq(mat->omegap) / (xi * (xi + mat->gamma)); /* libcaps.c:150 */
}

/* ------------------------------------------------------------------------- */
/* dense log-det (src/matrix.c:57-577)                                        */
/* ------------------------------------------------------------------------- */

/* log|det A| by LU with partial pivoting, A row-major n x n (overwritten) */
double oracle_logdet_lu(double *A, int n)
{
    double *lg = malloc(n * sizeof(double));
    for (int k = 0; k < n; k++) {
        int piv = k; double mx = fabs(A[(size_t)k * n + k]);
        for (int i = k + 1; i < n; i++) { double v = fabs(A[(size_t)i * n + k]); if (v > mx) { mx = v; piv = i; } }
        if (mx == 0) die("logdet_lu: singular");
        if (piv != k) for (int j = 0; j < n; j++) { double t = A[(size_t)k * n + j]; A[(size_t)k * n + j] = A[(size_t)piv * n + j]; A[(size_t)piv * n + j] = t; }
        const double inv = 1 / A[(size_t)k * n + k];
        for (int i = k + 1; i < n; i++) {
            double *ri = A + (size_t)i * n; const double *rk = A + (size_t)k * n;
            const double f = ri[k] * inv;
            ri[k] = f;
            if (f != 0) for (int j = k + 1; j < n; j++) ri[j] -= f * rk[j];
        }
        lg[k] = log(fabs(A[(size_t)k * n + k]));
    }
    double s = kahan(lg, n);
    free(lg);
    return s;
}

/* log det(1-M) for the dense path: trace shortcut, Mercator shortcut, LU.
 * M is row-major n x n and is overwritten (matrix.c:57-119, 489-577). */
double oracle_logdet_1mM(double *M, int n, int *path)
{
    double *d = malloc(n * sizeof(double));
    for (int i = 0; i < n; i++) d[i] = M[(size_t)i * n + i];
    const double tr = kahan(d, n);
    if (fabs(tr) < 1e-8) { free(d); if (path) *path = 1; return -tr; }
    double fro = 0;
    for (size_t i = 0; i < (size_t)n * n; i++) fro += sq(M[i]);
    fro = sqrt(fro);
    if (fro < 1) {
        /* z=-1: log det(1-M) ~ -tr M - tr M^2/2 */
        const double trA = -tr;
        for (int i = 0; i < n; i++) {
            double s = 0;
            for (int k = 0; k < n; k++) s += M[(size_t)i * n + k] * M[(size_t)k * n + i];
            d[i] = s;
        }
        const double trA2 = kahan(d, n);
        const double merc = trA - trA2 / 2;
        const double err = fabs(sq(fro) / 2 + fro + log1p(-fro));
        if (fabs(err / merc) < 1e-8) { free(d); if (path) *path = 2; return merc; }
    }
    free(d);
    for (size_t i = 0; i < (size_t)n * n; i++) M[i] = -M[i];
    for (int i = 0; i < n; i++) M[(size_t)i * n + i] += 1;
    if (path) *path = 3;
    return oracle_logdet_lu(M, n);
}

/* fill the full round-trip matrix M (row-major, dim = 2*ldim) */
void oracle_M_dense(const oracle_geom_t *g, double xi_, int m, double *M)
{
    ctx_t c; ctx_init(&c, g, xi_, m);
    const int n = 2 * g->ldim;
    /* same fill order as the reference: diagonal, then minor diagonals */
    for (int i = 0; i < n; i++) M[(size_t)i * n + i] = kernel_M(&c, i, i);
    for (int md = 1; md < n; md++)
        for (int k = 0; k < n - md; k++) {
            M[(size_t)k * n + md + k] = kernel_M(&c, k, md + k);
            M[(size_t)(md + k) * n + k] = kernel_M(&c, md + k, k);
        }
    ctx_free(&c);
}

double oracle_logdetD(const oracle_geom_t *g, double xi_, int m)
{
    if (xi_ <= 0) die("oracle_logdetD: xi must be positive");
    const int n = 2 * g->ldim;
    /* diagonal first: trace shortcut needs no off-diagonal elements */
    ctx_t c; ctx_init(&c, g, xi_, m);
    double *dg = malloc(n * sizeof(double));
    for (int i = 0; i < n; i++) dg[i] = kernel_M(&c, i, i);
    const double tr = kahan(dg, n);
    if (fabs(tr) < 1e-8) { free(dg); ctx_free(&c); return -tr; }
    double *M = malloc((size_t)n * n * sizeof(double));
    for (int i = 0; i < n; i++) M[(size_t)i * n + i] = dg[i];
    for (int md = 1; md < n; md++)
        for (int k = 0; k < n - md; k++) {
            M[(size_t)k * n + md + k] = kernel_M(&c, k, md + k);
            M[(size_t)(md + k) * n + k] = kernel_M(&c, md + k, k);
        }
    free(dg); ctx_free(&c);
    const double r = oracle_logdet_1mM(M, n, NULL);
    free(M);
    return r;
}

/* K and I tables of one (xi,m), for kernel-level parity checks.
 * logK[p*nnu + nu] for nu < nnu; logI[(p*nl + l1)*nl + l2], sign in sI. */
void oracle_K_table(const oracle_geom_t *g, double xi_, int m, int nu_lo, int nu_hi, double *logK_TE, double *logK_TM)
{
    ctx_t c; ctx_init(&c, g, xi_, m);
    for (int nu = nu_lo; nu <= nu_hi; nu++) {
        int s;
        logK_TM[nu - nu_lo] = integrate_K(nu, m, 1, c.alpha, c.epsm1_plate, &s, &c.nev);
        logK_TE[nu - nu_lo] = c.is_pr ? logK_TM[nu - nu_lo] : integrate_K(nu, m, 0, c.alpha, c.epsm1_plate, &s, &c.nev);
    }
    ctx_free(&c);
}

double oracle_I(const oracle_geom_t *g, double xi_, int m, int l1, int l2, int p, int *sign)
{
    ctx_t c; ctx_init(&c, g, xi_, m);
    double v = ctx_I(&c, l1, l2, p, sign);
    ctx_free(&c);
    return v;
}

/* ------------------------------------------------------------------------- */
/* xi = 0 and high-temperature terms (libcaps.c:860-1145)                     */
/* ------------------------------------------------------------------------- */
double oracle_ht_drude(double LbyR) /* libcaps.c:1043 */
{
    const double x = LbyR, x2 = x * x;
    const double Z = (1 + x) * (1 - sqrt((x2 + 2 * x) / (x2 + 2 * x + 1)));
    double s1 = 0, s2 = 0;
    for (int l = 1;; l++) {
        const double a = pow(Z, 2 * l), b = a * Z;
        const double v1 = (2 * l + 1) * log1p(-b), v2 = b * (1 - a) / (1 - b);
        s1 += v1; s2 += v2;
        if (fabs(v1 / s1) < 1e-15 && fabs(v2 / s2) < 1e-15) break;
    }
    return 0.5 * (s1 + log1p(-(1 - sq(Z)) * s2));
}

/* log det(1-M0) of the xi=0 MM block for perfect reflectors (libcaps.c:920, 985) */
double oracle_logdetD0_MM(const oracle_geom_t *g, int m)
{
    const double LbyR = g->L / g->R, y = -O_LOG2 - log1p(LbyR);
    const int n = g->ldim, lmin = oracle_lmin(LbyR, g->ldim, m);
    double *M = malloc((size_t)n * n * sizeof(double));
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const int l1 = i + lmin, l2 = j + lmin;
            M[(size_t)i * n + j] = exp((l1 + l2 + 1) * y + oracle_lfac(l1 + l2)
                                       - 0.5 * (oracle_lfac(l1 + m) + oracle_lfac(l1 - m) + oracle_lfac(l2 + m) + oracle_lfac(l2 - m)))
                                   * sqrt(((double)l1 * l2) / ((l1 + 1.) * (l2 + 1.)));
        }
    const double r = oracle_logdet_1mM(M, n, NULL);
    free(M);
    return r;
}

double oracle_ht_perf(const oracle_geom_t *g, double eps) /* libcaps.c:1089 */
{
    const double LbyR = g->L / g->R;
    const double drude = oracle_ht_drude(LbyR);
    double MM = 0;
    const double Z = 1. / (1 + LbyR + sqrt(LbyR * (2 + LbyR)));
    for (int l = 0;; l++) {
        const double v = 0.5 * log1p(-pow(Z, 2 * l + 3));
        MM += v;
        if (fabs(v / MM) < eps) break;
    }
    for (int m = 1;; m++) {
        const double v = oracle_logdetD0_MM(g, m);
        MM += v;
        if (fabs(v / MM) < eps) return drude + MM;
    }
}

/* ------------------------------------------------------------------------- */
/* plasma model, xi = 0 (integration.c:897-1031, libcaps.c:882-909, 1127-1145)  */
/* ------------------------------------------------------------------------- */
typedef struct { int nu; double omegap_, log_prefactor; } pargs_t;

/* -r_TE e^{-t} t^nu / nu!, r_TE = -b/(2+b), b = sqrtpm1((2 omegap_/t)^2) (integration.c:921) */
static double plasma_integrand(double t, const pargs_t *a)
{
    const double x = 2 * a->omegap_ / t;
    const double betam1 = sqrtpm1(x * x);
    return betam1 / (2 + betam1) * exp(a->log_prefactor - t + a->nu * log(t));
}

static double pl_panel(const pargs_t *a, double lo, double hi)
{
    const double h = (hi - lo) / 2, c = (lo + hi) / 2;
    double s = 0;
    for (int i = 0; i < GLN; i++) s += gl_w[i] * plasma_integrand(c + h * gl_x[i], a);
    return s * h;
}

static double pl_adapt(const pargs_t *a, double lo, double hi, double whole, double tol, int depth)
{
    const double mid = (lo + hi) / 2;
    const double l = pl_panel(a, lo, mid), r = pl_panel(a, mid, hi);
    if (fabs(l + r - whole) <= tol || depth >= 50) return l + r;
    return pl_adapt(a, lo, mid, l, tol / 1.4142135623730951, depth + 1) + pl_adapt(a, mid, hi, r, tol / 1.4142135623730951, depth + 1);
}

static double pl_integrate(const pargs_t *a, double lo, double hi, double tol_abs)
{
    const double w = pl_panel(a, lo, hi);
    return pl_adapt(a, lo, hi, w, fmax(tol_abs, 1e-14 * fabs(w)), 0);
}

/* I_nu = int_0^inf dt (-r_TE) e^{-t} t^nu / nu! on the reference's intervals [0,a],
 * [a,b], [b,inf) with a = max(0, nu - 5/sqrt(nu)), b = nu + 5/sqrt(nu)
 * (integration.c:979-1013); [b,inf) is cut where e^{-t} t^nu / nu! < 1e-40 */
double oracle_plasma_I(int nu, double omegap_)
{
    pthread_once(&tables_once, tables_init);
    pthread_once(&gl_once, gl_init);
    pargs_t args = { nu, omegap_, -oracle_lfac(nu) };
    const double width = 1 / sqrt((double)nu), a = fmax(0, nu - 5 * width), b = nu + 5 * width;
    const double I2 = pl_integrate(&args, a, b, 0);
    const double I1 = a > 0 ? pl_integrate(&args, 0, a, 1e-16 * I2) : 0;
    double c = b + 10;
    while (args.log_prefactor - c + nu * log(c) > -92) c += 10 + sqrt((double)nu);
    const double I3 = pl_integrate(&args, b, c, 1e-16 * I2);
    return I1 + I2 + I3;
}

/* log det(1-M0) of the plasma xi=0 MM block (libcaps.c:882-909, 985-1016);
 * Itab[nu] = oracle_plasma_I(nu, omegap_) for nu up to 2(lmin+ldim-1) */
static double logdetD0_MM_plasma_tab(const oracle_geom_t *g, int m, double omegap, const double *Itab)
{
    const double LbyR = g->L / g->R, y = -O_LOG2 - log1p(LbyR);
    const double omegap_ = omegap * (g->L + g->R) / O_C, alpha = omegap_ / (1 + LbyR);
    const int n = g->ldim, lmin = oracle_lmin(LbyR, g->ldim, m);
    double *f = malloc((size_t)n * sizeof(double));
    for (int i = 0; i < n; i++) {
        const int l = i + lmin;
        f[i] = 1 - (2 * l + 1.) / (alpha * oracle_ratioI(l - 0.5, alpha));
    }
    double *M = malloc((size_t)n * n * sizeof(double));
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) {
            const int l1 = i + lmin, l2 = j + lmin;
            const double factor = sqrt(l1 * f[i] / (l1 + 1.) * l2 * f[j] / (l2 + 1.));
            M[(size_t)i * n + j] = factor * exp(oracle_lfac(l1 + l2) - 0.5 * (oracle_lfac(l1 + m) + oracle_lfac(l1 - m) + oracle_lfac(l2 + m)
                                                                            + oracle_lfac(l2 - m)) + (l1 + l2 + 1) * y) * Itab[l1 + l2];
        }
    const double r = oracle_logdet_1mM(M, n, NULL);
    free(M); free(f);
    return r;
}

static double *plasma_table(const oracle_geom_t *g, int numax, double omegap)
{
    const double omegap_ = omegap * (g->L + g->R) / O_C;
    double *Itab = malloc((size_t)(numax + 1) * sizeof(double));
    Itab[0] = NAN;
    for (int nu = 1; nu <= numax; nu++) Itab[nu] = oracle_plasma_I(nu, omegap_);
    return Itab;
}

double oracle_logdetD0_MM_plasma(const oracle_geom_t *g, int m, double omegap)
{
    const int lmin = oracle_lmin(g->L / g->R, g->ldim, m);
    double *Itab = plasma_table(g, 2 * (lmin + g->ldim - 1), omegap);
    const double r = logdetD0_MM_plasma_tab(g, m, omegap, Itab);
    free(Itab);
    return r;
}

/* caps_ht_plasma (libcaps.c:1127): drude + sum'_m MM_plasma until |v/sum| < eps */
double oracle_ht_plasma(const oracle_geom_t *g, double omegap, double eps)
{
    const double drude = oracle_ht_drude(g->L / g->R);
    int numax = 0;
    double *Itab = NULL, sum = 0;
    for (int m = 0;; m++) {
        const int need = 2 * (oracle_lmin(g->L / g->R, g->ldim, m) + g->ldim - 1);
        if (need > numax) {
            free(Itab);
            numax = need + 256;
            Itab = plasma_table(g, numax, omegap);
        }
        const double v = logdetD0_MM_plasma_tab(g, m, omegap, Itab);
        sum += m == 0 ? v / 2 : v;
        if (fabs(v / sum) < eps) { free(Itab); return drude + sum; }
    }
}

/* ------------------------------------------------------------------------- */
/* batch evaluation on host threads (CPU baseline)                            */
/* ------------------------------------------------------------------------- */
typedef struct {
    const oracle_geom_t *g; const double *xi; const int *m; double *out;
    int n; int next; pthread_mutex_t lock;
} batch_t;

static void *batch_worker(void *arg)
{
    batch_t *b = (batch_t *)arg;
    for (;;) {
        pthread_mutex_lock(&b->lock);
        int i = b->next++;
        pthread_mutex_unlock(&b->lock);
        if (i >= b->n) break;
        b->out[i] = oracle_logdetD(b->g, b->xi[i], b->m[i]);
    }
    return NULL;
}

/* logdetD for n (xi,m) tasks on nthreads host threads, dynamic scheduling */
void oracle_logdetD_batch(const oracle_geom_t *g, int n, const double *xi, const int *m, double *out, int nthreads)
{
    pthread_once(&tables_once, tables_init);
    pthread_once(&gl_once, gl_init);
    if (nthreads < 1) nthreads = 1;
    batch_t b = { g, xi, m, out, n, 0, PTHREAD_MUTEX_INITIALIZER };
    pthread_t *th = malloc(nthreads * sizeof(pthread_t));
    for (int t = 0; t < nthreads; t++) pthread_create(&th[t], NULL, batch_worker, &b);
    for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
    free(th);
}

/* ------------------------------------------------------------------------- */
/* free energy, serial restatement of the caps driver (src/caps.c:307-396,   */
/* 749-852): Matsubara sum with m cutoff; xi=0 term per material model.       */
/* ------------------------------------------------------------------------- */
double oracle_free_energy(const oracle_geom_t *g, double T, double cutoff, double epsrel, int nthreads,
                          double *xi_out, double *v_out, int *nxi, int *ndet)
{
    const double hbar = 1.0545718e-34, kB = 1.38064852e-23, c = 299792458.;
    const double Ts = 2 * M_PI * kB * (g->R + g->L) * T / (hbar * c);
    const double LbyR = g->L / g->R;
    double v[4096]; int nv = 0, dets = 0;
    /* xi = 0 (caps.c:329-395): Drude (gamma > 0) analytic; perfect reflectors and the
     * plasma model (gamma = 0): drude_HT + sum'_m of the logdetD0 MM (resp. MM_plasma)
     * blocks with the m cutoff and half weight for m=0 */
    const int plasma = g->plate.kind == ORACLE_DRUDE && g->plate.gamma == 0;
    if (g->plate.kind == ORACLE_PERFECT || plasma) {
        double t0[4096]; int ms = -1, numax = 0;
        double *Itab = NULL;
        for (int m = 0; m < 4096; m++) {
            if (plasma) {
                const int need = 2 * (oracle_lmin(LbyR, g->ldim, m) + g->ldim - 1);
                if (need > numax) { free(Itab); numax = need + 256; Itab = plasma_table(g, numax, g->plate.omegap); }
                t0[m] = logdetD0_MM_plasma_tab(g, m, g->plate.omegap, Itab);
            } else
                t0[m] = oracle_logdetD0_MM(g, m);
            if (t0[m] == 0 || t0[m] / t0[0] < cutoff) { ms = m; break; }
        }
        free(Itab);
        t0[0] /= 2;
        v[nv++] = oracle_ht_drude(LbyR) + kahan(t0, ms + 1);
    } else
        v[nv++] = oracle_ht_drude(LbyR); /* Drude: analytic */
    if (xi_out) { xi_out[0] = 0; v_out[0] = v[0]; }
    for (int n = 1; n < 4096; n++) {
        const double xi_ = n * Ts;
        /* m loop in chunks of nthreads (the reference farms m speculatively;
         * only terms up to the first m meeting the cutoff are summed here) */
        double terms[4096]; int mstop = -1;
        for (int m0 = 0; m0 < 4096 && mstop < 0; m0 += nthreads) {
            int cnt = nthreads; double xs[256]; int ms[256]; double out[256];
            if (cnt > 256) cnt = 256;
            for (int k = 0; k < cnt; k++) { xs[k] = xi_; ms[k] = m0 + k; }
            oracle_logdetD_batch(g, cnt, xs, ms, out, nthreads);
            dets += cnt;
            for (int k = 0; k < cnt; k++) {
                terms[m0 + k] = out[k];
                if (mstop < 0 && (out[k] == 0 || out[k] / terms[0] < cutoff)) mstop = m0 + k;
            }
        }
        terms[0] /= 2;
        v[nv] = kahan(terms, mstop + 1);
        if (xi_out) { xi_out[nv] = xi_; v_out[nv] = v[nv]; }
        nv++;
        if (fabs(v[nv - 1] / v[0]) < epsrel) break;
    }
    if (nxi) *nxi = nv;
    if (ndet) *ndet = dets;
    v[0] /= 2;
    return Ts / M_PI * kahan(v, nv);
}

/* ------------------------------------------------------------------------- */
/* integer-order modified Bessel functions (src/bessel.c:283-633)             */
/*                                                                            */
/* The branch structure of bessel_logIn / bessel_logKn is restated: series    */
/* for x < 5 sqrt(n) (bessel.c:744), Miller's downward recurrence started     */
/* from the continued-fraction ratio (bessel.c:608-620), upward recurrence of */
/* K in the log domain (bessel.c:506-544), Debye asymptotics for n >= 100.    */
/* Orders 0 and 1: the reference evaluates Cephes Chebyshev fits              */
/* (bessel.c:283-461), which are not restated; here the power series for      */
/* x < 8 as the reference's I_0/I_1, I_1 = I_0 / ratio above, and for I_0 and */
/* K_0, K_1 the trapezoidal rule on the integral representations             */
/* (DLMF 10.32.3, 10.32.9) or Hankel's expansion (DLMF 10.40.1) at large x.   */
/* The values are pinned against the reference library's functions.         */
/* ------------------------------------------------------------------------- */
static double o_logInu_series(double nu, double x) /* bessel.c:744-759 */
{
    const double y = 0.25 * x * x;
    double v = 1, sum = 0;
    for (int m = 1; m < 2048; m++) {
        v *= y / (m * (m + nu));
        sum += v;
        if (v < 1e-16 * sum) return 0.5 * nu * log(y) - lgamma(1 + nu) + log1p(sum);
    }
    return NAN;
}

double oracle_bessel_logI0(double x)
{
    if (x < 0) return NAN;
    if (x == 0) return 0;
    if (x < 8) return o_logInu_series(0, x);
    if (x > 2000) {
        double term = 1, sum = 1;
        for (int k = 1; k < 60; k++) {
            term *= (2.0 * k - 1) * (2.0 * k - 1) / (8.0 * k * x);
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        return x - 0.5 * log(2 * M_PI * x) + log(sum);
    }
    /* (1/pi) int_0^pi exp(x (cos th - 1)) dth by the trapezoidal rule (aliasing I_{2N}) */
    const int N = 20 + (int)ceil(sqrt(25 * x));
    double s = 0.5 * (1 + exp(-2 * x));
    for (int k = 1; k < N; k++) s += exp(x * (cos(M_PI * k / N) - 1));
    return x + log(s / N);
}

double oracle_bessel_logI1(double x)
{
    if (x <= 0) return NAN;
    if (x < 8) return o_logInu_series(1, x);
    return oracle_bessel_logI0(x) - log(oracle_ratioI(0, x));
}

/* log K_nu(x), nu = 0 or 1: x + log int_0^inf exp(-x (cosh t - 1)) cosh(nu t) dt */
static double o_logK01(int nu, double x)
{
    if (x <= 0) return NAN;
    const double h = fmin(M_PI * M_PI / (42 + fmax(0, -log(x))), 0.6 / sqrt(x));
    double s = 0.5, prev = 1;
    for (int k = 1; k < 1000000; k++) {
        const double t = k * h;
        const double f = exp(-x * (cosh(t) - 1)) * (nu ? cosh(t) : 1.0);
        s += f;
        if (f < 1e-18 * s && f <= prev) break;
        prev = f;
    }
    return -x + log(h * s);
}
double oracle_bessel_logK0(double x) { return o_logK01(0, x); }
double oracle_bessel_logK1(double x) { return o_logK01(1, x); }

double oracle_bessel_logKn(int n, double x) /* bessel.c:506-581 */
{
    if (n < 0) n = -n;
    if (n == 0) return oracle_bessel_logK0(x);
    if (n == 1) return oracle_bessel_logK1(x);
    if (n >= 100) return oracle_logK_asymp(n, x);
    double Km = oracle_bessel_logK0(x), K = oracle_bessel_logK1(x);
    for (int j = 1; j < n; j++) {
        const double k = 0.5 * x / j;
        const double Kp = -log(k) + K + log1p(exp(Km - K) * k);
        Km = K;
        K = Kp;
    }
    return K;
}

double oracle_bessel_logIn(int n, double x) /* bessel.c:583-621 */
{
    if (n < 0) n = -n;
    if (n == 0) return oracle_bessel_logI0(x);
    if (n == 1) return oracle_bessel_logI1(x);
    if (x == 0) return -INFINITY;
    if (n >= 100) return oracle_logI_asymp(n, x);
    if (x < 5 * sqrt(n)) return o_logInu_series(n, x);
    double Ip = 1, I = oracle_ratioI(n - 1, x); /* I_n = 1, I_{n-1}/I_n */
    for (int k = n - 1; k > 0; k--) {
        const double Im = Ip + 2 * k / x * I;
        Ip = I;
        I = Im;
    }
    return oracle_bessel_logI0(x) - log(I);
}

/* ------------------------------------------------------------------------- */
/* cylinder-plane round trip (src/capc.cpp:47-127 and the kernel :155-177)    */
/* ------------------------------------------------------------------------- */

/* kernel_logdet's rules for a symmetric M (matrix.c:57-149): hodlr = 1 keeps the HODLR
 * branch's trace shortcut and final |tr| > |logdet| check around an exact LU */
static double o_kernel_logdet(double *M, int n, int hodlr)
{
    if (!hodlr) return oracle_logdet_1mM(M, n, NULL);
    double *d = malloc(n * sizeof(double));
    for (int i = 0; i < n; i++) d[i] = M[(size_t)i * n + i];
    const double tr = kahan(d, n);
    free(d);
    if (fabs(tr) < 1e-8) return -tr;
    for (size_t i = 0; i < (size_t)n * n; i++) M[i] = -M[i];
    for (int i = 0; i < n; i++) M[(size_t)i * n + i] += 1;
    const double ld = oracle_logdet_lu(M, n);
    return fabs(tr) > fabs(ld) ? -tr : ld;
}

double oracle_capc_logdet(double R, double d, int lmax, double q, char DN, int hodlr)
{
    const double calL = d + R, xr = R * q;
    const int dn = (DN == 'D' || DN == 'd');
    double *ratio = malloc((lmax + 1) * sizeof(double)), *K = malloc(2 * (lmax + 1) * sizeof(double));
    for (int j = 0; j < 2 * (lmax + 1); j++) K[j] = oracle_bessel_logKn(j, 2 * calL * q);
    if (dn) {
        for (int j = 0; j <= lmax; j++) ratio[j] = oracle_bessel_logIn(j, xr) - oracle_bessel_logKn(j, xr);
    } else {
        /* I'_0/K'_0 = -I_1/K_1; I'_j/(-K'_j) = (I_{j-1} + I_{j+1}) / (K_{j-1} + K_{j+1}) */
        ratio[0] = oracle_bessel_logI1(xr) - oracle_bessel_logK1(xr);
        for (int j = 1; j <= lmax; j++) {
            const double num = logadd(oracle_bessel_logIn(j - 1, xr), oracle_bessel_logIn(j + 1, xr));
            const double den = logadd(oracle_bessel_logKn(j - 1, xr), oracle_bessel_logKn(j + 1, xr));
            ratio[j] = num - den;
        }
    }
    const double M00 = exp(ratio[0] + K[0]);
    const double log_rho = log1p(-M00), alpha = 2 / (1 - M00);
    double *M = malloc((size_t)lmax * lmax * sizeof(double));
    double total = log_rho;
    for (int type = 0; type < 2; type++) {
        for (int i = 0; i < lmax; i++)
            for (int j = 0; j < lmax; j++) {
                const int mu1 = i + 1, mu2 = j + 1;
                const double term1 = 0.5 * (ratio[mu1] + ratio[mu2]);
                const double U = exp(term1 + K[mu1 + mu2]), V = exp(term1 + K[abs(mu1 - mu2)]);
                M[(size_t)i * lmax + j] = type == 0 ? U - V : U + V + alpha * exp(term1 + ratio[0] + K[mu1] + K[mu2]);
            }
        total += o_kernel_logdet(M, lmax, hodlr);
    }
    free(M); free(ratio); free(K);
    return total;
}
