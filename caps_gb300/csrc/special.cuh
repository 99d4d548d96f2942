// special.cuh -- modified Bessel functions of half-integer order and the Mie
// coefficients a_l, b_l (log-magnitudes), FP64 device code.
//
// Algorithms (the same as CaPS v0.5):
//  * K_{n+1/2}(x): upward recurrence K_{l+1/2} = (2l-1)/x K_{l-1/2} + K_{l-3/2}
//    from K_{1/2}, K_{3/2}, rescaled by 2^-600 on growth (bessel.c:781-821);
//    for n >= 100 the uniform asymptotic expansion DLMF 10.41.4 (bessel.c:706).
//  * I_{n+1/2}(x): Wronskian I_nu K_{nu+1} + I_{nu+1} K_nu = 1/x with the ratio
//    I_nu/I_{nu+1} from the continued fraction DLMF 10.33.1 (bessel.c:635,831);
//    for n >= 100 the uniform expansion DLMF 10.41.3 (bessel.c:673).
//  * Mie coefficients: perfect reflector (libcaps.c:485) and Drude-type metal
//    (libcaps.c:557), both as log|a_l|, log|b_l|.
#pragma once
#include "common.cuh"

namespace capsgpu {

// I_nu(x)/I_{nu+1}(x): 2(nu+1)/x + 1/(2(nu+2)/x + 1/(...)), modified Lentz
CAPS_DEV double ratioI(double nu, double x)
{
    const double t = 2.0 / x;
    double f = (nu + 1) * t, C = f, D = 0;
    for (int k = 2; k < 4000000; k++) {
        const double b = (nu + k) * t;
        D = 1.0 / (b + D);
        C = b + 1.0 / C;
        const double d = C * D;
        f *= d;
        if (fabs(d - 1.0) < 1e-17) break;
    }
    return f;
}

// Debye polynomials of DLMF 10.41.10 as polynomials in p^2 (p^k taken out),
// summed as log1p(sum_k U_k y^k)
CAPS_DEV double debye_sum(double p2, double y)
{
    const double U1 = (3 - 5 * p2) / 24;
    const double U2 = (81 + p2 * (-462 + 385 * p2)) / 1152;
    const double U3 = (30375 + p2 * (-369603 + p2 * (765765 - 425425 * p2))) / 414720;
    const double U4 = (4465125 + p2 * (-94121676 + p2 * (349922430 + p2 * (-446185740 + 185910725 * p2)))) / 39813120;
    const double U5 = (1519035525. + p2 * (-49286948607. + p2 * (284499769554. + p2 * (-614135872350. + p2 * (566098157625. - 188699385875. * p2))))) / 6688604160.;
    return log1p(y * (U1 + y * (U2 + y * (U3 + y * (U4 + y * U5)))));
}

CAPS_DEV double logI_asymp(double nu, double x)
{
    const double z = x / nu, a = sqrt(1 + z * z), p2 = 1 / (1 + z * z);
    const double s = debye_sum(p2, 1 / (nu * a));
    const double eta = a + log(z / (1 + a));
    return nu * eta - 0.5 * log(2 * PI * nu * a) + s;
}

CAPS_DEV double logK_asymp(double nu, double x)
{
    const double z = x / nu, a = sqrt(1 + z * z), p2 = 1 / (1 + z * z);
    const double s = debye_sum(p2, -1 / (nu * a));
    const double eta = a + log(z / (1 + a));
    return -nu * eta - 0.5 * log(a) + 0.5 * log(0.5 * PI / nu) + s;
}

// log I_{n+1/2}(x), log K_{n+1/2}(x)
CAPS_DEV void logIK_half(int n, double x, double *logI, double *logK)
{
    const double logx = log(x), invx = 1.0 / x;
    double lk, lkp;
    if (n >= 100) {
        lkp = logK_asymp(n + 1.5, x);
        lk = logK_asymp(n + 0.5, x);
    } else {
        double k0 = 1, k1 = 1 + invx;
        int sc = 0;
        for (int l = 2; l <= n + 1; l++) {
            const double kn = fma((2 * l - 1) * invx, k1, k0);
            k0 = k1; k1 = kn;
            if (k0 > 0x1p600) { k0 *= 0x1p-600; k1 *= 0x1p-600; sc += 600; }
        }
        const double pre = -x + 0.5 * (log(PI / 2) - logx) + sc * LN2;
        lk = pre + log(k0);
        lkp = pre + log(k1);
    }
    if (logK) *logK = lk;
    if (logI) {
        if (n >= 100) *logI = logI_asymp(n + 0.5, x);
        else *logI = -logx - lkp - log1p(exp(lk - lkp - log(ratioI(n + 0.5, x))));
    }
}

CAPS_DEV double logadd(double a, double b)
{
    if (isinf(a) && a < 0) return b;
    if (isinf(b) && b < 0) return a;
    return a > b ? a + log1p(exp(b - a)) : b + log1p(exp(a - b));
}

// log|a_l|, log|b_l| at chi = xi_/(1+L/R); epsm1 = +inf selects perfect reflectors
CAPS_DEV void mie(double LbyR, double xi_, int l, double epsm1, double *lna, double *lnb)
{
    const double chi = xi_ / (1 + LbyR);
    const double ln_chi = log(xi_) - log1p(LbyR);
    double lIp, lKp, lIm, lKm;
    logIK_half(l, chi, &lIp, &lKp);
    logIK_half(l - 1, chi, &lIm, &lKm);
    const double ratio = ratioI(l - 0.5, chi);
    if (isinf(epsm1)) {
        *lnb = LOGPI - LN2 + lIp - lKp;
        const double num = LOGPI - LN2 + lIp + log(chi * ratio - l);
        const double den = logadd(log((double)l) + lKp, ln_chi + lKm);
        *lna = num - den;
        return;
    }
    const double ln_n = log1p(epsm1) / 2, nr = exp(ln_n), ln_l = log((double)l);
    double lIp_n, lKp_n, lIm_n, lKm_n;
    logIK_half(l, nr * chi, &lIp_n, &lKp_n);
    logIK_half(l - 1, nr * chi, &lIm_n, &lKm_n);
    const double ratio_n = ratioI(l - 0.5, nr * chi);
    const double ln_gB = lIp_n + lIp + ln_chi + log(nr * ratio_n - ratio);
    const double ln_gC = log(epsm1) + lIp_n + logadd(ln_chi + lKm, ln_l + lKp);
    const double ln_gD = ln_chi + logadd(lIp_n + lKm, ln_n + lKp + lIm_n);
    const double num = lIp_n + lIp + log(-l * epsm1 + nr * chi * (nr * ratio - ratio_n));
    *lnb = LOGPI - LN2 + ln_gB - ln_gD;
    *lna = LOGPI - LN2 + num - logadd(ln_gC, ln_gD);
}

} // namespace capsgpu
