// common.cuh -- shared device helpers for the CaPS round-trip-matrix kernels (sm_103a).
//
// Large and tiny quantities (K integrals, I integrals, Mie/Lambda scale
// factors) are carried as "scaled doubles": a double mantissa times 2^e with a
// 32-bit integer exponent.  Products add exponents, sums align to the larger
// exponent with an exact power-of-two shift done on the bit pattern.  This
// replaces the reference's log-domain arithmetic (exp/log per operation) with
// integer work, which matters on a part whose FP64 pipe is the scarce unit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define CAPS_DEV __device__ __forceinline__

namespace capsgpu {

constexpr double LN2 = 0.69314718055994530942;
constexpr double INV_LN2 = 1.4426950408889634074;
constexpr double LOGPI = 1.14472988584940017414;
constexpr double HALF_LOG_2PI = 0.91893853320467274178;
constexpr double PI = 3.14159265358979323846;

// number of Gauss-Legendre nodes per panel of the K quadrature
constexpr int GLN = 16;

struct sd { double m; int e; };   // value = m * 2^e

// per (m, l1 >= l2) pair: a_1, a_2 and a_0 = a0m 2^a0e of the I q-sum
struct A012 { double a1, a2, a0m; int a0e, pad; };
// the same for the mixed form, as float-float: a_1, a_2, and a_0 = (a0h + a0l) 2^a0e
struct A012F { float a1h, a1l, a2h, a2l, a0h, a0l; int a0e, pad; };

// 2^k as a double for -1022 <= k <= 1023
CAPS_DEV double pow2i(int k) { return __longlong_as_double((long long)(k + 1023) << 52); }

// exponent of a normal nonzero double (value in [2^k, 2^(k+1)))
CAPS_DEV int expo(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff) - 1023; }

// x * 2^k for |x| normal and the result normal; flushes to 0 below 2^-1020.
// Integer work only (no FP64 instruction): zero and subnormal inputs give 0.
CAPS_DEV double shift2(double x, int k)
{
    const long long b = __double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0 || ex + k <= 2) return 0.0;
    return __longlong_as_double(b + ((long long)k << 52));
}

// x == 0 (either sign) tested on the bit pattern
CAPS_DEV bool dzero(double x) { return (__double_as_longlong(x) << 1) == 0; }

// normalise so that |m| is in [1,2)
CAPS_DEV sd sd_norm(double m, int e)
{
    if (m == 0.0 || !isfinite(m)) return sd{m, 0};
    int k = expo(m);
    return sd{shift2(m, -k), e + k};
}

CAPS_DEV sd sd_from_log(double lg, int sign)
{
    if (isinf(lg) && lg < 0) return sd{0.0, 0};
    double t = lg * INV_LN2;
    double fl = floor(t);
    double m = exp((t - fl) * LN2);
    return sd{sign < 0 ? -m : m, (int)fl};
}

CAPS_DEV sd sd_mul(sd a, sd b) { return sd_norm(a.m * b.m, a.e + b.e); }

// a + b
CAPS_DEV sd sd_add(sd a, sd b)
{
    if (a.m == 0.0) return b;
    if (b.m == 0.0) return a;
    if (a.e >= b.e) {
        int d = b.e - a.e;
        return sd_norm(a.m + (d < -1000 ? 0.0 : shift2(b.m, d)), a.e);
    }
    int d = a.e - b.e;
    return sd_norm(b.m + (d < -1000 ? 0.0 : shift2(a.m, d)), b.e);
}

CAPS_DEV double sd_to_double(sd a)
{
    if (a.m == 0.0) return 0.0;
    if (a.e > 1000) return a.m > 0 ? INFINITY : -INFINITY;
    if (a.e < -1000) {
        // two steps so that the intermediate stays normal
        return shift2(shift2(a.m, -500), a.e + 500);
    }
    return a.m * pow2i(a.e);
}

CAPS_DEV double sd_log(sd a) { return log(fabs(a.m)) + a.e * LN2; }

// log n! : table for n<1024 (uploaded), first-order Stirling above, the same
// split as the reference's logfac.c
CAPS_DEV double lfac(const double *__restrict__ tab, int n)
{
    if (n < 1024) return __ldg(tab + n);
    const double dn = (double)n;
    return (dn + 0.5) * log(dn) - dn + HALF_LOG_2PI + (1.0 / 12) / dn;
}

// description of one (xi, m) matrix of a batch
struct Task {
    double xi_;          // xi (L+R)/c
    double alpha;        // 2 xi_
    double epsm1_plate;  // eps(i xi) - 1 of the plate, +inf for perfect reflectors
    double epsm1_sphere; // same for the sphere
    int m;
    int lmin;            // first l of the window
    int mu;              // order of the Legendre function in K: 2 max(m,1)
    int s;               // K integrand carries 1/(x^2-1)^s: s = (m>0)
    int nu_max;          // largest degree of K needed: 2 (lmin+ldim)
    int xi_index;        // row of the Mie table
    int is_pr;           // plate is a perfect reflector: K_TE = -K_TM
    int npanel;          // number of quadrature panels of K
    int mgroup;          // row of the per-m table of a_0, a_1, a_2 in the current chunk
};

// per-task result/status slots
enum : int {
    ST_OK = 0,
    ST_TRACE = 1,     // trace shortcut |tr M| < 1e-8 used
    ST_MERCATOR = 2,  // Mercator shortcut used
    ST_FACTOR = 3,    // full factorisation
    ST_ERR_PIVOT = 16,   // non-positive pivot in the Cholesky factorisation
    ST_ERR_NONFINITE = 32, // non-finite matrix element or integral
    ST_ERR_GRID = 64,      // quadrature grid did not fit the node budget
    ST_ERR_WAIT = 128,     // a bounded wait for the tensor cores ran out
    ST_ERR_HODLR = 256,    // HODLR: an off-diagonal block needed more than the largest rank
    ST_ERR_RANGE = 512,    // mixed form: a factor entry |x| >= 4, outside the range of the FP16 panel images
};

} // namespace capsgpu
