// kgrid.cuh -- panel grid for the K integrals of one (xi, m) matrix.
//
// K_{nu,p}^{(m)}(alpha) = int_1^inf r_p(x) e^{-alpha x} P_nu^mu(x) (x^2-1)^{-s} dx,
// mu = 2 max(m,1), s = (m>0)  (integration.c:257-286).  With x = cosh t the
// integrand of degree nu is a single peak in t; its position moves right with nu
// and its width is ~ kappa(t)^{-1/2}.  All degrees nu = mu..nu_max share ONE
// panel grid in t whose panel width follows the local peak width:
//   kappa(t) = alpha cosh t + k_eff cosh t / sinh^2 t,
// the curvature of -log of the integrand from the e^{-alpha cosh t} factor and
// from the sinh^k t behaviour near t = 0 (k = mu + 1 - 2s).  Each panel carries
// GLN Gauss-Legendre nodes.  Because every degree uses the same nodes, the K
// kernel obtains all P_nu^mu(x_k) from one forward recurrence in nu per node.
//
// The grid starts where even the lowest degree is negligible (e^-46 of its
// peak) -- or at t = 0 when k is small and the sinh^k factor is a low-order
// polynomial -- and ends once the highest degree has decayed by e^-52 past
// its peak.  The host/device function below writes the panel edges.
#pragma once
#include <math.h>

#ifndef __CUDACC__
#define KG_HD inline
#else
#define KG_HD __host__ __device__ inline
#endif

namespace capsgpu {

struct KGridParams {
    double c_width;   // panel width in units of the local peak width
    double neg_left;  // log-ratio below the lowest peak where the grid starts
    double neg_right; // log-ratio below the highest peak where the grid ends
    int kpoly;        // k <= kpoly: start at t=0, no sinh^-2 term in kappa
};

KG_HD KGridParams kgrid_default() { return KGridParams{1.0, 46.0, 52.0, 12}; }

// log of the lowest-degree integrand up to a constant: k log sinh t - alpha cosh t
KG_HD double kg_g0(double t, int k, double alpha) { return k * log(sinh(t)) - alpha * cosh(t); }

// d/dt log of the degree-nu integrand, Liouville-Green estimate of P_nu^mu
KG_HD double kg_dlog(double t, double nu, double mu, int s, double alpha)
{
    const double sh = sinh(t), ch = cosh(t), ct = ch / sh;
    const double y = -0.5 * ct + sqrt(0.25 * ct * ct + nu * (nu + 1) + mu * mu / (sh * sh));
    return y - alpha * sh + (1 - 2 * s) * ct;
}

KG_HD double kg_kappa(double t, double alpha, double keff)
{
    const double sh = sinh(t), ch = cosh(t);
    return alpha * ch + keff * ch / (sh * sh);
}

// Writes panel edges edges[0..np] (np panels) and returns np, or -1 if more
// than max_panels would be needed.
KG_HD int kgrid_build(double alpha, int mu, int s, int nu_max, const KGridParams &P, double *edges, int max_panels)
{
    const int k = mu + 1 - 2 * s;
    const double keff = (k <= P.kpoly) ? 0.0 : (double)(mu + 1);

    // peak of the lowest degree: k coth t = alpha sinh t  <=> sinh t tanh t = k/alpha
    const double r = (double)k / alpha;
    const double u = 0.5 * (r * r + sqrt(r * r * r * r + 4 * r * r));
    const double tp0 = asinh(sqrt(u));

    double t0 = 0.0;
    if (k > P.kpoly) {
        // left edge: g0(t) = g0(tp0) - neg_left, bisection in log t
        const double gt = kg_g0(tp0, k, alpha) - P.neg_left;
        double lo = log(tp0) - 80.0, hi = log(tp0);
        for (int it = 0; it < 100; it++) {
            const double mid = 0.5 * (lo + hi);
            if (kg_g0(exp(mid), k, alpha) < gt) lo = mid; else hi = mid;
        }
        t0 = exp(lo);
    }

    // peak of the highest degree: dlog = 0 (dlog decreases in t)
    double tlo = 1e-6, thi = 1.0;
    while (kg_dlog(thi, nu_max, mu, s, alpha) > 0 && thi < 700) thi *= 2;
    if (kg_dlog(tlo, nu_max, mu, s, alpha) < 0) tlo = 1e-12;
    for (int it = 0; it < 200; it++) {
        const double mid = 0.5 * (tlo + thi);
        if (kg_dlog(mid, nu_max, mu, s, alpha) > 0) tlo = mid; else thi = mid;
    }
    const double tpk = 0.5 * (tlo + thi);

    int np = 0;
    double t = t0;
    edges[0] = t0;
    double drop = 0.0;           // integrated dlog of the highest degree past its peak
    bool past = false;
    while (np < max_panels) {
        double h1 = P.c_width / sqrt(kg_kappa(t > 0 ? t : 1e-300, alpha, keff));
        if (t == 0.0) h1 = P.c_width / sqrt(alpha + (k > 0 ? 0.0 : 0.0));
        const double h2 = P.c_width / sqrt(kg_kappa(t + h1, alpha, keff));
        double h = h1 < h2 ? h1 : h2;
        if (h2 < 0.25 * h1) {
            // the local width overshoots into a far narrower region (small alpha, where
            // kappa grows like e^t over one step): take the self-consistent width
            // h = c / sqrt(kappa(t + h)) instead of the look-ahead's, which would crawl
            double lo = 0.0, hi = h1;
            for (int it = 0; it < 60; it++) {
                const double mid = 0.5 * (lo + hi);
                if (mid < P.c_width / sqrt(kg_kappa(t + mid, alpha, keff))) lo = mid; else hi = mid;
            }
            if (lo > h) h = lo;
        }
        const double tn = t + h;
        if (past || tn > tpk) {
            const double a = past ? t : tpk;
            if (tn > a) drop += 0.5 * (tn - a) * (kg_dlog(a, nu_max, mu, s, alpha) + kg_dlog(tn, nu_max, mu, s, alpha));
            past = true;
        }
        t = tn;
        edges[++np] = t;
        if (past && drop < -P.neg_right) return np;
    }
    return -1;
}

#ifdef __CUDACC__
// [lo, hi] brackets the point where a monotone predicate `below` turns from true to false;
// each round the 32 lanes of the warp test the 32 inner points of 33 equal sub-intervals
// and all lanes keep the sub-interval that holds the turn (5 bits per round against a
// bisection's 1).  Every lane returns the same bracket.
template <class F> __device__ inline void kg_warp_section(double &lo, double &hi, int rounds, F below)
{
    const int lane = threadIdx.x & 31;
    for (int r = 0; r < rounds; r++) {
        const double x = lo + (hi - lo) * (double)(lane + 1) * (1.0 / 33.0);
        const int c = __popc(__ballot_sync(0xffffffffu, below(x)));
        const double xl = __shfl_sync(0xffffffffu, x, c > 0 ? c - 1 : 0);
        const double xh = __shfl_sync(0xffffffffu, x, c < 32 ? c : 31);
        if (c > 0) lo = xl;
        if (c < 32) hi = xh;
    }
}

// kgrid_build for one warp (all 32 lanes call it and get the same result; lane 0 writes
// the edges): the same grid rules, with the three root searches as warp multisections
__device__ inline int kgrid_build_warp(double alpha, int mu, int s, int nu_max, const KGridParams &P, double *edges, int max_panels)
{
    const bool writer = (threadIdx.x & 31) == 0;
    const int k = mu + 1 - 2 * s;
    const double keff = (k <= P.kpoly) ? 0.0 : (double)(mu + 1);
    const double r = (double)k / alpha;
    const double u = 0.5 * (r * r + sqrt(r * r * r * r + 4 * r * r));
    const double tp0 = asinh(sqrt(u));

    double t0 = 0.0;
    if (k > P.kpoly) {
        // left edge: g0(t) = g0(tp0) - neg_left, in log t
        const double gt = kg_g0(tp0, k, alpha) - P.neg_left;
        double lo = log(tp0) - 80.0, hi = log(tp0);
        kg_warp_section(lo, hi, 12, [&](double x) { return kg_g0(exp(x), k, alpha) < gt; });
        t0 = exp(lo);
    }

    // peak of the highest degree: dlog = 0 (dlog decreases in t)
    double tlo = 1e-6, thi = 1.0;
    while (kg_dlog(thi, nu_max, mu, s, alpha) > 0 && thi < 700) thi *= 2;
    if (kg_dlog(tlo, nu_max, mu, s, alpha) < 0) tlo = 1e-12;
    kg_warp_section(tlo, thi, 16, [&](double x) { return kg_dlog(x, nu_max, mu, s, alpha) > 0; });
    const double tpk = 0.5 * (tlo + thi);

    int np = 0;
    double t = t0;
    if (writer) edges[0] = t0;
    double drop = 0.0;
    bool past = false;
    while (np < max_panels) {
        double h1 = P.c_width / sqrt(kg_kappa(t > 0 ? t : 1e-300, alpha, keff));
        if (t == 0.0) h1 = P.c_width / sqrt(alpha);
        const double h2 = P.c_width / sqrt(kg_kappa(t + h1, alpha, keff));
        double h = h1 < h2 ? h1 : h2;
        if (h2 < 0.25 * h1) {
            // self-consistent width h = c / sqrt(kappa(t + h)) (see kgrid_build)
            double lo = 0.0, hi = h1;
            kg_warp_section(lo, hi, 12, [&](double x) { return x < P.c_width / sqrt(kg_kappa(t + x, alpha, keff)); });
            if (lo > h) h = lo;
        }
        const double tn = t + h;
        if (past || tn > tpk) {
            const double a = past ? t : tpk;
            if (tn > a) drop += 0.5 * (tn - a) * (kg_dlog(a, nu_max, mu, s, alpha) + kg_dlog(tn, nu_max, mu, s, alpha));
            past = true;
        }
        t = tn;
        ++np;
        if (writer) edges[np] = t;
        if (past && drop < -P.neg_right) return np;
    }
    return -1;
}
#endif

} // namespace capsgpu
