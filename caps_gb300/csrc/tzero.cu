// tzero.cu -- frequency integration around the batched logdetD engine.
//
// * T = 0: E = 1/(alpha pi) int_0^inf dx F(x/alpha), x = 2 xi L/c, alpha = 2L/(L+R)
//   (caps.c:722-748), with the reference's integrand rule (caps.c:235-267: F = 0 beyond
//   the PFA estimate of logdetD = 1e-100 when L/R < 0.1).  Quadrature: QUADPACK's qagi
//   (the reference's default) or the Fourier-Chebyshev scheme (fcqs.c:107).
// * finite T by Pade spectrum decomposition (caps.c:811-831, psd.c:80): F at the PSD
//   poles with the PSD weights instead of the Matsubara frequencies.
//
// The quadrature rules keep the reference's steps exactly (same abscissae, same
// adaptive decisions, same extrapolation), so that E agrees with the reference's to
// rounding; what changes is the grouping: every function value a step needs (30 for a
// qagi bisection, all new nodes of an fcqs level, all PSD poles) is one batch of F,
// and F itself batches the (xi, m) matrices of all its frequencies on the GPU.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <functional>
#include <vector>

#include "../../include/libcaps.h"
#include "internal.h"

namespace capsgpu {


// ---------------------------------------------------------------------------
// QUADPACK qagi (Piessens, de Doncker-Kapenga, Ueberhuber, Kahaner 1983), as the
// reference's vendored C translation runs it (cquadpack/src/dqagi.c, dqk15i.c,
// dqext.c, dqsort.c): [bound, inf) (or its mirror, or the whole line) mapped to
// (0,1] by x = bound + (1-t)/t, 15-point Gauss-Kronrod on sub-intervals, bisection of
// the interval with the largest error, epsilon-algorithm extrapolation.
// ---------------------------------------------------------------------------
namespace qp {

const double EPMACH = DBL_EPSILON, UFLOW = DBL_MIN, OFLOW = DBL_MAX;
constexpr int LIMIT = 500;

// Kronrod abscissae and weights of the 7/15-point pair (QUADPACK qk15i)
const double XK[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                      0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                      0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                      0.207784955007898467600689403773245, 0.0};
const double WK[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                      0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                      0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                      0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
// Gauss weights of the 7-point rule at XK[1], XK[3], XK[5] and the centre
const double WG[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                      0.381830050505118944950369775488975, 0.417959183673469387755102040816327};

struct Rule { double result, abserr, resabs, resasc; };

// abscissae x of the 15 nodes of [a,b] in (0,1]: centre first, then the pairs
// c -/+ h XK[j]; with inf == 2 the mirrored points follow (30 values)
static int nodes(double boun, int inf, double a, double b, double *x)
{
    const double dinf = std::min(1.0, (double)inf);
    const double c = 0.5 * (a + b), h = 0.5 * (b - a);
    double t[15];
    t[0] = c;
    for (int j = 0; j < 7; j++) { t[1 + 2 * j] = c - h * XK[j]; t[2 + 2 * j] = c + h * XK[j]; }
    for (int k = 0; k < 15; k++) x[k] = boun + dinf * (1.0 - t[k]) / t[k];
    if (inf == 2) { for (int k = 0; k < 15; k++) x[15 + k] = -x[k]; return 30; }
    return 15;
}

// the rule from the function values at nodes() (same operation order as qk15i)
static Rule rule(int inf, double a, double b, const double *f)
{
    const double c = 0.5 * (a + b), h = 0.5 * (b - a);
    auto val = [&](int k) { return inf == 2 ? f[k] + f[15 + k] : f[k]; };
    double fv1[7], fv2[7];
    const double fc = (val(0) / c) / c;
    double resg = fc * WG[3], resk = fc * WK[7], resabs = std::fabs(resk);
    for (int j = 0; j < 7; j++) {
        const double x1 = c - h * XK[j], x2 = c + h * XK[j];
        const double f1 = (val(1 + 2 * j) / x1) / x1, f2 = (val(2 + 2 * j) / x2) / x2;
        fv1[j] = f1; fv2[j] = f2;
        const double fsum = f1 + f2;
        if (j & 1) resg += WG[j / 2] * fsum;
        resk += WK[j] * fsum;
        resabs = resabs + WK[j] * (std::fabs(f1) + std::fabs(f2));
    }
    const double reskh = resk * 0.5;
    double resasc = WK[7] * std::fabs(fc - reskh);
    for (int j = 0; j < 7; j++) resasc = resasc + WK[j] * (std::fabs(fv1[j] - reskh) + std::fabs(fv2[j] - reskh));
    Rule r;
    r.result = resk * h;
    r.resabs = resabs * h;
    r.resasc = resasc * h;
    r.abserr = std::fabs((resk - resg) * h);
    if (r.resasc != 0.0 && r.abserr != 0.0) r.abserr = r.resasc * std::min(1.0, std::pow(200.0 * r.abserr / r.resasc, 1.5));
    if (r.resabs > UFLOW / (50.0 * EPMACH)) r.abserr = std::max(EPMACH * 50.0 * r.resabs, r.abserr);
    return r;
}

// epsilon algorithm on tab[0..*n] (Wynn; QUADPACK qelg): returns the extrapolated
// value, its error estimate in *err; tab holds up to 52 entries, last3 the last three
// results, *nres the call count
static double epsilon(int *n, double *tab, double *err, double *last3, int *nres)
{
    (*nres)++;
    int nn = *n + 1; // 1-based count of entries
    *err = OFLOW;
    double result = tab[*n];
    if (nn >= 3) {
        const int limexp = 50;
        tab[*n + 2] = tab[*n];
        const int newelm = *n / 2;
        tab[*n] = OFLOW;
        const int num = nn;
        int k1 = nn;
        bool early = false;
        for (int i = 1; i <= newelm; i++) {
            const int k2 = k1 - 1, k3 = k1 - 2;
            double res = tab[k1 + 1];
            const double e0 = tab[k3 - 1], e1 = tab[k2 - 1], e2 = res;
            const double e1abs = std::fabs(e1);
            const double delta2 = e2 - e1, err2 = std::fabs(delta2), tol2 = std::max(std::fabs(e2), e1abs) * EPMACH;
            const double delta3 = e1 - e0, err3 = std::fabs(delta3), tol3 = std::max(e1abs, std::fabs(e0)) * EPMACH;
            if (err2 <= tol2 && err3 <= tol3) { // convergence: the table has reached rounding
                result = res;
                *err = err2 + err3;
                early = true;
                break;
            }
            const double e3 = tab[k1 - 1];
            tab[k1 - 1] = e1;
            const double delta1 = e1 - e3, err1 = std::fabs(delta1), tol1 = std::max(e1abs, std::fabs(e3)) * EPMACH;
            double ss = 0.0;
            bool stop = err1 <= tol1 || err2 <= tol2 || err3 <= tol3;
            if (!stop) {
                ss = 1.0 / delta1 + 1.0 / delta2 - 1.0 / delta3;
                stop = !(std::fabs(ss * e1) > 1.0e-4);
            }
            if (stop) { nn = i + i - 1; break; }
            res = e1 + 1.0 / ss;
            tab[k1 - 1] = res;
            k1 -= 2;
            const double error = err2 + std::fabs(res - e2) + err3;
            if (error <= *err) { *err = error; result = res; }
        }
        if (!early) {
            if (nn == limexp) nn = 2 * (limexp / 2) - 1;
            int ib = (num / 2) * 2 == num ? 2 : 1;
            for (int i = 1; i <= newelm + 1; i++) { tab[ib - 1] = tab[ib + 1]; ib += 2; }
            if (num != nn) {
                int indx = num - nn + 1;
                for (int i = 1; i <= nn; i++) { tab[i - 1] = tab[indx - 1]; indx++; }
            }
            if (*nres <= 3) {
                last3[*nres - 1] = result;
                *err = OFLOW;
            } else {
                *err = std::fabs(result - last3[2]) + std::fabs(result - last3[1]) + std::fabs(result - last3[0]);
                last3[0] = last3[1]; last3[1] = last3[2]; last3[2] = result;
            }
        }
    }
    *err = std::max(*err, 5.0 * EPMACH * std::fabs(result));
    *n = nn - 1;
    return result;
}

// keep iord[] ordered by descending error; on return *maxerr is the interval with the
// nrmax-th largest error (QUADPACK qpsrt)
static void order(int limit, int last, int *maxerr, double *ermax, const double *elist, int *iord, int *nrmax)
{
    if (last <= 1) {
        iord[0] = 0; iord[1] = 1;
    } else {
        const double errmax = elist[*maxerr];
        if (*nrmax != 0) {
            const int ido = *nrmax - 1;
            for (int i = 0; i <= ido; i++) {
                const int isucc = iord[*nrmax - 1];
                if (errmax <= elist[isucc]) break;
                iord[*nrmax] = isucc;
                (*nrmax)--;
            }
        }
        const int jupbn = last > limit / 2 + 2 ? limit + 3 - last : last;
        const double errmin = elist[last];
        const int jbnd = jupbn - 1, ibeg = *nrmax + 1;
        int i = ibeg;
        bool placed = false;
        for (; i <= jbnd; i++) {
            const int isucc = iord[i];
            if (errmax >= elist[isucc]) { placed = true; break; }
            iord[i - 1] = isucc;
        }
        if (!placed) {
            iord[jbnd] = *maxerr;
            iord[jupbn] = last;
        } else {
            iord[i - 1] = *maxerr;
            int k = jbnd;
            bool put = false;
            for (int j = i; j <= jbnd; j++) {
                const int isucc = iord[k];
                if (errmin < elist[isucc]) { iord[k + 1] = last; put = true; break; }
                iord[k + 1] = isucc;
                k--;
            }
            if (!put) iord[i] = last;
        }
    }
    *maxerr = iord[*nrmax];
    *ermax = elist[*maxerr];
}

// f evaluated in batches of the 15 (30) nodes of one rule, or both halves of a bisection
static double qagi(const BatchFn &F, double bound, int inf, double epsabs, double epsrel, double *abserr, int *neval, int *ier)
{
    const int limit = LIMIT - 1;
    std::vector<double> alist(LIMIT), blist(LIMIT), elist(LIMIT), rlist(LIMIT);
    std::vector<int> iord(LIMIT);
    double rlist2[52] = {0}, last3[3] = {0};
    *ier = 0; *neval = 0; *abserr = 0.0;
    double result = 0.0;
    alist[0] = 0.0; blist[0] = 1.0;
    if ((epsabs < 0.0 && epsrel < 0.0) || (inf != 1 && inf != -1 && inf != 2)) { *ier = 6; return result; }
    const double boun = inf == 2 ? 0.0 : bound;
    double x[60], fx[60];

    auto one = [&](double a, double b) {
        const int k = nodes(boun, inf, a, b, x);
        F(x, k, fx);
        return rule(inf, a, b, fx);
    };
    const Rule r0 = one(0.0, 1.0);
    result = r0.result;
    *abserr = r0.abserr;
    const double defabs = r0.resabs, resabs0 = r0.resasc;
    rlist[0] = result; elist[0] = *abserr; iord[0] = 0;
    const double dres = std::fabs(result);
    double errbnd = std::max(epsabs, epsrel * dres);
    if (*abserr <= 100.0 * EPMACH * defabs && *abserr > errbnd) *ier = 2;
    if (limit == 0) *ier = 1;
    int last = 0;
    double area = result, errsum = *abserr;
    bool done_sum = false; // leave through the "sum of all intervals" exit
    if (!(*ier != 0 || (*abserr <= errbnd && *abserr != resabs0) || *abserr == 0.0)) {
        rlist2[0] = result;
        double errmax = *abserr, erlarg = 0, ertest = 0, small = 0, correc = 0;
        int maxerr = 0, nrmax = 0, nres = 0, ktmin = 0, numrl2 = 1, ierro = 0, iroff1 = 0, iroff2 = 0, iroff3 = 0;
        bool extrap = false, noext = false;
        *abserr = OFLOW;
        const int ksgn = dres > (1.0 - 50.0 * EPMACH) * defabs ? 1 : -1;
        for (last = 1; last <= limit; last++) {
            const double a1 = alist[maxerr], b1 = 0.5 * (alist[maxerr] + blist[maxerr]), a2 = b1, b2 = blist[maxerr];
            const double erlast = errmax;
            // both halves in one batch
            const int k1 = nodes(boun, inf, a1, b1, x), k2 = nodes(boun, inf, a2, b2, x + k1);
            F(x, k1 + k2, fx);
            const Rule R1 = rule(inf, a1, b1, fx), R2 = rule(inf, a2, b2, fx + k1);
            const double area1 = R1.result, area2 = R2.result, error1 = R1.abserr, error2 = R2.abserr;
            const double area12 = area1 + area2, erro12 = error1 + error2;
            errsum = errsum + erro12 - errmax;
            area = area + area12 - rlist[maxerr];
            if (!(R1.resasc == error1 || R2.resasc == error2)) {
                if (!(std::fabs(rlist[maxerr] - area12) > 1.0e-5 * std::fabs(area12) || erro12 < .99 * errmax)) {
                    if (extrap) iroff2++; else iroff1++;
                }
                if (last > 9 && erro12 > errmax) iroff3++;
            }
            rlist[maxerr] = area1;
            rlist[last] = area2;
            errbnd = std::max(epsabs, epsrel * std::fabs(area));
            if (iroff1 + iroff2 >= 10 || iroff3 >= 20) *ier = 2;
            if (iroff2 > 5) *ier = 3;
            if (last == limit) *ier = 1;
            if (std::max(std::fabs(a1), std::fabs(b2)) <= (1.0 + 1000.0 * EPMACH) * (std::fabs(a2) + 1000.0 * UFLOW)) *ier = 4;
            if (error2 <= error1) {
                alist[last] = a2; blist[maxerr] = b1; blist[last] = b2; elist[maxerr] = error1; elist[last] = error2;
            } else {
                alist[maxerr] = a2; alist[last] = a1; blist[last] = b1;
                rlist[maxerr] = area2; rlist[last] = area1; elist[maxerr] = error2; elist[last] = error1;
            }
            order(limit, last, &maxerr, &errmax, elist.data(), iord.data(), &nrmax);
            if (errsum <= errbnd) { done_sum = true; break; }
            if (*ier != 0) break;
            if (last == 1) { small = .375; erlarg = errsum; ertest = errbnd; rlist2[1] = area; continue; }
            if (noext) continue;
            erlarg -= erlast;
            if (std::fabs(b1 - a1) > small) erlarg += erro12;
            if (!extrap) {
                // is the interval to bisect next the smallest one?
                if (std::fabs(blist[maxerr] - alist[maxerr]) > small) continue;
                extrap = true;
                nrmax = 1;
            }
            if (!(ierro == 3 || erlarg <= ertest)) {
                // bisect the larger intervals first while they carry the error
                const int id = nrmax;
                const int jupbnd = last > 2 + limit / 2 ? limit + 3 - last : last;
                bool larger = false;
                for (int k = id; k <= jupbnd; k++) {
                    maxerr = iord[nrmax];
                    errmax = elist[maxerr];
                    if (std::fabs(blist[maxerr] - alist[maxerr]) > small) { larger = true; break; }
                    nrmax++;
                }
                if (larger) continue;
            }
            // extrapolate
            numrl2++;
            rlist2[numrl2] = area;
            double abseps;
            const double reseps = epsilon(&numrl2, rlist2, &abseps, last3, &nres);
            ktmin++;
            if (ktmin > 5 && *abserr < 1.0e-3 * errsum) *ier = 5;
            if (abseps < *abserr) {
                ktmin = 0;
                *abserr = abseps;
                result = reseps;
                correc = erlarg;
                ertest = std::max(epsabs, epsrel * std::fabs(reseps));
                if (*abserr <= ertest) break;
            }
            if (numrl2 == 0) noext = true;
            if (*ier == 5) break;
            maxerr = iord[0];
            errmax = elist[maxerr];
            nrmax = 0;
            extrap = false;
            small = small * 0.5;
            erlarg = errsum;
        }
        if (last > limit) last = limit;
        if (!done_sum) {
            // final tests (labels 100-110 of qagie)
            bool use_sum = false, finish = false;
            if (*abserr == OFLOW) use_sum = true;
            else if (*ier + ierro != 0) {
                if (ierro == 3) *abserr += correc;
                if (*ier == 0) *ier = 3;
                if (result != 0.0 && area != 0.0) {
                    if (*abserr / std::fabs(result) > errsum / std::fabs(area)) use_sum = true;
                } else if (*abserr > errsum) use_sum = true;
                else if (area == 0.0) finish = true;
            }
            if (!use_sum && !finish) {
                if (!(ksgn == -1 && std::max(std::fabs(result), std::fabs(area)) <= defabs * .01))
                    if (0.01 > result / area || result / area > 100.0 || errsum > std::fabs(area)) *ier = 6;
            }
            if (use_sum) done_sum = true;
        }
    }
    if (done_sum) {
        result = 0.0;
        for (int k = 0; k <= last; k++) result += rlist[k];
        *abserr = errsum;
    }
    *neval = 30 * last + 15;
    if (inf == 2) *neval *= 2;
    if (*ier > 2) (*ier)--;
    return result;
}

// ---------------------------------------------------------------------------
// Fourier-Chebyshev quadrature on [0, inf) (fcqs.c:107): x = L cot^2(t/2), nested
// levels M = 5, 10, ..., 2560 sharing nodes; stop when two levels agree to epsrel.
// The new nodes of a level are one batch.
// ---------------------------------------------------------------------------
static double fcqs_semiinf(const BatchFn &F, double *epsrel, int *neval, double L, int *ier)
{
    constexpr int MMIN = 5, MMAX = 2560;
    std::vector<double> cache(MMAX, NAN);
    if (neval) *neval = 0;
    if (*epsrel <= 0) { *ier = 1; return NAN; }
    double Ilast = NAN;
    for (int M = MMIN; M <= MMAX; M *= 2) {
        const int ratio = MMAX / M, N = M - 1;
        std::vector<double> x;
        std::vector<int> idx;
        for (int i = 1; i <= N; i++)
            if (std::isnan(cache[ratio * i])) {
                const double ti = M_PI * i / (N + 1);
                const double ct = std::cos(ti / 2) / std::sin(ti / 2);
                x.push_back(L * (ct * ct));
                idx.push_back(ratio * i);
            }
        std::vector<double> y(x.size());
        if (!x.empty()) F(x.data(), (int)x.size(), y.data());
        if (neval) *neval += (int)x.size();
        for (size_t k = 0; k < x.size(); k++) cache[idx[k]] = y[k];
        double I = 0;
        for (int i = 1; i <= N; i++) {
            const double fti = cache[ratio * i];
            if (std::isnan(fti)) { *ier = 2; return Ilast; }
            if (std::isinf(fti)) { *ier = 3; return Ilast; }
            const double ti = M_PI * i / (N + 1);
            double sum = 0;
            for (int j = 1; j <= N; j += 2) sum += std::sin(j * ti) / j;
            const double om = 1 - std::cos(ti);
            I += 8 * L * std::sin(ti) / (om * om) / (N + 1) * sum * fti;
        }
        if (!std::isnan(Ilast)) {
            const double eps = std::fabs(1 - Ilast / I);
            if (eps < *epsrel) { *ier = 0; *epsrel = eps; return I; }
        }
        Ilast = I;
    }
    *ier = 4;
    return Ilast;
}

// ---------------------------------------------------------------------------
// Pade spectrum decomposition (Hu, Xu, Yan, J. Chem. Phys. 133, 101106 (2010); psd.c):
// poles xi_j = -2/w_j from the N negative eigenvalues w_j of the 2N x 2N symmetric
// tridiagonal matrix with zero diagonal and off-diagonal 1/sqrt((2j+1)(2j+3)), and
// weights eta_j from the recurrence of eq. (12).  The eigenvalues are found by
// bisection on Sturm counts, which for a zero-diagonal tridiagonal matrix resolve
// every eigenvalue to high relative accuracy.
// ---------------------------------------------------------------------------
static int sturm_below(const std::vector<double> &e2, double lam)
{
    // number of eigenvalues < lam: negative pivots of the LDL^T factorisation of T - lam I
    int cnt = 0;
    double q = -lam;
    if (q < 0) cnt++;
    for (size_t i = 1; i < e2.size() + 1; i++) {
        if (q == 0) q = DBL_MIN;
        q = -lam - e2[i - 1] / q;
        if (q < 0) cnt++;
    }
    return cnt;
}

static double psd_eta(int N, double z)
{
    double Am = 1 / 4., A = 5 / 4., Bm = 3, B = 15 + z / 4, dBm = 0, dB = 1 / 4.;
    for (int M = 3; M <= N; M++) {
        const double Amm = Am, Bmm = Bm, dBmm = dBm;
        Am = A; Bm = B; dBm = dB;
        dB = (2 * M + 1) * dBm + Bmm / 4 + z * dBmm / 4;
        A = (2 * M + 1) * Am + z * Amm / 4;
        B = (2 * M + 1) * Bm + z * Bmm / 4;
        Am /= A; Bm /= A; B /= A; dBm /= A; dB /= A;
        A = 1;
    }
    return A / (2 * dB);
}

static int psd(int N, double *xi, double *eta)
{
    const int n = 2 * N;
    std::vector<double> e2(n - 1);
    double norm = 0;
    for (int j = 1; j <= n - 1; j++) {
        const double e = 1 / std::sqrt((double)((2 * j + 1) * (2 * j + 3)));
        e2[j - 1] = e * e;
        norm = std::max(norm, 2 * e);
    }
    for (int k = 0; k < N; k++) {
        // the (k+1)-th smallest eigenvalue lies in [-norm, 0)
        double lo = -norm - 1e-300, hi = 0.0;
        for (int it = 0; it < 2000; it++) {
            const double mid = 0.5 * (lo + hi);
            if (mid == lo || mid == hi) break;
            if (sturm_below(e2, mid) > k) hi = mid; else lo = mid;
        }
        const double w = 0.5 * (lo + hi);
        xi[k] = -2 / w;
        eta[k] = psd_eta(2 * N, -xi[k] * xi[k]);
    }
    return 0;
}

} // namespace qp

double qagi_batched(const BatchFn &F, double bound, int inf, double epsabs, double epsrel, double *abserr, int *neval, int *ier)
{
    return qp::qagi(F, bound, inf, epsabs, epsrel, abserr, neval, ier);
}
} // namespace capsgpu

// implemented in libcaps.cu
void fxi_batch(caps_t *self, const double *xi, int n, double cutoff, double *out, int *ndet, int *nwasted, int kind);
double xi0_term(caps_t *self, double cutoff, int *ndet, int *nwasted);

using namespace capsgpu;

static double seconds_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// ---- quadrature and PSD on host callbacks (the reference's cquadpack / fcqs / psd API) ----
extern "C" double caps_dqagi(double (*f)(double, void *), void *userdata, double bound, int inf, double epsabs, double epsrel,
                             double *abserr, int *neval, int *ier)
{
    const BatchFn F = [&](const double *x, int n, double *y) { for (int k = 0; k < n; k++) y[k] = f(x[k], userdata); };
    return qp::qagi(F, bound, inf, epsabs, epsrel, abserr, neval, ier);
}

extern "C" double caps_fcqs_semiinf(double (*f)(double, void *), void *userdata, double *epsrel, int *neval, double L, int *ier)
{
    const BatchFn F = [&](const double *x, int n, double *y) { for (int k = 0; k < n; k++) y[k] = f(x[k], userdata); };
    return qp::fcqs_semiinf(F, epsrel, neval, L, ier);
}

extern "C" int caps_psd(int N, double *xi, double *eta)
{
    if (N < 1) return -1;
    return qp::psd(N, xi, eta);
}

// ---- free energy at T = 0 ----
extern "C" double caps_free_energy_T0(caps_t *self, double cutoff, double epsrel, int method, caps_energy_info_t *info)
{
    const auto t0 = std::chrono::steady_clock::now();
    const double L = self->L, R = self->R, LbyR = L / R;
    const double alpha = 2 * L / (L + R);
    // PFA estimate of the frequency beyond which logdetD < 1e-100 (caps.c:252-262)
    const double logdet_cutoff = 1e-100;
    const double xi_cutoff = -(1 + 1 / LbyR) * std::log(2 * LbyR * logdet_cutoff) / 2;
    int ndet = 0, nwasted = 0, nrec = 0;
    const BatchFn F = [&](const double *x, int n, double *y) {
        std::vector<double> xs;
        std::vector<int> where;
        for (int k = 0; k < n; k++) {
            const double xi_ = x[k] / alpha;
            if (LbyR < 0.1 && xi_ > xi_cutoff) y[k] = 0;
            else { xs.push_back(xi_); where.push_back(k); }
        }
        std::vector<double> v(xs.size());
        if (!xs.empty()) fxi_batch(self, xs.data(), (int)xs.size(), cutoff, v.data(), &ndet, &nwasted, 0);
        for (size_t k = 0; k < xs.size(); k++) y[where[k]] = v[k];
        for (int k = 0; k < n && info; k++, nrec++)
            if (nrec < 4096) {
                if (info->xi) info->xi[nrec] = x[k] / alpha;
                if (info->logdetD) info->logdetD[nrec] = y[k];
            }
    };
    double integral, abserr = 0, eps = epsrel;
    int neval = 0, ier = 0;
    if (method == 1) integral = qp::fcqs_semiinf(F, &eps, &neval, 1, &ier);
    else integral = qp::qagi(F, 0, 1, 0, epsrel, &abserr, &neval, &ier);
    if (ier != 0) fprintf(stderr, "caps_free_energy_T0: quadrature ier=%d\n", ier);
    if (info) {
        info->nxi = neval;
        info->ndet = ndet;
        info->nwasted = nwasted;
        info->seconds = seconds_since(t0);
    }
    return integral / alpha / M_PI;
}

// ---- Gauss-Laguerre rule: int_0^inf e^{-x} f(x) dx ~ sum_i w_i f(x_i) ----
// Nodes: eigenvalues of the n x n Jacobi matrix of the Laguerre polynomials (diagonal 2k + 1,
// off-diagonal k; Golub and Welsch 1969), found by bisection on Sturm counts and polished by
// Newton's method on L_n; weights w_i = x_i / ((n + 1) L_{n+1}(x_i))^2.  The caller receives
// w_i e^{x_i} (the integrand without its e^{-x}), formed from logarithms.
static void laguerre(int n, double x, double *Ln, double *dLn, double *Ln1)
{
    double p0 = 1.0, p1 = 1.0 - x; // L_0, L_1
    if (n == 0) p1 = 1.0;
    for (int k = 1; k < n; k++) { const double p2 = ((2 * k + 1 - x) * p1 - k * p0) / (k + 1); p0 = p1; p1 = p2; }
    // p1 = L_n, p0 = L_{n-1}; L_n' = n (L_n - L_{n-1}) / x; L_{n+1} = ((2n + 1 - x) L_n - n L_{n-1}) / (n + 1)
    *Ln = p1;
    *dLn = n * (p1 - p0) / x;
    *Ln1 = ((2 * n + 1 - x) * p1 - n * p0) / (n + 1);
}

extern "C" int caps_gauss_laguerre(int n, double *x, double *w_ex)
{
    if (n < 1 || n > 200) return 0;
    // Sturm count of the symmetric tridiagonal matrix below lam: the number of negative
    // pivots of T - lam I
    auto below = [&](double lam) {
        int cnt = 0;
        double d = 1.0 - lam; // k = 0
        if (d < 0) cnt++;
        for (int k = 1; k < n; k++) {
            const double e2 = (double)k * k;
            d = (2 * k + 1 - lam) - e2 / (d == 0.0 ? 1e-300 : d);
            if (d < 0) cnt++;
        }
        return cnt;
    };
    const double hi0 = 4.0 * n + 2.0; // Gershgorin bound: 2n - 1 + 2(n - 1) < 4n
    for (int i = 0; i < n; i++) {
        double lo = 0.0, hi = hi0;
        for (int it = 0; it < 200 && hi - lo > 1e-15 * hi; it++) {
            const double mid = 0.5 * (lo + hi);
            if (below(mid) > i) hi = mid; else lo = mid;
        }
        double z = 0.5 * (lo + hi), Ln, dLn, Ln1;
        for (int it = 0; it < 3; it++) {
            laguerre(n, z, &Ln, &dLn, &Ln1);
            if (dLn == 0.0) break;
            const double dz = Ln / dLn;
            if (!(std::fabs(dz) < 1e-3 * (hi - lo + 1e-12) + 1e-12 * z)) break; // stay inside the bracket
            z -= dz;
        }
        laguerre(n, z, &Ln, &dLn, &Ln1);
        x[i] = z;
        w_ex[i] = std::exp(std::log(z) - 2 * std::log(std::fabs((n + 1) * Ln1)) + z);
    }
    return 1;
}

// ---- free energy at T = 0 by an n-point Gauss-Laguerre rule in x = 2 xi L / c ----
extern "C" double caps_free_energy_T0_gl(caps_t *self, double cutoff, int n, caps_energy_info_t *info)
{
    const auto t0 = std::chrono::steady_clock::now();
    const double L = self->L, R = self->R, LbyR = L / R;
    const double alpha = 2 * L / (L + R);
    const double xi_cutoff = -(1 + 1 / LbyR) * std::log(2 * LbyR * 1e-100) / 2; // PFA cut (caps.c:252-262)
    std::vector<double> x(n), w(n), xs, F(n, 0.0);
    TERMINATE(!caps_gauss_laguerre(n, x.data(), w.data()), "Gauss-Laguerre rule of %d points not supported", n);
    std::vector<int> where;
    for (int i = 0; i < n; i++) {
        const double xi_ = x[i] / alpha;
        if (!(LbyR < 0.1 && xi_ > xi_cutoff)) { xs.push_back(xi_); where.push_back(i); }
    }
    int ndet = 0, nwasted = 0;
    std::vector<double> v(xs.size());
    if (!xs.empty()) fxi_batch(self, xs.data(), (int)xs.size(), cutoff, v.data(), &ndet, &nwasted, 0);
    for (size_t k = 0; k < xs.size(); k++) F[where[k]] = v[k];
    double s = 0, c = 0;
    for (int i = 0; i < n; i++) { const double y = w[i] * F[i] - c, u = s + y; c = (u - s) - y; s = u; }
    if (info) {
        info->nxi = n;
        info->ndet = ndet;
        info->nwasted = nwasted;
        info->seconds = seconds_since(t0);
        for (int i = 0; i < n && i < 4096; i++) {
            if (info->xi) info->xi[i] = x[i] / alpha;
            if (info->logdetD) info->logdetD[i] = F[i];
        }
    }
    return s / alpha / M_PI;
}

// ---- free energy at T > 0 by Pade spectrum decomposition ----
extern "C" double caps_free_energy_psd(caps_t *self, double T, double cutoff, double epsrel, int order, caps_energy_info_t *info)
{
    const auto t0 = std::chrono::steady_clock::now();
    TERMINATE(!(T > 0), "temperature must be positive");
    if (order <= 0) {
        // automatic order (caps.c:635-639)
        const double Teff = 4 * M_PI * CAPS_kB / CAPS_hbar / CAPS_c * T * self->L;
        order = (int)std::ceil((1 - 1.5 * std::log10(epsrel)) / std::sqrt(Teff));
    }
    const double Ts = 2 * M_PI * CAPS_kB * (self->R + self->L) * T / (CAPS_hbar * CAPS_c);
    int ndet = 0, nwasted = 0;
    const double v0 = xi0_term(self, cutoff, &ndet, &nwasted);
    std::vector<double> pxi(order), peta(order), xs(order), v(order + 1);
    qp::psd(order, pxi.data(), peta.data());
    for (int n = 0; n < order; n++) xs[n] = pxi[n] * Ts / (2 * M_PI);
    std::vector<double> Fv(order);
    fxi_batch(self, xs.data(), order, cutoff, Fv.data(), &ndet, &nwasted, 0);
    v[0] = v0 / 2;
    for (int n = 0; n < order; n++) v[n + 1] = peta[n] * Fv[n];
    double s = 0, c = 0;
    for (double t : v) { const double y = t - c, u = s + y; c = (u - s) - y; s = u; }
    if (info) {
        info->nxi = order + 1;
        info->ndet = ndet;
        info->nwasted = nwasted;
        info->seconds = seconds_since(t0);
        for (int n = 0; n <= order && n < 4096; n++) {
            if (info->xi) info->xi[n] = n == 0 ? 0.0 : xs[n - 1];
            if (info->logdetD) info->logdetD[n] = n == 0 ? v0 : Fv[n - 1];
        }
    }
    return Ts / M_PI * s;
}

// ---- sphere-sphere at T = 0 (cass.c:66-223) ----
// Two spheres of the caps object's radius R at separation d = 2L (the caps object is
// made with L = d/2): E d/(hbar c) = 1/(2 pi) int_0^inf dy F2(y), y = xi d/c,
// F2 = 2 sum_m logdet(1 - M^2) - the m = 0 term, m cut as the plane-sphere sum;
// QUADPACK qagi with relative tolerance epsrel.
extern "C" double caps_sphere_sphere_T0(caps_t *self, double cutoff, double epsrel, caps_energy_info_t *info)
{
    const auto t0 = std::chrono::steady_clock::now();
    const double L = self->L, R = self->R;
    int ndet = 0, nwasted = 0, nrec = 0;
    const BatchFn F = [&](const double *x, int n, double *y) {
        std::vector<double> xs(n);
        for (int k = 0; k < n; k++) xs[k] = x[k] * (L + R) / (2 * L);
        fxi_batch(self, xs.data(), n, cutoff, y, &ndet, &nwasted, 1);
        for (int k = 0; k < n && info; k++, nrec++)
            if (nrec < 4096) {
                if (info->xi) info->xi[nrec] = xs[k];
                if (info->logdetD) info->logdetD[nrec] = y[k];
            }
    };
    double abserr = 0;
    int neval = 0, ier = 0;
    const double integral = qp::qagi(F, 0, 1, 0, epsrel, &abserr, &neval, &ier);
    if (ier != 0) fprintf(stderr, "caps_sphere_sphere_T0: quadrature ier=%d\n", ier);
    if (info) {
        info->nxi = neval;
        info->ndet = ndet;
        info->nwasted = nwasted;
        info->seconds = seconds_since(t0);
    }
    return integral / (2 * M_PI);
}
