// capc.cu -- the cylinder-plane geometry at T = 0 (the reference's capc.cpp:20-177).
//
// A cylinder of radius R at distance d from a plane, both perfect reflectors: scalar
// Dirichlet (D) and Neumann (N) modes decouple, and at wave number q along the axis the
// reference writes (capc.cpp:47-127, :155-177)
//   log det(1 - M(q)) = log(1 - M_00) + log det(1 - (U - V)) + log det(1 - (U + V + alpha v v^T))
// for mu1, mu2 = 1 .. lmax, with
//   U = r(mu1)^1/2 r(mu2)^1/2 K_{mu1+mu2}(2 calL q),  V = the same with K_{|mu1-mu2|},
//   v_mu = r(0)^1/2 r(mu)^1/2 K_mu(2 calL q),  M_00 = r(0) K_0(2 calL q),  alpha = 2/(1 - M_00),
// calL = R + d, r(n) = I_n(Rq)/K_n(Rq) (D) or I'_n(Rq)/|K'_n(Rq)| (N).  The energy per
// length is E/(hbar c) = 1/(8 pi d) int_0^inf dx q logdet(q), q = x/(2d), by QUADPACK qagi
// (capc.cpp:129-153).
//
// GPU form: per q the host builds three short tables as scaled doubles -- sqrt r(mu),
// K_k(2 calL q) for k <= 2 lmax, and sqrt(alpha r(0)) sqrt r(mu) K_mu(2 calL q) -- and one
// kernel writes 1 - M of both matrices of every q of a batch, each element a product of
// table entries (no exp or log per element); the batched FP64 Cholesky with
// kernel_logdet's rules (matrix.c:57-149) gives the log dets.  A batch is every node of
// one qagi step.
//
// Integer-order Bessel functions, own method (the reference evaluates Cephes Chebyshev
// fits for orders 0 and 1, bessel.c:283-461, and per-order recurrences or Debye
// asymptotics above, bessel.c:506-633):
//   * K_0, K_1: trapezoidal rule on K_nu(x) = int_0^inf exp(-x cosh t) cosh(nu t) dt
//     (DLMF 10.32.9), geometrically convergent in the step;
//   * I_0: trapezoidal rule on I_0(x) = (1/pi) int_0^pi exp(x cos th) dth (DLMF 10.32.3),
//     exact up to aliasing terms I_{2N}(x), and Hankel's expansion (DLMF 10.40.1) for
//     large x;
//   * K_n, n >= 2: upward recurrence K_{n+1} = K_{n-1} + (2n/x) K_n (all terms positive);
//   * I_{n+1}/I_n: backward recurrence of the ratio started high enough above the largest
//     order that the starting error has decayed (Miller's algorithm).
// Values are kept as mantissa x 2^exponent, so nothing overflows and no logarithm is
// taken: table entries are accurate to a few ulps, where exp(sum of logs) loses |log| ulps.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/libcaps.h"
#include "../../include/capc.h"
#include "../../include/bessel.h"
#include "internal.h"

namespace capsgpu {

namespace {

constexpr double H_LN2 = 0.69314718055994530942;
constexpr double H_INV_LN2 = 1.4426950408889634074;
constexpr double H_LN2_TAIL = 2.3190468138462996e-17; // ln 2 - (double)(ln 2)
constexpr double H_PI = 3.14159265358979323846;

struct hx { double m; long long e; }; // m 2^e with m in [0.5, 1), or m = 0

hx hnorm(double m, long long e)
{
    if (m == 0.0 || !std::isfinite(m)) return hx{m, 0};
    int k;
    const double f = std::frexp(m, &k);
    return hx{f, e + k};
}
hx hmul(hx a, hx b) { return hnorm(a.m * b.m, a.e + b.e); }
hx hdiv(hx a, hx b) { return hnorm(a.m / b.m, a.e - b.e); }
hx hadd(hx a, hx b) // a, b >= 0
{
    if (a.m == 0.0) return b;
    if (b.m == 0.0) return a;
    if (a.e < b.e) std::swap(a, b);
    const long long d = b.e - a.e;
    return hnorm(a.m + (d < -1100 ? 0.0 : std::ldexp(b.m, (int)d)), a.e);
}
hx hsqrt(hx a)
{
    if (a.e & 1) { a.m *= 2.0; a.e -= 1; }
    return hnorm(std::sqrt(a.m), a.e / 2);
}
double hlog(hx a) { return std::log(a.m) + (double)a.e * H_LN2; }
double hval(hx a)
{
    if (a.m == 0.0 || !std::isfinite(a.m)) return a.m;
    if (a.e > 1100) return INFINITY;
    if (a.e < -1100) return 0.0;
    return std::ldexp(a.m, (int)a.e);
}
// e^y for any finite y: y = n ln2 + r, with n ln2 carried exactly (fma) so that r keeps
// full relative accuracy however large n is
hx hexp(double y)
{
    const double n = std::floor(y * H_INV_LN2);
    const double p = n * H_LN2, perr = std::fma(n, H_LN2, -p);
    const double r = ((y - p) - perr) - n * H_LN2_TAIL;
    return hnorm(std::exp(r), (long long)n);
}

// e^x K_0(x) and e^x K_1(x): trapezoidal rule in t with step h.  The integrand is analytic
// in |Im t| < pi/2; the step keeps the discretisation error below e^-40 relative both for
// small x (strip error ~ e^{-pi^2/h} / x) and large x (Gaussian of width x^-1/2).
void k01_scaled(double x, double &S0, double &S1)
{
    const double h = std::min(9.8696044010893586 / (42.0 + std::max(0.0, -std::log(x))), 0.6 / std::sqrt(x));
    double s0 = 0.5, s1 = 0.5, prev = 1.0;
    for (int k = 1; k < 1000000; k++) {
        const double t = k * h, sh = std::sinh(0.5 * t);
        const double g = std::exp(-2.0 * x * sh * sh); // exp(-x (cosh t - 1))
        const double f1 = g * std::cosh(t);
        s0 += g;
        s1 += f1;
        if (f1 < 1e-18 * s1 && f1 <= prev) break; // past the peak and negligible
        prev = f1;
    }
    S0 = h * s0;
    S1 = h * s1;
}

// e^-x I_0(x)
double i0_scaled(double x)
{
    if (x > 2000.0) {
        // Hankel: sum_k a_k / x^k, a_k = a_{k-1} (2k-1)^2 / (8k), all terms positive
        double term = 1.0, sum = 1.0;
        for (int k = 1; k < 60; k++) {
            term *= (2.0 * k - 1) * (2.0 * k - 1) / (8.0 * k * x);
            sum += term;
            if (term < 1e-18 * sum) break;
        }
        return sum / std::sqrt(2.0 * H_PI * x);
    }
    // N intervals on [0, pi]: the rule adds I_{2N}(x) + I_{2N+2}... relative to I_0, which
    // is below e^-50 once (2N)^2 >= 100 x (large x) or 2N >= 40 (small x)
    const int N = 20 + (int)std::ceil(std::sqrt(25.0 * x));
    double s = 0.5 * (1.0 + std::exp(-2.0 * x));
    for (int k = 1; k < N; k++) {
        const double sh = std::sin(0.5 * H_PI * k / N);
        s += std::exp(-2.0 * x * sh * sh); // exp(x (cos th - 1))
    }
    return s / N;
}

// K_0 .. K_J at x > 0
void k_table(double x, int J, hx *K)
{
    double S0, S1;
    k01_scaled(x, S0, S1);
    const hx ex = hexp(-x);
    K[0] = hmul(ex, hnorm(S0, 0));
    if (J >= 1) K[1] = hmul(ex, hnorm(S1, 0));
    double a = S0, b = S1; // K_{j-1}, K_j in units of 2^e e^-x
    long long e = 0;
    for (int j = 1; j < J; j++) {
        const double c = a + (2.0 * j / x) * b;
        a = b;
        b = c;
        if (b > 0x1p500) { a = std::ldexp(a, -500); b = std::ldexp(b, -500); e += 500; }
        K[j + 1] = hmul(ex, hnorm(b, e));
    }
}

// I_0 .. I_J at x > 0
void i_table(double x, int J, hx *I)
{
    I[0] = hmul(hexp(x), hnorm(i0_scaled(x), 0));
    if (J < 1) return;
    // start of the ratio recurrence: the error of r_M = 0 reaches order j damped by
    // I_M K_j / (K_M I_j) < e^-50 for M^2 >= j^2 + 50 x
    const int M = (int)std::ceil(std::sqrt((double)J * J + 50.0 * x)) + 30;
    std::vector<double> r(J);
    double rr = 0.0; // I_{j+1}/I_j
    for (int j = M - 1; j >= 0; j--) {
        rr = 1.0 / (2.0 * (j + 1) / x + rr);
        if (j < J) r[j] = rr;
    }
    for (int j = 0; j < J; j++) I[j + 1] = hmul(I[j], hnorm(r[j], 0));
}

// ---- tables and batch ----

struct QTab {
    double log_rho; // log(1 - M_00)
    bool ok;
};

// device-side table of one q: S[0..n), KQ[0..2n], W[0..n) as scaled doubles (m 2^e)
int tab_stride(int n) { return 4 * n + 1; }

sd to_sd(hx a)
{
    if (a.m == 0.0 || !std::isfinite(a.m)) return sd{a.m, 0};
    const long long e = std::max(-(1LL << 30), std::min(1LL << 30, a.e));
    return sd{a.m, (int)e};
}

QTab build_tab(double R, double d, int n, double q, char DN, sd *T)
{
    const double calL = R + d, xR = R * q, xK = 2.0 * calL * q;
    std::vector<hx> KQ(2 * n + 2), KR(n + 2), IR(n + 2), rat(n + 1);
    k_table(xK, 2 * n + 1, KQ.data());
    k_table(xR, n + 1, KR.data());
    i_table(xR, n + 1, IR.data());
    if (DN == 'D')
        for (int j = 0; j <= n; j++) rat[j] = hdiv(IR[j], KR[j]);
    else {
        // I'_0 / |K'_0| = I_1 / K_1;  I'_j / |K'_j| = (I_{j-1} + I_{j+1}) / (K_{j-1} + K_{j+1})
        rat[0] = hdiv(IR[1], KR[1]);
        for (int j = 1; j <= n; j++) rat[j] = hdiv(hadd(IR[j - 1], IR[j + 1]), hadd(KR[j - 1], KR[j + 1]));
    }
    const double M00 = hval(hmul(rat[0], KQ[0]));
    QTab Q;
    Q.ok = M00 < 1.0 && std::isfinite(M00);
    Q.log_rho = std::log1p(-M00);
    const double alpha = 2.0 / (1.0 - M00);
    const hx c1 = hsqrt(hmul(hnorm(Q.ok ? alpha : 1.0, 0), rat[0]));
    for (int mu = 1; mu <= n; mu++) {
        const hx s = hsqrt(rat[mu]);
        T[mu - 1] = to_sd(s);
        T[3 * n + mu] = to_sd(hmul(c1, hmul(s, KQ[mu])));
    }
    for (int k = 0; k <= 2 * n; k++) T[n + k] = to_sd(KQ[k]);
    return Q;
}

std::mutex g_capc_mu;
struct Buf {
    void *p = nullptr;
    size_t bytes = 0;
    void *get(size_t need)
    {
        if (need > bytes) {
            if (p) CK(cudaFree(p));
            bytes = std::max(need, bytes + bytes / 4);
            CK(cudaMalloc(&p, bytes));
        }
        return p;
    }
};
Buf b_tab, b_A, b_md, b_ld, b_tr, b_res, b_st;

} // namespace

// 1 - M of matrix `task` = 2 iq + type (lower triangle, column-major) and M_ii.
// grid (ceil(n/128), n, 2 nq): thread (r, c) for r >= c
__global__ void __launch_bounds__(128) k_capc_elem(int ntask, int n, const sd *__restrict__ tab, int tstride, double *A,
                                                   size_t mstride, double *mdiag)
{
    const int task = blockIdx.z, c = blockIdx.y, r = blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= ntask || r >= n || r < c) return;
    const sd *T = tab + (size_t)(task >> 1) * tstride;
    const sd *S = T, *KQ = T + n, *W = T + 3 * n + 1;
    const sd P = sd_mul(S[r], S[c]);
    const double U = sd_to_double(sd_mul(P, KQ[r + c + 2])), V = sd_to_double(sd_mul(P, KQ[r - c]));
    const double M = (task & 1) ? U + V + sd_to_double(sd_mul(W[r], W[c])) : U - V;
    A[(size_t)task * mstride + (size_t)c * n + r] = (r == c) ? 1.0 - M : -M;
    if (r == c) mdiag[(size_t)task * n + r] = M;
}

// log det of the cylinder-plane round trip for nq wave numbers; returns the number of
// results that are NaN because of a numerical failure
int capc_batch(double R, double d, int n, const double *q, int nq, char DN, int mode, double *out)
{
    std::lock_guard<std::mutex> lk(g_capc_mu);
    const size_t mstride = (size_t)n * n;
    const int ts = tab_stride(n);
    // chunks of at most ~4 GB of matrices and 16384 wave numbers (grid z = 2 per q)
    const int chunk = (int)std::max<size_t>(
        1, std::min<size_t>(std::min<size_t>((size_t)nq, 16384), ((size_t)4 << 30) / (2 * mstride * sizeof(double))));
    std::vector<sd> htab((size_t)chunk * ts);
    std::vector<QTab> qt(chunk);
    std::vector<double> res(2 * (size_t)chunk);
    std::vector<int> hst(2 * (size_t)chunk);
    int nbad = 0;
    const cudaStream_t st = 0;
    for (int q0 = 0; q0 < nq; q0 += chunk) {
        const int nc = std::min(chunk, nq - q0), nt = 2 * nc;
        for (int k = 0; k < nc; k++) qt[k] = build_tab(R, d, n, q[q0 + k], DN, htab.data() + (size_t)k * ts);
        sd *d_tab = (sd *)b_tab.get((size_t)nc * ts * sizeof(sd));
        double *d_A = (double *)b_A.get((size_t)nt * mstride * sizeof(double));
        double *d_md = (double *)b_md.get((size_t)nt * n * sizeof(double));
        double *d_ld = (double *)b_ld.get((size_t)nt * n * sizeof(double));
        double *d_tr = (double *)b_tr.get((size_t)nt * sizeof(double));
        double *d_res = (double *)b_res.get((size_t)nt * sizeof(double));
        int *d_st = (int *)b_st.get((size_t)nt * sizeof(int));
        CK(cudaMemcpyAsync(d_tab, htab.data(), (size_t)nc * ts * sizeof(sd), cudaMemcpyHostToDevice, st));
        g_counters.h2d += (long long)nc * ts * sizeof(sd);
        CK(cudaMemsetAsync(d_st, 0, (size_t)nt * sizeof(int), st));
        dim3 g((n + 127) / 128, n, nt);
        k_capc_elem<<<g, 128, 0, st>>>(nt, n, d_tab, ts, d_A, mstride, d_md);
        COUNT_LAUNCH(1);
        CK(cudaGetLastError());
        launch_stats(nullptr, nt, n, d_A, n, mstride, d_md, mode, d_tr, d_res, d_st, st);
        launch_cholesky(nt, n, d_A, n, mstride, d_st, d_ld, st);
        launch_final(nt, n, d_ld, d_tr, d_st, d_res, mode, st);
        CK(cudaMemcpyAsync(res.data(), d_res, (size_t)nt * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hst.data(), d_st, (size_t)nt * sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        g_counters.d2h += (long long)nt * (sizeof(double) + sizeof(int));
        g_counters.nmat += nt;
        for (int k = 0; k < nc; k++) {
            const bool bad = !qt[k].ok || (hst[2 * k] & ~0xF) || (hst[2 * k + 1] & ~0xF);
            out[q0 + k] = bad ? NAN : qt[k].log_rho + res[2 * k] + res[2 * k + 1];
            nbad += bad;
        }
    }
    return nbad;
}

} // namespace capsgpu

using namespace capsgpu;

namespace {
char norm_dn(char DN) { return std::toupper((unsigned char)DN) == 'D' ? 'D' : 'N'; } // capc.cpp:51-53
int norm_lmax(double R, double d, int lmax) { return lmax > 0 ? lmax : std::max(25, (int)(5 * R / d)); } // capc.cpp:28
} // namespace

extern "C" int caps_capc_lmax(double R, double d, double eta)
{
    TERMINATE(!(R > 0) || !(d > 0) || !(eta > 0), "capc: R, d and eta must be positive");
    return std::max(25, (int)std::ceil(eta / d * R));
}

extern "C" double caps_capc_pfa(double R, double d)
{
    return -H_PI * H_PI * H_PI / 1920 * std::sqrt(R / (2 * d)) / (d * d);
}

extern "C" int caps_capc_logdet_batch(double R, double d, int lmax, const double *q, int nq, char DN, detalg_t detalg, double *out)
{
    TERMINATE(!(R > 0) || !(d > 0), "capc: R and d must be positive");
    if (nq <= 0) return 0;
    for (int k = 0; k < nq; k++) TERMINATE(!(q[k] > 0) || !std::isfinite(q[k]), "capc: wave number q must be positive and finite");
    return capc_batch(R, d, norm_lmax(R, d, lmax), q, nq, norm_dn(DN), detalg == DETALG_HODLR ? 1 : 0, out);
}

extern "C" double caps_capc_logdet(double R, double d, int lmax, double q, char DN, detalg_t detalg)
{
    double r = NAN;
    caps_capc_logdet_batch(R, d, lmax, &q, 1, DN, detalg, &r);
    return r;
}

extern "C" double caps_capc_energy_T0(double R, double d, int lmax, char p, double epsrel, detalg_t detalg, int *neval_out,
                                      int *ier_out)
{
    TERMINATE(!(R > 0) || !(d > 0), "capc: R and d must be positive");
    TERMINATE(!(epsrel > 0), "capc: epsrel must be positive");
    const int n = norm_lmax(R, d, lmax);
    const char DN = norm_dn(p);
    const int mode = detalg == DETALG_HODLR ? 1 : 0;
    // integrand x -> q logdet(q), q = x/(2d) (capc.cpp:180-194), every node of a qagi step in one batch
    const BatchFn F = [&](const double *x, int k, double *y) {
        std::vector<double> qs(k);
        for (int i = 0; i < k; i++) qs[i] = x[i] / (2 * d);
        capc_batch(R, d, n, qs.data(), k, DN, mode, y);
        for (int i = 0; i < k; i++) y[i] *= qs[i];
    };
    double abserr = 0;
    int neval = 0, ier = 0;
    const double integral = qagi_batched(F, 0, 1, 0, epsrel, &abserr, &neval, &ier);
    if (neval_out) *neval_out = neval;
    if (ier_out) *ier_out = ier;
    return integral / (4 * H_PI * 2 * d);
}

// ---- integer-order modified Bessel functions (the reference's bessel.h names) ----

extern "C" double bessel_logI0(double x)
{
    if (x < 0) return NAN;
    if (x == 0) return 0.0;
    std::vector<hx> I(1);
    i_table(x, 0, I.data());
    return hlog(I[0]);
}

extern "C" double bessel_logI1(double x)
{
    if (!(x > 0)) return NAN;
    std::vector<hx> I(2);
    i_table(x, 1, I.data());
    return hlog(I[1]);
}

extern "C" double bessel_logK0(double x)
{
    if (!(x > 0)) return NAN;
    hx K;
    k_table(x, 0, &K);
    return hlog(K);
}

extern "C" double bessel_logK1(double x)
{
    if (!(x > 0)) return NAN;
    hx K[2];
    k_table(x, 1, K);
    return hlog(K[1]);
}

extern "C" double bessel_logIn(int n, double x)
{
    if (n < 0) n = -n;
    if (n == 0) return bessel_logI0(x);
    if (n == 1) return bessel_logI1(x);
    if (x == 0) return -INFINITY;
    if (!(x > 0)) return NAN;
    std::vector<hx> I(n + 1);
    i_table(x, n, I.data());
    return hlog(I[n]);
}

extern "C" double bessel_logKn(int n, double x)
{
    if (n < 0) n = -n;
    if (!(x > 0)) return NAN;
    std::vector<hx> K(n + 1);
    k_table(x, n, K.data());
    return hlog(K[n]);
}
