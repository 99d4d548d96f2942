// assemble.cu -- FP64 assembly of the round-trip matrices M(xi,m) of a batch.
//
// Phases (each one launch over the whole batch):
//   k_setup   per task: K panel grid and the degree-recurrence coefficients
//   k_mie     per (xi, l): log|a_l|, log|b_l|                     (libcaps.c:485-602)
//   k_scale   per (task, l): symmetric scale factors sqrt(Lambda a_l), u(l), v(l)
//   k_ktab    per (task, 32 quadrature nodes): all K_{nu,p} partial sums
//   k_kred    per (task, nu): K table                             (integration.c:288-489)
//   k_itab    per (task, l1>=l2): I_{l1 l2,p} q-sums              (integration.c:491-671)
//   k_elem    per (task, 2x2 block): 1 - M, lower triangle        (libcaps.c:717-831,
//                                                                   integration.c:762-888)
//   k_stats   per task: Kahan trace, Frobenius norm, shortcut decision (matrix.c:57-119,489-505)
#include "common.cuh"
#include "ff.cuh"
#include "special.cuh"
#include "kgrid.cuh"
#include "qsum64.cuh"
#include "qsum_ff.cuh"
#include "internal.h"

namespace capsgpu {

__constant__ double c_glx[GLN];
__constant__ double c_glw[GLN];

void upload_gauss_legendre(const double *x, const double *w)
{
    CK(cudaMemcpyToSymbol(c_glx, x, GLN * sizeof(double)));
    CK(cudaMemcpyToSymbol(c_glw, w, GLN * sizeof(double)));
}

// ---------------------------------------------------------------------------
// setup: quadrature grid + recurrence coefficients for every task
// ---------------------------------------------------------------------------
__global__ void k_setup(Task *tasks, int ntask, double *edges, int max_panels, double2 *coefAB, int nu_stride,
                        double c_width, int *status)
{
    const int task = blockIdx.x;
    if (task >= ntask) return;
    Task &T = tasks[task];
    if (threadIdx.x < 32) { // warp 0 builds the grid
        KGridParams P = kgrid_default();
        P.c_width = c_width;
        const int np = kgrid_build_warp(T.alpha, T.mu, T.s, T.nu_max, P, edges + (size_t)task * (max_panels + 1), max_panels);
        if (threadIdx.x == 0) {
            if (np < 0) { T.npanel = 0; status[task] |= ST_ERR_GRID; }
            else T.npanel = np;
        }
    }
    // A_nu = (2nu+1)/(nu-mu+1), B_nu = (nu+mu)/(nu-mu+1): P_{nu+1} = A x P_nu - B P_{nu-1}
    const int nnu = T.nu_max - T.mu + 1;
    for (int i = threadIdx.x; i < nnu; i += blockDim.x) {
        const double nu = T.mu + i, d = 1.0 / (i + 1.0);
        coefAB[(size_t)task * nu_stride + i] = make_double2((2 * nu + 1) * d, (nu + T.mu) * d);
    }
}

// ---------------------------------------------------------------------------
// Mie coefficients per distinct xi
// ---------------------------------------------------------------------------
__global__ void k_mie(const double *xi_list, const double *epsm1_list, int nxi, double LbyR, int lmax,
                      double *lna, double *lnb)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x + 1;
    const int ix = blockIdx.y;
    if (l > lmax || ix >= nxi) return;
    double a, b;
    mie(LbyR, xi_list[ix], l, epsm1_list[ix], &a, &b);
    lna[(size_t)ix * (lmax + 1) + l] = a;
    lnb[(size_t)ix * (lmax + 1) + l] = b;
}

// per task and l in [lmin, lmin+ldim-1]: Sa = exp((f(l)+log a_l)/2), Sb likewise,
// f(l) = log(2l+1) - log l - log(l+1) + lfac(l-m) - lfac(l+m) so that
// exp(lnLambda + (log a1 + log a2)/2) = Sa(l1) Sa(l2)   (libcaps.c:45, :787)
__global__ void k_scale(const Task *tasks, int ntask, int ldim, const double *lna, const double *lnb, int lmax,
                        const double *lfac_tab, sd *Sa, sd *Sb, double2 *uv)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int task = blockIdx.y;
    if (a >= ldim + 2 || task >= ntask) return;
    const Task &T = tasks[task];
    const int l = T.lmin - 1 + a; // a indexes l-(lmin-1) in [0, ldim+1]
    const size_t o = (size_t)task * (ldim + 2) + a;
    const double m = T.m;
    uv[o] = make_double2(l >= 0 ? (l + 1.0) * (l + m) / (2 * l + 1.0) : 0.0,
                         l >= 0 ? (double)l * (l - m + 1.0) / (2 * l + 1.0) : 0.0);
    if (a == 0 || a == ldim + 1) { Sa[o] = sd{0, 0}; Sb[o] = sd{0, 0}; return; }
    const double f = log(2.0 * l + 1) - log((double)l) - log(l + 1.0) + lfac(lfac_tab, l - T.m) - lfac(lfac_tab, l + T.m);
    const size_t mo = (size_t)T.xi_index * (lmax + 1) + l;
    Sa[o] = sd_from_log(0.5 * (f + lna[mo]), 1);
    Sb[o] = sd_from_log(0.5 * (f + lnb[mo]), 1);
}

// ---------------------------------------------------------------------------
// K integrals on the shared panel grid
// ---------------------------------------------------------------------------
// One warp owns 32 nodes (two panels).  Each lane runs the degree recurrence of
// P_nu^mu at its node; at every degree the warp aligns the lane values to the
// warp-maximum binary exponent and parks them in shared memory; every 32
// degrees lane r folds row r with the node weights (times the Fresnel
// coefficient of each node) into the partial K sum of degree nu0+r.
constexpr int KT_WARPS = 8;

template <bool PR>
__global__ void __launch_bounds__(KT_WARPS * 32)
k_ktab(const Task *tasks, const double *edges, int max_panels, const double2 *coefAB, int nu_stride,
       const double *lfac_tab, double *partM, int *partE, int max_warps)
{
    extern __shared__ double smem[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *buf = smem + wib * (32 * 33);                    // [32][33]
    double *wTM = smem + KT_WARPS * 32 * 33 + wib * 64;      // [32]
    double *wTE = wTM + 32;                                  // [32]
    int *rowE = (int *)(smem + KT_WARPS * (32 * 33 + 64)) + wib * 32;

    const int task = blockIdx.y;
    const Task T = tasks[task];
    const int warp = blockIdx.x * KT_WARPS + wib;
    const int nwarp = (T.npanel + 1) / 2;
    if (warp >= nwarp) return;

    const int panel = warp * 2 + (lane >> 4), j = lane & 15;
    const bool valid = panel < T.npanel;
    double x = 1.0, WTM = 0.0, WTE = 0.0;
    int E = -(1 << 29);
    if (valid) {
        const double *ed = edges + (size_t)task * (max_panels + 1);
        const double a = ed[panel], b = ed[panel + 1];
        const double h = 0.5 * (b - a), c = 0.5 * (a + b);
        const double t = c + h * c_glx[j], w = h * c_glw[j];
        const double sh = sinh(t);
        x = cosh(t);
        // log of node weight times e^{-alpha x} sinh^{mu+1-2s} t (2mu-1)!!
        const double ldf = lfac(lfac_tab, 2 * T.mu) - T.mu * LN2 - lfac(lfac_tab, T.mu);
        const double lc = log(w) - T.alpha * x + (T.mu + 1 - 2 * T.s) * log(sh) + ldf;
        const double fl = floor(lc * INV_LN2);
        const double f = exp(lc - fl * LN2);
        E = (int)fl;
        double rTE = -1.0, rTM = 1.0;
        if (!PR) { // Fresnel at k = xi_ sinh t  (libcaps.c:616)
            const double eps = T.epsm1_plate;
            const double y = eps / (x * x);
            const double bm1 = y / (sqrt(1 + y) + 1);
            rTE = -bm1 / (2 + bm1);
            rTM = (eps - bm1) / (eps + 2 + bm1);
        }
        WTM = f * rTM;
        WTE = f * rTE;
    }
    wTM[lane] = WTM;
    wTE[lane] = WTE;

    double pp = 0.0, pc = valid ? 1.0 : 0.0;
    const int nnu = T.nu_max - T.mu + 1;
    const double2 *ab = coefAB + (size_t)task * nu_stride;
    const size_t pTM = ((size_t)(task * 2 + 1) * max_warps + warp) * nu_stride;
    const size_t pTE = ((size_t)(task * 2 + 0) * max_warps + warp) * nu_stride;

    for (int base = 0; base < nnu; base += 32) {
        const int rows = min(32, nnu - base);
        for (int r = 0; r < rows; r++) {
            const int e = (pc != 0.0) ? expo(pc) + E : -(1 << 29);
            const int emax = __reduce_max_sync(0xffffffffu, e);
            buf[r * 33 + lane] = (pc != 0.0 && e - emax > -1000) ? shift2(pc, E - emax) : 0.0;
            if (lane == 0) rowE[r] = emax;
            const double2 c = __ldg(ab + base + r);
            const double pn = fma(c.x * x, pc, -c.y * pp);
            pp = pc;
            pc = pn;
            if (fabs(pc) > 0x1p600) { pc *= 0x1p-600; pp *= 0x1p-600; E += 600; }
        }
        __syncwarp();
        if (lane < rows) {
            double sTM = 0.0, sTE = 0.0;
            const double *row = buf + lane * 33;
#pragma unroll 8
            for (int l = 0; l < 32; l++) {
                const double v = row[l];
                sTM = fma(v, wTM[l], sTM);
                if (!PR) sTE = fma(v, wTE[l], sTE);
            }
            partM[pTM + base + lane] = sTM;
            partE[pTM + base + lane] = rowE[lane];
            if (!PR) {
                partM[pTE + base + lane] = sTE;
                partE[pTE + base + lane] = rowE[lane];
            }
        }
        __syncwarp();
    }
}

// fold the per-warp partials into K_{nu,p} (scaled doubles)
// Mixed form of k_ktab: the same grid, node weights and row normalisation, with the
// Legendre recurrence and the 32-node dot products in float-float (~2^-48) on the FP32
// pipe.  P_nu^mu(x) > 0 for x >= 1 and every weight of one polarisation has one sign, so
// the sums do not cancel; the upward recurrence (dominant solution) loses at most a bit
// per step to its subtraction.  The node weights are still formed once per node in FP64.
// Partials: float-float (h, l) times 2^partE.
__global__ void k_coef_ff(int ntask, int nu_stride, const double2 *coefAB, float4 *coefF)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, task = blockIdx.y;
    if (i >= nu_stride || task >= ntask) return;
    const double2 c = coefAB[(size_t)task * nu_stride + i];
    const ff a = ff_from_d(c.x), b = ff_from_d(c.y);
    coefF[(size_t)task * nu_stride + i] = make_float4(a.h, a.l, b.h, b.l);
}

template <bool PR>
__global__ void __launch_bounds__(KT_WARPS * 32)
k_ktab_ff(const Task *tasks, const double *edges, int max_panels, const float4 *coefF, int nu_stride, const double *lfac_tab,
          float2 *partF, int *partE, int max_warps)
{
    extern __shared__ double smem[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *buf = reinterpret_cast<float2 *>(smem + wib * (32 * 33));      // [32][33]
    float2 *wTM = reinterpret_cast<float2 *>(smem + KT_WARPS * 32 * 33 + wib * 64); // [32]
    float2 *wTE = wTM + 32;                                                          // [32]
    int *rowE = (int *)(smem + KT_WARPS * (32 * 33 + 64)) + wib * 32;

    const int task = blockIdx.y;
    const Task T = tasks[task];
    const int warp = blockIdx.x * KT_WARPS + wib;
    const int nwarp = (T.npanel + 1) / 2;
    if (warp >= nwarp) return;

    const int panel = warp * 2 + (lane >> 4), j = lane & 15;
    const bool valid = panel < T.npanel;
    ff x{1.0f, 0.0f}, WTM{0.0f, 0.0f}, WTE{0.0f, 0.0f};
    int E = -(1 << 29);
    if (valid) {
        const double *ed = edges + (size_t)task * (max_panels + 1);
        const double a = ed[panel], b = ed[panel + 1];
        const double h = 0.5 * (b - a), c = 0.5 * (a + b);
        const double t = c + h * c_glx[j], w = h * c_glw[j];
        const double sh = sinh(t), xd = cosh(t);
        const double ldf = lfac(lfac_tab, 2 * T.mu) - T.mu * LN2 - lfac(lfac_tab, T.mu);
        const double lc = log(w) - T.alpha * xd + (T.mu + 1 - 2 * T.s) * log(sh) + ldf;
        const double fl = floor(lc * INV_LN2);
        const double f = exp(lc - fl * LN2);
        E = (int)fl;
        double rTE = -1.0, rTM = 1.0;
        if (!PR) { // Fresnel at k = xi_ sinh t  (libcaps.c:616)
            const double eps = T.epsm1_plate;
            const double y = eps / (xd * xd);
            const double bm1 = y / (sqrt(1 + y) + 1);
            rTE = -bm1 / (2 + bm1);
            rTM = (eps - bm1) / (eps + 2 + bm1);
        }
        x = ff_from_d(xd);
        WTM = ff_from_d(f * rTM);
        WTE = ff_from_d(f * rTE);
    }
    wTM[lane] = make_float2(WTM.h, WTM.l);
    wTE[lane] = make_float2(WTE.h, WTE.l);

    ff pp{0.0f, 0.0f}, pc{valid ? 1.0f : 0.0f, 0.0f};
    const int nnu = T.nu_max - T.mu + 1;
    const float4 *ab = coefF + (size_t)task * nu_stride;
    const size_t pTM = ((size_t)(task * 2 + 1) * max_warps + warp) * nu_stride;
    const size_t pTE = ((size_t)(task * 2 + 0) * max_warps + warp) * nu_stride;

    for (int base = 0; base < nnu; base += 32) {
        const int rows = min(32, nnu - base);
        for (int r = 0; r < rows; r++) {
            const int e = (pc.h != 0.0f) ? fexpo(pc.h) + E : -(1 << 29);
            const int emax = __reduce_max_sync(0xffffffffu, e);
            // align to the warp maximum by one multiply with 2^(E - emax) (0 below 2^-126; the
            // clamp at 2^127 only matters for a zero value, which stays zero)
            const float p2 = __uint_as_float((unsigned)min(max(127 + E - emax, 0), 254) << 23);
            const ff v{pc.h * p2, pc.l * p2};
            buf[r * 33 + lane] = make_float2(v.h, v.l);
            if (lane == 0) rowE[r] = emax;
            const float4 c = __ldg(ab + base + r);
            const ff pn = ff_add(ff_mul(ff_mul(ff{c.x, c.y}, x), pc), ff_neg(ff_mul(ff{c.z, c.w}, pp)));
            pp = pc;
            pc = pn;
            if (fabsf(pc.h) > 0x1p40f) { pc = ff_shift(pc, -40); pp = ff_shift(pp, -40); E += 40; }
        }
        __syncwarp();
        if (lane < rows) {
            ff sTM{0.0f, 0.0f}, sTE{0.0f, 0.0f};
            const float2 *row = buf + lane * 33;
#pragma unroll 8
            for (int l = 0; l < 32; l++) {
                const float2 v = row[l];
                const float2 wm = wTM[l];
                sTM = ff_add(sTM, ff_mul(ff{v.x, v.y}, ff{wm.x, wm.y}));
                if (!PR) {
                    const float2 we = wTE[l];
                    sTE = ff_add(sTE, ff_mul(ff{v.x, v.y}, ff{we.x, we.y}));
                }
            }
            partF[pTM + base + lane] = make_float2(sTM.h, sTM.l);
            partE[pTM + base + lane] = rowE[lane];
            if (!PR) {
                partF[pTE + base + lane] = make_float2(sTE.h, sTE.l);
                partE[pTE + base + lane] = rowE[lane];
            }
        }
        __syncwarp();
    }
}

// Mixed form of k_kred: the warps' float-float partials aligned to the largest exponent and
// summed in float-float, written as the paired table the q-sums read: TM and TE of one
// (task, nu) as one float4 (TM h, l, TE h, l; the larger of the two h in [1, 2)) under their
// common exponent (KPe), so that one alignment serves both polarisations
__global__ void k_kred_ff(const Task *tasks, int ntask, const float2 *partF, const int *partE, int max_warps, int nu_stride,
                          float4 *KP, int *KPe, int *status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int task = blockIdx.y;
    if (task >= ntask) return;
    const Task &T = tasks[task];
    const int nnu = T.nu_max - T.mu + 1;
    if (i >= nnu) return;
    const int nwarp = (T.npanel + 1) / 2;
    ffe kp[2];
    for (int p = 1; p >= 0; p--) {
        if (p == 0 && T.is_pr) { // K_TE = -K_TM for perfect reflectors (integration.c:638)
            kp[0] = ffe{-kp[1].h, -kp[1].l, kp[1].e, 0};
            continue;
        }
        const size_t base = (size_t)(task * 2 + p) * max_warps * nu_stride + i;
        int emax = -(1 << 29);
        for (int w = 0; w < nwarp; w++) {
            const float2 m = partF[base + (size_t)w * nu_stride];
            if (m.x != 0.0f) emax = max(emax, partE[base + (size_t)w * nu_stride]);
        }
        ff s{0.0f, 0.0f};
        for (int w = 0; w < nwarp; w++) {
            const float2 m = partF[base + (size_t)w * nu_stride];
            const int d = partE[base + (size_t)w * nu_stride] - emax;
            if (m.x != 0.0f && d > -100) s = ff_add(s, ff_shift(ff{m.x, m.y}, d));
        }
        const int k = fexpo(s.h);
        if (s.h == 0.0f || k == 128) {
            atomicOr(status + task, ST_ERR_NONFINITE);
            kp[p] = ffe{s.h, 0.0f, 0, 0};
        } else
            kp[p] = ffe{fshift(s.h, -k), fshift(s.l, -k), emax + k, 0};
    }
    const int e = max(kp[1].e, kp[0].e);
    const ff tm = ff_shift(ff{kp[1].h, kp[1].l}, kp[1].e - e), te = ff_shift(ff{kp[0].h, kp[0].l}, kp[0].e - e);
    KP[(size_t)task * nu_stride + i] = make_float4(tm.h, tm.l, te.h, te.l);
    KPe[(size_t)task * nu_stride + i] = e;
}

__global__ void k_kred(const Task *tasks, int ntask, const double *partM, const int *partE, int max_warps, int nu_stride,
                       sd *K, int *status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int task = blockIdx.y;
    if (task >= ntask) return;
    const Task &T = tasks[task];
    const int nnu = T.nu_max - T.mu + 1;
    if (i >= nnu) return;
    const int nwarp = (T.npanel + 1) / 2;
    for (int p = 1; p >= 0; p--) {
        sd *out = K + (size_t)(task * 2 + p) * nu_stride + i;
        if (p == 0 && T.is_pr) { // K_TE = -K_TM for perfect reflectors (integration.c:638)
            sd k = K[(size_t)(task * 2 + 1) * nu_stride + i];
            *out = sd{-k.m, k.e};
            continue;
        }
        const size_t base = (size_t)(task * 2 + p) * max_warps * nu_stride + i;
        int emax = -(1 << 29);
        for (int w = 0; w < nwarp; w++) {
            const double m = partM[base + (size_t)w * nu_stride];
            if (m != 0.0) emax = max(emax, partE[base + (size_t)w * nu_stride]);
        }
        double s = 0.0;
        for (int w = 0; w < nwarp; w++) {
            const double m = partM[base + (size_t)w * nu_stride];
            const int d = partE[base + (size_t)w * nu_stride] - emax;
            if (m != 0.0 && d > -1000) s += shift2(m, d);
        }
        if (s == 0.0 || !isfinite(s)) atomicOr(status + task, ST_ERR_NONFINITE);
        *out = sd_norm(s, emax);
    }
}

// ---------------------------------------------------------------------------
// I integrals: q-sum of K with the three-term a_q recurrence (integration.c:497)
// ---------------------------------------------------------------------------
// The recurrence coefficients of eqs. (26)-(28) are rewritten so that every
// factor that depends on p alone comes from tables (per task: the integer
// products K0..K3 of p, p1=p-2m, p2=p+2m; per batch: x^2 and 1/(4x^2-1)),
// the common factor Ap cancels, and alpha(p+3), alpha(p+4) are carried over
// from the previous step.  One division per step remains.  log n! comes from
// a table covering every argument of the batch.
// per task, for p in [0, pstride): the p-dependent factors of the recurrence with the
// alpha denominators 1/(4x^2-1) folded in.  Table 0 (l1 != l2, eqs. (26)-(27)):
//   {K0/(4(p+1)^2-1), K1/(4(p+2)^2-1), K2/(4(p+3)^2-1), K3/(4(p+4)^2-1)},
//   K0=(p+2)(p+3)(p1+1)(p1+2), K1=(p+1)(p+3)(p1+2)(p2+2), K2=(p+2)(p+4)(p1+3)(p2+3), K3=(p+2)(p+3)(p2+3)(p2+4);
// table 1 (l1 == l2, eq. (30)): {(p+2)(p1+1)/(4(p+1)^2-1), (p+1)(p2+2)/(4(p+2)^2-1), 0, 0};
// p1 = p-2m, p2 = p+2m.
// the q recurrence coefficients of degree index p for one m (they depend on m alone)
CAPS_DEV void ptab_entry(int mt, int p, double4 *tm, double4 *tp, float4 *fm, float4 *fp)
{
    const double m = mt > 0 ? mt : 1;
    const double pp = p, p1 = pp - 2 * m, p2 = pp + 2 * m;
    auto invD = [](double x) { return 1.0 / (4 * x * x - 1); };
    const double4 v0 = make_double4((pp + 2) * (pp + 3) * ((p1 + 1) * (p1 + 2)) * invD(pp + 1),
                                    (pp + 1) * (pp + 3) * ((p1 + 2) * (p2 + 2)) * invD(pp + 2),
                                    (pp + 2) * (pp + 4) * ((p1 + 3) * (p2 + 3)) * invD(pp + 3),
                                    (pp + 2) * (pp + 3) * ((p2 + 3) * (p2 + 4)) * invD(pp + 4));
    const double4 v1 = make_double4((pp + 2) * (p1 + 1) * invD(pp + 1), (pp + 1) * (p2 + 2) * invD(pp + 2), 0.0, 0.0);
    if (tm) { *tm = v0; *tp = v1; }
    if (fm) {
        const double s = 0x1p-30;
        for (int t = 0; t < 2; t++) {
            const double4 v = t ? v1 : v0;
            const ff x = ff_from_d(v.x * s), y = ff_from_d(v.y * s), z = ff_from_d(v.z * s), w = ff_from_d(v.w * s);
            float4 *f = t ? fp : fm;
            f[0] = make_float4(x.h, y.h, z.h, w.h);
            f[1] = make_float4(x.l, y.l, z.l, w.l);
        }
    }
}

__global__ void k_ptab(const Task *tasks, int ntask, double4 *ptab, float4 *ptabf, int pstride)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int task = blockIdx.y;
    if (p >= pstride || task >= ntask) return;
    ptab_entry(tasks[task].m, p, ptab + ((size_t)task * 2 + 0) * pstride + p, ptab + ((size_t)task * 2 + 1) * pstride + p,
               ptabf ? ptabf + (((size_t)task * 2 + 0) * pstride + p) * 2 : nullptr,
               ptabf ? ptabf + (((size_t)task * 2 + 1) * pstride + p) * 2 : nullptr);
}

// the float-float tables once per distinct m of a chunk (groups), indexed like the a_0..a_2 rows
__global__ void k_ptab_groups(const int *group_m, int ngroup, float4 *ptabf, int pstride)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int g = blockIdx.y;
    if (p >= pstride || g >= ngroup) return;
    ptab_entry(group_m[g], p, nullptr, nullptr, ptabf + (((size_t)g * 2 + 0) * pstride + p) * 2,
               ptabf + (((size_t)g * 2 + 1) * pstride + p) * 2);
}

// per distinct m of a chunk and per (l1>=l2) pair: a_0 (as a scaled double), a_1,
// a_2 of the q-sum (eqs. (20), (29), (35)) -- they depend on (l1, l2, m) but not on
// xi, so every frequency with the same m shares them.  Evaluated with the
// reference's formulas and order of operations: the m=0 q-sums cancel strongly
// and the reference's results carry exactly this rounding of a_2.

__global__ void k_a12(const int *group_m, const int *group_lmin, int ngroup, int ldim, const double *__restrict__ lft, A012 *tab)
{
    const int L = ldim + 2;
    const long long npair = (long long)L * (L + 1) / 2;
    const long long pid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int g = blockIdx.y;
    if (pid >= npair || g >= ngroup) return;
    int a1 = (int)((sqrt(8.0 * (double)pid + 1.0) - 1.0) * 0.5);
    while ((long long)(a1 + 1) * (a1 + 2) / 2 <= pid) a1++;
    while ((long long)a1 * (a1 + 1) / 2 > pid) a1--;
    const int a2 = (int)(pid - (long long)a1 * (a1 + 1) / 2);
    tab[(size_t)g * npair + pid] = a012_pair(group_m[g], group_lmin[g], a1, a2, lft);
}

// Mixed form: the same a_0, a_1, a_2 from O(L) tables per m.  With m' = max(m, 1),
// s = 2(l1 + l2), n4 = l1 + l2 - 2m',
//   F1(l) = (m'-l)(m'-l+1)/(2l-1),   F2(l) = F1(l) (m'-l+2)(m'-l+3)/(2l-3),
//   a_1 = (l1 + l2 - 3/2)(1 - (s-1)/(n4(n4-1)) (F1(l1) + F1(l2))),
//   a_2 = (s-1)(s-7)/4 ((s-3)/(n4(n4-1)) ((s-5)/(2(n4-2)(n4-3)) (F2(l1) + 2 F1(l1) F1(l2) + F2(l2))
//         - F1(l1) - F1(l2)) + 1/2),
//   a_0 = e^G(l1) e^G(l2) e^H(l1+l2),  G(l) = lfac(2l) - lfac(l) - lfac(l-m'),
//         H(j) = lfac(j) - lfac(2j) + lfac(j-2m'),
// which is k_a12's expression regrouped: every division and the exponential move into
// per-l and per-(l1+l2) tables, and a pair costs a few FP64 products.  The rounding
// differs from the reference's at the ulp level, far below the mixed form's 2^-44; the
// FP64 form keeps k_a12.  The mixed table is written as float-float (A012F), so the
// q-sum kernel needs no FP64 instruction.
// per-m tables of the mixed form, formed in FP64 and stored as float-float
CAPS_DEV ffe ffe_from_sd(sd v)
{
    if (v.m == 0.0) return ffe{0.0f, 0.0f, FFE_ZERO_E, 0};
    const ff x = ff_from_d(v.m);
    return ffe{x.h, x.l, v.e, 0};
}

// grid (ceil((2L-1)/128), ngroup)
__global__ void k_a12_tabs(const int *group_m, const int *group_lmin, int ngroup, int ldim, const double *__restrict__ lft,
                           A12L *tl, A12J *tj)
{
    const int L = ldim + 2, NJ = 2 * L - 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x, g = blockIdx.y;
    if (g >= ngroup || i >= NJ) return;
    const int mt = group_m[g], mm = mt > 0 ? mt : 1, l0 = group_lmin[g] - 1;
    const double m = mm;
    if (i < L) {
        const int l = l0 + i;
        const double dl = l, u = m - dl;
        const double F1 = u * (u + 1) / (2 * dl - 1);
        sd eG{0.0, 0};
        if (l >= mm) eG = sd_from_log(__ldg(lft + 2 * l) - __ldg(lft + l) - __ldg(lft + l - mm), 1);
        tl[(size_t)g * L + i] = A12L{ff_from_d(F1), ff_from_d(F1 * (u + 2) * (u + 3) / (2 * dl - 3)), ffe_from_sd(eG)};
    }
    const int j = 2 * l0 + i, n4 = j - 2 * mm;
    const double s = 2.0 * j, q = (double)n4 * (n4 - 1);
    double h1 = 0.0, pb = 0.0, pc = 0.0;
    sd eH{0.0, 0};
    if (n4 >= 2) { h1 = (s - 1) / q; pb = (s - 3) / q; }
    if (n4 >= 4) pc = (s - 5) / (2.0 * (n4 - 2) * (n4 - 3));
    if (n4 >= 0) eH = sd_from_log(__ldg(lft + j) - __ldg(lft + 2 * j) + __ldg(lft + n4), 1);
    tj[(size_t)g * NJ + i] = A12J{ff_from_d(h1), ff_from_d((s - 1) * (s - 7) / 4), ff_from_d(pb), ff_from_d(pc), ffe_from_sd(eH)};
}

// grid (ceil(npair/128), nlist); block row y fills group glist[y] (glist == nullptr: y)
__global__ void k_a12_mix(const int *group_m, const int *group_lmin, const int *glist, int nlist, int ldim, const A12L *__restrict__ tl,
                          const A12J *__restrict__ tj, A012F *tab)
{
    const int L = ldim + 2, NJ = 2 * L - 1;
    const long long npair = (long long)L * (L + 1) / 2;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((int)blockIdx.y >= nlist || tid >= npair) return;
    const int g = glist ? glist[blockIdx.y] : (int)blockIdx.y;
    const long long pid = tid;
    int a1 = (int)((sqrtf(8.0f * (float)pid + 1.0f) - 1.0f) * 0.5f);
    while ((long long)(a1 + 1) * (a1 + 2) / 2 <= pid) a1++;
    while ((long long)a1 * (a1 + 1) / 2 > pid) a1--;
    const int a2 = (int)(pid - (long long)a1 * (a1 + 1) / 2);
    const A012F r = a012f_pair(group_m[g], group_lmin[g], a1, a2, tl + (size_t)g * L, tj + (size_t)g * NJ);
    tab[(size_t)g * npair + pid] = r;
}

// grid (ceil(npair/128), nlist) or, for the band, (ceil(2L/128), nlist); block row y handles
// task tlist[y] (tlist == nullptr: task y).  BAND computes only the pairs that the
// diagonal of M reads (l1 - l2 in {0, 2}), each with the sum the full kernel forms.
template <bool BAND>
__global__ void __launch_bounds__(128) k_itab(const Task *tasks, const int *tlist, int nlist, int ldim, const sd *K, int nu_stride,
                                              const double *__restrict__ lft, const double2 *__restrict__ xtab,
                                              const double4 *__restrict__ ptab, int pstride, sd *I, int *status,
                                              const A012 *__restrict__ a12)
{
    const int L = ldim + 2;
    const long long npair = (long long)L * (L + 1) / 2;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if ((int)blockIdx.y >= nlist) return;
    const int task = tlist ? tlist[blockIdx.y] : (int)blockIdx.y;
    long long pid;
    int a1, a2;
    if (BAND) {
        // thread 2 a2 + d owns the pair (a2 + 2 d, a2)
        if (tid >= 2LL * L) return;
        a2 = (int)(tid >> 1);
        a1 = a2 + 2 * (int)(tid & 1);
        if (a1 >= L) return;
        pid = (long long)a1 * (a1 + 1) / 2 + a2;
    } else {
        if (tid >= npair) return;
        pid = tid;
        // pair index -> (a1 >= a2)
        a1 = (int)((sqrt(8.0 * (double)pid + 1.0) - 1.0) * 0.5);
        while ((long long)(a1 + 1) * (a1 + 2) / 2 <= pid) a1++;
        while ((long long)a1 * (a1 + 1) / 2 > pid) a1--;
        a2 = (int)(pid - (long long)a1 * (a1 + 1) / 2);
    }

    const Task &T = tasks[task];
    const int l1 = T.lmin - 1 + a1, l2 = T.lmin - 1 + a2;
    const int mm = T.m > 0 ? T.m : 1;
    sd *I_TM = I + (size_t)(task * 2 + 1) * L * L;
    sd *I_TE = I + (size_t)(task * 2 + 0) * L * L;
    const size_t o12 = (size_t)a1 * L + a2, o21 = (size_t)a2 * L + a1;
    if (l2 < mm || l2 < T.m || l1 < 1) { // I = 0 for l < m (integration.c:631)
        I_TM[o12] = I_TM[o21] = sd{0, 0};
        I_TE[o12] = I_TE[o21] = sd{0, 0};
        return;
    }
    sd rT, rE;
    if (qsum_pair(T, l1, l2, a12[(size_t)T.mgroup * npair + pid], K + (size_t)(task * 2 + 1) * nu_stride - T.mu,
                  K + (size_t)(task * 2 + 0) * nu_stride - T.mu, ptab + (size_t)task * 2 * pstride, pstride, rT, rE))
        atomicOr(status + task, ST_ERR_NONFINITE);
    I_TM[o12] = rT; I_TM[o21] = rT;
    I_TE[o12] = rE; I_TE[o21] = rE;
}

// per batch: log n! for n < nlf (table below 1024, Stirling above) and
// x^2, 1/(4x^2-1) for x < nx
__global__ void k_tables(const double *lfac_tab, double *lft, int nlf, double2 *xtab, int nx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nlf) lft[i] = lfac(lfac_tab, i);
    if (i < nx) { const double x = i; xtab[i] = make_double2(x * x, 1.0 / (4 * x * x - 1)); }
}

// ---------------------------------------------------------------------------
// elements of 1 - M (lower triangle, column-major, leading dimension lda)
// ---------------------------------------------------------------------------

// A = 1 - M (lower triangle); mdiag receives M_ii itself, so that the trace keeps its
// relative precision when M_ii is far below the unit diagonal of A.  Grid (ceil(ldim/128),
// ldim, nlist), block z on task tlist[z] (tlist == nullptr: task z).  DIAG: grid
// (ceil(ldim/128), 1, nlist), M_ii alone into mdiag (A untouched), from the band of I
// values that k_itab<true> leaves; the same arithmetic as the full assembly.
template <bool DIAG>
__global__ void k_elem(const Task *tasks, const int *tlist, int nlist, int ldim, const sd *I, const sd *Sa, const sd *Sb,
                       const double2 *uv, double *A, size_t lda, size_t mat_stride, double *mdiag, int *status)
{
    const int L = ldim + 2;
    const int a = blockIdx.x * blockDim.x + threadIdx.x; // row block
    const int b = DIAG ? a : (int)blockIdx.y;           // column block
    if (a >= ldim || b > a || (int)blockIdx.z >= nlist) return;
    const int task = tlist ? tlist[blockIdx.z] : (int)blockIdx.z;
    const Task &T = tasks[task];
    const sd *ITM = I + (size_t)(task * 2 + 1) * L * L;
    const sd *ITE = I + (size_t)(task * 2 + 0) * L * L;
    const int i1 = a + 1, i2 = b + 1; // index into [lmin-1, lmin+ldim]
    const size_t so = (size_t)task * L;
    const sd sa1 = Sa[so + i1], sa2 = Sa[so + i2], sb1 = Sb[so + i1], sb2 = Sb[so + i2];
    const double2 uv1 = uv[so + i1], uv2 = uv[so + i2];
    // the table is symmetric; I(x, y) is read at t[y L + x] so that consecutive threads
    // (consecutive x) read consecutive entries
    auto Iv = [&](int p, int x, int y) { return (p ? ITM : ITE)[(size_t)y * L + x]; };
    sd EE, MM, EM, ME;
    elem_block<DIAG>(T.m, i1, i2, sa1, sa2, sb1, sb2, uv1, uv2, Iv, EE, MM, EM, ME);
    if (DIAG) {
        const double ee = sd_to_double(EE), mm = sd_to_double(MM);
        if (!isfinite(ee) || !isfinite(mm)) atomicOr(status + task, ST_ERR_NONFINITE);
        mdiag[(size_t)task * 2 * ldim + 2 * a] = ee;
        mdiag[(size_t)task * 2 * ldim + 2 * a + 1] = mm;
        return;
    }
    double *Am = A + (size_t)task * mat_stride;
    const int r0 = 2 * a, c0 = 2 * b;
    const double ee = sd_to_double(EE), mm = sd_to_double(MM), me = sd_to_double(ME), em = sd_to_double(EM);
    if (!isfinite(ee) || !isfinite(mm) || !isfinite(me) || !isfinite(em)) atomicOr(status + task, ST_ERR_NONFINITE);
    Am[(size_t)c0 * lda + r0] = (a == b ? 1.0 : 0.0) - ee;
    Am[(size_t)c0 * lda + r0 + 1] = -me;
    Am[(size_t)(c0 + 1) * lda + r0 + 1] = (a == b ? 1.0 : 0.0) - mm;
    if (a != b) Am[(size_t)(c0 + 1) * lda + r0] = -em;
    else {
        mdiag[(size_t)task * 2 * ldim + r0] = ee;
        mdiag[(size_t)task * 2 * ldim + r0 + 1] = mm;
    }
}

// ---------------------------------------------------------------------------
// trace / Frobenius norm / shortcut decision (one block per task)
// ---------------------------------------------------------------------------
// mode: 0 = dense semantics (trace + Mercator shortcut), 1 = HODLR semantics
// (trace shortcut only; |tr| > |logdet| checked after the factorisation).
// trace and Frobenius norm of M from its strict lower triangle (-A) and its diagonal
// M_ii (mdiag, n per task), as the reference takes them from the elements of M
// (matrix.c:57-119): 1 - A_ii would lose every M_ii below the rounding of 1
// One block per listed task (tlist[x], or x without a list).  A == nullptr: the trace rule
// alone; a task it does not decide keeps status 0, to be assembled in full.
__global__ void k_stats(const int *tlist, int nlist, int n, const double *A, size_t lda, size_t mat_stride, int mode,
                        const double *mdiag, double *trace_out, double *result, int *status)
{
    if ((int)blockIdx.x >= nlist) return;
    const int task = tlist ? tlist[blockIdx.x] : (int)blockIdx.x;
    __shared__ double red[256];
    if (A) {
        const double *Am = A + (size_t)task * mat_stride;
        double s = 0.0;
        // sum of squares of M: diagonal once, strict lower twice (M is symmetric)
        for (int j = 0; j < n; j++) {
            const double *col = Am + (size_t)j * lda;
            for (int i = j + threadIdx.x; i < n; i += blockDim.x) {
                const double v = (i == j) ? mdiag[(size_t)task * n + i] : -col[i];
                s += (i == j ? 1.0 : 2.0) * v * v;
            }
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
    }
    if (threadIdx.x != 0) return;
    // Kahan trace in index order (misc.c:26)
    double tr = 0.0, c = 0.0;
    for (int i = 0; i < n; i++) {
        const double y = mdiag[(size_t)task * n + i] - c;
        const double t = tr + y;
        c = (t - tr) - y;
        tr = t;
    }
    trace_out[task] = tr;
    if (status[task] & ~0xF) { result[task] = NAN; return; }
    if (fabs(tr) < 1e-8) { result[task] = -tr; status[task] = ST_TRACE; return; }
    if (!A) return;
    const double fro2 = red[0], fro = sqrt(fro2);
    if (mode == 0 && fro < 1) {
        const double merc = -tr - fro2 / 2;
        const double err = fabs(fro2 / 2 + fro + log1p(-fro));
        if (fabs(err / merc) < 1e-8) { result[task] = merc; status[task] = ST_MERCATOR; return; }
    }
    status[task] = ST_FACTOR;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
void launch_setup(Task *tasks, int ntask, double *edges, int max_panels, double2 *coefAB, int nu_stride, double c_width,
                  int *status, cudaStream_t st)
{
    k_setup<<<ntask, 256, 0, st>>>(tasks, ntask, edges, max_panels, coefAB, nu_stride, c_width, status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_mie(const double *xi, const double *epsm1, int nxi, double LbyR, int lmax, double *lna, double *lnb, cudaStream_t st)
{
    dim3 g((lmax + 127) / 128, nxi);
    k_mie<<<g, 128, 0, st>>>(xi, epsm1, nxi, LbyR, lmax, lna, lnb);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_scale(const Task *tasks, int ntask, int ldim, const double *lna, const double *lnb, int lmax, const double *lfac_tab,
                  sd *Sa, sd *Sb, double2 *uv, cudaStream_t st)
{
    dim3 g((ldim + 2 + 127) / 128, ntask);
    k_scale<<<g, 128, 0, st>>>(tasks, ntask, ldim, lna, lnb, lmax, lfac_tab, Sa, Sb, uv);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

size_t ktab_smem_bytes() { return (size_t)KT_WARPS * (32 * 33 + 64) * sizeof(double) + KT_WARPS * 32 * sizeof(int); }

void launch_ktab(bool pr, const Task *tasks, int ntask, int max_warps, const double *edges, int max_panels, const double2 *coefAB,
                 int nu_stride, const double *lfac_tab, double *partM, int *partE, cudaStream_t st)
{
    static bool attr_set = false;
    const size_t sm = ktab_smem_bytes();
    if (!attr_set) {
        CK(cudaFuncSetAttribute(k_ktab<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        CK(cudaFuncSetAttribute(k_ktab<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        attr_set = true;
    }
    dim3 g((max_warps + KT_WARPS - 1) / KT_WARPS, ntask);
    if (pr) k_ktab<true><<<g, KT_WARPS * 32, sm, st>>>(tasks, edges, max_panels, coefAB, nu_stride, lfac_tab, partM, partE, max_warps);
    else k_ktab<false><<<g, KT_WARPS * 32, sm, st>>>(tasks, edges, max_panels, coefAB, nu_stride, lfac_tab, partM, partE, max_warps);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_kred(const Task *tasks, int ntask, int max_nnu, const double *partM, const int *partE, int max_warps, int nu_stride,
                 sd *K, int *status, cudaStream_t st)
{
    dim3 g((max_nnu + 127) / 128, ntask);
    k_kred<<<g, 128, 0, st>>>(tasks, ntask, partM, partE, max_warps, nu_stride, K, status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_tables(const double *lfac_tab, double *lft, int nlf, double2 *xtab, int nx, cudaStream_t st)
{
    const int n = nlf > nx ? nlf : nx;
    k_tables<<<(n + 255) / 256, 256, 0, st>>>(lfac_tab, lft, nlf, xtab, nx);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_a12(const int *group_m, const int *group_lmin, int ngroup, int ldim, const double *lft, void *tab, cudaStream_t st)
{
    const long long L = ldim + 2, npair = L * (L + 1) / 2;
    dim3 g((unsigned)((npair + 127) / 128), ngroup);
    k_a12<<<g, 128, 0, st>>>(group_m, group_lmin, ngroup, ldim, lft, (A012 *)tab);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

size_t a12_tab_bytes(int ldim, int ngroup)
{
    const size_t L = ldim + 2;
    return (L * sizeof(A12L) + (2 * L - 1) * sizeof(A12J)) * ngroup;
}

void launch_a12_mixed(const int *group_m, const int *group_lmin, int ngroup, int ldim, const double *lft, void *tab, void *work,
                      cudaStream_t st, bool tabs, const int *glist, int nlist)
{
    const long long L = ldim + 2, npair = L * (L + 1) / 2;
    A12L *tl = (A12L *)work;
    A12J *tj = (A12J *)((char *)work + (size_t)L * ngroup * sizeof(A12L));
    if (tabs) {
        dim3 gt((unsigned)((2 * L - 1 + 127) / 128), ngroup);
        k_a12_tabs<<<gt, 128, 0, st>>>(group_m, group_lmin, ngroup, ldim, lft, tl, tj);
        COUNT_LAUNCH(1);
    }
    if (nlist < 0) nlist = ngroup;
    if (nlist > 0) {
        dim3 g((unsigned)((npair + 127) / 128), nlist);
        k_a12_mix<<<g, 128, 0, st>>>(group_m, group_lmin, glist, nlist, ldim, tl, tj, (A012F *)tab);
        COUNT_LAUNCH(1);
    }
    CK(cudaGetLastError());
}

size_t a12_bytes(int ldim, int ngroup)
{
    const size_t L = ldim + 2;
    return L * (L + 1) / 2 * ngroup * sizeof(A012);
}

void launch_ptab_groups(const int *group_m, int ngroup, float4 *ptabf, int pstride, cudaStream_t st)
{
    dim3 gp((pstride + 127) / 128, ngroup);
    k_ptab_groups<<<gp, 128, 0, st>>>(group_m, ngroup, ptabf, pstride);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_ktab_ff(bool pr, const Task *tasks, int ntask, int max_warps, const double *edges, int max_panels, const double2 *coefAB,
                    float4 *coefF, int nu_stride, const double *lfac_tab, float2 *partF, int *partE, cudaStream_t st)
{
    static bool attr_set = false;
    const size_t sm = ktab_smem_bytes();
    if (!attr_set) {
        CK(cudaFuncSetAttribute(k_ktab_ff<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        CK(cudaFuncSetAttribute(k_ktab_ff<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        attr_set = true;
    }
    dim3 gc((nu_stride + 127) / 128, ntask);
    k_coef_ff<<<gc, 128, 0, st>>>(ntask, nu_stride, coefAB, coefF);
    dim3 g((max_warps + KT_WARPS - 1) / KT_WARPS, ntask);
    if (pr) k_ktab_ff<true><<<g, KT_WARPS * 32, sm, st>>>(tasks, edges, max_panels, coefF, nu_stride, lfac_tab, partF, partE, max_warps);
    else k_ktab_ff<false><<<g, KT_WARPS * 32, sm, st>>>(tasks, edges, max_panels, coefF, nu_stride, lfac_tab, partF, partE, max_warps);
    COUNT_LAUNCH(2);
    CK(cudaGetLastError());
}

void launch_kred_ff(const Task *tasks, int ntask, int max_nnu, const float2 *partF, const int *partE, int max_warps, int nu_stride,
                    float4 *KP, int *KPe, int *status, cudaStream_t st)
{
    dim3 g((max_nnu + 127) / 128, ntask);
    k_kred_ff<<<g, 128, 0, st>>>(tasks, ntask, partF, partE, max_warps, nu_stride, KP, KPe, status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_ptab(const Task *tasks, int ntask, double4 *ptab, int pstride, cudaStream_t st)
{
    dim3 gp((pstride + 127) / 128, ntask);
    k_ptab<<<gp, 128, 0, st>>>(tasks, ntask, ptab, nullptr, pstride);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_itab(const Task *tasks, const int *tlist, int nlist, int ldim, const sd *K, int nu_stride, const double *lft,
                 const double2 *xtab, const double4 *ptab, int pstride, sd *I, int *status, cudaStream_t st, const void *a12,
                 bool band)
{
    if (nlist <= 0) return;
    const long long L = ldim + 2, npair = L * (L + 1) / 2;
    dim3 g((unsigned)(((band ? 2 * L : npair) + 127) / 128), nlist);
    if (band)
        k_itab<true><<<g, 128, 0, st>>>(tasks, tlist, nlist, ldim, K, nu_stride, lft, xtab, ptab, pstride, I, status,
                                        (const A012 *)a12);
    else
        k_itab<false><<<g, 128, 0, st>>>(tasks, tlist, nlist, ldim, K, nu_stride, lft, xtab, ptab, pstride, I, status,
                                         (const A012 *)a12);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_elem(const Task *tasks, const int *tlist, int nlist, int ldim, const sd *I, const sd *Sa, const sd *Sb, const double2 *uv,
                 double *A, size_t lda, size_t mat_stride, double *mdiag, int *status, cudaStream_t st, bool diag_only)
{
    if (nlist <= 0) return;
    if (diag_only) {
        dim3 g((ldim + 127) / 128, 1, nlist);
        k_elem<true><<<g, 128, 0, st>>>(tasks, tlist, nlist, ldim, I, Sa, Sb, uv, A, lda, mat_stride, mdiag, status);
    } else {
        dim3 g((ldim + 127) / 128, ldim, nlist);
        k_elem<false><<<g, 128, 0, st>>>(tasks, tlist, nlist, ldim, I, Sa, Sb, uv, A, lda, mat_stride, mdiag, status);
    }
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_stats(const int *tlist, int nlist, int n, const double *A, size_t lda, size_t mat_stride, const double *mdiag, int mode,
                  double *trace, double *result, int *status, cudaStream_t st)
{
    if (nlist <= 0) return;
    k_stats<<<nlist, 256, 0, st>>>(tlist, nlist, n, A, lda, mat_stride, mode, mdiag, trace, result, status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
