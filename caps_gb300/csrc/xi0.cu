// xi0.cu -- the xi = 0 blocks: closed-form EE/MM elements and the plasma-model MM
// block (libcaps.c:860-928), assembled on the GPU and factored by the same batched
// Cholesky (caps_logdetD0, libcaps.c:985); the plasma integrals I_nu
// (integration.c:897-1031) by a fixed composite Gauss-Legendre rule on the GPU.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/libcaps.h"
#include "internal.h"
#include "special.cuh"

namespace capsgpu {

struct GL16 { double x[16], w[16]; };

// Gauss-Legendre nodes and weights on [-1,1] (Newton iteration on P_16)
static GL16 gl16()
{
    GL16 g;
    const int n = 16;
    for (int i = 0; i < n; i++) {
        double z = cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 1;
        for (int it = 0; it < 100; it++) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; j++) { const double p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
            pp = n * (z * p1 - p2) / (z * z - 1);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-16) break;
        }
        g.x[i] = z;
        g.w[i] = 2 / ((1 - z * z) * pp * pp);
    }
    return g;
}

// I_nu = int_0^inf dt (-r_TE) e^{-t} t^nu / nu!, -r_TE = b/(2+b), b = sqrt(1+(2w/t)^2) - 1
// (integration.c:921-1013), for nu = nu_lo .. nu_lo+nnu-1; one warp per nu.
// The weight t^nu e^{-t}/nu! peaks at t = nu with width sigma = sqrt(nu); -r_TE is
// analytic for t > 0 with its nearest singularities at t = +-2iw.  Panels cover
// [max(0, nu-14 sigma-10), nu+14 sigma+30] (the weight outside is below e^-90), are at
// most sigma/3 wide, and near t = 0 grow geometrically from 2w/8 (width <= t), so
// that every panel sees the singularity at >= 3 half-widths: GL-16 per panel then
// converges to rounding.  Lanes 0-15 take the nodes of one panel and 16-31 of the
// next; the warp sum is in a fixed order.
__global__ void k_plasma_I(int nu_lo, int nnu, double w, const double *lfac_tab, GL16 gl, double *I)
{
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= nnu) return;
    const int nu = nu_lo + warp;
    const double sigma = fmax(1.0, sqrt((double)nu));
    const double t_lo = fmax(0.0, nu - 14 * sigma - 10), t_hi = nu + 14 * sigma + 30;
    const double hmax = sigma / 3, hmin = fmax(0.25 * w, 1e-6 * hmax);
    const double lpre = -lfac(lfac_tab, nu);
    auto width = [&](double t) { return fmin(hmax, fmax(t, hmin)); };
    const int k = lane & 15;
    double acc = 0;
    double t = t_lo;
    for (int guard = 0; t < t_hi && guard < 1 << 20; guard++) {
        const double b0 = fmin(t + width(t), t_hi);
        const double b1 = b0 < t_hi ? fmin(b0 + width(b0), t_hi) : b0;
        const double lo = lane < 16 ? t : b0, hi = lane < 16 ? b0 : b1;
        if (hi > lo) {
            const double h = 0.5 * (hi - lo), x = 0.5 * (hi + lo) + h * gl.x[k];
            const double s = 2 * w / x, s2 = s * s;
            const double bm1 = s2 / (sqrt(1 + s2) + 1);
            acc += gl.w[k] * h * (bm1 / (2 + bm1)) * exp(lpre - x + nu * log(x));
        }
        t = b1;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) I[warp] = acc;
}

// ratio[l] = I_{l-1/2}(alpha)/I_{l+1/2}(alpha) and f[l] = 1 - (2l+1)/(alpha ratio[l])
// for l = 1 .. lmax (libcaps.c:897-900)
__global__ void k_plasma_ratio(int lmax, double alpha, double *ratio, double *f)
{
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l > lmax) return;
    if (l == 0) { ratio[0] = f[0] = NAN; return; }
    const double r = ratioI(l - 0.5, alpha);
    ratio[l] = r;
    f[l] = 1 - (2 * l + 1.) / (alpha * r);
}

// M0_EE(l1,l2) = exp((l1+l2+1) y + lfac(l1+l2) - (lfac(l1+m)+lfac(l1-m)+lfac(l2+m)+lfac(l2-m))/2)
// M0_MM = M0_EE sqrt(l1 l2 / ((l1+1)(l2+1)))
// M0_MM_plasma = sqrt(l1 f1/(l1+1) l2 f2/(l2+1)) exp(lfac(l1+l2) - (...)/2 + (l1+l2+1) y) I_{l1+l2}
__global__ void k_elem0(const int *ms, const int *lmins, int ntask, int ldim, double y, int which, const double *lfac_tab,
                        const double *Itab, const double *ftab, double *A, size_t mstride, double *mdiag, int *status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const int task = blockIdx.z;
    if (i >= ldim || j > i || task >= ntask) return;
    const int m = ms[task], l1 = i + lmins[task], l2 = j + lmins[task];
    double v;
    if (which == 2) {
        const double factor = sqrt(l1 * ftab[l1] / (l1 + 1.) * l2 * ftab[l2] / (l2 + 1.));
        v = factor * exp(lfac(lfac_tab, l1 + l2) - 0.5 * (lfac(lfac_tab, l1 + m) + lfac(lfac_tab, l1 - m) + lfac(lfac_tab, l2 + m)
                                                           + lfac(lfac_tab, l2 - m)) + (l1 + l2 + 1) * y) * Itab[l1 + l2];
    } else {
        v = exp((l1 + l2 + 1) * y + lfac(lfac_tab, l1 + l2)
                - 0.5 * (lfac(lfac_tab, l1 + m) + lfac(lfac_tab, l1 - m) + lfac(lfac_tab, l2 + m) + lfac(lfac_tab, l2 - m)));
        if (which == 1) v *= sqrt(((double)l1 * l2) / ((l1 + 1.) * (l2 + 1.)));
    }
    if (!isfinite(v)) atomicOr(status + task, ST_ERR_NONFINITE);
    A[(size_t)task * mstride + (size_t)j * ldim + i] = (i == j ? 1.0 : 0.0) - v;
    if (i == j) mdiag[(size_t)task * ldim + i] = v;
}

static double *lfac_table_device()
{
    static double *d_lfac = nullptr;
    if (!d_lfac) {
        double tab[1024];
        for (int k = 0; k < 1024; k++) tab[k] = lgamma(k + 1.0);
        CK(cudaMalloc(&d_lfac, sizeof tab));
        CK(cudaMemcpy(d_lfac, tab, sizeof tab, cudaMemcpyHostToDevice));
    }
    return d_lfac;
}

// grow-only device buffers of the xi = 0 path, reused by every call; g_xi0_mu serialises
// the calls that use them (the free energy calls the batch once per chunk of m)
struct Xi0Buf {
    void *p = nullptr;
    size_t bytes = 0;
    template <class T> T *get(size_t count)
    {
        const size_t need = count * sizeof(T);
        if (need > bytes) {
            if (p) CK(cudaFree(p));
            bytes = std::max(need, bytes + bytes / 4);
            CK(cudaMalloc(&p, bytes));
        }
        return (T *)p;
    }
};
static struct { Xi0Buf I, ratio, f, m, lmin, status, A, ld, md, tr, res; } g_x0;
static std::mutex g_xi0_mu;

// I_nu for nu = 0 .. numax and ratio_l, f_l for l = 0 .. lmax of the plasma xi=0 block,
// in the path's workspace (valid until the next call); omegap_ = omegap (L+R)/c,
// alpha = omegap_/(1+L/R)
static void plasma_tables_device(double omegap_, double alpha, int numax, int lmax, double **dI, double **dratio, double **df)
{
    *dI = g_x0.I.get<double>((size_t)numax + 1);
    *dratio = g_x0.ratio.get<double>((size_t)lmax + 1);
    *df = g_x0.f.get<double>((size_t)lmax + 1);
    const int nnu = numax + 1;
    k_plasma_I<<<(nnu + 3) / 4, 128>>>(0, nnu, omegap_, lfac_table_device(), gl16(), *dI);
    COUNT_LAUNCH(1);
    k_plasma_ratio<<<(lmax + 1 + 127) / 128, 128>>>(lmax, alpha, *dratio, *df);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu

using namespace capsgpu;

// implemented in libcaps.cu
struct Engine;

// which: 0 EE, 1 MM (perfect reflector), 2 MM of the plasma model with plasma frequency
// omegap (rad/s)
int logdetD0_batch(caps_t *self, const int *ms, int n, int which, double *out, double omegap)
{
    std::lock_guard<std::mutex> lk(g_xi0_mu);
    double *d_lfac = lfac_table_device();
    const int ldim = self->ldim;
    std::vector<int> lmins(n);
    int lmax = 1;
    for (int k = 0; k < n; k++) {
        size_t lo, hi;
        caps_estimate_lminmax(self, ms[k], &lo, &hi);
        lmins[k] = (int)lo;
        lmax = std::max(lmax, lmins[k] + ldim - 1);
    }
    double *d_I = nullptr, *d_ratio = nullptr, *d_f = nullptr;
    if (which == 2) {
        const double omegap_ = omegap * self->calL / CAPS_c;
        plasma_tables_device(omegap_, omegap_ / (1 + self->LbyR), 2 * lmax, lmax, &d_I, &d_ratio, &d_f);
    }
    const size_t mstride = (size_t)ldim * ldim;
    int *d_m = g_x0.m.get<int>(n), *d_lmin = g_x0.lmin.get<int>(n), *d_status = g_x0.status.get<int>(n);
    double *d_A = g_x0.A.get<double>(n * mstride);
    double *d_ld = g_x0.ld.get<double>((size_t)n * ldim), *d_md = g_x0.md.get<double>((size_t)n * ldim);
    double *d_tr = g_x0.tr.get<double>(n), *d_res = g_x0.res.get<double>(n);
    cudaStream_t st = 0;
    CK(cudaMemcpy(d_m, ms, n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_lmin, lmins.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemset(d_status, 0, n * sizeof(int)));
    dim3 g((ldim + 127) / 128, ldim, n);
    k_elem0<<<g, 128, 0, st>>>(d_m, d_lmin, n, ldim, self->y, which, d_lfac, d_I, d_f, d_A, mstride, d_md, d_status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
    const int mode = self->detalg == DETALG_HODLR ? 1 : 0;
    launch_stats(nullptr, n, ldim, d_A, ldim, mstride, d_md, mode, d_tr, d_res, d_status, st);
    launch_cholesky(n, ldim, d_A, ldim, mstride, d_status, d_ld, st);
    launch_final(n, ldim, d_ld, d_tr, d_status, d_res, mode, st);
    std::vector<int> hs(n);
    CK(cudaMemcpy(out, d_res, n * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hs.data(), d_status, n * sizeof(int), cudaMemcpyDeviceToHost));
    int nerr = 0;
    for (int k = 0; k < n; k++) nerr += (hs[k] & ~0xF) != 0;
    return nerr;
}

// host copies of the plasma tables for the element-wise interface
// (caps_integrate_plasma, caps_kernel_M0_MM_plasma)
void plasma_tables_host(double omegap_, double alpha, int numax, int lmax, std::vector<double> &I, std::vector<double> &ratio)
{
    std::lock_guard<std::mutex> lk(g_xi0_mu);
    double *d_I, *d_ratio, *d_f;
    plasma_tables_device(omegap_, alpha, numax, lmax, &d_I, &d_ratio, &d_f);
    I.resize(numax + 1);
    ratio.resize(lmax + 1);
    CK(cudaMemcpy(I.data(), d_I, I.size() * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(ratio.data(), d_ratio, ratio.size() * sizeof(double), cudaMemcpyDeviceToHost));
}
