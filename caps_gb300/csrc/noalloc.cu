// noalloc.cu -- log det(1-M) of one (xi, m) matrix without allocating memory.
//
// Who needs it: callers that must not allocate device memory while they run --
// code executing inside a framework that owns every byte of the device through
// its own pool allocator (a cudaMalloc behind its back can fail or fragment the
// pool), or a host that may not grow its heap at that point.  caps_logdetD()
// grows a workspace with cudaMalloc on first use; this entry point instead takes
// all of its scratch from one file-scope device array of fixed size,
// NOALLOC_SCRATCH_BYTES (32 MiB), which exists on every GPU that loads the
// library until the process exits.
//
// Limits (rejected with an error code and a message, never truncated):
//   ldim <= 512 (matrix dimension <= 1024), lmin + ldim <= 2048, and at most
//   256 quadrature panels for the K integrals.
//
// The scratch array is shared by all calls and keeps the last call's contents;
// everything that must start at zero is cleared at the start of each call.
// Calls that overlap on the GPU (several host threads, or several streams)
// race on the array: issue them one at a time.
//
// Set-up: the first call on a device (with that device current) resolves the
// device address of the scratch array with cudaGetSymbolAddress and uploads
// the log n! and Gauss-Legendre constants to fixed device symbols.  Make that
// first call before any stream capture begins.
//
// It runs the same kernels as caps_logdetD, with the same HODLR/LU semantics
// of caps_t::detalg, on the legacy default stream.  The call synchronises the
// host with that stream twice (once to read the quadrature panel count, once for
// the result) and copies the result to the caller's host double.  Rejected input
// and failed CUDA API calls return a negative code with a message; a kernel
// launch that fails aborts the process, as every launch of the library does.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "../../include/libcaps.h"
#include "internal.h"

using namespace capsgpu;

#define NOALLOC_SCRATCH_BYTES (32u << 20)
#define NOALLOC_MAX_LDIM 512
#define NOALLOC_MAX_LWINDOW 2048
#define NOALLOC_MAX_PANELS 256
#define NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];
static __device__ double g_noalloc_lfac[1024];

static void *g_scratch_ptr[NOALLOC_MAX_DEVICES];
static double *g_lfac_ptr[NOALLOC_MAX_DEVICES];
static thread_local char g_noalloc_err[256];   // per host thread, like caps_gpu_last_error

extern "C" const char *caps_noalloc_last_error(void) { return g_noalloc_err; }

static int noalloc_fail(int code, const char *msg)
{
    snprintf(g_noalloc_err, sizeof g_noalloc_err, "caps_logdetD_noalloc: %s", msg);
    fprintf(stderr, "libcaps_gb300: %s\n", g_noalloc_err);
    return code;
}

// once per device: device address of the scratch array and the constant tables
static int noalloc_setup(int dev)
{
    if (g_scratch_ptr[dev]) return 0;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
        return noalloc_fail(-3, "cudaGetSymbolAddress of the scratch array failed");
    void *lf = nullptr;
    if (cudaGetSymbolAddress(&lf, g_noalloc_lfac) != cudaSuccess || !lf)
        return noalloc_fail(-3, "cudaGetSymbolAddress of the log n! table failed");
    double tab[1024];
    for (int n = 0; n < 1024; n++) tab[n] = lgamma(n + 1.0);
    if (cudaMemcpyToSymbol(g_noalloc_lfac, tab, sizeof tab) != cudaSuccess)
        return noalloc_fail(-3, "upload of the log n! table failed");
    // Gauss-Legendre nodes of the K panels (Newton iteration on P_GLN)
    double x[GLN], w[GLN];
    for (int i = 0; i < GLN; i++) {
        double z = cos(PI * (i + 0.75) / (GLN + 0.5)), pp = 0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= GLN; j++) { double p3 = p2; p2 = p1; p1 = ((2 * j - 1) * z * p2 - (j - 1) * p3) / j; }
            pp = GLN * (z * p1 - p2) / (z * z - 1);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) < 1e-16) break;
        }
        x[i] = z;
        w[i] = 2 / ((1 - z * z) * pp * pp);
    }
    upload_gauss_legendre(x, w);
    g_lfac_ptr[dev] = (double *)lf;
    g_scratch_ptr[dev] = p;
    return 0;
}

// bump allocator over the scratch array (256-byte aligned pieces)
struct Carve {
    unsigned char *base;
    size_t off = 0;
    bool ok = true;
    template <class T> T *take(size_t count)
    {
        const size_t bytes = (count * sizeof(T) + 255) & ~(size_t)255;
        if (off + bytes > NOALLOC_SCRATCH_BYTES) { ok = false; return nullptr; }
        T *r = (T *)(base + off);
        off += bytes;
        return r;
    }
};

#define NA_CK(x) do { if ((x) != cudaSuccess) return noalloc_fail(-4, "CUDA call failed: " #x); } while (0)

extern "C" int caps_logdetD_noalloc(caps_t *self, double xi_, int m, double *logdet)
{
    g_noalloc_err[0] = 0;
    if (!(xi_ > 0)) {   // contract of caps_logdetD (libcaps.c:952)
        fprintf(stderr, "libcaps_gb300: Matsubara frequency must be positive\n");
        abort();
    }
    if (m < 0) return noalloc_fail(-1, "m must be non-negative");
    const int ldim = self->ldim, dim = 2 * ldim, L = ldim + 2;
    size_t lo, hi;
    caps_estimate_lminmax(self, m, &lo, &hi);
    const int lmin = (int)lo;
    if (ldim > NOALLOC_MAX_LDIM) return noalloc_fail(-2, "ldim exceeds the maximum of 512");
    if (lmin + ldim > NOALLOC_MAX_LWINDOW) return noalloc_fail(-2, "lmin+ldim exceeds the maximum of 2048");

    int dev = 0;
    NA_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return noalloc_fail(-3, "device index out of range");
    if (int e = noalloc_setup(dev)) return e;
    const cudaStream_t st = 0;

    // the task (same fields as the batch path)
    Task T;
    memset(&T, 0, sizeof T);
    T.xi_ = xi_;
    T.alpha = 2 * xi_;
    T.epsm1_plate = caps_epsilonm1_plate(self, xi_);
    T.epsm1_sphere = caps_epsilonm1_sphere(self, xi_);
    T.m = m;
    T.lmin = lmin;
    T.mu = 2 * (m > 1 ? m : 1);
    T.s = m > 0 ? 1 : 0;
    T.nu_max = 2 * (lmin + ldim);
    T.xi_index = 0;
    T.mgroup = 0;
    T.is_pr = std::isinf(caps_epsilonm1_plate(self, INFINITY)) ? 1 : 0;
    const int nnu = T.nu_max - T.mu + 1;
    const int nu_stride = (nnu + 31) / 32 * 32;
    const int lmax_mie = lmin + ldim;
    const int lmax_all = lmin + ldim + 2;
    const int nlf = 4 * lmax_all + 8, nx = 2 * lmax_all + 8, pstride = 2 * lmax_all + 8;
    const int max_warps = NOALLOC_MAX_PANELS / 2;

    Carve C{(unsigned char *)g_scratch_ptr[dev]};
    Task *d_task = C.take<Task>(1);
    int *d_status = C.take<int>(1);
    double *d_xi = C.take<double>(1), *d_eps = C.take<double>(1);
    double *d_lna = C.take<double>(lmax_mie + 1), *d_lnb = C.take<double>(lmax_mie + 1);
    double *d_edges = C.take<double>(NOALLOC_MAX_PANELS + 1);
    double2 *d_coef = C.take<double2>(nu_stride);
    sd *d_Sa = C.take<sd>(L), *d_Sb = C.take<sd>(L);
    double2 *d_uv = C.take<double2>(L);
    double *d_lft = C.take<double>(nlf);
    double2 *d_xtab = C.take<double2>(nx);
    double4 *d_ptab = C.take<double4>((size_t)2 * pstride);
    double *d_pM = C.take<double>((size_t)2 * max_warps * nu_stride);
    int *d_pE = C.take<int>((size_t)2 * max_warps * nu_stride);
    sd *d_K = C.take<sd>((size_t)2 * nu_stride);
    sd *d_I = C.take<sd>((size_t)2 * L * L);
    double *d_A = C.take<double>((size_t)dim * dim);
    double *d_ld = C.take<double>(dim);
    double *d_md = C.take<double>(dim);
    double *d_trace = C.take<double>(1), *d_res = C.take<double>(1);
    int *d_gm = C.take<int>(1), *d_glm = C.take<int>(1);
    // the a_0..a_2 table of this m reuses the K partial-sum region when it fits there
    // (k_kred has read the partials before k_a12 writes the table, both on one stream);
    // otherwise nu_stride is small and the table gets a region of its own
    void *d_a12 = d_pM;
    if (a12_bytes(ldim, 1) > (size_t)2 * max_warps * nu_stride * sizeof(double)) d_a12 = C.take<unsigned char>(a12_bytes(ldim, 1));
    if (!C.ok) return noalloc_fail(-2, "workspace of this geometry exceeds the 32 MiB scratch array");

    // only the status word must start at zero; every other piece is written before it is read
    NA_CK(cudaMemsetAsync(d_status, 0, sizeof(int), st));
    NA_CK(cudaMemcpyAsync(d_task, &T, sizeof T, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(d_xi, &T.xi_, sizeof(double), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(d_eps, &T.epsm1_sphere, sizeof(double), cudaMemcpyHostToDevice, st));
    launch_mie(d_xi, d_eps, 1, self->LbyR, lmax_mie, d_lna, d_lnb, st);
    launch_setup(d_task, 1, d_edges, NOALLOC_MAX_PANELS, d_coef, nu_stride, 2.0, d_status, st);
    Task back;
    NA_CK(cudaMemcpyAsync(&back, d_task, sizeof back, cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    if (back.npanel == 0) return noalloc_fail(-2, "the K quadrature needs more than 256 panels for this (xi, m)");
    launch_scale(d_task, 1, ldim, d_lna, d_lnb, lmax_mie, g_lfac_ptr[dev], d_Sa, d_Sb, d_uv, st);
    launch_tables(g_lfac_ptr[dev], d_lft, nlf, d_xtab, nx, st);
    launch_ktab(T.is_pr != 0, d_task, 1, max_warps, d_edges, NOALLOC_MAX_PANELS, d_coef, nu_stride, g_lfac_ptr[dev], d_pM, d_pE, st);
    launch_kred(d_task, 1, nnu, d_pM, d_pE, max_warps, nu_stride, d_K, d_status, st);
    const int gm_h[2] = {m, lmin};
    NA_CK(cudaMemcpyAsync(d_gm, &gm_h[0], sizeof(int), cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(d_glm, &gm_h[1], sizeof(int), cudaMemcpyHostToDevice, st));
    launch_a12(d_gm, d_glm, 1, ldim, d_lft, d_a12, st);
    launch_ptab(d_task, 1, d_ptab, pstride, st);
    launch_itab(d_task, nullptr, 1, ldim, d_K, nu_stride, d_lft, d_xtab, d_ptab, pstride, d_I, d_status, st, d_a12, false);
    launch_elem(d_task, nullptr, 1, ldim, d_I, d_Sa, d_Sb, d_uv, d_A, dim, (size_t)dim * dim, d_md, d_status, st, false);
    const int mode = self->detalg == DETALG_HODLR ? 1 : 0;
    launch_stats(nullptr, 1, dim, d_A, dim, (size_t)dim * dim, d_md, mode, d_trace, d_res, d_status, st);
    launch_cholesky(1, dim, d_A, dim, (size_t)dim * dim, d_status, d_ld, st);
    launch_final(1, dim, d_ld, d_trace, d_status, d_res, mode, st);
    int status = 0;
    double r = NAN;
    NA_CK(cudaMemcpyAsync(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaMemcpyAsync(&r, d_res, sizeof(double), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    *logdet = r;
    return (status & ~0xF) ? status : 0;
}
