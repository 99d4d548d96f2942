// libcaps.cu -- host side of the GB300 CaPS library: the reference's C API
// (src/include/libcaps.h) on top of the batched GPU pipeline.
//
// A batch is a list of (xi_, m) matrices of one geometry.  The host evaluates
// the dielectric callbacks once per distinct frequency (the reference calls
// them per quadrature node with the same argument, integration.c:277), then
// the device runs: setup -> Mie -> K -> I -> elements -> stats -> Cholesky ->
// log-det, in chunks sized to the free device memory.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/libcaps.h"
#include "internal.h"

using namespace capsgpu;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string g_last_error;

static void set_error(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

namespace capsgpu {
Counters g_counters;
[[noreturn]] void fatal(const char *file, int line, const char *what)
{
    fprintf(stderr, "libcaps_gb300: CUDA failure at %s:%d: %s\n", file, line, what);
    abort();
}
} // namespace capsgpu

extern "C" const char *caps_gpu_last_error(void) { return g_last_error.c_str(); }

// ---------------------------------------------------------------------------
// log n! table shared by host and device (logfac.c:66615-66628)
// ---------------------------------------------------------------------------
static double h_lfac_tab[1024];
static std::once_flag g_tab_once;
static void init_host_tables()
{
    for (int n = 0; n < 1024; n++) h_lfac_tab[n] = lgamma(n + 1.0);
}
static double host_lfac(unsigned n)
{
    std::call_once(g_tab_once, init_host_tables);
    if (n < 1024) return h_lfac_tab[n];
    const double dn = n;
    return (dn + 0.5) * log(dn) - dn + HALF_LOG_2PI + (1.0 / 12) / dn;
}

// ---------------------------------------------------------------------------
// device engine: stream, constant tables, grow-only workspace
// ---------------------------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    void *get(size_t need)
    {
        if (need > bytes) {
            if (p) CK(cudaFree(p));
            p = nullptr;
            // grow by a quarter at least (fewer reallocations as batches vary); where that
            // does not fit, exactly what is needed
            const size_t want = std::max(need, bytes + bytes / 4);
            bytes = 0;
            if (cudaMalloc(&p, want) == cudaSuccess) {
                bytes = want;
            } else {
                (void)cudaGetLastError(); // an allocation failure is not sticky: clear it
                p = nullptr;
                CK(cudaMalloc(&p, need));
                bytes = need;
            }
        }
        return p;
    }
    void release()
    {
        if (p) CK(cudaFree(p));
        p = nullptr;
        bytes = 0;
    }
};

struct Engine {
    bool ready = false;
    int device = 0;
    cudaStream_t own = nullptr, user = nullptr;
    cudaStream_t side = nullptr;          // Mie coefficients and scale factors, beside setup and K
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double *d_lfac = nullptr;
    DevBuf tasks, edges, coef, partM, partE, K, I, Sa, Sb, uv, A, logdiag, trace, result, status, mie_a, mie_b, xi, eps, lft, xtab, ptab, S32, ptabf, a12, gm, glmin, Saf, Sbf, uvf, part, diag, groups, B, diag2, mwork, a12t, coefF, tlist, groups2, glist2, KP, KPe, hwork, seed;
    std::vector<double> host_pinned_dummy;
    double timings[6] = {0, 0, 0, 0, 0, 0};
    double timings_cum[6] = {0, 0, 0, 0, 0, 0};
    static constexpr int NEV = 9;
    cudaEvent_t ev[NEV];
    uint64_t shape = 0; // of the last batch (dimension, precision, path), see run_batch
    std::mutex mu;
    cudaStream_t stream() const { return user ? user : own; }
};
static Engine g_eng;

// schedules chosen by caps_gpu_autotune, per (precision, matrix dimension): for the mixed form
// the trailing-update schedule (MIXED_SCHED_*); absent entries use MIXED_SCHED_IMAGES
static std::map<std::pair<int, int>, int> g_sched;
static std::mutex g_sched_mu;
static int schedule_for(int precision, int dim)
{
    std::lock_guard<std::mutex> lk(g_sched_mu);
    auto it = g_sched.find({precision, dim});
    return it == g_sched.end() ? MIXED_SCHED_IMAGES : it->second;
}

static void engine_init()
{
    if (g_eng.ready) return;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        fprintf(stderr, "libcaps_gb300: no CUDA device available (%s); this library has no CPU path\n",
                e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
        abort();
    }
    CK(cudaGetDevice(&g_eng.device));
    CK(cudaStreamCreateWithFlags(&g_eng.own, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&g_eng.side, cudaStreamNonBlocking));
    CK(cudaEventCreateWithFlags(&g_eng.ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&g_eng.ev_join, cudaEventDisableTiming));
    std::call_once(g_tab_once, init_host_tables);
    CK(cudaMalloc(&g_eng.d_lfac, 1024 * sizeof(double)));
    CK(cudaMemcpy(g_eng.d_lfac, h_lfac_tab, 1024 * sizeof(double), cudaMemcpyHostToDevice));
    // Gauss-Legendre nodes on [-1,1] by Newton iteration on P_GLN
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
    for (int i = 0; i < Engine::NEV; i++) CK(cudaEventCreate(&g_eng.ev[i]));
    g_eng.ready = true;
}

extern "C" void caps_gpu_set_stream(void *stream)
{
    std::lock_guard<std::mutex> lk(g_eng.mu);
    engine_init();
    g_eng.user = (cudaStream_t)stream;
}

extern "C" void caps_gpu_counters(long long *launches, long long *h2d_bytes, long long *d2h_bytes, int reset)
{
    if (launches) *launches = g_counters.launches;
    if (h2d_bytes) *h2d_bytes = g_counters.h2d;
    if (d2h_bytes) *d2h_bytes = g_counters.d2h;
    if (reset) g_counters = Counters();
}

extern "C" void caps_gpu_kernel_timing(int enable)
{
    std::lock_guard<std::mutex> lk(g_eng.mu);
    kernel_timer_enable(enable != 0);
}

extern "C" void caps_gpu_kernel_stats_kind(int kind, double *ms, double *bytes, long long *launches)
{
    kernel_timer_stats(kind, ms, bytes, launches);
}

extern "C" void caps_gpu_kernel_stats(double *ms, double *bytes, long long *launches)
{
    kernel_timer_stats(KT_SYRK, ms, bytes, launches);
}

extern "C" void caps_gpu_work(long long *nmat, long long *nfactor, double *factor_flops)
{
    if (nmat) *nmat = g_counters.nmat;
    if (nfactor) *nfactor = g_counters.nfactor;
    if (factor_flops) *factor_flops = g_counters.factor_flops;
}

// sustained FP64 FMA throughput of this device (independent FMA chains on every SM)
__global__ void k_fp64_probe(double *out, int iters, double a)
{
    double x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = threadIdx.x + k;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fma(x[k], a, 1.0);
    double s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_fp32_probe(float *out, int iters, float a)
{
    float x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = threadIdx.x + k;
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fmaf(x[k], a, 1.0f);
    float s = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) s += x[k];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// sustained FP32 FMA throughput (independent FMA chains on every SM), TFLOP/s
extern "C" double caps_gpu_fp32_peak(void)
{
    std::lock_guard<std::mutex> lk(g_eng.mu);
    engine_init();
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_eng.device));
    const int blocks = sms * 8, threads = 256, iters = 100000;
    float *d;
    CK(cudaMalloc(&d, (size_t)blocks * threads * sizeof(float)));
    cudaStream_t st = g_eng.stream();
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        CK(cudaEventRecord(g_eng.ev[0], st));
        k_fp32_probe<<<blocks, threads, 0, st>>>(d, iters, 0.999f);
        CK(cudaEventRecord(g_eng.ev[1], st));
        CK(cudaEventSynchronize(g_eng.ev[1]));
        float ms;
        CK(cudaEventElapsedTime(&ms, g_eng.ev[0], g_eng.ev[1]));
        best = std::min(best, ms);
    }
    CK(cudaFree(d));
    return 2.0 * 8 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
}

extern "C" double caps_gpu_fp64_peak(void)
{
    std::lock_guard<std::mutex> lk(g_eng.mu);
    engine_init();
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g_eng.device));
    const int blocks = sms * 8, threads = 256, iters = 20000;
    double *d;
    CK(cudaMalloc(&d, (size_t)blocks * threads * sizeof(double)));
    cudaStream_t st = g_eng.stream();
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        CK(cudaEventRecord(g_eng.ev[0], st));
        k_fp64_probe<<<blocks, threads, 0, st>>>(d, iters, 0.999);
        CK(cudaEventRecord(g_eng.ev[1], st));
        CK(cudaEventSynchronize(g_eng.ev[1]));
        float ms;
        CK(cudaEventElapsedTime(&ms, g_eng.ev[0], g_eng.ev[1]));
        best = std::min(best, ms);
    }
    CK(cudaFree(d));
    return 2.0 * 8 * iters * (double)blocks * threads / (best * 1e-3) / 1e12;
}

extern "C" int caps_gpu_timings(double *ms, int n)
{
    int k = std::min(n, 12);
    for (int i = 0; i < k; i++) ms[i] = i < 6 ? g_eng.timings[i] : g_eng.timings_cum[i - 6];
    return k;
}

extern "C" void caps_gpu_reset_timings(void)
{
    for (int i = 0; i < 6; i++) g_eng.timings_cum[i] = 0;
}

// ---------------------------------------------------------------------------
// caps_t API (libcaps.c:45-457)
// ---------------------------------------------------------------------------
extern "C" double caps_lnLambda(int l1, int l2, int m)
{
    return (log(2. * l1 + 1) + log(2. * l2 + 1) - log((double)l1) - log(l1 + 1.) - log((double)l2) - log(l2 + 1.)
            + host_lfac(l1 - m) + host_lfac(l2 - m) - host_lfac(l1 + m) - host_lfac(l2 + m)) / 2.0;
}

extern "C" int caps_estimate_lminmax(caps_t *self, int m, size_t *lmin_p, size_t *lmax_p)
{
    const int ldim = self->ldim;
    if (m == 0) { *lmin_p = 1; *lmax_p = 1 + ldim; return 0; }
    const int l = (int)round(m / sqrt(2 * self->LbyR));
    int lmin = l - ldim / 2;
    if (lmin < m) lmin = m;
    *lmin_p = lmin;
    *lmax_p = lmin + ldim;
    return l;
}

extern "C" double caps_epsilonm1_perf(double xi_, void *userdata) { (void)xi_; (void)userdata; return INFINITY; }

extern "C" double caps_epsilonm1_drude(double xi, void *userdata)
{
    const double *p = (const double *)userdata;
    return p[0] * p[0] / (xi * (xi + p[1]));
}

extern "C" caps_t *caps_init(double R, double L)
{
    if (L <= 0 || R <= 0) return NULL;
    caps_t *s = (caps_t *)calloc(1, sizeof(caps_t));
    if (!s) { fprintf(stderr, "libcaps_gb300: out of memory\n"); abort(); }
    const double LbyR = L / R;
    s->LbyR = LbyR; s->L = L; s->R = R; s->calL = L + R;
    s->y = -LN2 - log1p(LbyR);
    s->ldim = (int)ceil(std::max((double)CAPS_MINIMUM_LDIM, CAPS_FACTOR_LDIM / LbyR));
    s->epsilonm1_plate = caps_epsilonm1_perf;
    s->epsilonm1_sphere = caps_epsilonm1_perf;
    s->userdata_plate = s->userdata_sphere = NULL;
    s->epsrel = CAPS_EPSREL;
    s->detalg = DETALG_HODLR;
    s->precision = CAPS_PREC_FP64;
    s->path = CAPS_PATH_AUTO;
    return s;
}

extern "C" void caps_free(caps_t *self) { free(self); }

extern "C" void caps_build(FILE *stream, const char *prefix)
{
    if (!prefix) prefix = "";
    fprintf(stream, "%sversion: 0.5 (GB300 port of the logdetD path)\n", prefix);
    fprintf(stream, "%scompiler: nvcc %d.%d\n", prefix, __CUDACC_VER_MAJOR__, __CUDACC_VER_MINOR__);
    fprintf(stream, "%scompile time: %s %s\n", prefix, __DATE__, __TIME__);
}

extern "C" void caps_info(caps_t *self, FILE *stream, const char *prefix)
{
    const char *d;
    if (!prefix) prefix = "";
    switch (self->detalg) {
    case DETALG_HODLR: d = "HODLR"; break;
    case DETALG_LU: d = "LU"; break;
    case DETALG_QR: d = "QR"; break;
    case DETALG_CHOLESKY: d = "CHOLESKY"; break;
    default: d = "unknown";
    }
    fprintf(stream, "%sL/R    = %.16g\n", prefix, self->LbyR);
    fprintf(stream, "%sL      = %.16g\n", prefix, self->L);
    fprintf(stream, "%sR      = %.16g\n", prefix, self->R);
    fprintf(stream, "%sldim   = %d\n", prefix, self->ldim);
    fprintf(stream, "%sepsrel = %.1e\n", prefix, self->epsrel);
    fprintf(stream, "%sdetalg = %s\n", prefix, d);
}

extern "C" int caps_set_epsrel(caps_t *self, double epsrel) { if (epsrel <= 0) return 0; self->epsrel = epsrel; return 1; }
extern "C" double caps_get_epsrel(caps_t *self) { return self->epsrel; }
extern "C" void caps_set_epsilonm1_plate(caps_t *self, double (*f)(double, void *), void *ud) { self->epsilonm1_plate = f; self->userdata_plate = ud; }
extern "C" void caps_set_epsilonm1_sphere(caps_t *self, double (*f)(double, void *), void *ud) { self->epsilonm1_sphere = f; self->userdata_sphere = ud; }
extern "C" void caps_set_epsilonm1(caps_t *self, double (*f)(double, void *), void *ud) { caps_set_epsilonm1_plate(self, f, ud); caps_set_epsilonm1_sphere(self, f, ud); }
extern "C" int caps_set_detalg(caps_t *self, detalg_t d) { self->detalg = d; return 1; }
extern "C" detalg_t caps_get_detalg(caps_t *self) { return self->detalg; }
extern "C" int caps_set_ldim(caps_t *self, int ldim) { if (ldim < 1) return 0; self->ldim = ldim; return 1; }
extern "C" int caps_get_ldim(caps_t *self) { return self->ldim; }
extern "C" int caps_gpu_set_precision(caps_t *self, int p)
{
    if (p != CAPS_PREC_FP64 && p != CAPS_PREC_MIXED) return 0;
    self->precision = p;
    return 1;
}

extern "C" int caps_gpu_set_path(caps_t *self, int path)
{
    if (path != CAPS_PATH_AUTO && path != CAPS_PATH_HODLR && path != CAPS_PATH_DENSE) return 0;
    self->path = path;
    return 1;
}

extern "C" double caps_epsilonm1_plate(caps_t *self, double xi_) { return self->epsilonm1_plate(xi_ * CAPS_c / self->calL, self->userdata_plate); }
extern "C" double caps_epsilonm1_sphere(caps_t *self, double xi_) { return self->epsilonm1_sphere(xi_ * CAPS_c / self->calL, self->userdata_sphere); }

// Fresnel coefficients (libcaps.c:616): a scalar helper of the API; the GPU
// evaluates the same formula per quadrature node inside the K kernel
extern "C" void caps_fresnel(caps_t *self, double xi_, double k_, double *r_TE, double *r_TM)
{
    const double epsm1 = caps_epsilonm1_plate(self, xi_);
    if (std::isinf(epsm1)) { *r_TM = 1.0; *r_TE = -1.0; return; }
    const double x = xi_ * xi_ / (xi_ * xi_ + k_ * k_) * epsm1;
    const double bm1 = x / (sqrt(1 + x) + 1);
    *r_TE = -bm1 / (2 + bm1);
    *r_TM = (epsm1 - bm1) / (epsm1 + 2 + bm1);
}

// ---------------------------------------------------------------------------
// the batch pipeline
// ---------------------------------------------------------------------------
struct BatchOpts {
    int mode = 1;            // 0 dense semantics (Mercator shortcut), 1 HODLR semantics
    bool factor = true;      // false: stop after assembly (caps_M_init)
    double *M_out = nullptr; // host buffer for the dense M of a single task (row-major)
    double *mie_out_a = nullptr, *mie_out_b = nullptr; // Mie of task 0's window
    bool square = false;     // sphere-sphere: log det(1 - M^2) (FP64, dense rules)
    bool force_dense = false; // factor densely even where the HODLR path applies
};

static void h2d(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
    g_counters.h2d += (long long)bytes;
}
static void d2h(void *dst, const void *src, size_t bytes, cudaStream_t st)
{
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    g_counters.d2h += (long long)bytes;
}

// panel width of the K quadrature grid in units of the local peak width: the accuracy of K
// (|d log K| ~ 1e-13 against an adaptive quadrature) is the same from 1 to 3; the FP64 form
// keeps 2, the mixed form, where K is a fifth of a free energy's time, takes 3 (a third
// fewer nodes)
static const double KGRID_WIDTH = 2.0, KGRID_WIDTH_MIXED = 3.0;
static const int MAX_PANELS = 2048;

static int lmin_of(const caps_t *c, int m)
{
    size_t lo, hi;
    caps_estimate_lminmax(const_cast<caps_t *>(c), m, &lo, &hi);
    return (int)lo;
}

static int run_batch(caps_t *caps, const double *xi_, const int *ms, int n, double *out, int *status_out, const BatchOpts &O)
{
    std::lock_guard<std::mutex> lk(g_eng.mu);
    engine_init();
    g_last_error.clear();
    const cudaStream_t st = g_eng.stream();
    const int ldim = caps->ldim, dim = 2 * ldim, L = ldim + 2;
    for (int i = 0; i < n; i++) TERMINATE(!(xi_[i] > 0), "Matsubara frequency must be positive");

    // material per distinct xi (host callbacks, evaluated once per frequency)
    const bool is_pr = std::isinf(caps_epsilonm1_plate(caps, INFINITY));
    std::map<double, int> xi_index;
    std::vector<double> xis, eps_sphere;
    // tasks run in (m, xi) order: consecutive frequencies of one m share the I recurrence;
    // results go back to the caller's order through `order`
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return ms[a] != ms[b] ? ms[a] < ms[b] : xi_[a] < xi_[b]; });
    std::vector<Task> tasks(n);
    int lmax_mie = 1;
    for (int i = 0; i < n; i++) {
        const int src = order[i];
        auto it = xi_index.find(xi_[src]);
        int ix;
        if (it == xi_index.end()) {
            ix = (int)xis.size();
            xi_index[xi_[src]] = ix;
            xis.push_back(xi_[src]);
            eps_sphere.push_back(caps_epsilonm1_sphere(caps, xi_[src]));
        } else ix = it->second;
        Task &T = tasks[i];
        T.xi_ = xi_[src];
        T.alpha = 2 * xi_[src];
        T.epsm1_plate = caps_epsilonm1_plate(caps, xi_[src]);
        T.epsm1_sphere = eps_sphere[ix];
        T.m = ms[src];
        TERMINATE(ms[src] < 0, "m must be non-negative");
        T.lmin = lmin_of(caps, ms[src]);
        // the I recurrence forms (x^2-(l1+l2+1)^2)(x^2-(l1-l2)^2) exactly in 64-bit integers
        TERMINATE(T.lmin + ldim > 27000, "l window beyond 27000 (lmin+ldim=%d) is not supported", T.lmin + ldim);
        T.mu = 2 * std::max(ms[src], 1);
        T.s = ms[src] > 0 ? 1 : 0;
        T.nu_max = 2 * (T.lmin + ldim);
        T.xi_index = ix;
        T.is_pr = is_pr ? 1 : 0;
        T.npanel = 0;
        lmax_mie = std::max(lmax_mie, T.lmin + ldim);
    }
    const int nxi = (int)xis.size();
    int nnu_max = 0;
    for (auto &T : tasks) nnu_max = std::max(nnu_max, T.nu_max - T.mu + 1);
    const int nu_stride = (nnu_max + 31) / 32 * 32;

    // HODLR semantics: the HODLR path (elements on demand) where it applies; the FP64 form
    // takes it from CAPS_HODLR_AUTO_DIM on, the mixed form from CAPS_HODLR_AUTO_DIM_MIXED on
    const bool mixed = caps->precision == CAPS_PREC_MIXED;
    const bool hodlr = O.factor && !O.square && !O.M_out && !O.force_dense && caps->detalg == DETALG_HODLR &&
                       (caps->path == CAPS_PATH_HODLR ||
                        (caps->path == CAPS_PATH_AUTO && dim >= (mixed ? CAPS_HODLR_AUTO_DIM_MIXED : CAPS_HODLR_AUTO_DIM)));
    // mixed precision without a dense-M request: elements go straight into the FP32 delta
    // matrix (no FP64 matrix)
    const bool ff_elem = mixed && O.factor && !O.M_out && !O.square && !hodlr;
    // ... and, where the window fits its shared-memory ring, M comes from the I recurrence seeded
    // by 4 L q-sums per matrix (sweep.cu) instead of the q-sums of every pair
    const bool sweep = ff_elem && sweep_fits(ldim);
    // chunk size from free memory.  The budget counts the large work buffers held from earlier
    // batches as free for this one: true while batches keep one shape, each buffer serving the
    // same array again; when the shape (dimension, precision, path) changes they are released
    // first, since a buffer the new path does not use would stay held beside the new ones
    // (every batch ends synchronised with the device, so none is in use)
    const uint64_t shape = ((uint64_t)dim << 16) | (uint64_t)mixed | (uint64_t)hodlr << 1 | (uint64_t)sweep << 2 |
                           (uint64_t)ff_elem << 3 | (uint64_t)O.square << 4 | (uint64_t)O.M_out << 5 | (uint64_t)O.factor << 6;
    if (g_eng.shape != shape) {
        for (DevBuf *b : {&g_eng.A, &g_eng.I, &g_eng.partM, &g_eng.partE, &g_eng.S32, &g_eng.a12, &g_eng.part, &g_eng.B,
                          &g_eng.hwork, &g_eng.seed, &g_eng.mwork})
            b->release();
        g_eng.shape = shape;
    }
    size_t freeb = 0, totb = 0;
    CK(cudaMemGetInfo(&freeb, &totb));
    const size_t mat_bytes = O.square ? 16 : ff_elem ? 4 + 1 : (caps->precision == CAPS_PREC_MIXED ? 12 : 8);
    const size_t dense_bytes = hodlr ? hodlr_work_bytes(ldim, 1)
                             : sweep ? (size_t)dim * dim * 4 + seed_bytes(ldim, 1)
                                     : (size_t)dim * dim * mat_bytes + (size_t)2 * L * L * sizeof(sd)
                                           + (size_t)L * (L + 1) / 2 * 32; // a_0..a_2 table (one row per task)
    const size_t per_task = dense_bytes + (size_t)2 * nu_stride * sizeof(sd)
                          + (size_t)nu_stride * sizeof(double2) + (size_t)3 * L * sizeof(sd) + (size_t)dim * 8
                          + (size_t)2 * 256 * nu_stride * 12  // partial sums, up to 256 warps
                          + (size_t)(4 * (caps->ldim + 4096)) * sizeof(double4) // p tables
                          + (mixed && !hodlr ? mixed_work_bytes(1, dim) : 0);   // diagonal-block inverses, panel images
    size_t budget = (size_t)(0.70 * (double)(freeb + g_eng.A.bytes + g_eng.I.bytes + g_eng.partM.bytes + g_eng.partE.bytes + g_eng.S32.bytes
                                             + g_eng.a12.bytes + g_eng.part.bytes + g_eng.B.bytes + g_eng.hwork.bytes
                                             + g_eng.seed.bytes + g_eng.mwork.bytes));
    int chunk = (int)std::max<size_t>(1, std::min<size_t>(budget / per_task, 65535));
    chunk = std::min(chunk, n);

    // Mie table for all distinct xi at once
    double *d_xi = (double *)g_eng.xi.get(nxi * sizeof(double));
    double *d_eps = (double *)g_eng.eps.get(nxi * sizeof(double));
    h2d(d_xi, xis.data(), nxi * sizeof(double), st);
    h2d(d_eps, eps_sphere.data(), nxi * sizeof(double), st);
    double *d_lna = (double *)g_eng.mie_a.get((size_t)nxi * (lmax_mie + 1) * sizeof(double));
    double *d_lnb = (double *)g_eng.mie_b.get((size_t)nxi * (lmax_mie + 1) * sizeof(double));

    // batch tables: log n! over every argument of the I q-sums, x^2 and 1/(4x^2-1)
    int lmax_all = 0;
    for (auto &T : tasks) lmax_all = std::max(lmax_all, T.lmin + ldim + 2);
    const int nlf = 4 * lmax_all + 8, nx = 2 * lmax_all + 8, pstride = 2 * lmax_all + 8;
    double *d_lft = (double *)g_eng.lft.get((size_t)nlf * sizeof(double));
    double2 *d_xtab = (double2 *)g_eng.xtab.get((size_t)nx * sizeof(double2));
    launch_tables(g_eng.d_lfac, d_lft, nlf, d_xtab, nx, st);

    double tsum[6] = {0, 0, 0, 0, 0, 0};
    int nerr = 0;
    for (int c0 = 0; c0 < n; c0 += chunk) {
        const int nt = std::min(chunk, n - c0);
        CK(cudaEventRecord(g_eng.ev[0], st));
        // the Mie coefficients (first chunk) and the scale factors do not feed the quadrature
        // set-up or the K integrals: they run on a side stream beside them
        if (c0 == 0) {
            CK(cudaEventRecord(g_eng.ev_fork, st));
            CK(cudaStreamWaitEvent(g_eng.side, g_eng.ev_fork, 0));
            launch_mie(d_xi, d_eps, nxi, caps->LbyR, lmax_mie, d_lna, d_lnb, g_eng.side);
        }
        // group the chunk's tasks by m: a_0, a_1, a_2 of the q-sums depend on (l1, l2, m) only
        std::map<int, int> gidx;
        std::vector<int> gm, glm;
        for (int i = c0; i < c0 + nt; i++) {
            auto it = gidx.find(tasks[i].m);
            if (it == gidx.end()) {
                it = gidx.emplace(tasks[i].m, (int)gm.size()).first;
                gm.push_back(tasks[i].m);
                glm.push_back(tasks[i].lmin);
            }
            tasks[i].mgroup = it->second;
        }
        const int ngroup = (int)gm.size();
        // subgroups of at most itab_group_size() consecutive tasks of one m for the mixed q-sums
        std::vector<int4> sub;
        for (int i = c0; i < c0 + nt; i++) {
            if (sub.empty() || tasks[i].m != tasks[c0 + sub.back().x].m || sub.back().y == itab_group_size())
                sub.push_back(make_int4(i - c0, 0, tasks[i].mgroup, 0));
            sub.back().y++;
        }
        const int nsub = (int)sub.size();
        int *d_gm = (int *)g_eng.gm.get(ngroup * sizeof(int));
        int *d_glm = (int *)g_eng.glmin.get(ngroup * sizeof(int));
        h2d(d_gm, gm.data(), ngroup * sizeof(int), st);
        h2d(d_glm, glm.data(), ngroup * sizeof(int), st);
        Task *d_tasks = (Task *)g_eng.tasks.get(nt * sizeof(Task));
        h2d(d_tasks, tasks.data() + c0, nt * sizeof(Task), st);
        int4 *d_sub = (int4 *)g_eng.groups.get(nsub * sizeof(int4));
        h2d(d_sub, sub.data(), nsub * sizeof(int4), st);
        int *d_status = (int *)g_eng.status.get(nt * sizeof(int));
        CK(cudaMemsetAsync(d_status, 0, nt * sizeof(int), st));
        double *d_edges = (double *)g_eng.edges.get((size_t)nt * (MAX_PANELS + 1) * sizeof(double));
        double2 *d_coef = (double2 *)g_eng.coef.get((size_t)nt * nu_stride * sizeof(double2));
        launch_setup(d_tasks, nt, d_edges, MAX_PANELS, d_coef, nu_stride,
                     caps->precision == CAPS_PREC_MIXED ? KGRID_WIDTH_MIXED : KGRID_WIDTH, d_status, st);
        // panel counts decide the size of the partial-sum buffers
        std::vector<Task> tback(nt);
        d2h(tback.data(), d_tasks, nt * sizeof(Task), st);
        CK(cudaStreamSynchronize(st));
        int max_warps = 1;
        for (auto &T : tback) max_warps = std::max(max_warps, (T.npanel + 1) / 2);
        sd *d_Sa = (sd *)g_eng.Sa.get((size_t)nt * L * sizeof(sd));
        sd *d_Sb = (sd *)g_eng.Sb.get((size_t)nt * L * sizeof(sd));
        double2 *d_uv = (double2 *)g_eng.uv.get((size_t)nt * L * sizeof(double2));
        CK(cudaEventRecord(g_eng.ev_fork, st)); // the chunk's task table is on the device
        CK(cudaStreamWaitEvent(g_eng.side, g_eng.ev_fork, 0));
        launch_scale(d_tasks, nt, ldim, d_lna, d_lnb, lmax_mie, g_eng.d_lfac, d_Sa, d_Sb, d_uv, g_eng.side);
        CK(cudaEventRecord(g_eng.ev_join, g_eng.side));
        CK(cudaEventRecord(g_eng.ev[1], st));

        double *d_pM = (double *)g_eng.partM.get((size_t)nt * 2 * max_warps * nu_stride * sizeof(double));
        int *d_pE = (int *)g_eng.partE.get((size_t)nt * 2 * max_warps * nu_stride * sizeof(int));
        const bool mixed = caps->precision == CAPS_PREC_MIXED;
        sd *d_K = nullptr;
        float4 *d_KP = nullptr;
        int *d_KPe = nullptr;
        if (mixed) {
            // mixed form: float-float K, TM and TE paired, the table the q-sums read
            d_KP = (float4 *)g_eng.KP.get((size_t)nt * nu_stride * sizeof(float4));
            d_KPe = (int *)g_eng.KPe.get((size_t)nt * nu_stride * sizeof(int));
            float4 *d_coefF = (float4 *)g_eng.coefF.get((size_t)nt * nu_stride * sizeof(float4));
            launch_ktab_ff(is_pr, d_tasks, nt, max_warps, d_edges, MAX_PANELS, d_coef, d_coefF, nu_stride, g_eng.d_lfac,
                           (float2 *)d_pM, d_pE, st);
            launch_kred_ff(d_tasks, nt, nnu_max, (const float2 *)d_pM, d_pE, max_warps, nu_stride, d_KP, d_KPe, d_status, st);
        } else {
            d_K = (sd *)g_eng.K.get((size_t)nt * 2 * nu_stride * sizeof(sd));
            launch_ktab(is_pr, d_tasks, nt, max_warps, d_edges, MAX_PANELS, d_coef, nu_stride, g_eng.d_lfac, d_pM, d_pE, st);
            launch_kred(d_tasks, nt, nnu_max, d_pM, d_pE, max_warps, nu_stride, d_K, d_status, st);
        }
        CK(cudaEventRecord(g_eng.ev[2], st));
        CK(cudaStreamWaitEvent(st, g_eng.ev_join, 0)); // Mie and scale factors from here on

        sd *d_I = (hodlr || sweep) ? nullptr : (sd *)g_eng.I.get((size_t)nt * 2 * L * L * sizeof(sd));
        double4 *d_ptab = (double4 *)g_eng.ptab.get((size_t)nt * 2 * pstride * sizeof(double4));
        void *d_a12 = (hodlr || sweep) ? nullptr : g_eng.a12.get(a12_bytes(ldim, ngroup));
        // a_0..a_2 per m; the mixed form's trace rule first needs only the band of each m
        void *d_a12t = nullptr;
        if (caps->precision == CAPS_PREC_MIXED) {
            // (the HODLR path and the seeds need the per-m tables alone: their pairs combine them
            // on demand)
            d_a12t = g_eng.a12t.get(a12_tab_bytes(ldim, ngroup));
            launch_a12_mixed(d_gm, d_glm, ngroup, ldim, d_lft, d_a12, d_a12t, st, true, nullptr, (hodlr || ff_elem) ? 0 : -1);
        } else if (!hodlr)
            launch_a12(d_gm, d_glm, ngroup, ldim, d_lft, d_a12, st);
        const size_t lda = dim, mstride = (size_t)dim * dim;
        double *d_trace = (double *)g_eng.trace.get(nt * sizeof(double));
        double *d_res = (double *)g_eng.result.get(nt * sizeof(double));
        double *d_dg = (double *)g_eng.diag.get((size_t)nt * dim * sizeof(double));
        void *d_Saf = nullptr, *d_Sbf = nullptr, *d_seed = nullptr;
        float4 *d_uvf = nullptr;
        int nlist = nt;            // matrices assembled in full
        const int *d_list = nullptr; // their chunk indices (nullptr: all of them)
        std::vector<int> list;
        std::vector<int4> sub2;      // mixed form: q-sum subgroups of the listed matrices
        // A factorising request whose M is not wanted in full applies the trace rule to the
        // diagonal first, as kernel_logdet does (matrix.c:62-82): the band of the q-sums that
        // M_ii reads, M_ii, and the rule.  Only the matrices it leaves undecided are summed
        // and assembled in full.
        const bool diag_first = O.factor && !O.square && !O.M_out && (ff_elem || caps->precision != CAPS_PREC_MIXED);
        auto undecided = [&]() {
            std::vector<int> hs(nt);
            d2h(hs.data(), d_status, nt * sizeof(int), st);
            CK(cudaStreamSynchronize(st));
            for (int i = 0; i < nt; i++) {
                if (hs[i] != 0) continue;
                if (sub2.empty() || tasks[c0 + i].m != tasks[c0 + list[sub2.back().x]].m || sub2.back().y == itab_group_size())
                    sub2.push_back(make_int4((int)list.size(), 0, tasks[c0 + i].mgroup, 0));
                sub2.back().y++;
                list.push_back(i);
            }
            nlist = (int)list.size();
            if (nlist > 0) {
                int *dl = (int *)g_eng.tlist.get(nlist * sizeof(int));
                h2d(dl, list.data(), nlist * sizeof(int), st);
                d_list = dl;
            }
        };
        HodlrMixed hmx{};
        if (caps->precision == CAPS_PREC_MIXED && hodlr) {
            // mixed HODLR: M_ii for the trace rule and, for the undecided matrices, every sampled
            // element from float-float q-sums; compression and factorisation in FP64
            float4 *d_ptabf = (float4 *)g_eng.ptabf.get((size_t)nt * 2 * pstride * 2 * sizeof(float4));
            launch_ptab_groups(d_gm, ngroup, d_ptabf, pstride, st);
            hmx = HodlrMixed{d_KP, d_KPe, d_ptabf, d_a12t, ngroup};
            hodlr_diag(d_tasks, nt, ldim, nullptr, nu_stride, nullptr, pstride, d_lft, d_Sa, d_Sb, d_uv, d_dg, d_status, st, &hmx);
            CK(cudaEventRecord(g_eng.ev[3], st));
            launch_stats(nullptr, nt, dim, nullptr, lda, mstride, d_dg, O.mode, d_trace, d_res, d_status, st);
            CK(cudaEventRecord(g_eng.ev[4], st));
            undecided();
            CK(cudaEventRecord(g_eng.ev[5], st));
        } else if (caps->precision == CAPS_PREC_MIXED) {
            // mixed form: the q-sums in float-float on the FP32 pipe
            float4 *d_ptabf = (float4 *)g_eng.ptabf.get((size_t)nt * 2 * pstride * 2 * sizeof(float4));
            launch_ptab_groups(d_gm, ngroup, d_ptabf, pstride, st); // the recurrence tables depend on m alone
            if (diag_first) {
                d_Saf = g_eng.Saf.get((size_t)nt * L * 16);
                d_Sbf = g_eng.Sbf.get((size_t)nt * L * 16);
                d_uvf = (float4 *)g_eng.uvf.get((size_t)nt * L * sizeof(float4));
                launch_scale_ff(nt, ldim, d_Sa, d_Sb, d_uv, d_Saf, d_Sbf, d_uvf, st);
                // the band of q-sums that M_ii reads (l1 - l2 in {0, 2})
                d_seed = g_eng.seed.get(seed_bytes(ldim, nt));
                launch_seed_ff(d_tasks, nullptr, d_sub, nsub, ldim, d_KP, d_KPe, nu_stride, d_ptabf, pstride, d_a12t, ngroup, d_seed,
                               true, d_status, st);
                CK(cudaEventRecord(g_eng.ev[3], st));
                launch_diag_ff(d_tasks, nt, ldim, d_seed, d_Saf, d_Sbf, d_uvf, d_dg, d_status, st);
                launch_stats_ff(nullptr, nt, ldim, d_dg, nullptr, O.mode, d_trace, d_res, d_status, st);
                CK(cudaEventRecord(g_eng.ev[4], st));
                undecided();
                int4 *dg2 = nullptr;
                if (nlist > 0) {
                    dg2 = (int4 *)g_eng.groups2.get(sub2.size() * sizeof(int4));
                    h2d(dg2, sub2.data(), sub2.size() * sizeof(int4), st);
                }
                if (nlist > 0 && !sweep) {
                    // all pairs of the a_0..a_2 rows of the m that still need them
                    std::vector<int> gl;
                    for (const int4 &g : sub2)
                        if (gl.empty() || gl.back() != g.z) gl.push_back(g.z);
                    int *dgl = (int *)g_eng.glist2.get(gl.size() * sizeof(int));
                    h2d(dgl, gl.data(), gl.size() * sizeof(int), st);
                    launch_a12_mixed(d_gm, d_glm, ngroup, ldim, d_lft, d_a12, d_a12t, st, false, dgl, (int)gl.size());
                }
                CK(cudaEventRecord(g_eng.ev[5], st));
                if (sweep) // the rest of the recurrence's seeds: l1 - l2 = 1 and the first column
                    launch_seed_ff(d_tasks, d_list, dg2, nlist > 0 ? (int)sub2.size() : 0, ldim, d_KP, d_KPe, nu_stride, d_ptabf, pstride,
                                   d_a12t, ngroup, d_seed, false, d_status, st);
                else
                    launch_itab_grp(d_tasks, d_list, dg2, nlist > 0 ? (int)sub2.size() : 0, ldim, d_KP, d_KPe, nu_stride, d_ptabf, pstride,
                                    d_a12, d_I, true, d_status, st);
            } else {
                for (int k = 3; k <= 5; k++) CK(cudaEventRecord(g_eng.ev[k], st));
                launch_itab_grp(d_tasks, nullptr, d_sub, nsub, ldim, d_KP, d_KPe, nu_stride, d_ptabf, pstride, d_a12, d_I, ff_elem,
                                d_status, st);
            }
        } else if (hodlr) {
            // HODLR: M_ii for the trace rule, then the undecided matrices by HODLR with their
            // elements formed on demand (no I table, no dense matrix)
            launch_ptab(d_tasks, nt, d_ptab, pstride, st);
            hodlr_diag(d_tasks, nt, ldim, d_K, nu_stride, d_ptab, pstride, d_lft, d_Sa, d_Sb, d_uv, d_dg, d_status, st, nullptr);
            CK(cudaEventRecord(g_eng.ev[3], st));
            launch_stats(nullptr, nt, dim, nullptr, lda, mstride, d_dg, O.mode, d_trace, d_res, d_status, st);
            CK(cudaEventRecord(g_eng.ev[4], st));
            undecided();
            CK(cudaEventRecord(g_eng.ev[5], st));
        } else {
            launch_ptab(d_tasks, nt, d_ptab, pstride, st);
            if (diag_first) {
                launch_itab(d_tasks, nullptr, nt, ldim, d_K, nu_stride, d_lft, d_xtab, d_ptab, pstride, d_I, d_status, st, d_a12, true);
                CK(cudaEventRecord(g_eng.ev[3], st));
                launch_elem(d_tasks, nullptr, nt, ldim, d_I, d_Sa, d_Sb, d_uv, nullptr, lda, mstride, d_dg, d_status, st, true);
                launch_stats(nullptr, nt, dim, nullptr, lda, mstride, d_dg, O.mode, d_trace, d_res, d_status, st);
                CK(cudaEventRecord(g_eng.ev[4], st));
                undecided();
                CK(cudaEventRecord(g_eng.ev[5], st));
            } else
                for (int k = 3; k <= 5; k++) CK(cudaEventRecord(g_eng.ev[k], st));
            launch_itab(d_tasks, d_list, nlist, ldim, d_K, nu_stride, d_lft, d_xtab, d_ptab, pstride, d_I, d_status, st, d_a12, false);
        }
        CK(cudaEventRecord(g_eng.ev[6], st));

        double *d_A = nullptr;
        float *d_S = nullptr;
        if (hodlr) {
            // (no element phase)
        } else if (ff_elem && sweep) {
            d_S = (float *)g_eng.S32.get((size_t)nt * mstride * sizeof(float));
            float *d_part = (float *)g_eng.part.get((size_t)nt * sizeof(float));
            launch_sweep_ff(d_tasks, d_list, nlist, ldim, d_seed, d_Saf, d_Sbf, d_S, mstride, d_part, d_status, st);
            launch_stats_ff(d_list, nlist, ldim, d_dg, d_part, O.mode, d_trace, d_res, d_status, st, true);
        } else if (ff_elem) {
            d_S = (float *)g_eng.S32.get((size_t)nt * mstride * sizeof(float));
            float *d_part = (float *)g_eng.part.get((size_t)nt * elem_ff_part_floats(ldim) * sizeof(float));
            launch_elem_ff(d_tasks, d_list, nlist, ldim, d_Saf, d_Sbf, d_uvf, d_I, d_S, mstride, d_dg, d_part, d_status, st);
            launch_stats_ff(d_list, nlist, ldim, d_dg, d_part, O.mode, d_trace, d_res, d_status, st);
        } else {
            d_A = (double *)g_eng.A.get((size_t)nt * mstride * sizeof(double));
            launch_elem(d_tasks, d_list, nlist, ldim, d_I, d_Sa, d_Sb, d_uv, d_A, lda, mstride, d_dg, d_status, st, false);
            if (O.square) {
                // sphere-sphere: continue with B = 1 - M^2 in place of A
                double *d_B = (double *)g_eng.B.get((size_t)nt * mstride * sizeof(double));
                double *d_dg2 = (double *)g_eng.diag2.get((size_t)nt * dim * sizeof(double));
                launch_square(nt, dim, d_A, lda, mstride, d_dg, d_B, d_status, d_dg2, st);
                d_A = d_B;
                d_dg = d_dg2;
            }
            if (O.factor) launch_stats(d_list, nlist, dim, d_A, lda, mstride, d_dg, O.mode, d_trace, d_res, d_status, st);
        }
        CK(cudaEventRecord(g_eng.ev[7], st));

        // CAPS_MIXED_SIMT=1 selects the FP32 FFMA trailing update instead of split-TF32 tensor cores
        static const bool tc = getenv("CAPS_MIXED_SIMT") == nullptr;
        if (hodlr) {
            if (nlist > 0)
                hodlr_logdet_batch(d_tasks, d_list, nlist, ldim, d_K, nu_stride, d_ptab, pstride, d_lft, d_Sa, d_Sb, d_uv, d_trace,
                                   d_status, d_res, g_eng.hwork.get(hodlr_work_bytes(ldim, nlist)), st, mixed ? &hmx : nullptr);
        } else if (ff_elem) {
            void *d_work = g_eng.mwork.get(mixed_work_bytes(nt, dim));
            launch_cholesky_mixed(nt, dim, nullptr, 0, 0, d_status, d_S, mstride, d_dg, d_trace, d_res, O.mode, st, tc, false, d_work,
                                  schedule_for(caps->precision, dim));
        } else if (O.factor && caps->precision == CAPS_PREC_MIXED && !O.square) {
            d_S = (float *)g_eng.S32.get((size_t)nt * mstride * sizeof(float));
            void *d_work = g_eng.mwork.get(mixed_work_bytes(nt, dim));
            launch_cholesky_mixed(nt, dim, d_A, lda, mstride, d_status, d_S, mstride, d_dg, d_trace, d_res, O.mode, st, tc, true, d_work,
                                  schedule_for(caps->precision, dim));
        } else if (O.factor) {
            double *d_ld = (double *)g_eng.logdiag.get((size_t)nt * dim * sizeof(double));
            launch_cholesky(nt, dim, d_A, lda, mstride, d_status, d_ld, st);
            launch_final(nt, dim, d_ld, d_trace, d_status, d_res, O.mode, st);
        }
        CK(cudaEventRecord(g_eng.ev[8], st));

        std::vector<int> hst(nt);
        std::vector<double> hres(nt);
        d2h(hst.data(), d_status, nt * sizeof(int), st);
        if (O.factor) d2h(hres.data(), d_res, nt * sizeof(double), st);
        if (O.M_out) {
            // dense row-major M from the lower triangle of 1-M
            std::vector<double> Ah((size_t)dim * dim);
            d2h(Ah.data(), d_A, (size_t)dim * dim * sizeof(double), st);
            CK(cudaStreamSynchronize(st));
            for (int j = 0; j < dim; j++)
                for (int i = j; i < dim; i++) {
                    const double v = (i == j ? 1.0 : 0.0) - Ah[(size_t)j * dim + i];
                    O.M_out[(size_t)i * dim + j] = v;
                    O.M_out[(size_t)j * dim + i] = v;
                }
        }
        if (O.mie_out_a) {
            const Task &T = tasks[0];
            d2h(O.mie_out_a, d_lna + (size_t)T.xi_index * (lmax_mie + 1) + T.lmin, ldim * sizeof(double), st);
            d2h(O.mie_out_b, d_lnb + (size_t)T.xi_index * (lmax_mie + 1) + T.lmin, ldim * sizeof(double), st);
        }
        CK(cudaStreamSynchronize(st));
        // phases: setup+Mie, K, I (band, the host's look at the trace rule, the rest), elements
        // (diagonal, then the undecided matrices in full), factorisation, total
        auto el = [](int a, int b) { float f; CK(cudaEventElapsedTime(&f, g_eng.ev[a], g_eng.ev[b])); return (double)f; };
        tsum[0] += el(0, 1);
        tsum[1] += el(1, 2);
        tsum[2] += el(2, 3) + el(4, 6);
        tsum[3] += el(3, 4) + el(6, 7);
        tsum[4] += el(7, 8);
        tsum[5] += el(0, 8);
        g_counters.nmat += nt;
        long long nfac = 0;
        for (int i = 0; i < nt; i++) nfac += hst[i] == ST_FACTOR;
        kernel_timer_collect(nfac);
        for (int i = 0; i < nt; i++) {
            const int dst = order[c0 + i];
            if (O.factor) out[dst] = hres[i];
            if (hst[i] == ST_FACTOR) {
                g_counters.nfactor++;
                if (!hodlr) g_counters.factor_flops += (double)dim * dim * dim / 3.0;
            }
            if (status_out) status_out[dst] = hst[i];
            if (hst[i] & ~0xF) {
                nerr++;
                set_error("matrix %d (xi_=%.17g, m=%d): status %d", dst, tasks[c0 + i].xi_, tasks[c0 + i].m, hst[i]);
            }
        }
    }
    for (int k = 0; k < 6; k++) { g_eng.timings[k] = tsum[k]; g_eng.timings_cum[k] += tsum[k]; }
    return nerr;
}

static int detalg_mode(const caps_t *c) { return c->detalg == DETALG_HODLR ? 1 : 0; }

extern "C" int caps_logdetD_batch(caps_t *self, const double *xi_, const int *m, int n, double *out, int *status)
{
    if (n <= 0) return 0;
    BatchOpts O;
    O.mode = detalg_mode(self);
    std::vector<int> st_local;
    if (!status) { st_local.resize(n); status = st_local.data(); }
    int nerr = run_batch(self, xi_, m, n, out, status, O);
    // matrices whose HODLR compression ran over its rank limit: factored densely instead
    std::vector<double> rx;
    std::vector<int> rm, ri;
    for (int i = 0; i < n; i++)
        if (status[i] & ST_ERR_HODLR) { rx.push_back(xi_[i]); rm.push_back(m[i]); ri.push_back(i); }
    if (!ri.empty()) {
        O.force_dense = true;
        std::vector<double> ro(ri.size());
        std::vector<int> rs(ri.size());
        run_batch(self, rx.data(), rm.data(), (int)ri.size(), ro.data(), rs.data(), O);
        nerr = 0;
        for (size_t k = 0; k < ri.size(); k++) { out[ri[k]] = ro[k]; status[ri[k]] = rs[k]; }
        for (int i = 0; i < n; i++) nerr += (status[i] & ~0xF) != 0;
    }
    return nerr;
}

// Autotuner: for this object's dimension and precision, time each candidate schedule on a
// probe batch of the object's own workload (nprobe matrices at xi_, m = 0, 1, ... -- the
// low m of a frequency are the matrices that reach the factorisation) and keep the fastest:
// the trailing-update schedule of the mixed form (process-wide, per dimension), or the
// determinant path of the FP64 form under DETALG_HODLR (dense Cholesky or HODLR, stored in
// the object; under DETALG_HODLR the mixed form's candidates include its HODLR path too).
// Each candidate runs twice; the second run's device time of the batch counts.
// The schedules give the same result to the rounding of the FP32 update (mixed) or to the
// compression tolerance (HODLR); within a process a dimension keeps its choice.
extern "C" int caps_gpu_autotune(caps_t *self, double xi_, int nprobe, caps_autotune_info_t *info)
{
    if (nprobe <= 0 || !(xi_ > 0)) return 0;
    const int dim = 2 * self->ldim;
    std::vector<double> xs(nprobe, xi_), out(nprobe);
    std::vector<int> ms(nprobe), st(nprobe);
    for (int k = 0; k < nprobe; k++) ms[k] = k;
    const bool mixed = self->precision == CAPS_PREC_MIXED;
    const bool can_hodlr = self->detalg == DETALG_HODLR;
    // mixed: the dense schedules, then (under DETALG_HODLR) the HODLR path; FP64: dense, HODLR
    const int ncand = mixed ? MIXED_SCHED_COUNT + (can_hodlr ? 1 : 0) : (can_hodlr ? 2 : 1);
    std::vector<double> ms_per(ncand, 0.0);
    const int saved_path = self->path;
    for (int c = 0; c < ncand; c++) {
        if (mixed) {
            self->path = c < MIXED_SCHED_COUNT ? CAPS_PATH_DENSE : CAPS_PATH_HODLR;
            if (c < MIXED_SCHED_COUNT) {
                std::lock_guard<std::mutex> lk(g_sched_mu);
                g_sched[{CAPS_PREC_MIXED, dim}] = c;
            }
        } else
            self->path = c == 0 ? CAPS_PATH_DENSE : CAPS_PATH_HODLR;
        caps_logdetD_batch(self, xs.data(), ms.data(), nprobe, out.data(), st.data());
        caps_logdetD_batch(self, xs.data(), ms.data(), nprobe, out.data(), st.data());
        ms_per[c] = g_eng.timings[5] / nprobe;
    }
    int best = 0;
    for (int c = 1; c < ncand; c++)
        if (ms_per[c] < ms_per[best]) best = c;
    if (ncand == 1)
        self->path = saved_path;
    else if (mixed) {
        // the fastest dense schedule is kept for the dimension in any case
        int bs = 0;
        for (int c = 1; c < MIXED_SCHED_COUNT; c++)
            if (ms_per[c] < ms_per[bs]) bs = c;
        std::lock_guard<std::mutex> lk(g_sched_mu);
        g_sched[{CAPS_PREC_MIXED, dim}] = bs;
        self->path = best == MIXED_SCHED_COUNT ? CAPS_PATH_HODLR : CAPS_PATH_DENSE;
    } else
        self->path = best == 0 ? CAPS_PATH_DENSE : CAPS_PATH_HODLR;
    if (info) {
        info->ncand = ncand;
        info->chosen = best;
        for (int c = 0; c < ncand && c < 4; c++) info->ms_per_matrix[c] = ms_per[c];
    }
    return 1;
}

// sphere-sphere (cass.c:23-64): log det(1 - M^2) of the plane-sphere round trip M at
// the caps object's L (half the sphere-sphere separation), dense rules, FP64
extern "C" int caps_logdetD2_batch(caps_t *self, const double *xi_, const int *m, int n, double *out, int *status)
{
    if (n <= 0) return 0;
    for (int i = 0; i < n; i++) TERMINATE(!(xi_[i] > 0), "Matsubara frequency must be positive");
    BatchOpts O;
    O.mode = 0;
    O.square = true;
    return run_batch(self, xi_, m, n, out, status, O);
}

extern "C" double caps_logdetD(caps_t *self, double xi_, int m)
{
    TERMINATE(xi_ <= 0, "Matsubara frequency must be positive");
    double r = NAN;
    BatchOpts O;
    O.mode = detalg_mode(self);
    run_batch(self, &xi_, &m, 1, &r, NULL, O);
    return r;
}

// ---------------------------------------------------------------------------
// Mie coefficients through the device kernel (single evaluation)
// ---------------------------------------------------------------------------
static void mie_device(caps_t *self, double xi_, int l, double epsm1, double *lna, double *lnb)
{
    std::lock_guard<std::mutex> lk(g_eng.mu);
    engine_init();
    const cudaStream_t st = g_eng.stream();
    double *d_xi = (double *)g_eng.xi.get(sizeof(double));
    double *d_eps = (double *)g_eng.eps.get(sizeof(double));
    h2d(d_xi, &xi_, sizeof(double), st);
    h2d(d_eps, &epsm1, sizeof(double), st);
    double *d_a = (double *)g_eng.mie_a.get((size_t)(l + 1) * sizeof(double));
    double *d_b = (double *)g_eng.mie_b.get((size_t)(l + 1) * sizeof(double));
    launch_mie(d_xi, d_eps, 1, self->LbyR, l, d_a, d_b, st);
    d2h(lna, d_a + l, sizeof(double), st);
    d2h(lnb, d_b + l, sizeof(double), st);
    CK(cudaStreamSynchronize(st));
}

extern "C" void caps_mie(caps_t *self, double xi_, int l, double *lna, double *lnb)
{
    mie_device(self, xi_, l, caps_epsilonm1_sphere(self, xi_), lna, lnb);
}

extern "C" void caps_mie_perf(caps_t *self, double xi_, int l, double *lna, double *lnb)
{
    mie_device(self, xi_, l, INFINITY, lna, lnb);
}

// ---------------------------------------------------------------------------
// element API (libcaps.c:673-846): the GPU materialises the whole matrix
// ---------------------------------------------------------------------------
extern "C" caps_M_t *caps_M_init(caps_t *self, int m, double xi_)
{
    TERMINATE(xi_ <= 0, "Matsubara frequency must be positive");
    caps_M_t *M = (caps_M_t *)calloc(1, sizeof(caps_M_t));
    const int ldim = self->ldim, dim = 2 * ldim;
    M->caps = self; M->m = m; M->ldim = ldim; M->xi_ = xi_;
    M->lmin = lmin_of(self, m);
    M->al = (double *)malloc(ldim * sizeof(double));
    M->bl = (double *)malloc(ldim * sizeof(double));
    M->M = (double *)malloc((size_t)dim * dim * sizeof(double));
    BatchOpts O;
    O.factor = false;
    O.M_out = M->M;
    O.mie_out_a = M->al;
    O.mie_out_b = M->bl;
    run_batch(self, &xi_, &m, 1, NULL, NULL, O);
    return M;
}

extern "C" double caps_M_elem(caps_M_t *self, int l1, int l2, char p1, char p2)
{
    const int dim = 2 * self->ldim;
    const int i = 2 * (l1 - self->lmin) + (p1 == 'M'), j = 2 * (l2 - self->lmin) + (p2 == 'M');
    return self->M[(size_t)i * dim + j];
}

extern "C" double caps_kernel_M(int i, int j, void *args_)
{
    caps_M_t *a = (caps_M_t *)args_;
    return a->M[(size_t)i * 2 * a->ldim + j];
}

extern "C" void caps_M_free(caps_M_t *self)
{
    if (!self) return;
    free(self->al); free(self->bl); free(self->M); free(self);
}

// ---------------------------------------------------------------------------
// xi = 0 (libcaps.c:860-1145): closed-form EE/MM kernels; element callbacks
// ---------------------------------------------------------------------------
extern "C" double caps_kernel_M0_EE(int i, int j, void *args_)
{
    caps_M_t *a = (caps_M_t *)args_;
    const double y = a->caps->y;
    const int l1 = i + a->lmin, l2 = j + a->lmin, m = a->m;
    return exp((l1 + l2 + 1) * y + host_lfac(l1 + l2) - 0.5 * (host_lfac(l1 + m) + host_lfac(l1 - m) + host_lfac(l2 + m) + host_lfac(l2 - m)));
}

extern "C" double caps_kernel_M0_MM(int i, int j, void *args_)
{
    caps_M_t *a = (caps_M_t *)args_;
    const int l1 = i + a->lmin, l2 = j + a->lmin;
    return caps_kernel_M0_EE(i, j, args_) * sqrt(((double)l1 * l2) / ((l1 + 1.) * (l2 + 1.)));
}

// plasma xi=0 integrals for the element-wise interface: the tables I_nu and
// I_{l-1/2}/I_{l+1/2} are computed on the GPU (xi0.cu) and served from host copies,
// grown on demand (integration.c:897-1031)
void plasma_tables_host(double omegap_, double alpha, int numax, int lmax, std::vector<double> &I, std::vector<double> &ratio);
struct PlasmaTables { std::vector<double> I, ratio; };

extern "C" integration_plasma_t *caps_integrate_plasma_init(caps_t *caps, double omegap, double epsrel)
{
    integration_plasma_t *self = (integration_plasma_t *)calloc(1, sizeof(integration_plasma_t));
    self->LbyR = caps->LbyR;
    self->omegap_ = omegap * caps->calL / CAPS_c;
    self->alpha = self->omegap_ / (1 + caps->LbyR);
    self->epsrel = epsrel;
    self->cache = new PlasmaTables;
    self->cache_ratio = nullptr;
    return self;
}

extern "C" double caps_integrate_plasma(integration_plasma_t *self, int l1, int l2, int m, double *ratio1, double *ratio2)
{
    (void)m;
    PlasmaTables *t = (PlasmaTables *)self->cache;
    const int lmax = std::max(l1, l2), numax = l1 + l2;
    if ((int)t->I.size() <= numax || (int)t->ratio.size() <= lmax) {
        const int l = std::max(2 * lmax, 64);
        plasma_tables_host(self->omegap_, self->alpha, 2 * l, l, t->I, t->ratio);
    }
    if (ratio1) *ratio1 = t->ratio[l1];
    if (ratio2) *ratio2 = t->ratio[l2];
    return t->I[numax];
}

extern "C" void caps_integrate_plasma_free(integration_plasma_t *self)
{
    if (!self) return;
    delete (PlasmaTables *)self->cache;
    free(self);
}

extern "C" double caps_kernel_M0_MM_plasma(int i, int j, void *args_)
{
    caps_M_t *a = (caps_M_t *)args_;
    integration_plasma_t *ip = (integration_plasma_t *)a->integration_plasma;
    TERMINATE(!ip, "caps_kernel_M0_MM_plasma: integration_plasma not set (caps_integrate_plasma_init)");
    const double y = a->caps->y;
    const int l1 = i + a->lmin, l2 = j + a->lmin, m = a->m;
    double ratio1, ratio2;
    const double I = caps_integrate_plasma(ip, l1, l2, m, &ratio1, &ratio2);
    const double alpha = ip->alpha;
    const double factor1 = 1 - (2 * l1 + 1.) / (alpha * ratio1);
    const double factor2 = 1 - (2 * l2 + 1.) / (alpha * ratio2);
    const double factor = sqrt(l1 * factor1 / (l1 + 1.) * l2 * factor2 / (l2 + 1.));
    return factor * exp(host_lfac(l1 + l2) - 0.5 * (host_lfac(l1 + m) + host_lfac(l1 - m) + host_lfac(l2 + m) + host_lfac(l2 - m)) + (l1 + l2 + 1) * y) * I;
}

extern "C" double caps_ht_drude(caps_t *caps)
{
    const double x = caps->LbyR, x2 = x * x;
    const double Z = (1 + x) * (1 - sqrt((x2 + 2 * x) / (x2 + 2 * x + 1)));
    double s1 = 0, s2 = 0;
    for (int l = 1;; l++) {
        const double a = pow(Z, 2 * l), b = a * Z;
        const double v1 = (2 * l + 1) * log1p(-b), v2 = b * (1 - a) / (1 - b);
        s1 += v1; s2 += v2;
        if (fabs(v1 / s1) < 1e-15 && fabs(v2 / s2) < 1e-15) break;
    }
    return 0.5 * (s1 + log1p(-(1 - Z * Z) * s2));
}

// xi=0 EE/MM determinants are assembled and factored on the GPU
int logdetD0_batch(caps_t *self, const int *ms, int n, int which, double *out, double omegap);

extern "C" void caps_logdetD0(caps_t *self, int m, double omegap, double *EE, double *MM, double *MM_plasma)
{
    if (EE) logdetD0_batch(self, &m, 1, 0, EE, 0.0);
    if (MM) logdetD0_batch(self, &m, 1, 1, MM, 0.0);
    if (MM_plasma) logdetD0_batch(self, &m, 1, 2, MM_plasma, omegap);
}

extern "C" double caps_ht_perf(caps_t *caps, double eps)
{
    const double LbyR = caps->LbyR;
    const double drude = caps_ht_drude(caps);
    double MM = 0;
    const double Z = 1. / (1 + LbyR + sqrt(LbyR * (2 + LbyR)));
    for (int l = 0;; l++) {
        const double v = 0.5 * log1p(-pow(Z, 2 * l + 3));
        MM += v;
        if (fabs(v / MM) < eps) break;
    }
    // m = 1, 2, ... in batches of 16 on the GPU; summed up to the first m that meets the cutoff
    for (int m0 = 1;; m0 += 16) {
        int ms[16];
        double v[16];
        for (int k = 0; k < 16; k++) ms[k] = m0 + k;
        logdetD0_batch(caps, ms, 16, 1, v, 0.0);
        for (int k = 0; k < 16; k++) {
            MM += v[k];
            if (fabs(v[k] / MM) < eps) return drude + MM;
        }
    }
}

// libcaps.c:1127-1145: drude + sum'_m MM_plasma (m = 0 with weight 1/2) until the first m
// with |v / sum| < eps; m in batches of 16 on the GPU, summed in order up to that m
extern "C" double caps_ht_plasma(caps_t *caps, double omegap, double eps)
{
    const double drude = caps_ht_drude(caps);
    double sum = 0;
    for (int m0 = 0;; m0 += 16) {
        int ms[16];
        double v[16];
        for (int k = 0; k < 16; k++) ms[k] = m0 + k;
        logdetD0_batch(caps, ms, 16, 2, v, omegap);
        for (int k = 0; k < 16; k++) {
            sum += ms[k] == 0 ? v[k] / 2 : v[k];
            if (fabs(v[k] / sum) < eps) return drude + sum;
        }
    }
}

// ---------------------------------------------------------------------------
// free energy: Matsubara sum with the reference's truncation rules
// (src/caps.c:307-396 F_xi, :749-852 master), batched on the GPU
// ---------------------------------------------------------------------------
static double kahan_sum(const double *v, size_t n)
{
    double s = 0, c = 0;
    for (size_t i = 0; i < n; i++) { const double y = v[i] - c, t = s + y; c = (t - s) - y; s = t; }
    return s;
}

// which xi = 0 rule applies: 0 perfect reflectors, 1 Drude (analytic), 2 plasma; a
// tabulated material follows its low-frequency extrapolation (caps.c:782-803)
static int xi0_model(const caps_t *c)
{
    if (c->epsilonm1_plate == caps_epsilonm1_perf) return 0;
    if (c->epsilonm1_plate == caps_epsilonm1_drude && c->userdata_plate) {
        const double *p = (const double *)c->userdata_plate;
        return p[1] > 0 ? 1 : 2;
    }
    if (c->epsilonm1_plate == material_epsilonm1 && c->userdata_plate)
        return ((const material_t *)c->userdata_plate)->gamma_low > 0 ? 1 : 2;
    return 1;
}

// plasma frequency (rad/s) of the plasma model's xi = 0 term
static double xi0_omegap(const caps_t *c)
{
    if (c->epsilonm1_plate == material_epsilonm1) return ((const material_t *)c->userdata_plate)->omegap_low;
    return ((const double *)c->userdata_plate)[0];
}

struct MState {
    std::vector<double> v;  // logdetD per m (NAN = not yet computed)
    int mstop = -1;         // first m meeting the cutoff
    int next = 0;           // next m to schedule
    bool done() const { return mstop >= 0; }
};

// number of m to schedule next for one frequency, from the decay of the
// values so far (log-linear extrapolation to the cutoff), clamped
static int m_chunk(const MState &s, double cutoff)
{
    const int k = s.next;
    if (k < 8) return 32;
    const double v0 = s.v[0], a = fabs(s.v[k - 1]), b = fabs(s.v[k - 8]);
    if (!(a > 0) || !(b > a)) return 32;
    const double rate = log(b / a) / 7.0;          // e-folds per m
    const double need = log(a / (cutoff * fabs(v0))) / rate;
    int w = (int)ceil(need) + 4;
    return std::max(8, std::min(w, 256));
}

// first_chunk[i] (i < n_first): number of m to compute in the first batch for xi_{i+1}
// (from a proposal); nullptr: the extrapolating schedule of the plain method.
// F(xi_k) = sum'_m logdetD(xi_k, m) (m = 0 with weight 1/2) up to the first m with
// v_m == 0 or v_m / v_0 < cutoff, Kahan-summed in m order (caps.c:307-396), for n
// frequencies at once: the m chunks of every unfinished frequency share one GPU batch
// per round.  A non-finite term ends that frequency with F = NaN.
extern "C" int caps_logdetD2_batch(caps_t *self, const double *xi_, const int *m, int n, double *out, int *status);

// kind 1: the sphere-sphere sum of cass.c:78-92 instead -- logdet(1 - M^2) terms and
// 2 kahan(terms over 4096 slots) - term_0
void fxi_batch(caps_t *self, const double *xi, int n, double cutoff, double *out, int *ndet, int *nwasted, int kind)
{
    std::vector<MState> st(n);
    std::vector<char> bad(n, 0);
    for (;;) {
        std::vector<double> bx; std::vector<int> bm; std::vector<std::pair<int, int>> who;
        for (int i = 0; i < n; i++) {
            MState &s = st[i];
            if (s.done()) continue;
            TERMINATE(s.next >= 4096, "sum over m did not converge (xi_=%g)", xi[i]);
            const int w = std::min(m_chunk(s, cutoff), 4096 - s.next);
            for (int k = 0; k < w; k++) { bx.push_back(xi[i]); bm.push_back(s.next + k); who.push_back({i, s.next + k}); }
            s.next += w;
            s.v.resize(s.next, NAN);
        }
        if (bx.empty()) break;
        std::vector<double> r(bx.size());
        if (kind == 1) caps_logdetD2_batch(self, bx.data(), bm.data(), (int)bx.size(), r.data(), NULL);
        else caps_logdetD_batch(self, bx.data(), bm.data(), (int)bx.size(), r.data(), NULL);
        if (ndet) *ndet += (int)bx.size();
        for (size_t k = 0; k < bx.size(); k++) st[who[k].first].v[who[k].second] = r[k];
        for (int i = 0; i < n; i++) {
            MState &s = st[i];
            if (s.done()) continue;
            for (int m = 0; m < s.next; m++) {
                if (!std::isfinite(s.v[m])) { s.mstop = m; bad[i] = 1; break; }
                if (s.v[m] == 0 || s.v[m] / s.v[0] < cutoff) { s.mstop = m; break; }
            }
        }
    }
    for (int i = 0; i < n; i++) {
        MState &s = st[i];
        if (nwasted) *nwasted += s.next - (s.mstop + 1);
        if (bad[i]) { out[i] = NAN; continue; }
        std::vector<double> t(s.v.begin(), s.v.begin() + s.mstop + 1);
        if (kind == 1) {
            t.resize(4096, 0.0);
            out[i] = 2 * kahan_sum(t.data(), t.size()) - t[0];
            continue;
        }
        t[0] /= 2;
        out[i] = kahan_sum(t.data(), t.size());
    }
}

// xi = 0 term of the free energy by the reference's material rules (caps.c:329-395, 760-808)
double xi0_term(caps_t *self, double cutoff, int *ndet_, int *nwasted_)
{
    int ndet = 0, nwasted = 0;
    double v0;
    const int model = xi0_model(self);
    if (model == 1) v0 = caps_ht_drude(self);
    else {
        // drude_HT + sum'_m logdetD0 MM (perfect reflectors) or MM_plasma (plasma model)
        // with the m cutoff (caps.c:329-395, worker :921-929)
        const int which = model == 0 ? 1 : 2;
        const double omegap = model == 2 ? xi0_omegap(self) : 0.0;
        const double drude = caps_ht_drude(self);
        std::vector<double> terms;
        int mstop = -1;
        for (int m0 = 0; mstop < 0 && m0 < 4096; m0 += 32) {
            int ms[32]; double v[32];
            for (int k = 0; k < 32; k++) ms[k] = m0 + k;
            logdetD0_batch(self, ms, 32, which, v, omegap);
            ndet += 32;
            for (int k = 0; k < 32; k++) {
                terms.push_back(v[k]);
                if (mstop < 0 && (v[k] == 0 || v[k] / terms[0] < cutoff)) mstop = m0 + k;
            }
        }
        nwasted += (int)terms.size() - (mstop + 1);
        terms[0] /= 2;
        v0 = drude + kahan_sum(terms.data(), mstop + 1);
    }

    *ndet_ += ndet;
    *nwasted_ += nwasted;
    return v0;
}

static double energy_impl(caps_t *self, double T, double cutoff, double epsrel, const int *first_chunk, int n_first,
                          caps_energy_info_t *info)
{
    const auto t0 = std::chrono::steady_clock::now();
    TERMINATE(!(T > 0), "temperature must be positive");
    const double Ts = 2 * PI * CAPS_kB * (self->R + self->L) * T / (CAPS_hbar * CAPS_c);
    int ndet = 0, nwasted = 0;

    // xi = 0
    const double v0 = xi0_term(self, cutoff, &ndet, &nwasted);
    if (std::isnan(v0)) return NAN;

    std::vector<double> vn(1, v0);      // per-frequency sums, index n
    std::vector<MState> st;             // st[n-1] for xi_n
    int nmax_known = -1;                // n where |v_n/v_0| < epsrel
    int nactive = first_chunk ? std::max(1, n_first) : 4;
    st.resize(nactive);
    for (;;) {
        // schedule
        std::vector<double> bx; std::vector<int> bm; std::vector<std::pair<int, int>> who;
        const int nlim = nmax_known > 0 ? nmax_known : nactive;
        for (int i = 0; i < nlim; i++) {
            MState &s = st[i];
            if (s.done()) continue;
            int w = m_chunk(s, cutoff);
            if (s.next == 0 && first_chunk && i < n_first) w = std::max(1, first_chunk[i]);
            else if (s.next == 0 && !first_chunk)
                // a known cutoff of a neighbouring frequency sizes the first chunk
                for (int j = i - 1; j >= 0; j--)
                    if (st[j].done()) { w = std::min(w, st[j].mstop + 8); break; }
            for (int k = 0; k < w; k++) { bx.push_back((i + 1) * Ts); bm.push_back(s.next + k); who.push_back({i, s.next + k}); }
            s.next += w;
            s.v.resize(s.next, NAN);
        }
        if (bx.empty()) break;
        std::vector<double> out(bx.size());
        caps_logdetD_batch(self, bx.data(), bm.data(), (int)bx.size(), out.data(), NULL);
        ndet += (int)bx.size();
        for (size_t k = 0; k < bx.size(); k++) st[who[k].first].v[who[k].second] = out[k];
        for (int i = 0; i < nlim; i++) {
            MState &s = st[i];
            if (s.done()) continue;
            for (int m = 0; m < s.next; m++)
                if (s.v[m] == 0 || s.v[m] / s.v[0] < cutoff) { s.mstop = m; break; }
        }
        // Matsubara truncation in order of n
        if (nmax_known < 0) {
            bool grow = true;
            for (int i = 0; i < (int)st.size(); i++) {
                if (!st[i].done()) { grow = false; break; }
                std::vector<double> t(st[i].v.begin(), st[i].v.begin() + st[i].mstop + 1);
                t[0] /= 2;
                const double v = kahan_sum(t.data(), t.size());
                if (fabs(v / v0) < epsrel) { nmax_known = i + 1; grow = false; break; }
            }
            if (grow && nmax_known < 0) {
                // extrapolate |v_n/v_0| log-linearly from the last two complete frequencies
                int grow_to = nactive + 4;
                const int k = (int)st.size();
                if (k >= 2 && st[k - 1].done() && st[k - 2].done()) {
                    auto vsum = [&](const MState &s) {
                        std::vector<double> t(s.v.begin(), s.v.begin() + s.mstop + 1);
                        t[0] /= 2;
                        return fabs(kahan_sum(t.data(), t.size()));
                    };
                    const double a = vsum(st[k - 2]), b = vsum(st[k - 1]);
                    if (a > 0 && b > 0 && b < a) {
                        const double rate = log(a / b);
                        const double need = log(b / (epsrel * fabs(v0))) / rate;
                        grow_to = k + std::max(1, (int)ceil(need));
                    }
                }
                nactive = std::min(std::max(grow_to, nactive + 1), 2 * nactive);
                st.resize(nactive);
            }
        }
        if (nmax_known > 0) {
            bool all = true;
            for (int i = 0; i < nmax_known; i++) all = all && st[i].done();
            if (all) break;
        }
        TERMINATE(nactive > 4096, "Matsubara sum did not converge");
    }
    for (int i = 0; i < (int)st.size(); i++) {
        if (i < nmax_known) nwasted += st[i].next - (st[i].mstop + 1);
        else nwasted += st[i].next;
    }
    for (int i = 0; i < nmax_known; i++) {
        std::vector<double> t(st[i].v.begin(), st[i].v.begin() + st[i].mstop + 1);
        t[0] /= 2;
        vn.push_back(kahan_sum(t.data(), t.size()));
    }
    if (info) {
        info->nxi = (int)vn.size();
        info->ndet = ndet;
        info->nwasted = nwasted;
        for (size_t i = 0; i < vn.size() && i < 4096; i++) {
            if (info->xi) info->xi[i] = i * Ts;
            if (info->logdetD) info->logdetD[i] = vn[i];
        }
    }
    std::vector<double> w(vn);
    w[0] /= 2;
    const double E = Ts / PI * kahan_sum(w.data(), w.size());
    if (info) info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return E;
}

extern "C" double caps_free_energy(caps_t *self, double T, double cutoff, double epsrel, caps_energy_info_t *info)
{
    return energy_impl(self, T, cutoff, epsrel, nullptr, 0, info);
}

// material features of the learned proposal: perfect reflectors are encoded as
// omega_p = 50 eV, gamma = 0; Drude callbacks carry (omega_p, gamma) in rad/s
static bool material_features(const caps_t *c, double *wp_eV, double *g_eV)
{
    if (c->epsilonm1_plate == caps_epsilonm1_perf) { *wp_eV = 50.0; *g_eV = 0.0; return true; }
    if (c->epsilonm1_plate == caps_epsilonm1_drude && c->userdata_plate) {
        const double *p = (const double *)c->userdata_plate;
        *wp_eV = p[0] * CAPS_hbar_eV;
        *g_eV = p[1] * CAPS_hbar_eV;
        return true;
    }
    return false;
}

extern "C" void caps_mlp_features(double RbyL, double xi_, int m, double omegap_eV, double gamma_eV, float *x);
extern "C" void caps_mlp_predict(caps_mlp_t *m, const float *X, int n, float *y);

extern "C" int caps_mlp_proposal(caps_t *self, double T, double cutoff, double epsrel, caps_mlp_t *mlp, int nmax, int *mchunk)
{
    double wp, ga;
    if (!material_features(self, &wp, &ga)) return -1;
    const double Ts = 2 * PI * CAPS_kB * (self->R + self->L) * T / (CAPS_hbar * CAPS_c);
    const int MCAP = 1024, NPROBE = std::min(nmax, 256), NB = 16;
    // the xi = 0 term (analytic for Drude; drude term as the scale for other materials)
    const double v0 = fabs(caps_ht_drude(self));
    const double lc = log(cutoff);
    // frequencies in blocks of NB, stopping at the first block that reaches the Matsubara
    // cutoff; features as caps_mlp_features forms them
    std::vector<float> X((size_t)NB * MCAP * 5), Y((size_t)NB * MCAP);
    for (int n0 = 1; n0 <= NPROBE; n0 += NB) {
        const int nb = std::min(NB, NPROBE - n0 + 1);
        for (int k = 0; k < nb; k++)
            for (int m = 0; m < MCAP; m++)
                caps_mlp_features(1.0 / self->LbyR, (n0 + k) * Ts, m, wp, ga, &X[((size_t)k * MCAP + m) * 5]);
        caps_mlp_predict(mlp, X.data(), nb * MCAP, Y.data());
        for (int k = 0; k < nb; k++) {
            const int n = n0 + k;
            const float *y = &Y[(size_t)k * MCAP];
            int mstop = MCAP - 1;
            for (int m = 1; m < MCAP; m++)
                if (y[m] - y[0] < lc) { mstop = m; break; }
            mchunk[n - 1] = mstop + 1 + 2; // two extra m beyond the predicted cutoff
            double v = 0.5 * exp((double)y[0]);
            for (int m = 1; m <= mstop; m++) v += exp((double)y[m]);
            if (v / v0 < epsrel) return n;
        }
    }
    return NPROBE;
}

extern "C" double caps_free_energy_learned(caps_t *self, double T, double cutoff, double epsrel, caps_mlp_t *mlp,
                                           caps_energy_info_t *info)
{
    std::vector<int> chunk(256, 32);
    const int N = mlp ? caps_mlp_proposal(self, T, cutoff, epsrel, mlp, 256, chunk.data()) : -1;
    if (N <= 0) return energy_impl(self, T, cutoff, epsrel, nullptr, 0, info);
    return energy_impl(self, T, cutoff, epsrel, chunk.data(), N, info);
}
