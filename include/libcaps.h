/*
 * libcaps.h -- GB300 implementation of the CaPS v0.5 public C API for the
 * round-trip-matrix log-det path (plane-sphere Casimir geometry).
 *
 * Every reference prototype below keeps the reference's name, argument meaning
 * and error behaviour; the comment beside each names the reference
 * declaration (src/include/libcaps.h) and definition it replaces.  All
 * matrix assembly and factorisation runs on the GPU; the host evaluates the
 * dielectric callbacks once per frequency and ships the scalars.
 *
 * Error behaviour: contract violations (xi <= 0, as in the reference) print a
 * message and abort(); a missing or failing CUDA device prints and aborts (no
 * CPU fallback); numerical trouble inside a kernel yields NaN for that matrix
 * and a status code, readable through caps_gpu_last_error().
 */
#ifndef LIBCAPS_H
#define LIBCAPS_H

#include <stdarg.h>
#include <stdbool.h>
#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/include/libcaps.h:17 */
typedef enum { TE, TM } polarization_t;
/* src/include/matrix.h:14 */
typedef enum { DETALG_HODLR, DETALG_LU, DETALG_QR, DETALG_CHOLESKY } detalg_t;
/* src/include/constants.h:15 */
typedef signed char sign_t;

/* src/include/constants.h:45-48 */
#define CAPS_hbar    1.0545718e-34
#define CAPS_hbar_eV 6.582119514e-16
#define CAPS_kB      1.38064852e-23
#define CAPS_c       299792458.

/* src/include/libcaps.h:29-33 */
#define CAPS_MINIMUM_LDIM 20
#define CAPS_FACTOR_LDIM 5
#define CAPS_EPSREL 1e-8

/* The CaPS object.  The public fields keep the layout of the reference
 * (src/include/libcaps.h:41-78); private GPU settings follow them. */
typedef struct caps
{
    double L;    /* separation of plane and sphere */
    double R;    /* radius of sphere */
    double calL; /* L+R */
    double LbyR; /* L/R */
    double y;    /* log(R/(R+L)/2) */
    double (*epsilonm1_plate)(double xi_, void *userdata);
    void *userdata_plate;
    double (*epsilonm1_sphere)(double xi_, void *userdata);
    void *userdata_sphere;
    int ldim;
    double epsrel;
    detalg_t detalg;
    /* private: arithmetic of the factorisation, see caps_gpu_set_precision */
    int precision;
    /* private: determinant path under DETALG_HODLR, see caps_gpu_set_path */
    int path;
} caps_t;

/* Matrix object of one (xi, m) (src/include/libcaps.h:101-109).  The GPU
 * builds the whole matrix at caps_M_init; caps_M_elem serves it. */
typedef struct
{
    caps_t *caps;
    int m, lmin, ldim;
    void *integration;        /* unused; kept for layout */
    void *integration_plasma; /* unused; kept for layout */
    double xi_;
    double *al, *bl;          /* log|a_l|, log|b_l| for l = lmin .. lmin+ldim-1 */
    double *M;                /* private: dense M, row-major 2ldim x 2ldim */
} caps_M_t;

/* Plasma-model xi=0 integration object (src/include/libcaps.h:93-98).  The public
 * fields keep the reference's meaning; the two pointers are private (GPU-computed
 * tables served to the element-wise interface). */
typedef struct
{
    double LbyR, alpha, omegap_, epsrel;
    void *cache;
    void *cache_ratio;
} integration_plasma_t;

/* ---- reference API (src/include/libcaps.h:113-163) ---- */
void caps_build(FILE *stream, const char *prefix);                 /* libcaps.h:113, libcaps.c:239 */
void caps_info(caps_t *self, FILE *stream, const char *prefix);    /* libcaps.h:114, libcaps.c:273 */

double caps_lnLambda(int l1, int l2, int m);                        /* libcaps.h:116, libcaps.c:45 */

caps_t *caps_init(double R, double L);                              /* libcaps.h:118, libcaps.c:183 */
void caps_free(caps_t *self);                                       /* libcaps.h:119, libcaps.c:224 */

double caps_epsilonm1_plate(caps_t *self, double xi_);              /* libcaps.h:121, libcaps.c:104 */
double caps_epsilonm1_sphere(caps_t *self, double xi_);             /* libcaps.h:122, libcaps.c:116 */

void caps_set_epsilonm1(caps_t *self, double (*epsilonm1)(double xi_, void *userdata), void *userdata);        /* libcaps.h:124, libcaps.c:337 */
void caps_set_epsilonm1_plate(caps_t *self, double (*epsilonm1)(double xi_, void *userdata), void *userdata);  /* libcaps.h:125, libcaps.c:358 */
void caps_set_epsilonm1_sphere(caps_t *self, double (*epsilonm1)(double xi_, void *userdata), void *userdata); /* libcaps.h:126, libcaps.c:379 */

int caps_get_ldim(caps_t *self);                                    /* libcaps.h:128, libcaps.c:454 */
int caps_set_ldim(caps_t *self, int ldim);                          /* libcaps.h:129, libcaps.c:436 */

detalg_t caps_get_detalg(caps_t *self);                             /* libcaps.h:131, libcaps.c:418 */
int caps_set_detalg(caps_t *self, detalg_t detalg);                 /* libcaps.h:132, libcaps.c:400 */

double caps_get_epsrel(caps_t *self);                               /* libcaps.h:134, libcaps.c:322 */
int    caps_set_epsrel(caps_t *self, double epsrel);                /* libcaps.h:135, libcaps.c:306 */

void caps_mie(caps_t *self, double xi_, int l, double *lna, double *lnb);       /* libcaps.h:137, libcaps.c:557 */
void caps_mie_perf(caps_t *self, double xi_, int l, double *lna, double *lnb);  /* libcaps.h:138, libcaps.c:485 */

double caps_kernel_M(int i, int j, void *args_);                    /* libcaps.h:140, libcaps.c:717 */

caps_M_t *caps_M_init(caps_t *self, int m, double xi_);             /* libcaps.h:142, libcaps.c:673 */
double caps_M_elem(caps_M_t *self, int l1, int l2, char p1, char p2); /* libcaps.h:143, libcaps.c:761 */
void caps_M_free(caps_M_t *self);                                   /* libcaps.h:144, libcaps.c:840 */

double caps_logdetD(caps_t *self, double xi_, int m);               /* libcaps.h:146, libcaps.c:950 */

void caps_fresnel(caps_t *self, double xi_, double k, double *r_TE, double *r_TM); /* libcaps.h:148, libcaps.c:616 */

int caps_estimate_lminmax(caps_t *self, int m, size_t *lmin_p, size_t *lmax_p);   /* libcaps.h:150, libcaps.c:63 */

double caps_epsilonm1_perf(double xi_, void *userdata);             /* libcaps.h:152, libcaps.c:129 */
double caps_epsilonm1_drude(double xi_, void *userdata);            /* libcaps.h:153, libcaps.c:150 */

double caps_ht_drude(caps_t *caps);                                 /* libcaps.h:155, libcaps.c:1043 */
double caps_ht_perf(caps_t *caps, double eps);                      /* libcaps.h:156, libcaps.c:1089 */
double caps_ht_plasma(caps_t *caps, double omegap_, double eps);    /* libcaps.h:157, libcaps.c:1127 */

double caps_kernel_M0_EE(int i, int j, void *args);                 /* libcaps.h:159, libcaps.c:860 */
double caps_kernel_M0_MM(int i, int j, void *args);                 /* libcaps.h:160, libcaps.c:920 */
double caps_kernel_M0_MM_plasma(int i, int j, void *args_);         /* libcaps.h:161, libcaps.c:882 */

void caps_logdetD0(caps_t *self, int m, double omegap, double *EE, double *MM, double *MM_plasma); /* libcaps.h:163, libcaps.c:985 */

/* ---- tabulated materials (src/include/material.h:11-30) ---- */
typedef struct {
    char filename[512]; /* material file */
    double calL;        /* L+R */
    double xi_min;      /* lowest tabulated frequency (rad/s) */
    double xi_max;      /* highest tabulated frequency (rad/s) */
    size_t points;      /* number of tabulated points */
    double *xi;         /* tabulated frequencies (rad/s) */
    double *epsm1;      /* tabulated eps(i xi) - 1 */
    double omegap_low;  /* Drude extrapolation below the table (rad/s) */
    double gamma_low;
    double omegap_high; /* Drude extrapolation above the table (rad/s) */
    double gamma_high;
} material_t;
material_t *material_init(const char *filename, double calL);            /* material.h:24, material.c:63 */
void material_info(material_t *material, FILE *stream, const char *prefix); /* material.h:25, material.c:225 */
void material_free(material_t *material);                                 /* material.h:26, material.c:205 */
void material_get_extrapolation(material_t *material, double *omegap_low, double *gamma_low, double *omegap_high,
                                double *gamma_high);                      /* material.h:28, material.c:189 */
double material_epsilonm1(double xi, void *args);                         /* material.h:30, material.c:251 */

/* ---- plasma xi=0 integrals (src/include/integration.h:24-26) ---- */
integration_plasma_t *caps_integrate_plasma_init(caps_t *caps, double omegap, double epsrel); /* integration.h:24, integration.c:897 */
double caps_integrate_plasma(integration_plasma_t *self, int l1, int l2, int m, double *ratio1, double *ratio2); /* integration.h:25, integration.c:954 */
void caps_integrate_plasma_free(integration_plasma_t *self);                                   /* integration.h:26, integration.c:1026 */

/* ---- batch extensions (no reference counterpart; additive) ---- */

/* status codes of a batch entry */
#define CAPS_ST_TRACE     1   /* trace shortcut |tr M| < 1e-8 (matrix.c:78) */
#define CAPS_ST_MERCATOR  2   /* Mercator shortcut (matrix.c:494-505) */
#define CAPS_ST_FACTOR    3   /* full factorisation */
#define CAPS_ST_ERR_PIVOT 16  /* non-positive pivot: result NaN */
#define CAPS_ST_ERR_NONFINITE 32 /* non-finite integral or element: result NaN */
#define CAPS_ST_ERR_GRID  64  /* quadrature grid exceeded its node budget: result NaN */
#define CAPS_ST_ERR_WAIT  128 /* a bounded wait for the tensor cores ran out: result NaN */
#define CAPS_ST_ERR_HODLR 256 /* HODLR block rank over its limit (the batch call then factors it densely) */
#define CAPS_ST_ERR_RANGE 512 /* mixed form: a factor entry |x| >= 4 (impossible for 1-M positive definite
                                 with |M_ii| < 1), outside the range of its FP16 panel images: result NaN */

/* log det(1-M) for n (xi_[i], m[i]) pairs of one geometry, all matrices
 * assembled and factored as one GPU batch (replaces n calls of caps_logdetD,
 * the per-task worker at src/caps.c:946).  status may be NULL.
 * Returns the number of entries with an error status (0 on full success). */
int caps_logdetD_batch(caps_t *self, const double *xi_, const int *m, int n, double *out, int *status);

/* precision of the factorisation */
#define CAPS_PREC_FP64  0  /* plain FP64 Cholesky */
#define CAPS_PREC_MIXED 1  /* tensor-core factorisation + FP64 log-det correction */
int caps_gpu_set_precision(caps_t *self, int precision);

/* determinant path of an FP64 caps object with DETALG_HODLR (the default): a HODLR
 * factorisation with the elements evaluated on demand (src/libhodlr, matrix.c:125-147) or the
 * dense batched Cholesky with the same result rules.  Automatic: HODLR from dimension
 * CAPS_HODLR_AUTO_DIM on (where sampling the off-diagonal blocks needs fewer q-sums than the
 * dense I table).  The mixed form takes HODLR only when asked (CAPS_PATH_HODLR or the
 * autotuner); its sampled elements then come from the float-float q-sums, its compression and
 * factorisation stay FP64.  Returns 1, or 0 for an unknown path. */
#define CAPS_PATH_AUTO  0
#define CAPS_PATH_HODLR 1
#define CAPS_PATH_DENSE 2
#define CAPS_HODLR_AUTO_DIM 4000
#define CAPS_HODLR_AUTO_DIM_MIXED 1000000000 /* the mixed form factors densely unless asked */
int caps_gpu_set_path(caps_t *self, int path);

/* Autotuner (no reference counterpart): times the candidate schedules for this object's
 * dimension and precision on nprobe matrices of its own workload (xi_, m = 0 .. nprobe-1)
 * and keeps the fastest.  Mixed form: the tensor-core trailing update's schedule (0 panel
 * images by bulk copies, 1 panel staged through registers, 2 one CTA per tile), kept for the
 * dimension for the rest of the process, and under DETALG_HODLR candidate 3, the HODLR path;
 * FP64 under DETALG_HODLR: the determinant path (0 dense, 1 HODLR).  The chosen path is
 * stored in the object as by caps_gpu_set_path.  info (optional) receives
 * the device milliseconds per matrix of each candidate.  Returns 1, or 0 for bad arguments. */
typedef struct {
    int ncand;               /* candidates timed */
    int chosen;              /* index of the fastest */
    double ms_per_matrix[4]; /* device time per matrix of each candidate */
} caps_autotune_info_t;
int caps_gpu_autotune(caps_t *self, double xi_, int nprobe, caps_autotune_info_t *info);

/* Free energy E (L+R)/(hbar c) at temperature T via the Matsubara sum with the
 * reference's m cutoff and xi truncation (src/caps.c:307-396, 749-852).
 * The xi = 0 term follows the reference's material rules.  info arrays may be
 * NULL.  Returns E; nxi/ndet report the frequencies and determinants used. */
typedef struct {
    int nxi;          /* number of frequencies including xi = 0 */
    int ndet;         /* number of (xi,m) determinants evaluated on the GPU */
    int nwasted;      /* determinants computed beyond the cutoff (speculation) */
    double seconds;   /* wall time */
    double *xi;       /* optional [4096]: xi (L+R)/c per frequency */
    double *logdetD;  /* optional [4096]: m-summed term per frequency */
} caps_energy_info_t;
double caps_free_energy(caps_t *self, double T, double cutoff, double epsrel, caps_energy_info_t *info);

/* Free energy at T = 0 (src/caps.c:722-748): E = 1/(alpha pi) int_0^inf dx F(x/alpha),
 * x = 2 xi L/c, alpha = 2L/(L+R), with the reference's PFA cut of the integrand
 * (caps.c:235-267).  method 0: QUADPACK qagi with relative tolerance epsrel (the
 * reference's default); 1: Fourier-Chebyshev quadrature (fcqs.c:107).  Every step's
 * function values are evaluated as one GPU batch.  info (optional): nxi = integrand
 * evaluations; xi/logdetD record the first 4096 of them. */
double caps_free_energy_T0(caps_t *self, double cutoff, double epsrel, int method, caps_energy_info_t *info);
/* Free energy at T = 0 by an n-point Gauss-Laguerre rule in x = 2 xi L/c (no reference
 * counterpart; the reference integrates the same E = 1/(alpha pi) int_0^inf dx F(x/alpha)
 * adaptively): all n frequencies and their m sums in one batch, the PFA cut as above. */
double caps_free_energy_T0_gl(caps_t *self, double cutoff, int n, caps_energy_info_t *info);
/* the n-point Gauss-Laguerre rule (n <= 200): nodes x and weights times e^x; returns 1 */
int caps_gauss_laguerre(int n, double *x, double *w_ex);
/* Free energy at T > 0 by Pade spectrum decomposition (src/caps.c:811-831) of the given
 * order (<= 0: the reference's automatic order, caps.c:635-639); all poles in one batch. */
double caps_free_energy_psd(caps_t *self, double T, double cutoff, double epsrel, int order, caps_energy_info_t *info);

/* Sphere-sphere geometry (the reference's cass program, src/cass.c): two spheres of radius
 * R at separation d, for perfect reflectors as cass computes them.  Create the object with
 * caps_init(R, d/2): the round trip is M^2 with M the plane-sphere round trip at L = d/2.
 * caps_logdetD2_batch: log det(1 - M^2) per (xi, m) (cass.c:23-64: trace shortcut below
 * 1e-8, dense Mercator rule, else factorisation; FP64).  caps_sphere_sphere_T0: the T = 0
 * energy E d/(hbar c) (cass.c:66-92, 210-219: qagi over y = xi d/c of 2 sum_m - m=0 term). */
int caps_logdetD2_batch(caps_t *self, const double *xi_, const int *m, int n, double *out, int *status);
double caps_sphere_sphere_T0(caps_t *self, double cutoff, double epsrel, caps_energy_info_t *info);

/* The quadratures and PSD poles behind these drivers, on a host callback: the same
 * algorithms as the reference's dqagi (cquadpack/src/dqagi.c:40), fcqs_semiinf
 * (src/fcqs.c:107) and psd (src/psd.c:80), with the same arguments and results. */
double caps_dqagi(double (*f)(double, void *), void *userdata, double bound, int inf, double epsabs, double epsrel,
                  double *abserr, int *neval, int *ier);
double caps_fcqs_semiinf(double (*f)(double, void *), void *userdata, double *epsrel, int *neval, double L, int *ier);
int caps_psd(int N, double *xi, double *eta);

/* ---- learned truncation (no reference counterpart) ----
 * A 5-64-64-64-1 SiLU network (FP32), trained on the GPU by the library's own
 * forward/backward/Adam kernels on log|logdetD| values computed by the plain
 * method, predicts log|logdetD(xi, m)| from (log R/L, log xi_, m, omega_p,
 * gamma).  caps_free_energy_learned() uses it to propose the m cutoff of every
 * Matsubara frequency and the number of frequencies, computes the proposed
 * matrices as one GPU batch, then applies the reference's cutoff rules to the
 * computed values and extends the batch where the proposal fell short -- so
 * its result is the plain method's result. */
typedef struct caps_mlp caps_mlp_t;
caps_mlp_t *caps_mlp_create(unsigned seed);
void caps_mlp_free(caps_mlp_t *mlp);
int caps_mlp_nparams(void);
void caps_mlp_get_params(caps_mlp_t *mlp, float *out);
void caps_mlp_set_params(caps_mlp_t *mlp, const float *in);
/* features of one sample (5 floats) in the normalisation the network uses */
void caps_mlp_features(double RbyL, double xi_, int m, double omegap_eV, double gamma_eV, float *x);
/* mean squared error of a batch and (if grad != NULL) its gradient w.r.t. all parameters */
double caps_mlp_loss_grad(caps_mlp_t *mlp, const float *X, const float *y, int n, float *grad);
/* full-batch Adam for the given epochs; returns the final loss */
double caps_mlp_train(caps_mlp_t *mlp, const float *X, const float *y, int n, int epochs, float lr);
void caps_mlp_predict(caps_mlp_t *mlp, const float *X, int n, float *y);
/* proposal: mchunk[n-1] = number of m to compute for xi_n; returns the number of frequencies (<= nmax) */
int caps_mlp_proposal(caps_t *self, double T, double cutoff, double epsrel, caps_mlp_t *mlp, int nmax, int *mchunk);
double caps_free_energy_learned(caps_t *self, double T, double cutoff, double epsrel, caps_mlp_t *mlp, caps_energy_info_t *info);

/* last error text of this thread's most recent GPU call ("" if none) */
const char *caps_gpu_last_error(void);

/* run subsequent GPU work on this CUDA stream (a cudaStream_t; NULL = library stream) */
void caps_gpu_set_stream(void *stream);

/* device time of the phases, milliseconds, measured with CUDA events on the
 * library's stream: [0] setup+Mie, [1] K integrals, [2] I integrals,
 * [3] elements+stats, [4] factorisation, [5] total of the most recent batch;
 * [6..11] the same phases summed since caps_gpu_reset_timings(); returns the
 * number written (at most 12) */
int caps_gpu_timings(double *ms, int n);
void caps_gpu_reset_timings(void);

/* kernel launches and host<->device bytes since the last reset */
void caps_gpu_counters(long long *launches, long long *h2d_bytes, long long *d2h_bytes, int reset);

/* matrices assembled, matrices factored and the algorithmic flops of those
 * factorisations (n^3/3 each) since the last counter reset */
void caps_gpu_work(long long *nmat, long long *nfactor, double *factor_flops);

/* live timing of the mixed form's factorisation kernels: with caps_gpu_kernel_timing(1),
 * CUDA events on the library's stream bracket every launch; caps_gpu_kernel_stats returns
 * for the tcgen05 updates the summed device milliseconds, the algorithmic bytes (target
 * block read and written once plus the panel rows, per factored matrix) and the launch
 * count since the last enable; caps_gpu_kernel_stats_kind the same for kind 0 (updates),
 * 1 (panel solve: the panel rows read, X or its FP16 image written) or 2 (diagonal block:
 * read, written, its inverse written).
 * caps_gpu_kernel_timing(0) stops it. */
void caps_gpu_kernel_timing(int enable);
void caps_gpu_kernel_stats(double *ms, double *bytes, long long *launches);
void caps_gpu_kernel_stats_kind(int kind, double *ms, double *bytes, long long *launches);

/* measured FP64 FMA throughput of the current device, TFLOP/s (a short probe kernel) */
double caps_gpu_fp64_peak(void);
/* measured FP32 FMA throughput of the current device, TFLOP/s (a short probe kernel) */
double caps_gpu_fp32_peak(void);

/* log det(1-M) of one (xi_, m), like caps_logdetD, for callers that cannot
 * allocate device memory at call time (a framework that owns the whole device
 * through its own pool allocator, where an outside cudaMalloc can fail or
 * fragment the pool).  No counterpart in the reference.  All scratch lives in
 * one fixed 32 MiB file-scope device array (held on every GPU that loads the
 * library until exit); no cudaMalloc/cudaFree or allocating library call is made.
 * Limits: ldim <= 512, lmin+ldim <= 2048, <= 256 K-quadrature panels; larger
 * cases return a negative code with a message (caps_noalloc_last_error(), per
 * host thread).  The first call on a device resolves the array's address
 * (cudaGetSymbolAddress) and uploads constant tables: make it before any stream
 * capture.  Calls share the array: calls that overlap on the GPU race.  Runs on
 * the legacy default stream and synchronises the host with it before returning.
 * A failed kernel launch aborts, as in every entry point of the library.
 * Returns 0, a negative code for rejected input or a failed CUDA API call, or
 * the status bits of a numerical failure (CAPS_ST_ERR_*); *logdet receives the
 * result. */
int caps_logdetD_noalloc(caps_t *self, double xi_, int m, double *logdet);
const char *caps_noalloc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif
