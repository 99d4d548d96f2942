// internal.h -- launchers shared between the translation units of the library.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <cuda_runtime.h>
#include "common.cuh"

// contract violation: same behaviour as the reference's TERMINATE (utils.h:31)
#define TERMINATE(cond, ...)                                                              \
    do {                                                                                  \
        if (cond) {                                                                       \
            fprintf(stderr, "libcaps_gb300: %s:%d: ", __FILE__, __LINE__);               \
            fprintf(stderr, __VA_ARGS__);                                                 \
            fprintf(stderr, "\n");                                                        \
            abort();                                                                      \
        }                                                                                 \
    } while (0)

namespace capsgpu {

[[noreturn]] void fatal(const char *file, int line, const char *what);
#define CK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) ::capsgpu::fatal(__FILE__, __LINE__, cudaGetErrorString(e_)); } while (0)

// counters of kernel launches and host<->device bytes since the last reset
struct Counters { long long launches = 0, h2d = 0, d2h = 0, nfactor = 0, nmat = 0; double factor_flops = 0; };
extern Counters g_counters;
#define COUNT_LAUNCH(n) (::capsgpu::g_counters.launches += (n))

void upload_gauss_legendre(const double *x, const double *w);
void launch_setup(Task *tasks, int ntask, double *edges, int max_panels, double2 *coefAB, int nu_stride, double c_width,
                  int *status, cudaStream_t st);
void launch_mie(const double *xi, const double *epsm1, int nxi, double LbyR, int lmax, double *lna, double *lnb, cudaStream_t st);
void launch_scale(const Task *tasks, int ntask, int ldim, const double *lna, const double *lnb, int lmax, const double *lfac_tab,
                  sd *Sa, sd *Sb, double2 *uv, cudaStream_t st);
size_t ktab_smem_bytes();
void launch_ktab(bool pr, const Task *tasks, int ntask, int max_warps, const double *edges, int max_panels, const double2 *coefAB,
                 int nu_stride, const double *lfac_tab, double *partM, int *partE, cudaStream_t st);
void launch_kred(const Task *tasks, int ntask, int max_nnu, const double *partM, const int *partE, int max_warps, int nu_stride,
                 sd *K, int *status, cudaStream_t st);
// mixed form: the K integrals in float-float
struct ffe;
void launch_ktab_ff(bool pr, const Task *tasks, int ntask, int max_warps, const double *edges, int max_panels, const double2 *coefAB,
                    float4 *coefF, int nu_stride, const double *lfac_tab, float2 *partF, int *partE, cudaStream_t st);
// KP, KPe: TM and TE of one (task, nu) under one exponent, the table the q-sums read
void launch_kred_ff(const Task *tasks, int ntask, int max_nnu, const float2 *partF, const int *partE, int max_warps, int nu_stride,
                    float4 *KP, int *KPe, int *status, cudaStream_t st);
void launch_tables(const double *lfac_tab, double *lft, int nlf, double2 *xtab, int nx, cudaStream_t st);
struct ffe;
// FP64 q-sums of the listed tasks (tlist, nlist; tlist == nullptr: tasks 0..nlist-1); band:
// only the pairs the diagonal reads.  The p tables come first (launch_ptab).
void launch_ptab(const Task *tasks, int ntask, double4 *ptab, int pstride, cudaStream_t st);
void launch_itab(const Task *tasks, const int *tlist, int nlist, int ldim, const sd *K, int nu_stride, const double *lft,
                 const double2 *xtab, const double4 *ptab, int pstride, sd *I, int *status, cudaStream_t st, const void *a12,
                 bool band);
// float-float q recurrence tables once per distinct m (group_m), row g per group
void launch_ptab_groups(const int *group_m, int ngroup, float4 *ptabf, int pstride, cudaStream_t st);
// mixed form: q-sums of every pair with one a_q recurrence per (pair, subgroup of same-m tasks)
// (itab_ff.cu); groups index tlist (nullptr: the tasks themselves).  The p tables come first
// (launch_ptab_groups).
int itab_group_size();
void launch_itab_grp(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim, const float4 *KP,
                     const int *KPe, int nu_stride, const float4 *ptabf, int pstride, const void *a12, void *Iout, bool ffe_out,
                     int *status, cudaStream_t st);
// sphere-sphere: B = 1 - M^2 and (M^2)_ii from A = 1 - M and M_ii (square.cu)
void launch_square(int ntask, int n, const double *A, size_t lda, size_t mstride, const double *mdiag, double *B,
                   const int *status, double *mdiag2, cudaStream_t st);
// a_0, a_1, a_2 per distinct m of a chunk (groups), shared by all frequencies
void launch_a12(const int *group_m, const int *group_lmin, int ngroup, int ldim, const double *lft, void *tab, cudaStream_t st);
size_t a12_bytes(int ldim, int ngroup);
// mixed form: the same from per-m tables (work: a12_tab_bytes of scratch)
size_t a12_tab_bytes(int ldim, int ngroup);
// tabs: the per-m tables first; then every pair of the listed groups (glist == nullptr: groups
// 0..nlist-1, nlist < 0: all)
void launch_a12_mixed(const int *group_m, const int *group_lmin, int ngroup, int ldim, const double *lft, void *tab, void *work,
                      cudaStream_t st, bool tabs = true, const int *glist = nullptr, int nlist = -1);
// elements of the listed tasks into A = 1 - M and M_ii; diag_only: M_ii alone (from the band)
void launch_elem(const Task *tasks, const int *tlist, int nlist, int ldim, const sd *I, const sd *Sa, const sd *Sb, const double2 *uv,
                 double *A, size_t lda, size_t mat_stride, double *mdiag, int *status, cudaStream_t st, bool diag_only);
// shortcut decision of the listed tasks; A == nullptr: the trace rule alone, undecided tasks keep status 0
void launch_stats(const int *tlist, int nlist, int n, const double *A, size_t lda, size_t mat_stride, const double *mdiag, int mode,
                  double *trace, double *result, int *status, cudaStream_t st);
// mixed form: elements in float-float straight into the FP32 delta matrix (elem_ff.cu)
size_t elem_ff_part_floats(int ldim);
// float-float copies of the scale factors (Saf, Sbf: L ffe per task; uvf: L float4 per task)
void launch_scale_ff(int ntask, int ldim, const sd *Sa, const sd *Sb, const double2 *uv, void *Saf, void *Sbf, float4 *uvf,
                     cudaStream_t st);
// q-sums of seed pairs at every window index w (sweep.cu), one array of L float-float values per
// (task, polarisation, kind): seed[((task * 2 + pol) * SEED_KINDS + kind) * L + w] holds the pair
// (w, w), (w+1, w), (w+2, w) or (w, c), c the window index of the first l with I != 0
enum { SEED_D0 = 0, SEED_D1 = 1, SEED_D2 = 2, SEED_COL = 3, SEED_KINDS = 4 };
size_t seed_bytes(int ldim, int ntask);
// band: kinds D0 and D2 (what the diagonal of M reads); otherwise D1 and COL (the rest of the
// recurrence's seeds).  a12t: the per-m tables of launch_a12_mixed (ngroup_all groups)
void launch_seed_ff(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim, const float4 *KP, const int *KPe,
                    int nu_stride, const float4 *ptabf, int pstride, const void *a12t, int ngroup_all, void *seed, bool band,
                    int *status, cudaStream_t st);
// M of the listed tasks by the I recurrence from all four seed kinds, straight into the FP32
// delta matrix, with one sum of squares per task in part[task]; sweep_fits: the window fits the
// kernel's shared-memory ring
bool sweep_fits(int ldim);
void launch_sweep_ff(const Task *tasks, const int *tlist, int nlist, int ldim, const void *seed, const void *Saf, const void *Sbf,
                     float *S, size_t sstride, float *part, int *status, cudaStream_t st);
// the diagonal of M alone, from the band seeds
void launch_diag_ff(const Task *tasks, int ntask, int ldim, const void *seed, const void *Saf, const void *Sbf, const float4 *uvf,
                    double *diag, int *status, cudaStream_t st);
// the listed tasks (tlist, nlist; tlist == nullptr: tasks 0..nlist-1)
void launch_elem_ff(const Task *tasks, const int *tlist, int nlist, int ldim, const void *Saf, const void *Sbf, const float4 *uvf,
                    const void *I, float *S, size_t sstride, double *diag, float *part, int *status, cudaStream_t st);
// part == nullptr: the trace rule alone, undecided tasks keep status 0; part_per_task: part holds
// one sum of squares per task (launch_sweep_ff), otherwise k_elem_ff's per-warp partials
void launch_stats_ff(const int *tlist, int nlist, int ldim, const double *diag, const float *part, int mode, double *trace,
                     double *result, int *status, cudaStream_t st, bool part_per_task = false);
void launch_cholesky(int ntask, int n, double *A, size_t lda, size_t mstride, int *status, double *logdiag, cudaStream_t st);
size_t mixed_work_bytes(int ntask, int n);
// live CUDA-event timing of the tcgen05 trailing update (mixed.cu)
void kernel_timer_enable(bool on);
void kernel_timer_collect(long long nfactored);
enum { KT_SYRK = 0, KT_TRSM = 1, KT_POTF2 = 2, KT_KINDS = 3 };
void kernel_timer_stats(int kind, double *ms, double *bytes, long long *launches);
// schedules of the mixed form's trailing update
enum { MIXED_SCHED_IMAGES = 0, MIXED_SCHED_REGSTAGE = 1, MIXED_SCHED_PER_TILE = 2, MIXED_SCHED_COUNT = 3 };
void launch_cholesky_mixed(int ntask, int n, const double *A, size_t lda, size_t mstride, int *status, float *S, size_t sstride,
                           const double *mdiag, const double *trace, double *result, int mode, cudaStream_t st, bool tc,
                           bool convert, void *work, int sched);
void launch_final(int ntask, int n, const double *logdiag, const double *trace, int *status, double *result, int mode, cudaStream_t st);

// HODLR log-determinants of the listed tasks (hodlr.cu), elements on demand; the diagonal of
// M alone for the trace rule; workspace bytes for nbatch matrices.  mx == nullptr: the I
// values by the FP64 q-sums (K, ptab); otherwise by the float-float q-sums from these tables
struct HodlrMixed {
    const float4 *KP;    // paired K table (k_kred_ff)
    const int *KPe;
    const float4 *ptabf; // float-float p tables per m group (launch_ptab_groups)
    const void *a12t;    // a_0..a_2 tables per m group (launch_a12_mixed with tabs)
    int ngroup;
};
size_t hodlr_work_bytes(int ldim, int nbatch);
int hodlr_levels(int ldim);
void hodlr_diag(const Task *tasks, int ntask, int ldim, const sd *K, int nu_stride, const double4 *ptab, int pstride, const double *lft,
                const sd *Sa, const sd *Sb, const double2 *uv, double *mdiag, int *status, cudaStream_t st, const HodlrMixed *mx);
void hodlr_logdet_batch(const Task *tasks, const int *tlist, int nbatch, int ldim, const sd *K, int nu_stride, const double4 *ptab,
                        int pstride, const double *lft, const sd *Sa, const sd *Sb, const double2 *uv, const double *trace,
                        int *status, double *result, void *work, cudaStream_t st, const HodlrMixed *mx);

// F for n abscissae at once; QUADPACK qagi with every node of a step in one call (tzero.cu)
using BatchFn = std::function<void(const double *x, int n, double *y)>;
double qagi_batched(const BatchFn &F, double bound, int inf, double epsabs, double epsrel, double *abserr, int *neval, int *ier);

} // namespace capsgpu
