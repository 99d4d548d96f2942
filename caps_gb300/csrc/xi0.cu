// xi0.cu -- the xi = 0 blocks: closed-form EE/MM elements (libcaps.c:860-928)
// assembled on the GPU and factored by the same batched Cholesky
// (caps_logdetD0, libcaps.c:985).
#include <cmath>
#include <mutex>
#include <vector>

#include "../../include/libcaps.h"
#include "internal.h"

namespace capsgpu {

// M0_EE(l1,l2) = exp((l1+l2+1) y + lfac(l1+l2) - (lfac(l1+m)+lfac(l1-m)+lfac(l2+m)+lfac(l2-m))/2)
// M0_MM = M0_EE sqrt(l1 l2 / ((l1+1)(l2+1)))
__global__ void k_elem0(const int *ms, const int *lmins, int ntask, int ldim, double y, int which, const double *lfac_tab,
                        double *A, size_t mstride, int *status)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const int task = blockIdx.z;
    if (i >= ldim || j > i || task >= ntask) return;
    const int m = ms[task], l1 = i + lmins[task], l2 = j + lmins[task];
    double v = exp((l1 + l2 + 1) * y + lfac(lfac_tab, l1 + l2)
                   - 0.5 * (lfac(lfac_tab, l1 + m) + lfac(lfac_tab, l1 - m) + lfac(lfac_tab, l2 + m) + lfac(lfac_tab, l2 - m)));
    if (which == 1) v *= sqrt(((double)l1 * l2) / ((l1 + 1.) * (l2 + 1.)));
    if (!isfinite(v)) atomicOr(status + task, ST_ERR_NONFINITE);
    A[(size_t)task * mstride + (size_t)j * ldim + i] = (i == j ? 1.0 : 0.0) - v;
}

} // namespace capsgpu

using namespace capsgpu;

// implemented in libcaps.cu
struct Engine;

int logdetD0_batch(caps_t *self, const int *ms, int n, int which, double *out)
{
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    // the engine's stream/tables are initialised by any prior API call; make sure
    static double *d_lfac = nullptr;
    if (!d_lfac) {
        double tab[1024];
        for (int k = 0; k < 1024; k++) tab[k] = lgamma(k + 1.0);
        CK(cudaMalloc(&d_lfac, sizeof tab));
        CK(cudaMemcpy(d_lfac, tab, sizeof tab, cudaMemcpyHostToDevice));
    }
    const int ldim = self->ldim;
    std::vector<int> lmins(n);
    for (int k = 0; k < n; k++) {
        size_t lo, hi;
        caps_estimate_lminmax(self, ms[k], &lo, &hi);
        lmins[k] = (int)lo;
    }
    int *d_m, *d_lmin, *d_status;
    double *d_A, *d_ld, *d_tr, *d_res;
    const size_t mstride = (size_t)ldim * ldim;
    CK(cudaMalloc(&d_m, n * sizeof(int)));
    CK(cudaMalloc(&d_lmin, n * sizeof(int)));
    CK(cudaMalloc(&d_status, n * sizeof(int)));
    CK(cudaMalloc(&d_A, n * mstride * sizeof(double)));
    CK(cudaMalloc(&d_ld, (size_t)n * ldim * sizeof(double)));
    CK(cudaMalloc(&d_tr, n * sizeof(double)));
    CK(cudaMalloc(&d_res, n * sizeof(double)));
    cudaStream_t st = 0;
    CK(cudaMemcpy(d_m, ms, n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(d_lmin, lmins.data(), n * sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemset(d_status, 0, n * sizeof(int)));
    dim3 g((ldim + 127) / 128, ldim, n);
    k_elem0<<<g, 128, 0, st>>>(d_m, d_lmin, n, ldim, self->y, which, d_lfac, d_A, mstride, d_status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
    const int mode = self->detalg == DETALG_HODLR ? 1 : 0;
    launch_stats(nullptr, n, ldim, d_A, ldim, mstride, mode, d_tr, d_res, d_status, st);
    launch_cholesky(n, ldim, d_A, ldim, mstride, d_status, d_ld, st);
    launch_final(n, ldim, d_ld, d_tr, d_status, d_res, mode, st);
    std::vector<int> hs(n);
    CK(cudaMemcpy(out, d_res, n * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hs.data(), d_status, n * sizeof(int), cudaMemcpyDeviceToHost));
    CK(cudaFree(d_m)); CK(cudaFree(d_lmin)); CK(cudaFree(d_status)); CK(cudaFree(d_A));
    CK(cudaFree(d_ld)); CK(cudaFree(d_tr)); CK(cudaFree(d_res));
    int nerr = 0;
    for (int k = 0; k < n; k++) nerr += (hs[k] & ~0xF) != 0;
    return nerr;
}
