// cholesky.cu -- batched blocked right-looking Cholesky in FP64 and the log-det.
//
// A = 1 - M is symmetric positive definite (the reference calls kernel_logdet
// with sym_spd=2, libcaps.c:954, and its HODLR path factors LL^T).  Each panel
// step is three launches over the whole batch: factor the 64x64 diagonal block,
// solve the panel below it, update the trailing lower triangle tile by tile.
// log det A = 2 sum_j log L_jj, summed with Kahan in index order like
// matrix_logdet_triangular (matrix.c:462).  A non-positive pivot marks the task
// (ST_ERR_PIVOT) and its result becomes NaN; nothing traps.
#include "common.cuh"
#include "internal.h"

namespace capsgpu {

constexpr int NB = 64;

// diagonal block: one CTA per task
__global__ void __launch_bounds__(256) k_potf2(int ntask, int n, int k0, double *A, size_t lda, size_t mstride, int *status,
                                               double *logdiag)
{
    const int task = blockIdx.x;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    __shared__ double S[NB][NB + 1];
    __shared__ int bad;
    const int nb = min(NB, n - k0);
    double *Am = A + (size_t)task * mstride + (size_t)k0 * lda + k0;
    if (threadIdx.x == 0) bad = 0;
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
        const int c = e / nb, r = e % nb;
        if (r >= c) S[r][c] = Am[(size_t)c * lda + r];
    }
    __syncthreads();
    for (int j = 0; j < nb; j++) {
        const double d = S[j][j];
        if (!(d > 0.0)) { // not SPD (or NaN): record and continue on |d| so the launch stays well defined
            if (threadIdx.x == 0) bad = 1;
        }
        const double ljj = sqrt(fabs(d) > 0 ? fabs(d) : 1.0);
        __syncthreads();
        if (threadIdx.x == 0) {
            S[j][j] = ljj;
            logdiag[(size_t)task * n + k0 + j] = log(ljj);
        }
        const double inv = 1.0 / ljj;
        for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) S[i][j] *= inv;
        __syncthreads();
        const int m = nb - j - 1; // rank-1 update of the remaining lower triangle
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
            const int i = j + 1 + e / m, c = j + 1 + e % m;
            if (i >= c) S[i][c] -= S[i][j] * S[c][j];
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
        const int c = e / nb, r = e % nb;
        if (r >= c) Am[(size_t)c * lda + r] = S[r][c];
    }
    if (threadIdx.x == 0 && bad) atomicOr(status + task, ST_ERR_PIVOT);
}

// panel solve: L_ik = A_ik L_kk^{-T} for the rows below the diagonal block;
// one thread per row, the row and L_kk held in shared memory
constexpr int TRSM_T = 64;
__global__ void __launch_bounds__(TRSM_T) k_trsm(int ntask, int n, int k0, double *A, size_t lda, size_t mstride, const int *status)
{
    const int task = blockIdx.y;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    const int nb = min(NB, n - k0);
    const int r0 = k0 + nb + blockIdx.x * TRSM_T;
    if (r0 >= n) return;
    extern __shared__ double sm[];
    double *Lk = sm;                      // [NB][NB+1]
    double *X = sm + NB * (NB + 1);       // [TRSM_T][NB+1]
    double *Am = A + (size_t)task * mstride;
    for (int e = threadIdx.x; e < nb * nb; e += TRSM_T) {
        const int c = e / nb, r = e % nb;
        Lk[r * (NB + 1) + c] = (r >= c) ? Am[(size_t)(k0 + c) * lda + k0 + r] : 0.0;
    }
    const int rows = min(TRSM_T, n - r0);
    for (int c = 0; c < nb; c++)
        for (int r = threadIdx.x; r < rows; r += TRSM_T) X[r * (NB + 1) + c] = Am[(size_t)(k0 + c) * lda + r0 + r];
    __syncthreads();
    if (threadIdx.x < rows) {
        double *x = X + threadIdx.x * (NB + 1);
        for (int c = 0; c < nb; c++) {
            double v = x[c];
            for (int cc = 0; cc < c; cc++) v -= x[cc] * Lk[c * (NB + 1) + cc];
            x[c] = v / Lk[c * (NB + 1) + c];
        }
    }
    __syncthreads();
    for (int c = 0; c < nb; c++)
        for (int r = threadIdx.x; r < rows; r += TRSM_T) Am[(size_t)(k0 + c) * lda + r0 + r] = X[r * (NB + 1) + c];
}

// trailing update of the lower triangle: tile (ti >= tj) of 64x64,
// C -= L_i L_j^T over the 64 panel columns; 256 threads x (4x4) outputs
__global__ void __launch_bounds__(256) k_syrk(int ntask, int n, int k0, double *A, size_t lda, size_t mstride, const int *status)
{
    const int task = blockIdx.y;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    const int nb = min(NB, n - k0);
    const int t0 = k0 + nb;
    // tile pair from linear index
    const int p = blockIdx.x;
    int ti = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
    while ((ti + 1) * (ti + 2) / 2 <= p) ti++;
    while (ti * (ti + 1) / 2 > p) ti--;
    const int tj = p - ti * (ti + 1) / 2;
    const int row0 = t0 + ti * 64, col0 = t0 + tj * 64;
    if (row0 >= n) return;
    extern __shared__ double sy[];
    double (*As)[65] = reinterpret_cast<double (*)[65]>(sy);            // [k][r]
    double (*Bs)[65] = reinterpret_cast<double (*)[65]>(sy + NB * 65);  // [k][c]
    double *Am = A + (size_t)task * mstride;
    for (int e = threadIdx.x; e < nb * 64; e += 256) {
        const int k = e / 64, r = e % 64;
        As[k][r] = (row0 + r < n) ? Am[(size_t)(k0 + k) * lda + row0 + r] : 0.0;
        Bs[k][r] = (col0 + r < n) ? Am[(size_t)(k0 + k) * lda + col0 + r] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.0;
    for (int k = 0; k < nb; k++) {
        double a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; i++) { a[i] = As[k][ty + 16 * i]; b[i] = Bs[k][tx + 16 * i]; }
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = row0 + ty + 16 * i;
        if (r >= n) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = col0 + tx + 16 * j;
            if (c < n && r >= c) Am[(size_t)c * lda + r] -= acc[i][j];
        }
    }
}

// log det and the post-checks of kernel_logdet (matrix.c:78-82, :144-145)
__global__ void k_final(int ntask, int n, const double *logdiag, const double *trace, int *status, double *result, int mode)
{
    const int task = blockIdx.x * blockDim.x + threadIdx.x;
    if (task >= ntask) return;
    const int st = status[task];
    if (st & ~0xF) { result[task] = NAN; return; }
    if (st != ST_FACTOR) return; // trace or Mercator result already stored
    double s = 0.0, c = 0.0;
    for (int j = 0; j < n; j++) {
        const double y = logdiag[(size_t)task * n + j] - c;
        const double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    double ld = 2.0 * s;
    if (mode == 1 && fabs(trace[task]) > fabs(ld)) ld = -trace[task];
    result[task] = ld;
}

void launch_cholesky(int ntask, int n, double *A, size_t lda, size_t mstride, int *status, double *logdiag, cudaStream_t st)
{
    static bool attr = false;
    const size_t trsm_sm = (size_t)(NB * (NB + 1) + TRSM_T * (NB + 1)) * sizeof(double);
    const size_t syrk_sm = (size_t)2 * NB * 65 * sizeof(double);
    if (!attr) {
        CK(cudaFuncSetAttribute(k_trsm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)trsm_sm));
        CK(cudaFuncSetAttribute(k_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)syrk_sm));
        attr = true;
    }
    for (int k0 = 0; k0 < n; k0 += NB) {
        k_potf2<<<ntask, 256, 0, st>>>(ntask, n, k0, A, lda, mstride, status, logdiag);
        COUNT_LAUNCH(1);
        const int rest = n - k0 - NB;
        if (rest <= 0) break;
        dim3 gt((rest + TRSM_T - 1) / TRSM_T, ntask);
        k_trsm<<<gt, TRSM_T, trsm_sm, st>>>(ntask, n, k0, A, lda, mstride, status);
        COUNT_LAUNCH(1);
        const int nt = (rest + 63) / 64;
        dim3 gs(nt * (nt + 1) / 2, ntask);
        k_syrk<<<gs, 256, syrk_sm, st>>>(ntask, n, k0, A, lda, mstride, status);
        COUNT_LAUNCH(1);
    }
    CK(cudaGetLastError());
}

void launch_final(int ntask, int n, const double *logdiag, const double *trace, int *status, double *result, int mode, cudaStream_t st)
{
    k_final<<<(ntask + 127) / 128, 128, 0, st>>>(ntask, n, logdiag, trace, status, result, mode);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
