// square.cu -- the sphere-sphere round trip (the reference's cass.c:23-64).
//
// For two equal spheres at separation d the round-trip operator is M^2, with M the
// plane-sphere round trip at L = d/2, and the reference takes log det(1 - M^2) from the
// dense matrix M^2 = M M (matrix_mult + matrix_logdet_dense, cass.c:42-60).  Here the
// batch already holds A = 1 - M (lower triangle, FP64) and M_ii; this kernel forms
// B = 1 - M^2 in the same layout, reading M(r,k) = -A(r,k) off the diagonal and M_ii on
// it (no 2A - A^2 cancellation), and writes (M^2)_ii separately for the trace shortcut.
// B is symmetric positive definite (|eigenvalues of M| < 1) and goes to the batched
// Cholesky with the dense shortcut rules.
#include "common.cuh"
#include "internal.h"

namespace capsgpu {

constexpr int SQ = 32; // output tile edge; 16 x 16 threads, 2 x 2 outputs each

// grid (tiles of the lower triangle, ntask)
__global__ void __launch_bounds__(256) k_square(int ntask, int n, const double *A, size_t lda, size_t mstride, const double *mdiag,
                                                double *B, const int *status, double *mdiag2)
{
    const int task = blockIdx.y;
    if (task >= ntask || (status[task] & ~0xF)) return;
    const int p = blockIdx.x;
    int ti = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
    while ((ti + 1) * (ti + 2) / 2 <= p) ti++;
    while (ti * (ti + 1) / 2 > p) ti--;
    const int tj = p - ti * (ti + 1) / 2;
    const int row0 = ti * SQ, col0 = tj * SQ;
    if (row0 >= n) return;
    const double *Am = A + (size_t)task * mstride;
    const double *dg = mdiag + (size_t)task * n;
    // M(r, k) from the lower triangle of A = 1 - M
    auto Mv = [&](int r, int k) -> double {
        if (r == k) return dg[r];
        return r > k ? -Am[(size_t)k * lda + r] : -Am[(size_t)r * lda + k];
    };
    __shared__ double Rs[SQ][SQ + 1]; // [row][k]
    __shared__ double Cs[SQ][SQ + 1]; // [col][k]
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
    for (int k0 = 0; k0 < n; k0 += SQ) {
        for (int e = threadIdx.x; e < SQ * SQ; e += 256) {
            const int r = e % SQ, kk = e / SQ, k = k0 + kk;
            Rs[r][kk] = (row0 + r < n && k < n) ? Mv(row0 + r, k) : 0.0;
            Cs[r][kk] = (col0 + r < n && k < n) ? Mv(col0 + r, k) : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < SQ; kk++) {
            const double a0 = Rs[ty][kk], a1 = Rs[ty + 16][kk], b0 = Cs[tx][kk], b1 = Cs[tx + 16][kk];
            acc[0][0] = fma(a0, b0, acc[0][0]);
            acc[0][1] = fma(a0, b1, acc[0][1]);
            acc[1][0] = fma(a1, b0, acc[1][0]);
            acc[1][1] = fma(a1, b1, acc[1][1]);
        }
        __syncthreads();
    }
    double *Bm = B + (size_t)task * mstride;
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int r = row0 + ty + 16 * i, c = col0 + tx + 16 * j;
            if (r >= n || c >= n || r < c) continue;
            const double s = acc[i][j]; // (M^2)_rc
            if (r == c) {
                Bm[(size_t)c * lda + r] = 1.0 - s;
                mdiag2[(size_t)task * n + r] = s;
            } else
                Bm[(size_t)c * lda + r] = -s;
        }
}

void launch_square(int ntask, int n, const double *A, size_t lda, size_t mstride, const double *mdiag, double *B,
                   const int *status, double *mdiag2, cudaStream_t st)
{
    const int nt = (n + SQ - 1) / SQ;
    dim3 g(nt * (nt + 1) / 2, ntask);
    k_square<<<g, 256, 0, st>>>(ntask, n, A, lda, mstride, mdiag, B, status, mdiag2);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
