// mixed.cu -- mixed-precision log det(1-M): FP32 factorisation in "delta form"
// plus an FP64 correction.
//
// A = 1 - M is close to the identity (on the R/L=150 workload its condition
// number is 1.0-1.1).  The factorisation is written as A = (I+Lam)(I+Lam)^T and
// only Lam and S = A - I are held in FP32, so the unit diagonal never enters
// FP32 arithmetic: the pivot of column j is 1 + d with d = S_jj - sum_k Lam_jk^2,
// and Lam_jj = d/(sqrt(1+d)+1).  FP32 rounding then acts on O(|M|) quantities.
//
// log det A = 2 sum_j log1p(Lam_jj) + log det(I + X),  X = (I+Lam)^{-1} Delta (I+Lam)^{-T},
// Delta = A - (I+Lam)(I+Lam)^T.  The correction keeps the first term of the
// trace series, tr X ~ tr Delta, evaluated in FP64 from the FP32 factor
// (products of two FP32 numbers are exact in FP64):
//   tr Delta = tr(A - I) - 2 tr Lam - ||Lam||_F^2.
// The pivot logarithms and every sum are FP64.  The result agrees with the
// FP64 Cholesky to ~3e-9 absolute on the hardest matrices of the workload
// (log det ~ -1) and to <1e-12 on the rest.
#include <cstdlib>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "syrk_umma.cuh"
#include "syrk_pipe.cuh"

namespace capsgpu {

constexpr int MB = 64; // panel width
static_assert(MB == UM_K, "the tcgen05 trailing update is built for the panel width");
// ||Lam||_F^2 is summed where the final entries of Lam are written: one partial per
// diagonal block (k_potf2_w) and per 64-row block of each panel solve (k_trsm_inv), in
// slot p (NBR + 1) and p (NBR + 1) + 1 + b of a task's PS = NBR (NBR + 1) slots, NBR = ceil(n / 64)
__host__ __device__ inline int fro_nbr(int n) { return (n + MB - 1) / MB; }
__host__ __device__ inline int fro_slots(int n) { return fro_nbr(n) * (fro_nbr(n) + 1); }

// sum over the 256 threads of a block, fixed order; the result is valid in thread 0
__device__ __forceinline__ double block_sum256(double v, double *red8)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red8[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < 8; w++) s += red8[w];
    return s;
}

// Sums of squares of FP32 entries without the FP64 pipe (a few per cent of the FP32 rate on
// this GPU): x^2 = p + e exactly (p = fl(x x), e = fma(x, x, -p)), accumulated as a float-float
// pair by Knuth's two-sum on the high parts with the low parts summed in FP32 (relative error
// about 2^-48, as good as an FP64 sum of a few hundred terms).  The _rn intrinsics keep the
// compiler from fusing the additions into FMAs, which the two-sum must not see.
struct SqSum {
    float hi = 0.0f, lo = 0.0f;
    __device__ __forceinline__ void add2(float h2, float l2)
    {
        const float t = __fadd_rn(hi, h2), bp = __fsub_rn(t, hi);
        lo = __fadd_rn(__fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(h2, bp)), __fadd_rn(lo, l2));
        hi = t;
    }
    __device__ __forceinline__ void add_sq(float x)
    {
        const float p = __fmul_rn(x, x);
        add2(p, fmaf(x, x, -p));
    }
};
// SqSum over the NW warps of a block: float-float within each warp (fixed butterfly), then
// the warp sums in FP64 in warp order; the result is valid in thread 0
template <int NW> __device__ __forceinline__ double block_sq(SqSum q, double *red)
{
    for (int o = 16; o > 0; o >>= 1) q.add2(__shfl_xor_sync(0xffffffffu, q.hi, o), __shfl_xor_sync(0xffffffffu, q.lo, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = (double)q.hi + (double)q.lo;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < NW; w++) s += red[w];
    return s;
}

// S = A - I (lower triangle, FP32) for the tasks that need a factorisation
__global__ void k_to_delta32(int ntask, int n, const double *A, size_t lda, size_t mstride, const int *status, float *S,
                             size_t sstride)
{
    const int task = blockIdx.y;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    const size_t total = (size_t)n * n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(e / n), r = (int)(e % n);
        if (r < c) continue;
        const double v = A[(size_t)task * mstride + (size_t)c * lda + r];
        S[(size_t)task * sstride + (size_t)c * n + r] = (float)(r == c ? v - 1.0 : v);
    }
}

// diagonal block in delta form, one CTA of 256 threads per matrix; also writes W =
// (I + Lam_kk)^{-1} (lower triangular, MB x MB per task, stored transposed) for the panel solve and
// the block's share of ||Lam||_F^2.  The factorisation runs in 16-column sub-panels (warp-level
// diagonal block, substitution below it, rank-16 update of the rest); the updates take the
// entries (i, c) of the trailing triangle from a list of the whole triangle ordered by column
// (last column first), so that each sub-panel's entries are a prefix of it and the 256
// threads share them evenly (consecutive threads: consecutive rows of one column, T rows 65
// floats apart, distinct banks).  W follows blockwise (16 x 16 blocks).
__global__ void __launch_bounds__(256) k_potf2_w(int ntask, int n, int k0, float *S, size_t sstride, int *status, float *Winv,
                                                 double *fro)
{
    const int task = blockIdx.x;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    __shared__ float T[MB][MB + 1];
    __shared__ float W[MB][MB + 1];
    __shared__ float colj[MB];
    __shared__ float Yb[3][16][17]; // blocks of the blockwise inverse in progress
    __shared__ double red8[8];
    // the entries (i, c), 1 <= c <= i <= 63, as i | c << 8, columns 63, 62, ..., 1, rows
    // ascending within a column; column c starts at (63 - c)(64 - c) / 2
    __shared__ unsigned short tri[(MB - 1) * MB / 2];
    const int tid = threadIdx.x;
    const int nb = min(MB, n - k0);
    if (tid >= 1 && tid < MB) {
        const int c = tid, first = (MB - 1 - c) * (MB - c) / 2;
        for (int i = c; i < MB; i++) tri[first + i - c] = (unsigned short)(i | c << 8);
    }
    float *Sm = S + (size_t)task * sstride + (size_t)k0 * n + k0;
    {
        // the block's lower triangle, 16 loads in flight per thread
        float v[MB * MB / 256];
#pragma unroll
        for (int u = 0; u < MB * MB / 256; u++) {
            const int e = tid + 256 * u, c = e / MB, r = e % MB;
            v[u] = (c < nb && r >= c && r < nb) ? __ldg(Sm + (size_t)c * n + r) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < MB * MB / 256; u++) {
            const int e = tid + 256 * u, c = e / MB, r = e % MB;
            if (c < nb && r >= c && r < nb) T[r][c] = v[u];
        }
    }
    __syncthreads();
    bool bad = false;
    // blocked in 16-column sub-panels: (a) the sub-panel's diagonal block by warp 0 (lane i
    // holds its row i in registers, column entries broadcast by shuffles), (b) the rows below it
    // by forward substitution, one thread per row, (c) the rank-16 update of the rest of the
    // triangle from the tail of the entry list; three barriers per sub-panel
    constexpr int PB = 16;
    for (int o = 0; o < nb; o += PB) {
        const int w = min(PB, nb - o);
        if (tid < 32) {
            // every lane also keeps the sub-panel's future pivots dd[c] (pivot - 1), updated
            // with the same fma and order as lane c's own diagonal entry: the shuffles of the
            // update bring l_cj to every lane, so no pivot is broadcast, and the step's chain is
            // one shuffle, an fma, an add, a reciprocal square root and a product
            const int i = tid;
            float t[PB], dd[PB];
#pragma unroll
            for (int k = 0; k < PB; k++) {
                t[k] = (i < w && k <= i) ? T[o + i][o + k] : 0.0f;
                dd[k] = k < w ? T[o + k][o + k] : 0.0f;
            }
#pragma unroll
            for (int j = 0; j < PB; j++) {
                if (j < w) { // uniform
                const float d = dd[j]; // pivot - 1
                const float one_d = 1.0f + d;
                bad |= !(one_d > 0.0f);
                // inv = 1 / (1 + lam) = (1 + d)^(-1/2); lam = sqrt(1 + d) - 1 = d inv / (1 + inv)
                // (no quotient: one with a tiny numerator, as d is at high l, is slow)
                const float inv = __frsqrt_rn(fmaxf(one_d, 1e-30f));
                if (i > j) t[j] *= inv;
                else if (i == j) t[j] = d * inv * __frcp_rn(1.0f + inv);
                if (i == 0) colj[o + j] = inv;
                const float cj = t[j];
#pragma unroll
                for (int c = j + 1; c < PB; c++) {
                    const float v = __shfl_sync(0xffffffffu, cj, c); // column j of row c
                    if (i >= c && i < w) t[c] = fmaf(-cj, v, t[c]);
                    dd[c] = fmaf(-v, v, dd[c]);
                }
                }
            }
#pragma unroll
            for (int k = 0; k < PB; k++)
                if (i < w && k <= i) T[o + i][o + k] = t[k];
        }
        __syncthreads();
        const int c0 = o + w;
        if (tid < nb - c0) {
            const int r = c0 + tid;
            float x[PB];
#pragma unroll
            for (int k = 0; k < PB; k++) x[k] = k < w ? T[r][o + k] : 0.0f;
#pragma unroll
            for (int k = 0; k < PB; k++) {
                if (k < w) {
                    float a = x[k];
#pragma unroll
                    for (int j = 0; j < k; j++) a = fmaf(-x[j], T[o + k][o + j], a);
                    x[k] = a * colj[o + k];
                }
            }
#pragma unroll
            for (int k = 0; k < PB; k++)
                if (k < w) T[r][o + k] = x[k];
        }
        __syncthreads();
        if (c0 < nb) {
            // the entries (i, c), c0 <= c <= i, are the first (MB - c0)(MB - c0 + 1) / 2 of the list
            const int cnt = (MB - c0) * (MB - c0 + 1) / 2;
            for (int e = tid; e < cnt; e += 256) {
                const int v = tri[e], ri = v & 0xff, c = v >> 8;
                if (ri < nb) {
                    float acc = 0.0f;
#pragma unroll
                    for (int k = 0; k < PB; k++) acc = fmaf(T[ri][o + k], T[c][o + k], acc);
                    T[ri][c] -= acc;
                }
            }
        }
        __syncthreads();
    }
    SqSum q;
    for (int e = tid; e < MB * MB; e += 256) {
        const int c = e / MB, r = e % MB;
        if (c < nb && r >= c && r < nb) {
            Sm[(size_t)c * n + r] = T[r][c];
            q.add_sq(T[r][c]);
        }
    }
    const double sq = block_sq<8>(q, red8);
    if (tid == 0) fro[(size_t)task * fro_slots(n) + (size_t)(k0 / MB) * (fro_nbr(n) + 1)] = sq;
    // W = (I + Lam)^{-1} blockwise in 16 x 16 blocks: the four diagonal blocks by forward
    // substitution, one thread per column with the column in registers; then the blocks below,
    // by distance from the diagonal, X_ij = -X_ii sum_{k=j}^{i-1} L_ik X_kj (L = I + Lam).  Rows
    // past nb read entries of T that were never loaded; they feed only rows past nb (the
    // inverse of a lower triangular matrix is causal in the row index), which are not stored.
    constexpr int QB = 16;
    if (tid < MB) {
        const int o = (tid / QB) * QB, c = tid % QB;
        float x[QB], rdv[QB];
#pragma unroll
        for (int r = 0; r < QB; r++) rdv[r] = __frcp_rn(1.0f + T[o + r][o + r]); // off the chain below
#pragma unroll
        for (int r = 0; r < QB; r++) {
            float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
            for (int k = 0; k < r; k++) {
                if (k & 1) a1 = fmaf(T[o + r][o + k], x[k], a1);
                else a0 = fmaf(T[o + r][o + k], x[k], a0);
            }
            x[r] = r < c ? 0.0f : (r == c ? rdv[r] : -(a0 + a1) * rdv[r]); // a product, not a quotient: see above
            W[o + r][o + c] = x[r];
        }
    }
    __syncthreads();
    for (int dl = 1; dl < MB / QB; dl++) {
        const int np = MB / QB - dl; // block pairs (i, j) = (p + dl, p) at this distance
        for (int e = tid; e < np * QB * QB; e += 256) {
            const int p = e / (QB * QB), r = (e / QB) % QB, c = e % QB, i = p + dl;
            float acc = 0.0f;
            for (int k = p; k < i; k++)
#pragma unroll
                for (int q = 0; q < QB; q++) acc = fmaf(T[i * QB + r][k * QB + q], W[k * QB + q][p * QB + c], acc);
            Yb[p][r][c] = acc;
        }
        __syncthreads();
        for (int e = tid; e < np * QB * QB; e += 256) {
            const int p = e / (QB * QB), r = (e / QB) % QB, c = e % QB, i = p + dl;
            float acc = 0.0f;
#pragma unroll
            for (int q = 0; q < QB; q++)
                if (q <= r) acc = fmaf(W[i * QB + r][i * QB + q], Yb[p][q][c], acc);
            W[i * QB + r][p * QB + c] = -acc;
        }
        __syncthreads();
    }
    // stored transposed, Wt[k MB + c] = W[c][k] (zero outside the lower triangle and past nb): the
    // k-major layout in which the panel solve keeps it, so that its copy is a plain one
    float *Wt = Winv + (size_t)task * MB * MB;
    for (int e = tid; e < MB * MB; e += 256) {
        const int k = e / MB, c = e % MB;
        Wt[e] = (c < nb && k <= c) ? W[c][k] : 0.0f;
    }
    if (__syncthreads_or(bad) && tid == 0) atomicOr(status + task, ST_ERR_PIVOT);
}

// panel: X (I + Lam_kk)^T = S for the rows below the diagonal block, as X = S W^T with
// W = (I + Lam_kk)^{-1} from k_potf2_w (I + Lam_kk is within a few per cent of I, so the
// product is as accurate as the substitution).  64 rows per CTA of 128 threads; thread t
// computes rows t mod 16 + 16 i of the column groups g = t / 16 and 15 - g (columns 4 g + j
// and 4 (15 - g) + j).  W is lower triangular (column c takes k <= c), so the pair needs
// k < 4 g + 4 for both groups and k < 64 - 4 g for the second: 1088 FMAs for every thread, half
// the FMAs and shared-memory reads of the full product, in the same order per column.  The
// rows are kept in shared memory k-major with row r at position 4 (r mod 16) + r / 16 and W
// k-major, so per k a thread reads its four rows and four columns of a group as one float4.
constexpr int MT = 64, TRSM_THREADS = 128;
// img64 != nullptr: every row goes to the FP16 image of 64-column block blk64 of the 256-column
// panel (layout of syrk_pipe.cuh), which the left-looking updates of the panel's later blocks
// and the trailing update after the panel read.  An entry |x| >= 4, outside the images' range,
// marks the matrix ST_ERR_RANGE.  Rows past n are left unwritten there; they only reach
// accumulator rows and columns that are never stored.  store_x false: X is not written back
// to S (with the images, nothing reads it there again: later steps read S only in their own
// columns, the final sums only its diagonal).
__global__ void __launch_bounds__(TRSM_THREADS) k_trsm_inv(int ntask, int n, int k0, float *S, size_t sstride, int *status,
                                                  const float *Winv, double *fro, __half *img64, int blk64, bool store_x)
{
    const int task = blockIdx.y;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    const int nb = min(MB, n - k0);
    const int r0 = k0 + nb + blockIdx.x * MT;
    if (r0 >= n) return;
    __shared__ __align__(16) float Wk[MB][MB + 4]; // W[c][k] at Wk[k][c]
    __shared__ __align__(16) float Xk[MB][MT + 4]; // S[r0 + r][k0 + k] at Xk[k][4 (r mod 16) + r / 16]
    float *Sm = S + (size_t)task * sstride;
    const float *Wt = Winv + (size_t)task * MB * MB;
    const int rows = min(MT, n - r0);
    constexpr int NT = TRSM_THREADS;
    {
        float w[MB * MB / NT], x[MT * MB / NT];
#pragma unroll
        for (int u = 0; u < MB * MB / NT; u++) w[u] = __ldg(Wt + threadIdx.x + NT * u);
#pragma unroll
        for (int u = 0; u < MT * MB / NT; u++) {
            const int e = threadIdx.x + NT * u, c = e / MT, r = e % MT;
            x[u] = (r < rows && c < nb) ? __ldg(Sm + (size_t)(k0 + c) * n + r0 + r) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < MB * MB / NT; u++) {
            const int e = threadIdx.x + NT * u; // W stored transposed: e = k MB + c
            Wk[e / MB][e % MB] = w[u];
        }
#pragma unroll
        for (int u = 0; u < MT * MB / NT; u++) {
            const int e = threadIdx.x + NT * u, c = e / MT, r = e % MT;
            Xk[c][4 * (r & 15) + (r >> 4)] = x[u];
        }
    }
    __syncthreads();
    const int rg = threadIdx.x & 15, g = threadIdx.x >> 4, gh = 15 - g;
    float acl[4][4], ach[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acl[i][j] = ach[i][j] = 0.0f;
    const int k1 = min(nb, 4 * g + 4), k2 = min(nb, 4 * gh + 4);
    for (int k = 0; k < k1; k++) {
        const float4 a = *reinterpret_cast<const float4 *>(&Xk[k][4 * rg]);
        const float4 wl = *reinterpret_cast<const float4 *>(&Wk[k][4 * g]);
        const float4 wh = *reinterpret_cast<const float4 *>(&Wk[k][4 * gh]);
        const float av[4] = {a.x, a.y, a.z, a.w}, lv[4] = {wl.x, wl.y, wl.z, wl.w}, hv[4] = {wh.x, wh.y, wh.z, wh.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                acl[i][j] = fmaf(av[i], lv[j], acl[i][j]);
                ach[i][j] = fmaf(av[i], hv[j], ach[i][j]);
            }
    }
    for (int k = k1; k < k2; k++) {
        const float4 a = *reinterpret_cast<const float4 *>(&Xk[k][4 * rg]);
        const float4 wh = *reinterpret_cast<const float4 *>(&Wk[k][4 * gh]);
        const float av[4] = {a.x, a.y, a.z, a.w}, hv[4] = {wh.x, wh.y, wh.z, wh.w};
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) ach[i][j] = fmaf(av[i], hv[j], ach[i][j]);
    }
    SqSum q;
    bool big = false;
    // the outputs of column group cg (columns 4 cg .. 4 cg + 3) from its accumulators
    auto emit = [&](const float(&acc)[4][4], int cg) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = 4 * cg + j;
            if (c >= nb) continue;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = rg + 16 * i;
                if (r < rows) {
                    if (store_x) Sm[(size_t)(k0 + c) * n + r0 + r] = acc[i][j];
                    q.add_sq(acc[i][j]);
                }
            }
        }
        if (img64) {
            // this block's 64 rows are 64-row block blockIdx.x of the image (rows from k0 + 64);
            // columns 4 cg .. 4 cg + 3 are half of one 16-byte row of a core matrix (the groups
            // 2 w, 2 w + 1 or 14 - 2 w, 15 - 2 w of warp w fill it, its 16 rows two whole core
            // matrices)
            const int nrb64 = pipe_img64_nrb(n);
            __half *hi = img64 + (((size_t)blk64 * ntask + task) * 2 * nrb64 + blockIdx.x) * PIPE_IMG64_HALVES;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int r = rg + 16 * i;
                if (r < rows) {
                    const int e = ((r / 8) * 8 + cg / 2) * 64 + (r % 8) * 8 + 4 * (cg % 2);
                    uint32_t h[4], l[4];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        img_split16(acc[i][j], h[j], l[j]);
                        big |= !(fabsf(acc[i][j]) < PIPE_IMG_XMAX);
                    }
                    *reinterpret_cast<uint2 *>(hi + e) = make_uint2(h[0] | h[1] << 16, h[2] | h[3] << 16);
                    *reinterpret_cast<uint2 *>(hi + (size_t)nrb64 * PIPE_IMG64_HALVES + e) =
                        make_uint2(l[0] | l[1] << 16, l[2] | l[3] << 16);
                }
            }
        }
    };
    emit(acl, g);
    emit(ach, gh);
    if (big) atomicOr(status + task, ST_ERR_RANGE);
    __shared__ double red4[NT / 32];
    const double sq = block_sq<NT / 32>(q, red4);
    if (threadIdx.x == 0) fro[(size_t)task * fro_slots(n) + (size_t)(k0 / MB) * (fro_nbr(n) + 1) + 1 + blockIdx.x] = sq;
}

// trailing update S_ab -= sum_k Lam_ak Lam_bk over the panel, 64x64 tiles of the
// lower triangle, 64 threads x (8x8) outputs
__global__ void __launch_bounds__(64) k_syrk_f(int ntask, int n, int k0, float *S, size_t sstride, const int *status)
{
    const int task = blockIdx.y;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    const int nb = min(MB, n - k0);
    const int t0 = k0 + nb;
    const int p = blockIdx.x;
    int ti = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
    while ((ti + 1) * (ti + 2) / 2 <= p) ti++;
    while (ti * (ti + 1) / 2 > p) ti--;
    const int tj = p - ti * (ti + 1) / 2;
    const int row0 = t0 + ti * 64, col0 = t0 + tj * 64;
    if (row0 >= n) return;
    __shared__ float As[MB][64 + 4];
    __shared__ float Bs[MB][64 + 4];
    float *Sm = S + (size_t)task * sstride;
    for (int e = threadIdx.x; e < nb * 64; e += 64) {
        const int k = e / 64, r = e % 64;
        As[k][r] = (row0 + r < n) ? Sm[(size_t)(k0 + k) * n + row0 + r] : 0.0f;
        Bs[k][r] = (col0 + r < n) ? Sm[(size_t)(k0 + k) * n + col0 + r] : 0.0f;
    }
    __syncthreads();
    const int tx = threadIdx.x & 7, ty = threadIdx.x >> 3;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 8; j++) acc[i][j] = 0.0f;
    for (int k = 0; k < nb; k++) {
        float a[8], b[8];
#pragma unroll
        for (int i = 0; i < 8; i++) { a[i] = As[k][ty + 8 * i]; b[i] = Bs[k][tx + 8 * i]; }
#pragma unroll
        for (int i = 0; i < 8; i++)
#pragma unroll
            for (int j = 0; j < 8; j++) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const int r = row0 + ty + 8 * i;
        if (r >= n) continue;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int c = col0 + tx + 8 * j;
            if (c < n && r >= c) Sm[(size_t)c * n + r] -= acc[i][j];
        }
    }
}


// Tensor-core trailing update: S_tile -= A B^T over the 64 panel columns with
// split TF32 (x = hi + lo, both TF32; A B^T ~ hi hi + hi lo + lo hi, FP32
// accumulation) on mma.sync.m16n8k8.  64x64 output tile per CTA of 4 warps,
// each warp a 32x32 quadrant of 2x4 m16n8 fragments.
__device__ __forceinline__ unsigned tf32_of(float x)
{
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const unsigned (&a)[4], const unsigned (&b)[2])
{
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(128) k_syrk_tc(int ntask, int n, int k0, float *S, size_t sstride, const int *status)
{
    const int task = blockIdx.y;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    const int nb = min(MB, n - k0);
    const int t0 = k0 + nb;
    const int p = blockIdx.x;
    int ti = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
    while ((ti + 1) * (ti + 2) / 2 <= p) ti++;
    while (ti * (ti + 1) / 2 > p) ti--;
    const int tj = p - ti * (ti + 1) / 2;
    const int row0 = t0 + ti * 64, col0 = t0 + tj * 64;
    if (row0 >= n) return;
    __shared__ float As[64][MB + 4]; // [row][k]
    __shared__ float Bs[64][MB + 4]; // [col][k]
    float *Sm = S + (size_t)task * sstride;
    for (int e = threadIdx.x; e < 64 * MB; e += 128) {
        const int k = e / 64, r = e % 64;
        As[r][k] = (row0 + r < n && k < nb) ? Sm[(size_t)(k0 + k) * n + row0 + r] : 0.0f;
        Bs[r][k] = (col0 + r < n && k < nb) ? Sm[(size_t)(k0 + k) * n + col0 + r] : 0.0f;
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[i][j][q] = 0.0f;
#pragma unroll 2
    for (int ks = 0; ks < MB; ks += 8) {
        unsigned ah[2][4], al[2][4], bh[4][2], bl[4][2];
#pragma unroll
        for (int i = 0; i < 2; i++) {
            const int r = wm + i * 16 + g;
            const float x[4] = {As[r][ks + t], As[r + 8][ks + t], As[r][ks + t + 4], As[r + 8][ks + t + 4]};
#pragma unroll
            for (int q = 0; q < 4; q++) { ah[i][q] = tf32_of(x[q]); al[i][q] = tf32_of(x[q] - __uint_as_float(ah[i][q])); }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = wn + j * 8 + g;
            const float y[2] = {Bs[c][ks + t], Bs[c][ks + t + 4]};
#pragma unroll
            for (int q = 0; q < 2; q++) { bh[j][q] = tf32_of(y[q]); bl[j][q] = tf32_of(y[q] - __uint_as_float(bh[j][q])); }
        }
#pragma unroll
        for (int i = 0; i < 2; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                mma_tf32(acc[i][j], al[i], bh[j]);
                mma_tf32(acc[i][j], ah[i], bl[j]);
                mma_tf32(acc[i][j], ah[i], bh[j]);
            }
    }
#pragma unroll
    for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int r = row0 + wm + i * 16 + g + (q >= 2 ? 8 : 0);
                const int c = col0 + wn + j * 8 + 2 * t + (q & 1);
                if (r < n && c < n && r >= c) Sm[(size_t)c * n + r] -= acc[i][j][q];
            }
}

// log det = 2 sum log1p(Lam_jj) + tr(A-I) - 2 tr Lam - ||Lam||_F^2, all sums FP64;
// one CTA per task, fixed reduction order
__global__ void __launch_bounds__(256) k_final_mixed(int ntask, int n, const float *S, size_t sstride, const double *mdiag,
                                                     const double *trace, int *status, double *result, int mode,
                                                     const double *part)
{
    const int task = blockIdx.x;
    if (task >= ntask) return;
    const int st = status[task];
    if (st & ~0xF) { if (threadIdx.x == 0) result[task] = NAN; return; }
    if (st != ST_FACTOR) return;
    const float *Sm = S + (size_t)task * sstride;
    // per thread (strided j, fixed order): pivot logs, tr(A-I), tr Lam, and the Frobenius
    // partials; then one fixed-order block sum of each
    double sl = 0, sa = 0, st_ = 0, sf = 0;
    for (int j = threadIdx.x; j < n; j += 256) {
        const double lam = Sm[(size_t)j * n + j];
        sl += log1p(lam);
        sa -= mdiag[(size_t)task * n + j];
        st_ += lam;
    }
    const int PS = fro_slots(n);
    for (int i = threadIdx.x; i < PS; i += 256) sf += part[(size_t)task * PS + i];
    __shared__ double red8[8];
    sl = block_sum256(sl, red8);
    __syncthreads();
    sa = block_sum256(sa, red8);
    __syncthreads();
    st_ = block_sum256(st_, red8);
    __syncthreads();
    sf = block_sum256(sf, red8);
    if (threadIdx.x != 0) return;
    const double trDelta = sa - 2.0 * st_ - sf;
    double ld = 2.0 * sl + trDelta;
    if (mode == 1 && fabs(trace[task]) > fabs(ld)) ld = -trace[task];
    result[task] = ld;
}

// live timing of the factorisation's kernels (off unless caps_gpu_kernel_timing(1)): CUDA
// events on the launching stream around every launch of kind KT_SYRK (the tcgen05 trailing
// update), KT_TRSM (the panel solve k_trsm_inv) and KT_POTF2 (the diagonal block k_potf2_w),
// with each launch's algorithmic bytes per factored matrix; kernel_timer_collect() resolves
// the events of a finished batch and scales the bytes by the number of matrices it factored
namespace {
struct KernelTimer {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<double> per_matrix_bytes; // one per pending launch
    double ms = 0, bytes = 0;
    long long launches = 0;
    cudaEvent_t next()
    {
        if (used == pool.size()) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            pool.push_back(e);
        }
        return pool[used++];
    }
};
KernelTimer g_kts[KT_KINDS];
KernelTimer &g_kt = g_kts[KT_SYRK];
} // namespace

void kernel_timer_enable(bool on)
{
    for (KernelTimer &k : g_kts) {
        k.on = on;
        k.used = 0;
        k.per_matrix_bytes.clear();
        k.ms = k.bytes = 0;
        k.launches = 0;
    }
}

void kernel_timer_collect(long long nfactored)
{
    for (KernelTimer &k : g_kts) {
        if (!k.on) continue;
        for (size_t i = 0; i < k.per_matrix_bytes.size(); i++) {
            float f;
            CK(cudaEventElapsedTime(&f, k.pool[2 * i], k.pool[2 * i + 1]));
            k.ms += f;
            k.bytes += k.per_matrix_bytes[i] * (double)nfactored;
            k.launches++;
        }
        k.used = 0;
        k.per_matrix_bytes.clear();
    }
}

void kernel_timer_stats(int kind, double *ms, double *bytes, long long *launches)
{
    const KernelTimer &k = g_kts[kind >= 0 && kind < KT_KINDS ? kind : 0];
    if (ms) *ms = k.ms;
    if (bytes) *bytes = k.bytes;
    if (launches) *launches = k.launches;
}

// scratch: diagonal-block inverses, Frobenius partials, then (256-byte aligned) the panel
// images of the trailing update
static size_t mixed_img_offset(int ntask, int n)
{
    return ((size_t)ntask * (MB * MB * sizeof(float) + fro_slots(n) * sizeof(double)) + 255) / 256 * 256;
}
size_t mixed_work_bytes(int ntask, int n)
{
    return mixed_img_offset(ntask, n) + (size_t)ntask * pipe_img64_bytes(n);
}

void launch_cholesky_mixed(int ntask, int n, const double *A, size_t lda, size_t mstride, int *status, float *S, size_t sstride,
                           const double *mdiag, const double *trace, double *result, int mode, cudaStream_t st, bool tc, bool convert,
                           void *work, int sched)
{
    // work: mixed_work_bytes(ntask, n) of scratch (diagonal-block inverses, Frobenius partials,
    // panel images)
    float *Winv = (float *)work;
    double *part = (double *)((char *)work + (size_t)ntask * MB * MB * sizeof(float));
    __half *img64 = (__half *)((char *)work + mixed_img_offset(ntask, n));
    CK(cudaMemsetAsync(part, 0, (size_t)ntask * fro_slots(n) * sizeof(double), st));
    // convert: A is the FP64 matrix 1 - M and S receives its delta form here; otherwise S
    // already holds it.  mdiag: M_ii in FP64, n per task (tr(A - I) = -tr M).
    // Trailing update: tcgen05 (k_syrk_umma); CAPS_MIXED_MMASYNC=1 selects the mma.sync
    // kernel, tc = false (CAPS_MIXED_SIMT=1) the FFMA one.
    // The schedule of the trailing update (sched, chosen by the caller's autotuner):
    // MIXED_SCHED_IMAGES the persistent kernel fed by bulk copies of the panel images,
    // MIXED_SCHED_REGSTAGE the persistent kernel staging the panel through registers (16
    // producer warps), MIXED_SCHED_PER_TILE one CTA per tile.  The environment overrides it:
    // CAPS_MIXED_REGSTAGE=1, CAPS_MIXED_NOPIPE=1, CAPS_MIXED_MMASYNC=1 (mma.sync).
    static const bool legacy_mma = getenv("CAPS_MIXED_MMASYNC") != nullptr;
    static const bool env_no_pipe = getenv("CAPS_MIXED_NOPIPE") != nullptr;
    static const bool env_reg_stage = getenv("CAPS_MIXED_REGSTAGE") != nullptr;
    const bool no_pipe = env_no_pipe || (!env_reg_stage && sched == MIXED_SCHED_PER_TILE);
    const bool reg_stage = env_reg_stage || (!env_no_pipe && sched == MIXED_SCHED_REGSTAGE);
    // the persistent updates read the panel from images that the panel solves write (and X
    // then stays out of S); the register-staged and one-CTA-per-tile updates read S
    const bool use_img = !reg_stage && !no_pipe;
    static bool attr = false;
    static int nsm = 1;
    if (!attr) {
        CK(cudaFuncSetAttribute(k_syrk_umma, cudaFuncAttributeMaxDynamicSharedMemorySize, UM_SMEM));
        CK(cudaFuncSetAttribute(k_syrk_pipe<64, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, PIPE_SMEM));
        CK(cudaFuncSetAttribute(k_syrk_pipe<128, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, PIPE_SMEM_WIDE));
        CK(cudaFuncSetAttribute(k_syrk_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, PAIR_SMEM));
        CK(cudaFuncSetAttribute(k_syrk_blk, cudaFuncAttributeMaxDynamicSharedMemorySize, BLK_SMEM));
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        attr = true;
    }
    // update of S[t0.., t0..cmax) by the panel columns k0 .. k0 + kw - 1: the persistent
    // pipelined kernels (one CTA per SM), or with CAPS_MIXED_NOPIPE=1 one CTA per tile.  kind:
    // UPD_BLOCK the 64 columns t0 .. t0 + 64 (left-looking, inside a half panel), UPD_MID the
    // 256 columns t0 .. t0 + 256 (the first half of a panel onto the second half), UPD_TRAIL
    // the whole trailing matrix
    enum { UPD_BLOCK, UPD_MID, UPD_TRAIL };
    auto syrk = [&](int k0, int kw, int t0, int cmax, int kind) {
        const int nr = (n - t0 + UM_M - 1) / UM_M;
        if (g_kt.on) CK(cudaEventRecord(g_kt.next(), st));
        if (no_pipe)
            k_syrk_umma<<<dim3(kind == UPD_BLOCK ? nr : nr * (nr + 1), ntask), UM_THREADS, UM_SMEM, st>>>(
                ntask, n, k0, kw, t0, cmax, kind == UPD_BLOCK, S, sstride, status);
        else if (kind == UPD_BLOCK && use_img) // from the FP16 images of the half panel's earlier blocks
            k_syrk_blk<<<std::min(ntask * nr, nsm), BLK_THREADS, BLK_SMEM, st>>>(ntask, n, k0, t0, S, sstride, status, img64);
        else if (kind != UPD_TRAIL && use_img) // UPD_MID: row blocks against the two column blocks
            k_syrk_pair<<<std::min(ntask * nr, nsm), PAIR_THREADS, PAIR_SMEM, st>>>(ntask, n, t0, kw, 1, S, sstride, status, img64);
        else if (kind != UPD_TRAIL) { // the same from S: 128 x 64 tiles, 64-column chunks
            const int ncb = (cmax - t0 + 63) / 64;
            k_syrk_pipe<64, 64><<<std::min(ntask * nr * ncb, nsm), PIPE_THREADS, PIPE_SMEM, st>>>(ntask, n, k0, kw, t0, cmax, ncb, S,
                                                                                                  sstride, status);
        } else { // the whole trailing matrix: 128 x 128 tiles
            const int tw = ntask * pipe_tiles<128>(nr, 0);
            if (use_img && kw == PIPE_IMG_CH * PIPE_IMG_TK) // the panel solves left the panel's images: row-pair items
                k_syrk_pair<<<std::min(ntask * pair_items(nr), nsm), PAIR_THREADS, PAIR_SMEM, st>>>(ntask, n, t0, kw, 0, S, sstride,
                                                                                                  status, img64);
            else
                k_syrk_pipe<128, 32><<<std::min(tw, nsm), PIPE_THREADS, PIPE_SMEM_WIDE, st>>>(ntask, n, k0, kw, t0, cmax, 0, S,
                                                                                              sstride, status);
        }
        COUNT_LAUNCH(1);
        if (g_kt.on) {
            CK(cudaEventRecord(g_kt.next(), st));
            // lower part of the target block read and written in FP32, panel rows read once
            const double r = n - t0, w = std::min(cmax, n) - t0;
            g_kt.per_matrix_bytes.push_back(8.0 * (w * r - w * (w - 1) / 2) + 4.0 * r * kw);
        }
    };
    if (convert) {
        dim3 g(256, ntask);
        k_to_delta32<<<g, 256, 0, st>>>(ntask, n, A, lda, mstride, status, S, sstride);
        COUNT_LAUNCH(1);
    }
    // diagonal block k0 and the panel solve below it; false when nothing lies below.  With
    // images, the solve writes the FP16 image of its 64 columns (every row below the diagonal
    // block), which the panel's later blocks and the trailing update after the panel read.
    constexpr int PANEL = PIPE_IMG_CH * PIPE_IMG_TK; // outer panel width, 512
    auto factor_panel = [&](int k0, bool images) {
        KernelTimer &tp = g_kts[KT_POTF2], &tt = g_kts[KT_TRSM];
        if (tp.on) CK(cudaEventRecord(tp.next(), st));
        k_potf2_w<<<ntask, 256, 0, st>>>(ntask, n, k0, S, sstride, status, Winv, part);
        COUNT_LAUNCH(1);
        if (tp.on) { // the diagonal block read and written, its inverse written
            CK(cudaEventRecord(tp.next(), st));
            tp.per_matrix_bytes.push_back(3.0 * MB * MB * 4);
        }
        const int rest = n - k0 - MB;
        if (rest <= 0) return false;
        const int blk = (k0 % PANEL) / MB; // 64-column block of the 512-column panel
        dim3 gt((rest + MT - 1) / MT, ntask);
        if (tt.on) CK(cudaEventRecord(tt.next(), st));
        k_trsm_inv<<<gt, TRSM_THREADS, 0, st>>>(ntask, n, k0, S, sstride, status, Winv, part, images ? img64 : nullptr, blk,
                                                !images);
        COUNT_LAUNCH(1);
        if (tt.on) { // the panel's rows below read; written: X (without images) or the FP16 image
            CK(cudaEventRecord(tt.next(), st));
            double w = 0;
            if (!images) w = 4.0 * rest * MB;
            if (images) w += 4.0 * rest * MB;
            tt.per_matrix_bytes.push_back(4.0 * rest * MB + w);
        }
        return true;
    };
    if (tc && !legacy_mma) {
        // panels of OUTER = 512 columns in two halves of 256: factor 64 columns at a time,
        // each first updated with its half's earlier blocks (left-looking, so every column
        // block of S passes through one such update); between the halves the first half is
        // applied to the second half's 256 columns (all rows below), and after the panel one
        // K = 512 update of the trailing matrix, which therefore passes through DRAM once per
        // 512 columns
        constexpr int OUTER = 8 * MB, HALF = OUTER / 2;
        static_assert(OUTER == PANEL && OUTER / MB == PIPE_IMG64_BLOCKS, "outer panel = image panel");
        bool more = true; // columns remain below the last factored panel
        for (int k0 = 0; k0 < n && more; k0 += OUTER) {
            for (int kh = k0; more && kh < k0 + OUTER; kh += HALF) {
                if (kh > k0) syrk(k0, HALF, kh, std::min(kh + HALF, n), UPD_MID);
                for (int kj = kh; kj < kh + HALF; kj += MB) {
                    if (kj > kh) syrk(kh, kj - kh, kj, std::min(kj + MB, n), UPD_BLOCK);
                    if (!factor_panel(kj, use_img)) { more = false; break; }
                }
            }
            const int t2 = k0 + OUTER;
            if (!more || t2 >= n) break;
            syrk(k0, OUTER, t2, n, UPD_TRAIL);
        }
    } else {
        for (int k0 = 0; k0 < n; k0 += MB) {
            if (!factor_panel(k0, false)) break;
            const int rest = n - k0 - MB, nt = (rest + 63) / 64;
            dim3 gs(nt * (nt + 1) / 2, ntask);
            if (tc)
                k_syrk_tc<<<gs, 128, 0, st>>>(ntask, n, k0, S, sstride, status);
            else
                k_syrk_f<<<gs, 64, 0, st>>>(ntask, n, k0, S, sstride, status);
            COUNT_LAUNCH(1);
        }
    }
    k_final_mixed<<<ntask, 256, 0, st>>>(ntask, n, S, sstride, mdiag, trace, status, result, mode, part);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
