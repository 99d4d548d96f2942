// syrk_umma.cuh -- trailing update of the FP32 delta-form Cholesky on the tcgen05 tensor
// cores: S_tile -= P_rows P_cols^T over a panel P of kw = 64 or 128 columns (chunks of
// K = 64 accumulated in place), with the split-TF32 product hi*hi + hi*lo + lo*hi
// accumulated in FP32 in tensor memory.  Each tile of S is read and written once per
// call, so a 128-column panel halves the trailing matrix's DRAM traffic.
//
// One CTA of 256 threads owns a 128 x 64 tile of the lower triangle.  The threads stage
// the two panel slices into shared memory (16 independent loads in flight per thread),
// already split into TF32 hi and lo parts and laid out as the tensor cores read them
// (K-major, no swizzle: 8-row x 4-element core matrices of 128 B, 128 B apart along K
// and 2048 B apart along the rows).  Element e of a slice is the e-th float of that
// layout, so a warp writes one whole core matrix (conflict-free) and reads 8 consecutive
// rows of 4 columns (four full 32-byte sectors).  One thread issues 8 k-steps x 3 MMAs
// (M = 128, N = 64, K = 8) into a 64-column accumulator and commits them to an mbarrier;
// before the next chunk overwrites the slices every thread waits (bounded) for that
// commit.  While the last chunk's MMAs run every thread loads its 32 entries of the tile
// of S, then waits and the 8 warps subtract the accumulator: warp w reads tensor-memory
// lanes 32 (w mod 4) .. +31 (tile rows) and columns 32 (w / 4) .. +31.
#pragma once
#include "common.cuh"
#include "umma.cuh"

namespace capsgpu {

constexpr int UM_M = 128, UM_N = 64, UM_K = 64;
constexpr int UM_SMEM = 2 * (UM_M + UM_N) * UM_K * 4; // hi and lo of both slices: 96 KB
constexpr int UM_WAIT_ITERS = 1 << 20;
constexpr int UM_THREADS = 256, UM_ILP = 16;

// float offset of element (r, k) of a K-major slice with 16 core matrices along K
__device__ __forceinline__ int um_off(int r, int k) { return (((r >> 3) * (UM_K / 4) + (k >> 2)) << 5) + ((r & 7) << 2) + (k & 3); }

__device__ __forceinline__ void um_split(float x, float &hi, float &lo)
{
    uint32_t h;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(h) : "f"(x));
    hi = __uint_as_float(h);
    lo = x - hi;
}

// (r, k) of the e-th float of a slice in the layout of um_off
__device__ __forceinline__ void um_coord(int e, int &r, int &k)
{
    const int cm = e >> 5, lane = e & 31;
    r = (cm / (UM_K / 4)) * 8 + (lane >> 2);
    k = (cm % (UM_K / 4)) * 4 + (lane & 3);
}

// rows [row0, row0 + R) of the panel (columns k0 .. k0 + nb) into hi/lo slices
template <int R>
__device__ __forceinline__ void um_stage(const float *Sm, int n, int k0, int nb, int row0, float *hi_s, float *lo_s, int tid)
{
    static_assert((R * UM_K) % (UM_THREADS * UM_ILP) == 0, "whole staging rounds");
#pragma unroll 1
    for (int base = 0; base < R * UM_K; base += UM_THREADS * UM_ILP) {
        float x[UM_ILP];
#pragma unroll
        for (int u = 0; u < UM_ILP; u++) {
            int r, k;
            um_coord(base + u * UM_THREADS + tid, r, k);
            x[u] = (row0 + r < n && k < nb) ? __ldg(Sm + (size_t)(k0 + k) * n + row0 + r) : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < UM_ILP; u++) {
            const int e = base + u * UM_THREADS + tid;
            float hi, lo;
            um_split(x[u], hi, lo);
            hi_s[e] = hi;
            lo_s[e] = lo;
        }
    }
}

// S[t0.., t0..cmax) -= P P^T with P = columns k0 .. k0 + kw - 1 (rows >= t0), lower triangle.
// grid (nr (nr + 1), ntask) with nr = ceil((n - t0) / 128), tile p -> (row block ri, column
// block cj <= 2 ri + 1); with one_col, grid (nr, ntask) and tile p -> (p, 0), the single
// column block [t0, t0 + 64).  S column-major n x n per task.
__global__ void __launch_bounds__(UM_THREADS, 2) k_syrk_umma(int ntask, int n, int k0, int kw, int t0, int cmax, bool one_col,
                                                            float *S, size_t sstride, int *status)
{
    const int task = blockIdx.y;
    if (task >= ntask || status[task] != ST_FACTOR) return;
    const int p = blockIdx.x;
    int ri = p, cj = 0;
    if (!one_col) {
        ri = (int)((sqrtf(4.0f * p + 1.0f) - 1.0f) * 0.5f);
        while ((ri + 1) * (ri + 2) <= p) ri++;
        while (ri * (ri + 1) > p) ri--;
        cj = p - ri * (ri + 1);
    }
    const int cend = min(n, cmax);
    const int row0 = t0 + ri * UM_M, col0 = t0 + cj * UM_N;
    if (row0 >= n || col0 >= cend) return; // uniform per CTA

    extern __shared__ __align__(128) float um_sm[];
    float *Ahi = um_sm, *Alo = Ahi + UM_M * UM_K, *Bhi = Alo + UM_M * UM_K, *Blo = Bhi + UM_N * UM_K;
    __shared__ uint64_t mbar, drain;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    float *Sm = S + (size_t)task * sstride;

    if (warp == 0) umma::alloc(&tslot, UM_N);
    if (tid == 0) {
        umma::mbar_init(&mbar, 1);
        umma::mbar_init(&drain, 1);
    }
    const int nchunk = (kw + UM_K - 1) / UM_K;
    bool ok = true;
    for (int ch = 0; ch < nchunk; ch++) {
        if (ch > 0) {
            // the previous chunk's MMAs read the slices: wait for their commit (phase ch-1)
            // before overwriting; the decision to go on is taken by the whole CTA
            const bool mine = umma::mbar_wait(&mbar, (ch - 1) & 1, UM_WAIT_ITERS);
            if (!__syncthreads_and(mine)) { ok = false; break; }
            umma::fence_after();
        }
        const int kc = k0 + ch * UM_K, nb = min(UM_K, k0 + kw - kc);
        // stage both slices (coalesced along the rows), split into TF32 hi + lo
        um_stage<UM_M>(Sm, n, kc, nb, row0, Ahi, Alo, tid);
        um_stage<UM_N>(Sm, n, kc, nb, col0, Bhi, Blo, tid);
        umma::fence_smem_async();
        umma::fence_before();
        __syncthreads();
        umma::fence_after();
        if (tid == 0) {
            const uint32_t tmem = tslot;
            constexpr uint32_t idesc = umma::idesc_tf32(UM_M, UM_N);
            constexpr uint32_t LBO = 128, SBO = (UM_K / 4) * 128;
            const uint32_t ah = umma::smem_u32(Ahi), al = umma::smem_u32(Alo), bh = umma::smem_u32(Bhi), bl = umma::smem_u32(Blo);
            for (int ks = 0; ks < UM_K / 8; ks++) {
                const uint32_t o = ks * 256; // two core matrices along K per k-step of 8
                umma::mma_tf32(tmem, umma::desc_kmajor(al + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc,
                               ch > 0 || ks > 0);
                umma::mma_tf32(tmem, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bl + o, LBO, SBO), idesc, 1);
                umma::mma_tf32(tmem, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc, 1);
            }
            umma::commit(&mbar);
        }
    }
    const uint32_t tmem = tslot;
    // this thread's 32 entries of C, loaded while the MMAs run (the MMAs read only the
    // staged slices, never S)
    const int quad = warp & 3, half = warp >> 2;
    const int R = row0 + quad * 32 + lane, cb = col0 + half * 32;
    float c[32];
#pragma unroll
    for (int j = 0; j < 32; j++) {
        const int C = cb + j;
        c[j] = (ok && R < n && C < cend && R >= C) ? Sm[(size_t)C * n + R] : 0.0f;
    }
    if (ok) ok = umma::mbar_wait(&mbar, (nchunk - 1) & 1, UM_WAIT_ITERS);
    umma::fence_after();
    if (ok) {
        float v[32];
        umma::ld16(tmem + ((uint32_t)(quad * 32) << 16) + half * 32, *reinterpret_cast<float(*)[16]>(v));
        umma::ld16(tmem + ((uint32_t)(quad * 32) << 16) + half * 32 + 16, *reinterpret_cast<float(*)[16]>(v + 16));
#pragma unroll
        for (int j = 0; j < 32; j++) {
            const int C = cb + j;
            if (R < n && C < cend && R >= C) Sm[(size_t)C * n + R] = c[j] - v[j];
        }
    } else
        atomicOr(status + task, ST_ERR_WAIT);
    if (!ok && tid == 0) {
        // a wait gave up: the MMAs issued so far complete before tensor memory is freed
        umma::commit(&drain);
        umma::mbar_wait(&drain, 0, UM_WAIT_ITERS);
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after();
        umma::dealloc(tmem, UM_N);
    }
}

} // namespace capsgpu
