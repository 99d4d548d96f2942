// syrk_pipe.cuh -- persistent, warp-specialised form of the tcgen05 trailing update
// (same arithmetic as k_syrk_umma: S_tile -= P_rows P_cols^T over a panel of kw = 64 or 128
// columns, split TF32 hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory).
//
// One CTA per SM walks a static list of 128 x 64 tiles over all matrices of the batch
// (tile t = blockIdx.x, blockIdx.x + gridDim.x, ...), with three roles that overlap
// across tiles instead of running one after another:
//   * producer warps 0-15 stage each 64-column chunk of the two panel slices, split into
//     TF32 hi/lo in the canonical K-major layout, into one of two shared-memory stages
//     (96 KB each) and arrive on that stage's "full" mbarrier;
//   * warp 16 (one thread) waits for a full stage, issues the 8 k-steps x 3 MMAs into one
//     of two 64-column tensor-memory accumulators, and commits to the stage's "empty"
//     mbarrier (the slices may be overwritten once the MMAs have read them) and, after a
//     tile's last chunk, to the accumulator's "full" mbarrier;
//   * epilogue warps 17-24 load the tile of S, wait for the accumulator, read it back with
//     tcgen05.ld (warp w reads lanes 32 (w mod 4) .. +31, columns 32 ((w - 17) / 4) .. +31),
//     store S - acc and arrive on the accumulator's "empty" mbarrier.
// Every wait is bounded (PIPE_WAIT_ITERS polls of mbarrier.try_wait); a role that gives up
// marks the tile's matrix with ST_ERR_WAIT and leaves its loop, the others then give up at
// their next wait, and the CTA frees its tensor memory and returns.  All roles walk the
// same tile list and skip the same tiles (matrices whose factorisation already failed).
#pragma once
#include "common.cuh"
#include "umma.cuh"
#include "syrk_umma.cuh"

namespace capsgpu {

constexpr int PIPE_PRODUCER_WARPS = 16, PIPE_EPI_WARPS = 8;
constexpr int PIPE_THREADS = (PIPE_PRODUCER_WARPS + 1 + PIPE_EPI_WARPS) * 32; // 800
constexpr int PIPE_STAGE_FLOATS = 2 * (UM_M + UM_N) * UM_K;                  // hi + lo of both slices
constexpr int PIPE_SMEM = 2 * PIPE_STAGE_FLOATS * 4;                         // two stages: 192 KB
constexpr int PIPE_WAIT_ITERS = 1 << 22;
constexpr int PIPE_PRODUCERS = PIPE_PRODUCER_WARPS * 32;

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_u32(mbar)) : "memory");
}

// Stage layout: Ahi (128 x 64), Alo, Bhi (64 x 64), Blo, each slice in the layout of um_off.
constexpr int PIPE_A = UM_M * UM_K, PIPE_B = UM_N * UM_K;

// rows [row0, row0 + R) of the panel (columns kc .. kc + nb) into hi/lo slices, by the
// PIPE_PRODUCERS producer threads (ptid), 8 loads in flight per thread (measured: 12 loads
// over both slices at once ran slower under the 80-register budget of 800 threads, and
// 4-byte cp.async copies with an in-place split pass slower still).
// Element e = base + u PIPE_PRODUCERS + ptid of a round sits in core matrix e / 32 =
// (base + ptid) / 32 + 16 u: a thread keeps its column k through the round and its row
// steps by 8, so the loads and stores are one base address with immediate offsets.
template <int R>
__device__ __forceinline__ void pipe_stage(const float *Sm, int n, int kc, int nb, int row0, float *hi_s, float *lo_s, int ptid)
{
    constexpr int ILP = 8, CPR = UM_K / 4; // core matrices per 8-row group
    static_assert((R * UM_K) % (PIPE_PRODUCERS * ILP) == 0, "whole staging rounds");
    static_assert(PIPE_PRODUCERS / 32 == CPR, "a round advances one 8-row group per load");
    const int lane = ptid & 31;
#pragma unroll 1
    for (int base = 0; base < R * UM_K; base += PIPE_PRODUCERS * ILP) {
        const int cm0 = (base + ptid) >> 5;
        const int k = (cm0 % CPR) * 4 + (lane & 3), r0 = row0 + (cm0 / CPR) * 8 + (lane >> 2);
        const float *src = Sm + (size_t)(kc + k) * n + r0;
        const bool kok = k < nb;
        float x[ILP];
#pragma unroll
        for (int u = 0; u < ILP; u++) x[u] = (kok && r0 + 8 * u < n) ? __ldg(src + 8 * u) : 0.0f;
        float *hd = hi_s + base + ptid, *ld = lo_s + base + ptid;
#pragma unroll
        for (int u = 0; u < ILP; u++) {
            float hi, lo;
            um_split(x[u], hi, lo);
            hd[u * PIPE_PRODUCERS] = hi;
            ld[u * PIPE_PRODUCERS] = lo;
        }
    }
}

struct PipeTile {
    int task, row0, col0;
    bool valid;
};

// tile t of the launch: tpt tiles per matrix; ncb > 0: tile p -> (p / ncb, p mod ncb), the
// first ncb column blocks; ncb = 0: p -> (ri, cj <= 2 ri + 1), the whole lower triangle
__device__ __forceinline__ PipeTile pipe_tile(int t, int tpt, int ncb, int n, int t0, int cend, const int *status)
{
    PipeTile T;
    T.task = t / tpt;
    const int p = t - T.task * tpt;
    int ri = p, cj = 0;
    if (ncb > 0) {
        ri = p / ncb;
        cj = p - ri * ncb;
    } else {
        ri = (int)((sqrtf(4.0f * p + 1.0f) - 1.0f) * 0.5f);
        while ((ri + 1) * (ri + 2) <= p) ri++;
        while (ri * (ri + 1) > p) ri--;
        cj = p - ri * (ri + 1);
    }
    T.row0 = t0 + ri * UM_M;
    T.col0 = t0 + cj * UM_N;
    // skip matrices that are not being factored or failed before this launch; a wait
    // error set during this launch (ST_ERR_WAIT) does not change the walk
    const int st = status[T.task] & ~ST_ERR_WAIT;
    T.valid = st == ST_FACTOR && T.row0 < n && T.col0 < cend && T.col0 < T.row0 + UM_M;
    return T;
}

// S[t0.., t0..cmax) -= P P^T, P = columns k0 .. k0 + kw - 1; grid = min(tiles, SMs), 800 threads
__global__ void __launch_bounds__(PIPE_THREADS, 1) k_syrk_pipe(int ntask, int n, int k0, int kw, int t0, int cmax, int ncb,
                                                               float *S, size_t sstride, int *status)
{
    extern __shared__ __align__(1024) float pipe_sm[];
    __shared__ uint64_t full[2], empty[2], tfull[2], tempty[2];
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int cend = min(n, cmax);
    const int nr = (n - t0 + UM_M - 1) / UM_M;
    const int tpt = ncb > 0 ? nr * ncb : nr * (nr + 1);
    const int ntile = ntask * tpt;
    const int nchunk = (kw + UM_K - 1) / UM_K;

    if (warp == 0) umma::alloc(&tslot, 2 * UM_N);
    if (tid == 0) {
        for (int i = 0; i < 2; i++) {
            umma::mbar_init(&full[i], PIPE_PRODUCERS);
            umma::mbar_init(&empty[i], 1);
            umma::mbar_init(&tfull[i], 1);
            umma::mbar_init(&tempty[i], PIPE_EPI_WARPS * 32);
        }
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;

    if (warp < PIPE_PRODUCER_WARPS) {
        // ---- producers ----
        const int ptid = tid;
        int it = 0; // chunk counter (stage ring)
        for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
            const PipeTile T = pipe_tile(t, tpt, ncb, n, t0, cend, status);
            if (!T.valid) continue;
            const float *Sm = S + (size_t)T.task * sstride;
            bool ok = true;
            for (int ch = 0; ch < nchunk; ch++, it++) {
                const int s = it & 1, use = it >> 1;
                if (use > 0 && !umma::mbar_wait(&empty[s], (use - 1) & 1, PIPE_WAIT_ITERS)) { ok = false; break; }
                float *st = pipe_sm + s * PIPE_STAGE_FLOATS;
                float *Ahi = st, *Alo = Ahi + PIPE_A, *Bhi = Alo + PIPE_A, *Blo = Bhi + PIPE_B;
                const int kc = k0 + ch * UM_K, nb = min(UM_K, k0 + kw - kc);
                pipe_stage<UM_M>(Sm, n, kc, nb, T.row0, Ahi, Alo, ptid);
                pipe_stage<UM_N>(Sm, n, kc, nb, T.col0, Bhi, Blo, ptid);
                umma::fence_smem_async();
                mbar_arrive(&full[s]);
            }
            if (!ok) { atomicOr(status + T.task, ST_ERR_WAIT); break; }
        }
    } else if (warp == PIPE_PRODUCER_WARPS) {
        // ---- MMA issue (one thread) ----
        if (lane == 0) {
            int it = 0, tt = 0;
            constexpr uint32_t idesc = umma::idesc_tf32(UM_M, UM_N);
            constexpr uint32_t LBO = 128, SBO = (UM_K / 4) * 128;
            for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
                const PipeTile T = pipe_tile(t, tpt, ncb, n, t0, cend, status);
                if (!T.valid) continue;
                const int b = tt & 1, ub = tt >> 1;
                bool ok = ub == 0 || umma::mbar_wait(&tempty[b], (ub - 1) & 1, PIPE_WAIT_ITERS);
                umma::fence_after();
                const uint32_t acc = tmem + b * UM_N;
                for (int ch = 0; ok && ch < nchunk; ch++, it++) {
                    const int s = it & 1, use = it >> 1;
                    if (!umma::mbar_wait(&full[s], use & 1, PIPE_WAIT_ITERS)) { ok = false; break; }
                    umma::fence_after();
                    const float *st = pipe_sm + s * PIPE_STAGE_FLOATS;
                    const uint32_t ah = umma::smem_u32(st), al = ah + PIPE_A * 4, bh = al + PIPE_A * 4, bl = bh + PIPE_B * 4;
                    for (int ks = 0; ks < UM_K / 8; ks++) {
                        const uint32_t o = ks * 256;
                        umma::mma_tf32(acc, umma::desc_kmajor(al + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc,
                                       ch > 0 || ks > 0);
                        umma::mma_tf32(acc, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bl + o, LBO, SBO), idesc, 1);
                        umma::mma_tf32(acc, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc, 1);
                    }
                    umma::commit(&empty[s]);
                }
                if (!ok) { atomicOr(status + T.task, ST_ERR_WAIT); break; }
                umma::commit(&tfull[b]);
                tt++;
            }
        }
    } else {
        // ---- epilogue: warp w reads lane quadrant w mod 4 and column half (w - 17) / 4 ----
        const int quad = warp & 3, half = (warp - PIPE_PRODUCER_WARPS - 1) >> 2;
        int tt = 0;
        for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
            const PipeTile T = pipe_tile(t, tpt, ncb, n, t0, cend, status);
            if (!T.valid) continue;
            float *Sm = S + (size_t)T.task * sstride;
            const int b = tt & 1, ub = tt >> 1;
            const int R = T.row0 + quad * 32 + lane;
            bool ok = true;
            for (int part = 0; part < 2; part++) {
                const int cb = T.col0 + half * 32 + part * 16;
                float c[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int C = cb + j;
                    c[j] = (R < n && C < cend && R >= C) ? Sm[(size_t)C * n + R] : 0.0f;
                }
                if (part == 0) {
                    ok = umma::mbar_wait(&tfull[b], ub & 1, PIPE_WAIT_ITERS);
                    umma::fence_after();
                    if (!ok) break;
                }
                float v[16];
                umma::ld16(tmem + ((uint32_t)(quad * 32) << 16) + b * UM_N + half * 32 + part * 16, v);
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const int C = cb + j;
                    if (R < n && C < cend && R >= C) Sm[(size_t)C * n + R] = c[j] - v[j];
                }
            }
            if (!ok) { atomicOr(status + T.task, ST_ERR_WAIT); break; }
            umma::fence_before();
            mbar_arrive(&tempty[b]);
            tt++;
        }
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after();
        umma::dealloc(tmem, 2 * UM_N);
    }
}

} // namespace capsgpu
