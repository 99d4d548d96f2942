// syrk_pipe.cuh -- persistent, warp-specialised tcgen05 trailing updates of the mixed-form
// Cholesky: S_tile -= P_rows P_cols^T over panel columns k0 .. k0+kw, three products
// hi*hi + hi*lo + lo*hi accumulated in FP32 in tensor memory.
//
// One CTA per SM walks a static list of tiles (or items of two tiles) over all matrices of
// the batch (t = blockIdx.x, blockIdx.x + gridDim.x, ...), with three roles that overlap
// across tiles instead of running one after another:
//   * producers fill shared-memory stages with the hi/lo slices of a chunk of panel columns
//     in the canonical K-major layout (8-row x 16-byte core matrices);
//   * one thread waits for a full stage, issues the chunk's MMAs into a tensor-memory
//     accumulator, and commits to the stage's "empty" mbarrier (the slices may be
//     overwritten once the MMAs have read them) and, after a tile's last chunk, to the
//     accumulator's "full" mbarrier;
//   * epilogue warps load the tile of S, wait for the accumulator, read it back with
//     tcgen05.ld (warp w reads lanes 32 (w mod 4) .. +31 and its share of the columns), store
//     S - acc and arrive on the accumulator's "empty" mbarrier.
// Three kernels:
//   * k_syrk_pair (whole trailing matrix) and k_syrk_blk (left-looking block updates inside a
//     256-column panel) read FP16 panel images hi + lo of 2^14 x that the panel solves write:
//     one thread fills each stage with cp.async.bulk copies (completion counted on the stage's
//     "full" mbarrier by transaction bytes), kind::f16 MMAs;
//   * k_syrk_pipe (the register-staged schedule) splits the panel itself: 16 producer warps
//     load S, split each entry into TF32 hi and lo and store through registers; kind::tf32
//     MMAs (warp 16), epilogue warps 17-24.
// Every wait is bounded (PIPE_WAIT_ITERS polls of mbarrier.try_wait); a role that gives up
// marks the tile's matrix with ST_ERR_WAIT and leaves its loop, the others then give up at
// their next wait, the bulk-copy thread waits (bounded) for its last copies, the MMA thread
// waits (bounded) for the MMAs it issued, and the CTA frees its tensor memory and returns.  All roles walk the same tile list and skip the same
// tiles (matrices whose factorisation already failed).
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"
#include "umma.cuh"
#include "syrk_umma.cuh"

namespace capsgpu {

constexpr int PIPE_PRODUCER_WARPS = 16, PIPE_EPI_WARPS = 8;
constexpr int PIPE_THREADS = (PIPE_PRODUCER_WARPS + 1 + PIPE_EPI_WARPS) * 32; // 800
// tile width TN (columns of S per tile) and chunk depth TK (panel columns per stage): a
// stage holds hi + lo of the 128-row and the TN-row slice; two stages
// stage; NS stages
template <int TN, int TK, int NS = 2> struct PipeShape {
    static constexpr int STAGE = 2 * (UM_M + TN) * TK; // floats
    static constexpr int SMEM = NS * STAGE * 4;        // bytes
};
constexpr int PIPE_SMEM = PipeShape<64, 64>::SMEM;   // 192 KB
constexpr int PIPE_SMEM_WIDE = PipeShape<128, 32>::SMEM; // 128 KB
constexpr int PIPE_WAIT_ITERS = 1 << 22;
constexpr int PIPE_PRODUCERS = PIPE_PRODUCER_WARPS * 32;

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_u32(mbar)) : "memory");
}

// Stage layout: Ahi (128 x TK), Alo, Bhi (TN x TK), Blo, each slice K-major in 8-row x
// 4-column core matrices (core matrix (r / 8) (TK / 4) + k / 4, 32 floats each).

// rows [row0, row0 + R) of the panel (columns kc .. kc + nb, nb <= TK) into hi/lo slices,
// by the PIPE_PRODUCERS producer threads (ptid), 8 loads in flight per thread (measured:
// 12 loads over both slices at once ran slower under the 80-register budget of 800
// threads, and 4-byte cp.async copies with an in-place split pass slower still).
// Element e = base + u PIPE_PRODUCERS + ptid of a round sits in core matrix e / 32 =
// (base + ptid) / 32 + 16 u: a thread keeps its column k through the round and its row
// steps by 8 x 16 / (TK / 4), so the loads and stores are one base address with immediate
// offsets.
template <int R, int TK>
__device__ __forceinline__ void pipe_stage(const float *Sm, int n, int kc, int nb, int row0, float *hi_s, float *lo_s, int ptid)
{
    constexpr int ILP = 8, CPR = TK / 4; // core matrices per 8-row group
    constexpr int STEP = 8 * (PIPE_PRODUCERS / 32) / CPR;
    static_assert((R * TK) % (PIPE_PRODUCERS * ILP) == 0, "whole staging rounds");
    static_assert((PIPE_PRODUCERS / 32) % CPR == 0, "a thread keeps its column through a round");
    const int lane = ptid & 31;
#pragma unroll 1
    for (int base = 0; base < R * TK; base += PIPE_PRODUCERS * ILP) {
        const int cm0 = (base + ptid) >> 5;
        const int k = (cm0 % CPR) * 4 + (lane & 3), r0 = row0 + (cm0 / CPR) * 8 + (lane >> 2);
        const float *src = Sm + (size_t)(kc + k) * n + r0;
        const bool kok = k < nb;
        float x[ILP];
#pragma unroll
        for (int u = 0; u < ILP; u++) x[u] = (kok && r0 + STEP * u < n) ? __ldg(src + STEP * u) : 0.0f;
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

// Panel images, read by both image-fed updates (k_syrk_blk and k_syrk_pair below): 64-column
// block b = 0 .. 7 of a 512-column panel (columns k0 + 64 b ..) scaled by 2^14, rows from
// t1 = k0 + 64 (b + 1), each entry split into FP16 hi = fp16(2^14 x) and lo = fp16(2^14 x - hi),
// cut into 64-row blocks of 8 KB in the shared-memory layout of the MMA operands (K-major core
// matrices of 8 rows x 8 halves, 8-row groups 1024 B apart), all hi blocks of a matrix and then
// all lo blocks, so that a 128-row slice is two consecutive blocks:
// img[(((b ntask + task) 2 + part) pipe_img64_nrb(n) + rb) PIPE_IMG64_HALVES + e],
// e = ((q / 8) 8 + k / 8) 64 + (q mod 8) 8 + k mod 8 for row q of the block and column k.
// The left-looking update of block j reads the earlier blocks b of its 256-column half from
// their images; the middle update (the first half applied to the second half's columns, rows
// from k0 + 256) reads chunk b < 4 from 64-row block 3 - b + 2 rb, the trailing update after
// the panel (rows from k0 + 512) chunk b from 64-row block 7 - b + 2 rb.
// The panel solves that produce the panel write them (k_trsm_inv in mixed.cu).
// Range: the panel holds entries of a Cholesky factor of A = 1 - M, |x| <= sqrt(A_ii) <
// sqrt(2) for |M_ii| < 1, so 2^14 x stays below the FP16 maximum 65504 (the writer flags
// |x| >= 4).  Entries from 2^-17 up have both halves normal: 22 significant bits, as many as
// a split-TF32 pair; smaller ones keep an absolute resolution of 2^-38.  The products of two
// scaled entries are exact in the FP32 accumulator, which the update scales back by 2^-28.
constexpr int PIPE_IMG_TK = 64, PIPE_IMG_CH = 8;                        // chunk width, chunks (blocks) per panel
constexpr float PIPE_IMG_SCALE = 16384.0f, PIPE_IMG_UNSCALE2 = 1.0f / (16384.0f * 16384.0f), PIPE_IMG_XMAX = 4.0f;
constexpr int PIPE_IMG64_HALVES = 64 * 64, PIPE_IMG64_BLOCKS = PIPE_IMG_CH;
__host__ __device__ inline int pipe_img64_nrb(int n) { return 2 * ((n + UM_M - 1) / UM_M) + 2; }
// bytes of image space per matrix of dimension n
__host__ __device__ inline size_t pipe_img64_bytes(int n)
{
    return (size_t)PIPE_IMG64_BLOCKS * 2 * pipe_img64_nrb(n) * PIPE_IMG64_HALVES * 2;
}
// the FP16 pair of 2^14 x (bits of hi, lo)
__device__ __forceinline__ void img_split16(float x, uint32_t &hi, uint32_t &lo)
{
    const float s = x * PIPE_IMG_SCALE;
    const __half h = __float2half_rn(s);
    hi = __half_as_ushort(h);
    lo = __half_as_ushort(__float2half_rn(s - __half2float(h)));
}

struct PipeTile {
    int task, row0, col0;
    bool valid;
};

// tiles per matrix: ncb > 0 the first ncb column blocks of every row block, else the whole
// lower triangle (128 / TN column blocks per row block)
template <int TN> __host__ __device__ inline int pipe_tiles(int nr, int ncb)
{
    return ncb > 0 ? nr * ncb : (TN == UM_M ? nr * (nr + 1) / 2 : nr * (nr + 1));
}

// tile t of the launch: tpt tiles per matrix; ncb > 0: tile p -> (p / ncb, p mod ncb); ncb =
// 0: p -> (ri, cj) over the lower triangle (cj <= 2 ri + 1 for TN = 64, cj <= ri for TN = 128)
template <int TN>
__device__ __forceinline__ PipeTile pipe_tile(int t, int tpt, int ncb, int n, int t0, int cend, const int *status)
{
    static_assert(TN == UM_M || 2 * TN == UM_M, "tile width 64 or 128");
    PipeTile T;
    T.task = t / tpt;
    const int p = t - T.task * tpt;
    int ri = p, cj = 0;
    if (ncb > 0) {
        ri = p / ncb;
        cj = p - ri * ncb;
    } else if (TN == UM_M) {
        ri = (int)((sqrtf(8.0f * p + 1.0f) - 1.0f) * 0.5f);
        while ((ri + 1) * (ri + 2) / 2 <= p) ri++;
        while (ri * (ri + 1) / 2 > p) ri--;
        cj = p - ri * (ri + 1) / 2;
    } else {
        ri = (int)((sqrtf(4.0f * p + 1.0f) - 1.0f) * 0.5f);
        while ((ri + 1) * (ri + 2) <= p) ri++;
        while (ri * (ri + 1) > p) ri--;
        cj = p - ri * (ri + 1);
    }
    T.row0 = t0 + ri * UM_M;
    T.col0 = t0 + cj * TN;
    // skip matrices that are not being factored or failed before this launch; a wait
    // error set during this launch (ST_ERR_WAIT) does not change the walk
    const int st = status[T.task] & ~ST_ERR_WAIT;
    T.valid = st == ST_FACTOR && T.row0 < n && T.col0 < cend && T.col0 < T.row0 + UM_M;
    return T;
}

// S[t0.., t0..cmax) -= P P^T, P = columns k0 .. k0 + kw - 1, in 128 x TN tiles and TK-column
// chunks staged through registers from S; grid = min(tiles, SMs), 800 threads.  (The
// image-fed updates are k_syrk_pair and k_syrk_blk below.)
template <int TN, int TK, int NS = 2>
__global__ void __launch_bounds__(PIPE_THREADS, 1) k_syrk_pipe(int ntask, int n, int k0, int kw, int t0, int cmax, int ncb,
                                                               float *S, size_t sstride, int *status)
{
    using Shape = PipeShape<TN, TK, NS>;
    constexpr int PA = UM_M * TK, PB = TN * TK;
    extern __shared__ __align__(1024) float pipe_sm[];
    __shared__ uint64_t full[NS], empty[NS], tfull[2], tempty[2], drain;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int cend = min(n, cmax);
    const int nr = (n - t0 + UM_M - 1) / UM_M;
    const int tpt = pipe_tiles<TN>(nr, ncb);
    const int ntile = ntask * tpt;
    const int nchunk = (kw + TK - 1) / TK;

    if (warp == 0) umma::alloc(&tslot, 2 * TN);
    if (tid == 0) {
        for (int i = 0; i < NS; i++) {
            umma::mbar_init(&full[i], PIPE_PRODUCERS);
            umma::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; i++) {
            umma::mbar_init(&tfull[i], 1);
            umma::mbar_init(&tempty[i], PIPE_EPI_WARPS * 32);
        }
        umma::mbar_init(&drain, 1);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;

    // epilogue warps: 17-24; warp w reads TMEM lane quadrant w mod 4, and the two warps of
    // one quadrant take half of the tile's columns each
    const int eidx = warp > PIPE_PRODUCER_WARPS ? warp - PIPE_PRODUCER_WARPS - 1 : -1;
    if (eidx >= 0) {
        // ---- epilogue ----
        const int HW = TN / (PIPE_EPI_WARPS / 4); // columns per warp
        const int quad = warp & 3, half = eidx >> 2;
        int tt = 0;
        for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
            const PipeTile T = pipe_tile<TN>(t, tpt, ncb, n, t0, cend, status);
            if (!T.valid) continue;
            float *Sm = S + (size_t)T.task * sstride;
            const int b = tt & 1, ub = tt >> 1;
            const int R = T.row0 + quad * 32 + lane;
            bool ok = true;
            for (int part = 0; part < HW / 16; part++) {
                const int cb = T.col0 + half * HW + part * 16;
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
                umma::ld16(tmem + ((uint32_t)(quad * 32) << 16) + b * TN + half * HW + part * 16, v);
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
    } else if (warp < PIPE_PRODUCER_WARPS) {
        // ---- producers ----
        const int ptid = tid;
        int it = 0; // chunk counter (stage ring)
        for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
            const PipeTile T = pipe_tile<TN>(t, tpt, ncb, n, t0, cend, status);
            if (!T.valid) continue;
            const float *Sm = S + (size_t)T.task * sstride;
            bool ok = true;
            for (int ch = 0; ch < nchunk; ch++, it++) {
                const int s = it % NS, use = it / NS;
                if (use > 0 && !umma::mbar_wait(&empty[s], (use - 1) & 1, PIPE_WAIT_ITERS)) { ok = false; break; }
                float *st = pipe_sm + s * Shape::STAGE;
                float *Ahi = st, *Alo = Ahi + PA, *Bhi = Alo + PA, *Blo = Bhi + PB;
                const int kc = k0 + ch * TK, nb = min(TK, k0 + kw - kc);
                pipe_stage<UM_M, TK>(Sm, n, kc, nb, T.row0, Ahi, Alo, ptid);
                pipe_stage<TN, TK>(Sm, n, kc, nb, T.col0, Bhi, Blo, ptid);
                umma::fence_smem_async();
                mbar_arrive(&full[s]);
            }
            if (!ok) { atomicOr(status + T.task, ST_ERR_WAIT); break; }
        }
    } else if (warp == PIPE_PRODUCER_WARPS) {
        // ---- MMA issue (one thread) ----
        if (lane == 0) {
            int it = 0, tt = 0;
            constexpr uint32_t idesc = umma::idesc_tf32(UM_M, TN);
            constexpr uint32_t LBO = 128, SBO = (TK / 4) * 128;
            for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
                const PipeTile T = pipe_tile<TN>(t, tpt, ncb, n, t0, cend, status);
                if (!T.valid) continue;
                const int b = tt & 1, ub = tt >> 1;
                bool ok = ub == 0 || umma::mbar_wait(&tempty[b], (ub - 1) & 1, PIPE_WAIT_ITERS);
                umma::fence_after();
                const uint32_t acc = tmem + b * TN;
                for (int ch = 0; ok && ch < nchunk; ch++, it++) {
                    const int s = it % NS, use = it / NS;
                    if (!umma::mbar_wait(&full[s], use & 1, PIPE_WAIT_ITERS)) { ok = false; break; }
                    umma::fence_after();
                    const float *st = pipe_sm + s * Shape::STAGE;
                    const uint32_t ah = umma::smem_u32(st), al = ah + PA * 4, bh = al + PA * 4, bl = bh + PB * 4;
                    for (int ks = 0; ks < TK / 8; ks++) {
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
            // every MMA this thread issued completes before the CTA frees tensor memory,
            // also when a wait gave up with MMAs still in flight (bounded like every wait)
            umma::commit(&drain);
            umma::mbar_wait(&drain, 0, PIPE_WAIT_ITERS);
        }
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after();
        umma::dealloc(tmem, 2 * TN);
    }
}

// ---------------------------------------------------------------------------
// Row-pair items for the image-fed whole-trailing-matrix update
// ---------------------------------------------------------------------------
// A 128 x 128 tile needs two 128-row slices of the panel (its rows and its columns); copying
// them from L2 into shared memory bounds the update.  Here a work item is row blocks 2q and
// 2q + 1 against one column block j <= 2q, sharing the column block's slice: three slices per
// chunk for two tiles.  The diagonal tile (2q + 1, 2q + 1) and, for an odd number of row
// blocks, the last row block's tiles are items of one tile.  Row pair q has 2q + 2 items
// (columns 0 .. 2q paired, then the diagonal single), starting at item q (q + 1).  Roles:
// warp 0 lane 0 fills PAIR_STAGES stages of 64 panel columns with two bulk copies per slice
// (hi and lo of the FP16 panel images), warp 1 lane 0 issues the FP16 MMAs (hi hi + hi lo +
// lo hi, FP32 accumulation) into one 128-column accumulator per tile of the item
// (double-buffered: all 512 columns of tensor memory), warps 2..17 are the epilogue
// (warp w reads tensor-memory lanes 32 (w mod 4); the four warps of a lane quadrant split the
// columns).  Waits and failure handling as in k_syrk_pipe.
constexpr int PAIR_STAGES = 2, PAIR_EPI_WARPS = 16;
constexpr int PAIR_THREADS = (2 + PAIR_EPI_WARPS) * 32;                 // 576
constexpr int PAIR_SLICE = UM_M * PIPE_IMG_TK * 2;                      // bytes of one hi or lo slice: 16 KB
constexpr int PAIR_STAGE = 6 * PAIR_SLICE;                              // A0, A1, B (hi, lo each): 96 KB
constexpr int PAIR_SMEM = PAIR_STAGES * PAIR_STAGE;                     // 192 KB

struct PairTile {
    int task, ra, rb, col0; // rb < 0: one tile
    bool valid;
};
__host__ __device__ inline int pair_items(int nr)
{
    const int np = nr / 2;
    return np * (np + 1) + ((nr & 1) ? nr : 0);
}
__device__ __forceinline__ PairTile pair_tile(int t, int ipt, int nr, int t0, const int *status)
{
    PairTile T;
    T.task = t / ipt;
    const int p = t - T.task * ipt, np = nr / 2;
    int ra, rb = -1, cj;
    if (p < np * (np + 1)) {
        int q = (int)((sqrtf(4.0f * p + 1.0f) - 1.0f) * 0.5f);
        while ((q + 1) * (q + 2) <= p) q++;
        while (q * (q + 1) > p) q--;
        const int off = p - q * (q + 1);
        if (off <= 2 * q) { ra = 2 * q; rb = 2 * q + 1; cj = off; }
        else { ra = 2 * q + 1; cj = 2 * q + 1; }
    } else {
        ra = 2 * np;
        cj = p - np * (np + 1);
    }
    T.ra = t0 + ra * UM_M;
    T.rb = rb >= 0 ? t0 + rb * UM_M : -1;
    T.col0 = t0 + cj * UM_M;
    // skip matrices that are not being factored or failed before this launch
    T.valid = (status[T.task] & ~ST_ERR_WAIT) == ST_FACTOR;
    return T;
}
// the middle update's items: item t is row block t mod nr of matrix t / nr against the two
// column blocks t0 .. t0 + 256 (ra = rb = the rows; rb < 0 when the second block lies past n)
__device__ __forceinline__ PairTile mid_tile(int t, int nr, int n, int t0, const int *status)
{
    PairTile T;
    T.task = t / nr;
    T.ra = t0 + (t - T.task * nr) * UM_M;
    T.rb = t0 + UM_M < n ? T.ra : -1;
    T.col0 = t0;
    T.valid = (status[T.task] & ~ST_ERR_WAIT) == ST_FACTOR;
    return T;
}

// mid = 0: S[t0.., t0..) -= P P^T over the kw panel columns t0 - kw .. t0 (the start of a panel,
// so that chunk ch is image block ch); mid = 1: the same for columns t0 .. t0 + 256 only (the
// middle update of a 512-column panel: the first half applied to the second half's columns),
// items of one row block against the two column blocks, which share the row block's slice:
// the stage holds the two column slices and the row slice, and the MMAs take the row slice
// as A.  Grid = min(items, SMs), PAIR_THREADS threads, PAIR_SMEM bytes of dynamic shared memory.
__global__ void __launch_bounds__(PAIR_THREADS, 1) k_syrk_pair(int ntask, int n, int t0, int kw, int mid, float *S, size_t sstride,
                                                               int *status, const __half *img)
{
    constexpr int PA = PAIR_SLICE;
    const int nch = kw / PIPE_IMG_TK;
    extern __shared__ __align__(1024) unsigned char pair_sm[];
    __shared__ uint64_t full[PAIR_STAGES], empty[PAIR_STAGES], tfull[2], tempty[2], drain;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nr = (n - t0 + UM_M - 1) / UM_M;
    const int ipt = mid ? nr : pair_items(nr);
    const int nitem = ntask * ipt;
    auto item = [&](int t) { return mid ? mid_tile(t, nr, n, t0, status) : pair_tile(t, ipt, nr, t0, status); };

    if (warp == 0) umma::alloc(&tslot, 512);
    if (tid == 0) {
        for (int i = 0; i < PAIR_STAGES; i++) {
            umma::mbar_init(&full[i], 1);
            umma::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; i++) {
            umma::mbar_init(&tfull[i], 1);
            umma::mbar_init(&tempty[i], PAIR_EPI_WARPS * 32);
        }
        umma::mbar_init(&drain, 1);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    const int nrb64 = pipe_img64_nrb(n);
    auto slice = [&](int task, int rblock, int ch) { // hi slice of row block rblock, chunk ch (the lo slice is nrb64 blocks on)
        return img + (((size_t)ch * ntask + task) * 2 * nrb64 + nch - 1 - ch + 2 * rblock) * PIPE_IMG64_HALVES;
    };

    if (warp >= 2) {
        // ---- epilogue ----
        const int quad = warp & 3, part4 = (warp - 2) >> 2; // four warps per lane quadrant, 32 columns each
        int tt = 0;
        for (int t = blockIdx.x; t < nitem; t += gridDim.x) {
            const PairTile T = item(t);
            if (!T.valid) continue;
            float *Sm = S + (size_t)T.task * sstride;
            const int b = tt & 1, ub = tt >> 1;
            // parts p = 2 h + half: tile h (rows ra, then rb; in the middle update the column
            // blocks col0, then col0 + 128), this warp's columns 32 part4 + 16 half; the loads of
            // part p + 1 go out before the stores of part p
            const int np = T.rb >= 0 ? 4 : 2;
            // row R of part p and its columns cb + j, j < jm (inside the matrix and R >= C)
            auto row = [&](int p) { return ((p >> 1) ? T.rb : T.ra) + quad * 32 + lane; };
            auto col = [&](int p) { return T.col0 + (mid ? (p >> 1) * UM_M : 0) + part4 * 32 + (p & 1) * 16; };
            auto lim = [&](int R, int cb) { return R < n ? min(n - cb, R - cb + 1) : 0; };
            auto load = [&](int p, float (&d)[16]) {
                const int R = row(p), cb = col(p), jm = lim(R, cb);
                const float *src = Sm + (size_t)cb * n + R;
#pragma unroll
                for (int j = 0; j < 16; j++, src += n) d[j] = j < jm ? *src : 0.0f;
            };
            float cc[16], cn[16];
            load(0, cc);
            if (!umma::mbar_wait(&tfull[b], ub & 1, PIPE_WAIT_ITERS)) {
                atomicOr(status + T.task, ST_ERR_WAIT);
                break;
            }
            umma::fence_after();
#pragma unroll 1
            for (int p = 0; p < np; p++) {
                if (p + 1 < np) load(p + 1, cn);
                float v[16];
                umma::ld16(tmem + ((uint32_t)(quad * 32) << 16) + b * 256 + (p >> 1) * 128 + part4 * 32 + (p & 1) * 16, v);
                const int R = row(p), cb = col(p), jm = lim(R, cb);
                float *dst = Sm + (size_t)cb * n + R;
#pragma unroll
                for (int j = 0; j < 16; j++, dst += n)
                    if (j < jm) *dst = fmaf(v[j], -PIPE_IMG_UNSCALE2, cc[j]);
#pragma unroll
                for (int j = 0; j < 16; j++) cc[j] = cn[j];
            }
            umma::fence_before();
            mbar_arrive(&tempty[b]);
            tt++;
        }
    } else if (warp == 0) {
        // ---- producer: bulk copies of the images (one thread) ----
        if (lane == 0) {
            int it = 0, last[PAIR_STAGES];
            for (int s = 0; s < PAIR_STAGES; s++) last[s] = -1;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < nitem; t += gridDim.x) {
                const PairTile T = item(t);
                if (!T.valid) continue;
                // image row blocks of the three slices: A0, A1 (the item's rows) and B (its
                // columns); in the middle update the two column blocks and then the rows
                const int br = (T.ra - t0) / UM_M;
                const int s0 = mid ? 0 : br, s1 = mid ? 1 : (T.rb - t0) / UM_M, s2 = mid ? br : (T.col0 - t0) / UM_M;
                const bool two = T.rb >= 0;
                for (int ch = 0; ch < nch; ch++, it++) {
                    const int s = it % PAIR_STAGES, use = it / PAIR_STAGES;
                    if (use > 0 && !umma::mbar_wait(&empty[s], (use - 1) & 1, PIPE_WAIT_ITERS)) {
                        ok = false;
                        atomicOr(status + T.task, ST_ERR_WAIT);
                        break;
                    }
                    unsigned char *st = pair_sm + s * PAIR_STAGE;
                    umma::mbar_arrive_tx(&full[s], (two ? 6 : 4) * PA);
                    const size_t lo = (size_t)nrb64 * PIPE_IMG64_HALVES;
                    const __half *a0 = slice(T.task, s0, ch), *b0 = slice(T.task, s2, ch);
                    umma::bulk_g2s(st, a0, PA, &full[s]); // A0 hi, lo
                    umma::bulk_g2s(st + PA, a0 + lo, PA, &full[s]);
                    if (two) { // A1 hi, lo
                        const __half *a1 = slice(T.task, s1, ch);
                        umma::bulk_g2s(st + 2 * PA, a1, PA, &full[s]);
                        umma::bulk_g2s(st + 3 * PA, a1 + lo, PA, &full[s]);
                    }
                    umma::bulk_g2s(st + 4 * PA, b0, PA, &full[s]); // B hi, lo
                    umma::bulk_g2s(st + 5 * PA, b0 + lo, PA, &full[s]);
                    last[s] = use;
                }
            }
            // the copies complete whatever the other roles do: wait (bounded) for the last fill of
            // each stage, so that none is in flight when the CTA leaves
            for (int s = 0; s < PAIR_STAGES; s++)
                if (last[s] >= 0) umma::mbar_wait(&full[s], last[s] & 1, PIPE_WAIT_ITERS);
        }
    } else {
        // ---- MMA issue (warp 1, one thread) ----
        if (lane == 0) {
            int it = 0, tt = 0;
            constexpr uint32_t idesc = umma::idesc_f16(UM_M, UM_M);
            constexpr uint32_t LBO = 128, SBO = (PIPE_IMG_TK / 8) * 128;
            for (int t = blockIdx.x; t < nitem; t += gridDim.x) {
                const PairTile T = item(t);
                if (!T.valid) continue;
                const int b = tt & 1, ub = tt >> 1, nh = T.rb >= 0 ? 2 : 1;
                bool ok = ub == 0 || umma::mbar_wait(&tempty[b], (ub - 1) & 1, PIPE_WAIT_ITERS);
                umma::fence_after();
                for (int ch = 0; ok && ch < nch; ch++, it++) {
                    const int s = it % PAIR_STAGES, use = it / PAIR_STAGES;
                    if (!umma::mbar_wait(&full[s], use & 1, PIPE_WAIT_ITERS)) { ok = false; break; }
                    umma::fence_after();
                    const uint32_t base = umma::smem_u32(pair_sm + s * PAIR_STAGE);
                    for (int h = 0; h < nh; h++) {
                        // tile h: slot h against slot 2 (the shared slice); the middle update
                        // takes the shared row slice as A
                        const uint32_t sh = base + h * 2 * PA, sc = base + 4 * PA;
                        const uint32_t ah = mid ? sc : sh, al = ah + PA, bh = mid ? sh : sc, bl = bh + PA;
                        const uint32_t acc = tmem + b * 256 + h * 128;
                        for (int ks = 0; ks < PIPE_IMG_TK / 16; ks++) { // K = 16 halves: two core matrices
                            const uint32_t o = ks * 256;
                            umma::mma_f16(acc, umma::desc_kmajor(al + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc,
                                          ch > 0 || ks > 0);
                            umma::mma_f16(acc, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bl + o, LBO, SBO), idesc, 1);
                            umma::mma_f16(acc, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc, 1);
                        }
                    }
                    umma::commit(&empty[s]);
                }
                if (!ok) { atomicOr(status + T.task, ST_ERR_WAIT); break; }
                umma::commit(&tfull[b]);
                tt++;
            }
            // every MMA this thread issued completes before the CTA frees tensor memory
            umma::commit(&drain);
            umma::mbar_wait(&drain, 0, PIPE_WAIT_ITERS);
        }
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after();
        umma::dealloc(tmem, 512);
    }
}

// ---------------------------------------------------------------------------
// Left-looking block update from the FP16 images
// ---------------------------------------------------------------------------
// S[t0.., t0 .. t0 + 64) -= P P^T with P = columns k0 .. t0 of the current 256-column half
// of a panel (t0 - k0 = 64, 128 or 192: one 64-column chunk per earlier block of the half,
// read from that block's images), one 128 x 64 tile per row block.  Roles as in k_syrk_pair: warp 0 lane
// 0 fills BLK_STAGES stages of 48 KB with four bulk copies (A hi, A lo: two consecutive 64-row
// image blocks of 8 KB each; B hi, B lo: one block each), warp 1 lane 0 issues the FP16 MMAs
// into one of BLK_ACC 64-column accumulators, warps 2..17 are the epilogue (warp w reads lane
// quadrant w mod 4, 16 of the 64 columns).  Waits and failure handling as in k_syrk_pipe.
constexpr int BLK_STAGES = 4, BLK_ACC = 4, BLK_EPI_WARPS = 16;
constexpr int BLK_THREADS = (2 + BLK_EPI_WARPS) * 32;                     // 576
constexpr int BLK_A = UM_M * 64 * 2, BLK_B = 64 * 64 * 2;                 // bytes of one hi or lo slice
constexpr int BLK_STAGE = 2 * (BLK_A + BLK_B);                            // 48 KB
constexpr int BLK_SMEM = BLK_STAGES * BLK_STAGE;                          // 192 KB
__global__ void __launch_bounds__(BLK_THREADS, 1) k_syrk_blk(int ntask, int n, int k0, int t0, float *S, size_t sstride, int *status,
                                                             const __half *img)
{
    extern __shared__ __align__(1024) unsigned char blk_sm[];
    __shared__ uint64_t full[BLK_STAGES], empty[BLK_STAGES], tfull[BLK_ACC], tempty[BLK_ACC], drain;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int cend = min(n, t0 + 64);
    const int nr = (n - t0 + UM_M - 1) / UM_M; // row blocks: tile t -> (task t / nr, row block t mod nr)
    const int ntile = ntask * nr;
    const int nchunk = (t0 - k0) / 64;
    const int nrb64 = pipe_img64_nrb(n);

    if (warp == 0) umma::alloc(&tslot, BLK_ACC * 64);
    if (tid == 0) {
        for (int i = 0; i < BLK_STAGES; i++) {
            umma::mbar_init(&full[i], 1);
            umma::mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < BLK_ACC; i++) {
            umma::mbar_init(&tfull[i], 1);
            umma::mbar_init(&tempty[i], BLK_EPI_WARPS * 32);
        }
        umma::mbar_init(&drain, 1);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    // skip matrices that are not being factored or failed before this launch
    auto valid = [&](int task) { return (status[task] & ~ST_ERR_WAIT) == ST_FACTOR; };

    if (warp >= 2) {
        // ---- epilogue ----
        const int quad = warp & 3, part = (warp - 2) >> 2;
        // the loads of the next tile go out before the wait for this one
        // this thread's row R of tile t and its columns cb + j, j < jm (inside the block and R >= C)
        const int cb = t0 + part * 16;
        auto lim = [&](int R) { return R < n ? min(cend - cb, R - cb + 1) : 0; };
        auto load = [&](int t, float (&d)[16]) {
            const int task = t / nr, R = t0 + (t - task * nr) * UM_M + quad * 32 + lane, jm = lim(R);
            const float *src = S + (size_t)task * sstride + (size_t)cb * n + R;
#pragma unroll
            for (int j = 0; j < 16; j++) d[j] = j < jm ? src[j * n] : 0.0f;
        };
        auto next = [&](int t) {
            while (t < ntile && !valid(t / nr)) t += gridDim.x;
            return t;
        };
        int tt = 0;
        float cn[16];
        int t = next(blockIdx.x);
        if (t < ntile) load(t, cn);
        while (t < ntile) {
            float c[16];
#pragma unroll
            for (int j = 0; j < 16; j++) c[j] = cn[j];
            const int tn = next(t + gridDim.x);
            if (tn < ntile) load(tn, cn);
            const int task = t / nr, R = t0 + (t - task * nr) * UM_M + quad * 32 + lane, jm = lim(R);
            float *dst = S + (size_t)task * sstride + (size_t)cb * n + R;
            const int b = tt % BLK_ACC, ub = tt / BLK_ACC;
            if (!umma::mbar_wait(&tfull[b], ub & 1, PIPE_WAIT_ITERS)) {
                atomicOr(status + task, ST_ERR_WAIT);
                break;
            }
            umma::fence_after();
            float v[16];
            umma::ld16(tmem + ((uint32_t)(quad * 32) << 16) + b * 64 + part * 16, v);
#pragma unroll
            for (int j = 0; j < 16; j++)
                if (j < jm) dst[j * n] = fmaf(v[j], -PIPE_IMG_UNSCALE2, c[j]);
            umma::fence_before();
            mbar_arrive(&tempty[b]);
            tt++;
            t = tn;
        }
    } else if (warp == 0) {
        // ---- producer: bulk copies of the images (one thread) ----
        if (lane == 0) {
            int it = 0, last[BLK_STAGES];
            for (int s = 0; s < BLK_STAGES; s++) last[s] = -1;
            bool ok = true;
            for (int t = blockIdx.x; ok && t < ntile; t += gridDim.x) {
                const int task = t / nr, row0 = t0 + (t - task * nr) * UM_M;
                if (!valid(task)) continue;
                for (int ch = 0; ch < nchunk; ch++, it++) {
                    // chunk ch is the image of block k0 / 64 + ch of the panel, its rows counted
                    // from k0 + 64 (ch + 1)
                    const int t1 = k0 + 64 * (ch + 1), blk = (k0 % (PIPE_IMG_CH * PIPE_IMG_TK)) / 64 + ch;
                    const __half *hi0 = img + ((size_t)blk * ntask + task) * 2 * nrb64 * PIPE_IMG64_HALVES;
                    const __half *ahi = hi0 + (size_t)((row0 - t1) / 64) * PIPE_IMG64_HALVES;
                    const __half *bhi = hi0 + (size_t)((t0 - t1) / 64) * PIPE_IMG64_HALVES;
                    const int s = it % BLK_STAGES, use = it / BLK_STAGES;
                    if (use > 0 && !umma::mbar_wait(&empty[s], (use - 1) & 1, PIPE_WAIT_ITERS)) {
                        ok = false;
                        atomicOr(status + task, ST_ERR_WAIT);
                        break;
                    }
                    unsigned char *st = blk_sm + s * BLK_STAGE;
                    umma::mbar_arrive_tx(&full[s], BLK_STAGE);
                    umma::bulk_g2s(st, ahi, BLK_A, &full[s]);
                    umma::bulk_g2s(st + BLK_A, ahi + (size_t)nrb64 * PIPE_IMG64_HALVES, BLK_A, &full[s]);
                    umma::bulk_g2s(st + 2 * BLK_A, bhi, BLK_B, &full[s]);
                    umma::bulk_g2s(st + 2 * BLK_A + BLK_B, bhi + (size_t)nrb64 * PIPE_IMG64_HALVES, BLK_B, &full[s]);
                    last[s] = use;
                }
            }
            // the copies complete whatever the other roles do: wait (bounded) for the last fill of
            // each stage, so that none is in flight when the CTA leaves
            for (int s = 0; s < BLK_STAGES; s++)
                if (last[s] >= 0) umma::mbar_wait(&full[s], last[s] & 1, PIPE_WAIT_ITERS);
        }
    } else {
        // ---- MMA issue (warp 1, one thread) ----
        if (lane == 0) {
            int it = 0, tt = 0;
            constexpr uint32_t idesc = umma::idesc_f16(UM_M, 64);
            constexpr uint32_t LBO = 128, SBO = 8 * 128;
            for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
                const int task = t / nr;
                if (!valid(task)) continue;
                const int b = tt % BLK_ACC, ub = tt / BLK_ACC;
                bool ok = ub == 0 || umma::mbar_wait(&tempty[b], (ub - 1) & 1, PIPE_WAIT_ITERS);
                umma::fence_after();
                const uint32_t acc = tmem + b * 64;
                for (int ch = 0; ok && ch < nchunk; ch++, it++) {
                    const int s = it % BLK_STAGES, use = it / BLK_STAGES;
                    if (!umma::mbar_wait(&full[s], use & 1, PIPE_WAIT_ITERS)) { ok = false; break; }
                    umma::fence_after();
                    const uint32_t ah = umma::smem_u32(blk_sm + s * BLK_STAGE), al = ah + BLK_A, bh = al + BLK_A, bl = bh + BLK_B;
                    for (int ks = 0; ks < 4; ks++) { // K = 16 halves: two core matrices
                        const uint32_t o = ks * 256;
                        umma::mma_f16(acc, umma::desc_kmajor(al + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc,
                                      ch > 0 || ks > 0);
                        umma::mma_f16(acc, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bl + o, LBO, SBO), idesc, 1);
                        umma::mma_f16(acc, umma::desc_kmajor(ah + o, LBO, SBO), umma::desc_kmajor(bh + o, LBO, SBO), idesc, 1);
                    }
                    umma::commit(&empty[s]);
                }
                if (!ok) { atomicOr(status + task, ST_ERR_WAIT); break; }
                umma::commit(&tfull[b]);
                tt++;
            }
            // every MMA this thread issued completes before the CTA frees tensor memory
            umma::commit(&drain);
            umma::mbar_wait(&drain, 0, PIPE_WAIT_ITERS);
        }
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) {
        umma::fence_after();
        umma::dealloc(tmem, BLK_ACC * 64);
    }
}

} // namespace capsgpu
