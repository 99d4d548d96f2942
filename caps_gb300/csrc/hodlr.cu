// hodlr.cu -- batched HODLR log-determinant of 1 - M on the GPU, FP64, with the matrix
// elements evaluated on demand (libhodlr: src/libhodlr/src/hodlr.cpp:34-55, HODLR_Tree.cpp,
// HODLR_Node.cpp, HODLR_Matrix.cpp:66-389 rookPiv, HODLR_Tree_SPD.cpp:6-454).
//
// A = 1 - M (symmetric positive definite) is split recursively in halves down to leaves of at
// most HL_LEAF rows.  Every off-diagonal block of a node, B = A[child 0, child 1], is
// compressed as U V^T by adaptive cross approximation with rook pivoting: the rows and columns
// it visits are the only elements of B that are ever formed, each from I values computed for
// that row or column alone (qsum64.cuh, the same arithmetic as the dense path).  The
// determinant then follows the symmetric factorisation A = W W^T: leaves by dense Cholesky,
// each node by a thin QR of its two bases whitened by the factors below it (Q0 R0 = W_0^{-1} U,
// Q1 R1 = W_1^{-1} V), K = R0 R1^T and the Cholesky factor of I - K^T K, so that
//   log det A = 2 sum_leaves sum log L_ii + 2 sum_nodes sum log Lk_ii.
// Each factor is applied to the row slices of its ancestors' bases before they are used.
//
// GPU form: one CUDA block per (matrix, node) for the compression and per (matrix, node) of
// one level for the factorisation, all matrices of a batch and all nodes of a level in one
// launch.  Row and column requests compute a strip of I values (three consecutive l of one
// index, a range of the other) with one q-sum per thread, then the elements.
//
// Compression rule (HODLR_Matrix.cpp:66-389): pivot row first row of the block; the residual
// row's largest unused entry is the pivot column; the residual column's largest unused entry
// the next pivot row; a pivot below the tolerance is replaced by another row (the ends of
// the block, then the midpoint of the widest gap between chosen rows; the reference
// alternates that midpoint with a random row); the loop stops when
//   rank (n0 + n1) |row| |col| <= |pivot| tol ||U V^T||_F^2 (estimated as the reference does)
// or the rank reaches min(n0, n1); a rank of min(n0, n1) - 1 or more stores the block exactly.
// tol = max(1e-13, 1e-13 tr M) (matrix.c:133-139).  A block whose rank would exceed HL_RMAX
// marks its matrix with ST_ERR_HODLR; the caller factors those matrices densely.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "qsum64.cuh"
#include "qsum_ff.cuh"

namespace capsgpu {

constexpr int HL_LEAF = 128; // largest leaf
constexpr int HL_RMAX = 128; // largest rank of an off-diagonal block
constexpr int HL_T = 256;    // threads per block
constexpr int HL_MAX_TRIES = 200;

struct HNode {
    int start, size, c0;   // rows [start, start + size), first child c0 rows
    long long qoff;        // offset (doubles) of the bases in a matrix's area: U (c0 x RMAX) then V
};

struct HCtx {
    const Task *tasks;
    const int *tlist; // chunk index of batch entry h
    int ldim;
    const sd *K;
    int nu_stride;
    const double4 *ptab;
    int pstride;
    const double *lft;
    const sd *Sa, *Sb;
    const double2 *uv;
    const HNode *nodes; // 2^(NL+1) - 1 nodes, level-major
    int NL;
    long long qstride;  // doubles of basis storage per matrix
    double *Q;
    int *rank;          // per matrix and node
    const double *trace;
    int *status;
    double *part;       // per matrix: one log-det partial per node (leaves included), level-major
    // mixed form: the I values by the float-float q-sums (paired K table, float-float p
    // tables and a_0..a_2 tables per m group); the rest of the path stays FP64
    int mixed;
    const float4 *KP;
    const int *KPe;
    const float4 *ptabf;
    const A12L *tl;
    const A12J *tj;
};

__device__ __forceinline__ int node_id(int level, int k) { return (1 << level) - 1 + k; }

// ---------------------------------------------------------------------------------------
// block-wide reductions (HL_T threads)
// ---------------------------------------------------------------------------------------
__device__ double blk_sum(double v, double *red)
{
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < HL_T / 32; i++) s += red[i];
        red[0] = s;
    }
    __syncthreads();
    s = red[0];
    __syncthreads();
    return s;
}

// largest |v| over the threads' candidates (index < 0: none); ties go to the lowest index
__device__ void blk_argmax(double v, int idx, double *redv, int *redi, double &vmax, int &imax)
{
    double a = idx >= 0 ? fabs(v) : -1.0;
    int i = idx;
    double sv = v;
    for (int o = 16; o; o >>= 1) {
        const double a2 = __shfl_xor_sync(0xffffffffu, a, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, i, o);
        const double s2 = __shfl_xor_sync(0xffffffffu, sv, o);
        if (a2 > a || (a2 == a && i2 >= 0 && (i < 0 || i2 < i))) { a = a2; i = i2; sv = s2; }
    }
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) { redv[2 * w] = a; redv[2 * w + 1] = sv; redi[w] = i; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ba = -1.0, bs = 0.0;
        int bi = -1;
        for (int k = 0; k < HL_T / 32; k++) {
            const double ak = redv[2 * k];
            const int ik = redi[k];
            if (ak > ba || (ak == ba && ik >= 0 && (bi < 0 || ik < bi))) { ba = ak; bi = ik; bs = redv[2 * k + 1]; }
        }
        redv[0] = bs;
        redi[0] = bi;
    }
    __syncthreads();
    vmax = redv[0];
    imax = redi[0];
    __syncthreads();
}

// ---------------------------------------------------------------------------------------
// elements on demand
// ---------------------------------------------------------------------------------------
// I(x, y) (TM, TE) of chunk task `task`, x, y indices into [lmin-1, lmin+ldim]
__device__ void hl_ipair(const HCtx &C, int task, int x, int y, sd &tm, sd &te)
{
    const Task &T = C.tasks[task];
    const int a1 = max(x, y), a2 = min(x, y);
    const int l1 = T.lmin - 1 + a1, l2 = T.lmin - 1 + a2;
    const int mm = T.m > 0 ? T.m : 1;
    if (l2 < mm || l2 < T.m || l1 < 1) { // I = 0 for l < m (integration.c:631)
        tm = te = sd{0, 0};
        return;
    }
    if (C.mixed) {
        const int g = T.mgroup, L = C.ldim + 2;
        const A012F A = a012f_pair(T.m, T.lmin, a1, a2, C.tl + (size_t)g * L, C.tj + (size_t)g * (2 * L - 1));
        auto put = [&](int, int pol, float h, float l, int e) { (pol ? tm : te) = sd_norm((double)h + (double)l, e); };
        if (qsum_ff_pair<1>(T, &task, 1, l1, l2, A, C.KP, C.KPe, C.nu_stride, C.ptabf + (size_t)g * 2 * C.pstride * 2, C.pstride,
                            QSUM_FF_STOP_BITS, put))
            atomicOr(C.status + task, ST_ERR_NONFINITE);
        return;
    }
    const A012 A = a012_pair(T.m, T.lmin, a1, a2, C.lft);
    if (qsum_pair(T, l1, l2, A, C.K + (size_t)(task * 2 + 1) * C.nu_stride - T.mu, C.K + (size_t)(task * 2) * C.nu_stride - T.mu,
                  C.ptab + (size_t)task * 2 * C.pstride, C.pstride, tm, te))
        atomicOr(C.status + task, ST_ERR_NONFINITE);
}

// strip[k][w] = I(t0 + k, v0 + w), k = 0..2 (only k = 1 for m = 0), w < W; TM then TE
__device__ void hl_strip(const HCtx &C, int task, int t0, int v0, int W, sd *strip)
{
    const bool m0 = C.tasks[task].m == 0;
    for (int it = threadIdx.x; it < 3 * W; it += HL_T) {
        const int k = it / W, w = it - k * W;
        if (m0 && k != 1) continue;
        sd tm, te;
        hl_ipair(C, task, t0 + k, v0 + w, tm, te);
        strip[(size_t)(2 * k) * W + w] = tm;
        strip[(size_t)(2 * k + 1) * W + w] = te;
    }
}

// M(r, c), r >= c matrix indices, from an I lookup Iv(pol, x, y) (pol 1 = TM): the entry
// (r mod 2, c mod 2) of the 2x2 block at l-indices (r/2, c/2) -- EE, ME, EM, MM as the dense
// assembly stores the lower triangle (assemble.cu k_elem)
template <class IV> __device__ double hl_lower(const HCtx &C, int task, int r, int c, IV Iv)
{
    const Task &T = C.tasks[task];
    const int a = r >> 1, b = c >> 1, i1 = a + 1, i2 = b + 1;
    const int L = C.ldim + 2;
    const size_t so = (size_t)task * L;
    sd EE, MM, EM, ME;
    elem_block<false>(T.m, i1, i2, C.Sa[so + i1], C.Sa[so + i2], C.Sb[so + i1], C.Sb[so + i2], C.uv[so + i1], C.uv[so + i2], Iv, EE,
                      MM, EM, ME);
    const int pr = r & 1, pc = c & 1;
    const sd v = pr == 0 ? (pc == 0 ? EE : EM) : (pc == 0 ? ME : MM);
    const double d = sd_to_double(v);
    if (!isfinite(d)) atomicOr(C.status + task, ST_ERR_NONFINITE);
    return d;
}

// ---------------------------------------------------------------------------------------
// compression of the off-diagonal block of every node of one level
// ---------------------------------------------------------------------------------------
// per block scratch: row (n1), col (n0), two strips (6 W sd each: rows, columns), used rows
// (n0), used columns (n1)
__host__ __device__ inline size_t hl_aca_scratch(int n0, int n1)
{
    const int W = max(n0, n1) / 2 + 4;
    return ((size_t)(n0 + n1) * 8 + (size_t)12 * W * sizeof(sd) + (size_t)(n0 + n1) + 255) & ~(size_t)255;
}

// grid (nodes of the level, batch); blockIdx.x = node k of level `level`
__global__ void __launch_bounds__(HL_T) k_hodlr_aca(HCtx C, int level, unsigned char *scratch, size_t scratch_per)
{
    const int h = blockIdx.y, k = blockIdx.x;
    const int task = C.tlist[h];
    const int nid = node_id(level, k);
    const HNode N = C.nodes[nid];
    const int n0 = N.c0, n1 = N.size - N.c0;
    const int r0s = N.start, c1s = N.start + N.c0;
    __shared__ double redv[2 * HL_T / 32];
    __shared__ int redi[HL_T / 32];
    __shared__ double red[HL_T / 32];
    __shared__ int s_rows[4]; // the replacement row picked by thread 0
    __shared__ int s_skip;
    // the block decides once (other blocks may set status bits meanwhile)
    if (threadIdx.x == 0) s_skip = (C.status[task] & ~0xF) != 0;
    __syncthreads();
    if (s_skip) return;

    unsigned char *sc = scratch + ((size_t)h * gridDim.x + k) * scratch_per;
    double *row = (double *)sc, *col = row + n1;
    const int W = max(n0, n1) / 2 + 4;
    sd *stripR = (sd *)(col + n0), *stripC = stripR + (size_t)6 * W;
    unsigned char *usedR = (unsigned char *)(stripC + (size_t)6 * W), *usedC = usedR + n0;
    // the strip of the last row (column) request: the two polarisation rows (columns) of one l
    // read the same I values, so a request for the other one reuses them
    int strip_row_l = -1, strip_col_l = -1;
    double *U = C.Q + (size_t)h * C.qstride + N.qoff, *V = U + (size_t)n0 * HL_RMAX;
    for (int i = threadIdx.x; i < n0; i += HL_T) usedR[i] = 0;
    for (int j = threadIdx.x; j < n1; j += HL_T) usedC[j] = 0;
    const double tol = fmax(1e-13, C.trace[task] * 1e-13);
    const int rmin = min(n0, n1);
    __syncthreads();

    // residual row i over the block's columns: -M(r0s + i, c1s + j) - sum_k U[i,k] V[j,k]
    auto get_row = [&](int i, int rank) {
        const int gi = r0s + i, b = gi >> 1;
        const int v0 = c1s >> 1, Wr = ((c1s + n1 - 1) >> 1) - v0 + 3;
        if (b != strip_row_l) {
            hl_strip(C, task, b, v0, Wr, stripR);
            strip_row_l = b;
            __syncthreads();
        }
        // M(gi, gj) = lower(gj, gi): x = gj/2 + {0,1,2} varies, y = b + {0,1,2} fixed
        auto Iv = [&](int p, int x, int y) { return stripR[(size_t)(2 * (y - b) + (p ? 0 : 1)) * Wr + (x - v0)]; };
        for (int j = threadIdx.x; j < n1; j += HL_T) {
            double v = -hl_lower(C, task, c1s + j, gi, Iv);
            for (int q = 0; q < rank; q++) v -= U[(size_t)q * n0 + i] * V[(size_t)q * n1 + j];
            row[j] = v;
        }
        __syncthreads();
    };
    // residual column j over the block's rows
    auto get_col = [&](int j, int rank) {
        const int gj = c1s + j, a = gj >> 1;
        const int v0 = r0s >> 1, Wc = ((r0s + n0 - 1) >> 1) - v0 + 3;
        if (a != strip_col_l) {
            hl_strip(C, task, a, v0, Wc, stripC);
            strip_col_l = a;
            __syncthreads();
        }
        // M(gi, gj) = lower(gj, gi): x = a + {0,1,2} fixed, y = gi/2 + {0,1,2} varies
        auto Iv = [&](int p, int x, int y) { return stripC[(size_t)(2 * (x - a) + (p ? 0 : 1)) * Wc + (y - v0)]; };
        for (int i = threadIdx.x; i < n0; i += HL_T) {
            double v = -hl_lower(C, task, gj, r0s + i, Iv);
            for (int q = 0; q < rank; q++) v -= V[(size_t)q * n1 + j] * U[(size_t)q * n0 + i];
            col[i] = v;
        }
        __syncthreads();
    };

    int rank = 0, irow = 0, nrows_chosen = 0;
    double norm2 = 0.0;
    bool overflow = false;
    bool at_end = false; // thread 0 alone uses it
    if (threadIdx.x == 0) usedR[0] = 1;
    nrows_chosen = 1;
    __syncthreads();
    for (;;) {
        get_row(irow, rank);
        double mx;
        int jp;
        {
            double best = 0.0;
            int bi = -1;
            for (int j = threadIdx.x; j < n1; j += HL_T)
                if (!usedC[j] && (bi < 0 || fabs(row[j]) > fabs(best))) { best = row[j]; bi = j; }
            blk_argmax(best, bi, redv, redi, mx, jp);
        }
        int tries = 0;
        while (fabs(mx) < tol && tries < HL_MAX_TRIES && jp >= 0) {
            // replace the row: the ends of the block while fewer than three rows are chosen,
            // then the midpoint of the widest gap between chosen rows (nearest unused row)
            if (threadIdx.x == 0) {
                int pick = -1;
                if (nrows_chosen < 3) {
                    if (at_end) { for (int i = n0 - 1; i >= 0; i--) if (!usedR[i]) { pick = i; break; } }
                    else { for (int i = 0; i < n0; i++) if (!usedR[i]) { pick = i; break; } }
                    at_end = !at_end;
                } else {
                    int prev = -1, gbest = -1, gl = 0;
                    for (int i = 0; i < n0; i++)
                        if (usedR[i]) {
                            if (prev >= 0 && i - prev > gbest) { gbest = i - prev; gl = prev; }
                            prev = i;
                        }
                    const int mid = gl + gbest / 2;
                    for (int d = 0; d < n0 && pick < 0; d++) {
                        if (mid + d < n0 && !usedR[mid + d]) pick = mid + d;
                        else if (mid - d >= 0 && !usedR[mid - d]) pick = mid - d;
                    }
                }
                if (pick >= 0) usedR[pick] = 1;
                s_rows[0] = pick;
            }
            __syncthreads();
            const int pick = s_rows[0];
            __syncthreads();
            if (pick < 0) { jp = -1; break; }
            irow = pick;
            nrows_chosen++;
            get_row(irow, rank);
            double best = 0.0;
            int bi = -1;
            for (int j = threadIdx.x; j < n1; j += HL_T)
                if (!usedC[j] && (bi < 0 || fabs(row[j]) > fabs(best))) { best = row[j]; bi = j; }
            blk_argmax(best, bi, redv, redi, mx, jp);
            tries++;
        }
        if (jp < 0 || tries == HL_MAX_TRIES || fabs(mx) < tol) break;
        if (rank == HL_RMAX) { overflow = true; break; }
        if (threadIdx.x == 0) usedC[jp] = 1;
        __syncthreads();
        get_col(jp, rank);
        double cmx;
        int inext;
        {
            double best = 0.0;
            int bi = -1;
            for (int i = threadIdx.x; i < n0; i += HL_T)
                if (!usedR[i] && (bi < 0 || fabs(col[i]) > fabs(best))) { best = col[i]; bi = i; }
            blk_argmax(best, bi, redv, redi, cmx, inext);
        }
        // new basis vectors: U_rank = col / pivot, V_rank = row
        const double g = 1.0 / mx;
        double rs = 0.0, cs = 0.0;
        for (int j = threadIdx.x; j < n1; j += HL_T) { V[(size_t)rank * n1 + j] = row[j]; rs += row[j] * row[j]; }
        for (int i = threadIdx.x; i < n0; i += HL_T) { U[(size_t)rank * n0 + i] = g * col[i]; cs += col[i] * col[i]; }
        rs = blk_sum(rs, red);
        cs = blk_sum(cs, red);
        double add = fabs(g * g * rs * cs);
        for (int q = 0; q < rank; q++) {
            double du = 0.0, dv = 0.0;
            for (int i = threadIdx.x; i < n0; i += HL_T) du += U[(size_t)q * n0 + i] * U[(size_t)rank * n0 + i];
            for (int j = threadIdx.x; j < n1; j += HL_T) dv += V[(size_t)q * n1 + j] * V[(size_t)rank * n1 + j];
            du = blk_sum(du, red);
            dv = blk_sum(dv, red);
            add += 2.0 * fabs(du) * fabs(dv);
        }
        norm2 += add;
        rank++;
        if (!(rank * (double)(n0 + n1) * sqrt(rs) * sqrt(cs) > fabs(mx) * tol * norm2 && rank < rmin)) break;
        if (inext < 0) break;
        irow = inext;
        if (threadIdx.x == 0) usedR[irow] = 1;
        nrows_chosen++;
        __syncthreads();
    }
    if (!overflow && rank >= rmin - 1) {
        // the block stored exactly (HODLR_Matrix.cpp:360-375): identity on the shorter side
        if (rmin > HL_RMAX) overflow = true;
        else if (n0 <= n1) {
            for (int q = 0; q < n0; q++) {
                for (int i = threadIdx.x; i < n0; i += HL_T) U[(size_t)q * n0 + i] = i == q ? 1.0 : 0.0;
                get_row(q, 0);
                for (int j = threadIdx.x; j < n1; j += HL_T) V[(size_t)q * n1 + j] = row[j];
                __syncthreads();
            }
            rank = n0;
        } else {
            for (int q = 0; q < n1; q++) {
                for (int j = threadIdx.x; j < n1; j += HL_T) V[(size_t)q * n1 + j] = j == q ? 1.0 : 0.0;
                get_col(q, 0);
                for (int i = threadIdx.x; i < n0; i += HL_T) U[(size_t)q * n0 + i] = col[i];
                __syncthreads();
            }
            rank = n1;
        }
    }
    if (threadIdx.x == 0) {
        C.rank[(size_t)h * ((2 << C.NL) - 1) + nid] = overflow ? 0 : rank;
        if (overflow) atomicOr(C.status + task, ST_ERR_HODLR);
    }
}

// ---------------------------------------------------------------------------------------
// leaves: dense block, Cholesky, whitening of the ancestors' bases
// ---------------------------------------------------------------------------------------
// scratch per block: the I window (W x W, both polarisations), W = HL_LEAF / 2 + 4
__host__ __device__ inline size_t hl_leaf_scratch() { return (size_t)2 * (HL_LEAF / 2 + 4) * (HL_LEAF / 2 + 4) * sizeof(sd); }

// grid (leaves, batch), dynamic shared memory HL_LEAF^2 doubles
__global__ void __launch_bounds__(HL_T) k_hodlr_leaf(HCtx C, unsigned char *scratch)
{
    extern __shared__ double Lf[];
    const int h = blockIdx.y, k = blockIdx.x;
    const int task = C.tlist[h];
    const int nid = node_id(C.NL, k);
    const HNode N = C.nodes[nid];
    const int s = N.size, s0 = N.start;
    __shared__ int bad, s_skip;
    if (threadIdx.x == 0) s_skip = (C.status[task] & ~0xF) != 0;
    __syncthreads();
    if (s_skip) return;
    // I window over l-indices [lo, lo + W)
    const int lo = s0 >> 1, W = ((s0 + s - 1) >> 1) - lo + 3;
    sd *Iw = (sd *)(scratch + ((size_t)h * gridDim.x + k) * hl_leaf_scratch());
    for (int it = threadIdx.x; it < W * W; it += HL_T) {
        const int x = it / W, y = it - x * W;
        if (x < y) continue;
        sd tm, te;
        hl_ipair(C, task, lo + x, lo + y, tm, te);
        Iw[(size_t)(x * W + y) * 2] = tm;
        Iw[(size_t)(x * W + y) * 2 + 1] = te;
        Iw[(size_t)(y * W + x) * 2] = tm;
        Iw[(size_t)(y * W + x) * 2 + 1] = te;
    }
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    auto Iv = [&](int p, int x, int y) { return Iw[(size_t)((x - lo) * W + (y - lo)) * 2 + (p ? 0 : 1)]; };
    // A = 1 - M, lower triangle, column-major s x s
    for (int it = threadIdx.x; it < s * s; it += HL_T) {
        const int r = it % s, c = it / s;
        if (r < c) continue;
        const double mv = hl_lower(C, task, s0 + r, s0 + c, Iv);
        Lf[(size_t)c * s + r] = (r == c ? 1.0 : 0.0) - mv;
    }
    __syncthreads();
    // right-looking Cholesky in shared memory
    for (int j = 0; j < s; j++) {
        if (threadIdx.x == 0) {
            const double d = Lf[(size_t)j * s + j];
            if (!(d > 0.0)) bad = 1;
            Lf[(size_t)j * s + j] = d > 0.0 ? sqrt(d) : 1.0;
        }
        __syncthreads();
        const double piv = Lf[(size_t)j * s + j];
        for (int i = j + 1 + threadIdx.x; i < s; i += HL_T) Lf[(size_t)j * s + i] /= piv;
        __syncthreads();
        const int rest = s - j - 1;
        for (int it = threadIdx.x; it < rest * rest; it += HL_T) {
            const int r = j + 1 + it % rest, c = j + 1 + it / rest;
            if (r >= c) Lf[(size_t)c * s + r] -= Lf[(size_t)j * s + r] * Lf[(size_t)j * s + c];
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) atomicOr(C.status + task, ST_ERR_PIVOT);
        return;
    }
    if (threadIdx.x == 0) {
        double sum = 0.0, cc = 0.0;
        for (int j = 0; j < s; j++) { // Kahan, in index order
            const double y = log(Lf[(size_t)j * s + j]) - cc, t = sum + y;
            cc = (t - sum) - y;
            sum = t;
        }
        C.part[(size_t)h * ((2 << C.NL) - 1) + nid] = 2.0 * sum;
    }
    // whiten the ancestors' bases: rows of this leaf, L^{-1} X
    int child = k, parent = k;
    for (int l = C.NL - 1; l >= 0; l--) {
        child = parent & 1;
        parent >>= 1;
        const int pid = node_id(l, parent);
        const HNode P = C.nodes[pid];
        const int r = C.rank[(size_t)h * ((2 << C.NL) - 1) + pid];
        const int cs = child ? P.size - P.c0 : P.c0, cstart = child ? P.start + P.c0 : P.start;
        double *X = C.Q + (size_t)h * C.qstride + P.qoff + (child ? (size_t)P.c0 * HL_RMAX : 0) + (s0 - cstart);
        for (int q = threadIdx.x; q < r; q += HL_T) {
            double *x = X + (size_t)q * cs;
            for (int i = 0; i < s; i++) {
                double v = x[i];
                for (int t = 0; t < i; t++) v -= Lf[(size_t)t * s + i] * x[t];
                x[i] = v / Lf[(size_t)i * s + i];
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------------------
// nodes of one level: thin QR of both whitened bases, K = R0 R1^T, chol(I - K^T K), and the
// node's factor applied to its ancestors' bases
// ---------------------------------------------------------------------------------------
// scratch per block: R0, R1, K, Lk (RMAX^2 each) and two vectors of 2 RMAX
__host__ __device__ inline size_t hl_node_scratch(int r) { return ((size_t)4 * r * r + 4 * HL_RMAX) * sizeof(double); }

// thin QR of X (rows x r, column-major, ld rows) in place by classical Gram-Schmidt with one
// reorthogonalisation; R (r x r, column-major) upper triangular
__device__ void hl_qr(double *X, int rows, int r, double *R, double *red, double *hv)
{
    for (int i = threadIdx.x; i < r * r; i += HL_T) R[i] = 0.0;
    __syncthreads();
    for (int c = 0; c < r; c++) {
        double *v = X + (size_t)c * rows;
        for (int pass = 0; pass < 2; pass++) {
            // h = Q[:, :c]^T v, one warp per coefficient
            const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
            for (int q = w; q < c; q += HL_T / 32) {
                double d = 0.0;
                for (int i = ln; i < rows; i += 32) d += X[(size_t)q * rows + i] * v[i];
                for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
                if (ln == 0) hv[q] = d;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < rows; i += HL_T) {
                double s = v[i];
                for (int q = 0; q < c; q++) s -= X[(size_t)q * rows + i] * hv[q];
                v[i] = s;
            }
            for (int q = threadIdx.x; q < c; q += HL_T) R[(size_t)c * r + q] += hv[q];
            __syncthreads();
        }
        double nn = 0.0;
        for (int i = threadIdx.x; i < rows; i += HL_T) nn += v[i] * v[i];
        nn = sqrt(blk_sum(nn, red));
        const double inv = nn > 0.0 ? 1.0 / nn : 0.0;
        for (int i = threadIdx.x; i < rows; i += HL_T) v[i] *= inv;
        if (threadIdx.x == 0) R[(size_t)c * r + c] = nn;
        __syncthreads();
    }
}

// grid (nodes of the level, batch); dynamic shared memory none
__global__ void __launch_bounds__(HL_T) k_hodlr_node(HCtx C, int level, unsigned char *scratch, size_t scratch_per)
{
    const int h = blockIdx.y, k = blockIdx.x;
    const int task = C.tlist[h];
    const int nid = node_id(level, k);
    const HNode N = C.nodes[nid];
    const int n0 = N.c0, n1 = N.size - N.c0;
    const int r = C.rank[(size_t)h * ((2 << C.NL) - 1) + nid];
    __shared__ double red[HL_T / 32];
    __shared__ int bad, s_skip;
    if (threadIdx.x == 0) s_skip = (C.status[task] & ~0xF) != 0;
    __syncthreads();
    if (s_skip) return;
    double *sc = (double *)(scratch + ((size_t)h * gridDim.x + k) * scratch_per);
    double *R0 = sc, *R1 = R0 + (size_t)r * r, *Km = R1 + (size_t)r * r, *Lk = Km + (size_t)r * r;
    double *hv = Lk + (size_t)r * r, *tv = hv + HL_RMAX, *sv = tv + HL_RMAX, *wv = sv + HL_RMAX;
    double *Q0 = C.Q + (size_t)h * C.qstride + N.qoff, *Q1 = Q0 + (size_t)n0 * HL_RMAX;
    if (r == 0) {
        if (threadIdx.x == 0) C.part[(size_t)h * ((2 << C.NL) - 1) + nid] = 0.0;
        return; // a zero block: the node's factor is the identity
    }
    hl_qr(Q0, n0, r, R0, red, hv);
    hl_qr(Q1, n1, r, R1, red, hv);
    // K = R0 R1^T; G = I - K^T K (lower triangle into Lk), then Cholesky in place
    for (int it = threadIdx.x; it < r * r; it += HL_T) {
        const int i = it % r, j = it / r;
        double s = 0.0;
        for (int t = max(i, j); t < r; t++) s += R0[(size_t)t * r + i] * R1[(size_t)t * r + j];
        Km[(size_t)j * r + i] = s;
    }
    __syncthreads();
    for (int it = threadIdx.x; it < r * r; it += HL_T) {
        const int i = it % r, j = it / r;
        if (i < j) continue;
        double s = i == j ? 1.0 : 0.0;
        for (int t = 0; t < r; t++) s -= Km[(size_t)i * r + t] * Km[(size_t)j * r + t];
        Lk[(size_t)j * r + i] = s;
    }
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < r; j++) {
        if (threadIdx.x == 0) {
            const double d = Lk[(size_t)j * r + j];
            if (!(d > 0.0)) bad = 1;
            Lk[(size_t)j * r + j] = d > 0.0 ? sqrt(d) : 1.0;
        }
        __syncthreads();
        const double piv = Lk[(size_t)j * r + j];
        for (int i = j + 1 + threadIdx.x; i < r; i += HL_T) Lk[(size_t)j * r + i] /= piv;
        __syncthreads();
        const int rest = r - j - 1;
        for (int it = threadIdx.x; it < rest * rest; it += HL_T) {
            const int a = j + 1 + it % rest, b = j + 1 + it / rest;
            if (a >= b) Lk[(size_t)b * r + a] -= Lk[(size_t)j * r + a] * Lk[(size_t)j * r + b];
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) atomicOr(C.status + task, ST_ERR_PIVOT);
        return;
    }
    if (threadIdx.x == 0) {
        double sum = 0.0, cc = 0.0;
        for (int j = 0; j < r; j++) {
            const double y = log(Lk[(size_t)j * r + j]) - cc, t = sum + y;
            cc = (t - sum) - y;
            sum = t;
        }
        C.part[(size_t)h * ((2 << C.NL) - 1) + nid] = 2.0 * sum;
    }
    // the node's factor W = [I 0; Q1 K^T Q0^T, I + Q1 (Lk - I) Q1^T] applied to each ancestor's
    // slice b = [b1; b2] over this node's rows (HODLR_Tree_SPD.cpp:170-186):
    //   t = Q1^T b2, u = K^T Q0^T b1 - t, b2 -= Q1 (Lk^{-1} u + t)
    int parent = k, child;
    for (int l = level - 1; l >= 0; l--) {
        child = parent & 1;
        parent >>= 1;
        const int pid = node_id(l, parent);
        const HNode P = C.nodes[pid];
        const int ra = C.rank[(size_t)h * ((2 << C.NL) - 1) + pid];
        const int cs = child ? P.size - P.c0 : P.c0, cstart = child ? P.start + P.c0 : P.start;
        double *X = C.Q + (size_t)h * C.qstride + P.qoff + (child ? (size_t)P.c0 * HL_RMAX : 0) + (N.start - cstart);
        for (int q = 0; q < ra; q++) {
            double *b1 = X + (size_t)q * cs, *b2 = b1 + n0;
            const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
            for (int e = w; e < 2 * r; e += HL_T / 32) { // s = Q0^T b1 (e < r), t = Q1^T b2
                const double *qq = e < r ? Q0 + (size_t)e * n0 : Q1 + (size_t)(e - r) * n1;
                const double *bb = e < r ? b1 : b2;
                const int len = e < r ? n0 : n1;
                double d = 0.0;
                for (int i = ln; i < len; i += 32) d += qq[i] * bb[i];
                for (int o = 16; o; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
                if (ln == 0) { if (e < r) sv[e] = d; else tv[e - r] = d; }
            }
            __syncthreads();
            for (int i = threadIdx.x; i < r; i += HL_T) { // u = K^T s - t
                double u = -tv[i];
                for (int t = 0; t < r; t++) u += Km[(size_t)i * r + t] * sv[t];
                hv[i] = u;
            }
            __syncthreads();
            if (threadIdx.x == 0) { // w = Lk^{-1} u + t
                for (int i = 0; i < r; i++) {
                    double v = hv[i];
                    for (int t = 0; t < i; t++) v -= Lk[(size_t)t * r + i] * wv[t];
                    wv[i] = v / Lk[(size_t)i * r + i];
                }
                for (int i = 0; i < r; i++) wv[i] += tv[i];
            }
            __syncthreads();
            for (int i = threadIdx.x; i < n1; i += HL_T) {
                double v = b2[i];
                for (int t = 0; t < r; t++) v -= Q1[(size_t)t * n1 + i] * wv[t];
                b2[i] = v;
            }
            __syncthreads();
        }
    }
}

// log det of every matrix: the partials in fixed order (leaves, then levels bottom-up), the
// HODLR rule |tr M| > |log det| -> -tr M (matrix.c:144-146)
__global__ void k_hodlr_final(HCtx C, int nbatch, double *result)
{
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= nbatch) return;
    const int task = C.tlist[h];
    const int st = C.status[task];
    if (st & ~0xF) { result[task] = NAN; return; }
    const double *p = C.part + (size_t)h * ((2 << C.NL) - 1);
    double s = 0.0, cc = 0.0;
    for (int l = C.NL; l >= 0; l--)
        for (int k = 0; k < (1 << l); k++) {
            const double y = p[node_id(l, k)] - cc, t = s + y;
            cc = (t - s) - y;
            s = t;
        }
    double ld = s;
    if (fabs(C.trace[task]) > fabs(ld)) ld = -C.trace[task];
    C.status[task] = ST_FACTOR;
    result[task] = ld;
}

// ---------------------------------------------------------------------------------------
// the diagonal of M alone, for the trace rule: I over the 3 x 3 window of each l
// ---------------------------------------------------------------------------------------
// grid (ceil(ldim / 128), ntask); mdiag[task dim + 2a] = EE(a, a), + 1 = MM(a, a)
__global__ void __launch_bounds__(128) k_hodlr_diag(HCtx C, int ntask, double *mdiag)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x, task = blockIdx.y;
    if (a >= C.ldim || task >= ntask) return;
    const bool m0 = C.tasks[task].m == 0;
    sd w[3][3][2];
    for (int x = 0; x < 3; x++)
        for (int y = 0; y <= x; y++) {
            sd tm{0, 0}, te{0, 0};
            if (!m0 || (x == 1 && y == 1)) hl_ipair(C, task, a + x, a + y, tm, te);
            w[x][y][0] = w[y][x][0] = tm;
            w[x][y][1] = w[y][x][1] = te;
        }
    auto Iv = [&](int p, int x, int y) { return w[x - a][y - a][p ? 0 : 1]; };
    const Task &T = C.tasks[task];
    const int i1 = a + 1;
    const size_t so = (size_t)task * (C.ldim + 2);
    sd EE, MM, EM, ME;
    elem_block<true>(T.m, i1, i1, C.Sa[so + i1], C.Sa[so + i1], C.Sb[so + i1], C.Sb[so + i1], C.uv[so + i1], C.uv[so + i1], Iv, EE,
                     MM, EM, ME);
    const double ee = sd_to_double(EE), mm = sd_to_double(MM);
    if (!isfinite(ee) || !isfinite(mm)) atomicOr(C.status + task, ST_ERR_NONFINITE);
    mdiag[(size_t)task * 2 * C.ldim + 2 * a] = ee;
    mdiag[(size_t)task * 2 * C.ldim + 2 * a + 1] = mm;
}

// ---------------------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------------------
struct HTree {
    int NL = 0;
    std::vector<HNode> nodes;
    long long qstride = 0;
};

// levels: ceil(log2(n / HL_LEAF)), at least one; children split at floor(size/2) as the
// reference does (HODLR_Node.cpp:14-17)
static HTree hodlr_tree(int n)
{
    HTree T;
    int NL = 1;
    while ((double)n / (1 << NL) > HL_LEAF) NL++;
    T.NL = NL;
    T.nodes.resize((2 << NL) - 1);
    T.nodes[0] = HNode{0, n, n / 2, 0};
    long long off = 0;
    for (int l = 0; l <= NL; l++)
        for (int k = 0; k < (1 << l); k++) {
            HNode &N = T.nodes[(1 << l) - 1 + k];
            if (l > 0) {
                const HNode &P = T.nodes[(1 << (l - 1)) - 1 + k / 2];
                N.start = (k & 1) ? P.start + P.c0 : P.start;
                N.size = (k & 1) ? P.size - P.c0 : P.c0;
            }
            N.c0 = N.size / 2;
            N.qoff = l < NL ? off : 0;
            if (l < NL) off += (long long)N.size * HL_RMAX;
        }
    T.qstride = off;
    return T;
}

// largest rank a node of level l can hold: its shorter side (its sizes differ by at most one
// from the level's first node), at most HL_RMAX
static int hl_level_rank(const HTree &T, int l)
{
    const HNode &N = T.nodes[(1 << l) - 1];
    return std::min(HL_RMAX, N.size - N.c0 + 1);
}

size_t hodlr_work_bytes(int ldim, int nbatch)
{
    const HTree T = hodlr_tree(2 * ldim);
    const int nn = (2 << T.NL) - 1;
    size_t aca = 0;
    for (int l = 0; l < T.NL; l++) {
        const HNode &N = T.nodes[(1 << l) - 1];
        aca = std::max(aca, (size_t)(1 << l) * hl_aca_scratch(N.c0 + 1, N.size - N.c0 + 1));
    }
    const size_t leaf = (size_t)(1 << T.NL) * hl_leaf_scratch();
    size_t node = 0;
    for (int l = 0; l < T.NL; l++) node = std::max(node, (size_t)(1 << l) * hl_node_scratch(hl_level_rank(T, l)));
    const size_t scratch = std::max(aca, std::max(leaf, node));
    return (size_t)nbatch * ((size_t)T.qstride * 8 + (size_t)nn * (sizeof(int) + sizeof(double)) + scratch) + nn * sizeof(HNode) + 4096;
}

int hodlr_levels(int ldim) { return hodlr_tree(2 * ldim).NL; }

static HCtx hodlr_ctx(const Task *tasks, const int *tlist, int ldim, const sd *K, int nu_stride, const double4 *ptab, int pstride,
                      const double *lft, const sd *Sa, const sd *Sb, const double2 *uv, const double *trace, int *status,
                      const HodlrMixed *mx)
{
    HCtx C{};
    if (mx) {
        C.mixed = 1;
        C.KP = mx->KP;
        C.KPe = mx->KPe;
        C.ptabf = mx->ptabf;
        C.tl = (const A12L *)mx->a12t;
        C.tj = (const A12J *)((const char *)mx->a12t + (size_t)(ldim + 2) * mx->ngroup * sizeof(A12L));
    }
    C.tasks = tasks;
    C.tlist = tlist;
    C.ldim = ldim;
    C.K = K;
    C.nu_stride = nu_stride;
    C.ptab = ptab;
    C.pstride = pstride;
    C.lft = lft;
    C.Sa = Sa;
    C.Sb = Sb;
    C.uv = uv;
    C.trace = trace;
    C.status = status;
    return C;
}

void hodlr_diag(const Task *tasks, int ntask, int ldim, const sd *K, int nu_stride, const double4 *ptab, int pstride, const double *lft,
                const sd *Sa, const sd *Sb, const double2 *uv, double *mdiag, int *status, cudaStream_t st, const HodlrMixed *mx)
{
    const HCtx C = hodlr_ctx(tasks, nullptr, ldim, K, nu_stride, ptab, pstride, lft, Sa, Sb, uv, nullptr, status, mx);
    k_hodlr_diag<<<dim3((ldim + 127) / 128, ntask), 128, 0, st>>>(C, ntask, mdiag);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

// log det(1 - M) of the listed tasks by HODLR; tasks with status bits above 0xF are skipped;
// ST_ERR_HODLR marks a matrix whose compression exceeded HL_RMAX
void hodlr_logdet_batch(const Task *tasks, const int *tlist, int nbatch, int ldim, const sd *K, int nu_stride, const double4 *ptab,
                        int pstride, const double *lft, const sd *Sa, const sd *Sb, const double2 *uv, const double *trace,
                        int *status, double *result, void *work, cudaStream_t st, const HodlrMixed *mx)
{
    if (nbatch <= 0) return;
    static bool attr = false;
    if (!attr) {
        CK(cudaFuncSetAttribute(k_hodlr_leaf, cudaFuncAttributeMaxDynamicSharedMemorySize, HL_LEAF * HL_LEAF * 8));
        attr = true;
    }
    const HTree T = hodlr_tree(2 * ldim);
    const int nn = (2 << T.NL) - 1;
    unsigned char *w = (unsigned char *)(((uintptr_t)work + 255) & ~(uintptr_t)255);
    HNode *d_nodes = (HNode *)w;
    w += (nn * sizeof(HNode) + 255) & ~(size_t)255;
    CK(cudaMemcpyAsync(d_nodes, T.nodes.data(), nn * sizeof(HNode), cudaMemcpyHostToDevice, st));
    HCtx C = hodlr_ctx(tasks, tlist, ldim, K, nu_stride, ptab, pstride, lft, Sa, Sb, uv, trace, status, mx);
    C.nodes = d_nodes;
    C.NL = T.NL;
    C.qstride = T.qstride;
    C.Q = (double *)w;
    w += (size_t)nbatch * T.qstride * 8;
    C.rank = (int *)w;
    w += ((size_t)nbatch * nn * sizeof(int) + 255) & ~(size_t)255;
    C.part = (double *)w;
    w += ((size_t)nbatch * nn * sizeof(double) + 255) & ~(size_t)255;
    unsigned char *scratch = w;
    CK(cudaMemsetAsync(C.rank, 0, (size_t)nbatch * nn * sizeof(int), st));
    CK(cudaMemsetAsync(C.part, 0, (size_t)nbatch * nn * sizeof(double), st));
    // compression of every node
    for (int l = 0; l < T.NL; l++) {
        const HNode &N = T.nodes[(1 << l) - 1];
        const size_t per = hl_aca_scratch(N.c0 + 1, N.size - N.c0 + 1);
        k_hodlr_aca<<<dim3(1 << l, nbatch), HL_T, 0, st>>>(C, l, scratch, per);
        COUNT_LAUNCH(1);
    }
    // leaves
    k_hodlr_leaf<<<dim3(1 << T.NL, nbatch), HL_T, HL_LEAF * HL_LEAF * 8, st>>>(C, scratch);
    COUNT_LAUNCH(1);
    // nodes, bottom-up
    for (int l = T.NL - 1; l >= 0; l--) {
        k_hodlr_node<<<dim3(1 << l, nbatch), HL_T, 0, st>>>(C, l, scratch, hl_node_scratch(hl_level_rank(T, l)));
        COUNT_LAUNCH(1);
    }
    k_hodlr_final<<<(nbatch + 127) / 128, 128, 0, st>>>(C, nbatch, result);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
