// elem_ff.cu -- mixed-precision assembly of 1 - M(xi, m).
//
// The mixed form factorises A = 1 - M in FP32 delta form (A - I = -M, see mixed.cu),
// so an element only has to reach FP32 accuracy once it is assembled; what it must
// survive on the way is the cancellation inside the B, C, D combinations (up to ~1e5
// for m = 0).  The combinations are therefore formed in float-float with a separate
// power-of-two exponent ("fe" below, ~48-bit mantissa) from the float-float I table
// that k_itab_pk writes, and the result goes straight into the FP32 delta matrix:
// no FP64 matrix is formed, and the FP64 pipe is used only for the diagonal, which
// the logdet correction needs in FP64.  Per element block the kernel also leaves a
// per-warp sum of squares, from which k_stats_ff takes the Frobenius norm for the
// reference's trace / Mercator shortcuts.
//
// Formulas: elements as in libcaps.c:717-831 (caps_M_elem / caps_kernel_M) with A, B,
// C, D from integration.c:762-888; shortcut decision as in matrix.c:57-119
// (kernel_logdet) and matrix.c:489-505 (Mercator bound).
#include "common.cuh"
#include "ff.cuh"
#include "internal.h"

namespace capsgpu {

constexpr int EB = 128; // threads per element block (one 2x2 block of M each)

// (h + l) 2^e.  Table values (I, scale factors) arrive with |h| in [1,2); products and
// combinations are left unnormalised -- a product of three such mantissas stays below 8,
// a combination of a few terms with float-float coefficients below 2^30 -- and only the
// final conversion to FP32 / FP64 applies the exponent, so no renormalisation is spent in
// between (float-float precision does not depend on the binary scale).
struct fe { float h, l; int e; };

CAPS_DEV fe fe_ld(const ffe &v) { return fe{v.h, v.l, v.e}; }
CAPS_DEV fe fe_neg(fe a) { return fe{-a.h, -a.l, a.e}; }
CAPS_DEV fe fe_mul(fe a, fe b)
{
    const ff p = ff_mul(ff{a.h, a.l}, ff{b.h, b.l});
    return fe{p.h, p.l, a.e + b.e};
}
// sum_k c_k x_k for float-float coefficients c_k and table values x_k (|h| in [1,2), zeros
// with exponent FFE_ZERO_E): every x_k is rescaled to the largest exponent among them by one
// exact multiply with 2^d, d <= 0 (terms more than 2^126 below it, zeros among them, scale
// to 0), then float-float products and sums
template <int N>
CAPS_DEV fe fe_lincomb(const ff (&c)[N], const fe (&x)[N])
{
    int emax = x[0].e;
#pragma unroll
    for (int k = 1; k < N; k++) emax = max(emax, x[k].e);
    ff s{0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < N; k++) {
        const int d = x[k].e - emax;
        const float p2 = __uint_as_float((unsigned)max(127 + d, 0) << 23);
        s = ff_add(s, ff_mul(c[k], ff{x[k].h * p2, x[k].l * p2}));
    }
    return fe{s.h, s.l, emax};
}

// to FP32: values below 2^-120 flush to 0 (as do subnormal mantissas left by cancellation);
// non-finite or >= 2^126 set *bad
CAPS_DEV float fe_to_float(fe a, bool &bad)
{
    const int k = fexpo(a.h);
    if (k == -127) return 0.0f;
    if (k == 128 || a.e + k > 125) { bad = true; return a.h; }
    if (a.e + k < -120) return 0.0f;
    return fshift(a.h + a.l, a.e);
}
CAPS_DEV double fe_to_double(fe a)
{
    if (a.h == 0.0f) return 0.0;
    return shift2((double)a.h + (double)a.l, a.e);
}

// float-float copies of the per-l scale factors and u, v coefficients (k_scale)
__global__ void k_scale_ff(int ntask, int L, const sd *Sa, const sd *Sb, const double2 *uv, ffe *Saf, ffe *Sbf, float4 *uvf)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    const int task = blockIdx.y;
    if (a >= L || task >= ntask) return;
    const size_t o = (size_t)task * L + a;
    const sd sa = Sa[o], sb = Sb[o];
    const ff fa = ff_from_d(sa.m), fb = ff_from_d(sb.m);
    Saf[o] = ffe{fa.h, fa.l, sa.e, 0};
    Sbf[o] = ffe{fb.h, fb.l, sb.e, 0};
    const double2 w = uv[o];
    const ff u = ff_from_d(w.x), v = ff_from_d(w.y);
    uvf[o] = make_float4(u.h, u.l, v.h, v.l);
}

// EE and MM (with OFFD also EM and ME) of the 2x2 block of M at rows lmin + i1 - 1 and
// columns lmin + i2 - 1 (i1, i2 index [lmin-1, lmin+ldim]); each is one linear combination
// of I values times the scale factors.  One routine for the full assembly and for the
// diagonal that the trace shortcut reads, so that both give the same numbers.
// Iv(pol, x, y) returns I of polarisation pol (1 = TM, 0 = TE) at window indices (x, y).
template <bool OFFD, class IV>
CAPS_DEV void elem_block(const Task &T, int i1, int i2, size_t so, const ffe *__restrict__ Saf, const ffe *__restrict__ Sbf,
                         const float4 *__restrict__ uvf, IV Iv, fe &EE, fe &MM, fe &EM, fe &ME)
{
    const fe sa1 = fe_ld(Saf[so + i1]), sa2 = fe_ld(Saf[so + i2]);
    const fe sb1 = fe_ld(Sbf[so + i1]), sb2 = fe_ld(Sbf[so + i2]);
    const int ITM = 1, ITE = 0;
    EM = fe{0.0f, 0.0f, 0};
    ME = fe{0.0f, 0.0f, 0};
    if (T.m == 0) {
        EE = fe_mul(fe_mul(sa1, sa2), Iv(ITM, i1, i2));          // B_TM, A = 0
        MM = fe_neg(fe_mul(fe_mul(sb1, sb2), Iv(ITE, i1, i2)));  // -B_TE
        return;
    }
    const float mf = (float)T.m, m2h = mf * mf;
    const ff m1{mf, 0.0f}, m2{m2h, fmaf(mf, mf, -m2h)};
    const float4 w1 = uvf[so + i1], w2 = uvf[so + i2];
    const ff U1{w1.x, w1.y}, V1{w1.z, w1.w}, U2{w2.x, w2.y}, V2{w2.z, w2.w};
    const ff cUU = ff_mul(U1, U2), cVU = ff_mul(V1, U2), cUV = ff_mul(U1, V2), cVV = ff_mul(V1, V2);
    // B_p = u1 u2 I(l1-1,l2-1) - v1 u2 I(l1+1,l2-1) - u1 v2 I(l1-1,l2+1) + v1 v2 I(l1+1,l2+1)
    // C_p(l1,l2) = m (v2 I(l1,l2+1) - u2 I(l1,l2-1)); D_p(l1,l2) = C_p(l2,l1)
    // EE = B_TM - m^2 I_TE,  MM = m^2 I_TM - B_TE,  EM = D_TM - C_TE,  ME = C_TM - D_TE
    // (times the scale factors), each one linear combination of the I values
    {
        const ff c[5] = {cUU, ff_neg(cVU), ff_neg(cUV), cVV, ff_neg(m2)};
        const fe x[5] = {Iv(ITM, i1 - 1, i2 - 1), Iv(ITM, i1 + 1, i2 - 1), Iv(ITM, i1 - 1, i2 + 1), Iv(ITM, i1 + 1, i2 + 1),
                         Iv(ITE, i1, i2)};
        EE = fe_mul(fe_mul(sa1, sa2), fe_lincomb(c, x));
    }
    {
        const ff c[5] = {m2, ff_neg(cUU), cVU, cUV, ff_neg(cVV)};
        const fe x[5] = {Iv(ITM, i1, i2), Iv(ITE, i1 - 1, i2 - 1), Iv(ITE, i1 + 1, i2 - 1), Iv(ITE, i1 - 1, i2 + 1),
                         Iv(ITE, i1 + 1, i2 + 1)};
        MM = fe_mul(fe_mul(sb1, sb2), fe_lincomb(c, x));
    }
    if (!OFFD) return;
    const ff mU1 = ff_mul(m1, U1), mV1 = ff_mul(m1, V1), mU2 = ff_mul(m1, U2), mV2 = ff_mul(m1, V2);
    {
        const ff c[4] = {mV1, ff_neg(mU1), ff_neg(mV2), mU2};
        const fe x[4] = {Iv(ITM, i1 + 1, i2), Iv(ITM, i1 - 1, i2), Iv(ITE, i1, i2 + 1), Iv(ITE, i1, i2 - 1)};
        EM = fe_mul(fe_mul(sa1, sb2), fe_lincomb(c, x));
    }
    {
        const ff c[4] = {mV2, ff_neg(mU2), ff_neg(mV1), mU1};
        const fe x[4] = {Iv(ITM, i1, i2 + 1), Iv(ITM, i1, i2 - 1), Iv(ITE, i1 + 1, i2), Iv(ITE, i1 - 1, i2)};
        ME = fe_mul(fe_mul(sb1, sa2), fe_lincomb(c, x));
    }
}

// grid (ceil(ldim/EB), ldim, nlist); block z handles task tlist[z] (tlist == nullptr: task
// z); thread (a, b) with a >= b owns rows 2a, 2a+1 and
// columns 2b, 2b+1 of M.  S receives -M (the delta form of A = 1 - M), lower triangle,
// column-major with leading dimension n; diag receives M_ii in FP64; part
// receives, per warp, the sum of squares of M over the warp's blocks (strict lower
// entries twice).  Blocks entirely above the diagonal exit before doing anything.
__global__ void __launch_bounds__(EB) k_elem_ff(const Task *tasks, const int *tlist, int nlist, int ldim, const ffe *__restrict__ I,
                                                const ffe *__restrict__ Saf, const ffe *__restrict__ Sbf,
                                                const float4 *__restrict__ uvf, float *S, size_t sstride, double *diag,
                                                float *part, int *status)
{
    const int L = ldim + 2, n = 2 * ldim;
    const int b = blockIdx.y;
    if ((int)blockIdx.z >= nlist || (int)blockIdx.x < b / EB) return; // uniform per block
    const int task = tlist ? tlist[blockIdx.z] : (int)blockIdx.z;
    const int a = blockIdx.x * EB + threadIdx.x;
    const bool valid = a < ldim && b <= a;
    float wsum = 0.0f;
    if (valid) {
        const Task &T = tasks[task];
        // the table is symmetric; I(x, y) is read at t[y L + x] so that consecutive
        // threads (consecutive x) read consecutive entries
        const ffe *It = I + (size_t)task * 2 * L * L;
        auto Iv = [&](int p, int x, int y) { return fe_ld(It[(size_t)p * L * L + (size_t)y * L + x]); };
        fe EE, MM, EM, ME;
        elem_block<true>(T, a + 1, b + 1, (size_t)task * L, Saf, Sbf, uvf, Iv, EE, MM, EM, ME);
        bool bad = false;
        const float ee = fe_to_float(EE, bad), mm = fe_to_float(MM, bad);
        const float em = fe_to_float(EM, bad), me = fe_to_float(ME, bad);
        if (bad) atomicOr(status + task, ST_ERR_NONFINITE);
        float *Sm = S + (size_t)task * sstride;
        const int r0 = 2 * a, c0 = 2 * b;
        Sm[(size_t)c0 * n + r0] = -ee;
        Sm[(size_t)c0 * n + r0 + 1] = -me;
        Sm[(size_t)(c0 + 1) * n + r0 + 1] = -mm;
        if (a != b) {
            Sm[(size_t)(c0 + 1) * n + r0] = -em;
            wsum = 2.0f * (ee * ee + me * me + mm * mm + em * em);
        } else {
            diag[(size_t)task * n + r0] = fe_to_double(EE);
            diag[(size_t)task * n + r0 + 1] = fe_to_double(MM);
            wsum = ee * ee + mm * mm + 2.0f * me * me;
        }
    }
    for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
    if ((threadIdx.x & 31) == 0)
        part[(((size_t)task * ldim + b) * gridDim.x + blockIdx.x) * (EB / 32) + threadIdx.x / 32] = wsum;
}

// the diagonal of M alone (kernel_logdet computes it first, matrix.c:62-66): grid
// (ceil(ldim/EB), ntask), thread a writes M_ii of the diagonal block (a, a) in FP64, from
// the band seeds (pairs l1 - l2 in {0, 2}, sweep.cu's k_seed_ff)
__global__ void __launch_bounds__(EB) k_diag_ff(const Task *tasks, int ntask, int ldim, const ffe *__restrict__ seed,
                                                const ffe *__restrict__ Saf, const ffe *__restrict__ Sbf,
                                                const float4 *__restrict__ uvf, double *diag, int *status)
{
    const int L = ldim + 2, n = 2 * ldim;
    const int task = blockIdx.y;
    const int a = blockIdx.x * EB + threadIdx.x;
    if (task >= ntask || a >= ldim) return;
    const Task &T = tasks[task];
    // the diagonal block reads I at |x - y| in {0, 2} only
    auto Iv = [&](int p, int x, int y) {
        const int kind = x == y ? SEED_D0 : SEED_D2;
        return fe_ld(seed[((size_t)(task * 2 + p) * SEED_KINDS + kind) * L + min(x, y)]);
    };
    fe EE, MM, EM, ME;
    elem_block<false>(T, a + 1, a + 1, (size_t)task * L, Saf, Sbf, uvf, Iv, EE, MM, EM, ME);
    bool bad = false;
    fe_to_float(EE, bad);
    fe_to_float(MM, bad);
    if (bad) atomicOr(status + task, ST_ERR_NONFINITE);
    diag[(size_t)task * n + 2 * a] = fe_to_double(EE);
    diag[(size_t)task * n + 2 * a + 1] = fe_to_double(MM);
}

// per task (tlist[blockIdx.x], or blockIdx.x without a list): Kahan trace of M over its
// FP64 diagonal (index order, misc.c:26), the Frobenius norm from the element partials
// (fixed order), and the reference's shortcut decision: |tr| < 1e-8 -> -tr; dense modes:
// Mercator when its error bound is below 1e-8 relative; otherwise factorise.  Without
// partials (part == nullptr) only the trace rule is applied: a matrix it does not decide
// keeps status 0, to be assembled in full.
__global__ void k_stats_ff(const int *tlist, int nlist, int ldim, const double *diag, const float *part, int nbx, int mode,
                           double *trace_out, double *result, int *status)
{
    if ((int)blockIdx.x >= nlist) return;
    const int task = tlist ? tlist[blockIdx.x] : (int)blockIdx.x;
    const int n = 2 * ldim, per_b = nbx * (EB / 32);
    __shared__ double red[256];
    if (part && nbx == 0) { // one sum per task (k_sweep_ff)
        if (threadIdx.x == 0) red[0] = (double)part[task];
        __syncthreads();
    } else if (part) {
        const float *p = part + (size_t)task * ldim * per_b;
        double s = 0.0;
        for (int i = threadIdx.x; i < ldim * per_b; i += blockDim.x) {
            const int b = i / per_b, x = (i % per_b) / (EB / 32);
            if (x >= b / EB) s += p[i];
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int w = blockDim.x / 2; w > 0; w >>= 1) {
            if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
    }
    if (threadIdx.x >= 32) return;
    // Kahan trace (misc.c:26) over the diagonal, split across the 32 lanes of warp 0: lane l
    // sums the l-th contiguous chunk, lane 0 then adds the 32 compensated partials in order
    const double *dg = diag + (size_t)task * n;
    const int lane = threadIdx.x, per = (n + 31) / 32;
    double tr = 0.0, c = 0.0;
    for (int i = lane * per; i < min(n, (lane + 1) * per); i++) {
        const double y = dg[i] - c;
        const double t = tr + y;
        c = (t - tr) - y;
        tr = t;
    }
    const double partial = tr - c;
    tr = 0.0;
    c = 0.0;
    for (int l = 0; l < 32; l++) {
        const double y = __shfl_sync(0xffffffffu, partial, l) - c;
        const double t = tr + y;
        c = (t - tr) - y;
        tr = t;
    }
    if (lane != 0) return;
    trace_out[task] = tr;
    if (status[task] & ~0xF) { result[task] = NAN; return; }
    if (fabs(tr) < 1e-8) { result[task] = -tr; status[task] = ST_TRACE; return; }
    if (!part) return;
    const double fro2 = red[0], fro = sqrt(fro2);
    if (mode == 0 && fro < 1) {
        const double merc = -tr - fro2 / 2;
        const double err = fabs(fro2 / 2 + fro + log1p(-fro));
        if (fabs(err / merc) < 1e-8) { result[task] = merc; status[task] = ST_MERCATOR; return; }
    }
    status[task] = ST_FACTOR;
}

size_t elem_ff_part_floats(int ldim) { return (size_t)ldim * ((ldim + EB - 1) / EB) * (EB / 32); }

void launch_scale_ff(int ntask, int ldim, const sd *Sa, const sd *Sb, const double2 *uv, void *Saf, void *Sbf, float4 *uvf,
                     cudaStream_t st)
{
    const int L = ldim + 2;
    dim3 gs((L + 127) / 128, ntask);
    k_scale_ff<<<gs, 128, 0, st>>>(ntask, L, Sa, Sb, uv, (ffe *)Saf, (ffe *)Sbf, uvf);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_diag_ff(const Task *tasks, int ntask, int ldim, const void *seed, const void *Saf, const void *Sbf, const float4 *uvf,
                    double *diag, int *status, cudaStream_t st)
{
    dim3 g((ldim + EB - 1) / EB, ntask);
    k_diag_ff<<<g, EB, 0, st>>>(tasks, ntask, ldim, (const ffe *)seed, (const ffe *)Saf, (const ffe *)Sbf, uvf, diag, status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_elem_ff(const Task *tasks, const int *tlist, int nlist, int ldim, const void *Saf, const void *Sbf, const float4 *uvf,
                    const void *I, float *S, size_t sstride, double *diag, float *part, int *status, cudaStream_t st)
{
    if (nlist <= 0) return;
    dim3 g((ldim + EB - 1) / EB, ldim, nlist);
    k_elem_ff<<<g, EB, 0, st>>>(tasks, tlist, nlist, ldim, (const ffe *)I, (const ffe *)Saf, (const ffe *)Sbf, uvf, S, sstride,
                                diag, part, status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_stats_ff(const int *tlist, int nlist, int ldim, const double *diag, const float *part, int mode, double *trace,
                     double *result, int *status, cudaStream_t st, bool part_per_task)
{
    if (nlist <= 0) return;
    k_stats_ff<<<nlist, 256, 0, st>>>(tlist, nlist, ldim, diag, part, part_per_task ? 0 : (ldim + EB - 1) / EB, mode, trace, result,
                                      status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
