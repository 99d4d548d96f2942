// itab_ff.cu -- mixed-precision I q-sums, one a_q recurrence shared by every
// frequency of the same m.
//
// I_{l1 l2,p}^{(m)}(xi) = a_0 sum_q a_q K_{l1+l2-2q,p}(xi)        (integration.c:491-609)
//
// The coefficients a_q (eqs. (26)-(30) of the reference's integration.c) depend on
// (l1, l2, m) only; the frequency enters through K alone.  A thread therefore owns one
// (l1 >= l2) pair and a subgroup of up to G tasks that share m: it runs the projective
// recurrence b_q = X b_{q-1} - Y Z_{q-1} b_{q-2}, D_q = Z D_{q-1} once, forms
// a_q = b_q / D_q with one float-float division per q, and each task only accumulates
// a_q K_q for its two polarisations and applies the reference's early stop to its own terms.
// Everything is float-float (two FP32 words) with separate power-of-two exponents;
// the FP64 pipe is touched only by per-pair set-up.
//
// The early stop is the reference's rule (three consecutive terms below a threshold
// relative to the q = 0 term, integration.c:563-575) with the threshold 2^-44 (about
// e^-30.5) instead of e^-60, tested on exponents only.  The I values feed elements that
// the mixed form stores in FP32 (2^-24), so terms below 2^-44 of the q = 0 term leave 20
// bits of headroom for cancellation in the B, C, D combinations of the elements.  On
// the R/L=150 free energy the result does not move between 2^-58 and 2^-38 (|dE/E|
// 5.58e-11 throughout) while the term count falls by a quarter.
#include "common.cuh"
#include "ff.cuh"
#include "internal.h"
#include "qsum_ff.cuh"

namespace capsgpu {

// The q-sums (qsum_ff.cuh) with both polarisations of a task under one exponent frame: the paired K
// table (KP: TM h, l, TE h, l; KPe: their common exponent) lets one alignment serve both, and
// a_q is scaled into the task's frame once (an exact power of two) before the two float-float
// products.  Per task the state is the two float-float sums, the frame exponent, the two stop
// thresholds (in frame units) and the last q with a significant term.  The early stop keeps
// the reference's form (three consecutive terms below 2^-stop_bits of the q = 0 term,
// integration.c:563-575), applied to the pair of polarisations: a task stops once neither
// polarisation has had a significant term for three steps.  Each sum is a function of its own
// (pair, task) alone, so results do not depend on how tasks are grouped.
//
// grid (ceil(npair/128), ngroups); groups[g] = {first list position, count <= G, a_0..a_2 and
// p-table row}: the group's tasks are tlist[x], ..., tlist[x + count - 1] (tlist == nullptr:
// tasks x, ..., x + count - 1).  They share m (hence lmin, mu, the p table and the a_0..a_2 row)
// and the material.  Output: I tables as float-float (ffe) or, with ffe_out false, as scaled
// doubles.  The kernel is bound by FP32/ALU issue and the latency of float-float dependency
// chains, so occupancy pays (MINB blocks of 128 per SM).
template <int G, int MINB>
__global__ void __launch_bounds__(128, MINB) k_itab_pk(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim,
                                                 const float4 *__restrict__ KP, const int *__restrict__ KPe, int nu_stride,
                                                 const float4 *__restrict__ ptabf, int pstride, const A012F *__restrict__ a12,
                                                 void *Iout, bool ffe_out, int *status, int stop_bits)
{
    const int L = ldim + 2;
    const long long npair = (long long)L * (L + 1) / 2;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int gi = blockIdx.y;
    if (gi >= ngroups || tid >= npair) return;
    const long long pid = tid;
    int a1 = (int)((sqrtf(8.0f * (float)pid + 1.0f) - 1.0f) * 0.5f);
    while ((long long)(a1 + 1) * (a1 + 2) / 2 <= pid) a1++;
    while ((long long)a1 * (a1 + 1) / 2 > pid) a1--;
    const int a2 = (int)(pid - (long long)a1 * (a1 + 1) / 2);
    const int4 grp = groups[gi];
    const int ng = grp.y;
    int tk[G];
#pragma unroll
    for (int g = 0; g < G; g++) tk[g] = g < ng ? (tlist ? tlist[grp.x + g] : grp.x + g) : 0;

    const Task &T = tasks[tk[0]];
    const int l1 = T.lmin - 1 + a1, l2 = T.lmin - 1 + a2;
    const int mm = T.m > 0 ? T.m : 1;
    const size_t o12 = (size_t)a1 * L + a2, o21 = (size_t)a2 * L + a1;
    const size_t LL = (size_t)L * L;
    auto store = [&](int g, int pol, float h, float l, int e) { // pol 1 = TM, 0 = TE
        const size_t base = (size_t)(tk[g] * 2 + pol) * LL;
        if (ffe_out) {
            ffe *F = reinterpret_cast<ffe *>(Iout) + base;
            F[o12] = F[o21] = ffe{h, l, e, 0};
        } else {
            sd *D = reinterpret_cast<sd *>(Iout) + base;
            const sd v = sd_norm((double)h + (double)l, e);
            D[o12] = D[o21] = v;
        }
    };
    if (l2 < mm || l2 < T.m || l1 < 1) { // I = 0 for l < m (integration.c:631)
        for (int g = 0; g < ng; g++) { store(g, 1, 0.0f, 0.0f, FFE_ZERO_E); store(g, 0, 0.0f, 0.0f, FFE_ZERO_E); }
        return;
    }
    const unsigned bad = qsum_ff_pair<G>(T, tk, ng, l1, l2, a12[(size_t)grp.z * npair + pid], KP, KPe, nu_stride,
                                          ptabf + (size_t)grp.z * 2 * pstride * 2, pstride, stop_bits, store);
#pragma unroll
    for (int g = 0; g < G; g++)
        if (g < ng && (bad & (1u << g))) atomicOr(status + tk[g], ST_ERR_NONFINITE);
}

// tasks per subgroup.  q-sums of the R/L=150 free energy (ms), first float-float version:
// G = 3 at six blocks per SM 119.7, at five 123.8, at seven 122.3; G = 2 at seven 124.1, at
// five 136.6; G = 4 at five 134.6, at six 137.9.  With the packed stop state and the trace
// rule first (q-sum phase of the undecided matrices): G = 3 at seven 57.1, at six 59.3, at
// eight 57.7; G = 4 at six 61.0, at five 62.9; G = 2 at seven 62.0, at eight 62.3.  More
// tasks share the recurrence, but the registers cost occupancy and a subgroup runs to the
// term count of its slowest frequency.  The paired-K kernel (k_itab_pk, one frame per task):
// G = 3 at seven blocks 40.6, G = 4 at six 43.0, G = 5 at five 42.9, G = 6 at five 44.8,
// against 55.4 for the per-polarisation kernel in the same run; E identical in all five.
constexpr int IGRP = 3;
constexpr int ITAB_STOP_BITS = QSUM_FF_STOP_BITS;
int itab_group_size() { return IGRP; }

void launch_itab_grp(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim, const float4 *KP, const int *KPe,
                     int nu_stride, const float4 *ptabf, int pstride, const void *a12, void *Iout, bool ffe_out, int *status,
                     cudaStream_t st)
{
    if (ngroups <= 0) return;
    const long long L = ldim + 2, npair = L * (L + 1) / 2;
    dim3 g((unsigned)((npair + 127) / 128), ngroups);
    k_itab_pk<IGRP, 7><<<g, 128, 0, st>>>(tasks, tlist, groups, ngroups, (int)ldim, KP, KPe, nu_stride, ptabf, pstride,
                                          (const A012F *)a12, Iout, ffe_out, status, ITAB_STOP_BITS);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
