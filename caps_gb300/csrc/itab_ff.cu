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

namespace capsgpu {

// float-float quotient x / y (Dekker 1971: one correction of the leading quotient).  The
// reciprocal is the hardware approximation (relative error ~2^-23): the correction
// q2 = (x - q1 y) r then leaves a relative error ~2^-45, below the 2^-44 the q-sums keep.
CAPS_DEV ff ff_div(ff x, ff y)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y.h));
    const float q1 = x.h * r;
    const ff p = ff_mul(ff{q1, 0.0f}, y);
    const ff rem = ff_add(x, ff_neg(p));
    return ff_fast2(q1, rem.h * r);
}

// The q-sums with both polarisations of a task under one exponent frame: the paired K
// table (KP: TM h, l, TE h, l; KPe: their common exponent) lets one alignment serve both, and
// a_q is scaled into the task's frame once (an exact power of two) before the two float-float
// products.  Per task the state is the two float-float sums, the frame exponent, the two stop
// thresholds (in frame units) and the last q with a significant term.  The early stop keeps
// the reference's form (three consecutive terms below 2^-stop_bits of the q = 0 term,
// integration.c:563-575), applied to the pair of polarisations: a task stops once neither
// polarisation has had a significant term for three steps.  Each sum is a function of its own
// (pair, task) alone, so results do not depend on how tasks are grouped.
//
// grid (ceil(npair/128), ngroups) or, for the band, (ceil(2L/128), ngroups);
// groups[g] = {first list position, count <= G, a_0..a_2 and p-table row}: the group's tasks are
// tlist[x], ..., tlist[x + count - 1] (tlist == nullptr: tasks x, ..., x + count - 1).
// They share m (hence lmin, mu, the p table and the a_0..a_2 row) and the material.
// BAND computes only the pairs that the diagonal of M reads, l1 - l2 in {0, 2} (the EE and
// MM entries of a diagonal 2x2 block, integration.c:762-888); each pair's sum is the one
// the full kernel forms.  Output: I tables as float-float (ffe) or, with ffe_out false, as
// scaled doubles.  The kernel is bound by FP32/ALU issue and the latency of float-float
// dependency chains, so occupancy pays (MINB blocks of 128 per SM).
struct PAcc {
    float th, tl, eh, el; // TM and TE sums, (h + l) 2^e
    int e;
    int thr_t, thr_e;     // exponent (frame units) below which a term is insignificant
    int last;             // last q with a significant term (2 before the loop: q = 3, 4, 5 may stop it)
};

template <int G, bool BAND, int MINB>
__global__ void __launch_bounds__(128, MINB) k_itab_pk(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim,
                                                 const float4 *__restrict__ KP, const int *__restrict__ KPe, int nu_stride,
                                                 const float4 *__restrict__ ptabf, int pstride, const A012F *__restrict__ a12,
                                                 void *Iout, bool ffe_out, int *status, int stop_bits)
{
    const int L = ldim + 2;
    const long long npair = (long long)L * (L + 1) / 2;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int gi = blockIdx.y;
    if (gi >= ngroups) return;
    long long pid;
    int a1, a2;
    if (BAND) {
        if (tid >= 2LL * L) return;
        a2 = (int)(tid >> 1);
        a1 = a2 + 2 * (int)(tid & 1);
        if (a1 >= L) return;
        pid = (long long)a1 * (a1 + 1) / 2 + a2;
    } else {
        if (tid >= npair) return;
        pid = tid;
        a1 = (int)((sqrtf(8.0f * (float)pid + 1.0f) - 1.0f) * 0.5f);
        while ((long long)(a1 + 1) * (a1 + 2) / 2 <= pid) a1++;
        while ((long long)a1 * (a1 + 1) / 2 > pid) a1--;
        a2 = (int)(pid - (long long)a1 * (a1 + 1) / 2);
    }
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
    const bool both = !T.is_pr;
    const int l12 = l1 + l2;
    const int qmax = min(min(l1, l2), (l12 - 2 * mm) / 2);
    const A012F A12 = a12[(size_t)grp.z * npair + pid];
    const ff a1f{A12.a1h, A12.a1l}, a2f{A12.a2h, A12.a2l};
    const int koff = -T.mu;

    // add c K(nu) (c in frame units of exponent ec) to task g's sums; true if significant
    auto add = [&](PAcc &A, int g, ff c, int ec, int nu) {
        const size_t k = (size_t)tk[g] * nu_stride + (nu + koff);
        const float4 kv = KP[k];
        int d = ec + KPe[k] - A.e;
        if (d > 30) { // a term far above the frame: move the frame up (exact shifts)
            A.th = fshift(A.th, -d); A.tl = fshift(A.tl, -d); A.eh = fshift(A.eh, -d); A.el = fshift(A.el, -d);
            A.thr_t -= d; A.thr_e -= d; A.e += d; d = 0;
        }
        const float p2 = __uint_as_float((unsigned)max(127 + d, 0) << 23);
        const ff cs{c.h * p2, c.l * p2};
        const ff tT = ff_mul(cs, ff{kv.x, kv.y});
        const ff sT = ff_add(ff{A.th, A.tl}, tT);
        A.th = sT.h; A.tl = sT.l;
        bool sig = fexpo(tT.h) >= A.thr_t;
        if (both) {
            const ff tE = ff_mul(cs, ff{kv.z, kv.w});
            const ff sE = ff_add(ff{A.eh, A.el}, tE);
            A.eh = sE.h; A.el = sE.l;
            sig |= fexpo(tE.h) >= A.thr_e;
        }
        return sig;
    };

    PAcc acc[G];
#pragma unroll
    for (int g = 0; g < G; g++) {
        PAcc &A = acc[g];
        A = PAcc{0.0f, 0.0f, 0.0f, 0.0f, 0, 0, 0, -(1 << 30)};
        if (g >= ng) continue;
        const size_t k = (size_t)tk[g] * nu_stride + (l12 + koff);
        const float4 k0 = KP[k];
        A.th = k0.x; A.tl = k0.y; A.eh = k0.z; A.el = k0.w; A.e = KPe[k];
        A.thr_t = fexpo(k0.x) - stop_bits;
        A.thr_e = fexpo(k0.z) - stop_bits;
        A.last = 2;
        if (qmax >= 1) add(A, g, a1f, 0, l12 - 2);
        if (qmax >= 2) add(A, g, a2f, 0, l12 - 4);
    }

    if (qmax >= 3) {
        const long long Si = l1 + l2 + 1, Di = l1 - l2;
        int ip = l12 - 6; // p of q = 3
        const long long n1st = ((long long)(ip + 1 - Si) * (ip + 1 + Si)) * ((long long)(ip + 1 - Di) * (ip + 1 + Di));
        const int sig = (n1st == 0 ? 0 : (63 - __clzll(n1st < 0 ? -n1st : n1st))) - 20;
        const int sa = sig / 2, sc = sig - sa;
        const float fS = (float)Si, fD = (float)Di;
        const float sA = __uint_as_float((unsigned)(127 - sa) << 23), sC = __uint_as_float((unsigned)(127 - sc) << 23);
        auto Nf = [&](float x) {
            const float p1 = x - fS, p2 = x + fS, q1 = x - fD, q2 = x + fD;
            const float ah = p1 * p2, ch = q1 * q2;
            const ff av{ah * sA, fmaf(p1, p2, -ah) * sA}, cv{ch * sC, fmaf(q1, q2, -ch) * sC};
            return ff_mul(av, cv);
        };
        const bool diag = (l1 == l2);
        const float m2f = 2.0f * mm, dlf = (float)(l1 - l2), pA = m2f * dlf;
        const ff ApF = ff_mul(ff{pA, fmaf(m2f, dlf, -pA)}, ff{(float)(l1 + l2 + 1), 0.0f});
        const ff Ap2 = diag ? ff{0.0f, 0.0f} : ff_shift(ff_mul(ApF, ApF), -30 - sig);
        const float4 *pt = ptabf + ((size_t)grp.z * 2 + (diag ? 1 : 0)) * pstride * 2;
        const int e_b = fexpo(A12.a2h);
        ff bm2 = ff_shift(a1f, -e_b), bm1 = ff_shift(a2f, -e_b);
        int eb = e_b, eD = 0;
        ff Dq{1.0f, 0.0f}, Zprev{1.0f, 0.0f};
        float fx = (float)(ip + 1);
        ff N3 = Nf(fx + 2.0f), N4 = Nf(fx + 3.0f);
        bool any = true;
        for (int q = 3; q <= qmax && any; q++, ip -= 2, fx -= 2.0f) {
            const ff N1 = Nf(fx), N2 = Nf(fx + 1.0f);
            const float4 kh = pt[2 * ip], kl = pt[2 * ip + 1];
            const ff X = ff_add(Ap2, ff_add(ff_mul(ff{kh.y, kl.y}, N2), ff_mul(ff{kh.z, kl.z}, N3)));
            const ff Y = ff_mul(ff{kh.w, kl.w}, N4);
            const ff Z = ff_mul(ff{kh.x, kl.x}, N1);
            const ff b = ff_add(ff_mul(X, bm1), ff_neg(ff_mul(ff_mul(Y, Zprev), bm2)));
            Dq = ff_mul(Dq, Z);
            N3 = N1; N4 = N2; Zprev = Z;
            bm2 = bm1; bm1 = b;
            {
                const int kb = fexpo(bm1.h);
                if (kb > 40 || (kb < -40 && kb > -127)) { bm1 = ff_shift(bm1, -kb); bm2 = ff_shift(bm2, -kb); eb += kb; }
                const int kd = fexpo(Dq.h);
                if (kd > 40 || kd < -40) { Dq = ff_shift(Dq, -kd); eD += kd; }
            }
            const ff aq = ff_div(bm1, Dq);
            const int ea = eb - eD;
            any = false;
#pragma unroll
            for (int g = 0; g < G; g++) {
                PAcc &A = acc[g];
                if (q - A.last > 3) continue; // stopped (never true for g >= ng: last = -2^30)
                if (add(A, g, aq, ea, ip)) A.last = q;
                any |= q + 1 - A.last <= 3;
            }
        }
    }

    // I = a_0 sum; TE of a perfect reflector is -TM
    const ff a0f{A12.a0h, A12.a0l};
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (g >= ng) break;
        const PAcc &A = acc[g];
        ff r = ff_mul(a0f, ff{A.th, A.tl});
        int k = fexpo(r.h);
        if (k == -127 || k == 128) atomicOr(status + tk[g], ST_ERR_NONFINITE);
        if (k == 128 || k == -127) k = 0;
        r = ff_shift(r, -k);
        const int eT = r.h == 0.0f ? FFE_ZERO_E : A.e + A12.a0e + k;
        store(g, 1, r.h, r.l, eT);
        if (both) {
            ff s = ff_mul(a0f, ff{A.eh, A.el});
            int ke = fexpo(s.h);
            if (ke == 128 || ke == -127) ke = 0;
            s = ff_shift(s, -ke);
            store(g, 0, s.h, s.l, s.h == 0.0f ? FFE_ZERO_E : A.e + A12.a0e + ke);
        } else
            store(g, 0, -r.h, -r.l, eT);
    }
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
constexpr int ITAB_STOP_BITS = 44; // early stop below 2^-44 of the q = 0 term
int itab_group_size() { return IGRP; }

void launch_itab_grp(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim, const float4 *KP, const int *KPe,
                     int nu_stride, const float4 *ptabf, int pstride, const void *a12, void *Iout, bool ffe_out, bool band,
                     int *status, cudaStream_t st)
{
    if (ngroups <= 0) return;
    const long long L = ldim + 2, npair = L * (L + 1) / 2;
    dim3 g((unsigned)(((band ? 2 * L : npair) + 127) / 128), ngroups);
    const A012F *A = (const A012F *)a12;
    if (band)
        k_itab_pk<IGRP, true, 7><<<g, 128, 0, st>>>(tasks, tlist, groups, ngroups, (int)ldim, KP, KPe, nu_stride, ptabf, pstride, A,
                                                    Iout, ffe_out, status, ITAB_STOP_BITS);
    else
        k_itab_pk<IGRP, false, 7><<<g, 128, 0, st>>>(tasks, tlist, groups, ngroups, (int)ldim, KP, KPe, nu_stride, ptabf, pstride, A,
                                                     Iout, ffe_out, status, ITAB_STOP_BITS);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
