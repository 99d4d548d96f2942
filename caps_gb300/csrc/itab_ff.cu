// itab_ff.cu -- mixed-precision I q-sums, one a_q recurrence shared by every
// frequency of the same m.
//
// I_{l1 l2,p}^{(m)}(xi) = a_0 sum_q a_q K_{l1+l2-2q,p}(xi)        (integration.c:491-609)
//
// The coefficients a_q (eqs. (26)-(30) of the reference's integration.c) depend on
// (l1, l2, m) only; the frequency enters through K alone.  A thread therefore owns one
// (l1 >= l2) pair and a subgroup of up to G tasks that share m: it runs the projective
// recurrence b_q = X b_{q-1} - Y Z_{q-1} b_{q-2}, D_q = Z D_{q-1} once, forms
// a_q = b_q / D_q with one float-float division per q, and each task and polarisation
// only accumulates a_q K_q and applies the reference's early stop to its own terms.
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

struct IAcc {
    float h, l; // running sum (h + l) 2^e
    int e;
    int st; // 8 thr + 2 count + on: a term t stops counting as significant once exponent(t) < thr;
            // count = consecutive such terms, on = still summing
};

// sum += t 2^et.  The sum's exponent frame moves up (an exact power-of-two shift of the
// sum) only when a term lies more than 2^30 above it; otherwise the term is aligned to the
// frame by one exact multiply.  No renormalisation is needed for range: a term adds at most
// ~2^32 in frame units, so |h| stays below 2^32 times the number of terms, far inside float
// range, and float-float precision does not depend on the binary scale.  A zero term adds
// zero; a zero sum takes the term at the frame's exponent.
CAPS_DEV void iacc_add(IAcc &A, ff t, int et)
{
    int d = et - A.e;
    if (d > 30) {
        const ff s = ff_shift(ff{A.h, A.l}, -d);
        A.h = s.h; A.l = s.l; A.e = et; d = 0;
    }
    // 2^d for -126 <= d <= 30 is a normal float: the alignment is one exact multiply; below,
    // where the term lies more than 2^126 under the sum's frame, p2 = 0 drops it
    const float p2 = __uint_as_float((unsigned)max(127 + d, 0) << 23);
    const ff s = ff_add(ff{A.h, A.l}, ff{t.h * p2, t.l * p2});
    A.h = s.h; A.l = s.l;
}

// grid (ceil(npair/128), ngroups) or, for the band, (ceil(2L/128), ngroups);
// groups[g] = {first list position, count <= G, a_0..a_2 and p-table row}: the group's tasks are
// tlist[x], ..., tlist[x + count - 1] (tlist == nullptr: tasks x, ..., x + count - 1).
// They share m (hence lmin, mu, the p table and the a_0..a_2 row) and the material.
// BAND computes only the pairs that the diagonal of M reads, l1 - l2 in {0, 2} (the EE and
// MM entries of a diagonal 2x2 block, integration.c:762-888); each pair's sum is the one
// the full kernel forms.  Output: I tables as float-float (ffe) or, with ffe_out false, as
// scaled doubles.  The kernel is bound by FP32/ALU issue and the latency of float-float
// dependency chains, so occupancy pays: at G = 3, seven blocks of 128 per SM (72 registers;
// the stop state of an accumulator packed into one register).
template <int G, bool BAND>
__global__ void __launch_bounds__(128, 7) k_itab_grp(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim,
                                                  const ffe *__restrict__ KF, int nu_stride, const float4 *__restrict__ ptabf,
                                                  int pstride, const A012F *__restrict__ a12, void *Iout, bool ffe_out,
                                                  int *status, int stop_bits)
{
    const int L = ldim + 2;
    const long long npair = (long long)L * (L + 1) / 2;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int gi = blockIdx.y;
    if (gi >= ngroups) return;
    long long pid;
    int a1, a2;
    if (BAND) {
        // thread 2 a2 + d owns the pair (a2 + 2 d, a2)
        if (tid >= 2LL * L) return;
        a2 = (int)(tid >> 1);
        a1 = a2 + 2 * (int)(tid & 1);
        if (a1 >= L) return;
        pid = (long long)a1 * (a1 + 1) / 2 + a2;
    } else {
        if (tid >= npair) return;
        pid = tid;
        // pair index -> (a1 >= a2); the float root is exact to +-1 and corrected in integers
        a1 = (int)((sqrtf(8.0f * (float)pid + 1.0f) - 1.0f) * 0.5f);
        while ((long long)(a1 + 1) * (a1 + 2) / 2 <= pid) a1++;
        while ((long long)a1 * (a1 + 1) / 2 > pid) a1--;
        a2 = (int)(pid - (long long)a1 * (a1 + 1) / 2);
    }
    const int4 grp = groups[gi];
    const int ng = grp.y;
    int tk[G]; // task index of each member
#pragma unroll
    for (int g = 0; g < G; g++) tk[g] = g < ng ? (tlist ? tlist[grp.x + g] : grp.x + g) : 0;
    const int t0 = tk[0];

    const Task &T = tasks[t0];
    const int l1 = T.lmin - 1 + a1, l2 = T.lmin - 1 + a2;
    const int mm = T.m > 0 ? T.m : 1;
    const size_t o12 = (size_t)a1 * L + a2, o21 = (size_t)a2 * L + a1;
    const size_t LL = (size_t)L * L;
    auto store = [&](int g, int pol, float h, float l, int e) { // pol 1 = TM, 0 = TE (table order of K and I)
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

    // accumulators: j = 2 g + (0: TM, 1: TE); K table of task t, polarisation p at
    // KF[(t*2 + p) nu_stride - mu + nu] with p = 1 for TM
    IAcc acc[2 * G];
    auto Kat = [&](int j, int nu) { return KF[(size_t)(tk[j >> 1] * 2 + ((j & 1) ? 0 : 1)) * nu_stride + (nu - T.mu)]; };
#pragma unroll
    for (int j = 0; j < 2 * G; j++) {
        const bool live = (j >> 1) < ng && ((j & 1) == 0 || both);
        IAcc &A = acc[j];
        A = IAcc{0.0f, 0.0f, 0, 0};
        if (!live) continue;
        const ffe k0 = Kat(j, l12);
        A.h = k0.h; A.l = k0.l; A.e = k0.e; A.st = (fexpo(k0.h) + k0.e - stop_bits) * 8 + 1;
        if (qmax >= 1) { const ffe k = Kat(j, l12 - 2); iacc_add(A, ff_mul(a1f, ff{k.h, k.l}), k.e); }
        if (qmax >= 2) { const ffe k = Kat(j, l12 - 4); iacc_add(A, ff_mul(a2f, ff{k.h, k.l}), k.e); }
    }

    if (qmax >= 3) {
        // X, Y, Z carry lam = 2^-(30+sig) (p table 2^-30, N(x) 2^-sig); b_q and D_q both
        // pick up lam^(q-2), so a_q = b_q / D_q is unchanged
        const long long Si = l1 + l2 + 1, Di = l1 - l2;
        int ip = l12 - 6; // p of q = 3
        const long long n1st = ((long long)(ip + 1 - Si) * (ip + 1 + Si)) * ((long long)(ip + 1 - Di) * (ip + 1 + Di));
        const int sig = (n1st == 0 ? 0 : (63 - __clzll(n1st < 0 ? -n1st : n1st))) - 20;
        const int sa = sig / 2, sc = sig - sa;
        const float fS = (float)Si, fD = (float)Di;
        const float sA = __uint_as_float((unsigned)(127 - sa) << 23), sC = __uint_as_float((unsigned)(127 - sc) << 23);
        // N(x) = (x^2 - S^2)(x^2 - D^2): each factor is an exact float-float product of
        // two integers below 2^24 (fmaf gives the rounding error exactly), scaled by a
        // power of two (-20 <= sig <= 41, so 2^-sa and 2^-sc are normal and the scaling exact)
        auto Nf = [&](float x) {
            const float p1 = x - fS, p2 = x + fS, q1 = x - fD, q2 = x + fD;
            const float ah = p1 * p2, ch = q1 * q2;
            const ff av{ah * sA, fmaf(p1, p2, -ah) * sA}, cv{ch * sC, fmaf(q1, q2, -ch) * sC};
            return ff_mul(av, cv);
        };
        const bool diag = (l1 == l2);
        // Ap = -2 m (l1 - l2)(l1 + l2 + 1): 2m (l1 - l2) as an exact two-product of integers
        // below 2^24, times l1 + l2 + 1 in float-float; Ap^2 lam to ~2^-48 (sign irrelevant)
        const float m2f = 2.0f * mm, dlf = (float)(l1 - l2), pA = m2f * dlf;
        const ff ApF = ff_mul(ff{pA, fmaf(m2f, dlf, -pA)}, ff{(float)(l1 + l2 + 1), 0.0f});
        const ff Ap2 = diag ? ff{0.0f, 0.0f} : ff_shift(ff_mul(ApF, ApF), -30 - sig);
        const float4 *pt = ptabf + ((size_t)grp.z * 2 + (diag ? 1 : 0)) * pstride * 2; // the m's table
        // b_{q-2} = a_1, b_{q-1} = a_2, D_2 = 1, normalised by the exponent of a_2
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
            for (int j = 0; j < 2 * G; j++) {
                IAcc &A = acc[j];
                if (!(A.st & 1)) continue;
                const ffe Kv = Kat(j, ip);
                const ff t = ff_mul(aq, ff{Kv.h, Kv.l});
                const int et = ea + Kv.e;
                iacc_add(A, t, et);
                // exponent(t) < exponent(q=0 term) - stop_bits: |t| below 2^-stop_bits of the
                // q = 0 term (and above 2^-stop_bits-2 of it when not); a zero term counts as
                // below, as log 0 = -inf does in the reference's test
                const int cnt = fexpo(t.h) + et < (A.st >> 3) ? ((A.st >> 1) & 3) + 1 : 0;
                A.st = (A.st & ~7) | (cnt << 1) | (cnt < 3 ? 1 : 0);
                any |= (A.st & 1) != 0;
            }
        }
    }

    // I = a_0 sum; TE of a perfect reflector is -TM
    const ff a0f{A12.a0h, A12.a0l};
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (g >= ng) break;
        const IAcc &AT = acc[2 * g];
        ff r = ff_mul(a0f, ff{AT.h, AT.l});
        int k = fexpo(r.h);
        if (k == -127 || k == 128) atomicOr(status + tk[g], ST_ERR_NONFINITE);
        if (k == 128 || k == -127) k = 0;
        r = ff_shift(r, -k);
        const int eT = r.h == 0.0f ? FFE_ZERO_E : AT.e + A12.a0e + k;
        store(g, 1, r.h, r.l, eT);
        if (both) {
            const IAcc &AE = acc[2 * g + 1];
            ff s = ff_mul(a0f, ff{AE.h, AE.l});
            int ke = fexpo(s.h);
            if (ke == 128 || ke == -127) ke = 0;
            s = ff_shift(s, -ke);
            store(g, 0, s.h, s.l, s.h == 0.0f ? FFE_ZERO_E : AE.e + A12.a0e + ke);
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
// term count of its slowest frequency.
constexpr int IGRP = 3;
constexpr int ITAB_STOP_BITS = 44; // early stop below 2^-44 of the q = 0 term
int itab_group_size() { return IGRP; }

void launch_itab_grp(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim, const ffe *KF, int nu_stride,
                     const float4 *ptabf, int pstride, const void *a12, void *Iout, bool ffe_out, bool band, int *status,
                     cudaStream_t st)
{
    if (ngroups <= 0) return;
    const long long L = ldim + 2, npair = L * (L + 1) / 2;
    dim3 g((unsigned)(((band ? 2 * L : npair) + 127) / 128), ngroups);
    if (band)
        k_itab_grp<IGRP, true><<<g, 128, 0, st>>>(tasks, tlist, groups, ngroups, (int)ldim, KF, nu_stride, ptabf, pstride,
                                                  (const A012F *)a12, Iout, ffe_out, status, ITAB_STOP_BITS);
    else
        k_itab_grp<IGRP, false><<<g, 128, 0, st>>>(tasks, tlist, groups, ngroups, (int)ldim, KF, nu_stride, ptabf, pstride,
                                                   (const A012F *)a12, Iout, ffe_out, status, ITAB_STOP_BITS);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
