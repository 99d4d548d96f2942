// qsum_ff.cuh -- the float-float q-sum of one (l1, l2) pair for up to G frequencies of one m
// (integration.c:491-609), and its a_0, a_1, a_2 from the per-m tables, shared by the mixed
// form's I-table kernel (itab_ff.cu) and the HODLR path's on-demand elements (hodlr.cu).
//
// The recurrence b_q = X b_{q-1} - Y Z_{q-1} b_{q-2}, D_q = Z D_{q-1} runs once for the pair,
// a_q = b_q / D_q by one float-float division per q, and each frequency accumulates a_q K_q for
// its two polarisations under one exponent frame (the paired K table: KP = TM h, l, TE h, l,
// KPe their common exponent), with the reference's early stop (three consecutive terms below
// 2^-stop_bits of the q = 0 term, integration.c:563-575) applied to the pair of polarisations.
// Everything is float-float (two FP32 words) with separate power-of-two exponents; no FP64
// instruction.  Each sum depends on its own (pair, frequency) only.
#pragma once
#include "common.cuh"
#include "ff.cuh"

namespace capsgpu {

// early stop below 2^-44 of the q = 0 term (the mixed form's elements end in FP32, 2^-24)
constexpr int QSUM_FF_STOP_BITS = 44;

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

// Per task the state is the two float-float sums, the frame exponent, the two stop thresholds
// (in frame units) and the last q with a significant term.  A sum's frame moves up (exact
// power-of-two shifts) only when a term lies more than 2^30 above it.
struct PAcc {
    float th, tl, eh, el; // TM and TE sums, (h + l) 2^e
    int e;
    int thr_t, thr_e;     // exponent (frame units) below which a term is insignificant
    int last;             // last q with a significant term (2 before the loop: q = 3, 4, 5 may stop it)
};


// per-m tables of the mixed a_0, a_1, a_2 (assemble.cu k_a12_tabs), formed in FP64 and stored
// as float-float: per l (index l - (lmin - 1)) and per l1 + l2 (index l1 + l2 - 2(lmin - 1))
struct A12L { ff F1, F2; ffe eG; };
struct A12J { ff h1, pa, pb, pc; ffe eH; };

// a_0, a_1, a_2 of the pair at window indices (a1 >= a2) for azimuthal number mt from the m's
// tables tl (L entries) and tj (2L - 1 entries); zero when I = 0
CAPS_DEV A012F a012f_pair(int mt, int lmin, int a1, int a2, const A12L *__restrict__ tl, const A12J *__restrict__ tj)
{
    const int mm = mt > 0 ? mt : 1;
    const int l1 = lmin - 1 + a1, l2 = lmin - 1 + a2;
    A012F r{0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0, 0};
    if (!(l2 < mm || l2 < mt || l1 < 1)) {
        const int qmax = min(min(l1, l2), (l1 + l2 - 2 * mm) / 2);
        // the closed forms of a_0, a_1, a_2 in float-float (FP32 pipe) from the per-m tables
        const A12L x = tl[a1], y = tl[a2];
        const A12J z = tj[a1 + a2];
        ff p = ff_mul(ff_mul(ff{x.eG.h, x.eG.l}, ff{y.eG.h, y.eG.l}), ff{z.eH.h, z.eH.l});
        int e = x.eG.e + y.eG.e + z.eH.e;
        const int k = fexpo(p.h);
        if (k > -127) { p = ff_shift(p, -k); e += k; }
        r.a0h = p.h;
        r.a0l = p.l;
        r.a0e = e;
        const ff f = ff_add(x.F1, y.F1);
        if (qmax >= 1) {
            const ff v = ff_mul(ff{(float)(l1 + l2) - 1.5f, 0.0f}, ff_add(ff{1.0f, 0.0f}, ff_neg(ff_mul(z.h1, f))));
            r.a1h = v.h;
            r.a1l = v.l;
        }
        if (qmax >= 2) {
            const ff t = ff_add(ff_add(x.F2, ff_mul(ff{2.0f * x.F1.h, 2.0f * x.F1.l}, y.F1)), y.F2);
            const ff v = ff_mul(z.pa, ff_add(ff_mul(z.pb, ff_add(ff_mul(z.pc, t), ff_neg(f))), ff{0.5f, 0.0f}));
            r.a2h = v.h;
            r.a2l = v.l;
        }
    }
    return r;
}

// I = a_0 sum_q a_q K_q of the pair (l1 >= l2 >= m', l1 >= 1) for the ng <= G tasks tk[] that
// share T's m, handed to out(g, pol, h, l, e) (pol 1 TM, 0 TE; value (h + l) 2^e) as each is
// done.  ptm: the m's float-float p table (two rows of 2 pstride float4: l1 != l2, l1 == l2).
// Returns a bit per task whose TM sum is zero or not finite.
template <int G, class OUT>
CAPS_DEV unsigned qsum_ff_pair(const Task &T, const int *tk, int ng, int l1, int l2, const A012F &A12, const float4 *__restrict__ KP,
                               const int *__restrict__ KPe, int nu_stride, const float4 *__restrict__ ptm, int pstride, int stop_bits,
                               OUT out)
{
    const int mm = T.m > 0 ? T.m : 1;
    const bool both = !T.is_pr;
    const int l12 = l1 + l2;
    const int qmax = min(min(l1, l2), (l12 - 2 * mm) / 2);
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
        const float4 *pt = ptm + (diag ? (size_t)pstride * 2 : 0);
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
    unsigned bad = 0;
#pragma unroll
    for (int g = 0; g < G; g++) {
        if (g >= ng) break;
        const PAcc &A = acc[g];
        ff r = ff_mul(a0f, ff{A.th, A.tl});
        int k = fexpo(r.h);
        if (k == -127 || k == 128) bad |= 1u << g;
        if (k == 128 || k == -127) k = 0;
        r = ff_shift(r, -k);
        const int eT = r.h == 0.0f ? FFE_ZERO_E : A.e + A12.a0e + k;
        out(g, 1, r.h, r.l, eT);
        if (both) {
            ff s = ff_mul(a0f, ff{A.eh, A.el});
            int ke = fexpo(s.h);
            if (ke == 128 || ke == -127) ke = 0;
            s = ff_shift(s, -ke);
            out(g, 0, s.h, s.l, s.h == 0.0f ? FFE_ZERO_E : A.e + A12.a0e + ke);
        } else
            out(g, 0, -r.h, -r.l, eT);
    }
    return bad;
}

} // namespace capsgpu
