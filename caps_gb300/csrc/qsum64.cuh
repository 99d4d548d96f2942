// qsum64.cuh -- the FP64 q-sum of one (l1, l2) pair and its a_0, a_1, a_2 (integration.c:
// 491-609), shared by the dense I-table kernels (assemble.cu) and the HODLR path, which
// evaluates matrix elements on demand (hodlr.cu): both form every I value with the same
// arithmetic, so the two paths differ only by HODLR's compression.
//
// The recurrence coefficients of eqs. (26)-(28) are rewritten so that every factor that
// depends on p alone comes from tables (per task: the integer products K0..K3 of p,
// p1=p-2m, p2=p+2m, with 1/(4x^2-1) folded in), the common factor Ap cancels, and alpha is
// formed from an exact integer numerator.  One division per pair remains.
#pragma once
#include "common.cuh"

namespace capsgpu {

struct QAcc {
    double s; int e; bool on; int count;
};

CAPS_DEV void qacc_add(QAcc &A, double mant, int ex)
{
    if (mant == 0.0) return;
    if (A.s == 0.0) { A.s = mant; A.e = ex; return; }
    int d = ex - A.e;
    if (d > 64) { A.s = (A.e - ex < -1000) ? 0.0 : shift2(A.s, A.e - ex); A.e = ex; d = 0; }
    if (d > -1000) A.s += shift2(mant, d);
}


// a_0 (as a scaled double), a_1, a_2 of the q-sum of the pair (l1, l2) = (lmin - 1 + a1,
// lmin - 1 + a2), l1 >= l2, for azimuthal number mt (eqs. (20), (29), (35)); zero when I = 0
CAPS_DEV A012 a012_pair(int mt, int lmin, int a1, int a2, const double *__restrict__ lft)
{
    const int l1 = lmin - 1 + a1, l2 = lmin - 1 + a2;
    const int mm = mt > 0 ? mt : 1;
    A012 r{0.0, 0.0, 0.0, 0, 0};
    if (!(l2 < mm || l2 < mt || l1 < 1)) {
        const double n = l1, nu = l2, m = mm;
        const double n4 = l1 + l2 - 2 * mm;
        const int l12 = l1 + l2;
        const int qmax = min(min(l1, l2), (l12 - 2 * mm) / 2);
        const double log_a0 = __ldg(lft + 2 * l1) - __ldg(lft + l1) + __ldg(lft + 2 * l2) - __ldg(lft + l2) + __ldg(lft + l12)
                            - __ldg(lft + 2 * l12) + __ldg(lft + l12 - 2 * mm) - __ldg(lft + l1 - mm) - __ldg(lft + l2 - mm);
        const sd a0 = sd_from_log(log_a0, 1);
        r.a0m = a0.m;
        r.a0e = a0.e;
        if (qmax >= 1)
            r.a1 = (n + nu - 1.5) * (1 - (2 * n + 2 * nu - 1) / (n4 * (n4 - 1)) * ((m - n) * (m - n + 1) / (2 * n - 1) + (m - nu) * (m - nu + 1) / (2 * nu - 1)));
        if (qmax >= 2)
            r.a2 = (2 * n + 2 * nu - 1) * (2 * n + 2 * nu - 7) / 4 * ((2 * n + 2 * nu - 3) / (n4 * (n4 - 1)) * ((2 * n + 2 * nu - 5) / (2 * (n4 - 2) * (n4 - 3))
                  * ((m - n) * (m - n + 1) * (m - n + 2) * (m - n + 3) / (2 * n - 1) / (2 * n - 3)
                  + 2 * (m - n) * (m - n + 1) * (m - nu) * (m - nu + 1) / ((2 * n - 1) * (2 * nu - 1))
                  + (m - nu) * (m - nu + 1) * (m - nu + 2) * (m - nu + 3) / (2 * nu - 1) / (2 * nu - 3)) - (m - n) * (m - n + 1) / (2 * n - 1)
                  - (m - nu) * (m - nu + 1) / (2 * nu - 1)) + 0.5);
    }
    return r;
}

// the FP64 q-sum of one pair (integration.c:497-609): I_TM and I_TE of (l1, l2), l1 >= l2 >= m,
// l1 >= 1, with a_0..a_2 from a012_pair; KTM, KTE indexed by the degree nu; pt: the task's
// p table (two rows of pstride: l1 != l2, l1 == l2).  Returns true when the result is zero or
// not finite (a numerical failure).
CAPS_DEV bool qsum_pair(const Task &T, int l1, int l2, const A012 &A12, const sd *KTM, const sd *KTE, const double4 *ptab,
                        int pstride, sd &rT, sd &rE)
{
    const int mm = T.m > 0 ? T.m : 1;
    const double n = l1, nu = l2, m = mm;
    const int l12 = l1 + l2;
    const int qmax = min(min(l1, l2), (l12 - 2 * mm) / 2);
    const double Ap = -2 * m * (n - nu) * (n + nu + 1);
    const bool both = !T.is_pr;

    QAcc aT, aE;
    {
        const sd k0 = KTM[l12];
        aT = QAcc{k0.m, k0.e, true, 0};
        if (both) { const sd e0 = KTE[l12]; aE = QAcc{e0.m, e0.e, true, 0}; }
        else aE = QAcc{0, 0, false, 0};
    }
    double aqm2 = 0, aqm1 = 1; // a_{q-2}, a_{q-1}
    if (qmax >= 1) {
        const double a1q = A12.a1;
        const sd kt = KTM[l12 - 2];
        qacc_add(aT, a1q * kt.m, kt.e);
        if (both) { const sd ke = KTE[l12 - 2]; qacc_add(aE, a1q * ke.m, ke.e); }
        aqm2 = 1; aqm1 = a1q;
    }
    if (qmax >= 2) {
        const double a2q = A12.a2;
        const sd kt = KTM[l12 - 4];
        qacc_add(aT, a2q * kt.m, kt.e);
        if (both) { const sd ke = KTE[l12 - 4]; qacc_add(aE, a2q * ke.m, ke.e); }
        aqm2 = aqm1; aqm1 = a2q;
    }
    if (qmax >= 3) {
        // Division-free form of the recurrence: a_q = b_q / D_q with
        //   b_q = X_q b_{q-1} - Y_q Z_{q-1} b_{q-2},  D_q = D_{q-1} Z_q,
        //   X_q = Ap^2 + K1 alpha(p+2) + K2 alpha(p+3), Y_q = K3 alpha(p+4), Z_q = K0 alpha(p+1)
        // (eqs. (26)-(28) with the common factor Ap divided out), and the partial
        // sums carried as S_q = D_q sum_{j<=q} a_j K_j = Z_q S_{q-1} + b_q K_q.
        // b, D and each S keep their own power-of-two exponent; the reference's
        // early stop (term 60 e-folds below the q=0 term, three times in a row)
        // is decided on those exponents, with logarithms only inside the +-2
        // binade band around the threshold.  One division per pair remains.
        // alpha(x) = N(x)/(4x^2-1) with the integer numerator
        // N(x) = (x-S)(x+S)(x-Dd)(x+Dd), S = l1+l2+1, Dd = l1-l2, formed exactly in int64
        // (|N| < 2^62 for every degree this library accepts) and converted once.
        const long long Si = l1 + l2 + 1, Di = l1 - l2;
        auto Nf = [&](int x) -> double {
            const long long a = (long long)(x - Si) * (x + Si), c = (long long)(x - Di) * (x + Di);
            return (double)(a * c);
        };
        const bool diag = (l1 == l2); // Ap == 0: eq. (30)
        const double Ap2 = diag ? 0.0 : Ap * Ap;
        const double4 *pt = ptab + (diag ? pstride : 0);
        struct PS { double S; int eS; bool on; int count; double D; int eD; int e0; const sd *K0; };
        PS P[2] = {{aT.s, aT.e, true, 0, 1.0, 0, 0, KTM + l12}, {aE.s, aE.e, both, 0, 1.0, 0, 0, KTE + l12}};
        P[0].e0 = KTM[l12].e;
        if (both) P[1].e0 = KTE[l12].e;
        const sd *Kp[2] = {KTM, KTE};
        double bm2 = aqm2, bm1 = aqm1, Dq = 1.0, Zprev = 1.0;
        int eb = 0, eD = 0;
        int ip = l12 - 6; // p of q = 3
        double N3 = Nf(ip + 3), N4 = Nf(ip + 4);
        for (int q = 3; q <= qmax && (P[0].on || P[1].on); q++, ip -= 2) {
            const double N1 = Nf(ip + 1), N2 = Nf(ip + 2);
            const double4 k = pt[ip];
            const double X = fma(k.z, N3, fma(k.y, N2, Ap2));
            const double Y = k.w * N4;
            const double Z = k.x * N1;
            const double b = fma(X, bm1, -(Y * Zprev) * bm2);
            Dq *= Z;
            N3 = N1; N4 = N2; Zprev = Z;
            bm2 = bm1; bm1 = b;
            {   // exact rescaling of b (with b_{q-1}) and D
                const int kb = expo(b);
                if (kb > 300 || (kb < -300 && kb > -1023)) { bm1 = shift2(bm1, -kb); bm2 = shift2(bm2, -kb); eb += kb; }
                const int kd = expo(Dq);
                if (kd > 300 || kd < -300) { Dq = shift2(Dq, -kd); eD += kd; }
            }
            const int eb1 = expo(bm1);
            const int eDq = expo(Dq) + eD;
#pragma unroll
            for (int pi = 0; pi < 2; pi++) {
                PS &A = P[pi];
                if (!A.on) continue;
                const sd Kv = Kp[pi][ip];
                const double t = bm1 * Kv.m;          // term * D_q / 2^(eb+Ke)
                const int et = eb + Kv.e;
                // S_q = Z S_{q-1} + t 2^(et - eS)
                int d = et - A.eS;
                const int es = expo(A.S);
                if (es == -1023) { A.eS = et; d = 0; }
                else if (d > 64) { A.S = shift2(A.S, -d); A.eS = et; d = 0; }
                A.S = fma(Z, A.S, shift2(t, d));
                const int ks = expo(A.S);
                if (ks > 300 || (ks < -300 && ks > -1023)) { A.S = shift2(A.S, -ks); A.eS += ks; }
                // early stop on |a_q K_q| / |K_0| < e^-60, i.e. log2 ratio < -86.5617; a zero
                // term counts as below, as log 0 = -inf does in the reference's test
                {
                    const int approx = eb1 + eb + Kv.e - eDq - A.e0; // true log2 ratio in (approx-2, approx+2)
                    bool below;
                    if (eb1 == -1023) below = true;
                    else if (approx <= -89) below = true;
                    else if (approx >= -84) below = false;
                    else {
                        // exact test without logarithms: with mantissas in [1,2),
                        // ratio = 2^approx * (mb mK)/(mD m0) < e^-60  <=>  mb mK < 2^(-60/ln2 - approx) mD m0
                        const double c = approx == -88 ? 2.710008819393852 : approx == -87 ? 1.355004409696926
                                       : approx == -86 ? 0.677502204848463 : 0.3387511024242315;
                        const double mb = shift2(bm1, -eb1), mD = shift2(Dq, -expo(Dq));
                        below = fabs(mb * Kv.m) < c * fabs(mD * A.K0->m);
                    }
                    if (below) { if (++A.count >= 3) { A.on = false; A.D = Dq; A.eD = eD; } }
                    else A.count = 0;
                }
            }
        }
        for (int pi = 0; pi < 2; pi++) {
            PS &A = P[pi];
            if (A.on) { A.D = Dq; A.eD = eD; }
            const sd r = sd_norm(A.S / A.D, A.eS - A.eD);
            if (pi == 0) { aT.s = r.m; aT.e = r.e; } else { aE.s = r.m; aE.e = r.e; }
        }
    }
    const sd a0 = sd{A12.a0m, A12.a0e};
    rT = sd_mul(a0, sd_norm(aT.s, aT.e));
    if (both) rE = sd_mul(a0, sd_norm(aE.s, aE.e));
    else rE = sd{-rT.m, rT.e};
    return !isfinite(rT.m) || rT.m == 0.0;
}

CAPS_DEV sd sdx(double c, sd a) { return sd_norm(c * a.m, a.e); }
CAPS_DEV sd sd_neg(sd a) { return sd{-a.m, a.e}; }

// The 2x2 block of M at l-indices (a, b), a >= b, index i = a + 1 into [lmin-1, lmin+ldim]
// (libcaps.c:761-831, integration.c:762-888): EE, MM and (unless DIAG) EM, ME, from the I
// values that Iv(pol, x, y) returns (pol 1 = TM, 0 = TE; x, y indices into the window) and the
// per-l scale factors Sa, Sb (symmetric scaling) and uv (the B, C, D coefficients).
template <bool DIAG, class IV>
CAPS_DEV void elem_block(int mt, int i1, int i2, sd sa1, sd sa2, sd sb1, sd sb2, double2 uv1, double2 uv2, IV Iv, sd &EE, sd &MM,
                         sd &EM, sd &ME)
{
    const double m = mt;
    EM = sd{0, 0};
    ME = sd{0, 0};
    if (mt == 0) {
        EE = sd_mul(sd_mul(sa1, sa2), Iv(1, i1, i2));          // B_TM, A = 0
        MM = sd_neg(sd_mul(sd_mul(sb1, sb2), Iv(0, i1, i2)));  // -B_TE
    } else {
        const double m2 = m * m;
        auto Bv = [&](int p) {
            sd r = sdx(uv1.x * uv2.x, Iv(p, i1 - 1, i2 - 1));
            r = sd_add(r, sdx(-uv1.y * uv2.x, Iv(p, i1 + 1, i2 - 1)));
            r = sd_add(r, sdx(-uv1.x * uv2.y, Iv(p, i1 - 1, i2 + 1)));
            r = sd_add(r, sdx(uv1.y * uv2.y, Iv(p, i1 + 1, i2 + 1)));
            return r;
        };
        // C_p(l1,l2) = m (v(l2) I(l1,l2+1) - u(l2) I(l1,l2-1)); D_p(l1,l2) = C_p(l2,l1)
        auto Cv = [&](int p) { return sdx(m, sd_add(sdx(uv2.y, Iv(p, i1, i2 + 1)), sdx(-uv2.x, Iv(p, i1, i2 - 1)))); };
        auto Dv = [&](int p) { return sdx(m, sd_add(sdx(uv1.y, Iv(p, i1 + 1, i2)), sdx(-uv1.x, Iv(p, i1 - 1, i2)))); };
        EE = sd_mul(sd_mul(sa1, sa2), sd_add(Bv(1), sdx(-m2, Iv(0, i1, i2))));
        MM = sd_mul(sd_mul(sb1, sb2), sd_add(sdx(m2, Iv(1, i1, i2)), sd_neg(Bv(0))));
        if (!DIAG) {
            EM = sd_mul(sd_mul(sa1, sb2), sd_add(Dv(1), sd_neg(Cv(0))));
            ME = sd_mul(sd_mul(sb1, sa2), sd_add(Cv(1), sd_neg(Dv(0))));
        }
    }
}

} // namespace capsgpu
