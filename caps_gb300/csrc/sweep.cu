// sweep.cu -- the mixed form's round-trip matrix from a band of q-sums and a three-term
// recurrence of the I integrals, with the elements formed as the rows of the table appear.
//
// The q-sum of every (l1, l2) pair (integration.c:491-609) costs O(l) terms, O(ldim^3) per
// matrix.  The I integrals also obey the three-term recurrence of the associated Legendre
// functions in either degree, (2l+1) x P_l^m = (l-m+1) P_{l+1}^m + (l+m) P_{l-1}^m, which,
// applied once in each degree of I_{l1 l2} = int w(x) P_{l1}^{m'} P_{l2}^{m'} (m' = max(m,1)),
// links four neighbours:
//   (l1-m'+1) I(l1+1, l2) = (2l1+1)/(2l2+1) [(l2-m'+1) I(l1, l2+1) + (l2+m') I(l1, l2-1)]
//                           - (l1+m') I(l1-1, l2).
// Seeded with q-sums on the diagonal (l1 = l2), the first subdiagonal (l1 = l2 + 1) and the
// first column of the window, it fills the lower triangle row by row, moving away from the
// diagonal.  Against the q-sums of the reference's algorithm the filled values agree to ~1e-11
// relative (also 1000 rows from the seeds, from xi = 0.1 to 1119, m = 0 to 400), and
// log det(1 - M) built from them moves by <= 5e-14 relative in float-float arithmetic -- far
// below the FP32 storage of M, which dominates the mixed form's error.  The recurrence costs
// O(1) per pair: the q-sums shrink to 4 L pairs per matrix (two of which the trace rule's
// diagonal reads anyway).
//
// Scaling.  The table is held as T(w1, w2) = I(w1, w2) 2^{k(w1) + k(w2)} (w: index into the
// window [lmin-1, lmin+ldim]) with k(w) = -floor(log2 I_TM(w, w) / 2), so that T_TM(w, w) lies in
// [1, 4).  For a plate of real dielectric function the weight w(x) of the integral has one sign
// per polarisation, so I_p is a signed Gram matrix and |T(w1, w2)| <= sqrt(T(w1,w1) T(w2,w2)) < 4:
// every value sits in one fixed float-float frame (no per-entry exponent); far entries that
// fall below 2^-121 of that frame flush to zero, as they do in the FP32 matrix.  The powers of
// two enter the recurrence coefficients exactly.
//
// Elements (libcaps.c:761-831, integration.c:762-888) in this frame.  With
// Um(w) = u(w) 2^{k(w) - k(w-1)}, Vp(w) = v(w) 2^{k(w) - k(w+1)} (u, v the coefficients of the
// B, C, D combinations), dA(w) = Sa(w) 2^{-k(w)}, dB(w) = Sb(w) 2^{-k(w)} (Sa, Sb the symmetric
// Mie and normalisation factors), and per polarisation
//   J(x, y) = Um(x) T(x-1, y) - Vp(x) T(x+1, y)      (B, C, D differentiate in l1 ...)
//   H(x, y) = Um(y) T(x, y-1) - Vp(y) T(x, y+1)      (... and in l2)
//   B(x, y) = Um(y) J(x, y-1) - Vp(y) J(x, y+1),
// the 2x2 block at window row x, column y is
//   EE = dA(x) dA(y) [B_TM - m^2 T_TE],          MM = dB(x) dB(y) [m^2 T_TM - B_TE],
//   EM = m dA(x) dB(y) [H_TE - J_TM],            ME = m dB(x) dA(y) [J_TE - H_TM]
// (m = 0: EE = dA dA T_TM, MM = -dB dB T_TE).  Um = (l+1) Cm and Vp = l Cp for m >= 1, Cp and Cm
// the column coefficients of the recurrence, so one pair of tables serves both.
//
// k_sweep_ff: one CTA per matrix, warp-specialised.  Producer warps form the rows of T into a
// ring of four shared-memory rows (both polarisations) and publish each on an mbarrier;
// consumer warps form the elements of row x once row x + 1 is published, 30 columns per pass
// of 32 lanes (J of the neighbours by shuffles), and release row x - 1 for reuse, so that
// they wait only for a producer that falls behind, never for one another.  The elements go
// straight into the FP32 delta matrix (-M, lower triangle, column-major), with a per-matrix
// sum of squares for the reference's Mercator bound; the FP64 diagonal comes from the band
// (k_diag_ff).
#include "common.cuh"
#include "ff.cuh"
#include "internal.h"
#include "qsum_ff.cuh"
#include "umma.cuh"

namespace capsgpu {

// window index of the first l with I != 0: l = max(lmin - 1, m')
CAPS_DEV int seed_col(const Task &T)
{
    const int mm = T.m > 0 ? T.m : 1;
    return T.lmin - 1 >= mm ? 0 : 1;
}

// ---------------------------------------------------------------------------
// seeds: q-sums of the pairs of two kinds per window index w
// ---------------------------------------------------------------------------
// grid (2 ceil(L/128), ngroups): the first half of the blocks computes kind0, the second kind1
// (so that a warp runs sums of one kind and similar length).  groups as in launch_itab_grp; a_0,
// a_1, a_2 come from the per-m tables (a012f_pair), so no pair table is formed.  seed[((task *
// 2 + pol) * SEED_KINDS + kind) * L + w] receives the pair's value as float-float with exponent;
// pairs outside the window are not written (nothing reads them).
template <int G>
__global__ void __launch_bounds__(128, 7) k_seed_ff(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim,
                                                    const float4 *__restrict__ KP, const int *__restrict__ KPe, int nu_stride,
                                                    const float4 *__restrict__ ptabf, int pstride, const A12L *__restrict__ tl,
                                                    const A12J *__restrict__ tj, int kind0, int kind1, ffe *seed, int *status,
                                                    int stop_bits)
{
    const int L = ldim + 2, NJ = 2 * L - 1, nbw = (L + 127) / 128;
    const int gi = blockIdx.y;
    if (gi >= ngroups) return;
    const int kind = (int)blockIdx.x < nbw ? kind0 : kind1;
    const int w = ((int)blockIdx.x % nbw) * 128 + threadIdx.x;
    if (w >= L) return;
    const int4 grp = groups[gi];
    const int ng = grp.y;
    int tk[G];
#pragma unroll
    for (int g = 0; g < G; g++) tk[g] = g < ng ? (tlist ? tlist[grp.x + g] : grp.x + g) : 0;
    const Task &T = tasks[tk[0]];
    int a1 = w, a2 = w;
    if (kind == SEED_D1) a1 = w + 1;
    else if (kind == SEED_D2) a1 = w + 2;
    else if (kind == SEED_COL) a2 = seed_col(T);
    if (a1 >= L) return;
    auto store = [&](int g, int pol, float h, float l, int e) {
        seed[((size_t)(tk[g] * 2 + pol) * SEED_KINDS + kind) * L + w] = ffe{h, l, e, 0};
    };
    const int mm = T.m > 0 ? T.m : 1, l1 = T.lmin - 1 + a1, l2 = T.lmin - 1 + a2;
    if (a1 < a2 || l2 < mm || l2 < T.m || l1 < 1) { // I = 0 for l < m (integration.c:631)
        for (int g = 0; g < ng; g++) { store(g, 1, 0.0f, 0.0f, FFE_ZERO_E); store(g, 0, 0.0f, 0.0f, FFE_ZERO_E); }
        return;
    }
    const A012F A12 = a012f_pair(T.m, T.lmin, a1, a2, tl + (size_t)grp.z * L, tj + (size_t)grp.z * NJ);
    const unsigned bad = qsum_ff_pair<G>(T, tk, ng, l1, l2, A12, KP, KPe, nu_stride, ptabf + (size_t)grp.z * 2 * pstride * 2,
                                          pstride, stop_bits, store);
#pragma unroll
    for (int g = 0; g < G; g++)
        if (g < ng && (bad & (1u << g))) atomicOr(status + tk[g], ST_ERR_NONFINITE);
}

// ---------------------------------------------------------------------------
// the sweep
// ---------------------------------------------------------------------------
constexpr int SW_NT = 320, SW_NW = SW_NT / 32; // threads, warps per CTA
constexpr int SW_PW = 3, SW_CW = SW_NW - SW_PW;  // producer (recurrence) and consumer (element) warps
constexpr int SW_CH = 30;                       // output columns of a consumer pass (32 lanes)
constexpr int SW_RING = 4;                      // rows of T held in shared memory
constexpr int SW_WAIT_ITERS = 1 << 22;          // polls of a bounded mbarrier wait
constexpr size_t SW_BYTES_PER_L = SW_RING * 2 * sizeof(float2) + 2 * sizeof(float4) + 2 * sizeof(int);

CAPS_DEV ff ff_sub(ff x, ff y) { return ff_add(x, ff_neg(y)); }
// x c for c exactly representable in FP32 (small integers)
CAPS_DEV ff ff_mulf(ff x, float c)
{
    const float p = x.h * c;
    float e = fmaf(x.h, c, -p);
    e = fmaf(x.l, c, e);
    return ff_fast2(p, e);
}
// a x + b y: the two products with their rounding errors (fmaf), one exact sum of the leading
// parts and one renormalisation (the float-float error of ff_add(ff_mul, ff_mul), fewer steps)
CAPS_DEV ff ff_dot2(ff a, ff x, ff b, ff y)
{
    const float p = a.h * x.h, q = b.h * y.h;
    float ep = fmaf(a.h, x.h, -p);
    ep = fmaf(a.h, x.l, ep);
    ep = fmaf(a.l, x.h, ep);
    float eq = fmaf(b.h, y.h, -q);
    eq = fmaf(b.h, y.l, eq);
    eq = fmaf(b.l, y.h, eq);
    const float s = p + q, bb = s - p;
    const float t = (p - (s - bb)) + (q - bb);
    return ff_fast2(s, t + (ep + eq));
}
// a x + b y + c z, c exactly representable in FP32
CAPS_DEV ff ff_dot3f(ff a, ff x, ff b, ff y, float c, ff z)
{
    const float p = a.h * x.h, q = b.h * y.h, u = c * z.h;
    float ep = fmaf(a.h, x.h, -p);
    ep = fmaf(a.h, x.l, ep);
    ep = fmaf(a.l, x.h, ep);
    float eq = fmaf(b.h, y.h, -q);
    eq = fmaf(b.h, y.l, eq);
    eq = fmaf(b.l, y.h, eq);
    float eu = fmaf(c, z.h, -u);
    eu = fmaf(c, z.l, eu);
    const float s1 = p + q, b1 = s1 - p, t1 = (p - (s1 - b1)) + (q - b1);
    const float s2 = s1 + u, b2 = s2 - s1, t2 = (s1 - (s2 - b2)) + (u - b2);
    return ff_fast2(s2, (t1 + t2) + (ep + (eq + eu)));
}

// 1 / y in float-float: the hardware reciprocal and two corrections (relative error ~2^-48)
CAPS_DEV ff ff_rcp(ff y)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y.h));
    ff q{r, 0.0f};
#pragma unroll
    for (int it = 0; it < 2; it++) {
        const ff e = ff_sub(ff{1.0f, 0.0f}, ff_mul(q, y));
        q = ff_add(q, ff_mul(q, e));
    }
    return q;
}

// k(w) of the scaling: I_TM(w, w) 2^{2 k(w)} in [1, 4).  Window indices below the first
// column (zero rows) take the first column's k.
CAPS_DEV int sw_k(const ffe *__restrict__ d0tm, int w, int c)
{
    const ffe v = d0tm[w < c ? c : w];
    return v.h == 0.0f ? 0 : -(v.e >> 1);
}

// a seed (h + l) 2^e in the frame: times 2^{k1 + k2}
CAPS_DEV ff sw_seed(const ffe &v, int k12) { return v.h == 0.0f ? ff{0.0f, 0.0f} : ff_shift(ff{v.h, v.l}, v.e + k12); }

// FP32 of (d1 d2 2^e) v: the float-float product d1 d2 unrounded, times v with one rounding
// (error ~0.5 ulp); below 2^-120 -> 0, non-finite or above 2^125 sets bad
CAPS_DEV float sw_out(ff d1, ff d2, int e, ff v, bool &bad)
{
    const float a = d1.h * d2.h;
    float ea = fmaf(d1.h, d2.h, -a);
    ea = fmaf(d1.h, d2.l, ea);
    ea = fmaf(d1.l, d2.h, ea);
    const float h = fmaf(a, v.h, fmaf(ea, v.h, a * v.l));
    const int k = fexpo(h);
    if (k == -127) return 0.0f;
    if (k == 128 || k + e > 125) { bad = true; return h; }
    return fshift(h, e);
}

CAPS_DEV ff ldff(const float2 *p) { const float2 v = *p; return ff{v.x, v.y}; }

// bounded wait for phase `parity` of an mbarrier that also gives up once another role has
// given up (*abort); a wait that runs out sets *abort
CAPS_DEV bool sw_wait(uint64_t *mbar, uint32_t parity, volatile int *abort)
{
    const uint32_t a = umma::smem_u32(mbar);
    for (int it = 0; it < SW_WAIT_ITERS; it++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done) return true;
        if ((it & 63) == 63 && *abort) return false;
    }
    *abort = 1;
    return false;
}
CAPS_DEV void sw_arrive(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_u32(mbar)) : "memory");
}
// barrier of the SW_PW producer warps alone (hardware barrier 1)
CAPS_DEV void sw_producer_bar() { asm volatile("bar.sync 1, %0;" ::"n"(SW_PW * 32) : "memory"); }

// grid nlist (task tlist[b], or b), SW_NT threads, SW_BYTES_PER_L * L bytes of dynamic shared memory.
// S receives -M (lower triangle, column-major, leading dimension 2 ldim); part[task] the sum of
// squares of M (both triangles).  Tasks with an error status are skipped.
//
// Warp-specialised: SW_PW producer warps form the rows of T (lane y forms T(r, y) from rows r-1
// and r-2) into a ring of SW_RING rows and publish each on its slot's "ready" mbarrier; SW_CW
// consumer warps form the elements of row x once row x + 1 is ready, in passes of 30 columns
// (32 lanes, the two outer ones repeating the neighbours' edges, J of the neighbours by
// shuffles), and release row x - 1 on its slot's "free" mbarrier, which the producers wait
// for before they reuse the slot.  Consumers therefore never wait for one another, only for a
// producer that falls behind.  Row r also writes T(r, r-1) and T(r, r-2) past the diagonals
// of rows r-1 and r-2 (index r), so that the consumers read rows x-1, x, x+1 up to column
// x + 1 directly.  Every wait is bounded; a role that gives up flags the others, and the
// matrix gets ST_ERR_WAIT.
__global__ void __launch_bounds__(SW_NT, 2) k_sweep_ff(const Task *tasks, const int *tlist, int nlist, int ldim,
                                                       const ffe *__restrict__ seed, const ffe *__restrict__ Saf,
                                                       const ffe *__restrict__ Sbf, float *S, size_t sstride, float *part,
                                                       int *status)
{
    extern __shared__ __align__(16) unsigned char sw_smem[];
    __shared__ uint64_t rready[SW_RING], rfree[SW_RING];
    __shared__ int s_abort, s_ok;
    __shared__ float2 seedrow[2][3][2]; // scaled seeds of the producers' next row: [row parity][D0, D1, COL][TE, TM]
    __shared__ float red[SW_NW];
    const int L = ldim + 2, n = 2 * ldim;
    if ((int)blockIdx.x >= nlist) return;
    const int task = tlist ? tlist[blockIdx.x] : (int)blockIdx.x;
    if (status[task] & ~0xF) return; // uniform per block
    const Task &T = tasks[task];
    const int mt = T.m, mm = mt > 0 ? mt : 1, lm1 = T.lmin - 1, c = seed_col(T);
    float2 *ring = reinterpret_cast<float2 *>(sw_smem);   // [SW_RING][pol][L], pol 1 = TM, 0 = TE
    float4 *cpm = reinterpret_cast<float4 *>(ring + (size_t)SW_RING * 2 * L); // Cp h, l, Cm h, l
    float4 *dab = cpm + L;                                                   // dA h, l, dB h, l
    int *eab = reinterpret_cast<int *>(dab + L);                             // exponents of dA (low 16 bits), dB
    int *ktab = eab + L;                                                     // k(w) of the scaling
    auto sp = [&](int pol, int kind) { return seed + ((size_t)(task * 2 + pol) * SEED_KINDS + kind) * L; };
    auto rowp = [&](int r) { return ring + (size_t)((r % SW_RING) * 2) * L; }; // row r (r >= 0): TE at +0, TM at +L
    const ffe *d0tm = sp(1, SEED_D0);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    // per window index: k(w), then the recurrence's column coefficients and the element factors
    for (int w = tid; w < L; w += SW_NT) ktab[w] = sw_k(d0tm, w, c);
    __syncthreads();
    for (int w = tid; w < L; w += SW_NT) {
        const int l = lm1 + w, kw = ktab[w];
        ff cp{0.0f, 0.0f}, cmv{0.0f, 0.0f};
        if (w >= c && w + 1 < L) cp = ff_shift(ff_from_d((double)(l - mm + 1) / (2.0 * l + 1)), kw - ktab[w + 1]);
        if (w >= c + 1) cmv = ff_shift(ff_from_d((double)(l + mm) / (2.0 * l + 1)), kw - ktab[w - 1]);
        cpm[w] = make_float4(cp.h, cp.l, cmv.h, cmv.l);
        const ffe a = Saf[(size_t)task * L + w], b = Sbf[(size_t)task * L + w];
        dab[w] = make_float4(a.h, a.l, b.h, b.l);
        const int ea = a.h == 0.0f ? 0 : min(max(a.e - kw, -30000), 30000);
        const int eb = b.h == 0.0f ? 0 : min(max(b.e - kw, -30000), 30000);
        eab[w] = (int)(((unsigned)ea & 0xffffu) | ((unsigned)eb << 16));
    }
    if (tid == 0) {
        for (int i = 0; i < SW_RING; i++) {
            umma::mbar_init(&rready[i], 1);
            umma::mbar_init(&rfree[i], SW_CW);
        }
        s_abort = 0;
    }
    __syncthreads();
    volatile int *abort = &s_abort;
    const ff zero{0.0f, 0.0f};
    float fro = 0.0f;
    bool bad = false;

    if (warp < SW_PW) {
        // ---- producers: rows of T ----
        // the seeds of row r (pairs (r, r), (r, r-1), (r, c)), scaled into the frame, into
        // seedrow[r & 1] by threads 0..5 one row ahead, so that their loads are off the row's path
        auto fetch_seeds = [&](int r) {
            if (tid < 6 && r < L) {
                const int kind = tid >> 1, pol = tid & 1;
                const int y = kind == 0 ? r : (kind == 1 ? r - 1 : c), wi = kind == 2 ? r : y;
                const int skind = kind == 0 ? SEED_D0 : (kind == 1 ? SEED_D1 : SEED_COL);
                ff v = zero;
                if (y >= c && wi >= 0) v = sw_seed(sp(pol, skind)[wi], ktab[r] + ktab[y]);
                seedrow[r & 1][kind][pol] = make_float2(v.h, v.l);
            }
        };
        fetch_seeds(0);
        sw_producer_bar();
        for (int r = 0; r < L; r++) {
            const int s = r % SW_RING;
            if (r >= SW_RING) { // slot s held row r - SW_RING: every consumer warp has released it
                if (tid == 0) s_ok = sw_wait(&rfree[s], (r / SW_RING - 1) & 1, abort) ? 1 : 0;
                sw_producer_bar();
                if (!s_ok) break; // uniform over the producer warps
            }
            float2 *W = rowp(r);
            const float2 *P1 = r >= 1 ? rowp(r - 1) : W, *P2 = r >= 2 ? rowp(r - 2) : W;
            float2 *X1 = const_cast<float2 *>(P1), *X2 = const_cast<float2 *>(P2);
            // the recurrence of row r divided by its row coefficient: R1 = 1 / Cp(r-1), R2 = R1 Cm(r-1)
            ff R1 = zero, nR2 = zero;
            if (r >= c + 3) {
                const float4 q = cpm[r - 1];
                R1 = ff_rcp(ff{q.x, q.y});
                nR2 = ff_neg(ff_mul(R1, ff{q.z, q.w}));
            }
            fetch_seeds(r + 1); // read at row r + 1, after the barriers below
            for (int y = tid; y <= r; y += SW_PW * 32) {
                ff vT = zero, vE = zero;
                if (y < c) {
                } else if (y == r || y == r - 1 || y == c) {
                    const int kind = y == r ? 0 : (y == r - 1 ? 1 : 2);
                    const float2 t1 = seedrow[r & 1][kind][1], t0 = seedrow[r & 1][kind][0];
                    vT = ff{t1.x, t1.y};
                    vE = ff{t0.x, t0.y};
                } else {
                    const float4 q = cpm[y];
                    const ff Cp{q.x, q.y}, Cm{q.z, q.w};
                    vT = ff_dot2(R1, ff_dot2(Cp, ldff(P1 + L + y + 1), Cm, ldff(P1 + L + y - 1)), nR2, ldff(P2 + L + y));
                    vE = ff_dot2(R1, ff_dot2(Cp, ldff(P1 + y + 1), Cm, ldff(P1 + y - 1)), nR2, ldff(P2 + y));
                }
                W[L + y] = make_float2(vT.h, vT.l);
                W[y] = make_float2(vE.h, vE.l);
                // T(r, r-1) and T(r, r-2) past the diagonals of rows r-1 and r-2
                if (y == r - 1) { X1[L + r] = make_float2(vT.h, vT.l); X1[r] = make_float2(vE.h, vE.l); }
                if (y == r - 2) { X2[L + r] = make_float2(vT.h, vT.l); X2[r] = make_float2(vE.h, vE.l); }
            }
            sw_producer_bar(); // row r complete before the next row reads it, and before it is published
            if (tid == 0) sw_arrive(&rready[s]);
        }
    } else {
        // ---- consumers: elements of rows x = 1 .. ldim ----
        const int cw = warp - SW_PW;
        const float m2 = (float)mt * (float)mt; // exact for m < 4096
        float *Sm = S + (size_t)task * sstride;
        bool ok = __all_sync(0xffffffffu, sw_wait(&rready[0], 0, abort) && sw_wait(&rready[1], 0, abort));
        for (int x = 1; ok && x <= ldim; x++) {
            ok = __all_sync(0xffffffffu, sw_wait(&rready[(x + 1) % SW_RING], ((x + 1) / SW_RING) & 1, abort));
            if (!ok) break;
            const float2 *Rm = rowp(x - 1), *R0 = rowp(x), *Rp = rowp(x + 1);
            const float4 qx = cpm[x], dx = dab[x];
            const int ex = eab[x];
            const ff Umx = ff_mulf(ff{qx.z, qx.w}, (float)(lm1 + x + 1)), nVpx = ff_neg(ff_mulf(ff{qx.x, qx.y}, (float)(lm1 + x)));
            const ff dAx{dx.x, dx.y}, dBx{dx.z, dx.w};
            const ff mdAx = ff_mulf(dAx, (float)mt), mdBx = ff_mulf(dBx, (float)mt);
            const int eAx = (int)(short)(ex & 0xffff), eBx = ex >> 16;
            const int r0 = 2 * (x - 1);
            for (int k = cw; k * SW_CH <= x; k += SW_CW) {
                const int y = k * SW_CH - 1 + lane;
                // J(x, y) = Um(x) T(x-1, y) - Vp(x) T(x+1, y), y in [0, x+1]
                ff JT = zero, JE = zero;
                if (mt > 0 && y >= 0 && y <= x + 1) {
                    JT = ff_dot2(Umx, ldff(Rm + L + y), nVpx, ldff(Rp + L + y));
                    JE = ff_dot2(Umx, ldff(Rm + y), nVpx, ldff(Rp + y));
                }
                const ff JTm{__shfl_up_sync(0xffffffffu, JT.h, 1), __shfl_up_sync(0xffffffffu, JT.l, 1)};
                const ff JTp{__shfl_down_sync(0xffffffffu, JT.h, 1), __shfl_down_sync(0xffffffffu, JT.l, 1)};
                const ff JEm{__shfl_up_sync(0xffffffffu, JE.h, 1), __shfl_up_sync(0xffffffffu, JE.l, 1)};
                const ff JEp{__shfl_down_sync(0xffffffffu, JE.h, 1), __shfl_down_sync(0xffffffffu, JE.l, 1)};
                if (lane == 0 || lane == 31 || y < 1 || y > x) continue;
                const float4 dy = dab[y];
                const int ey = eab[y];
                const ff dAy{dy.x, dy.y}, dBy{dy.z, dy.w};
                const int eAy = (int)(short)(ey & 0xffff), eBy = ey >> 16;
                const ff c1T = ldff(R0 + L + y), c1E = ldff(R0 + y);
                float ee, mmv, em = 0.0f, me = 0.0f;
                if (mt == 0) {
                    ee = sw_out(dAx, dAy, eAx + eAy, c1T, bad);
                    mmv = sw_out(dBx, dBy, eBx + eBy, ff_neg(c1E), bad);
                } else {
                    const float4 qy = cpm[y];
                    const int ly = lm1 + y;
                    const ff Umy = ff_mulf(ff{qy.z, qy.w}, (float)(ly + 1)), nVpy = ff_neg(ff_mulf(ff{qy.x, qy.y}, (float)ly));
                    const ff HT = ff_dot2(Umy, ldff(R0 + L + y - 1), nVpy, ldff(R0 + L + y + 1));
                    const ff HE = ff_dot2(Umy, ldff(R0 + y - 1), nVpy, ldff(R0 + y + 1));
                    // EE = dA dA [B_TM - m^2 T_TE], MM = dB dB [m^2 T_TM - B_TE], B(x, y) = Um(y) J(x, y-1) - Vp(y) J(x, y+1)
                    const ff iEE = ff_dot3f(Umy, JTm, nVpy, JTp, -m2, c1E);
                    const ff iMM = ff_neg(ff_dot3f(Umy, JEm, nVpy, JEp, -m2, c1T));
                    ee = sw_out(dAx, dAy, eAx + eAy, iEE, bad);
                    mmv = sw_out(dBx, dBy, eBx + eBy, iMM, bad);
                    em = sw_out(mdAx, dBy, eAx + eBy, ff_sub(HE, JT), bad);
                    me = sw_out(mdBx, dAy, eBx + eAy, ff_sub(JE, HT), bad);
                }
                const int c0 = 2 * (y - 1);
                *reinterpret_cast<float2 *>(Sm + (size_t)c0 * n + r0) = make_float2(-ee, -me);
                if (y != x) {
                    *reinterpret_cast<float2 *>(Sm + (size_t)(c0 + 1) * n + r0) = make_float2(-em, -mmv);
                    fro += 2.0f * (ee * ee + me * me + mmv * mmv + em * em);
                } else {
                    Sm[(size_t)(c0 + 1) * n + r0 + 1] = -mmv;
                    fro += ee * ee + mmv * mmv + 2.0f * me * me;
                }
            }
            __syncwarp();
            if (lane == 0) sw_arrive(&rfree[(x - 1) % SW_RING]); // row x - 1 is done with
        }
    }
    __syncthreads();
    for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
    if (lane == 0) red[warp] = fro;
    const int anybad = __syncthreads_or(bad);
    if (tid == 0) {
        float sum = 0.0f;
        for (int w = 0; w < SW_NW; w++) sum += red[w];
        part[task] = sum;
        if (anybad) atomicOr(status + task, ST_ERR_NONFINITE);
        if (s_abort) atomicOr(status + task, ST_ERR_WAIT);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
size_t seed_bytes(int ldim, int ntask) { return (size_t)ntask * 2 * SEED_KINDS * (ldim + 2) * sizeof(ffe); }

size_t sweep_smem_bytes(int ldim) { return SW_BYTES_PER_L * (size_t)(ldim + 2); }

bool sweep_fits(int ldim)
{
    static int smax = -1;
    if (smax < 0) {
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    }
    return sweep_smem_bytes(ldim) + 256 <= (size_t)smax;
}

void launch_seed_ff(const Task *tasks, const int *tlist, const int4 *groups, int ngroups, int ldim, const float4 *KP, const int *KPe,
                    int nu_stride, const float4 *ptabf, int pstride, const void *a12t, int ngroup_all, void *seed, bool band,
                    int *status, cudaStream_t st)
{
    if (ngroups <= 0) return;
    const int L = ldim + 2;
    const A12L *tl = (const A12L *)a12t;
    const A12J *tj = (const A12J *)((const char *)a12t + (size_t)L * ngroup_all * sizeof(A12L));
    dim3 g(2 * ((L + 127) / 128), ngroups);
    k_seed_ff<3><<<g, 128, 0, st>>>(tasks, tlist, groups, ngroups, ldim, KP, KPe, nu_stride, ptabf, pstride, tl, tj,
                                    band ? SEED_D0 : SEED_D1, band ? SEED_D2 : SEED_COL, (ffe *)seed, status, QSUM_FF_STOP_BITS);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

void launch_sweep_ff(const Task *tasks, const int *tlist, int nlist, int ldim, const void *seed, const void *Saf, const void *Sbf,
                     float *S, size_t sstride, float *part, int *status, cudaStream_t st)
{
    if (nlist <= 0) return;
    static size_t attr = 0;
    const size_t smem = sweep_smem_bytes(ldim);
    if (smem > attr) {
        CK(cudaFuncSetAttribute(k_sweep_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = smem;
    }
    k_sweep_ff<<<nlist, SW_NT, smem, st>>>(tasks, tlist, nlist, ldim, (const ffe *)seed, (const ffe *)Saf, (const ffe *)Sbf, S, sstride,
                                           part, status);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
}

} // namespace capsgpu
