// mlp.cu -- a small MLP trained on the GPU that predicts log|logdetD(xi, m)|.
//
// Network: 5 inputs -> 64 -> 64 -> 64 -> 1, SiLU activations, FP32.  Inputs are
// the normalised features (log R/L, 2 xi L/c, m/sqrt(R/L), omega_p, gamma) built by the
// caller.  Hand-written kernels:
//   k_mlp_fwdbwd  one CTA of 64 threads (one per neuron) walks a slice of the
//                 batch: forward pass, MSE loss, backward pass; per-CTA gradient
//                 partials are kept in shared memory (each thread owns the rows of
//                 its neuron, so no atomics) and written out per CTA;
//   k_mlp_reduce  fixed-order sum of the CTA partials (deterministic gradients);
//   k_mlp_adam    Adam update, one thread per parameter;
//   k_mlp_fwd     inference.
// Parameter layout (floats): W1[64][5] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[64] b4[1].
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "../../include/libcaps.h"
#include "internal.h"

namespace capsgpu {

constexpr int HN = 64, NIN = 5;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + HN * NIN, OFF_W2 = OFF_B1 + HN, OFF_B2 = OFF_W2 + HN * HN,
              OFF_W3 = OFF_B2 + HN, OFF_B3 = OFF_W3 + HN * HN, OFF_W4 = OFF_B3 + HN, OFF_B4 = OFF_W4 + HN,
              NPARAM = OFF_B4 + 1;

__device__ __forceinline__ float sig(float x) { return 1.0f / (1.0f + expf(-x)); }

// forward (and optionally backward) of the samples [blockIdx.x*per, ...); y == nullptr: inference only
__global__ void __launch_bounds__(HN) k_mlp_fwdbwd(const float *__restrict__ P, const float *__restrict__ X, const float *__restrict__ Y,
                                                   int n, int per, float *out, float *gpart, float *lpart)
{
    extern __shared__ float sm[];
    float *w = sm;                      // parameters
    float *g = sm + NPARAM;             // gradient accumulators (backward only)
    float *h1 = g + (Y ? NPARAM : 0), *h2 = h1 + HN, *h3 = h2 + HN, *d3 = h3 + HN, *d2 = d3 + HN, *red = d2 + HN;
    const int j = threadIdx.x;
    for (int i = j; i < NPARAM; i += HN) { w[i] = P[i]; if (Y) g[i] = 0.0f; }
    __syncthreads();
    const int s0 = blockIdx.x * per, s1 = min(n, s0 + per);
    float loss = 0.0f;
    for (int s = s0; s < s1; s++) {
        const float *x = X + (size_t)s * NIN;
        float z1 = w[OFF_B1 + j];
#pragma unroll
        for (int c = 0; c < NIN; c++) z1 = fmaf(w[OFF_W1 + j * NIN + c], x[c], z1);
        const float s1g = sig(z1);
        h1[j] = z1 * s1g;
        __syncthreads();
        float z2 = w[OFF_B2 + j];
        for (int k = 0; k < HN; k++) z2 = fmaf(w[OFF_W2 + j * HN + k], h1[k], z2);
        const float s2g = sig(z2);
        h2[j] = z2 * s2g;
        __syncthreads();
        float z3 = w[OFF_B3 + j];
        for (int k = 0; k < HN; k++) z3 = fmaf(w[OFF_W3 + j * HN + k], h2[k], z3);
        const float s3g = sig(z3);
        h3[j] = z3 * s3g;
        // output: b4 + sum_j W4[j] h3[j]  (fixed-order reduction through shared memory)
        red[j] = w[OFF_W4 + j] * h3[j];
        __syncthreads();
        for (int st = HN / 2; st > 0; st >>= 1) {
            if (j < st) red[j] += red[j + st];
            __syncthreads();
        }
        const float yhat = red[0] + w[OFF_B4];
        __syncthreads();
        if (!Y) {
            if (j == 0) out[s] = yhat;
            continue;
        }
        const float r = yhat - Y[s];
        loss += r * r;
        const float d4 = 2.0f * r / n;          // d loss / d yhat, loss = mean (yhat - y)^2
        // layer 4
        g[OFF_W4 + j] += d4 * h3[j];
        if (j == 0) g[OFF_B4] += d4;
        const float dz3 = d4 * w[OFF_W4 + j] * s3g * (1.0f + z3 * (1.0f - s3g));
        d3[j] = dz3;
        __syncthreads();
        for (int k = 0; k < HN; k++) g[OFF_W3 + j * HN + k] += dz3 * h2[k];
        g[OFF_B3 + j] += dz3;
        float a2 = 0.0f;
        for (int i = 0; i < HN; i++) a2 = fmaf(w[OFF_W3 + i * HN + j], d3[i], a2);
        const float dz2 = a2 * s2g * (1.0f + z2 * (1.0f - s2g));
        d2[j] = dz2;
        __syncthreads();
        for (int k = 0; k < HN; k++) g[OFF_W2 + j * HN + k] += dz2 * h1[k];
        g[OFF_B2 + j] += dz2;
        float a1 = 0.0f;
        for (int i = 0; i < HN; i++) a1 = fmaf(w[OFF_W2 + i * HN + j], d2[i], a1);
        const float dz1 = a1 * s1g * (1.0f + z1 * (1.0f - s1g));
#pragma unroll
        for (int c = 0; c < NIN; c++) g[OFF_W1 + j * NIN + c] += dz1 * x[c];
        g[OFF_B1 + j] += dz1;
        __syncthreads();
    }
    if (!Y) return;
    for (int i = j; i < NPARAM; i += HN) gpart[(size_t)blockIdx.x * NPARAM + i] = g[i];
    if (j == 0) lpart[blockIdx.x] = loss;
}

__global__ void k_mlp_reduce(const float *gpart, const float *lpart, int nblk, float *grad, float *loss, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < NPARAM) {
        float s = 0.0f;
        for (int b = 0; b < nblk; b++) s += gpart[(size_t)b * NPARAM + i];
        grad[i] = s;
    }
    if (i == 0) {
        float s = 0.0f;
        for (int b = 0; b < nblk; b++) s += lpart[b];
        *loss = s / n;
    }
}

__global__ void k_mlp_adam(float *P, const float *grad, float *m1, float *m2, int t, float lr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NPARAM) return;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float gi = grad[i];
    m1[i] = b1 * m1[i] + (1 - b1) * gi;
    m2[i] = b2 * m2[i] + (1 - b2) * gi * gi;
    const float mh = m1[i] / (1 - powf(b1, (float)t)), vh = m2[i] / (1 - powf(b2, (float)t));
    P[i] -= lr * mh / (sqrtf(vh) + eps);
}

} // namespace capsgpu

using namespace capsgpu;

struct caps_mlp {
    float *P = nullptr, *G = nullptr, *M1 = nullptr, *M2 = nullptr, *loss = nullptr;
    float *X = nullptr, *Y = nullptr, *out = nullptr, *gpart = nullptr, *lpart = nullptr;
    size_t cap = 0, blk_cap = 0;
    int t = 0;
};

static void mlp_reserve(caps_mlp_t *m, size_t n)
{
    if (n > m->cap) {
        if (m->X) { CK(cudaFree(m->X)); CK(cudaFree(m->Y)); CK(cudaFree(m->out)); }
        m->cap = std::max(n, (size_t)1024);
        CK(cudaMalloc(&m->X, m->cap * NIN * sizeof(float)));
        CK(cudaMalloc(&m->Y, m->cap * sizeof(float)));
        CK(cudaMalloc(&m->out, m->cap * sizeof(float)));
    }
}

static int mlp_blocks(int n, int *per)
{
    const int nblk = std::max(1, std::min(304, (n + 15) / 16));
    *per = (n + nblk - 1) / nblk;
    return (n + *per - 1) / *per;
}

static void mlp_reserve_blocks(caps_mlp_t *m, size_t nblk)
{
    if (nblk > m->blk_cap) {
        if (m->gpart) { CK(cudaFree(m->gpart)); CK(cudaFree(m->lpart)); }
        m->blk_cap = std::max(nblk, (size_t)304);
        CK(cudaMalloc(&m->gpart, m->blk_cap * NPARAM * sizeof(float)));
        CK(cudaMalloc(&m->lpart, m->blk_cap * sizeof(float)));
    }
}

static size_t mlp_smem(bool train) { return (size_t)(NPARAM * (train ? 2 : 1) + 6 * HN) * sizeof(float); }

extern "C" int caps_mlp_nparams(void) { return NPARAM; }

extern "C" caps_mlp_t *caps_mlp_create(unsigned seed)
{
    caps_mlp_t *m = new caps_mlp_t();
    std::vector<float> p(NPARAM, 0.0f);
    std::mt19937 rng(seed);
    auto init = [&](int off, int fan_in, int count) {
        std::normal_distribution<float> d(0.0f, std::sqrt(2.0f / fan_in));
        for (int i = 0; i < count; i++) p[off + i] = d(rng);
    };
    init(OFF_W1, NIN, HN * NIN);
    init(OFF_W2, HN, HN * HN);
    init(OFF_W3, HN, HN * HN);
    init(OFF_W4, HN, HN);
    CK(cudaMalloc(&m->P, NPARAM * sizeof(float)));
    CK(cudaMalloc(&m->G, NPARAM * sizeof(float)));
    CK(cudaMalloc(&m->M1, NPARAM * sizeof(float)));
    CK(cudaMalloc(&m->M2, NPARAM * sizeof(float)));
    CK(cudaMalloc(&m->loss, sizeof(float)));
    CK(cudaMemcpy(m->P, p.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemset(m->M1, 0, NPARAM * sizeof(float)));
    CK(cudaMemset(m->M2, 0, NPARAM * sizeof(float)));
    static bool attr = false;
    if (!attr) {
        CK(cudaFuncSetAttribute(k_mlp_fwdbwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem(true)));
        attr = true;
    }
    return m;
}

extern "C" void caps_mlp_free(caps_mlp_t *m)
{
    if (!m) return;
    for (float *p : {m->P, m->G, m->M1, m->M2, m->loss, m->X, m->Y, m->out, m->gpart, m->lpart})
        if (p) CK(cudaFree(p));
    delete m;
}

extern "C" void caps_mlp_get_params(caps_mlp_t *m, float *out) { CK(cudaMemcpy(out, m->P, NPARAM * sizeof(float), cudaMemcpyDeviceToHost)); }
extern "C" void caps_mlp_set_params(caps_mlp_t *m, const float *in) { CK(cudaMemcpy(m->P, in, NPARAM * sizeof(float), cudaMemcpyHostToDevice)); }

static double mlp_fwdbwd(caps_mlp_t *m, int n)
{
    int per;
    const int nblk = mlp_blocks(n, &per);
    mlp_reserve_blocks(m, nblk);
    k_mlp_fwdbwd<<<nblk, HN, mlp_smem(true)>>>(m->P, m->X, m->Y, n, per, nullptr, m->gpart, m->lpart);
    COUNT_LAUNCH(1);
    k_mlp_reduce<<<(NPARAM + 255) / 256, 256>>>(m->gpart, m->lpart, nblk, m->G, m->loss, n);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
    float l;
    CK(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    return l;
}

extern "C" double caps_mlp_loss_grad(caps_mlp_t *m, const float *X, const float *y, int n, float *grad)
{
    mlp_reserve(m, n);
    CK(cudaMemcpy(m->X, X, (size_t)n * NIN * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->Y, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
    const double l = mlp_fwdbwd(m, n);
    if (grad) CK(cudaMemcpy(grad, m->G, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return l;
}

extern "C" double caps_mlp_train(caps_mlp_t *m, const float *X, const float *y, int n, int epochs, float lr)
{
    mlp_reserve(m, n);
    CK(cudaMemcpy(m->X, X, (size_t)n * NIN * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(m->Y, y, (size_t)n * sizeof(float), cudaMemcpyHostToDevice));
    double l = 0;
    int per;
    const int nblk = mlp_blocks(n, &per);
    mlp_reserve_blocks(m, nblk);
    for (int e = 0; e < epochs; e++) {
        // full-batch Adam; cosine-decayed step size
        const float lr_e = lr * 0.5f * (1.0f + cosf(3.14159265f * e / epochs)) + 1e-5f;
        k_mlp_fwdbwd<<<nblk, HN, mlp_smem(true)>>>(m->P, m->X, m->Y, n, per, nullptr, m->gpart, m->lpart);
        k_mlp_reduce<<<(NPARAM + 255) / 256, 256>>>(m->gpart, m->lpart, nblk, m->G, m->loss, n);
        k_mlp_adam<<<(NPARAM + 255) / 256, 256>>>(m->P, m->G, m->M1, m->M2, ++m->t, lr_e);
        COUNT_LAUNCH(3);
    }
    CK(cudaGetLastError());
    float lf;
    CK(cudaMemcpy(&lf, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
    l = lf;
    return l;
}

extern "C" void caps_mlp_predict(caps_mlp_t *m, const float *X, int n, float *y)
{
    if (n <= 0) return;
    mlp_reserve(m, n);
    CK(cudaMemcpy(m->X, X, (size_t)n * NIN * sizeof(float), cudaMemcpyHostToDevice));
    int per;
    const int nblk = mlp_blocks(n, &per);
    k_mlp_fwdbwd<<<nblk, HN, mlp_smem(false)>>>(m->P, m->X, nullptr, n, per, m->out, nullptr, nullptr);
    COUNT_LAUNCH(1);
    CK(cudaGetLastError());
    CK(cudaMemcpy(y, m->out, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost));
}

// features of one (geometry, material, xi_, m): the normalisation the network is trained with.
// The frequency enters as 2 xi L / c = 2 xi_ / (1 + R/L), the exponent of the round trip's
// decay e^{-2 xi L / c}, and m as m / sqrt(R/L), the scale on which the m sum of a
// plane-sphere geometry ends; log(R/L) carries what is left.  With these, geometries of
// different R/L put their values on nearly the same surface, so a network trained on small
// R/L serves larger ones.
extern "C" void caps_mlp_features(double RbyL, double xi_, int m, double omegap_eV, double gamma_eV, float *x)
{
    x[0] = (float)(log(RbyL) / 5.0);
    x[1] = (float)(2.0 * xi_ / (1.0 + RbyL) / 8.0);
    x[2] = (float)(m / sqrt(RbyL) / 10.0);
    x[3] = (float)(omegap_eV / 10.0);
    x[4] = (float)(gamma_eV / 0.05);
}
