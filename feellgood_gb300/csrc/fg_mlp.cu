// Learned initial guess for the per-step solve.
//
// A per-node MLP (12 -> 64 -> 64 -> 3, tanh) predicts the velocity v of the coming step
// from local features of the current state:
//   m_i (3), H_eff,i / Ms (3) with H_eff,i = BE_i / A_i (the Galerkin effective field the
//   element kernel assembles: exchange + demag + applied + anisotropy), v_prev,i / V0 (3)
//   and the 1-ring mean of m (3);  V0 = gamma0 * Ms.
// The network predicts the correction of the second-order extrapolation
// v_e = 2 v_prev - v_prev2 (in units of the RMS of that correction over the last solve),
// so the candidate is v_e + scale * MLP(features), projected on the new tangent basis and
// divided by gamma0. The reference's guess (previous v on the new basis,
// src/linear_algebra.cpp:13-24) is the fallback and the referee: the candidate is used only
// when its FP64 initial residual |b - K x| is smaller than the fallback's. The network is
// trained online on (features, solved v) pairs with hand-written kernels: BF16 weights
// (FP32 master copy, Adam), FP32 accumulation, deterministic fixed-order reductions.
#include <cuda_bf16.h>

#include <cmath>
#include <cstdint>
#include <vector>

#include "fg_device.cuh"
#include "fg_internal.h"

namespace fg {

constexpr int NF = 12, NH = 64, NO = 3;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, NPARAM = OFF_B3 + NO;
constexpr int SB = 128;  // samples per training block

struct MlpState {
    float *master = nullptr, *m1 = nullptr, *m2 = nullptr;  // FP32 master weights, Adam moments
    __nv_bfloat16 *w = nullptr;                             // BF16 weights used by the kernels
    float *feat = nullptr;                                  // nn x 12
    float *gpart = nullptr;                                 // per-block gradient partials
    float *lpart = nullptr;                                 // per-block loss partials
    double *xm = nullptr, *Wm = nullptr;                    // candidate guess and its tangent vectors
    double *rpart = nullptr;                                // residual partials
    int *flag = nullptr;                                    // [0] accepted
    double *res2 = nullptr;                                 // [0] |r_mlp|^2, [1] |r_prev|^2
    double *vprev2 = nullptr;                               // v of the step before the previous one
    double *scale = nullptr;                                // RMS of the extrapolation correction
    double *spart = nullptr;                                // its block partials
    int nblk_train = 0, nblk_res = 0;
    bool primed = false;   // vprev2 holds a real previous velocity
    long long t = 0;       // Adam steps
    long long steps = 0;   // training steps done
    double loss = 0.0;
    float *hloss = nullptr;  // pinned
};

__device__ __forceinline__ float bf(const __nv_bfloat16 *w, int k) { return __bfloat162float(w[k]); }

// Features of node i (magnetic nodes; others get zeros).
__device__ __forceinline__ void node_features(int i, const unsigned char *__restrict__ mag,
                                              const double *__restrict__ u0, const double *__restrict__ heff,
                                              const double *__restrict__ vprev, const int *__restrict__ Sptr,
                                              const int *__restrict__ Scol, double inv_ms, double inv_v0,
                                              float (&f)[NF]) {
#pragma unroll
    for (int k = 0; k < NF; k++) f[k] = 0.0f;
    if (!mag[i]) return;
    double mb[3] = {0, 0, 0};
    int deg = 0;
    for (int k = Sptr[i]; k < Sptr[i + 1]; k++) {
        const int j = Scol[k];
        if (j == i) continue;
        mb[0] += u0[3 * j]; mb[1] += u0[3 * j + 1]; mb[2] += u0[3 * j + 2];
        deg++;
    }
    const double id = deg ? 1.0 / deg : 0.0;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        f[c] = (float)u0[3 * i + c];
        f[3 + c] = (float)(heff[3 * i + c] * inv_ms);
        f[6 + c] = (float)(vprev[3 * i + c] * inv_v0);
        f[9 + c] = (float)(mb[c] * id);
    }
}

// Features of every node, for the training of a step that runs no inference.
__global__ void k_features(int nn, const unsigned char *__restrict__ mag, const double *__restrict__ u0,
                           const double *__restrict__ heff, const double *__restrict__ vprev,
                           const int *__restrict__ Sptr, const int *__restrict__ Scol, double inv_ms,
                           double inv_v0, float *__restrict__ feat) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    float f[NF];
    node_features(i, mag, u0, heff, vprev, Sptr, Scol, inv_ms, inv_v0, f);
#pragma unroll
    for (int k = 0; k < NF; k++) feat[(size_t)i * NF + k] = f[k];
}

// tanh on the SFU (tanh.approx.f32, relative error about 2^-11): the guess only has to be
// good, the referee below decides on its FP64 residual.
__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Inference: one thread per node, features formed in place (and stored for the training
// when feat is given), weights staged in shared memory as FP32 (from BF16). Writes the
// candidate x (2 per node) and its tangent vectors W.
__global__ void __launch_bounds__(256) k_mlp_infer(int nn, const unsigned char *__restrict__ mag,
                                                   const double *__restrict__ u0, const double *__restrict__ heff,
                                                   const int *__restrict__ Sptr, const int *__restrict__ Scol,
                                                   double inv_ms, double inv_v0, float *__restrict__ feat,
                                                   const __nv_bfloat16 *__restrict__ w, const double *__restrict__ ep,
                                                   const double *__restrict__ eq, const double *__restrict__ vprev,
                                                   const double *__restrict__ vprev2, const double *__restrict__ scale,
                                                   double *__restrict__ xm, double *__restrict__ Wm) {
    __shared__ __align__(16) float sw[NPARAM];
    for (int k = threadIdx.x; k < NPARAM; k += blockDim.x) sw[k] = bf(w, k);
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    float x[NF];
    node_features(i, mag, u0, heff, vprev, Sptr, Scol, inv_ms, inv_v0, x);
    if (feat)
#pragma unroll
        for (int k = 0; k < NF; k++) feat[(size_t)i * NF + k] = x[k];
    if (!mag[i]) {
        xm[2 * i] = xm[2 * i + 1] = 0.0;
        Wm[3 * i] = Wm[3 * i + 1] = Wm[3 * i + 2] = 0.0;
        return;
    }
    float h1[NH];
#pragma unroll
    for (int j = 0; j < NH; j++) {
        float z = sw[OFF_B1 + j];
#pragma unroll
        for (int k = 0; k < NF; k++) z += sw[OFF_W1 + j * NF + k] * x[k];
        h1[j] = tanh_sfu(z);
    }
    float o0 = sw[OFF_B3], o1 = sw[OFF_B3 + 1], o2 = sw[OFF_B3 + 2];
    for (int j = 0; j < NH; j++) {
        float z = sw[OFF_B2 + j];
#pragma unroll
        for (int k = 0; k < NH; k++) z += sw[OFF_W2 + j * NH + k] * h1[k];
        const float h2 = tanh_sfu(z);
        o0 += sw[OFF_W3 + j] * h2;
        o1 += sw[OFF_W3 + NH + j] * h2;
        o2 += sw[OFF_W3 + 2 * NH + j] * h2;
    }
    // v = 2 v_prev - v_prev2 + scale * o; x = (v . ep, v . eq) / gamma0
    const double sc = scale[0];
    double v[3];
    const double oo[3] = {o0, o1, o2};
#pragma unroll
    for (int c = 0; c < 3; c++) v[c] = 2.0 * vprev[3 * i + c] - vprev2[3 * i + c] + sc * oo[c];
    const double e0 = ep[3 * i], e1 = ep[3 * i + 1], e2 = ep[3 * i + 2];
    const double q0 = eq[3 * i], q1 = eq[3 * i + 1], q2 = eq[3 * i + 2];
    const double xp = (v[0] * e0 + v[1] * e1 + v[2] * e2) / FG_GAMMA0;
    const double xq = (v[0] * q0 + v[1] * q1 + v[2] * q2) / FG_GAMMA0;
    xm[2 * i] = xp;
    xm[2 * i + 1] = xq;
    Wm[3 * i] = xp * e0 + xq * q0;
    Wm[3 * i + 1] = xp * e1 + xq * q1;
    Wm[3 * i + 2] = xp * e2 + xq * q2;
}

// |b - K x|^2 for the candidate and for the fallback guess (FP64, masked), block partials.
__global__ void __launch_bounds__(256) k_resid2(int nn, const int *__restrict__ Sptr, const int *__restrict__ Scol,
                                                const double *__restrict__ Sval, const double *__restrict__ ep,
                                                const double *__restrict__ eq, const double *__restrict__ A,
                                                const double *__restrict__ Dl, const unsigned char *__restrict__ mag,
                                                double c0, const double *__restrict__ b, const double *__restrict__ xa,
                                                const double *Wa, const double *__restrict__ xb, const double *Wb,
                                                double *__restrict__ partial) {
    double acc[2] = {0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        if (!mag[i]) continue;
        double y0, y1;
        apply_row<double>(i, Sptr, Scol, Sval, Wa, ep, eq, A, Dl, c0, xa[2 * i], xa[2 * i + 1], y0, y1);
        acc[0] += (b[2 * i] - y0) * (b[2 * i] - y0) + (b[2 * i + 1] - y1) * (b[2 * i + 1] - y1);
        apply_row<double>(i, Sptr, Scol, Sval, Wb, ep, eq, A, Dl, c0, xb[2 * i], xb[2 * i + 1], y0, y1);
        acc[1] += (b[2 * i] - y0) * (b[2 * i] - y0) + (b[2 * i + 1] - y1) * (b[2 * i + 1] - y1);
    }
    block_store<2>(acc, partial, gridDim.x);
}

// Decision (one block): accept the candidate when its residual is smaller.
__global__ void k_choose(int G, const double *partial, int *flag, double *res2) {
    double s[2];
    grid_sum<2>(partial, G, s);
    if (threadIdx.x == 0) {
        res2[0] = s[0];
        res2[1] = s[1];
        flag[0] = (s[0] < s[1]) ? 1 : 0;
    }
}

__global__ void k_take(int nn, const int *__restrict__ flag, const double *__restrict__ xm,
                       const double *__restrict__ Wm, double *__restrict__ x, double *__restrict__ W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn || !flag[0]) return;
    x[2 * i] = xm[2 * i];
    x[2 * i + 1] = xm[2 * i + 1];
    W[3 * i] = Wm[3 * i];
    W[3 * i + 1] = Wm[3 * i + 1];
    W[3 * i + 2] = Wm[3 * i + 2];
}

__device__ __forceinline__ uint32_t hash32(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return (uint32_t)(x ^ (x >> 31));
}

// One training minibatch: each block takes SB nodes drawn by a counter-based hash,
// runs forward and backward with activations in shared memory and writes its summed
// gradient (per parameter, summed over its samples in a fixed order) and loss.
__global__ void __launch_bounds__(256) k_mlp_grad(int nmag, const int *__restrict__ mag_nodes,
                                                  const float *__restrict__ feat, const double *__restrict__ vtrue,
                                                  const double *__restrict__ vprev, const double *__restrict__ vprev2,
                                                  const double *__restrict__ scale,
                                                  const __nv_bfloat16 *__restrict__ w, uint64_t seed,
                                                  float inv_batch, float *__restrict__ gpart,
                                                  float *__restrict__ lpart, const float *__restrict__ xin,
                                                  const float *__restrict__ yin) {
    extern __shared__ float sm[];
    float *sw = sm;                 // NPARAM
    float *X = sw + NPARAM;         // SB x NF
    float *H1 = X + SB * NF;        // SB x NH
    float *H2 = H1 + SB * NH;       // SB x NH
    float *D3 = H2 + SB * NH;       // SB x NO
    float *Y = D3 + SB * NO;        // SB x NO
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int k = tid; k < NPARAM; k += nt) sw[k] = bf(w, k);
    for (int s = tid; s < SB; s += nt) {
        if (xin) {  // caller-given samples (gradient checks)
            const size_t g = (size_t)blockIdx.x * SB + s;
#pragma unroll
            for (int k = 0; k < NF; k++) X[s * NF + k] = xin[g * NF + k];
#pragma unroll
            for (int c = 0; c < NO; c++) Y[s * NO + c] = yin[g * NO + c];
            continue;
        }
        const int node = mag_nodes[hash32(seed * 1000003ull + (uint64_t)blockIdx.x * SB + s) % (uint32_t)nmag];
#pragma unroll
        for (int k = 0; k < NF; k++) X[s * NF + k] = feat[(size_t)node * NF + k];
        const double isc = 1.0 / scale[0];
#pragma unroll
        for (int c = 0; c < NO; c++) {
            const size_t q = 3 * (size_t)node + c;
            Y[s * NO + c] = (float)((vtrue[q] - (2.0 * vprev[q] - vprev2[q])) * isc);
        }
    }
    __syncthreads();
    for (int e = tid; e < SB * NH; e += nt) {
        const int s = e / NH, j = e % NH;
        float z = sw[OFF_B1 + j];
#pragma unroll
        for (int k = 0; k < NF; k++) z += sw[OFF_W1 + j * NF + k] * X[s * NF + k];
        H1[e] = tanhf(z);
    }
    __syncthreads();
    for (int e = tid; e < SB * NH; e += nt) {
        const int s = e / NH, j = e % NH;
        float z = sw[OFF_B2 + j];
        for (int k = 0; k < NH; k++) z += sw[OFF_W2 + j * NH + k] * H1[s * NH + k];
        H2[e] = tanhf(z);
    }
    __syncthreads();
    float lsum = 0.0f;
    for (int e = tid; e < SB * NO; e += nt) {
        const int s = e / NO, c = e % NO;
        float o = sw[OFF_B3 + c];
        for (int k = 0; k < NH; k++) o += sw[OFF_W3 + c * NH + k] * H2[s * NH + k];
        const float d = o - Y[e];
        D3[e] = 2.0f * d * inv_batch;
        lsum += d * d;
    }
    __syncthreads();
    float *G = gpart + (size_t)blockIdx.x * NPARAM;
    // layer 3 gradients
    for (int p = tid; p < NO * NH + NO; p += nt) {
        float g = 0.0f;
        if (p < NO * NH) {
            const int c = p / NH, k = p % NH;
            for (int s = 0; s < SB; s++) g += D3[s * NO + c] * H2[s * NH + k];
            G[OFF_W3 + p] = g;
        } else {
            const int c = p - NO * NH;
            for (int s = 0; s < SB; s++) g += D3[s * NO + c];
            G[OFF_B3 + c] = g;
        }
    }
    __syncthreads();
    // delta2 = (W3^T d3) * (1 - h2^2), in place of H2
    for (int e = tid; e < SB * NH; e += nt) {
        const int s = e / NH, k = e % NH;
        float d = 0.0f;
#pragma unroll
        for (int c = 0; c < NO; c++) d += sw[OFF_W3 + c * NH + k] * D3[s * NO + c];
        const float h = H2[e];
        H2[e] = d * (1.0f - h * h);
    }
    __syncthreads();
    for (int p = tid; p < NH * NH + NH; p += nt) {
        float g = 0.0f;
        if (p < NH * NH) {
            const int j = p / NH, k = p % NH;
            for (int s = 0; s < SB; s++) g += H2[s * NH + j] * H1[s * NH + k];
            G[OFF_W2 + p] = g;
        } else {
            const int j = p - NH * NH;
            for (int s = 0; s < SB; s++) g += H2[s * NH + j];
            G[OFF_B2 + j] = g;
        }
    }
    __syncthreads();
    // delta1 = (W2^T delta2) * (1 - h1^2), in place of H1
    for (int e = tid; e < SB * NH; e += nt) {
        const int s = e / NH, k = e % NH;
        float d = 0.0f;
        for (int j = 0; j < NH; j++) d += sw[OFF_W2 + j * NH + k] * H2[s * NH + j];
        const float h = H1[e];
        H1[e] = d * (1.0f - h * h);
    }
    __syncthreads();
    for (int p = tid; p < NH * NF + NH; p += nt) {
        float g = 0.0f;
        if (p < NH * NF) {
            const int j = p / NF, k = p % NF;
            for (int s = 0; s < SB; s++) g += H1[s * NH + j] * X[s * NF + k];
            G[OFF_W1 + p] = g;
        } else {
            const int j = p - NH * NF;
            for (int s = 0; s < SB; s++) g += H1[s * NH + j];
            G[OFF_B1 + j] = g;
        }
    }
    // loss partial (fixed-order block reduction)
    __shared__ float red[256];
    red[tid] = lsum;
    __syncthreads();
    if (tid == 0) {
        float t = 0.0f;
        for (int k = 0; k < nt; k++) t += red[k];
        lpart[blockIdx.x] = t;
    }
}

// Sum of |v_new - (2 v_prev - v_prev2)|^2 over magnetic nodes (block partials), then the
// RMS in one block; a zero RMS (first steps, no motion) keeps the previous scale.
__global__ void __launch_bounds__(256) k_corr2(int nn, const unsigned char *__restrict__ mag,
                                               const double *__restrict__ vnew, const double *__restrict__ vprev,
                                               const double *__restrict__ vprev2, double *__restrict__ partial) {
    double acc[1] = {0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nn; i += gridDim.x * blockDim.x) {
        if (!mag[i]) continue;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const double d = vnew[3 * i + c] - (2.0 * vprev[3 * i + c] - vprev2[3 * i + c]);
            acc[0] += d * d;
        }
    }
    block_store<1>(acc, partial, gridDim.x);
}
__global__ void k_scale(int G, const double *partial, int nmag, double *scale) {
    double s[1];
    grid_sum<1>(partial, G, s);
    if (threadIdx.x == 0) {
        const double r = sqrt(s[0] / (3.0 * nmag));
        if (r > 0.0 && isfinite(r)) scale[0] = r;
    }
}

// Sum the block gradients in block order and apply Adam; refresh the BF16 weights.
__global__ void k_adam(int nblk, const float *__restrict__ gpart, float *__restrict__ master, float *__restrict__ m1,
                       float *__restrict__ m2, __nv_bfloat16 *__restrict__ w, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    float g = 0.0f;
    for (int b = 0; b < nblk; b++) g += gpart[(size_t)b * NPARAM + p];
    const float a = b1 * m1[p] + (1.0f - b1) * g;
    const float v = b2 * m2[p] + (1.0f - b2) * g * g;
    m1[p] = a;
    m2[p] = v;
    const float upd = lr * (a / bc1) / (sqrtf(v / bc2) + eps);
    const float nw = master[p] - upd;
    master[p] = nw;
    w[p] = __float2bfloat16(nw);
}

// ---------------------------------------------------------------------------------
// host side

static inline int nb(long n, int b) { return (int)((n + b - 1) / b); }

int mlp_create(Ctx &c) {
    MlpState *s = new MlpState();
    c.mlp = s;
    const int batch = c.opts.mlp_batch > 0 ? c.opts.mlp_batch : 16384;
    s->nblk_train = std::max(1, batch / SB);
    s->nblk_res = std::max(1, std::min(2 * c.nsm, nb(c.nn, 256)));
    // Xavier-uniform initialisation from a fixed counter-based stream
    std::vector<float> w0(NPARAM, 0.0f);
    uint64_t st = 0x5eed1234abcdull;
    auto uni = [&]() {
        st += 0x9e3779b97f4a7c15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int fan_out, int fan_in) {
        const double a = std::sqrt(6.0 / (fan_in + fan_out));
        for (int k = 0; k < fan_out * fan_in; k++) w0[off + k] = (float)((2 * uni() - 1) * a);
    };
    fill(OFF_W1, NH, NF);
    fill(OFF_W2, NH, NH);
    fill(OFF_W3, NO, NH);
    std::vector<__nv_bfloat16> wb(NPARAM);
    for (int k = 0; k < NPARAM; k++) wb[k] = __float2bfloat16(w0[k]);
    if (cudaMalloc(&s->master, NPARAM * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->m1, NPARAM * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->m2, NPARAM * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->w, NPARAM * sizeof(__nv_bfloat16)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->feat, (size_t)c.nn * NF * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->gpart, (size_t)s->nblk_train * NPARAM * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->lpart, (size_t)s->nblk_train * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->xm, 2 * (size_t)c.nn * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->Wm, 3 * (size_t)c.nn * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->rpart, 2 * (size_t)s->nblk_res * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->flag, sizeof(int)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->res2, 2 * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMallocHost(&s->hloss, (size_t)s->nblk_train * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->vprev2, 3 * (size_t)c.nn * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->scale, sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->spart, (size_t)s->nblk_res * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    {
        const double one = FG_GAMMA0 * c.ms_ref * 1e-3;
        cudaMemcpy(s->scale, &one, sizeof(double), cudaMemcpyHostToDevice);
        cudaMemset(s->vprev2, 0, 3 * (size_t)c.nn * sizeof(double));
    }
    s->primed = false;
    cudaMemcpy(s->master, w0.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(s->w, wb.data(), NPARAM * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
    cudaMemset(s->m1, 0, NPARAM * sizeof(float));
    cudaMemset(s->m2, 0, NPARAM * sizeof(float));
    cudaMemset(s->flag, 0, sizeof(int));
    const int smem = (NPARAM + SB * NF + 2 * SB * NH + 2 * SB * NO) * (int)sizeof(float);
    if (cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
        return FG_ECUDA;
    return cudaGetLastError() == cudaSuccess ? FG_OK : FG_ECUDA;
}

void mlp_free(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s) return;
    void *p[] = {s->master, s->m1, s->m2, s->w, s->feat, s->gpart, s->lpart, s->xm, s->Wm, s->rpart, s->flag,
                 s->res2, s->vprev2, s->scale, s->spart};
    for (void *q : p)
        if (q) cudaFree(q);
    if (s->hloss) cudaFreeHost(s->hloss);
    delete s;
    c.mlp = nullptr;
}

static double v0_scale(const Ctx &c) { return FG_GAMMA0 * c.ms_ref; }

// With use != 0 the candidate guess and the decision against the fallback guess already in
// c.x (writes c.x / c.W when the candidate wins); the features of the current state are
// stored for the training when train is set (formed inside the inference when it runs).
cudaError_t mlp_before_solve(Ctx &c, double c0, bool use, bool train) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!use) {
        if (train) {
            k_features<<<nb(c.nn, 256), 256, 0, c.stream>>>(c.nn, c.mag, c.u[0], c.heff, c.v[1], c.Sptr, c.Scol,
                                                              1.0 / c.ms_ref, 1.0 / v0_scale(c), s->feat);
            c.launches += 1;
        }
        return cudaGetLastError();
    }
    if (!s->primed) {  // no history yet: the extrapolation degenerates to v_prev
        cudaMemcpyAsync(s->vprev2, c.v[0], 3 * (size_t)c.nn * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
        s->primed = true;
    }
    k_mlp_infer<<<nb(c.nn, 256), 256, 0, c.stream>>>(c.nn, c.mag, c.u[0], c.heff, c.Sptr, c.Scol, 1.0 / c.ms_ref,
                                                      1.0 / v0_scale(c), train ? s->feat : nullptr, s->w, c.ep, c.eq,
                                                      c.v[0], s->vprev2, s->scale, s->xm, s->Wm);
    k_resid2<<<s->nblk_res, 256, 0, c.stream>>>(c.nn, c.Sptr, c.Scol, c.Sval, c.ep, c.eq, c.A, c.Dl, c.mag, c0,
                                                c.rhs, s->xm, s->Wm, c.x, c.W, s->rpart);
    k_choose<<<1, 32, 0, c.stream>>>(s->nblk_res, s->rpart, s->flag, s->res2);
    k_take<<<nb(c.nn, 256), 256, 0, c.stream>>>(c.nn, s->flag, s->xm, s->Wm, c.x, c.W);
    c.launches += 4;
    return cudaGetLastError();
}

// One Adam step on a minibatch of (features at the start of the step, solved v).
cudaError_t mlp_train(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    const int smem = (NPARAM + SB * NF + 2 * SB * NH + 2 * SB * NO) * (int)sizeof(float);
    const float inv_batch = 1.0f / (float)(s->nblk_train * SB * NO);
    if (!s->primed) {
        cudaMemcpyAsync(s->vprev2, c.v[0], 3 * (size_t)c.nn * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
        s->primed = true;
    }
    k_corr2<<<s->nblk_res, 256, 0, c.stream>>>(c.nn, c.mag, c.v[1], c.v[0], s->vprev2, s->spart);
    k_scale<<<1, 32, 0, c.stream>>>(s->nblk_res, s->spart, c.n_mag_nodes, s->scale);
    k_mlp_grad<<<s->nblk_train, 256, smem, c.stream>>>(c.n_mag_nodes, c.mag_nodes, s->feat, c.v[1], c.v[0],
                                                        s->vprev2, s->scale, s->w, (uint64_t)s->steps + 1, inv_batch,
                                                        s->gpart, s->lpart, nullptr, nullptr);
    c.launches += 2;
    s->t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float lr = c.opts.mlp_lr > 0 ? (float)c.opts.mlp_lr : 1e-3f;
    k_adam<<<nb(NPARAM, 256), 256, 0, c.stream>>>(s->nblk_train, s->gpart, s->master, s->m1, s->m2, s->w, lr, b1, b2,
                                                   1e-8f, 1.0f - powf(b1, (float)s->t), 1.0f - powf(b2, (float)s->t));
    cudaMemcpyAsync(s->hloss, s->lpart, s->nblk_train * sizeof(float), cudaMemcpyDeviceToHost, c.stream);
    s->steps++;
    c.launches += 2;
    return cudaGetLastError();
}

void mlp_after_sync(Ctx &c, int *accepted, double *res0_mlp, double *res0_prev, double *loss) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s) return;
    double l = 0.0;
    for (int b = 0; b < s->nblk_train; b++) l += s->hloss[b];
    s->loss = l / (s->nblk_train * SB * NO);
    if (loss) *loss = s->loss;
    if (accepted) {
        int f = 0;
        double r2[2] = {0, 0};
        cudaMemcpy(&f, s->flag, sizeof(int), cudaMemcpyDeviceToHost);
        cudaMemcpy(r2, s->res2, 2 * sizeof(double), cudaMemcpyDeviceToHost);
        *accepted = f;
        *res0_mlp = std::sqrt(r2[0]);
        *res0_prev = std::sqrt(r2[1]);
    }
}

// Gradient of the mean-squared loss for caller-given samples (nblk*SB of them, device
// arrays), summed over the blocks on the host; returns the BF16 weights used as FP32.
int mlp_debug_grad(Ctx &c, int nsamples, const float *hx, const float *hy, float *w_out, float *g_out, float *loss) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s || nsamples <= 0 || nsamples % SB) return FG_EINVAL;
    const int nblk = nsamples / SB;
    float *dx = nullptr, *dy = nullptr, *dg = nullptr, *dl = nullptr;
    cudaMalloc(&dx, sizeof(float) * nsamples * NF);
    cudaMalloc(&dy, sizeof(float) * nsamples * NO);
    cudaMalloc(&dg, sizeof(float) * nblk * NPARAM);
    cudaMalloc(&dl, sizeof(float) * nblk);
    cudaMemcpy(dx, hx, sizeof(float) * nsamples * NF, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, hy, sizeof(float) * nsamples * NO, cudaMemcpyHostToDevice);
    const int smem = (NPARAM + SB * NF + 2 * SB * NH + 2 * SB * NO) * (int)sizeof(float);
    k_mlp_grad<<<nblk, 256, smem, c.stream>>>(1, c.mag_nodes, s->feat, c.v[1], c.v[0], s->vprev2, s->scale, s->w, 1,
                                              1.0f / (nsamples * NO), dg, dl, dx, dy);
    std::vector<float> g((size_t)nblk * NPARAM), l(nblk);
    std::vector<__nv_bfloat16> wb(NPARAM);
    cudaStreamSynchronize(c.stream);
    cudaMemcpy(g.data(), dg, sizeof(float) * g.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(l.data(), dl, sizeof(float) * nblk, cudaMemcpyDeviceToHost);
    cudaMemcpy(wb.data(), s->w, sizeof(__nv_bfloat16) * NPARAM, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    cudaFree(dg);
    cudaFree(dl);
    for (int p = 0; p < NPARAM; p++) {
        float t = 0.0f;
        for (int b = 0; b < nblk; b++) t += g[(size_t)b * NPARAM + p];
        g_out[p] = t;
        w_out[p] = __bfloat162float(wb[p]);
    }
    float lt = 0.0f;
    for (int b = 0; b < nblk; b++) lt += l[b];
    *loss = lt / (nsamples * NO);
    return cudaGetLastError() == cudaSuccess ? FG_OK : FG_ECUDA;
}

int mlp_nparam() { return NPARAM; }

// Fem::evolution is about to overwrite v_prev: keep it as v_prev2 for the extrapolation.
cudaError_t mlp_before_evolution(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s) return cudaSuccess;
    s->primed = true;
    return cudaMemcpyAsync(s->vprev2, c.v[0], 3 * (size_t)c.nn * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
}

long long mlp_steps(const Ctx &c) {
    const MlpState *s = static_cast<const MlpState *>(c.mlp);
    return s ? s->steps : 0;
}

double mlp_loss(const Ctx &c) {
    const MlpState *s = static_cast<const MlpState *>(c.mlp);
    return s ? s->loss : 0.0;
}

}  // namespace fg
