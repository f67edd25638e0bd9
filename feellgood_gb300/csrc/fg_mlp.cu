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
// divided by gamma0; the correction is averaged over the node and its magnetic neighbours
// first (the network's per-node errors are rough, and rough initial errors are what BiCGSTAB
// removes slowest). The reference's guess (previous v on the new basis,
// src/linear_algebra.cpp:13-24) is the fallback and the referee: on the FP32 + refinement
// path the solver forms the candidate in its first phase and, in its first FP64 residual
// pass, takes the blend of the two guesses with the smallest residual norm; on the FP64 path
// separate kernels keep the candidate only when its FP64 initial residual is smaller. The
// node kernel forms each node's own features; the inference adds the 1-ring mean of m from
// the neighbours' rows (FP32 sums, so that the FP64 node kernel gathers nothing more) and
// runs the network's three GEMMs on the tensor cores (BF16 operands, FP32 accumulation in
// tensor memory). The network is trained online
// on (features, solved v)
// pairs with hand-written kernels: BF16 weights (FP32 master copy, Adam), FP32
// accumulation, deterministic fixed-order reductions.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "fg_device.cuh"
#include "fg_internal.h"
#include "fg_tcgen05.cuh"

namespace fg {

constexpr int NF = 12, NH = 64, NO = 3;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NF, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NO * NH, NPARAM = OFF_B3 + NO;
constexpr int SB = 128;  // samples per training block

// The per-step results read back at the step's one host synchronisation (one copy), for
// each of the nflag systems (the samples of a batch): one block of
//   int tc_err (FG_ETIMEDOUT from a tensor-core wait), int pad,
//   int flag[nflag] (the candidate guess was taken: blend weight > 0), padded to 8 bytes,
//   double res2[2 nflag] (|r_cand|^2, |r_fallback|^2 of the first FP64 residual).
struct MlpFlagsLayout {
    size_t flag_off, res2_off, bytes;
    explicit MlpFlagsLayout(int n) {
        flag_off = 8;
        res2_off = flag_off + 8 * (((size_t)n + 1) / 2);
        bytes = res2_off + 16 * (size_t)n;
    }
};

struct MlpState {
    float *master = nullptr, *m1 = nullptr, *m2 = nullptr;  // FP32 master weights, Adam moments
    __nv_bfloat16 *w = nullptr;                             // BF16 weights used by the kernels
    unsigned char *wimg = nullptr;                          // their image for the inference
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
    int *tc_err = nullptr;                                  // FG_ETIMEDOUT from a tensor-core wait
    double *rc = nullptr;                                   // the candidate's residual (judged in the solver)
    float *out = nullptr;                                   // the network's outputs [nn][3]
    int nblk_train = 0, nblk_res = 0;
    bool primed = false;   // vprev2 holds a real previous velocity
    bool timed_out = false;  // a tensor-core wait of the last inference expired
    long long t = 0;       // Adam steps
    long long steps = 0;   // training steps done
    double loss = 0.0;
    float *hloss = nullptr;  // pinned
    unsigned char *dflags = nullptr, *hflags = nullptr;  // device, pinned copy (flag, res2, tc_err point into dflags)
    int nflag = 1;                                         // systems: 1, or the samples of a batch
};

__device__ __forceinline__ float bf(const __nv_bfloat16 *w, int k) { return __bfloat162float(w[k]); }

// tanh on the SFU (tanh.approx.f32, relative error about 2^-11): the guess only has to be
// good, the referee below decides on its FP64 residual.
__device__ __forceinline__ float tanh_sfu(float x) {
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// ---- forward pass on the tensor cores --------------------------------------------
// A tile of 128 nodes is the M = 128 side of three tcgen05.mma kind::f16 GEMMs with BF16
// operands and FP32 accumulators in tensor memory:
//   layer 1  D1[128 x 64] = X[128 x 16] W1^T      (12 features padded to K = 16), 1 MMA
//   layer 2  D2[128 x 64] = H1[128 x 64] W2^T     4 MMAs of K = 16
//   layer 3  D3[128 x 16] = H2[128 x 64] W3^T     (3 outputs padded to N = 16), 4 MMAs
// Thread t of the CTA owns node t of the tile: it reads the node's features (forming the
// 1-ring mean of m from its neighbours' rows in FP32), writes its BF16
// row of X, drains its row of D1 / D2 with tcgen05.ld (TMEM lane t), adds the bias, applies
// tanh and writes its BF16 row of H for the next layer; one thread issues the MMAs.
// Operands sit in shared memory in the no-swizzle K-major layout of 8-row x 16-byte core
// matrices (LBO 128 bytes along K; SBO = bytes of one 8-row group). TMEM: 64 columns, D1,
// D2 and D3 in turn (each is drained before the next layer's MMAs are issued), so that six
// CTAs (the shared-memory limit) fit on an SM.
constexpr int TM = 128;        // nodes per tile
constexpr int K1 = 16;         // layer-1 K (features padded)
constexpr int NO3 = 16;        // layer-3 N (outputs padded)
constexpr uint32_t TC_LBO = 128;
constexpr uint32_t SBO_K16 = 2 * TC_LBO, SBO_K64 = 8 * TC_LBO;
constexpr int A1_OFF = 0, A1_BYTES = TM * K1 * 2;                   // 4 KB
constexpr int A2_OFF = A1_OFF + A1_BYTES, A2_BYTES = TM * NH * 2;   // 16 KB: H1, then H2
constexpr int B1_OFF = A2_OFF + A2_BYTES, B1_BYTES = NH * K1 * 2;   // 2 KB
constexpr int B2_OFF = B1_OFF + B1_BYTES, B2_BYTES = NH * NH * 2;   // 8 KB
constexpr int B3_OFF = B2_OFF + B2_BYTES, B3_BYTES = NO3 * NH * 2;  // 2 KB
constexpr int BIAS_OFF = B3_OFF + B3_BYTES;                         // b1, b2, b3 as FP32
constexpr int TC_SMEM = BIAS_OFF + (NH + NH + NO3) * 4 + 1024;      // + alignment slack
constexpr int TC_TMEM_COLS = 64;

// Byte offset of element (row, k) in a K-major image whose 8-row groups are sbo bytes apart.
__device__ __forceinline__ int kmaj(int row, int k, uint32_t sbo) {
    return (row >> 3) * (int)sbo + (k >> 3) * (int)TC_LBO + (row & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t *>(&h);
}

// Writes the 8 BF16 values v[0..7] (K = k0..k0+7 of one row) as one 16-byte store.
__device__ __forceinline__ void store8(unsigned char *img, int row, int k0, uint32_t sbo, const float *v) {
    uint4 q;
    q.x = pack_bf16(v[0], v[1]);
    q.y = pack_bf16(v[2], v[3]);
    q.z = pack_bf16(v[4], v[5]);
    q.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4 *>(img + kmaj(row, k0, sbo)) = q;
}

// The forward pass's weights as the kernel's shared memory holds them: B1 | B2 | B3 (BF16,
// K-major core-matrix images, zero padding) | b1, b2, b3 (FP32 values of the BF16 biases).
// Written once at creation and by every Adam update (k_adam), so that each CTA of the
// inference copies one contiguous 12.6 KB block with 16-byte loads instead of gathering and
// re-laying out the parameters itself.
constexpr int IMG_BYTES = BIAS_OFF - B1_OFF + (NH + NH + NO3) * 4;
static_assert(IMG_BYTES % 16 == 0 && B1_OFF % 16 == 0, "16-byte copies of the weight image");

// Byte offset of parameter p in the weight image; *bias: stored as FP32 (else BF16).
__device__ __forceinline__ int img_offset(int p, bool *bias) {
    *bias = false;
    if (p < OFF_B1) return kmaj((p - OFF_W1) / NF, (p - OFF_W1) % NF, SBO_K16);
    if (p < OFF_W2) { *bias = true; return BIAS_OFF - B1_OFF + 4 * (p - OFF_B1); }
    if (p < OFF_B2) return B2_OFF - B1_OFF + kmaj((p - OFF_W2) / NH, (p - OFF_W2) % NH, SBO_K64);
    if (p < OFF_W3) { *bias = true; return BIAS_OFF - B1_OFF + 4 * (NH + p - OFF_B2); }
    if (p < OFF_B3) return B3_OFF - B1_OFF + kmaj((p - OFF_W3) / NH, (p - OFF_W3) % NH, SBO_K64);
    *bias = true;
    return BIAS_OFF - B1_OFF + 4 * (2 * NH + p - OFF_B3);
}

__device__ __forceinline__ void img_store(unsigned char *img, int p, __nv_bfloat16 wb) {
    bool bias;
    const int o = img_offset(p, &bias);
    if (bias) *reinterpret_cast<float *>(img + o) = __bfloat162float(wb);
    else *reinterpret_cast<__nv_bfloat16 *>(img + o) = wb;
}

// The image of the BF16 weights w (the padding must be zero already).
__global__ void k_mlp_pack(const __nv_bfloat16 *__restrict__ w, unsigned char *__restrict__ img) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < NPARAM) img_store(img, p, w[p]);
}

struct MlpTcArgs {
    int nn;                      // feature rows
    const uint4 *wimg;           // the weight image (IMG_BYTES)
    float *xin;                  // feature rows [nn][12]
    // with Sptr set, features 9..11 of a row are formed here: the mean of features 0..2 (m)
    // over the node's neighbours in the stiffness pattern (written back when ring_out is set)
    const int *Sptr, *Scol;
    int ring_out;
    float *yout;                 // the network's outputs [nn][3]
    int *err;                    // FG_ETIMEDOUT after an expired wait
};

// Features 9..11 of node i: the mean of m (features 0..2, FP32) over i's neighbours in the
// stiffness pattern (the nodes sharing a magnetic tetrahedron with i; zero rows elsewhere).
__device__ __forceinline__ void ring_mean(int i, const int *__restrict__ Sptr, const int *__restrict__ Scol,
                                          const float *feat, float *mean) {
    float m0 = 0.f, m1 = 0.f, m2 = 0.f;
    int deg = 0;
    const int k0 = Sptr[i], k1 = Sptr[i + 1];
#pragma unroll 4
    for (int k = k0; k < k1; k++) {
        const int j = Scol[k];
        if (j == i) continue;
        // m_j and one more feature as one 16-byte load (rows are 48 bytes)
        const float4 f = *reinterpret_cast<const float4 *>(feat + NF * (size_t)j);
        m0 += f.x;
        m1 += f.y;
        m2 += f.z;
        deg++;
    }
    const float id = deg ? 1.0f / (float)deg : 0.0f;
    mean[0] = m0 * id;
    mean[1] = m1 * id;
    mean[2] = m2 * id;
}

// Features 9..11 of every node (steps that train the network without using it).
__global__ void k_feat_ring(int nn, const int *__restrict__ Sptr, const int *__restrict__ Scol, float *feat) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    float m[3];
    ring_mean(i, Sptr, Scol, feat, m);
#pragma unroll
    for (int c = 0; c < 3; c++) feat[NF * (size_t)i + 9 + c] = m[c];
}

// Drains 16 TMEM columns of this thread's lane (row) into v[0..15].
__device__ __forceinline__ void drain16(uint32_t taddr, float *v) {
    uint32_t r[16];
    tc::tmem_ld16(taddr, r);
    tc::tmem_wait_ld();
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

__global__ void __launch_bounds__(TM) k_mlp_infer_tc(MlpTcArgs a) {
    using namespace tc;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *A1 = sm + A1_OFF, *A2 = sm + A2_OFF, *B1 = sm + B1_OFF, *B2 = sm + B2_OFF, *B3 = sm + B3_OFF;
    float *bias = reinterpret_cast<float *>(sm + BIAS_OFF);  // b1 [64], b2 [64], b3 [16]
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int bail;
    const int tid = threadIdx.x, warp = tid >> 5;
    // weights and biases: one contiguous copy of the prepared image
    {
        uint4 *dst = reinterpret_cast<uint4 *>(B1);
#pragma unroll 4
        for (int e = tid; e < IMG_BYTES / 16; e += TM) dst[e] = __ldg(a.wimg + e);
    }
    if (tid == 0) {
        mbar_init(&bar, 1);
        bail = 0;
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(&tmem_base, TC_TMEM_COLS);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
    const uint32_t sA1 = smem_u32(A1), sA2 = smem_u32(A2), sB1 = smem_u32(B1), sB2 = smem_u32(B2),
                   sB3 = smem_u32(B3);
    uint32_t parity = 0;
    // all threads reach this after their shared-memory writes: the issuer's MMAs see them
    auto issue_and_wait = [&](int layer) -> bool {
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            if (layer == 1) {
                mma_bf16(tmem, sdesc_kmajor(sA1, TC_LBO, SBO_K16), sdesc_kmajor(sB1, TC_LBO, SBO_K16),
                         idesc_bf16(TM, NH), 0u);
            } else {
                const uint32_t d = tmem;
                const uint32_t sB = layer == 2 ? sB2 : sB3;
                const uint32_t id = idesc_bf16(TM, layer == 2 ? NH : NO3);
#pragma unroll
                for (int k = 0; k < NH / 16; k++)
                    mma_bf16(d, sdesc_kmajor(sA2 + 256 * k, TC_LBO, SBO_K64), sdesc_kmajor(sB + 256 * k, TC_LBO, SBO_K64),
                             id, k > 0 ? 1u : 0u);
            }
            mma_commit(&bar);
        }
        const bool ok = mbar_wait(&bar, parity, a.err, &bail);
        if (!ok && tid == 0) mbar_drain(&bar, parity);  // the MMAs still own TMEM and the operands
        parity ^= 1u;
        const bool all = __syncthreads_and(ok) != 0;
        tc_fence_after();
        return all;
    };
    const int ntiles = (a.nn + TM - 1) / TM;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int i = tile * TM + tid;
        const bool live = i < a.nn;
        float x[NF];
        {
            // the row as three 16-byte loads (features 9..11 are replaced below when Sptr is set)
            const float4 *row = reinterpret_cast<const float4 *>(a.xin + (size_t)(live ? i : 0) * NF);
            const float4 r0 = row[0], r1 = row[1], r2 = row[2];
            const float v[NF] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
#pragma unroll
            for (int k = 0; k < NF; k++) x[k] = live ? v[k] : 0.f;
        }
        if (a.Sptr && live) {
            ring_mean(i, a.Sptr, a.Scol, a.xin, x + 9);
            if (a.ring_out) {
#pragma unroll
                for (int c = 0; c < 3; c++) a.xin[(size_t)i * NF + 9 + c] = x[9 + c];
            }
        }
        {
            const float x2[8] = {x[8], x[9], x[10], x[11], 0.f, 0.f, 0.f, 0.f};
            store8(A1, tid, 0, SBO_K16, x);
            store8(A1, tid, 8, SBO_K16, x2);
        }
        if (!issue_and_wait(1)) break;
        // H1 = tanh(D1 + b1) -> A2
#pragma unroll
        for (int c = 0; c < NH / 16; c++) {
            float v[16];
            drain16(lane_addr + 16 * c, v);
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] = tanh_sfu(v[k] + bias[16 * c + k]);
            store8(A2, tid, 16 * c, SBO_K64, v);
            store8(A2, tid, 16 * c + 8, SBO_K64, v + 8);
        }
        if (!issue_and_wait(2)) break;
        // H2 = tanh(D2 + b2) -> A2 (layer 2's MMAs have completed: A2 is free)
#pragma unroll
        for (int c = 0; c < NH / 16; c++) {
            float v[16];
            drain16(lane_addr + 16 * c, v);
#pragma unroll
            for (int k = 0; k < 16; k++) v[k] = tanh_sfu(v[k] + bias[NH + 16 * c + k]);
            store8(A2, tid, 16 * c, SBO_K64, v);
            store8(A2, tid, 16 * c + 8, SBO_K64, v + 8);
        }
        if (!issue_and_wait(3)) break;
        float o[16];
        drain16(lane_addr, o);
        if (live) {
#pragma unroll
            for (int c = 0; c < NO; c++) a.yout[NO * (size_t)i + c] = o[c] + bias[2 * NH + c];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, TC_TMEM_COLS);
    }
}

// The candidate guess from the network's outputs: the correction of the extrapolation,
// averaged over the node and its magnetic neighbours (a low-pass filter: the network's
// per-node errors are uncorrelated from node to node, and rough initial errors are what
// BiCGSTAB removes slowest), v = 2 v_prev - v_prev2 + scale * mean(o), projected on the new
// tangent basis: x = (v . ep, v . eq) / gamma0, and its tangent vectors W.
__global__ void __launch_bounds__(256) k_mlp_candidate(int nn, const unsigned char *__restrict__ mag,
                                                       const int *__restrict__ Sptr, const int *__restrict__ Scol,
                                                       const float *__restrict__ o, const double *__restrict__ vprev,
                                                       const double *__restrict__ vprev2,
                                                       const double *__restrict__ scale, const double *__restrict__ ep,
                                                       const double *__restrict__ eq, double *__restrict__ xm,
                                                       double *__restrict__ Wm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    if (!mag[i]) {
        xm[2 * i] = xm[2 * i + 1] = 0.0;
        Wm[3 * i] = Wm[3 * i + 1] = Wm[3 * i + 2] = 0.0;
        return;
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f;
    int cnt = 0;
    for (int k = Sptr[i]; k < Sptr[i + 1]; k++) {  // the row holds the node itself and its neighbours
        const int j = Scol[k];
        if (!mag[j]) continue;
        s0 += o[3 * (size_t)j];
        s1 += o[3 * (size_t)j + 1];
        s2 += o[3 * (size_t)j + 2];
        cnt++;
    }
    const double sc = scale[0] / (double)max(cnt, 1);
    const double oo[3] = {s0, s1, s2};
    double v[3];
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

static cudaError_t launch_mlp_infer_tc(Ctx &c, const MlpTcArgs &a) {
    static bool attr_set = false;  // per process; the attribute is a property of the function
    if (!attr_set) {
        const cudaError_t e = cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    const int ntiles = (a.nn + TM - 1) / TM;
    const int grid = std::max(1, std::min(ntiles, 6 * c.nsm));  // 6 CTAs of 64 TMEM columns per SM
    k_mlp_infer_tc<<<grid, TM, TC_SMEM, c.stream>>>(a);
    return cudaGetLastError();
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

// One training minibatch tile on the tensor cores: each CTA takes SB = 128 nodes drawn by a
// counter-based hash (thread s owns sample s), runs the forward pass of the inference
// kernel (BF16 operand images X, H1, H2 kept in shared memory) and the backward pass, and
// writes its summed gradient (per parameter, a fixed summation order) and loss:
//   d3 = 2 (o - y) / (batch x 3)                                        FP32, per sample
//   [gW3 | gb3] [3 x 65]  = d3^T [H2 | 1]         M = 128 (rows 0..2 used), N = 80, K = 128 samples
//   delta2 = (d3 W3) (1 - h2^2)                                         CUDA cores (K = 3)
//   [gW2 | gb2] [64 x 65] = delta2^T [H1 | 1]     M = 128 (rows 0..63 used), N = 80, K = 128
//   delta1 = (delta2 W2) (1 - h1^2)               M = 128 samples, N = 64, K = 64
//   [gW1 | gb1] [64 x 13] = delta1^T [X | 1]      M = 128 (rows 0..63 used), N = 16, K = 128
// The transposed operands (delta^T with samples along K, and [H | 1]^T, [X | 1]^T) are
// written column by column, each thread its own sample; the ones rows make the bias
// gradients come out of the same MMAs. Rows of D that are not read never need clearing:
// an output row depends on its own row of A only. BF16 operands, FP32 accumulation in TMEM.
constexpr uint32_t SBO_K128 = 16 * TC_LBO;
constexpr int NB80 = 80;  // N of the [H | 1] operands (65 used)
constexpr int G_A1 = 0;                          // X [128 x 16]
constexpr int G_H1 = G_A1 + TM * K1 * 2;         // H1 [128 x 64]
constexpr int G_H2 = G_H1 + TM * NH * 2;         // H2 [128 x 64]
constexpr int G_D2 = G_H2 + TM * NH * 2;         // delta2 [128 x 64]
constexpr int G_B1 = G_D2 + TM * NH * 2;         // W1 [64 x 16]
constexpr int G_B2 = G_B1 + NH * K1 * 2;         // W2 [64 x 64]
constexpr int G_B3 = G_B2 + NH * NH * 2;         // W3 [16 x 64]
constexpr int G_B2T = G_B3 + NO3 * NH * 2;       // W2^T [64 x 64]
constexpr int G_AT = G_B2T + NH * NH * 2;        // delta^T [128 x 128 samples]
constexpr int G_H1T = G_AT + 128 * SB * 2;       // [H1 | 1]^T [80 x 128 samples]
constexpr int G_H2T = G_H1T + NB80 * SB * 2;     // [H2 | 1]^T [80 x 128 samples]
constexpr int G_XT = G_H2T + NB80 * SB * 2;      // [X | 1]^T [16 x 128 samples]
constexpr int G_F32 = G_XT + K1 * SB * 2;        // b1, b2, b3 (16), W3 [3][64] as FP32, loss [128]
constexpr int GRAD_SMEM = G_F32 + (NH + NH + NO3 + NO * NH + SB) * 4 + 1024;
constexpr int GRAD_TMEM_COLS = 256;

__device__ __forceinline__ void store_bf16(unsigned char *img, int row, int k, uint32_t sbo, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(img + kmaj(row, k, sbo)) = __float2bfloat16(v);
}
__device__ __forceinline__ float load_bf16(const unsigned char *img, int row, int k, uint32_t sbo) {
    return __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(img + kmaj(row, k, sbo)));
}

__global__ void __launch_bounds__(SB) k_mlp_grad_tc(int nmag, const int *__restrict__ mag_nodes,
                                                    const float *__restrict__ feat, const double *__restrict__ vtrue,
                                                    const double *__restrict__ vprev,
                                                    const double *__restrict__ vprev2,
                                                    const double *__restrict__ scale,
                                                    const __nv_bfloat16 *__restrict__ w, uint64_t seed,
                                                    float inv_batch, float *__restrict__ gpart,
                                                    float *__restrict__ lpart, const float *__restrict__ xin,
                                                    const float *__restrict__ yin, int *err) {
    using namespace tc;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *A1 = sm + G_A1, *H1 = sm + G_H1, *H2 = sm + G_H2, *D2 = sm + G_D2, *B1 = sm + G_B1,
                  *B2 = sm + G_B2, *B3 = sm + G_B3, *B2T = sm + G_B2T, *AT = sm + G_AT, *H1T = sm + G_H1T,
                  *H2T = sm + G_H2T, *XT = sm + G_XT;
    float *bias = reinterpret_cast<float *>(sm + G_F32);  // b1 [64], b2 [64], b3 [16]
    float *w3f = bias + NH + NH + NO3;                    // W3 [3][64]
    float *red = w3f + NO * NH;                           // loss per sample
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int bail;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int e = tid; e < NH * K1; e += SB) {
        const int j = e / K1, k = e % K1;
        *reinterpret_cast<__nv_bfloat16 *>(B1 + kmaj(j, k, SBO_K16)) =
            k < NF ? w[OFF_W1 + j * NF + k] : __float2bfloat16(0.f);
    }
    for (int e = tid; e < NH * NH; e += SB) {
        const int j = e / NH, k = e % NH;
        const __nv_bfloat16 v = w[OFF_W2 + j * NH + k];
        *reinterpret_cast<__nv_bfloat16 *>(B2 + kmaj(j, k, SBO_K64)) = v;   // rows j (outputs), K = k
        *reinterpret_cast<__nv_bfloat16 *>(B2T + kmaj(k, j, SBO_K64)) = v;  // rows k (inputs), K = j
    }
    for (int e = tid; e < NO3 * NH; e += SB) {
        const int j = e / NH, k = e % NH;
        *reinterpret_cast<__nv_bfloat16 *>(B3 + kmaj(j, k, SBO_K64)) =
            j < NO ? w[OFF_W3 + j * NH + k] : __float2bfloat16(0.f);
    }
    for (int e = tid; e < NH + NH + NO3; e += SB)
        bias[e] = e < NH ? bf(w, OFF_B1 + e) : e < 2 * NH ? bf(w, OFF_B2 + e - NH)
                                                           : (e - 2 * NH < NO ? bf(w, OFF_B3 + e - 2 * NH) : 0.f);
    for (int e = tid; e < NO * NH; e += SB) w3f[e] = bf(w, OFF_W3 + e);
    if (tid == 0) {
        mbar_init(&bar, 1);
        bail = 0;
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(&tmem_base, GRAD_TMEM_COLS);
    // this thread's sample: features and target
    float x[NF], y[NO];
    if (xin) {
        const size_t g = (size_t)blockIdx.x * SB + tid;
#pragma unroll
        for (int k = 0; k < NF; k++) x[k] = xin[g * NF + k];
#pragma unroll
        for (int c = 0; c < NO; c++) y[c] = yin[g * NO + c];
    } else {
        const int node = mag_nodes[hash32(seed * 1000003ull + (uint64_t)blockIdx.x * SB + tid) % (uint32_t)nmag];
#pragma unroll
        for (int k = 0; k < NF; k++) x[k] = feat[(size_t)node * NF + k];
        const double isc = 1.0 / scale[0];
#pragma unroll
        for (int c = 0; c < NO; c++) {
            const size_t q = 3 * (size_t)node + c;
            y[c] = (float)((vtrue[q] - (2.0 * vprev[q] - vprev2[q])) * isc);
        }
    }
    {
        const float x2[8] = {x[8], x[9], x[10], x[11], 0.f, 0.f, 0.f, 0.f};
        store8(A1, tid, 0, SBO_K16, x);
        store8(A1, tid, 8, SBO_K16, x2);
#pragma unroll
        for (int k = 0; k < NF; k++) store_bf16(XT, k, tid, SBO_K128, x[k]);
        store_bf16(XT, NF, tid, SBO_K128, 1.0f);  // ones row: the bias gradient gb1
        store_bf16(H1T, NH, tid, SBO_K128, 1.0f);
        store_bf16(H2T, NH, tid, SBO_K128, 1.0f);
    }
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t lane_addr = tmem + ((uint32_t)(32 * warp) << 16);
    uint32_t parity = 0;
    const uint32_t sA1 = smem_u32(A1), sH1 = smem_u32(H1), sH2 = smem_u32(H2), sD2 = smem_u32(D2),
                   sB1 = smem_u32(B1), sB2 = smem_u32(B2), sB3 = smem_u32(B3), sB2T = smem_u32(B2T),
                   sAT = smem_u32(AT), sH1T = smem_u32(H1T), sH2T = smem_u32(H2T), sXT = smem_u32(XT);
    // D (+)= A B over K = 16 ksteps; A and B K-major images with 8-row groups sboA / sboB apart
    auto gemm = [&](uint32_t d, uint32_t sa, uint32_t sboA, uint32_t sb, uint32_t sboB, int n, int ksteps) {
        for (int k = 0; k < ksteps; k++)
            mma_bf16(d, sdesc_kmajor(sa + 256 * k, TC_LBO, sboA), sdesc_kmajor(sb + 256 * k, TC_LBO, sboB),
                     idesc_bf16(TM, n), k > 0 ? 1u : 0u);
    };
    // all threads: make the shared-memory writes visible, issue (thread 0), wait for the MMAs
    auto sync_issue_wait = [&](int stage) -> bool {
        fence_proxy_async();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            if (stage == 1) gemm(tmem, sA1, SBO_K16, sB1, SBO_K16, NH, 1);
            else if (stage == 2) gemm(tmem + 64, sH1, SBO_K64, sB2, SBO_K64, NH, 4);
            else if (stage == 3) gemm(tmem + 128, sH2, SBO_K64, sB3, SBO_K64, NO3, 4);
            else if (stage == 4) gemm(tmem + 144, sAT, SBO_K128, sH2T, SBO_K128, NB80, 8);  // gW3 | gb3
            else if (stage == 5) {
                gemm(tmem, sAT, SBO_K128, sH1T, SBO_K128, NB80, 8);      // gW2 | gb2
                gemm(tmem + 80, sD2, SBO_K64, sB2T, SBO_K64, NH, 4);     // delta2 W2
            } else {
                gemm(tmem + 144, sAT, SBO_K128, sXT, SBO_K128, K1, 8);   // gW1 | gb1
            }
            mma_commit(&bar);
        }
        const bool ok = mbar_wait(&bar, parity, err, &bail);
        if (!ok && tid == 0) mbar_drain(&bar, parity);
        parity ^= 1u;
        const bool all = __syncthreads_and(ok) != 0;
        tc_fence_after();
        return all;
    };
    float *G = gpart + (size_t)blockIdx.x * NPARAM;
    float lsum = 0.f;
    do {
        if (!sync_issue_wait(1)) break;
#pragma unroll
        for (int c = 0; c < NH / 16; c++) {  // H1 = tanh(D1 + b1)
            float v[16];
            drain16(lane_addr + 16 * c, v);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                v[k] = tanh_sfu(v[k] + bias[16 * c + k]);
                store_bf16(H1T, 16 * c + k, tid, SBO_K128, v[k]);
            }
            store8(H1, tid, 16 * c, SBO_K64, v);
            store8(H1, tid, 16 * c + 8, SBO_K64, v + 8);
        }
        if (!sync_issue_wait(2)) break;
#pragma unroll
        for (int c = 0; c < NH / 16; c++) {  // H2 = tanh(D2 + b2)
            float v[16];
            drain16(lane_addr + 64 + 16 * c, v);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                v[k] = tanh_sfu(v[k] + bias[NH + 16 * c + k]);
                store_bf16(H2T, 16 * c + k, tid, SBO_K128, v[k]);
            }
            store8(H2, tid, 16 * c, SBO_K64, v);
            store8(H2, tid, 16 * c + 8, SBO_K64, v + 8);
        }
        if (!sync_issue_wait(3)) break;
        float d3[NO];
        {
            float o[16];
            drain16(lane_addr + 128, o);
#pragma unroll
            for (int c = 0; c < NO; c++) {
                const float d = o[c] + bias[2 * NH + c] - y[c];
                lsum += d * d;
                d3[c] = 2.0f * d * inv_batch;
                store_bf16(AT, c, tid, SBO_K128, d3[c]);
            }
        }
        // delta2 = (d3 W3) (1 - h2^2) with this sample's BF16 h2
#pragma unroll 4
        for (int k0 = 0; k0 < NH; k0 += 8) {
            float v[8];
#pragma unroll
            for (int q = 0; q < 8; q++) {
                const int k = k0 + q;
                const float h = load_bf16(H2, tid, k, SBO_K64);
                v[q] = (d3[0] * w3f[k] + d3[1] * w3f[NH + k] + d3[2] * w3f[2 * NH + k]) * (1.0f - h * h);
            }
            store8(D2, tid, k0, SBO_K64, v);
        }
        if (!sync_issue_wait(4)) break;
        if (warp == 0) {  // rows 0..2 of [gW3 | gb3]
            float g[16];
#pragma unroll
            for (int c = 0; c < 5; c++) {
                drain16(lane_addr + 144 + 16 * c, g);
                if (tid < NO)
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        const int col = 16 * c + k;
                        if (col < NH) G[OFF_W3 + tid * NH + col] = g[k];
                        else if (col == NH) G[OFF_B3 + tid] = g[k];
                    }
            }
        }
        // delta2^T into AT (the gW3 MMAs have read it)
#pragma unroll 4
        for (int k = 0; k < NH; k++) store_bf16(AT, k, tid, SBO_K128, load_bf16(D2, tid, k, SBO_K64));
        if (!sync_issue_wait(5)) break;
        if (warp < 2) {  // rows 0..63 of [gW2 | gb2]
            float g[16];
#pragma unroll
            for (int c = 0; c < 5; c++) {
                drain16(lane_addr + 16 * c, g);
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int col = 16 * c + k;
                    if (col < NH) G[OFF_W2 + tid * NH + col] = g[k];
                    else if (col == NH) G[OFF_B2 + tid] = g[k];
                }
            }
        }
        // delta1 = (delta2 W2) (1 - h1^2), transposed into AT (the gW2 MMAs have read it)
#pragma unroll
        for (int c = 0; c < NH / 16; c++) {
            float v[16];
            drain16(lane_addr + 80 + 16 * c, v);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                const float h = load_bf16(H1, tid, 16 * c + k, SBO_K64);
                store_bf16(AT, 16 * c + k, tid, SBO_K128, v[k] * (1.0f - h * h));
            }
        }
        if (!sync_issue_wait(6)) break;
        if (warp < 2) {  // rows 0..63 of [gW1 | gb1]
            float g[16];
            drain16(lane_addr + 144, g);
#pragma unroll
            for (int k = 0; k < 16; k++) {
                if (k < NF) G[OFF_W1 + tid * NF + k] = g[k];
                else if (k == NF) G[OFF_B1 + tid] = g[k];
            }
        }
    } while (false);
    // loss partial (fixed-order block reduction)
    red[tid] = lsum;
    __syncthreads();
    if (tid == 0) {
        float t = 0.0f;
        for (int k = 0; k < SB; k++) t += red[k];
        lpart[blockIdx.x] = t;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, GRAD_TMEM_COLS);
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
                       float *__restrict__ m2, __nv_bfloat16 *__restrict__ w, unsigned char *__restrict__ img, float lr,
                       float b1, float b2, float eps, float bc1, float bc2) {
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
    const __nv_bfloat16 wb = __float2bfloat16(nw);
    w[p] = wb;
    img_store(img, p, wb);
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
    if (cudaMalloc(&s->wimg, IMG_BYTES) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->feat, (size_t)c.nn * NF * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->gpart, (size_t)s->nblk_train * NPARAM * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->lpart, (size_t)s->nblk_train * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->xm, 2 * (size_t)c.nn * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->Wm, 3 * (size_t)c.nn * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->rpart, 2 * (size_t)s->nblk_res * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    s->nflag = c.batch ? std::max(1, c.nseg) : 1;
    {
        const MlpFlagsLayout lay(s->nflag);
        if (cudaMalloc(&s->dflags, lay.bytes) != cudaSuccess) return FG_ECUDA;
        if (cudaMallocHost(&s->hflags, lay.bytes) != cudaSuccess) return FG_ECUDA;
        cudaMemset(s->dflags, 0, lay.bytes);
        std::memset(s->hflags, 0, lay.bytes);
        s->tc_err = reinterpret_cast<int *>(s->dflags);
        s->flag = reinterpret_cast<int *>(s->dflags + lay.flag_off);
        s->res2 = reinterpret_cast<double *>(s->dflags + lay.res2_off);
    }
    if (cudaMallocHost(&s->hloss, (size_t)s->nblk_train * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->vprev2, 3 * (size_t)c.nn * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->scale, sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->spart, (size_t)s->nblk_res * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->rc, 2 * (size_t)c.nn * sizeof(double)) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&s->out, 3 * (size_t)c.nn * sizeof(float)) != cudaSuccess) return FG_ECUDA;
    cudaMemset(s->tc_err, 0, sizeof(int));
    {
        const double one = FG_GAMMA0 * c.ms_ref * 1e-3;
        cudaMemcpy(s->scale, &one, sizeof(double), cudaMemcpyHostToDevice);
        cudaMemset(s->vprev2, 0, 3 * (size_t)c.nn * sizeof(double));
    }
    s->primed = false;
    cudaMemcpy(s->master, w0.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(s->w, wb.data(), NPARAM * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice);
    cudaMemset(s->wimg, 0, IMG_BYTES);
    k_mlp_pack<<<nb(NPARAM, 256), 256, 0, c.stream>>>(s->w, s->wimg);
    cudaStreamSynchronize(c.stream);
    cudaMemset(s->m1, 0, NPARAM * sizeof(float));
    cudaMemset(s->m2, 0, NPARAM * sizeof(float));
    cudaMemset(s->flag, 0, sizeof(int));
    if (cudaFuncSetAttribute(k_mlp_grad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, GRAD_SMEM) != cudaSuccess)
        return FG_ECUDA;
    return cudaGetLastError() == cudaSuccess ? FG_OK : FG_ECUDA;
}

void mlp_free(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s) return;
    void *p[] = {s->master, s->m1, s->m2, s->w, s->feat, s->gpart, s->lpart, s->xm, s->Wm, s->rpart, s->dflags,
                 s->vprev2, s->scale, s->spart, s->rc, s->out, s->wimg};
    for (void *q : p)
        if (q) cudaFree(q);
    if (s->hloss) cudaFreeHost(s->hloss);
    if (s->hflags) cudaFreeHost(s->hflags);
    delete s;
    c.mlp = nullptr;
}

static double v0_scale(const Ctx &c) { return FG_GAMMA0 * c.ms_ref; }

// Where the node kernel stores the features of the current state (inference and training).
NodeFeat mlp_node_features(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    return NodeFeat{s->feat, 1.0 / c.ms_ref, 1.0 / v0_scale(c)};
}

// With use set: the network's outputs on the features this step's node kernel formed, and
// the candidate guess for the solve to judge (FP32 + refinement: the solver forms and blends
// it; FP64: formed here and kept by the referee kernels when its residual is smaller).
cudaError_t mlp_before_solve(Ctx &c, double c0, bool use, bool train) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!use) {
        if (!train) return cudaSuccess;
        k_feat_ring<<<nb(c.nn, 256), 256, 0, c.stream>>>(c.nn, c.Sptr, c.Scol, s->feat);
        c.launches += 1;
        return cudaGetLastError();
    }
    if (!s->primed) {  // no history yet: the extrapolation degenerates to v_prev
        cudaMemcpyAsync(s->vprev2, c.v[0], 3 * (size_t)c.nn * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
        s->primed = true;
    }
    // the network's three GEMMs on the tensor cores, on the features the node kernel formed
    MlpTcArgs a{};
    a.nn = c.nn; a.wimg = reinterpret_cast<const uint4 *>(s->wimg); a.xin = s->feat; a.yout = s->out; a.err = s->tc_err;
    a.Sptr = c.Sptr; a.Scol = c.Scol; a.ring_out = train ? 1 : 0;
    cudaError_t e = launch_mlp_infer_tc(c, a);
    if (e != cudaSuccess) return e;
    c.launches += 1;
    if (c.opts.precision == FG_PREC_FP32_REFINE) {
        // the FP32 + refinement solver forms the smoothed candidate in its first phase and
        // judges it on its first FP64 residual
        c.cand_x = s->xm;
        c.cand_W = s->Wm;
        c.cand_r = s->rc;
        c.cand_flag = s->flag;
        c.cand_res2 = s->res2;
        c.cand_o = s->out;
        c.cand_vprev = c.v[0];
        c.cand_vprev2 = s->vprev2;
        c.cand_scale = s->scale;
        return cudaSuccess;
    }
    k_mlp_candidate<<<nb(c.nn, 256), 256, 0, c.stream>>>(c.nn, c.mag, c.Sptr, c.Scol, s->out, c.v[0], s->vprev2,
                                                           s->scale, c.ep, c.eq, s->xm, s->Wm);
    c.launches += 1;
    k_resid2<<<s->nblk_res, 256, 0, c.stream>>>(c.nn, c.Sptr, c.Scol, c.Sval, c.ep, c.eq, c.A, c.Dl, c.mag, c0,
                                                c.rhs, s->xm, s->Wm, c.x, c.W, s->rpart);
    k_choose<<<1, 32, 0, c.stream>>>(s->nblk_res, s->rpart, s->flag, s->res2);
    k_take<<<nb(c.nn, 256), 256, 0, c.stream>>>(c.nn, s->flag, s->xm, s->Wm, c.x, c.W);
    c.launches += 3;
    return cudaGetLastError();
}

// One Adam step on a minibatch of (features at the start of the step, solved v).
cudaError_t mlp_train(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    const float inv_batch = 1.0f / (float)(s->nblk_train * SB * NO);
    if (!s->primed) {
        cudaMemcpyAsync(s->vprev2, c.v[0], 3 * (size_t)c.nn * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
        s->primed = true;
    }
    k_corr2<<<s->nblk_res, 256, 0, c.stream>>>(c.nn, c.mag, c.v[1], c.v[0], s->vprev2, s->spart);
    k_scale<<<1, 32, 0, c.stream>>>(s->nblk_res, s->spart, c.n_mag_nodes, s->scale);
    k_mlp_grad_tc<<<s->nblk_train, SB, GRAD_SMEM, c.stream>>>(c.n_mag_nodes, c.mag_nodes, s->feat, c.v[1], c.v[0],
                                                                s->vprev2, s->scale, s->w, (uint64_t)s->steps + 1,
                                                                inv_batch, s->gpart, s->lpart, nullptr, nullptr,
                                                                s->tc_err);
    c.launches += 2;
    s->t++;
    const float b1 = 0.9f, b2 = 0.999f;
    const float lr = c.opts.mlp_lr > 0 ? (float)c.opts.mlp_lr : 1e-3f;
    k_adam<<<nb(NPARAM, 256), 256, 0, c.stream>>>(s->nblk_train, s->gpart, s->master, s->m1, s->m2, s->w, s->wimg, lr, b1, b2,
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
    if (*reinterpret_cast<const int *>(s->hflags)) {  // copied by mlp_before_sync
        s->timed_out = true;
        cudaMemsetAsync(s->tc_err, 0, sizeof(int), c.stream);
    }
    if (accepted) mlp_sample_flags(c, 0, accepted, res0_mlp, res0_prev);
}

// The learned guess's result for system g of the last step (0: a single context; a sample of
// a batch), from the copy read at the step's sync.
void mlp_sample_flags(const Ctx &c, int g, int *accepted, double *res0_mlp, double *res0_prev) {
    const MlpState *s = static_cast<const MlpState *>(c.mlp);
    if (!s || g < 0 || g >= s->nflag) return;
    const MlpFlagsLayout lay(s->nflag);
    const int *flag = reinterpret_cast<const int *>(s->hflags + lay.flag_off);
    const double *res2 = reinterpret_cast<const double *>(s->hflags + lay.res2_off);
    *accepted = flag[g];
    *res0_mlp = std::sqrt(res2[2 * g]);
    *res0_prev = std::sqrt(res2[2 * g + 1]);
}

// Enqueues the copy of this step's flags that mlp_after_sync reads after the step's sync.
cudaError_t mlp_before_sync(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s) return cudaSuccess;
    return cudaMemcpyAsync(s->hflags, s->dflags, MlpFlagsLayout(s->nflag).bytes, cudaMemcpyDeviceToHost, c.stream);
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
    k_mlp_grad_tc<<<nblk, SB, GRAD_SMEM, c.stream>>>(1, c.mag_nodes, s->feat, c.v[1], c.v[0], s->vprev2, s->scale,
                                                      s->w, 1, 1.0f / (nsamples * NO), dg, dl, dx, dy, s->tc_err);
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
    int terr = 0;
    cudaMemcpy(&terr, s->tc_err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemset(s->tc_err, 0, sizeof(int));
    if (cudaGetLastError() != cudaSuccess) return FG_ECUDA;
    return terr ? FG_ETIMEDOUT : FG_OK;
}

int mlp_nparam() { return NPARAM; }

// Fem::evolution is about to overwrite v_prev: keep it as v_prev2 for the extrapolation.
cudaError_t mlp_before_evolution(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s) return cudaSuccess;
    s->primed = true;
    return cudaMemcpyAsync(s->vprev2, c.v[0], 3 * (size_t)c.nn * sizeof(double), cudaMemcpyDeviceToDevice, c.stream);
}

bool mlp_take_timeout(Ctx &c) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s || !s->timed_out) return false;
    s->timed_out = false;
    return true;
}

// The tensor-core forward pass on caller-given feature rows: out [n][3] (scaled units, the
// network's raw outputs).
int mlp_debug_infer(Ctx &c, int n, const float *hx, float *hy) {
    MlpState *s = static_cast<MlpState *>(c.mlp);
    if (!s || n <= 0) return FG_EINVAL;
    float *dx = nullptr, *dy = nullptr;
    if (cudaMalloc(&dx, sizeof(float) * (size_t)n * NF) != cudaSuccess) return FG_ECUDA;
    if (cudaMalloc(&dy, sizeof(float) * (size_t)n * NO) != cudaSuccess) {
        cudaFree(dx);
        return FG_ECUDA;
    }
    cudaMemcpy(dx, hx, sizeof(float) * (size_t)n * NF, cudaMemcpyHostToDevice);
    MlpTcArgs a{};
    a.nn = n; a.wimg = reinterpret_cast<const uint4 *>(s->wimg); a.xin = dx; a.yout = dy; a.err = s->tc_err;
    a.Sptr = a.Scol = nullptr;  // the caller's rows are complete
    a.ring_out = 0;
    cudaError_t e = launch_mlp_infer_tc(c, a);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    if (e == cudaSuccess) e = cudaMemcpy(hy, dy, sizeof(float) * (size_t)n * NO, cudaMemcpyDeviceToHost);
    int terr = 0;
    cudaMemcpy(&terr, s->tc_err, sizeof(int), cudaMemcpyDeviceToHost);
    cudaMemset(s->tc_err, 0, sizeof(int));
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return FG_ECUDA;
    return terr ? FG_ETIMEDOUT : FG_OK;
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
