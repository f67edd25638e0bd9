// Device helpers shared by the persistent kernels: bounded grid barrier and
// deterministic reductions.
#pragma once

#include "fg_internal.h"

namespace fg {

// ---------------------------------------------------------------------------------
// small helpers

__device__ __forceinline__ unsigned long long gtimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for cooperative (co-resident) launches. The wait is bounded: after
// 2 s without progress it records FG_ETIMEDOUT and returns false; every block then
// leaves the kernel, so no launch can hang the GPU.
__device__ inline bool grid_sync(GridBar *gb) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = &gb->gen;
        volatile int *verr = &gb->err;
        unsigned int g = *vgen;
        __threadfence();
        unsigned int arrived = atomicAdd(&gb->count, 1u);
        if (arrived == gridDim.x - 1) {
            atomicExch(&gb->count, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            unsigned long long t0 = gtimer();
            while (*vgen == g) {
                if (*verr) break;
                if (gtimer() - t0 > 2000000000ull) {
                    atomicExch(&gb->err, FG_ETIMEDOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *(volatile int *)&gb->err == 0;
}

// Deterministic block reduction of NV sums into partial[k*G + blockIdx.x].
template <int NV>
__device__ __forceinline__ void block_store(double (&val)[NV], double *partial, int G) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
        for (int o = 16; o > 0; o >>= 1) val[k] += __shfl_down_sync(0xffffffffu, val[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) sh[k][warp] = val[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double x = lane < nw ? sh[k][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) partial[k * G + blockIdx.x] = x;
        }
    }
    __syncthreads();
}

// The same from FP32 per-thread sums: the warp stage adds in FP32, the block and grid
// stages in FP64. GB300's FP64 pipe runs at 1/64 of the FP32 rate, so converting and
// accumulating every element in FP64 would bound an FP32 Krylov body on that pipe.
template <int NV>
__device__ __forceinline__ void block_store_f(float (&val)[NV], double *partial, int G) {
    __shared__ double shf[NV][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++)
        for (int o = 16; o > 0; o >>= 1) val[k] += __shfl_down_sync(0xffffffffu, val[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; k++) shf[k][warp] = (double)val[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double x = lane < nw ? shf[k][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) partial[k * G + blockIdx.x] = x;
        }
    }
    __syncthreads();
}

// Scalar FP64 work (divisions, square roots of the Krylov recurrences) evaluated once per
// block by thread 0 and handed to every thread, instead of 256 copies on the 1/64-rate FP64
// pipe. Every thread of the block must make the call.
template <typename F>
__device__ __forceinline__ double block_once(F f) {
    __shared__ double v;
    if (threadIdx.x == 0) v = f();
    __syncthreads();
    const double r = v;
    __syncthreads();
    return r;
}

// Every block sums the G partials of each of the NV slots in the same fixed order.
template <int NV>
__device__ __forceinline__ void grid_sum(const double *partial, int G, double (&out)[NV]) {
    __shared__ double res[NV];
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double x = 0.0;
            for (int b = lane; b < G; b += 32) x += *(volatile const double *)&partial[k * G + b];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) res[k] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = res[k];
    __syncthreads();
}

// Sum of the partials of blocks [b0, b1) only (one sample of a batch), same fixed order.
template <int NV>
__device__ __forceinline__ void range_sum(const double *partial, int G, int b0, int b1, double (&out)[NV]) {
    __shared__ double res[NV];
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double x = 0.0;
            for (int b = b0 + lane; b < b1; b += 32) x += *(volatile const double *)&partial[k * G + b];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if (lane == 0) res[k] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) out[k] = res[k];
    __syncthreads();
}

__device__ __forceinline__ double dmax_reduce_block(double v) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        v = lane < nw ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    __syncthreads();
    return v;
}


template <typename T>
__device__ __forceinline__ void tangent(int i, const T *ep, const T *eq, T xp, T xq, T *W) {
    W[3 * i] = xp * ep[3 * i] + xq * eq[3 * i];
    W[3 * i + 1] = xp * ep[3 * i + 1] + xq * eq[3 * i + 1];
    W[3 * i + 2] = xp * ep[3 * i + 2] + xq * eq[3 * i + 2];
}

// (K x)_i for node i from the tangent vectors W of x: the 2x2 block row of node i in the
// factorised form (c0 S W projected on (eq_i, ep_i) plus the diagonal block). W is written
// by other blocks of the persistent kernels, so it is read through L2 (ld.cg).
template <typename T>
__device__ __forceinline__ void apply_row(int i, const int *__restrict__ Sptr, const int *__restrict__ Scol,
                                          const T *__restrict__ Sval, const T *W, const T *ep, const T *eq,
                                          const T *A, const T *Dl, T c0, T xp, T xq, T &y0, T &y1) {
    T a0 = 0, a1 = 0, a2 = 0;
    const int k1 = Sptr[i + 1];
    for (int k = Sptr[i]; k < k1; k++) {
        const int j = Scol[k];
        const T s = Sval[k];
        a0 += s * __ldcg(W + 3 * j);
        a1 += s * __ldcg(W + 3 * j + 1);
        a2 += s * __ldcg(W + 3 * j + 2);
    }
    const T q0 = eq[3 * i], q1 = eq[3 * i + 1], q2 = eq[3 * i + 2];
    const T e0 = ep[3 * i], e1 = ep[3 * i + 1], e2 = ep[3 * i + 2];
    const T ai = A[i], di = Dl[i];
    y0 = c0 * (q0 * a0 + q1 * a1 + q2 * a2) + ai * xp + di * xq;
    y1 = c0 * (e0 * a0 + e1 * a1 + e2 * a2) + di * xp - ai * xq;
}

// apply_row for a group of LPR consecutive lanes sharing row i (LPR = 1: thread per row):
// the lanes split the row's neighbour list and add their partial sums with shuffles, so a
// row's column indices and values are read by adjacent lanes. Every lane of the warp must
// call it (valid = false for lanes without a row); all lanes of the group get y0, y1.
template <typename T, int LPR>
__device__ __forceinline__ void apply_row_g(bool valid, int i, int sub, const int *__restrict__ Sptr,
                                            const int *__restrict__ Scol, const T *__restrict__ Sval, const T *W,
                                            const T *ep, const T *eq, const T *A, const T *Dl, T c0, T xp, T xq,
                                            T &y0, T &y1) {
    if constexpr (LPR == 1) {
        if (valid) apply_row<T>(i, Sptr, Scol, Sval, W, ep, eq, A, Dl, c0, xp, xq, y0, y1);
        return;
    }
    T a0 = 0, a1 = 0, a2 = 0;
    if (valid) {
        const int k1 = Sptr[i + 1];
        for (int k = Sptr[i] + sub; k < k1; k += LPR) {
            const int j = Scol[k];
            const T s = Sval[k];
            a0 += s * __ldcg(W + 3 * j);
            a1 += s * __ldcg(W + 3 * j + 1);
            a2 += s * __ldcg(W + 3 * j + 2);
        }
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (valid) {
        const T q0 = eq[3 * i], q1 = eq[3 * i + 1], q2 = eq[3 * i + 2];
        const T e0 = ep[3 * i], e1 = ep[3 * i + 1], e2 = ep[3 * i + 2];
        const T ai = A[i], di = Dl[i];
        y0 = c0 * (q0 * a0 + q1 * a1 + q2 * a2) + ai * xp + di * xq;
        y1 = c0 * (e0 * a0 + e1 * a1 + e2 * a2) + di * xp - ai * xq;
    }
}

}  // namespace fg
