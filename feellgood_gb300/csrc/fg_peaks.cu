// Measured compute roofs of the GPU the library runs on (fg_measure_peaks): throughput
// microbenchmarks of the instructions the compute-bound kernels are made of, counted per SM
// and per clock cycle (clock64 over each run), so that a roofline can be drawn at any clock:
// the FP32 fused multiply-add (scalar and packed f32x2, the near field's pair arithmetic),
// the SFU reciprocal square root (one per near-field pair) and tcgen05.mma kind::tf32 (the
// FMM translations). Each run is one launch of a few ms with enough independent chains per
// thread and resident warps to keep the pipe busy; the chains' results are kept live.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "fg_f32x2.cuh"
#include "fg_internal.h"

namespace fg {
namespace {

constexpr int CH = 8;      // independent chains per thread
constexpr int BLK = 256;   // threads per block
constexpr int BPSM = 8;    // blocks per SM: 64 resident warps

__device__ __forceinline__ void keep(float s, float *sink) {
    if (s == 1234.5678f) sink[0] = s;  // never true for these chains: keeps them from being removed
}

__global__ void __launch_bounds__(BLK) k_peak_ffma(int iters, float *sink, long long *cyc) {
    float a[CH];
#pragma unroll
    for (int k = 0; k < CH; k++) a[k] = 0.5f + 1e-3f * k + 1e-7f * threadIdx.x;
    const float b = 0.999f, c = 1e-3f;  // fixed point 1: the chains stay finite and normal
    __syncthreads();
    const long long t0 = clock64();
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int k = 0; k < CH; k++) asm volatile("fma.rn.f32 %0, %0, %1, %2;" : "+f"(a[k]) : "f"(b), "f"(c));
    __syncthreads();
    const long long t1 = clock64();
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < CH; k++) s += a[k];
    keep(s, sink);
    if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

__global__ void __launch_bounds__(BLK) k_peak_ffma2(int iters, float *sink, long long *cyc) {
    u64 a[CH];
#pragma unroll
    for (int k = 0; k < CH; k++) a[k] = pk2(0.5f + 1e-3f * k, 0.25f + 1e-7f * threadIdx.x);
    const u64 b = pk2(0.999f, 0.999f), c = pk2(1e-3f, 1e-3f);
    __syncthreads();
    const long long t0 = clock64();
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int k = 0; k < CH; k++) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(a[k]) : "l"(b), "l"(c));
    __syncthreads();
    const long long t1 = clock64();
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < CH; k++) {
        float x, y;
        upk2(a[k], x, y);
        s += x + y;
    }
    keep(s, sink);
    if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

__global__ void __launch_bounds__(BLK) k_peak_rsqrt(int iters, float *sink, long long *cyc) {
    float a[CH];
#pragma unroll
    for (int k = 0; k < CH; k++) a[k] = 2.0f + 0.1f * k + 1e-6f * threadIdx.x;  // x -> x^-1/2 tends to 1
    __syncthreads();
    const long long t0 = clock64();
    for (int i = 0; i < iters; i++)
#pragma unroll
        for (int k = 0; k < CH; k++) asm volatile("rsqrt.approx.ftz.f32 %0, %0;" : "+f"(a[k]));
    __syncthreads();
    const long long t1 = clock64();
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < CH; k++) s += a[k];
    keep(s, sink);
    if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

struct Scratch {
    float *sink = nullptr;
    long long *cyc = nullptr;
    int *err = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t st = nullptr;
    ~Scratch() {
        if (sink) cudaFree(sink);
        if (cyc) cudaFree(cyc);
        if (err) cudaFree(err);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (st) cudaStreamDestroy(st);
    }
};

// Longest block duration in cycles of the last launch (every block is resident from the
// start, so this is the launch's duration); -1 if a block reported a failed wait.
long long max_cycles(const Scratch &S, int nblk) {
    std::vector<long long> h(nblk);
    if (cudaMemcpy(h.data(), S.cyc, sizeof(long long) * nblk, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    long long m = 0;
    for (long long x : h) {
        if (x < 0) return -1;
        m = std::max(m, x);
    }
    return m;
}

}  // namespace
}  // namespace fg

using namespace fg;

extern "C" int fg_measure_peaks(double out[7]) {
    if (!out) return FG_EINVAL;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
        return FG_ECUDA;
    Scratch S;
    const int nblk = nsm * BPSM;
    if (cudaMalloc(&S.sink, sizeof(float)) != cudaSuccess ||
        cudaMalloc(&S.cyc, sizeof(long long) * nblk) != cudaSuccess || cudaMalloc(&S.err, sizeof(int)) != cudaSuccess ||
        cudaMemset(S.err, 0, sizeof(int)) != cudaSuccess || cudaEventCreate(&S.e0) != cudaSuccess ||
        cudaEventCreate(&S.e1) != cudaSuccess || cudaStreamCreateWithFlags(&S.st, cudaStreamNonBlocking) != cudaSuccess)
        return FG_ECUDA;
    const double lanes = (double)nblk * BLK * CH;
    // scalar FMA, packed FMA (2 lane operations each), SFU reciprocal square root
    const int it_fma = 20000, it_rsq = 3000;
    double per_clk[3], mhz = 0.0;
    for (int kind = 0; kind < 3; kind++) {
        const int iters = kind == 2 ? it_rsq : it_fma;
        for (int rep = 0; rep < 2; rep++) {  // the first run warms the clocks up
            cudaEventRecord(S.e0, S.st);
            if (kind == 0) k_peak_ffma<<<nblk, BLK, 0, S.st>>>(iters, S.sink, S.cyc);
            else if (kind == 1) k_peak_ffma2<<<nblk, BLK, 0, S.st>>>(iters, S.sink, S.cyc);
            else k_peak_rsqrt<<<nblk, BLK, 0, S.st>>>(iters, S.sink, S.cyc);
            cudaEventRecord(S.e1, S.st);
            if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(S.st) != cudaSuccess) return FG_ECUDA;
        }
        const long long cyc = max_cycles(S, nblk);
        if (cyc <= 0) return FG_ECUDA;
        const double ops = lanes * iters * (kind == 1 ? 2.0 : 1.0);
        per_clk[kind] = ops / ((double)cyc * nsm);
        if (kind == 0) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, S.e0, S.e1);
            mhz = ms > 0 ? (double)cyc / (ms * 1e3) : 0.0;
        }
    }
    // tensor pipe, kind::tf32 at the translations' N = 128 and at N = 256
    double tc[2];
    const int ns[2] = {128, 256};
    for (int k = 0; k < 2; k++) {
        const int iters = 40000;
        for (int rep = 0; rep < 2; rep++) {
            if (launch_peak_mma_tf32(S.st, nsm, ns[k], iters, S.cyc, S.err) != cudaSuccess ||
                cudaStreamSynchronize(S.st) != cudaSuccess)
                return FG_ECUDA;
        }
        int herr = 0;
        cudaMemcpy(&herr, S.err, sizeof(int), cudaMemcpyDeviceToHost);
        if (herr) return FG_ETIMEDOUT;
        const long long cyc = max_cycles(S, nsm);
        if (cyc <= 0) return FG_ETIMEDOUT;
        tc[k] = 2.0 * 128 * ns[k] * 8 * (double)iters / (double)cyc;  // flops per clock per SM
    }
    out[0] = per_clk[0];
    out[1] = per_clk[1];
    out[2] = per_clk[2];
    out[3] = tc[0];
    out[4] = tc[1];
    out[5] = mhz;
    out[6] = nsm;
    return FG_OK;
}
