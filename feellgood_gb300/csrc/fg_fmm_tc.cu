// FMM translations on the 5th-generation tensor cores (tcgen05) for the FP32 path.
//
// Every translation of the FMM (M2L for each cell offset, M2M and L2L for each child
// octant) applies a fixed real 100x100 operator to 100-coefficient expansions. For a tile
// of 64 output cells the work of one operator code is one GEMM
//     D[128 x 64] += Op_code[128 x 104] * X_code[104 x 64],
// rows = output coefficients (100 used), columns = the 64 cells, X_code = the input
// expansions that this code brings to each of the 64 cells (zero where there is none),
// K = input coefficients padded to 104. D lives in tensor memory (TMEM, 64 columns of
// FP32) and accumulates over all the codes of the tile, so each output is written once.
//
// Precision: the FP32 expansions are split as x = hi + lo with hi = tf32(x) (round to
// nearest) and lo = x - hi; D += Ah Bh + Ah Bl + Al Bh (kind::tf32 MMAs with FP32
// accumulation) keeps about 21 bits of every product, the accuracy of the FP32 CUDA-core
// translation.
//
// Pipeline (one CTA of 9 warps per tile, 4 shared-memory stages of K = 32):
//   warps 0-3  load one K-chunk of the operator and of the 64 gathered inputs with vector
//              loads, split hi/lo, store them in the no-swizzle K-major core-matrix layout
//              (8 rows x 16 bytes per core matrix), fence the async proxy, arrive on full[s];
//   warp 4     one lane waits full[s], issues the MMAs of each K-step of 8 and
//              tcgen05.commit arrives on empty[s] when they have read the stage; each code
//              accumulates into its own TMEM buffer (two, used in turn), committed to tfull;
//   warps 5-8  drain a finished code buffer with tcgen05.ld (warp w owns TMEM lanes
//              32(w%4)..+31 = coefficient rows), add it to FP32 registers with round to
//              nearest, release it (tfree), and finally store (or add to) the outputs.
// The tensor core's FP32 accumulation rounds toward zero, so an accumulator summed over
// all codes in place drifts by about 2.4e-7 per 13 K-steps (measured); one accumulator per
// code and per term group keeps the translation at FP32 rounding level.
// Every wait on an mbarrier is bounded (about 1 s): on expiry the CTA records FG_ETIMEDOUT
// in *err, stops issuing work, frees its TMEM and returns.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "fg_internal.h"

namespace fg {

namespace {

constexpr int NRC = 100;  // reals per expansion (P = 9)
constexpr int NC = 64;    // output cells per CTA = MMA N
constexpr int MR = 128;   // MMA M
constexpr int KC = 32;    // K per pipeline item
constexpr int NCHUNK = 4; // K = 104 = 32 + 32 + 32 + 8
constexpr int NSTAGE = 4;
constexpr int A_BYTES = MR * KC * 4;                    // 16 KB per part (hi or lo)
constexpr int B_BYTES = NC * KC * 4;                    // 8 KB per part
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // 48 KB
constexpr uint32_t LBO = 128;                           // next core matrix along K
constexpr uint32_t SBO = 1024;                          // next group of 8 rows
constexpr int TMEM_COLS = 256;  // 2 buffers x (main, corr) x 64 columns

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared-memory matrix descriptor: no swizzle, K-major core matrices of 8 rows x 16 bytes.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((LBO >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((SBO >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
    return d;                // base offset 0, absolute LBO mode, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::tf32: D f32, A and B tf32, both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(b))
                 : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the completion of the phase with the given parity.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, int *err, volatile int *bail) {
    if (mbar_test(b, parity)) return true;
    const unsigned long long t0 = now_ns();
    for (;;) {
        if (mbar_test(b, parity)) return true;
        if (*bail) return false;
        if (now_ns() - t0 > 1000000000ull) {
            *bail = 1;
            atomicExch(err, FG_ETIMEDOUT);
            return false;
        }
    }
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *b) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
                 : "memory");
}

// 16 consecutive TMEM columns of this warp's 32 lanes: one register per column.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// x rounded to the 10 explicit mantissa bits of TF32 (nearest, ties away from zero), as an
// FP32 bit pattern whose 13 low bits are zero; x - tf32_rn(x) is then exact in FP32.
__device__ __forceinline__ float tf32_rn(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// hi/lo split of 4 consecutive K values, stored at the same offset of the hi and lo images.
__device__ __forceinline__ void store_split(unsigned char *hi, unsigned char *lo, int off, float4 v) {
    const float h0 = tf32_rn(v.x), h1 = tf32_rn(v.y), h2 = tf32_rn(v.z), h3 = tf32_rn(v.w);
    *reinterpret_cast<float4 *>(hi + off) = make_float4(h0, h1, h2, h3);
    *reinterpret_cast<float4 *>(lo + off) = make_float4(v.x - h0, v.y - h1, v.z - h2, v.w - h3);
}

// One K-chunk (KQN quads of K) of the operator rows 0..103 and of the 64 gathered inputs.
// Thread mapping: 8 consecutive threads take the 8 rows of one core matrix (conflict-free
// 16-byte shared stores); 4 such groups of a warp read 64 contiguous bytes of each row.
template <int KQN>
__device__ __forceinline__ void load_chunk(unsigned char *st, int tid, const float *__restrict__ op, int k0,
                                           const int *__restrict__ tab, int ncode, int code, int out0, int c_begin,
                                           int n_out, const float *in) {
    for (int e = tid; e < 104 * KQN; e += 128) {
        const int il = e & 7, r = e >> 3, kq = r % KQN, ig = r / KQN, i = ig * 8 + il;
        const int j = k0 + 4 * kq;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < NRC && j < NRC) v = __ldg(reinterpret_cast<const float4 *>(op + i * NRC + j));
        store_split(st, st + A_BYTES, ig * 1024 + kq * 128 + il * 16, v);
    }
    unsigned char *bs = st + 2 * A_BYTES;
    for (int e = tid; e < NC * KQN; e += 128) {
        const int il = e & 7, r = e >> 3, kq = r % KQN, cg = r / KQN, n = cg * 8 + il;
        const int j = k0 + 4 * kq;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        const int cell = c_begin + n;
        if (cell < n_out && j < NRC) {
            const int sc = __ldg(tab + (size_t)(out0 + cell) * ncode + code);
            if (sc >= 0) v = *reinterpret_cast<const float4 *>(in + (size_t)sc * NRC + j);
        }
        store_split(bs, bs + B_BYTES, cg * 1024 + kq * 128 + il * 16, v);
    }
}

__device__ __forceinline__ void translate_tc_body(int n_out, int out0, int ncode, const int *__restrict__ tab,
                                                  const float *__restrict__ ops, const float *in, float *out,
                                                  int accumulate, const int *__restrict__ tile_ptr,
                                                  const int *__restrict__ tile_code, int *err, int terms) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[NSTAGE], empty[NSTAGE], tfull[2], tfree[2];
    __shared__ uint32_t tmem_base;
    __shared__ volatile int bail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int c_begin = blockIdx.x * NC;
    const int q0 = tile_ptr[blockIdx.x], q1 = tile_ptr[blockIdx.x + 1];
    const int ncodes = q1 - q0, nitems = ncodes * NCHUNK;
    if (nitems == 0) {  // no input reaches these cells: a stored result is zero
        if (!accumulate)
            for (int e = tid; e < NC * NRC; e += blockDim.x) {
                const int cell = c_begin + e / NRC;
                if (cell < n_out) out[(size_t)(out0 + cell) * NRC + e % NRC] = 0.f;
            }
        return;
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; s++) {
            mbar_init(&full[s], 128);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tfree[b], 128);
        }
        bail = 0;
        fence_mbar_init();
    }
    // rows 104..127 of the operator images are read by the M = 128 MMA: keep them zero
    for (int e = tid; e < NSTAGE * 2 * 192; e += blockDim.x) {
        const int s = e / 384, part = (e / 192) & 1, k = e % 192;
        *reinterpret_cast<uint4 *>(sm + s * STAGE_BYTES + part * A_BYTES + 13 * 1024 + k * 16) = make_uint4(0, 0, 0, 0);
    }
    if (warp == 4) tmem_alloc(&tmem_base, TMEM_COLS);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp < 4) {
        // producers: operator and gathered inputs, one K-chunk per pipeline item
        for (int it = 0; it < nitems; it++) {
            const int s = it % NSTAGE;
            if (it >= NSTAGE && !mbar_wait(&empty[s], ((it / NSTAGE) - 1) & 1, err, &bail)) break;
            const int code = tile_code[q0 + it / NCHUNK], q = it % NCHUNK;
            const float *op = ops + (size_t)code * NRC * NRC;
            unsigned char *st = sm + s * STAGE_BYTES;
            if (q < 3) load_chunk<8>(st, tid, op, 32 * q, tab, ncode, code, out0, c_begin, n_out, in);
            else load_chunk<2>(st, tid, op, 96, tab, ncode, code, out0, c_begin, n_out, in);
            fence_proxy_async();
            mbar_arrive(&full[s]);
        }
    } else if (warp == 4) {
        if (lane == 0) {
            // MMA issuer. Each code accumulates into a fresh pair of TMEM accumulators
            // (buffer ci & 1): main = hi*hi, corr = hi*lo + lo*hi. The tensor core's FP32
            // accumulation truncates, so its error grows with the number of MMAs summed in
            // place; 13 K-steps per accumulator keep it at FP32 rounding level, and the drain
            // warps add the per-code results with round-to-nearest.
            const uint32_t idesc = idesc_tf32(MR, NC);
            bool ok = true;
            for (int ci = 0; ci < ncodes && ok; ci++) {
                const int b = ci & 1;
                if (ci >= 2 && !mbar_wait(&tfree[b], ((ci >> 1) - 1) & 1, err, &bail)) break;
                tc_fence_after();
                const uint32_t dmain = tmem + b * 2 * NC, dcorr = dmain + NC;
                for (int q = 0; q < NCHUNK; q++) {
                    const int it = ci * NCHUNK + q, s = it % NSTAGE;
                    if (!mbar_wait(&full[s], (it / NSTAGE) & 1, err, &bail)) { ok = false; break; }
                    tc_fence_after();
                    const int ksteps = q < 3 ? 4 : 1;
                    const uint32_t base = smem_u32(sm + s * STAGE_BYTES);
                    for (int k = 0; k < ksteps; k++) {
                        const uint64_t ah = sdesc(base + k * 256), al = sdesc(base + A_BYTES + k * 256);
                        const uint64_t bh = sdesc(base + 2 * A_BYTES + k * 256);
                        const uint64_t bl = sdesc(base + 2 * A_BYTES + B_BYTES + k * 256);
                        const bool first = (q == 0 && k == 0);
                        if (terms & 1) mma_tf32(dmain, ah, bh, idesc, first ? 0u : 1u);
                        if (terms & 2) mma_tf32(dcorr, ah, bl, idesc, first ? 0u : 1u);
                        if (terms & 4) mma_tf32(dcorr, al, bh, idesc, (first && !(terms & 2)) ? 0u : 1u);
                    }
                    mma_commit(&empty[s]);
                }
                mma_commit(&tfull[b]);
            }
        }
    } else {
        // drain warps 5..8: warp w reads TMEM lanes 32 (w % 4) .. +31 (coefficient rows)
        const int quarter = warp & 3;
        const int row = 32 * quarter + lane;
        const uint32_t lane_off = (uint32_t)(32 * quarter) << 16;
        float acc[NC];
#pragma unroll
        for (int j = 0; j < NC; j++) acc[j] = 0.f;
        int drained = 0;
        for (int ci = 0; ci < ncodes; ci++) {
            const int b = ci & 1;
            const bool mine = mbar_wait(&tfull[b], (ci >> 1) & 1, err, &bail);
            if (!__all_sync(0xffffffffu, mine && !bail)) break;
            tc_fence_after();
            const uint32_t dmain = tmem + lane_off + b * 2 * NC, dcorr = dmain + NC;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                uint32_t rm[16], rc[16];
                tmem_ld16(dmain + 16 * j, rm);
                tmem_ld16(dcorr + 16 * j, rc);
                tmem_wait_ld();
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const float m = (terms & 1) ? __uint_as_float(rm[k]) : 0.f;
                    const float cr = (terms & 6) ? __uint_as_float(rc[k]) : 0.f;
                    acc[16 * j + k] += m + cr;
                }
            }
            tc_fence_before();
            mbar_arrive(&tfree[b]);
            drained++;
        }
        if (drained == ncodes && row < NRC) {
#pragma unroll
            for (int j = 0; j < NC; j++) {
                const int cell = c_begin + j;
                if (cell < n_out) {
                    float *o = out + (size_t)(out0 + cell) * NRC + row;
                    *o = accumulate ? *o + acc[j] : acc[j];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

// One entry per translation kind, so that profiles tell them apart.
#define FG_TC_KERNEL(name)                                                                                       \
    __global__ void __launch_bounds__(288, 1)                                                                    \
        name(int n_out, int out0, int ncode, const int *__restrict__ tab, const float *__restrict__ ops,          \
             const float *in, float *out, int accumulate, const int *__restrict__ tile_ptr,                     \
             const int *__restrict__ tile_code, int *err, int terms) {                                          \
        translate_tc_body(n_out, out0, ncode, tab, ops, in, out, accumulate, tile_ptr, tile_code, err, terms); \
    }
FG_TC_KERNEL(k_m2m_tc)
FG_TC_KERNEL(k_m2l_tc)
FG_TC_KERNEL(k_l2l_tc)
#undef FG_TC_KERNEL

}  // namespace

int translate_tc_smem() { return NSTAGE * STAGE_BYTES + 1024; }

cudaError_t translate_tc_setup() {
    cudaError_t e = cudaFuncSetAttribute(k_m2m_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, translate_tc_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_m2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, translate_tc_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_l2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, translate_tc_smem());
    return e;
}

cudaError_t launch_translate_tc(cudaStream_t st, int n_out, int out0, int ncode, const int *tab, const float *ops,
                                const float *in, float *out, int accumulate, const int *tile_ptr,
                                const int *tile_code, int *err, int terms) {
    if (n_out <= 0) return cudaSuccess;
    const int ntile = (n_out + NC - 1) / NC;
    auto k = accumulate ? k_l2l_tc : (ncode == 8 ? k_m2m_tc : k_m2l_tc);
    k<<<ntile, 288, translate_tc_smem(), st>>>(n_out, out0, ncode, tab, ops, in, out, accumulate, tile_ptr,
                                               tile_code, err, terms);
    return cudaGetLastError();
}

}  // namespace fg

// Diagnostic entry: one tensor-core translation launch on caller data (host arrays),
// out[c] = sum_code ops[code] in[tab[c][code]] for n_out cells, with the chosen product
// terms of the hi/lo split. Returns FG_* status.
extern "C" int fg_debug_translate_tc(int n_in, int n_out, int ncode, const float *ops, const int *tab,
                                     const float *in, float *out, int terms) {
    using namespace fg;
    if (n_in <= 0 || n_out <= 0 || ncode <= 0 || !ops || !tab || !in || !out) return FG_EINVAL;
    for (long k = 0; k < (long)n_out * ncode; k++)
        if (tab[k] < -1 || tab[k] >= n_in) return FG_EINVAL;
    std::vector<int> ptr, codes;
    const int ntile = (n_out + NC - 1) / NC;
    for (int b = 0; b < ntile; b++) {
        ptr.push_back((int)codes.size());
        for (int code = 0; code < ncode; code++) {
            bool any = false;
            for (int cc = b * NC; cc < std::min(n_out, b * NC + NC) && !any; cc++) any = tab[(size_t)cc * ncode + code] >= 0;
            if (any) codes.push_back(code);
        }
    }
    ptr.push_back((int)codes.size());
    float *d_ops = nullptr, *d_in = nullptr, *d_out = nullptr;
    int *d_tab = nullptr, *d_ptr = nullptr, *d_code = nullptr, *d_err = nullptr;
    int status = FG_OK, herr = 0;
    auto ok = [&](cudaError_t e) { if (e != cudaSuccess && status == FG_OK) status = FG_ECUDA; return e == cudaSuccess; };
    if (ok(cudaMalloc(&d_ops, sizeof(float) * (size_t)ncode * NRC * NRC)) &&
        ok(cudaMalloc(&d_in, sizeof(float) * (size_t)n_in * NRC)) &&
        ok(cudaMalloc(&d_out, sizeof(float) * (size_t)n_out * NRC)) &&
        ok(cudaMalloc(&d_tab, sizeof(int) * (size_t)n_out * ncode)) &&
        ok(cudaMalloc(&d_ptr, sizeof(int) * ptr.size())) &&
        ok(cudaMalloc(&d_code, sizeof(int) * std::max<size_t>(1, codes.size()))) &&
        ok(cudaMalloc(&d_err, sizeof(int))) &&
        ok(cudaMemcpy(d_ops, ops, sizeof(float) * (size_t)ncode * NRC * NRC, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_in, in, sizeof(float) * (size_t)n_in * NRC, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_tab, tab, sizeof(int) * (size_t)n_out * ncode, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_ptr, ptr.data(), sizeof(int) * ptr.size(), cudaMemcpyHostToDevice)) &&
        (codes.empty() || ok(cudaMemcpy(d_code, codes.data(), sizeof(int) * codes.size(), cudaMemcpyHostToDevice))) &&
        ok(cudaMemset(d_err, 0, sizeof(int))) && ok(translate_tc_setup()) &&
        ok(launch_translate_tc(0, n_out, 0, ncode, d_tab, d_ops, d_in, d_out, 0, d_ptr, d_code, d_err, terms)) &&
        ok(cudaDeviceSynchronize()) &&
        ok(cudaMemcpy(out, d_out, sizeof(float) * (size_t)n_out * NRC, cudaMemcpyDeviceToHost)) &&
        ok(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost))) {
        if (herr) status = FG_ETIMEDOUT;
    }
    void *ptrs[] = {d_ops, d_in, d_out, d_tab, d_ptr, d_code, d_err};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    return status;
}

namespace fg {

}  // namespace fg
