// FMM translations on the 5th-generation tensor cores (tcgen05) for the FP32 path.
//
// Every translation of the FMM (M2L for each cell offset, M2M and L2L for each child
// octant) applies a fixed real 100x100 operator to 100-coefficient expansions. For a tile
// of 64 output cells the work of one operator code is one GEMM
//     D[128 x 64 ns] += Op_code[128 x 104] * X_code[104 x 64 ns],
// rows = output coefficients (100 used), columns = the 64 cells of each of the ns sets of
// expansions evaluated together (the FMM evaluates the charges of m and of v at once: set s
// takes columns 64 s .. 64 s + 63, so the operator image is read once for both), X_code =
// the input expansions that this code brings to each cell (zero where there is none),
// K = input coefficients padded to 104. D lives in tensor memory (TMEM, 64 ns columns of
// FP32) and accumulates over all the codes of the tile, so each output is written once.
//
// Precision: the FP32 expansions are split as x = hi + lo with hi = tf32(x) (round to
// nearest) and lo = x - hi; D += Ah Bh + Ah Bl + Al Bh (kind::tf32 MMAs with FP32
// accumulation) keeps about 21 bits of every product, the accuracy of the FP32 CUDA-core
// translation.
//
// Pipeline (one CTA of 9 warps per tile, one CTA per SM, 6 shared-memory stages of K = 16):
//   warps 0-3  fill one stage per item: thread 0 starts two bulk copies
//              (cp.async.bulk, completion counted in bytes on bfull[s]) of the operator
//              item, stored pre-split (hi, lo) in global memory in exactly the shared-memory
//              image the MMA reads (no-swizzle K-major core matrices, 8 rows x 16 bytes);
//              all 128 threads gather the 64 ns input expansions' item with 16-byte cp.async
//              from pre-split hi/lo arrays into the same layout (zero fill where a cell has
//              no input). A thread arrives on full[s] once its copies for that item have
//              landed, LAG items later and before it waits for the next free stage, so
//              LAG items per CTA are in flight and the MMAs of an item never wait for those
//              of the item before it to complete;
//   warp 4     one lane waits full[s] and bfull[s], issues the MMAs of each K-step of 8 and
//              tcgen05.commit arrives on empty[s] when they have read the stage; each code
//              accumulates into its own TMEM buffer (two, used in turn), committed to tfull;
//   warps 5-8  drain a finished code buffer with tcgen05.ld (warp w owns TMEM lanes
//              32(w%4)..+31 = coefficient rows), add it to FP32 registers with round to
//              nearest, release it (tfree), and finally store (or add to) the outputs and
//              their hi/lo split for the next translation.
// The tensor core's FP32 accumulation rounds toward zero, so an accumulator summed over
// all codes in place drifts by about 2.4e-7 per 13 K-steps (measured); one accumulator per
// code and per term group keeps the translation at FP32 rounding level.
// Every wait on an mbarrier is bounded (about 1 s): on expiry the CTA records FG_ETIMEDOUT
// in *err and stops issuing work; before it frees its TMEM and returns, the issuer waits
// (bounded) for the MMAs it started (tcgen05.commit on tdone) and thread 0 for the bytes of
// the bulk copies it started (bfull), so no asynchronous write is left in flight.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "fg_internal.h"
#include "fg_tcgen05.cuh"

namespace fg {

namespace {

constexpr int NRC = 100;  // reals per expansion (P = 9)
constexpr int NC = 64;    // output cells per CTA
constexpr int NSET = 2;   // sets of expansions per CTA at most (MMA N = 64 sets)
constexpr int NB = NC * NSET;
constexpr int MR = 128;   // MMA M
constexpr int KI = 16;    // K per pipeline item (2 MMA K-steps of 8)
constexpr int IPC = 7;    // items per code: K = 104 = 6 x 16 + 8
constexpr int KQ = KI / 4;                              // 16-byte quads of K per row and item
constexpr int NSTAGE = 6;                               // 192 KB of stages: one CTA per SM
constexpr uint32_t LBO = 128;                           // next core matrix along K
constexpr uint32_t SBO = KQ * 128;                      // next group of 8 rows (512 B)
constexpr int A_BYTES = 16 * SBO;                       // 8 KB per part (hi or lo), rows 0..127
constexpr int B_BYTES = (NB / 8) * SBO;                 // 8 KB per part
constexpr int STAGE_BYTES = 2 * A_BYTES + 2 * B_BYTES;  // 32 KB
constexpr int TMEM_COLS = 512;  // 2 buffers x (main, corr) x 128 columns: all of an SM's TMEM
constexpr int IMG_BYTES = 13 * SBO;  // one operator image part: rows 0..103 (13 groups of 8)
constexpr int LAG = NSTAGE - 1;      // items whose gathers may still be in flight

using namespace tc;

// Shared-memory descriptor of this file's operand layout (LBO / SBO above).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) { return sdesc_kmajor(saddr, LBO, SBO); }

// x rounded to the 10 explicit mantissa bits of TF32 (nearest, ties away from zero), as an
// FP32 bit pattern whose 13 low bits are zero; x - tf32_rn(x) is then exact in FP32.
__device__ __forceinline__ float tf32_rn(float x) {
    return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// Gather of one item (K = 16) of the 64 input expansions of each set, hi and lo parts, with
// 16-byte async copies into the core-matrix layout: thread t copies quads 2(t&1), 2(t&1)+1
// of cell t>>1 of every set (column t>>1 + 64 set; zero fill beyond coefficient 99 or where
// the cell has no input, sc < 0). The sets share the tables: one source cell for all.
__device__ __forceinline__ void gather_item(unsigned char *bs, int tid, int k0, int sc, const float *in_hi,
                                            const float *in_lo, int ns, size_t set_io) {
    const int n = tid >> 1;
#pragma unroll
    for (int y = 0; y < NSET; y++) {
        if (y >= ns) break;
        const int col = n + NC * y;
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int kq = 2 * (tid & 1) + h, j = k0 + 4 * kq;
            const bool ok = sc >= 0 && j < NRC;
            const size_t o = ok ? y * set_io + (size_t)sc * NRC + j : 0;
            unsigned char *d = bs + (col >> 3) * SBO + kq * 128 + (col & 7) * 16;
            cp16(d, in_hi + o, ok ? 16u : 0u);
            cp16(d + B_BYTES, in_lo + o, ok ? 16u : 0u);
        }
    }
}

__device__ __forceinline__ void translate_tc_body(const TcArgs &a) {
    const int n_out = a.n_out, out0 = a.out0, ncode = a.ncode, accumulate = a.accumulate, terms = a.terms;
    const int *__restrict__ tab = a.tab;
    const int *__restrict__ tile_code = a.tile_code;
    // ns sets of expansions: the same tables and operators on ns sets of inputs and outputs,
    // set_io floats apart (set_scratch in the scratch array)
    const int ns = a.nset > 1 ? NSET : 1;
    const size_t set_io = a.set_io;
    float *out = a.out, *out_hi = a.out_hi, *out_lo = a.out_lo;
    const float *in_hi = a.in_hi, *in_lo = a.in_lo;
    float *scratch = a.scratch;
    int *err = a.err;
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    // full: the 128 gathering threads of a stage; bfull: the operator's bulk copies (bytes);
    // tdone: every MMA the issuer started has completed (checked before TMEM is freed)
    __shared__ __align__(8) uint64_t full[NSTAGE], bfull[NSTAGE], empty[NSTAGE], tfull[2], tfree[2], tdone;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int bail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int4 unit = a.units[blockIdx.x];
    const int c_begin = unit.x * NC;
    const int q0 = unit.y, q1 = unit.z, slot = unit.w;
    const int ncodes = q1 - q0, nitems = ncodes * IPC;
    if (nitems == 0) {  // no input reaches these cells: a stored result is zero
        if (!accumulate)
            for (int e = tid; e < ns * NC * NRC; e += blockDim.x) {
                const int y = e / (NC * NRC), r = e % (NC * NRC);
                const int cell = c_begin + r / NRC;
                if (cell < n_out) {
                    const size_t o = y * set_io + (size_t)(out0 + cell) * NRC + r % NRC;
                    out[o] = 0.f;
                    out_hi[o] = 0.f;
                    out_lo[o] = 0.f;
                }
            }
        return;
    }
    if (tid == 0) {
        for (int s = 0; s < NSTAGE; s++) {
            mbar_init(&full[s], 128);  // the 128 gathering threads
            mbar_init(&bfull[s], 1);   // thread 0's expect_tx, completed by the bulk copies' bytes
            mbar_init(&empty[s], 1);
        }
        mbar_init(&tdone, 1);
        for (int b = 0; b < 2; b++) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tfree[b], 128);
        }
        bail = 0;
        fence_mbar_init();
    }
    // rows 104..127 of the operator images are read by the M = 128 MMA: keep them zero
    constexpr int ZQ = 3 * SBO / 16;  // 16-byte words of groups 13..15
    for (int e = tid; e < NSTAGE * 2 * ZQ; e += blockDim.x) {
        const int s = e / (2 * ZQ), part = (e / ZQ) & 1, k = e % ZQ;
        *reinterpret_cast<uint4 *>(sm + s * STAGE_BYTES + part * A_BYTES + 13 * SBO + k * 16) = make_uint4(0, 0, 0, 0);
    }
    if (warp == 4) tmem_alloc(&tmem_base, TMEM_COLS);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp < 4) {
        // producers: one item (K = 16) per pipeline step; a thread's gathers of item it are
        // complete (cp.async.wait_group) when it arrives for that item, LAG items later.
        // The source cell of this thread's output cell is read once per code.
        bool live = true;
        // source cell of this thread's output cell for the current code; the next code's is
        // loaded one code ahead so that its latency is hidden behind the current code's items
        const int mycell = c_begin + (tid >> 1);
        auto src_of = [&](int ci) {
            return (ci < ncodes && mycell < n_out) ? __ldg(tab + (size_t)(out0 + mycell) * ncode + tile_code[q0 + ci])
                                                   : -1;
        };
        int sc = src_of(0), sc_next = src_of(1);
        int armed = 0;  // thread 0: items whose bulk copies were started (in order)
        for (int it = 0; it < nitems + LAG; it++) {
            // arrive for item it - LAG first: its copies were issued LAG items ago, and the
            // arrival must not wait behind this iteration's wait for a free stage (that wait
            // follows the MMAs of item it - NSTAGE; arriving after it would hold the MMAs of
            // item it - LAG until those of the item before it had completed)
            if (it >= LAG) {
                cp_wait<LAG - 1>();  // it groups committed: item it - LAG's has landed
                fence_proxy_async();
                if (live) mbar_arrive(&full[(it - LAG) % NSTAGE]);
            }
            if (it < nitems && live) {
                const int s = it % NSTAGE;
                if (it >= NSTAGE && !mbar_wait(&empty[s], ((it / NSTAGE) - 1) & 1, err, &bail)) live = false;
                if (live) {
                    const int ci = it / IPC, q = it % IPC;
                    const int code = tile_code[q0 + ci];
                    if (q == 0 && ci > 0) {
                        sc = sc_next;
                        sc_next = src_of(ci + 1);
                    }
                    unsigned char *st = sm + s * STAGE_BYTES;
                    if (tid == 0) {
                        const unsigned char *img = a.op_img + ((size_t)code * IPC + q) * 2 * IMG_BYTES;
                        mbar_arrive_expect_tx(&bfull[s], 2 * IMG_BYTES);
                        bulk_g2s(st, img, IMG_BYTES, &bfull[s]);
                        bulk_g2s(st + A_BYTES, img + IMG_BYTES, IMG_BYTES, &bfull[s]);
                        armed = it + 1;
                    }
                    gather_item(st + 2 * A_BYTES, tid, KI * q, sc, in_hi, in_lo, ns, set_io);
                }
            }
            cp_commit();
        }
        cp_wait<0>();
        // after a bail the issuer may not have consumed the last stages: wait (bounded) until
        // the bytes of every bulk copy still owed to a stage have landed before the CTA exits
        if (tid == 0 && bail)
            for (int it = armed > NSTAGE ? armed - NSTAGE : 0; it < armed; it++)
                mbar_drain(&bfull[it % NSTAGE], (it / NSTAGE) & 1);
    } else if (warp == 4) {
        if (lane == 0) {
            // MMA issuer. Each code accumulates into a fresh pair of TMEM accumulators
            // (buffer ci & 1): main = hi*hi, corr = hi*lo + lo*hi. The tensor core's FP32
            // accumulation truncates, so its error grows with the number of MMAs summed in
            // place; 13 K-steps per accumulator keep it at FP32 rounding level, and the drain
            // warps add the per-code results with round-to-nearest.
            const uint32_t idesc = idesc_tf32(MR, NC * ns);
            bool ok = true;
            for (int ci = 0; ci < ncodes && ok; ci++) {
                const int b = ci & 1;
                if (ci >= 2 && !mbar_wait(&tfree[b], ((ci >> 1) - 1) & 1, err, &bail)) break;
                tc_fence_after();
                const uint32_t dmain = tmem + b * 2 * NB, dcorr = dmain + NB;
                for (int q = 0; q < IPC; q++) {
                    const int it = ci * IPC + q, s = it % NSTAGE;
                    if (!mbar_wait(&full[s], (it / NSTAGE) & 1, err, &bail) ||
                        !mbar_wait(&bfull[s], (it / NSTAGE) & 1, err, &bail)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const int ksteps = q < IPC - 1 ? KI / 8 : 1;
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
            // tdone arrives once every MMA started above has completed (also after a bail,
            // when the drain warps no longer wait for them): TMEM is freed only after that
            mma_commit(&tdone);
            mbar_drain(&tdone, 0);
        }
    } else {
        // drain warps 5..8: warp w reads TMEM lanes 32 (w % 4) .. +31 (coefficient rows)
        const int quarter = warp & 3;
        const int row = 32 * quarter + lane;
        const uint32_t lane_off = (uint32_t)(32 * quarter) << 16;
        float acc[NB];
#pragma unroll
        for (int j = 0; j < NB; j++) acc[j] = 0.f;
        int drained = 0;
        for (int ci = 0; ci < ncodes; ci++) {
            const int b = ci & 1;
            const bool mine = mbar_wait(&tfull[b], (ci >> 1) & 1, err, &bail);
            if (!__all_sync(0xffffffffu, mine && !bail)) break;
            tc_fence_after();
            const uint32_t dmain = tmem + lane_off + b * 2 * NB, dcorr = dmain + NB;
#pragma unroll
            for (int j = 0; j < NB / 16; j++) {
                if (j >= ns * (NC / 16)) break;
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
            for (int y = 0; y < NSET; y++) {
                if (y >= ns) break;
                if (slot >= 0) {  // one of several units of this tile: partial result
                    float *p = scratch + y * a.set_scratch + (size_t)slot * NC * NRC + row;
#pragma unroll
                    for (int j = 0; j < NC; j++) p[j * NRC] = acc[NC * y + j];
                } else {
#pragma unroll
                    for (int j = 0; j < NC; j++) {
                        const int cell = c_begin + j;
                        if (cell < n_out) {
                            const size_t o = y * set_io + (size_t)(out0 + cell) * NRC + row;
                            const float v = accumulate ? out[o] + acc[NC * y + j] : acc[NC * y + j];
                            out[o] = v;
                            const float h = tf32_rn(v);
                            out_hi[o] = h;
                            out_lo[o] = v - h;
                        }
                    }
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
#define FG_TC_KERNEL(name) \
    __global__ void __launch_bounds__(288, 1) name(TcArgs a) { translate_tc_body(a); }
FG_TC_KERNEL(k_m2m_tc)
FG_TC_KERNEL(k_m2l_tc)
FG_TC_KERNEL(k_l2l_tc)
#undef FG_TC_KERNEL

// Sum of the partial results of tiles split over several units, in slot order.
__global__ void __launch_bounds__(256) k_tc_combine(TcArgs a) {
    const int4 ct = a.comb[blockIdx.x];
    const size_t io = blockIdx.y * a.set_io;
    const float *scratch = a.scratch + blockIdx.y * a.set_scratch;
    float *out = a.out + io, *out_hi = a.out_hi + io, *out_lo = a.out_lo + io;
    // four coefficients per thread and step: 100 per cell keeps every float4 inside one cell,
    // and every base (slot, set, output cell) is a multiple of 4 floats
    static_assert(NRC % 4 == 0, "float4 steps stay inside a cell");
    for (int e4 = threadIdx.x; e4 < NC * NRC / 4; e4 += blockDim.x) {
        const int e = 4 * e4;
        const int cell = ct.x * NC + e / NRC;
        if (cell >= a.n_out) continue;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        for (int u = 0; u < ct.z; u++) {
            const float4 w = __ldg(reinterpret_cast<const float4 *>(scratch + (size_t)(ct.y + u) * NC * NRC + e));
            v.x += w.x; v.y += w.y; v.z += w.z; v.w += w.w;
        }
        const size_t o = (size_t)(a.out0 + cell) * NRC + e % NRC;
        if (a.accumulate) {
            const float4 b = *reinterpret_cast<const float4 *>(out + o);
            v.x += b.x; v.y += b.y; v.z += b.z; v.w += b.w;
        }
        *reinterpret_cast<float4 *>(out + o) = v;
        const float4 h = make_float4(tf32_rn(v.x), tf32_rn(v.y), tf32_rn(v.z), tf32_rn(v.w));
        *reinterpret_cast<float4 *>(out_hi + o) = h;
        *reinterpret_cast<float4 *>(out_lo + o) = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
    }
}

// Failure-path probe: an mbarrier on which nothing ever arrives. The bounded wait must
// expire (about 1 s), record FG_ETIMEDOUT in *err and return.
__global__ void k_mbar_timeout_probe(int *err) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ volatile int bail;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        bail = 0;
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait(&bar, 0, err, &bail);
}

}  // namespace

// Tensor-pipe throughput of kind::tf32, the instruction of the translations: one CTA per SM
// issues `iters` MMAs of M = 128, N = n, K = 8 from fixed shared-memory operands (FP32 ones,
// the no-swizzle K-major layout of the translations) into one TMEM accumulator and waits
// (bounded) for their completion; cyc[block] = clock64 cycles from the first issue to the
// completion (-1 when the wait expired).
__global__ void __launch_bounds__(128, 1) k_peak_mma_tf32(int n, int iters, long long *cyc, int *err) {
    extern __shared__ unsigned char smem_raw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t done;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int bail;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int a_bytes = 16 * (int)SBO, b_bytes = (n / 8) * (int)SBO;  // K = 16 of A (128 rows) and B (n rows)
    for (int e = tid; e < (a_bytes + b_bytes) / 4; e += blockDim.x) reinterpret_cast<float *>(sm)[e] = 1.0f;
    if (tid == 0) {
        mbar_init(&done, 1);
        bail = 0;
        fence_mbar_init();
    }
    if (warp == 0) tmem_alloc(&tmem_base, 256);
    fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    if (tid == 0) {
        const uint32_t idesc = idesc_tf32(MR, n);
        const uint32_t base = smem_u32(sm);
        const uint64_t a0 = sdesc(base), a1 = sdesc(base + 256);
        const uint64_t b0 = sdesc(base + a_bytes), b1 = sdesc(base + a_bytes + 256);
        const long long t0 = clock64();
        for (int i = 0; i < iters; i++) mma_tf32(tmem, (i & 1) ? a1 : a0, (i & 1) ? b1 : b0, idesc, i > 0 ? 1u : 0u);
        mma_commit(&done);
        const bool ok = mbar_wait(&done, 0, err, &bail);
        const long long t1 = clock64();
        if (!ok) mbar_drain(&done, 0);  // the MMAs still own TMEM: wait again before freeing it
        cyc[blockIdx.x] = ok ? t1 - t0 : -1;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 256);
    }
}

int peak_mma_smem() { return 120 * 1024; }  // one CTA per SM

cudaError_t launch_peak_mma_tf32(cudaStream_t st, int grid, int n, int iters, long long *cyc, int *err) {
    if (n % 16 != 0 || n < 16 || n > 256) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_peak_mma_tf32, cudaFuncAttributeMaxDynamicSharedMemorySize, peak_mma_smem());
    if (e != cudaSuccess) return e;
    k_peak_mma_tf32<<<grid, 128, peak_mma_smem(), st>>>(n, iters, cyc, err);
    return cudaGetLastError();
}

cudaError_t launch_mbar_timeout_probe(cudaStream_t st, int *err) {
    k_mbar_timeout_probe<<<1, 32, 0, st>>>(err);
    return cudaGetLastError();
}

int translate_tc_smem() { return NSTAGE * STAGE_BYTES + 1024; }
int translate_tc_tile() { return NC; }

cudaError_t translate_tc_setup() {
    cudaError_t e = cudaFuncSetAttribute(k_m2m_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, translate_tc_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_m2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, translate_tc_smem());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_l2l_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, translate_tc_smem());
    return e;
}

cudaError_t launch_translate_tc(cudaStream_t st, const TcArgs &a) {
    if (a.n_out <= 0 || a.nunits <= 0) return cudaSuccess;
    auto k = a.accumulate ? k_l2l_tc : (a.ncode == 8 ? k_m2m_tc : k_m2l_tc);
    if (a.nset > NSET) return cudaErrorInvalidValue;
    const unsigned nset = a.nset > 1 ? (unsigned)a.nset : 1u;
    k<<<a.nunits, 288, translate_tc_smem(), st>>>(a);  // every CTA takes all sets of its tile
    if (a.ncomb > 0) k_tc_combine<<<dim3(a.ncomb, nset), 256, 0, st>>>(a);
    return cudaGetLastError();
}

void translate_tc_units(int n_out, int ncode, const int *tab, int out0, int max_codes, std::vector<int> &codes,
                        std::vector<int4> &units, std::vector<int4> &comb, int &nslot) {
    const int ntile = (n_out + NC - 1) / NC;
    for (int b = 0; b < ntile; b++) {
        const int first = (int)codes.size();
        const int c0 = b * NC, c1 = std::min(n_out, c0 + NC);
        for (int code = 0; code < ncode; code++) {
            bool any = false;
            for (int cc = c0; cc < c1 && !any; cc++) any = tab[(size_t)(out0 + cc) * ncode + code] >= 0;
            if (any) codes.push_back(code);
        }
        const int n = (int)codes.size() - first;
        const int nu = std::max(1, (n + max_codes - 1) / max_codes);
        if (nu == 1) {
            units.push_back(make_int4(b, first, first + n, -1));
        } else {
            comb.push_back(make_int4(b, nslot, nu, 0));
            for (int u = 0; u < nu; u++)
                units.push_back(make_int4(b, first + (int)((long)n * u / nu), first + (int)((long)n * (u + 1) / nu),
                                          nslot + u));
            nslot += nu;
        }
    }
}

// Pre-split operator images: for each code and item (K = 16), the hi and lo parts of
// operator rows 0..103 exactly as the MMA reads them from shared memory (core matrix
// (g, kq) at g*SBO + kq*128, row r of the group at + 16 r, four K values per row).
std::vector<float> translate_tc_images(const std::vector<double> &ops, int ncode) {
    std::vector<float> img((size_t)ncode * IPC * 2 * (IMG_BYTES / 4), 0.f);
    for (int code = 0; code < ncode; code++)
        for (int q = 0; q < IPC; q++) {
            float *hi = img.data() + ((size_t)code * IPC + q) * 2 * (IMG_BYTES / 4);
            float *lo = hi + IMG_BYTES / 4;
            for (int i = 0; i < NRC; i++)
                for (int kk = 0; kk < KI; kk++) {
                    const int j = KI * q + kk;
                    if (j >= NRC) continue;
                    const float v = (float)ops[((size_t)code * NRC + i) * NRC + j];
                    uint32_t bits;
                    std::memcpy(&bits, &v, 4);
                    bits = (bits + 0x1000u) & 0xFFFFE000u;
                    float h;
                    std::memcpy(&h, &bits, 4);
                    const size_t off = ((i >> 3) * SBO + (kk >> 2) * 128 + (i & 7) * 16 + (kk & 3) * 4) / 4;
                    hi[off] = h;
                    lo[off] = v - h;
                }
        }
    return img;
}

}  // namespace fg

extern "C" int fg_debug_tc_resources(int attrs[8]) {
    using namespace fg;
    if (!attrs) return FG_EINVAL;
    if (translate_tc_setup() != cudaSuccess) return FG_ECUDA;
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, k_m2l_tc) != cudaSuccess) return FG_ECUDA;
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_m2l_tc, 288, translate_tc_smem()) != cudaSuccess)
        blocks = -1;
    attrs[0] = fa.numRegs;
    attrs[1] = fa.maxThreadsPerBlock;
    attrs[2] = (int)fa.sharedSizeBytes;
    attrs[3] = fa.maxDynamicSharedSizeBytes;
    attrs[4] = (int)fa.localSizeBytes;
    attrs[5] = translate_tc_smem();
    attrs[6] = 288;
    attrs[7] = blocks;
    cudaGetLastError();
    return FG_OK;
}

// Diagnostic entry: one tensor-core translation launch on caller data (host arrays),
// out[c] = sum_code ops[code] in[tab[c][code]] for n_out cells, with the chosen product
// terms of the hi/lo split. Returns FG_* status.
extern "C" int fg_debug_translate_tc(int n_in, int n_out, int ncode, const float *ops, const int *tab,
                                     const float *in, float *out, int terms) {
    using namespace fg;
    if (n_in <= 0 || n_out <= 0 || ncode <= 0 || !ops || !tab || !in || !out) return FG_EINVAL;
    for (long k = 0; k < (long)n_out * ncode; k++)
        if (tab[k] < -1 || tab[k] >= n_in) return FG_EINVAL;
    std::vector<int> codes;
    std::vector<int4> units, comb;
    int nslot = 0;
    translate_tc_units(n_out, ncode, tab, 0, 3, codes, units, comb, nslot);  // small units: exercise the combine
    const std::vector<double> opd(ops, ops + (size_t)ncode * NRC * NRC);
    const std::vector<float> img = translate_tc_images(opd, ncode);
    std::vector<float> xh((size_t)n_in * NRC), xl((size_t)n_in * NRC);
    for (size_t k = 0; k < xh.size(); k++) {
        uint32_t bits;
        std::memcpy(&bits, &in[k], 4);
        bits = (bits + 0x1000u) & 0xFFFFE000u;
        std::memcpy(&xh[k], &bits, 4);
        xl[k] = in[k] - xh[k];
    }
    float *d_img = nullptr, *d_xh = nullptr, *d_xl = nullptr, *d_out = nullptr, *d_oh = nullptr, *d_ol = nullptr;
    int *d_tab = nullptr, *d_code = nullptr, *d_err = nullptr;
    int4 *d_units = nullptr, *d_comb = nullptr;
    float *d_scr = nullptr;
    int status = FG_OK, herr = 0;
    auto ok = [&](cudaError_t e) { if (e != cudaSuccess && status == FG_OK) status = FG_ECUDA; return e == cudaSuccess; };
    const size_t nx = (size_t)n_in * NRC, no = (size_t)n_out * NRC;
    if (ok(cudaMalloc(&d_img, sizeof(float) * img.size())) && ok(cudaMalloc(&d_xh, sizeof(float) * nx)) &&
        ok(cudaMalloc(&d_xl, sizeof(float) * nx)) && ok(cudaMalloc(&d_out, sizeof(float) * no)) &&
        ok(cudaMalloc(&d_oh, sizeof(float) * no)) && ok(cudaMalloc(&d_ol, sizeof(float) * no)) &&
        ok(cudaMalloc(&d_tab, sizeof(int) * (size_t)n_out * ncode)) &&
        ok(cudaMalloc(&d_units, sizeof(int4) * units.size())) &&
        ok(cudaMalloc(&d_comb, sizeof(int4) * std::max<size_t>(1, comb.size()))) &&
        ok(cudaMalloc(&d_scr, sizeof(float) * std::max(1, nslot) * NC * NRC)) &&
        ok(cudaMalloc(&d_code, sizeof(int) * std::max<size_t>(1, codes.size()))) &&
        ok(cudaMalloc(&d_err, sizeof(int))) &&
        ok(cudaMemcpy(d_img, img.data(), sizeof(float) * img.size(), cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_xh, xh.data(), sizeof(float) * nx, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_xl, xl.data(), sizeof(float) * nx, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_tab, tab, sizeof(int) * (size_t)n_out * ncode, cudaMemcpyHostToDevice)) &&
        ok(cudaMemcpy(d_units, units.data(), sizeof(int4) * units.size(), cudaMemcpyHostToDevice)) &&
        (comb.empty() || ok(cudaMemcpy(d_comb, comb.data(), sizeof(int4) * comb.size(), cudaMemcpyHostToDevice))) &&
        (codes.empty() || ok(cudaMemcpy(d_code, codes.data(), sizeof(int) * codes.size(), cudaMemcpyHostToDevice))) &&
        ok(cudaMemset(d_err, 0, sizeof(int))) && ok(translate_tc_setup())) {
        TcArgs a{};
        a.n_out = n_out; a.out0 = 0; a.ncode = ncode; a.tab = d_tab;
        a.op_img = reinterpret_cast<const unsigned char *>(d_img);
        a.in_hi = d_xh; a.in_lo = d_xl; a.out = d_out; a.out_hi = d_oh; a.out_lo = d_ol;
        a.accumulate = 0; a.tile_code = d_code; a.err = d_err; a.terms = terms;
        a.units = d_units; a.nunits = (int)units.size(); a.scratch = d_scr;
        a.comb = d_comb; a.ncomb = (int)comb.size();
        if (ok(launch_translate_tc(0, a)) && ok(cudaDeviceSynchronize()) &&
            ok(cudaMemcpy(out, d_out, sizeof(float) * no, cudaMemcpyDeviceToHost)) &&
            ok(cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost)) && herr)
            status = FG_ETIMEDOUT;
    }
    void *ptrs[] = {d_img, d_xh, d_xl, d_out, d_oh, d_ol, d_tab, d_code, d_err, d_units, d_comb, d_scr};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    return status;
}
