// Morton keys and their radix sort on the device: the ordering step of the FMM octree
// build. The reference hands its points to ScalFMM, which sorts them into its octree by
// Morton index (src/fmm_demag.h:52-80 inserts the scaled source and target points); here
// every point gets the 64-bit key (sample << 3L) | morton(cell at depth L), computed from
// the sample's root cube, and the (key, point index) pairs are sorted by a stable LSD radix
// sort, 8 bits per pass, over only the bits the keys use. Stable and fed in index order, it
// yields the order of a comparison sort of the pairs (key, then index): the host builds the
// same octree tables from it as from std::sort.
#include <cstdint>
#include <vector>

#include "fg_internal.h"

namespace fg {

namespace {

constexpr int SORT_THREADS = 256;
constexpr int SORT_ROUNDS = 16;  // items per thread and tile: a tile is 4096 pairs
constexpr int SORT_TILE = SORT_THREADS * SORT_ROUNDS;

__device__ __forceinline__ uint64_t spread3(uint32_t v) {
    // bit k of v to bit 3k (v < 2^21)
    uint64_t x = v & 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

// Key of point k: its sample in the bits above 3L, the Morton code of its cell at depth L
// below (x in the lowest bit of every triple, as the host's morton()). Points with
// keep[k] == 0 get the largest key and sort to the end.
__global__ void k_morton_keys(int n, int L, const double *__restrict__ xyz, const int *__restrict__ seg,
                              const double4 *__restrict__ root, const unsigned char *__restrict__ keep,
                              uint64_t *__restrict__ key, int *__restrict__ idx) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    idx[k] = k;
    if (keep && !keep[k]) {
        key[k] = ~0ull;
        return;
    }
    const int g = seg ? seg[k] : 0;
    const double4 R = root[g];  // centre x, y, z and side of the sample's root cube
    const int nside = 1 << L;
    const double c[3] = {R.x, R.y, R.z};
    uint32_t ijk[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        // ((p - c) / side + 1/2) * nside, each operation rounded as on the host (no contraction)
        const double q = __dmul_rn(__dadd_rn(__ddiv_rn(__dsub_rn(xyz[3 * (size_t)k + d], c[d]), R.w), 0.5), (double)nside);
        const int v = (int)q;
        ijk[d] = (uint32_t)min(nside - 1, max(0, v));
    }
    key[k] = ((uint64_t)g << (3 * L)) | spread3(ijk[0]) | (spread3(ijk[1]) << 1) | (spread3(ijk[2]) << 2);
}

// Histogram of the digit (key >> shift) & 255 over each tile, digit-major: hist[d * nblk + b].
__global__ void __launch_bounds__(SORT_THREADS) k_digit_hist(int n, int shift, const uint64_t *__restrict__ key,
                                                              int *__restrict__ hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ROUNDS; r++) {
        const int k = base + r * SORT_THREADS + threadIdx.x;
        if (k < n) atomicAdd(&h[(int)((key[k] >> shift) & 255)], 1);
    }
    __syncthreads();
    hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m counts in one block of 1024 threads (m is 256 x tiles: a few
// hundred thousand at most for the meshes of this library).
__global__ void __launch_bounds__(1024) k_scan_counts(int m, int *__restrict__ a) {
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int chunk = (m + 1023) / 1024;
    const int lo = min(m, t * chunk), hi = min(m, lo + chunk);
    int s = 0;
    for (int k = lo; k < hi; k++) s += a[k];
    part[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int v = t >= off ? part[t - off] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = part[t] - s;
    for (int k = lo; k < hi; k++) {
        const int v = a[k];
        a[k] = run;
        run += v;
    }
}

// Stable scatter of each tile by digit: the tile is read in rounds of 256 pairs (round-major,
// then warp, then lane), so a pair's rank among the tile's pairs of the same digit is the
// count of those before it in that order.
__global__ void __launch_bounds__(SORT_THREADS) k_digit_scatter(int n, int shift, const uint64_t *__restrict__ key,
                                                                 const int *__restrict__ val,
                                                                 const int *__restrict__ offs,
                                                                 uint64_t *__restrict__ key_out,
                                                                 int *__restrict__ val_out) {
    constexpr int NW = SORT_THREADS / 32;
    __shared__ int base[256];
    __shared__ int cnt[NW][256];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    base[t] = offs[t * gridDim.x + blockIdx.x];
    const unsigned lt = (1u << lane) - 1u;
    const int tile = blockIdx.x * SORT_TILE;
    for (int r = 0; r < SORT_ROUNDS; r++) {
#pragma unroll
        for (int q = 0; q < NW; q++) cnt[q][t] = 0;
        __syncthreads();
        const int k = tile + r * SORT_THREADS + t;
        const bool valid = k < n;
        uint64_t kv = 0;
        int vv = 0, d = 256;  // 256: no pair (never matches a digit)
        if (valid) {
            kv = key[k];
            vv = val[k];
            d = (int)((kv >> shift) & 255);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt);
        if (valid && rank == 0) cnt[w][d] = __popc(peers);
        __syncthreads();
        {
            // thread t owns digit t: the offsets of each warp's pairs of that digit in this round
            int run = base[t];
#pragma unroll
            for (int q = 0; q < NW; q++) {
                const int c = cnt[q][t];
                cnt[q][t] = run;
                run += c;
            }
            base[t] = run;
        }
        __syncthreads();
        if (valid) {
            const int pos = cnt[w][d] + rank;
            key_out[pos] = kv;
            val_out[pos] = vv;
        }
        __syncthreads();
    }
}

}  // namespace

// Sorted keys and point indices of n points (xyz on the device, seg: sample of each point on
// the device or nullptr, roots[g] = centre and side of sample g's root cube, keep: 0 for the
// points to leave out, nullptr to keep all). On return keys/idx hold the kept pairs in key order;
// *dev_ms adds the device time of the key and sort kernels.
cudaError_t morton_sort(Ctx &c, int n, int L, int nseg, const double *xyz, const int *seg,
                        const std::vector<double4> &roots, const unsigned char *keep, std::vector<uint64_t> &keys,
                        std::vector<int> &idx, double *dev_ms) {
    keys.clear();
    idx.clear();
    if (n <= 0) return cudaSuccess;
    // sorted bits: the cell's 3L and enough above them for the sample ids, and for one id more
    // when points are left out (their key, all ones, then sorts strictly after every kept key)
    int bits = 3 * L;
    while ((1ll << (bits - 3 * L)) < (long long)nseg + (keep ? 1 : 0)) bits++;
    const int passes = (bits + 7) / 8;
    const int nblk = (n + SORT_TILE - 1) / SORT_TILE;
    uint64_t *k0 = nullptr, *k1 = nullptr;
    int *v0 = nullptr, *v1 = nullptr, *hist = nullptr;
    double4 *droot = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaSuccess;
    auto ok = [&](cudaError_t x) {
        if (e == cudaSuccess && x != cudaSuccess) e = x;
        return e == cudaSuccess;
    };
    if (ok(cudaMalloc(&k0, sizeof(uint64_t) * n)) && ok(cudaMalloc(&k1, sizeof(uint64_t) * n)) &&
        ok(cudaMalloc(&v0, sizeof(int) * n)) && ok(cudaMalloc(&v1, sizeof(int) * n)) &&
        ok(cudaMalloc(&hist, sizeof(int) * 256 * (size_t)nblk)) && ok(cudaMalloc(&droot, sizeof(double4) * roots.size())) &&
        ok(cudaEventCreate(&e0)) && ok(cudaEventCreate(&e1)) &&
        ok(cudaMemcpyAsync(droot, roots.data(), sizeof(double4) * roots.size(), cudaMemcpyHostToDevice, c.stream)) &&
        ok(cudaEventRecord(e0, c.stream))) {
        k_morton_keys<<<(n + 255) / 256, 256, 0, c.stream>>>(n, L, xyz, seg, droot, keep, k0, v0);
        ok(cudaGetLastError());
        for (int p = 0; p < passes && e == cudaSuccess; p++) {
            const int shift = 8 * p;
            k_digit_hist<<<nblk, SORT_THREADS, 0, c.stream>>>(n, shift, k0, hist);
            k_scan_counts<<<1, 1024, 0, c.stream>>>(256 * nblk, hist);
            k_digit_scatter<<<nblk, SORT_THREADS, 0, c.stream>>>(n, shift, k0, v0, hist, k1, v1);
            if (!ok(cudaGetLastError())) break;
            std::swap(k0, k1);
            std::swap(v0, v1);
        }
        if (ok(cudaEventRecord(e1, c.stream))) {
            keys.resize(n);
            idx.resize(n);
            if (ok(cudaMemcpyAsync(keys.data(), k0, sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, c.stream)) &&
                ok(cudaMemcpyAsync(idx.data(), v0, sizeof(int) * n, cudaMemcpyDeviceToHost, c.stream)) &&
                ok(cudaStreamSynchronize(c.stream))) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (dev_ms) *dev_ms += ms;
            }
        }
    }
    if (e == cudaSuccess && keep) {
        size_t m = keys.size();
        while (m > 0 && keys[m - 1] == ~0ull) m--;
        keys.resize(m);
        idx.resize(m);
    }
    void *bufs[] = {k0, k1, v0, v1, hist, droot};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return e;
}

}  // namespace fg
