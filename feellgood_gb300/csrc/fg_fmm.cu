// Fast multipole evaluation of the demagnetising potential on the GPU.
//
// Replaces the ScalFMM octree + rotation kernel that fmm::demag calls
// (src/fmm_demag.h:184-224: P2M, M2M, M2L, L2L, L2P of 1/r plus the P2P near field).
// The potential computed is the same sum pot_i = sum_s q_s / |x_i - y_s| over the
// Gauss-point sources; only the evaluator differs.
//
// Expansions use the scaled solid harmonics
//   Ups_n^m(r) = (-1)^m r^n P_n^m(cos t) e^{i m p} / (n+m)!        (regular)
//   The_n^m(r) = (-1)^m (n-m)! P_n^m(cos t) e^{i m p} / r^{n+1}     (irregular)
// (P_n^m with the Condon-Shortley phase), for which 1/|x-y| = sum Ups_n^m*(y) The_n^m(x),
// Ups(a+b) = sum_kl Ups_k^l(a) Ups_{n-k}^{m-l}(b) and The(x-y) = sum Ups_k^l*(y) The_{n+k}^{m+l}(x).
// Multipoles M_n^m = sum q Ups_n^m*(y - z); locals F_n^m with phi = sum F_n^m Ups_n^m*(x - z).
// For real charges X_n^-m = (-1)^m conj X_n^m, so each expansion is stored as (P+1)^2 reals:
// Re X_n^0, then Re/Im X_n^m for m = 1..n. Coefficients of a cell of width w are stored
// scaled (M/w^n, F*w^(n+1)), which makes every translation independent of the level.
//
// Every translation (M2L for each of the 316 cell offsets, M2M and L2L for the 8 child
// octants) is then a fixed real 100x100 matrix, built once on the host. One kernel applies
// them: a block owns 64 output cells, walks the operator codes, gathers the 64 input
// expansions of that code and accumulates a register-tiled 100x100 x 100x64 product in a
// fixed order (deterministic, no atomics).
//
// The octree is uniform (all leaves on one level) and built once per mesh on the host
// (geometry is static). Interaction lists follow the one-cell separation: M2L over the
// children of the parent's neighbours that are not adjacent, P2P over adjacent leaves.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <queue>
#include <vector>

#include "fg_ds.cuh"
#include "fg_f32x2.cuh"
#include "fg_internal.h"

namespace fg {

constexpr int FMM_P = 9;
constexpr int NR = (FMM_P + 1) * (FMM_P + 1);  // reals per expansion (100)
constexpr int NCODE_M2L = 343;                   // offsets in [-3,3]^3 (27 unused)
// CUDA-core translations: output cells per block and per thread. FP64 uses narrow blocks
// of 16 cells (the FP64 pipe bounds them, so operator reuse matters less than spreading
// the blocks evenly over the SMs, two per SM); FP32 blocks of 64 cells.
template <typename T> struct TrShape;
template <> struct TrShape<float> { static constexpr int TB = 64, CT = 4; };
template <> struct TrShape<double> { static constexpr int TB = 16, CT = 1; };
template <typename T> constexpr int tr_smem() { return (int)((100 * 100 + 100 * (TrShape<T>::TB + 4)) * sizeof(T)); }

__host__ __device__ constexpr int cidx(int n, int m) { return n * (n + 1) / 2 + m; }
// real layout: Re X_n^0 at n*n; Re/Im X_n^m (m>0) at n*n + 2m-1, n*n + 2m
__host__ __device__ constexpr int ridx(int n, int m, int part) { return m == 0 ? n * n : n * n + 2 * m - 1 + part; }

struct FmmTree {
    int L = 0, nleaf = 0, ncell = 0, leaf0 = 0, nsrc = 0;
    double s0 = 1, c0[3] = {0, 0, 0};
    std::vector<int> lev_begin;
    size_t n_m2l = 0, n_p2p_pairs = 0;
    bool fp32 = false;
    double eval_ms = 0;
    // profiling: two sets of stage events used in turn (recorded without synchronising); a
    // set is read back when it is about to be reused or when the timings are requested
    cudaEvent_t ev[2][6] = {};
    cudaEvent_t evn[2][2] = {};          // the near field on the second stream (overlapped evaluation)
    bool ev_pending[2] = {false, false};
    bool ev_split[2] = {false, false};  // the set timed an overlapped evaluation
    int ev_next = 0;
    double stage_sum[5] = {0, 0, 0, 0, 0};
    long long stage_n = 0;
    // device
    int *leaf_src = nullptr, *leaf_tgt = nullptr, *tgt_node = nullptr;
    void *sloc = nullptr;  // 4 x nsrc: leaf-local source coordinates (T), w: charge of set 0
    void *tloc = nullptr;  // 4 x ntgt: leaf-local target coordinates (T)
    // FP64 path, near field in double-single arithmetic: every coordinate split as
    // hi (on a 2^-20 grid of leaf units) + lo, the charge as hi + lo; (x, y, z, q) per part
    bool ds = false;
    float4 *ds_src_hi = nullptr, *ds_src_lo = nullptr, *ds_tgt_hi = nullptr, *ds_tgt_lo = nullptr;
    int *leaf_ijk = nullptr;  // 3 x nleaf integer leaf coordinates (within the leaf's own tree)
    double *leaf_scale = nullptr;  // 1 / physical leaf width of the leaf's tree
    int *m2l_tab = nullptr;   // [ncell][343] source cell or -1
    int *m2m_tab = nullptr;   // [ncell][8] child per octant or -1
    int *l2l_tab = nullptr;   // [ncell][8] parent at the own octant, -1 elsewhere
    int *near_ptr = nullptr, *near_leaf = nullptr;
    void *M = nullptr, *F = nullptr;
    void *op_m2l = nullptr, *op_m2m = nullptr, *op_l2l = nullptr;  // [code][NR][NR] (out x in)
    // tensor-core translations (FP32 path): per launch, for each tile of 64 output cells,
    // the list of operator codes that bring any input to the tile
    bool tc = false;
    int *tc_code = nullptr;                      // codes per tile, all launches
    int4 *tc_units = nullptr, *tc_comb = nullptr;
    float *tc_scratch = nullptr;
    struct TcLaunch { int unit0 = 0, nunit = 0, comb0 = 0, ncomb = 0; };
    std::vector<TcLaunch> tc_m2m, tc_l2l;        // per level
    TcLaunch tc_m2l;
    int *tc_err = nullptr;                       // FG_ETIMEDOUT when a pipeline wait expired
    float *Mh = nullptr, *Ml = nullptr, *Fh = nullptr, *Fl = nullptr;  // hi/lo splits of M and F
    unsigned char *img_m2l = nullptr, *img_m2m = nullptr, *img_l2l = nullptr;  // operator images
    int *dst_keep = nullptr;
    // charge sets evaluated together (2: demag of m and of v in one pass): M, F, Mh, Ml, Fh,
    // Fl and tc_scratch hold nq sets one after the other; the second set's charges for the
    // near field are in sq2 (T) and, double-single, in ds_q2 (hi [nsrc] then lo [nsrc])
    int nq = 1;
    void *sq2 = nullptr;
    float *ds_q2 = nullptr;
    size_t nslot_floats = 0;  // floats of tc_scratch per set
};

// ---------------------------------------------------------------------------------
// host: complex operators (checked against a direct sum in the tests)

using cd = std::complex<double>;

static void ups_host(double x, double y, double z, int P, std::vector<cd> &U) {
    const double r2 = x * x + y * y + z * z;
    U.assign((P + 1) * (P + 2) / 2, 0.0);
    U[0] = 1.0;
    const cd w(x, y);
    for (int m = 0; m <= P; m++) {
        if (m > 0) U[cidx(m, m)] = w / (2.0 * m) * U[cidx(m - 1, m - 1)];
        if (m + 1 <= P) U[cidx(m + 1, m)] = z * U[cidx(m, m)];
        for (int n = m + 2; n <= P; n++)
            U[cidx(n, m)] = ((2.0 * n - 1) * z * U[cidx(n - 1, m)] - r2 * U[cidx(n - 2, m)]) / double((n + m) * (n - m));
    }
}
static void the_host(double x, double y, double z, int P, std::vector<cd> &T) {
    const double r2 = x * x + y * y + z * z, ir2 = 1.0 / r2;
    T.assign((P + 1) * (P + 2) / 2, 0.0);
    T[0] = 1.0 / std::sqrt(r2);
    const cd w(x, y);
    for (int m = 0; m <= P; m++) {
        if (m > 0) T[cidx(m, m)] = (2.0 * m - 1) * w * ir2 * T[cidx(m - 1, m - 1)];
        if (m + 1 <= P) T[cidx(m + 1, m)] = (2.0 * m + 1) * z * ir2 * T[cidx(m, m)];
        for (int n = m + 2; n <= P; n++)
            T[cidx(n, m)] = ((2.0 * n - 1) * z * T[cidx(n - 1, m)] - double((n + m - 1) * (n - m - 1)) * T[cidx(n - 2, m)]) * ir2;
    }
}
static inline cd getc(const std::vector<cd> &A, int n, int m) {
    if (m >= 0) return A[cidx(n, m)];
    const cd v = std::conj(A[cidx(n, -m)]);
    return (m & 1) ? -v : v;
}
static void to_complex(const double *r, int P, std::vector<cd> &A) {
    A.assign((P + 1) * (P + 2) / 2, 0.0);
    for (int n = 0; n <= P; n++)
        for (int m = 0; m <= n; m++) A[cidx(n, m)] = m == 0 ? cd(r[ridx(n, 0, 0)], 0) : cd(r[ridx(n, m, 0)], r[ridx(n, m, 1)]);
}
static void to_real(const std::vector<cd> &A, int P, double *r) {
    for (int n = 0; n <= P; n++)
        for (int m = 0; m <= n; m++) {
            r[ridx(n, m, 0)] = A[cidx(n, m)].real();
            if (m) r[ridx(n, m, 1)] = A[cidx(n, m)].imag();
        }
}
// F_n^m = (-1)^n sum_kl M_k^l The_{n+k}^{m+l}(t), t = target centre - source centre (cell units)
static void m2l_c(const std::vector<cd> &M, const std::vector<cd> &T, int P, std::vector<cd> &F) {
    F.assign((P + 1) * (P + 2) / 2, 0.0);
    for (int n = 0; n <= P; n++)
        for (int m = 0; m <= n; m++) {
            cd s = 0;
            for (int k = 0; k <= P; k++)
                for (int l = -k; l <= k; l++) s += getc(M, k, l) * getc(T, n + k, m + l);
            F[cidx(n, m)] = (n & 1) ? -s : s;
        }
}
// parent M from a child: M_n^m = sum conj(Ups_k^l(t)) 2^-(n-k) M_{n-k}^{m-l}, t = child - parent (parent units)
static void m2m_c(const std::vector<cd> &M, const std::vector<cd> &U, int P, std::vector<cd> &O) {
    O.assign((P + 1) * (P + 2) / 2, 0.0);
    for (int n = 0; n <= P; n++)
        for (int m = 0; m <= n; m++) {
            cd s = 0;
            for (int k = 0; k <= n; k++)
                for (int l = -k; l <= k; l++)
                    if (std::abs(m - l) <= n - k) s += std::conj(getc(U, k, l)) * std::ldexp(1.0, -(n - k)) * getc(M, n - k, m - l);
            O[cidx(n, m)] = s;
        }
}
// child F from the parent: F_k^l = sum_{n>=k} F_n^m 2^-(k+1) conj(Ups_{n-k}^{m-l}(t)), t = child - parent
static void l2l_c(const std::vector<cd> &F, const std::vector<cd> &U, int P, std::vector<cd> &O) {
    O.assign((P + 1) * (P + 2) / 2, 0.0);
    for (int k = 0; k <= P; k++)
        for (int l = 0; l <= k; l++) {
            cd s = 0;
            for (int n = k; n <= P; n++)
                for (int m = -n; m <= n; m++)
                    if (std::abs(m - l) <= n - k) s += getc(F, n, m) * std::conj(getc(U, n - k, m - l));
            O[cidx(k, l)] = s * std::ldexp(1.0, -(k + 1));
        }
}

// ---------------------------------------------------------------------------------
// device

template <typename T, int M, typename Fn>
__device__ __forceinline__ void ups_col(T x, T y, T z, T r2, T &dre, T &dim, Fn &f) {
    if constexpr (M > 0) {
        const T s = T(1) / T(2 * M);
        const T nre = (x * dre - y * dim) * s, nim = (x * dim + y * dre) * s;
        dre = nre;
        dim = nim;
    }
    f(M, M, dre, dim);
    if constexpr (M + 1 <= FMM_P) {
        T p2re = dre, p2im = dim;
        T p1re = z * dre, p1im = z * dim;
        f(M + 1, M, p1re, p1im);
#pragma unroll
        for (int n = M + 2; n <= FMM_P; n++) {
            const T a = T(2 * n - 1), b = T(1) / T((n + M) * (n - M));
            const T cre = (a * z * p1re - r2 * p2re) * b, cim = (a * z * p1im - r2 * p2im) * b;
            f(n, M, cre, cim);
            p2re = p1re; p2im = p1im;
            p1re = cre; p1im = cim;
        }
    }
    if constexpr (M < FMM_P) ups_col<T, M + 1>(x, y, z, r2, dre, dim, f);
}

// Every Ups_n^m(x, y, z), 0 <= m <= n <= P, passed to f(n, m, re, im) by the recurrences
// in m (diagonal) and n (columns); the column index m is a template parameter so that
// callers accumulating into register arrays see constant indices.
template <typename T, typename Fn>
__device__ __forceinline__ void ups_cols(T x, T y, T z, Fn &&f) {
    const T r2 = x * x + y * y + z * z;
    T dre = 1, dim = 0;
    ups_col<T, 0>(x, y, z, r2, dre, dim, f);
}


// P2M: one warp per leaf; each lane forms q*conj(Ups) of every 32nd source of the leaf into
// 100 register accumulators, which are then reduced over the warp in a fixed order (lane
// k mod 32 stores coefficient k). The charge is also stored for the near field (beside the
// source coordinates for the first set), and with the tensor-core translations the hi/lo
// split of M. Grid y selects the charge set.
template <typename T>
struct P2mSet {
    const double *q;        // charges (storage order)
    const float *qf;        // FP32 charges read instead of q (FP32 path, incremental demag), or nullptr
    T *M;                   // expansions of this set
    float *Mh, *Ml;         // their split (tensor-core translations) or nullptr
    T *qn;                  // charge for the near field, element s at qn[s * qn_stride]
    int qn_stride;
    float *qh, *ql;         // double-single charge for the FP64 near field (or nullptr)
    int qd_stride;
};

template <typename T>
__global__ void __launch_bounds__(128) k_p2m(int nleaf, const int *__restrict__ leaf_src, const T *__restrict__ sloc,
                                             int leaf0, P2mSet<T> set0, P2mSet<T> set1) {
    const P2mSet<T> st = blockIdx.y ? set1 : set0;
    const int lane = threadIdx.x & 31;
    const int leaf = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (leaf >= nleaf) return;
    const int s0 = leaf_src[leaf], s1 = leaf_src[leaf + 1];
    const double *__restrict__ q = st.q;
    T acc[NR];
#pragma unroll
    for (int k = 0; k < NR; k++) acc[k] = 0;
    for (int s = s0 + lane; s < s1; s += 32) {
        const T x = sloc[4 * (size_t)s], y = sloc[4 * (size_t)s + 1], z = sloc[4 * (size_t)s + 2];
        const T qq = T(q[s]);
        st.qn[(size_t)s * st.qn_stride] = qq;
        if (st.qh) {  // charge as hi + lo for the double-single near field
            const float qh = (float)q[s];
            st.qh[(size_t)s * st.qd_stride] = qh;
            st.ql[(size_t)s * st.qd_stride] = (float)(q[s] - (double)qh);
        }
        ups_cols<T>(x, y, z, [&](int n, int m, T re, T im) {
            acc[ridx(n, m, 0)] += qq * re;
            if (m) acc[ridx(n, m, 1)] -= qq * im;
        });
    }
    const size_t base = (size_t)(leaf0 + leaf) * NR;
#pragma unroll
    for (int k = 0; k < NR; k++) {
        T v = acc[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((k & 31) == lane) {
            st.M[base + k] = v;
            if (st.Mh) {  // split for the tensor-core translations: hi = tf32(x), lo = x - hi
                const float xf = (float)v;
                const float hi = __uint_as_float((__float_as_uint(xf) + 0x1000u) & 0xFFFFE000u);
                st.Mh[base + k] = hi;
                st.Ml[base + k] = xf - hi;
            }
        }
    }
}

// The same harmonics restricted to the columns M0..M1 (the diagonal recurrence still runs
// from m = 0): f(n, m, re, im) for M0 <= m <= M1 only, with the values and the order of
// operations of ups_cols.
template <typename T, int M, int M0, int M1, typename Fn>
__device__ __forceinline__ void ups_col_r(T x, T y, T z, T r2, T &dre, T &dim, Fn &f) {
    if constexpr (M > 0) {
        const T s = T(1) / T(2 * M);
        const T nre = (x * dre - y * dim) * s, nim = (x * dim + y * dre) * s;
        dre = nre;
        dim = nim;
    }
    if constexpr (M >= M0) {
        f(M, M, dre, dim);
        if constexpr (M + 1 <= FMM_P) {
            T p2re = dre, p2im = dim;
            T p1re = z * dre, p1im = z * dim;
            f(M + 1, M, p1re, p1im);
#pragma unroll
            for (int n = M + 2; n <= FMM_P; n++) {
                const T a = T(2 * n - 1), b = T(1) / T((n + M) * (n - M));
                const T cre = (a * z * p1re - r2 * p2re) * b, cim = (a * z * p1im - r2 * p2im) * b;
                f(n, M, cre, cim);
                p2re = p1re; p2im = p1im;
                p1re = cre; p1im = cim;
            }
        }
    }
    if constexpr (M < M1) ups_col_r<T, M + 1, M0, M1>(x, y, z, r2, dre, dim, f);
}

// Reals of harmonic column m (n = m..P; real and imaginary parts for m > 0).
__host__ __device__ constexpr int col_reals(int m) { return m == 0 ? FMM_P + 1 : 2 * (FMM_P + 1 - m); }
// Index of (n, m, part) among the reals of the columns M0.. (column-major).
__host__ __device__ constexpr int lidx(int M0, int n, int m, int part) {
    int k = 0;
    for (int c = M0; c < m; c++) k += col_reals(c);
    return k + (m == 0 ? n : 2 * (n - m) + part);
}

// One pass of k_p2m2 over the columns M0..M1 of the NS charge sets of a leaf's sources.
template <int NS, int M0, int M1>
__device__ __forceinline__ void p2m2_pass(int lane, int s0, int s1, const float *__restrict__ sloc, size_t base,
                                          const P2mSet<float> &a, const P2mSet<float> &b) {
    constexpr int NPR = lidx(M0, FMM_P, M1, 1) + 1;
    float acc0[NPR], acc1[NS == 2 ? NPR : 1];
#pragma unroll
    for (int k = 0; k < NPR; k++) acc0[k] = 0.f;
#pragma unroll
    for (int k = 0; k < (NS == 2 ? NPR : 1); k++) acc1[k] = 0.f;
    for (int s = s0 + lane; s < s1; s += 32) {
        const float x = sloc[4 * (size_t)s], y = sloc[4 * (size_t)s + 1], z = sloc[4 * (size_t)s + 2];
        const float qa = a.qf ? a.qf[s] : float(a.q[s]);
        const float qb = NS == 2 ? (b.qf ? b.qf[s] : float(b.q[s])) : 0.f;
        if constexpr (M0 == 0) {  // the charges for the near field, once
            a.qn[(size_t)s * a.qn_stride] = qa;
            if constexpr (NS == 2) b.qn[(size_t)s * b.qn_stride] = qb;
        }
        const float r2 = x * x + y * y + z * z;
        float dre = 1, dim = 0;
        auto f = [&](int n, int m, float re, float im) {
            const int k = lidx(M0, n, m, 0);
            acc0[k] += qa * re;
            if constexpr (NS == 2) acc1[k] += qb * re;
            if (m) {
                acc0[k + 1] -= qa * im;
                if constexpr (NS == 2) acc1[k + 1] -= qb * im;
            }
        };
        ups_col_r<float, 0, M0, M1>(x, y, z, r2, dre, dim, f);
    }
    auto put = [&](const P2mSet<float> &st, int g, float v) {
        st.M[base + g] = v;
        if (st.Mh) {  // split for the tensor-core translations: hi = tf32(x), lo = x - hi
            const float hi = __uint_as_float((__float_as_uint(v) + 0x1000u) & 0xFFFFE000u);
            st.Mh[base + g] = hi;
            st.Ml[base + g] = v - hi;
        }
    };
#pragma unroll
    for (int m = M0; m <= M1; m++)
#pragma unroll
        for (int n = m; n <= FMM_P; n++)
#pragma unroll
            for (int part = 0; part < (m ? 2 : 1); part++) {
                const int k = lidx(M0, n, m, part), g = ridx(n, m, part);
                float v0 = acc0[k], v1 = NS == 2 ? acc1[NS == 2 ? k : 0] : 0.f;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    v0 += __shfl_xor_sync(0xffffffffu, v0, o);
                    if constexpr (NS == 2) v1 += __shfl_xor_sync(0xffffffffu, v1, o);
                }
                if ((g & 31) == lane) {
                    put(a, g, v0);
                    if constexpr (NS == 2) put(b, g, v1);
                }
            }
}

// P2M of the FP32 path, the NS charge sets in one pass over the sources: the harmonics of a
// source are formed once for both sets (k_p2m forms them once per set), in three passes over
// the harmonic columns (0-2, 3-5, 6-9: 88, 72 and 40 register accumulators for two sets)
// that repeat the cheap diagonal recurrence. Each coefficient sums the terms of k_p2m in the
// same order; one set (fg_demag) and two (fg_compute_all) run the same code, so a set's
// expansion does not depend on whether the other is evaluated beside it.
template <int NS>
__global__ void __launch_bounds__(128) k_p2m2(int nleaf, const int *__restrict__ leaf_src,
                                              const float *__restrict__ sloc, int leaf0, P2mSet<float> set0,
                                              P2mSet<float> set1) {
    const int lane = threadIdx.x & 31;
    const int leaf = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (leaf >= nleaf) return;
    const int s0 = leaf_src[leaf], s1 = leaf_src[leaf + 1];
    const size_t base = (size_t)(leaf0 + leaf) * NR;
    p2m2_pass<NS, 0, 2>(lane, s0, s1, sloc, base, set0, set1);
    p2m2_pass<NS, 3, 5>(lane, s0, s1, sloc, base, set0, set1);
    p2m2_pass<NS, 6, FMM_P>(lane, s0, s1, sloc, base, set0, set1);
}

// ---- P2M of the FP64 path in double-single arithmetic -------------------------------
// The harmonics and the accumulation of k_p2m's FP64 form on the FP32 pipes (GB300's FP64
// pipe, 2 DFMA per clock and SM, made the FP64 P2M 9.9 ms of the film's FP64 evaluation):
// the recurrences of ups_cols with every operation a double-single one (about 48 bits), the
// coordinates as the normalised pair of their stored hi + lo parts, the charge split once.

__device__ __forceinline__ dsf dsc(double x) {  // a double constant as a double-single pair
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

template <int M, int M0, int M1, typename Fn>
__device__ __forceinline__ void ups_col_ds(dsf x, dsf y, dsf z, dsf r2, dsf &dre, dsf &dim, Fn &f) {
    if constexpr (M > 0) {
        const dsf s = dsc(1.0 / (2 * M));
        const dsf nre = ds_mul(ds_sub(ds_mul(x, dre), ds_mul(y, dim)), s);
        const dsf nim = ds_mul(ds_add(ds_mul(x, dim), ds_mul(y, dre)), s);
        dre = nre;
        dim = nim;
    }
    if constexpr (M >= M0) {
        f(M, M, dre, dim);
        if constexpr (M + 1 <= FMM_P) {
            dsf p2re = dre, p2im = dim;
            dsf p1re = ds_mul(z, dre), p1im = ds_mul(z, dim);
            f(M + 1, M, p1re, p1im);
#pragma unroll
            for (int n = M + 2; n <= FMM_P; n++) {
                const dsf az = ds_mul(dsf{(float)(2 * n - 1), 0.f}, z);
                const dsf b = dsc(1.0 / ((n + M) * (n - M)));
                const dsf cre = ds_mul(ds_sub(ds_mul(az, p1re), ds_mul(r2, p2re)), b);
                const dsf cim = ds_mul(ds_sub(ds_mul(az, p1im), ds_mul(r2, p2im)), b);
                f(n, M, cre, cim);
                p2re = p1re; p2im = p1im;
                p1re = cre; p1im = cim;
            }
        }
    }
    if constexpr (M < M1) ups_col_ds<M + 1, M0, M1>(x, y, z, r2, dre, dim, f);
}

template <int NS, int M0, int M1>
__device__ __forceinline__ void p2m_ds_pass(int lane, int s0, int s1, const float4 *__restrict__ shi,
                                            const float4 *__restrict__ slo, size_t base, const P2mSet<double> &a,
                                            const P2mSet<double> &b) {
    constexpr int NPR = lidx(M0, FMM_P, M1, 1) + 1;
    dsf acc0[NPR], acc1[NS == 2 ? NPR : 1];
#pragma unroll
    for (int k = 0; k < NPR; k++) acc0[k] = dsf{0.f, 0.f};
#pragma unroll
    for (int k = 0; k < (NS == 2 ? NPR : 1); k++) acc1[k] = dsf{0.f, 0.f};
    for (int s = s0 + lane; s < s1; s += 32) {
        const float4 h = shi[s], l = slo[s];
        const dsf x = ds_two_sum_f(h.x, l.x), y = ds_two_sum_f(h.y, l.y), z = ds_two_sum_f(h.z, l.z);
        const double qa_d = a.q[s], qb_d = NS == 2 ? b.q[s] : 0.0;
        const dsf qa = dsc(qa_d), qb = dsc(qb_d);
        if constexpr (M0 == 0) {  // the charges for the near field, as k_p2m stores them
            a.qn[(size_t)s * a.qn_stride] = qa_d;
            if (a.qh) {
                a.qh[(size_t)s * a.qd_stride] = qa.h;
                a.ql[(size_t)s * a.qd_stride] = (float)(qa_d - (double)qa.h);
            }
            if constexpr (NS == 2) {
                b.qn[(size_t)s * b.qn_stride] = qb_d;
                if (b.qh) {
                    b.qh[(size_t)s * b.qd_stride] = qb.h;
                    b.ql[(size_t)s * b.qd_stride] = (float)(qb_d - (double)qb.h);
                }
            }
        }
        const dsf r2 = ds_add(ds_add(ds_mul(x, x), ds_mul(y, y)), ds_mul(z, z));
        dsf dre = {1.f, 0.f}, dim = {0.f, 0.f};
        auto f = [&](int n, int m, dsf re, dsf im) {
            const int k = lidx(M0, n, m, 0);
            acc0[k] = ds_add(acc0[k], ds_mul(qa, re));
            if constexpr (NS == 2) acc1[k] = ds_add(acc1[k], ds_mul(qb, re));
            if (m) {
                acc0[k + 1] = ds_sub(acc0[k + 1], ds_mul(qa, im));
                if constexpr (NS == 2) acc1[k + 1] = ds_sub(acc1[k + 1], ds_mul(qb, im));
            }
        };
        ups_col_ds<0, M0, M1>(x, y, z, r2, dre, dim, f);
    }
    auto red = [&](dsf v) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v = ds_add(v, dsf{__shfl_xor_sync(0xffffffffu, v.h, o), __shfl_xor_sync(0xffffffffu, v.l, o)});
        return v;
    };
#pragma unroll
    for (int m = M0; m <= M1; m++)
#pragma unroll
        for (int n = m; n <= FMM_P; n++)
#pragma unroll
            for (int part = 0; part < (m ? 2 : 1); part++) {
                const int k = lidx(M0, n, m, part), g = ridx(n, m, part);
                const dsf v0 = red(acc0[k]);
                dsf v1 = {0.f, 0.f};
                if constexpr (NS == 2) v1 = red(acc1[k]);
                if ((g & 31) == lane) {
                    a.M[base + g] = ds_to(v0);
                    if constexpr (NS == 2) b.M[base + g] = ds_to(v1);
                }
            }
}

// One warp per leaf, the NS charge sets in one pass over the sources (the FP64 tree's
// sources as hi/lo float4 pairs): the harmonics of a source are formed once for both sets,
// in six passes over the harmonic columns (0, 1, 2, 3, 4-5, 6-9: at most 22 reals, 88 floats
// of accumulators for two sets); one set and two run the same code, so a set's expansion
// does not depend on whether the other is evaluated beside it.
template <int NS>
__global__ void __launch_bounds__(128) k_p2m_ds(int nleaf, const int *__restrict__ leaf_src,
                                                const float4 *__restrict__ shi, const float4 *__restrict__ slo,
                                                int leaf0, P2mSet<double> set0, P2mSet<double> set1) {
    const int lane = threadIdx.x & 31;
    const int leaf = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (leaf >= nleaf) return;
    const int s0 = leaf_src[leaf], s1 = leaf_src[leaf + 1];
    const size_t base = (size_t)(leaf0 + leaf) * NR;
    p2m_ds_pass<NS, 0, 0>(lane, s0, s1, shi, slo, base, set0, set1);
    p2m_ds_pass<NS, 1, 1>(lane, s0, s1, shi, slo, base, set0, set1);
    p2m_ds_pass<NS, 2, 2>(lane, s0, s1, shi, slo, base, set0, set1);
    p2m_ds_pass<NS, 3, 3>(lane, s0, s1, shi, slo, base, set0, set1);
    p2m_ds_pass<NS, 4, 5>(lane, s0, s1, shi, slo, base, set0, set1);
    p2m_ds_pass<NS, 6, FMM_P>(lane, s0, s1, shi, slo, base, set0, set1);
}

// Batched translation out[c] (+)= sum_code Op[code] in[tab[c][code]] for TB output cells
// per block. 160 threads: 10 row groups (10 rows each) x 16 column groups (CT cells each).
template <typename T>
__global__ void __launch_bounds__(160) k_translate(int n_out, int out0, int ncode, const int *__restrict__ tab,
                                                   const T *__restrict__ ops, const T *in, T *out,
                                                   int accumulate) {
    // in and out may be the same array (M2M, L2L): the cells read and written are disjoint.
    constexpr int TB = TrShape<T>::TB, CT = TrShape<T>::CT, RT = 10, BLD = TB + 4;
    extern __shared__ unsigned char smem_raw[];
    T *AT = reinterpret_cast<T *>(smem_raw);  // [NR][NR]: AT[k*NR + row] = Op[row][k]
    T *Bs = AT + NR * NR;                      // [NR][BLD]
    __shared__ int srcs[TB];
    const int tid = threadIdx.x, rg = tid / 16, cg = tid % 16;
    const int c_begin = blockIdx.x * TB;
    T acc[RT][CT];
#pragma unroll
    for (int i = 0; i < RT; i++)
#pragma unroll
        for (int j = 0; j < CT; j++) acc[i][j] = 0;
    for (int code = 0; code < ncode; code++) {
        int s = -1;
        if (tid < TB && c_begin + tid < n_out) s = tab[(size_t)(out0 + c_begin + tid) * ncode + code];
        if (tid < TB) srcs[tid] = s;
        if (!__syncthreads_or(s >= 0)) continue;
        for (int e = tid; e < NR * NR; e += blockDim.x) {
            const int row = e / NR, k = e % NR;
            AT[k * NR + row] = ops[(size_t)code * NR * NR + e];
        }
        for (int e = tid; e < NR * TB; e += blockDim.x) {
            const int col = e / NR, k = e % NR;
            const int sc = srcs[col];
            Bs[k * BLD + col] = sc >= 0 ? in[(size_t)sc * NR + k] : T(0);
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < NR; k++) {
            T a[RT], b[CT];
#pragma unroll
            for (int i = 0; i < RT; i++) a[i] = AT[k * NR + rg * RT + i];
#pragma unroll
            for (int j = 0; j < CT; j++) b[j] = Bs[k * BLD + cg * CT + j];
#pragma unroll
            for (int i = 0; i < RT; i++)
#pragma unroll
                for (int j = 0; j < CT; j++) acc[i][j] += a[i] * b[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < CT; j++) {
        const int c = c_begin + cg * CT + j;
        if (c >= n_out) continue;
        T *o = out + (size_t)(out0 + c) * NR + rg * RT;
#pragma unroll
        for (int i = 0; i < RT; i++) o[i] = accumulate ? o[i] + acc[i][j] : acc[i][j];
    }
}

// FP64-path translations in double-single arithmetic on the FP32 pipes (GB300's FP64 pipe
// does 2 DFMA per clock and SM, 1/64 of its FP32 rate): the same batched GEMM as
// k_translate, both charge sets of a block of DS_TB output cells as its 2 DS_TB columns, the
// operator and the inputs split into FP32 pairs hi + lo on their way into shared memory,
// every product exact through fma (Dekker's TwoProduct) and summed with Knuth's two-sum,
// the running sum renormalised once per code (about 44 significant bits), the result
// rounded to FP64 once.
constexpr int DS_TB = 16, DS_COLS = 2 * DS_TB, DS_CT = 2, DS_BLD = DS_COLS + 1;
constexpr int tr_ds_smem() { return (NR * NR + NR * DS_BLD) * (int)sizeof(float2); }

__device__ __forceinline__ float2 ds_split(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

__global__ void __launch_bounds__(160, 2) k_translate_ds(int n_out, int out0, int ncode, const int *__restrict__ tab,
                                                         const double *__restrict__ ops, const double *in,
                                                         double *out, int accumulate, int nset, size_t set_stride) {
    // in and out may be the same array (M2M, L2L): the cells read and written are disjoint.
    constexpr int RT = 10;
    extern __shared__ unsigned char smem_raw[];
    float2 *AT = reinterpret_cast<float2 *>(smem_raw);  // AT[k * NR + row] = Op[row][k]
    float2 *Bs = AT + NR * NR;                           // [NR][DS_BLD]: column set * DS_TB + cell
    __shared__ int srcs[DS_TB];
    const int tid = threadIdx.x, rg = tid / 16, cg = tid % 16;
    const int c_begin = blockIdx.x * DS_TB;
    float ah[RT][DS_CT], al[RT][DS_CT];
#pragma unroll
    for (int i = 0; i < RT; i++)
#pragma unroll
        for (int j = 0; j < DS_CT; j++) ah[i][j] = al[i][j] = 0.f;
    for (int code = 0; code < ncode; code++) {
        int sc = -1;
        if (tid < DS_TB && c_begin + tid < n_out) sc = tab[(size_t)(out0 + c_begin + tid) * ncode + code];
        if (tid < DS_TB) srcs[tid] = sc;
        if (!__syncthreads_or(sc >= 0)) continue;
        for (int e = tid; e < NR * NR; e += blockDim.x) {
            const int row = e / NR, k = e % NR;
            AT[k * NR + row] = ds_split(ops[(size_t)code * NR * NR + e]);
        }
        for (int e = tid; e < NR * DS_COLS; e += blockDim.x) {
            const int col = e / NR, k = e % NR, cell = col % DS_TB, set = col / DS_TB;
            const int src = srcs[cell];
            Bs[k * DS_BLD + col] = (src >= 0 && set < nset) ? ds_split(in[set * set_stride + (size_t)src * NR + k])
                                                              : make_float2(0.f, 0.f);
        }
        __syncthreads();
#pragma unroll 2
        for (int k = 0; k < NR; k++) {
            float2 a[RT], b[DS_CT];
#pragma unroll
            for (int i = 0; i < RT; i++) a[i] = AT[k * NR + rg * RT + i];
#pragma unroll
            for (int j = 0; j < DS_CT; j++) b[j] = Bs[k * DS_BLD + cg * DS_CT + j];
#pragma unroll
            for (int i = 0; i < RT; i++)
#pragma unroll
                for (int j = 0; j < DS_CT; j++) {
                    // (ah, al) += a b: exact leading product and cross terms, two-sum into hi
                    const float p = a[i].x * b[j].x;
                    float e = fmaf(a[i].x, b[j].x, -p);
                    e = fmaf(a[i].x, b[j].y, e);
                    e = fmaf(a[i].y, b[j].x, e);
                    const float s = ah[i][j] + p;
                    const float bb = s - ah[i][j];
                    const float err = (ah[i][j] - (s - bb)) + (p - bb);
                    ah[i][j] = s;
                    al[i][j] += e + err;
                }
        }
#pragma unroll
        for (int i = 0; i < RT; i++)
#pragma unroll
            for (int j = 0; j < DS_CT; j++) {  // renormalise: |lo| back to half an ulp of hi
                const float s = ah[i][j] + al[i][j];
                al[i][j] = al[i][j] - (s - ah[i][j]);
                ah[i][j] = s;
            }
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < DS_CT; j++) {
        const int col = cg * DS_CT + j, cell = col % DS_TB, set = col / DS_TB;
        const int c = c_begin + cell;
        if (c >= n_out || set >= nset) continue;
        double *o = out + set * set_stride + (size_t)(out0 + c) * NR + rg * RT;
#pragma unroll
        for (int i = 0; i < RT; i++) {
            const double v = (double)ah[i][j] + (double)al[i][j];
            o[i] = accumulate ? o[i] + v : v;
        }
    }
}

// 1/sqrt in the precision of the path.
template <typename T> __device__ __forceinline__ T rsqrt_p(T x);
template <> __device__ __forceinline__ float rsqrt_p<float>(float x) {
    float r;  // the SFU reciprocal square root (relative error below 2^-22), denormals flushed
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// FP64: CUDA's rsqrt (a single-precision-seeded Newton step written out here measured
// slower: the FP64 <-> FP32 conversions cost more than they save).
template <> __device__ __forceinline__ double rsqrt_p<double>(double x) { return rsqrt(x); }

template <typename T> struct Vec4;
template <> struct Vec4<float> { using type = float4; };
template <> struct Vec4<double> { using type = double4; };

// Charge sets of one near-field launch: the first set's charge rides in the w of the source
// coordinates, the second (demag of v beside that of m) in its own array; the local
// expansions and potentials of each set.
template <typename T>
struct NearSets {
    const T *q2;            // second set's charges (NQ = 2)
    const T *F[2];          // local expansions per set
    double *pot[2];         // potentials per set
    int near_only;          // 1: write the near-field sums only (k_l2p adds the far field later)
};

// One pass of the near field and L2P over up to NT targets tb.. of a leaf (nt of them real,
// the rest padding), for NQ charge sets at once (the pair geometry and the reciprocal
// distance are shared; each set keeps its own sums in the same order as alone): one warp;
// sources of the adjacent leaves spread over the lanes (x, y, z, q in one vector load; each
// lane takes two sources per step and already loads the next two); targets in registers;
// coordinates leaf-local (leaf units), so FP32 keeps the relative precision of close
// pairs. The per-lane sums are reduced over the warp in a fixed order, lane j then
// evaluates the local expansion(s) at target j.
template <typename T, int NT, int NQ>
__device__ __forceinline__ void l2p_p2p_pass(int leaf, int tb, int nt, int lane, int li, int lj, int lk,
                                             const int *__restrict__ leaf_src, const int *__restrict__ tgt_node,
                                             const T *__restrict__ tloc, const T *__restrict__ sloc,
                                             const int *__restrict__ leaf_ijk, const double *__restrict__ leaf_scale,
                                             const int *__restrict__ near_ptr, const int *__restrict__ near_leaf,
                                             size_t fbase, const NearSets<T> &sets) {
    using V4 = typename Vec4<T>::type;
    const V4 *__restrict__ src4 = reinterpret_cast<const V4 *>(sloc);
    const T *__restrict__ q2 = sets.q2;
    T tx[NT], ty[NT], tz[NT], ns[NQ][NT];
#pragma unroll
    for (int j = 0; j < NT; j++) {
        const int ti = tb + (j < nt ? j : 0);
        tx[j] = tloc[4 * (size_t)ti];
        ty[j] = tloc[4 * (size_t)ti + 1];
        tz[j] = tloc[4 * (size_t)ti + 2];
#pragma unroll
        for (int k = 0; k < NQ; k++) ns[k][j] = 0;
    }
    for (int e = near_ptr[leaf]; e < near_ptr[leaf + 1]; e++) {
        const int nl = near_leaf[e];
        // source coordinates relative to this leaf: own leaf-local + integer leaf offset
        const T ox = T(leaf_ijk[3 * nl] - li), oy = T(leaf_ijk[3 * nl + 1] - lj), oz = T(leaf_ijk[3 * nl + 2] - lk);
        const int s0 = leaf_src[nl], s1 = leaf_src[nl + 1];
        T acc[NQ][NT];
#pragma unroll
        for (int j = 0; j < NT; j++)
#pragma unroll
            for (int k = 0; k < NQ; k++) acc[k][j] = 0;
        // a missing source is a zero charge far away
        V4 far;
        far.x = far.y = far.z = T(1e4);
        far.w = T(0);
        int s = s0 + lane;
        V4 na = s < s1 ? src4[s] : far, nb = s + 32 < s1 ? src4[s + 32] : far;
        T na2 = 0, nb2 = 0;
        if constexpr (NQ == 2) {
            na2 = s < s1 ? q2[s] : T(0);
            nb2 = s + 32 < s1 ? q2[s + 32] : T(0);
        }
        for (; s < s1; s += 64) {
            const V4 sa = na, sb = nb;
            const T aq2 = na2, bq2 = nb2;
            na = s + 64 < s1 ? src4[s + 64] : far;
            nb = s + 96 < s1 ? src4[s + 96] : far;
            if constexpr (NQ == 2) {
                na2 = s + 64 < s1 ? q2[s + 64] : T(0);
                nb2 = s + 96 < s1 ? q2[s + 96] : T(0);
            }
            const T ax = sa.x + ox, ay = sa.y + oy, az = sa.z + oz, aq = sa.w;
            const T bx = sb.x + ox, by = sb.y + oy, bz = sb.z + oz, bq = sb.w;
#pragma unroll
            for (int j = 0; j < NT; j++) {
                const T dx = tx[j] - ax, dy = ty[j] - ay, dz = tz[j] - az;
                const T ex = tx[j] - bx, ey = ty[j] - by, ez = tz[j] - bz;
                const T ra = rsqrt_p<T>(dx * dx + dy * dy + dz * dz);
                const T rb = rsqrt_p<T>(ex * ex + ey * ey + ez * ez);
                acc[0][j] += aq * ra;
                acc[0][j] += bq * rb;
                if constexpr (NQ == 2) {
                    acc[1][j] += aq2 * ra;
                    acc[1][j] += bq2 * rb;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < NT; j++)
#pragma unroll
            for (int k = 0; k < NQ; k++) ns[k][j] += acc[k][j];
    }
    // warp sums in the path's precision (fixed butterfly order), then FP64
    double near[NQ][NT];
#pragma unroll
    for (int k = 0; k < NQ; k++)
#pragma unroll
        for (int j = 0; j < NT; j++) {
            T v = ns[k][j];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            near[k][j] = double(v);
        }
    if (lane < nt) {
        T x = 0, y = 0, z = 0;
        double nr[NQ];
#pragma unroll
        for (int k = 0; k < NQ; k++) nr[k] = 0;
#pragma unroll
        for (int j = 0; j < NT; j++)
            if (j == lane) {
                x = tx[j]; y = ty[j]; z = tz[j];
#pragma unroll
                for (int k = 0; k < NQ; k++) nr[k] = near[k][j];
            }
        if (sets.near_only) {
            const int node = tgt_node[tb + lane];
#pragma unroll
            for (int k = 0; k < NQ; k++) sets.pot[k][node] = nr[k];
            return;
        }
        const T *__restrict__ Fa = sets.F[0] + fbase;
        const T *__restrict__ Fb = sets.F[NQ - 1] + fbase;
        T fa = 0, fb = 0;
        ups_cols<T>(x, y, z, [&](int n, int m, T re, T im) {
            if (m == 0) {
                fa += Fa[ridx(n, 0, 0)] * re;
                if constexpr (NQ == 2) fb += Fb[ridx(n, 0, 0)] * re;
            } else {
                fa += T(2) * (Fa[ridx(n, m, 0)] * re + Fa[ridx(n, m, 1)] * im);
                if constexpr (NQ == 2) fb += T(2) * (Fb[ridx(n, m, 0)] * re + Fb[ridx(n, m, 1)] * im);
            }
        });
        const double sc = leaf_scale[leaf];
        const int node = tgt_node[tb + lane];
        sets.pot[0][node] = (double(fa) + nr[0]) * sc;
        if constexpr (NQ == 2) sets.pot[1][node] = (double(fb) + nr[NQ - 1]) * sc;
    }
}

// The FP32 pass of l2p_p2p_pass with the pair arithmetic on packed target pairs: per two
// pairs 3 subtractions, 3 for r^2 (d_x^2, then + d_y^2, + d_z^2 as fused multiply-adds),
// two SFU reciprocal square roots and one fused multiply-add per charge set, the pair
// arithmetic of the scalar pass. The terms go straight into the pass sums (no per-leaf
// partial sums as in the scalar pass): 128 registers, so four blocks fit on an SM, or one
// beside a tensor-core translation CTA (1.61 -> 1.49 ms on the film; the FP32 FMM's error
// against the FP64 FMM stays 4.7e-7 for the potential of m, 1.1e-6 instead of 7e-7 for the
// potential of v).
template <int NT, int NQ>
__device__ __forceinline__ void l2p_p2p_pass_x2(int leaf, int tb, int nt, int lane, int li, int lj, int lk,
                                                const int *__restrict__ leaf_src, const int *__restrict__ tgt_node,
                                                const float *__restrict__ tloc, const float *__restrict__ sloc,
                                                const int *__restrict__ leaf_ijk,
                                                const double *__restrict__ leaf_scale,
                                                const int *__restrict__ near_ptr, const int *__restrict__ near_leaf,
                                                size_t fbase, const NearSets<float> &sets) {
    static_assert(NT % 2 == 0, "targets come in pairs");
    constexpr int NP = NT / 2;
    const float4 *__restrict__ src4 = reinterpret_cast<const float4 *>(sloc);
    const float *__restrict__ q2 = sets.q2;
    u64 TX[NP], TY[NP], TZ[NP], NS[NQ][NP];
#pragma unroll
    for (int p = 0; p < NP; p++) {
        const int t0 = tb + (2 * p < nt ? 2 * p : 0), t1 = tb + (2 * p + 1 < nt ? 2 * p + 1 : 0);
        TX[p] = pk2(tloc[4 * (size_t)t0], tloc[4 * (size_t)t1]);
        TY[p] = pk2(tloc[4 * (size_t)t0 + 1], tloc[4 * (size_t)t1 + 1]);
        TZ[p] = pk2(tloc[4 * (size_t)t0 + 2], tloc[4 * (size_t)t1 + 2]);
#pragma unroll
        for (int k = 0; k < NQ; k++) NS[k][p] = 0ull;
    }
    for (int e = near_ptr[leaf]; e < near_ptr[leaf + 1]; e++) {
        const int nl = near_leaf[e];
        const float ox = float(leaf_ijk[3 * nl] - li), oy = float(leaf_ijk[3 * nl + 1] - lj),
                    oz = float(leaf_ijk[3 * nl + 2] - lk);
        const int s0 = leaf_src[nl], s1 = leaf_src[nl + 1];
        const float4 far = make_float4(1e4f, 1e4f, 1e4f, 0.f);  // a missing source: zero charge far away
        int s = s0 + lane;
        float4 na = s < s1 ? src4[s] : far, nb = s + 32 < s1 ? src4[s + 32] : far;
        float na2 = 0.f, nb2 = 0.f;
        if constexpr (NQ == 2) {
            na2 = s < s1 ? q2[s] : 0.f;
            nb2 = s + 32 < s1 ? q2[s + 32] : 0.f;
        }
        for (; s < s1; s += 64) {
            const float4 sa = na, sb = nb;
            const float aq2 = na2, bq2 = nb2;
            na = s + 64 < s1 ? src4[s + 64] : far;
            nb = s + 96 < s1 ? src4[s + 96] : far;
            if constexpr (NQ == 2) {
                na2 = s + 64 < s1 ? q2[s + 64] : 0.f;
                nb2 = s + 96 < s1 ? q2[s + 96] : 0.f;
            }
            const float ax = sa.x + ox, ay = sa.y + oy, az = sa.z + oz;
            const float bx = sb.x + ox, by = sb.y + oy, bz = sb.z + oz;
            const u64 AX = pk2(ax, ax), AY = pk2(ay, ay), AZ = pk2(az, az), AQ = pk2(sa.w, sa.w);
            const u64 BX = pk2(bx, bx), BY = pk2(by, by), BZ = pk2(bz, bz), BQ = pk2(sb.w, sb.w);
            const u64 AQ2 = pk2(aq2, aq2), BQ2 = pk2(bq2, bq2);
#pragma unroll
            for (int p = 0; p < NP; p++) {
                const u64 dx = sub2(TX[p], AX), dy = sub2(TY[p], AY), dz = sub2(TZ[p], AZ);
                const u64 ex = sub2(TX[p], BX), ey = sub2(TY[p], BY), ez = sub2(TZ[p], BZ);
                const u64 da = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
                const u64 db = fma2(ez, ez, fma2(ey, ey, mul2(ex, ex)));
                float a0, a1, b0, b1;
                upk2(da, a0, a1);
                upk2(db, b0, b1);
                const u64 RA = pk2(rsqrt_p<float>(a0), rsqrt_p<float>(a1));
                const u64 RB = pk2(rsqrt_p<float>(b0), rsqrt_p<float>(b1));
                NS[0][p] = fma2(AQ, RA, NS[0][p]);
                NS[0][p] = fma2(BQ, RB, NS[0][p]);
                if constexpr (NQ == 2) {
                    NS[1][p] = fma2(AQ2, RA, NS[1][p]);
                    NS[1][p] = fma2(BQ2, RB, NS[1][p]);
                }
            }
        }
    }
    // warp sums (fixed butterfly order), then FP64
    double near[NQ][NT];
#pragma unroll
    for (int k = 0; k < NQ; k++)
#pragma unroll
        for (int p = 0; p < NP; p++) {
            float v0, v1;
            upk2(NS[k][p], v0, v1);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                v0 += __shfl_xor_sync(0xffffffffu, v0, o);
                v1 += __shfl_xor_sync(0xffffffffu, v1, o);
            }
            near[k][2 * p] = double(v0);
            near[k][2 * p + 1] = double(v1);
        }
    if (lane < nt) {
        float x = 0, y = 0, z = 0;
        double nr[NQ];
#pragma unroll
        for (int k = 0; k < NQ; k++) nr[k] = 0;
#pragma unroll
        for (int p = 0; p < NP; p++) {
            float x0, x1, y0, y1, z0, z1;
            upk2(TX[p], x0, x1);
            upk2(TY[p], y0, y1);
            upk2(TZ[p], z0, z1);
            if (2 * p == lane) {
                x = x0; y = y0; z = z0;
#pragma unroll
                for (int k = 0; k < NQ; k++) nr[k] = near[k][2 * p];
            }
            if (2 * p + 1 == lane) {
                x = x1; y = y1; z = z1;
#pragma unroll
                for (int k = 0; k < NQ; k++) nr[k] = near[k][2 * p + 1];
            }
        }
        if (sets.near_only) {
            const int node = tgt_node[tb + lane];
#pragma unroll
            for (int k = 0; k < NQ; k++) sets.pot[k][node] = nr[k];
            return;
        }
        const float *__restrict__ Fa = sets.F[0] + fbase;
        const float *__restrict__ Fb = sets.F[NQ - 1] + fbase;
        float fa = 0, fb = 0;
        ups_cols<float>(x, y, z, [&](int n, int m, float re, float im) {
            if (m == 0) {
                fa += Fa[ridx(n, 0, 0)] * re;
                if constexpr (NQ == 2) fb += Fb[ridx(n, 0, 0)] * re;
            } else {
                fa += 2.f * (Fa[ridx(n, m, 0)] * re + Fa[ridx(n, m, 1)] * im);
                if constexpr (NQ == 2) fb += 2.f * (Fb[ridx(n, m, 0)] * re + Fb[ridx(n, m, 1)] * im);
            }
        });
        const double sc = leaf_scale[leaf];
        const int node = tgt_node[tb + lane];
        sets.pot[0][node] = (double(fa) + nr[0]) * sc;
        if constexpr (NQ == 2) sets.pot[1][node] = (double(fb) + nr[NQ - 1]) * sc;
    }
}

// L2P + P2P: one warp per target leaf, its targets in passes of 16 and a tail pass of 8
// or 4 (a leaf of the film holds 18 to 64 nodes: fixed passes of 16 would spend about a
// fifth of the pair work on padding).
template <typename T, int NQ>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 4 : 2)  // FP32: 128 registers, 4 blocks per SM
    k_l2p_p2p(int nleaf, const int *__restrict__ leaf_src, const int *__restrict__ leaf_tgt,
              const int *__restrict__ tgt_node, const T *__restrict__ tloc, const T *__restrict__ sloc,
              const int *__restrict__ leaf_ijk, int leaf0, const double *__restrict__ leaf_scale,
              const int *__restrict__ near_ptr, const int *__restrict__ near_leaf, NearSets<T> sets) {
    const int lane = threadIdx.x & 31;
    const int leaf = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (leaf >= nleaf) return;
    const int t0 = leaf_tgt[leaf], t1 = leaf_tgt[leaf + 1];
    if (t0 == t1) return;
    const int li = leaf_ijk[3 * leaf], lj = leaf_ijk[3 * leaf + 1], lk = leaf_ijk[3 * leaf + 2];
    const size_t fbase = (size_t)(leaf0 + leaf) * NR;
    for (int tb = t0; tb < t1;) {
        const int r = t1 - tb;
        const int nt = r > 8 ? 16 : r > 4 ? 8 : 4;
        if constexpr (sizeof(T) == 4) {
            if (nt == 16)
                l2p_p2p_pass_x2<16, NQ>(leaf, tb, min(16, r), lane, li, lj, lk, leaf_src, tgt_node, tloc, sloc,
                                        leaf_ijk, leaf_scale, near_ptr, near_leaf, fbase, sets);
            else if (nt == 8)
                l2p_p2p_pass_x2<8, NQ>(leaf, tb, r, lane, li, lj, lk, leaf_src, tgt_node, tloc, sloc, leaf_ijk,
                                       leaf_scale, near_ptr, near_leaf, fbase, sets);
            else
                l2p_p2p_pass_x2<4, NQ>(leaf, tb, r, lane, li, lj, lk, leaf_src, tgt_node, tloc, sloc, leaf_ijk,
                                       leaf_scale, near_ptr, near_leaf, fbase, sets);
        } else {
            if (nt == 16)
                l2p_p2p_pass<T, 16, NQ>(leaf, tb, min(16, r), lane, li, lj, lk, leaf_src, tgt_node, tloc, sloc,
                                        leaf_ijk, leaf_scale, near_ptr, near_leaf, fbase, sets);
            else if (nt == 8)
                l2p_p2p_pass<T, 8, NQ>(leaf, tb, r, lane, li, lj, lk, leaf_src, tgt_node, tloc, sloc, leaf_ijk,
                                       leaf_scale, near_ptr, near_leaf, fbase, sets);
            else
                l2p_p2p_pass<T, 4, NQ>(leaf, tb, r, lane, li, lj, lk, leaf_src, tgt_node, tloc, sloc, leaf_ijk,
                                       leaf_scale, near_ptr, near_leaf, fbase, sets);
        }
        tb += nt;
    }
}

// Double-single arithmetic on the FP32 pipes: an FP64-accurate near field for the FP64
// path, whose FP64 pipe (2 DFMA per clock and SM on this GPU) would otherwise bound it.
// A value is hi + lo with |lo| <= ulp(hi)/2 (Dekker, "A floating-point technique for
// extending the available precision", 1971; Knuth's two-sum).
__device__ __forceinline__ void ds_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// L2P + P2P of the FP64 path in double-single arithmetic. Coordinates are leaf-local with
// hi parts on a 2^-20 grid (|x| < 4, so hi - hi' is exact in FP32) and lo = x - hi
// (|lo| <= 2^-21, held to 2^-45); per pair: dx = (hi - hi') + (lo - lo'), r^2 as a
// double-single sum of the squares (the leading products exact through fma), 1/r from the
// SFU estimate and one Newton step evaluated in double-single (error ~1e-13), q/r as a
// double-single product, summed with two-sum. One warp per target leaf, 8 targets per
// lane pass, sources spread over the lanes; per-lane sums reduced over the warp in FP64.
// NQ charge sets share the pair geometry and 1/r (the second set's charge hi/lo in q2h/q2l).
template <int NQ>
__global__ void __launch_bounds__(128) k_l2p_p2p_ds(int nleaf, const int *__restrict__ leaf_src,
                                                    const int *__restrict__ leaf_tgt,
                                                    const int *__restrict__ tgt_node,
                                                    const double *__restrict__ tloc,
                                                    const float4 *__restrict__ th4, const float4 *__restrict__ tl4,
                                                    const float4 *__restrict__ sh4, const float4 *__restrict__ sl4,
                                                    const float *__restrict__ q2h, const float *__restrict__ q2l,
                                                    const int *__restrict__ leaf_ijk, int leaf0,
                                                    const double *__restrict__ leaf_scale,
                                                    const int *__restrict__ near_ptr,
                                                    const int *__restrict__ near_leaf, NearSets<double> sets) {
    constexpr int NT = 8;
    const int lane = threadIdx.x & 31;
    const int leaf = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (leaf >= nleaf) return;
    const int t0 = leaf_tgt[leaf], t1 = leaf_tgt[leaf + 1];
    if (t0 == t1) return;
    const int li = leaf_ijk[3 * leaf], lj = leaf_ijk[3 * leaf + 1], lk = leaf_ijk[3 * leaf + 2];
    const size_t fbase = (size_t)(leaf0 + leaf) * NR;
    for (int tb = t0; tb < t1; tb += NT) {
        const int nt = min(NT, t1 - tb);
        float thx[NT], thy[NT], thz[NT], tlx[NT], tly[NT], tlz[NT], ah[NQ][NT], al[NQ][NT];
#pragma unroll
        for (int j = 0; j < NT; j++) {
            const int ti = tb + (j < nt ? j : 0);
            const float4 h = th4[ti], l = tl4[ti];
            thx[j] = h.x; thy[j] = h.y; thz[j] = h.z;
            tlx[j] = l.x; tly[j] = l.y; tlz[j] = l.z;
#pragma unroll
            for (int k = 0; k < NQ; k++) ah[k][j] = al[k][j] = 0.f;
        }
        for (int e = near_ptr[leaf]; e < near_ptr[leaf + 1]; e++) {
            const int nl = near_leaf[e];
            // integer offset of the adjacent leaf, added exactly to the hi parts
            const float ox = float(leaf_ijk[3 * nl] - li), oy = float(leaf_ijk[3 * nl + 1] - lj),
                        oz = float(leaf_ijk[3 * nl + 2] - lk);
            const int s0 = leaf_src[nl], s1 = leaf_src[nl + 1];
            for (int s = s0 + lane; s < s1; s += 32) {
                const float4 h = sh4[s], l = sl4[s];
                const float sx = h.x + ox, sy = h.y + oy, sz = h.z + oz;
                float qh[NQ], ql[NQ];
                qh[0] = h.w;
                ql[0] = l.w;
                if constexpr (NQ == 2) {
                    qh[1] = q2h[s];
                    ql[1] = q2l[s];
                }
#pragma unroll
                for (int j = 0; j < NT; j++) {
                    const float d1x = thx[j] - sx, d1y = thy[j] - sy, d1z = thz[j] - sz;  // exact
                    const float d2x = tlx[j] - l.x, d2y = tly[j] - l.y, d2z = tlz[j] - l.z;
                    // squares: d^2 = d1^2 + d2 (2 d1 + d2), leading products exact
                    const float px = d1x * d1x, py = d1y * d1y, pz = d1z * d1z;
                    float ex = fmaf(d1x, d1x, -px), ey = fmaf(d1y, d1y, -py), ez = fmaf(d1z, d1z, -pz);
                    ex = fmaf(d2x, 2.f * d1x + d2x, ex);
                    ey = fmaf(d2y, 2.f * d1y + d2y, ey);
                    ez = fmaf(d2z, 2.f * d1z + d2z, ez);
                    float s1_, e1, s2_, e2;
                    ds_two_sum(px, py, s1_, e1);
                    ds_two_sum(s1_, pz, s2_, e2);
                    const float el = (e1 + e2) + (ex + ey + ez);
                    const float Sh = s2_ + el, Sl = el - (Sh - s2_);
                    // 1/sqrt(S): SFU estimate y, then y (1 + (1 - S y^2) / 2) with S y^2 in
                    // double-single (1 - S y^2 is small and exact to ~2^-46)
                    float y;
                    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(Sh));
                    const float t1_ = y * y, t2_ = fmaf(y, y, -t1_);
                    const float u1 = Sh * t1_;
                    const float u2 = fmaf(Sh, t1_, -u1) + fmaf(Sh, t2_, Sl * t1_);
                    const float delta = (1.f - u1) - u2;
                    const float yl = 0.5f * y * delta;
                    // q / r = (qh + ql)(y + yl), accumulated with two-sum
#pragma unroll
                    for (int k = 0; k < NQ; k++) {
                        const float c1 = qh[k] * y;
                        const float c2 = fmaf(qh[k], y, -c1) + fmaf(qh[k], yl, ql[k] * y);
                        float sn, en;
                        ds_two_sum(ah[k][j], c1, sn, en);
                        ah[k][j] = sn;
                        al[k][j] += en + c2;
                    }
                }
            }
        }
        double near[NQ][NT];
#pragma unroll
        for (int k = 0; k < NQ; k++)
#pragma unroll
            for (int j = 0; j < NT; j++) {
                near[k][j] = double(ah[k][j]) + double(al[k][j]);
                for (int o = 16; o > 0; o >>= 1) near[k][j] += __shfl_xor_sync(0xffffffffu, near[k][j], o);
            }
        // L2P in FP64: lane j evaluates target j
        if (lane < nt) {
            double nr[NQ];
#pragma unroll
            for (int k = 0; k < NQ; k++) nr[k] = 0;
#pragma unroll
            for (int j = 0; j < NT; j++)
                if (j == lane)
#pragma unroll
                    for (int k = 0; k < NQ; k++) nr[k] = near[k][j];
            const int ti = tb + lane;
            if (sets.near_only) {
#pragma unroll
                for (int k = 0; k < NQ; k++) sets.pot[k][tgt_node[ti]] = nr[k];
                continue;
            }
            const double x = tloc[4 * (size_t)ti], y = tloc[4 * (size_t)ti + 1], z = tloc[4 * (size_t)ti + 2];
            const double *__restrict__ Fa = sets.F[0] + fbase;
            const double *__restrict__ Fb = sets.F[NQ - 1] + fbase;
            double fa = 0, fb = 0;
            ups_cols<double>(x, y, z, [&](int n, int m, double re, double im) {
                if (m == 0) {
                    fa += Fa[ridx(n, 0, 0)] * re;
                    if constexpr (NQ == 2) fb += Fb[ridx(n, 0, 0)] * re;
                } else {
                    fa += 2.0 * (Fa[ridx(n, m, 0)] * re + Fa[ridx(n, m, 1)] * im);
                    if constexpr (NQ == 2) fb += 2.0 * (Fb[ridx(n, m, 0)] * re + Fb[ridx(n, m, 1)] * im);
                }
            });
            const double sc = leaf_scale[leaf];
            sets.pot[0][tgt_node[ti]] = (fa + nr[0]) * sc;
            if constexpr (NQ == 2) sets.pot[1][tgt_node[ti]] = (fb + nr[NQ - 1]) * sc;
        }
    }
}

// L2P after a near-field-only pass: one warp per target leaf, lane j of a pass evaluates
// the local expansion(s) at target j and forms the potential from the stored near sum with
// the same operations as the fused pass, pot = (far + near) * scale.
template <typename T, int NQ>
__global__ void __launch_bounds__(128) k_l2p(int nleaf, const int *__restrict__ leaf_tgt,
                                             const int *__restrict__ tgt_node, const T *__restrict__ tloc,
                                             int leaf0, const double *__restrict__ leaf_scale, NearSets<T> sets) {
    const int lane = threadIdx.x & 31;
    const int leaf = blockIdx.x * 4 + (threadIdx.x >> 5);
    if (leaf >= nleaf) return;
    const int t0 = leaf_tgt[leaf], t1 = leaf_tgt[leaf + 1];
    const size_t fbase = (size_t)(leaf0 + leaf) * NR;
    const double sc = leaf_scale[leaf];
    const T *__restrict__ Fa = sets.F[0] + fbase;
    const T *__restrict__ Fb = sets.F[NQ - 1] + fbase;
    for (int ti = t0 + lane; ti < t1; ti += 32) {
        const T x = tloc[4 * (size_t)ti], y = tloc[4 * (size_t)ti + 1], z = tloc[4 * (size_t)ti + 2];
        T fa = 0, fb = 0;
        ups_cols<T>(x, y, z, [&](int n, int m, T re, T im) {
            if (m == 0) {
                fa += Fa[ridx(n, 0, 0)] * re;
                if constexpr (NQ == 2) fb += Fb[ridx(n, 0, 0)] * re;
            } else {
                fa += T(2) * (Fa[ridx(n, m, 0)] * re + Fa[ridx(n, m, 1)] * im);
                if constexpr (NQ == 2) fb += T(2) * (Fb[ridx(n, m, 0)] * re + Fb[ridx(n, m, 1)] * im);
            }
        });
        const int node = tgt_node[ti];
        sets.pot[0][node] = (double(fa) + sets.pot[0][node]) * sc;
        if constexpr (NQ == 2) sets.pot[1][node] = (double(fb) + sets.pot[1][node]) * sc;
    }
}

// ---------------------------------------------------------------------------------
// host: tree construction

static inline uint64_t spread3(uint64_t v) {
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffull;
    v = (v | v << 16) & 0x1f0000ff0000ffull;
    v = (v | v << 8) & 0x100f00f00f00f00full;
    v = (v | v << 4) & 0x10c30c30c30c30c3ull;
    v = (v | v << 2) & 0x1249249249249249ull;
    return v;
}
static inline uint64_t morton(int x, int y, int z) { return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2); }
static void decode(uint64_t k, int *ijk) {
    ijk[0] = ijk[1] = ijk[2] = 0;
    for (int b = 0; b < 21; b++) {
        ijk[0] |= (int)((k >> (3 * b)) & 1) << b;
        ijk[1] |= (int)((k >> (3 * b + 1)) & 1) << b;
        ijk[2] |= (int)((k >> (3 * b + 2)) & 1) << b;
    }
}

template <typename T>
static cudaError_t up(T **p, const std::vector<T> &h) {
    cudaError_t e = cudaMalloc((void **)p, std::max<size_t>(1, h.size()) * sizeof(T));
    if (e != cudaSuccess) return e;
    if (!h.empty()) e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}
template <typename T>
static cudaError_t up_as(void **p, const std::vector<double> &h, bool fp32) {
    if (fp32) {
        std::vector<float> f(h.begin(), h.end());
        return up((float **)p, f);
    }
    return up((double **)p, h);
}

#define FCK(call)                                                                   \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess) {                                                    \
            c.err = std::string("fmm: ") + #call + ": " + cudaGetErrorString(e_);   \
            return FG_ECUDA;                                                        \
        }                                                                           \
    } while (0)

// Operator matrices (level independent), [code][out][in], in the real layout.
struct FmmOps {
    std::vector<double> m2l, m2m, l2l;
};
static const FmmOps &fmm_ops() {
    static FmmOps ops;
    if (!ops.m2l.empty()) return ops;
    const int P = FMM_P;
    ops.m2l.assign((size_t)NCODE_M2L * NR * NR, 0.0);
    ops.m2m.assign((size_t)8 * NR * NR, 0.0);
    ops.l2l.assign((size_t)8 * NR * NR, 0.0);
    std::vector<cd> T, U, in, out;
    std::vector<double> e(NR), r(NR);
    for (int dx = -3; dx <= 3; dx++)
        for (int dy = -3; dy <= 3; dy++)
            for (int dz = -3; dz <= 3; dz++) {
                if (std::abs(dx) <= 1 && std::abs(dy) <= 1 && std::abs(dz) <= 1) continue;
                const int code = (dx + 3) * 49 + (dy + 3) * 7 + (dz + 3);
                the_host(dx, dy, dz, 2 * P, T);
                for (int j = 0; j < NR; j++) {
                    std::fill(e.begin(), e.end(), 0.0);
                    e[j] = 1.0;
                    to_complex(e.data(), P, in);
                    m2l_c(in, T, P, out);
                    to_real(out, P, r.data());
                    for (int i = 0; i < NR; i++) ops.m2l[(size_t)code * NR * NR + (size_t)i * NR + j] = r[i];
                }
            }
    for (int oc = 0; oc < 8; oc++) {
        ups_host((oc & 1) ? 0.25 : -0.25, (oc & 2) ? 0.25 : -0.25, (oc & 4) ? 0.25 : -0.25, P, U);
        for (int j = 0; j < NR; j++) {
            std::fill(e.begin(), e.end(), 0.0);
            e[j] = 1.0;
            to_complex(e.data(), P, in);
            m2m_c(in, U, P, out);
            to_real(out, P, r.data());
            for (int i = 0; i < NR; i++) ops.m2m[(size_t)oc * NR * NR + (size_t)i * NR + j] = r[i];
            l2l_c(in, U, P, out);
            to_real(out, P, r.data());
            for (int i = 0; i < NR; i++) ops.l2l[(size_t)oc * NR * NR + (size_t)i * NR + j] = r[i];
        }
    }
    return ops;
}

void fmm_free(Ctx &c);
static int fmm_build_forest(Ctx &c, int L);
template <typename T>
static cudaError_t fmm_eval_t(Ctx &c, FmmTree &t, int nq);

// Points of each sample (sources and target nodes) and the sample's root cube. A batch of
// independent meshes gets one octree per sample (a forest); a single mesh is one tree.
struct SamplePts {
    std::vector<int> src, tgt;  // source indices, target node ids
    double c0[3] = {0, 0, 0}, side = 1.0;
};

// Centre and side of every sample's root cube.
static std::vector<double4> sample_roots(const std::vector<SamplePts> &S) {
    std::vector<double4> r(S.size());
    for (size_t g = 0; g < S.size(); g++) r[g] = make_double4(S[g].c0[0], S[g].c0[1], S[g].c0[2], S[g].side);
    return r;
}

static std::vector<SamplePts> split_samples(const Ctx &c) {
    const int nseg = std::max(1, c.nseg);
    std::vector<SamplePts> S(nseg);
    for (int s = 0; s < c.nsrc; s++) S[c.h_src_seg.empty() ? 0 : c.h_src_seg[s]].src.push_back(s);
    for (int i = 0; i < c.nn; i++)
        if (c.h_mag[i]) S[c.h_node_seg.empty() ? 0 : c.h_node_seg[i]].tgt.push_back(i);
    for (auto &P : S) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int s : P.src)
            for (int d = 0; d < 3; d++) {
                lo[d] = std::min(lo[d], c.h_src_xyz[3 * (size_t)s + d]);
                hi[d] = std::max(hi[d], c.h_src_xyz[3 * (size_t)s + d]);
            }
        for (int i : P.tgt)
            for (int d = 0; d < 3; d++) {
                lo[d] = std::min(lo[d], c.h_xyz[3 * (size_t)i + d]);
                hi[d] = std::max(hi[d], c.h_xyz[3 * (size_t)i + d]);
            }
        if (P.src.empty() && P.tgt.empty()) continue;
        // the root cube of the reference: the points scaled by 2 / max(l) about the centre
        // into a box of width 2.01 (src/fmm_demag.h:52-53, 72), i.e. 1.005 max(l)
        P.side = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2])) * (2.01 / 2.0);
        if (!(P.side > 0)) P.side = 1.0;
        for (int d = 0; d < 3; d++) P.c0[d] = 0.5 * (lo[d] + hi[d]);
    }
    return S;
}

int fmm_build(Ctx &c) {
    const bool fp32 = (c.opts.precision == FG_PREC_FP32_REFINE);
    if (c.opts.fmm_order != 0 && c.opts.fmm_order != FMM_P) {
        c.err = "fmm: only expansion order P=9 is built";
        return FG_EINVAL;
    }
    const auto t_begin = std::chrono::steady_clock::now();
    c.tree_wall_ms = c.tree_sort_ms = 0.0;
    const std::vector<SamplePts> S = split_samples(c);
    // mean number of sources per occupied leaf at each depth, over all samples
    std::vector<double> occ(11, 0.0);
    {
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<std::vector<uint64_t>> keys;
        if (c.opts.fmm_tree_host) {
            for (const SamplePts &P : S) {
                const int n10 = 1 << 10;
                keys.emplace_back();
                keys.back().reserve(P.src.size());
                for (int s : P.src) {
                    int ijk[3];
                    for (int d = 0; d < 3; d++)
                        ijk[d] = std::min(n10 - 1, std::max(0, (int)(((c.h_src_xyz[3 * (size_t)s + d] - P.c0[d]) / P.side + 0.5) * n10)));
                    keys.back().push_back(morton(ijk[0], ijk[1], ijk[2]));
                }
                std::sort(keys.back().begin(), keys.back().end());
            }
        } else {
            // one device sort of all samples' keys (the sample in the bits above the cell's):
            // the distinct prefixes of the sorted keys are the occupied cells of every sample
            keys.emplace_back();
            std::vector<int> idx;
            int *dseg = nullptr;
            cudaError_t e = c.h_src_seg.empty() ? cudaSuccess : up(&dseg, c.h_src_seg);
            if (e == cudaSuccess)
                e = morton_sort(c, c.nsrc, 10, (int)S.size(), c.src_xyz, dseg, sample_roots(S), nullptr, keys.back(),
                                idx, &c.tree_sort_ms);
            if (dseg) cudaFree(dseg);
            FCK(e);
        }
        for (const auto &K : keys)
            for (int l = 2; l <= 10; l++) {
                const int sh = 3 * (10 - l);
                uint64_t prev = ~0ull;
                for (uint64_t k : K)
                    if ((k >> sh) != prev) { occ[l] += 1; prev = k >> sh; }
            }
        c.tree_wall_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    auto closest = [&](double target) {
        int best = 2;
        double bd = 1e300;
        for (int l = 2; l <= 10; l++) {
            const double mean = c.nsrc / std::max(1.0, occ[l]);
            const double d = std::fabs(std::log(mean / target));
            if (d < bd) { bd = d; best = l; }
        }
        return best;
    };
    std::vector<int> cands;
    if (c.opts.fmm_leaf < 0) cands.push_back(std::min(10, std::max(2, -c.opts.fmm_leaf)));  // fixed depth
    else if (c.opts.fmm_leaf > 0) cands.push_back(closest(c.opts.fmm_leaf));
    else {
        const int l0 = closest(fp32 ? 400.0 : 300.0);
        for (int l = std::max(2, l0 - 1); l <= std::min(10, l0 + 1); l++) cands.push_back(l);
    }
    cudaMemsetAsync(c.src_q, 0, sizeof(double) * std::max(1, c.nsrc), c.stream);
    if (c.src_q2) cudaMemsetAsync(c.src_q2, 0, sizeof(double) * std::max(1, c.nsrc), c.stream);
    int bestL = cands[0];
    double bestms = 1e300;
    for (size_t k = 0; k < cands.size(); k++) {
        fmm_free(c);
        FmmTree *t = new FmmTree();
        c.fmm = t;
        t->fp32 = fp32;
        int s = fmm_build_forest(c, cands[k]);
        if (s != FG_OK) return s;
        if (cands.size() == 1) {
            c.fmm_setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_begin).count();
            return FG_OK;
        }
        // autotune: time two evaluations (of all charge sets, as the steps run them) with
        // the current charges (values do not matter)
        cudaEvent_t a, b;
        FCK(cudaEventCreate(&a));
        FCK(cudaEventCreate(&b));
        FCK(fp32 ? fmm_eval_t<float>(c, *t, t->nq) : fmm_eval_t<double>(c, *t, t->nq));
        FCK(cudaEventRecord(a, c.stream));
        for (int r = 0; r < 2; r++)
            FCK(fp32 ? fmm_eval_t<float>(c, *t, t->nq) : fmm_eval_t<double>(c, *t, t->nq));
        FCK(cudaEventRecord(b, c.stream));
        FCK(cudaEventSynchronize(b));
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        if (c.opts.verbose) fprintf(stderr, "fmm autotune: L=%d %.3f ms/eval\n", cands[k], ms / 2);
        if (ms < bestms) { bestms = ms; bestL = cands[k]; }
    }
    fmm_free(c);
    FmmTree *t = new FmmTree();
    c.fmm = t;
    t->fp32 = fp32;
    const int s = fmm_build_forest(c, bestL);
    c.fmm_setup_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_begin).count();
    return s;
}

// Per-sample octree of depth L (host vectors, sample-local indices).
struct TreeH {
    std::vector<uint64_t> leaf_keys;
    std::vector<std::vector<uint64_t>> keys;  // per level
    std::vector<std::pair<uint64_t, int>> sk, tk;  // (leaf key, source index / node id), sorted
    std::vector<int> leaf_src, leaf_tgt;           // CSR over sk / tk
};

static int fmm_build_forest(Ctx &c, int L) {
    const auto t_tree = std::chrono::steady_clock::now();
    FmmTree *t = static_cast<FmmTree *>(c.fmm);
    const bool fp32 = t->fp32;
    t->L = L;
    t->nsrc = c.nsrc;
    t->nq = (c.opts.first_order || !c.src_q2 || !c.pot2) ? 1 : 2;  // m, and v beside it
    const int nside = 1 << L;
    const std::vector<SamplePts> SP = split_samples(c);
    const int nseg = (int)SP.size();
    t->s0 = SP[0].side;
    for (int d = 0; d < 3; d++) t->c0[d] = SP[0].c0[d];
    std::vector<TreeH> T(nseg);
    if (!c.opts.fmm_tree_host) {
        // (leaf key, point) pairs of every sample in key order, from the device radix sort of
        // the sources and of the magnetic nodes
        const uint64_t cell_mask = (1ull << (3 * L)) - 1ull;
        std::vector<uint64_t> keys;
        std::vector<int> idx;
        int *dseg = nullptr;
        cudaError_t e = c.h_src_seg.empty() ? cudaSuccess : up(&dseg, c.h_src_seg);
        if (e == cudaSuccess)
            e = morton_sort(c, c.nsrc, L, nseg, c.src_xyz, dseg, sample_roots(SP), nullptr, keys, idx, &c.tree_sort_ms);
        if (dseg) cudaFree(dseg);
        FCK(e);
        for (size_t k = 0; k < keys.size(); k++) T[keys[k] >> (3 * L)].sk.push_back({keys[k] & cell_mask, idx[k]});
        FCK(morton_sort(c, c.nn, L, nseg, c.xyz, c.batch ? c.node_seg : nullptr, sample_roots(SP), c.mag, keys, idx,
                        &c.tree_sort_ms));
        for (size_t k = 0; k < keys.size(); k++) T[keys[k] >> (3 * L)].tk.push_back({keys[k] & cell_mask, idx[k]});
    }
    for (int g = 0; g < nseg; g++) {
        const SamplePts &P = SP[g];
        TreeH &H = T[g];
        if (c.opts.fmm_tree_host) {
            auto cell_of = [&](const double *p) {
                int ijk[3];
                for (int d = 0; d < 3; d++) ijk[d] = std::min(nside - 1, std::max(0, (int)(((p[d] - P.c0[d]) / P.side + 0.5) * nside)));
                return morton(ijk[0], ijk[1], ijk[2]);
            };
            for (int s : P.src) H.sk.push_back({cell_of(&c.h_src_xyz[3 * (size_t)s]), s});
            for (int i : P.tgt) H.tk.push_back({cell_of(&c.h_xyz[3 * (size_t)i]), i});
            std::sort(H.sk.begin(), H.sk.end());
            std::sort(H.tk.begin(), H.tk.end());
        }
        std::vector<uint64_t> a, b;
        for (auto &p : H.sk) if (a.empty() || a.back() != p.first) a.push_back(p.first);
        for (auto &p : H.tk) if (b.empty() || b.back() != p.first) b.push_back(p.first);
        std::set_union(a.begin(), a.end(), b.begin(), b.end(), std::back_inserter(H.leaf_keys));
        H.leaf_src.assign(H.leaf_keys.size() + 1, 0);
        H.leaf_tgt.assign(H.leaf_keys.size() + 1, 0);
        size_t ia = 0, ib = 0;
        for (size_t l = 0; l < H.leaf_keys.size(); l++) {
            H.leaf_src[l] = (int)ia;
            while (ia < H.sk.size() && H.sk[ia].first == H.leaf_keys[l]) ia++;
            H.leaf_tgt[l] = (int)ib;
            while (ib < H.tk.size() && H.tk[ib].first == H.leaf_keys[l]) ib++;
        }
        H.leaf_src.back() = (int)ia;
        H.leaf_tgt.back() = (int)ib;
        H.keys.assign(L + 1, {});
        H.keys[L] = H.leaf_keys;
        for (int l = L - 1; l >= 2; l--)
            for (uint64_t k : H.keys[l + 1])
                if (H.keys[l].empty() || H.keys[l].back() != (k >> 3)) H.keys[l].push_back(k >> 3);
    }
    // global numbering: level-major, then sample, then Morton order
    t->lev_begin.assign(L + 2, 0);
    std::vector<std::vector<int>> base(L + 1, std::vector<int>(nseg, 0));  // first global id of (level, sample)
    int next = 0;
    for (int l = 2; l <= L; l++) {
        t->lev_begin[l] = next;
        for (int g = 0; g < nseg; g++) {
            base[l][g] = next;
            next += (int)T[g].keys[l].size();
        }
    }
    t->lev_begin[L + 1] = next;
    const int ncell = next;
    t->ncell = ncell;
    t->leaf0 = t->lev_begin[L];
    int nleaf = ncell - t->leaf0;
    t->nleaf = nleaf;
    std::vector<int> leaf_src(nleaf + 1, 0), leaf_tgt(nleaf + 1, 0), leaf_ijk(3 * (size_t)nleaf, 0);
    std::vector<double> leaf_scale(nleaf, 0.0);
    std::vector<int> src_dst(c.nsrc, 0), tgt_node;
    std::vector<double> sloc(4 * (size_t)c.nsrc, 0.0), tloc;
    std::vector<int> nsub_src(ncell, 0), nsub_tgt(ncell, 0);
    std::vector<int> m2m_tab((size_t)ncell * 8, -1), l2l_tab((size_t)ncell * 8, -1);
    std::vector<int> m2l_tab((size_t)ncell * NCODE_M2L, -1);
    std::vector<int> near_ptr(nleaf + 1, 0), near_leaf;
    size_t src_off = 0, tgt_off = 0, nm2l = 0, np2p = 0;
    int ijk[3];
    for (int g = 0; g < nseg; g++) {
        TreeH &H = T[g];
        const SamplePts &P = SP[g];
        const double w = P.side / nside;
        std::vector<std::unordered_map<uint64_t, int>> where(L + 1);
        for (int l = 2; l <= L; l++) {
            where[l].reserve(H.keys[l].size() * 2);
            for (size_t i = 0; i < H.keys[l].size(); i++) where[l][H.keys[l][i]] = base[l][g] + (int)i;
        }
        const int lf0 = base[L][g] - t->leaf0;  // first global leaf index of the sample
        for (size_t l = 0; l < H.leaf_keys.size(); l++) {
            const int gl = lf0 + (int)l;
            leaf_src[gl] = (int)src_off + H.leaf_src[l];
            leaf_tgt[gl] = (int)tgt_off + H.leaf_tgt[l];
            decode(H.leaf_keys[l], &leaf_ijk[3 * (size_t)gl]);
            leaf_scale[gl] = 1.0 / w;
            const int *q = &leaf_ijk[3 * (size_t)gl];
            double cc[3];
            for (int d = 0; d < 3; d++) cc[d] = P.c0[d] - 0.5 * P.side + (q[d] + 0.5) * w;
            for (int k = H.leaf_src[l]; k < H.leaf_src[l + 1]; k++) {
                const size_t gk = src_off + k;
                const int s = H.sk[k].second;
                src_dst[s] = (int)gk;
                for (int d = 0; d < 3; d++) sloc[4 * gk + d] = (c.h_src_xyz[3 * (size_t)s + d] - cc[d]) / w;
            }
            for (int k = H.leaf_tgt[l]; k < H.leaf_tgt[l + 1]; k++) {
                const int i = H.tk[k].second;
                tgt_node.push_back(i);
                for (int d = 0; d < 3; d++) tloc.push_back((c.h_xyz[3 * (size_t)i + d] - cc[d]) / w);
                tloc.push_back(0.0);
            }
            nsub_src[base[L][g] + (int)l] = H.leaf_src[l + 1] - H.leaf_src[l];
            nsub_tgt[base[L][g] + (int)l] = H.leaf_tgt[l + 1] - H.leaf_tgt[l];
        }
        for (int l = L; l >= 3; l--)
            for (size_t i = 0; i < H.keys[l].size(); i++) {
                const int gc = base[l][g] + (int)i;
                const int p = where[l - 1][H.keys[l][i] >> 3];
                const int oc = (int)(H.keys[l][i] & 7);
                nsub_src[p] += nsub_src[gc];
                nsub_tgt[p] += nsub_tgt[gc];
                if (nsub_src[gc] > 0) m2m_tab[(size_t)p * 8 + oc] = gc;
                l2l_tab[(size_t)gc * 8 + oc] = p;
            }
        for (int l = 2; l <= L; l++) {
            const int n = 1 << l;
            for (size_t i = 0; i < H.keys[l].size(); i++) {
                const int gc = base[l][g] + (int)i;
                if (nsub_tgt[gc] == 0) continue;
                decode(H.keys[l][i], ijk);
                const int px = ijk[0] >> 1, py = ijk[1] >> 1, pz = ijk[2] >> 1;
                for (int ax = 2 * (px - 1); ax <= 2 * (px + 1) + 1; ax++)
                    for (int ay = 2 * (py - 1); ay <= 2 * (py + 1) + 1; ay++)
                        for (int az = 2 * (pz - 1); az <= 2 * (pz + 1) + 1; az++) {
                            if (ax < 0 || ay < 0 || az < 0 || ax >= n || ay >= n || az >= n) continue;
                            const int dx = ijk[0] - ax, dy = ijk[1] - ay, dz = ijk[2] - az;
                            if (std::abs(dx) <= 1 && std::abs(dy) <= 1 && std::abs(dz) <= 1) continue;
                            auto it = where[l].find(morton(ax, ay, az));
                            if (it == where[l].end() || nsub_src[it->second] == 0) continue;
                            m2l_tab[(size_t)gc * NCODE_M2L + (dx + 3) * 49 + (dy + 3) * 7 + (dz + 3)] = it->second;
                            nm2l++;
                        }
            }
        }
        for (size_t l = 0; l < H.leaf_keys.size(); l++) {
            const int gl = lf0 + (int)l;
            std::vector<int> nb;
            if (H.leaf_tgt[l + 1] > H.leaf_tgt[l]) {
                const int *q = &leaf_ijk[3 * (size_t)gl];
                for (int dx = -1; dx <= 1; dx++)
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dz = -1; dz <= 1; dz++) {
                            const int ax = q[0] + dx, ay = q[1] + dy, az = q[2] + dz;
                            if (ax < 0 || ay < 0 || az < 0 || ax >= nside || ay >= nside || az >= nside) continue;
                            auto it = where[L].find(morton(ax, ay, az));
                            if (it == where[L].end()) continue;
                            const int nl = it->second - t->leaf0;
                            const int ls = nl - lf0;
                            if (H.leaf_src[ls + 1] == H.leaf_src[ls]) continue;
                            nb.push_back(nl);
                            np2p += (size_t)(H.leaf_src[ls + 1] - H.leaf_src[ls]) * (H.leaf_tgt[l + 1] - H.leaf_tgt[l]);
                        }
            }
            near_leaf.insert(near_leaf.end(), nb.begin(), nb.end());
            near_ptr[gl + 1] = (int)near_leaf.size();
        }
        src_off += H.sk.size();
        tgt_off += H.tk.size();
    }
    leaf_src[nleaf] = (int)src_off;
    leaf_tgt[nleaf] = (int)tgt_off;
    t->n_m2l = nm2l;
    t->n_p2p_pairs = np2p;
    const FmmOps &ops = fmm_ops();
    t->tc = fp32 && c.opts.fmm_tensor != 0;
    if (t->tc) {
        std::vector<int> codes;
        std::vector<int4> units, comb;
        int nslot = 0;
        auto plan = [&](int n_out, int out0, int ncode, const std::vector<int> &tab, int max_codes) {
            FmmTree::TcLaunch l;
            l.unit0 = (int)units.size();
            l.comb0 = (int)comb.size();
            translate_tc_units(n_out, ncode, tab.data(), out0, max_codes, codes, units, comb, nslot);
            l.nunit = (int)units.size() - l.unit0;
            l.ncomb = (int)comb.size() - l.comb0;
            return l;
        };
        t->tc_m2m.assign(L + 1, FmmTree::TcLaunch());
        t->tc_l2l.assign(L + 1, FmmTree::TcLaunch());
        // M2M and L2L run level by level, each level a short launch: units of 2 codes keep
        // its critical path short. M2L has the whole tree in one launch; its unit size is
        // the one whose units, handed in launch order to the earliest free of the SMs' CTA
        // slots (one per SM), finish first: a unit costs its codes plus about 3 codes of
        // pipeline fill, drain and output, and a split tile adds a combine pass
        int m2l_codes = 48;
        {
            std::vector<int> cs;  // codes per tile: one unit per tile
            std::vector<int4> us, cb;
            int ns = 0;
            translate_tc_units(ncell, NCODE_M2L, m2l_tab.data(), 0, 1 << 30, cs, us, cb, ns);
            double best = 1e300;
            const int slots = std::max(1, c.nsm);
            for (int mc : {64, 48, 32, 24, 16, 12, 8}) {
                std::priority_queue<double, std::vector<double>, std::greater<double>> free_at;
                for (int k = 0; k < slots; k++) free_at.push(0.0);
                double span = 0.0;
                bool split = false;
                for (const int4 &u : us) {  // the split of translate_tc_units, unit by unit
                    const int n = u.z - u.y, nu = std::max(1, (n + mc - 1) / mc);
                    split = split || nu > 1;
                    for (int k = 0; k < nu; k++) {
                        const int cnt = (int)((long)n * (k + 1) / nu - (long)n * k / nu);
                        const double t0 = free_at.top();
                        free_at.pop();
                        const double t1 = t0 + 3.0 + cnt;
                        span = std::max(span, t1);
                        free_at.push(t1);
                    }
                }
                span += split ? 1.0 : 0.0;
                if (span < best) {
                    best = span;
                    m2l_codes = mc;
                }
            }
        }
        for (int l = L - 1; l >= 2; l--)
            t->tc_m2m[l] = plan(t->lev_begin[l + 1] - t->lev_begin[l], t->lev_begin[l], 8, m2m_tab, 2);
        t->tc_m2l = plan(ncell, 0, NCODE_M2L, m2l_tab, m2l_codes);
        for (int l = 3; l <= L; l++)
            t->tc_l2l[l] = plan(t->lev_begin[l + 1] - t->lev_begin[l], t->lev_begin[l], 8, l2l_tab, 2);
        FCK(up(&t->tc_code, codes));
        FCK(up(&t->tc_units, units));
        FCK(up(&t->tc_comb, comb));
        t->nslot_floats = (size_t)std::max(1, nslot) * translate_tc_tile() * NR;
        FCK(cudaMalloc(&t->tc_scratch, sizeof(float) * t->nslot_floats * t->nq));
        FCK(cudaMalloc(&t->tc_err, sizeof(int)));
        FCK(cudaMemset(t->tc_err, 0, sizeof(int)));
        FCK(translate_tc_setup());
        const size_t nexp = (size_t)ncell * NR * t->nq;
        FCK(cudaMalloc(&t->Mh, nexp * sizeof(float)));
        FCK(cudaMalloc(&t->Ml, nexp * sizeof(float)));
        FCK(cudaMalloc(&t->Fh, nexp * sizeof(float)));
        FCK(cudaMalloc(&t->Fl, nexp * sizeof(float)));
        FCK(cudaMemset(t->Mh, 0, nexp * sizeof(float)));
        FCK(cudaMemset(t->Ml, 0, nexp * sizeof(float)));
        FCK(cudaMemset(t->Fh, 0, nexp * sizeof(float)));
        FCK(cudaMemset(t->Fl, 0, nexp * sizeof(float)));
        static const std::vector<float> im2l = translate_tc_images(ops.m2l, NCODE_M2L);
        static const std::vector<float> im2m = translate_tc_images(ops.m2m, 8);
        static const std::vector<float> il2l = translate_tc_images(ops.l2l, 8);
        FCK(up((float **)&t->img_m2l, im2l));
        FCK(up((float **)&t->img_m2m, im2m));
        FCK(up((float **)&t->img_l2l, il2l));
    }
    FCK(up(&t->leaf_src, leaf_src));
    FCK(up(&t->leaf_tgt, leaf_tgt));
    FCK(up(&t->tgt_node, tgt_node));
    FCK(up(&t->leaf_ijk, leaf_ijk));
    FCK(up(&t->leaf_scale, leaf_scale));
    FCK(up(&t->m2l_tab, m2l_tab));
    FCK(up(&t->m2m_tab, m2m_tab));
    FCK(up(&t->l2l_tab, l2l_tab));
    FCK(up(&t->near_ptr, near_ptr));
    FCK(up(&t->near_leaf, near_leaf));
    FCK(up_as<double>(&t->sloc, sloc, fp32));
    FCK(up_as<double>(&t->tloc, tloc, fp32));
    t->ds = !fp32 && c.opts.fmm_native_fp64 == 0;
    if (t->ds) {
        // x = hi + lo, hi on the 2^-20 grid (|x| < 4 leaf units: exact in FP32)
        auto split = [](const std::vector<double> &v, std::vector<float4> &hi, std::vector<float4> &lo) {
            const size_t n = v.size() / 4;
            hi.resize(n);
            lo.resize(n);
            for (size_t k = 0; k < n; k++) {
                float h[3], l[3];
                for (int d = 0; d < 3; d++) {
                    const double x = v[4 * k + d];
                    const double xh = std::nearbyint(x * 1048576.0) / 1048576.0;
                    h[d] = (float)xh;
                    l[d] = (float)(x - xh);
                }
                hi[k] = make_float4(h[0], h[1], h[2], 0.f);
                lo[k] = make_float4(l[0], l[1], l[2], 0.f);
            }
        };
        std::vector<float4> sh, sl, th, tl;
        split(sloc, sh, sl);
        split(tloc, th, tl);
        FCK(up(&t->ds_src_hi, sh));
        FCK(up(&t->ds_src_lo, sl));
        FCK(up(&t->ds_tgt_hi, th));
        FCK(up(&t->ds_tgt_lo, tl));
    }
    FCK(up_as<double>(&t->op_m2l, ops.m2l, fp32));
    FCK(up_as<double>(&t->op_m2m, ops.m2m, fp32));
    FCK(up_as<double>(&t->op_l2l, ops.l2l, fp32));
    if (c.src_dst) cudaFree(c.src_dst);
    c.src_dst = nullptr;
    FCK(up(&c.src_dst, src_dst));
    const size_t esz = fp32 ? sizeof(float) : sizeof(double);
    const size_t nexp_all = (size_t)ncell * NR * t->nq;
    FCK(cudaMalloc(&t->M, nexp_all * esz));
    FCK(cudaMalloc(&t->F, nexp_all * esz));
    FCK(cudaMemset(t->M, 0, nexp_all * esz));
    FCK(cudaMemset(t->F, 0, nexp_all * esz));
    if (t->nq == 2) {
        FCK(cudaMalloc(&t->sq2, std::max(1, c.nsrc) * esz));
        FCK(cudaMemset(t->sq2, 0, std::max(1, c.nsrc) * esz));
        if (t->ds) {
            FCK(cudaMalloc(&t->ds_q2, 2 * sizeof(float) * std::max(1, c.nsrc)));
            FCK(cudaMemset(t->ds_q2, 0, 2 * sizeof(float) * std::max(1, c.nsrc)));
        }
    }
    if (fp32) {
        FCK(cudaFuncSetAttribute(k_translate<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, tr_smem<float>()));
    } else {
        FCK(cudaFuncSetAttribute(k_translate<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, tr_smem<double>()));
        FCK(cudaFuncSetAttribute(k_translate_ds, cudaFuncAttributeMaxDynamicSharedMemorySize, tr_ds_smem()));
    }
    if (c.opts.profile)
        for (auto &set : t->ev)
            for (auto &e : set) FCK(cudaEventCreate(&e));
    if (c.opts.profile)
        for (auto &set : t->evn)
            for (auto &e : set) FCK(cudaEventCreate(&e));
    if (c.opts.verbose)
        fprintf(stderr, "fmm: L=%d trees=%d leaves=%d cells=%d m2l=%zu p2p_pairs=%zu (%s)\n", L, nseg, nleaf, ncell,
                t->n_m2l, t->n_p2p_pairs, fp32 ? "fp32" : "fp64");
    c.tree_wall_ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_tree).count();
    return FG_OK;
}

void fmm_free(Ctx &c) {
    FmmTree *t = static_cast<FmmTree *>(c.fmm);
    if (!t) return;
    void *ptrs[] = {t->leaf_scale, t->leaf_src, t->leaf_tgt, t->tgt_node, t->sloc, t->tloc, t->leaf_ijk, t->m2l_tab, t->m2m_tab,
                    t->l2l_tab, t->near_ptr, t->near_leaf, t->M, t->F, t->op_m2l, t->op_m2m, t->op_l2l,
                    t->tc_code, t->tc_units, t->tc_comb, t->tc_scratch, t->tc_err, t->Mh, t->Ml, t->Fh, t->Fl,
                    t->img_m2l, t->img_m2m, t->img_l2l, t->ds_src_hi, t->ds_src_lo, t->ds_tgt_hi, t->ds_tgt_lo,
                    t->sq2, t->ds_q2};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &set : t->ev)
        for (auto &e : set)
            if (e) cudaEventDestroy(e);
    for (auto &set : t->evn)
        for (auto &e : set)
            if (e) cudaEventDestroy(e);
    delete t;
    c.fmm = nullptr;
}

template <typename T> static bool tc_path(const FmmTree &t);
template <> bool tc_path<float>(const FmmTree &t) { return t.tc; }
template <> bool tc_path<double>(const FmmTree &) { return false; }

// Adds the stage times of a recorded event set to the running sums (waits for its last event).
static void harvest_set(FmmTree &t, int k) {
    if (!t.ev_pending[k]) return;
    cudaEventSynchronize(t.ev[k][5]);
    for (int s = 0; s < 5; s++) {
        float ms = 0.f;
        if (s == 4 && t.ev_split[k]) cudaEventElapsedTime(&ms, t.evn[k][0], t.evn[k][1]);  // near field, own stream
        else cudaEventElapsedTime(&ms, t.ev[k][s], t.ev[k][s + 1]);
        t.stage_sum[s] += ms;
    }
    t.stage_n++;
    t.ev_pending[k] = false;
}

// One FMM evaluation of nq charge sets: set 0 from c.src_q into c.pot, set 1 (nq = 2) from
// c.src_q2 into c.pot2. The sets share every table, operator image and launch (grid y of
// P2M and of the tensor-core translations; one near-field pass computes both).
template <typename T>
static cudaError_t fmm_eval_t(Ctx &c, FmmTree &t, int nq) {
    if (nq < 1 || nq > t.nq || (nq == 2 && (!c.src_q2 || !c.pot2))) return cudaErrorInvalidValue;
    const int L = t.L;
    T *M = (T *)t.M, *F = (T *)t.F;
    constexpr int TB = TrShape<T>::TB;
    const size_t sstride = (size_t)t.ncell * NR;  // elements between the sets' expansions
    const bool prof = c.opts.profile && t.ev[0][0];
    cudaEvent_t *ev = t.ev[t.ev_next];
    if (prof) {
        harvest_set(t, t.ev_next);
        cudaEventRecord(ev[0], c.stream);
    }
    const bool tc = tc_path<T>(t);
    P2mSet<T> ps[2];
    for (int k = 0; k < 2; k++) {
        const int q = k < nq ? k : 0;
        P2mSet<T> &p = ps[k];
        p.q = q ? c.src_q2 : c.src_q;
        p.qf = (sizeof(T) == 4 && c.charges32) ? (q ? c.src_q2f : c.src_qf) : nullptr;
        p.M = M + q * sstride;
        p.Mh = tc ? t.Mh + q * sstride : nullptr;
        p.Ml = tc ? t.Ml + q * sstride : nullptr;
        p.qn = q ? (T *)t.sq2 : (T *)t.sloc + 3;
        p.qn_stride = q ? 1 : 4;
        p.qh = p.ql = nullptr;
        p.qd_stride = q ? 1 : 4;
        if (t.ds) {
            p.qh = q ? t.ds_q2 : (float *)t.ds_src_hi + 3;
            p.ql = q ? t.ds_q2 + t.nsrc : (float *)t.ds_src_lo + 3;
        }
    }
    // overlapped evaluation: after P2M (which stores the near field's charges) and M2M, the
    // near field runs on the second, lower-priority stream beside M2L and L2L: an FP32
    // near-field block (128 threads x 128 registers) fits on an SM beside a tensor-core
    // translation CTA (288 x 168), so the FP32 and SFU pipes work while the tensor pipe
    // does; L2P follows once both are done. (Forked before P2M, the near field's blocks took
    // every SM first and the short M2M launches waited behind them.)
    const bool split = c.opts.fmm_overlap != 0 && c.stream2 != nullptr;
    NearSets<T> ns;
    ns.q2 = nq == 2 ? (const T *)t.sq2 : nullptr;
    ns.F[0] = F;
    ns.F[1] = F + (nq == 2 ? sstride : 0);
    ns.pot[0] = c.pot;
    ns.pot[1] = nq == 2 ? c.pot2 : c.pot;
    ns.near_only = 0;
    const int nb = (t.nleaf + 3) / 4;
    auto near_field = [&](cudaStream_t st) {
        if constexpr (sizeof(T) == 8) {
            if (t.ds) {
                auto k = nq == 2 ? k_l2p_p2p_ds<2> : k_l2p_p2p_ds<1>;
                k<<<nb, 128, 0, st>>>(t.nleaf, t.leaf_src, t.leaf_tgt, t.tgt_node, (const double *)t.tloc, t.ds_tgt_hi,
                                      t.ds_tgt_lo, t.ds_src_hi, t.ds_src_lo, t.ds_q2,
                                      t.ds_q2 ? t.ds_q2 + t.nsrc : nullptr, t.leaf_ijk, t.leaf0, t.leaf_scale,
                                      t.near_ptr, t.near_leaf, ns);
            }
        }
        if (!t.ds) {
            auto k = nq == 2 ? k_l2p_p2p<T, 2> : k_l2p_p2p<T, 1>;
            k<<<nb, 128, 0, st>>>(t.nleaf, t.leaf_src, t.leaf_tgt, t.tgt_node, (const T *)t.tloc, (const T *)t.sloc,
                                  t.leaf_ijk, t.leaf0, t.leaf_scale, t.near_ptr, t.near_leaf, ns);
        }
    };
    t.ev_split[t.ev_next] = split && prof;
    if constexpr (sizeof(T) == 4) {
        (nq == 2 ? k_p2m2<2> : k_p2m2<1>)<<<(t.nleaf + 3) / 4, 128, 0, c.stream>>>(
            t.nleaf, t.leaf_src, (const float *)t.sloc, t.leaf0, ps[0], ps[1]);
    } else if (t.ds) {
        (nq == 2 ? k_p2m_ds<2> : k_p2m_ds<1>)<<<(t.nleaf + 3) / 4, 128, 0, c.stream>>>(
            t.nleaf, t.leaf_src, (const float4 *)t.ds_src_hi, (const float4 *)t.ds_src_lo, t.leaf0, ps[0], ps[1]);
    } else {
        k_p2m<T><<<dim3((t.nleaf + 3) / 4, nq), 128, 0, c.stream>>>(t.nleaf, t.leaf_src, (const T *)t.sloc, t.leaf0,
                                                                     ps[0], ps[1]);
    }
    if (prof) cudaEventRecord(ev[1], c.stream);
    // out (+)= sum_code Op[code] in[tab[cell][code]] over n output cells from out0; the
    // tensor-core form reads the inputs' hi/lo split and writes the outputs' split
    enum { M2M, M2L, L2L };
    cudaError_t terr = cudaSuccess;  // first failed translation launch
    auto translate = [&](int kind, int n, int out0, const FmmTree::TcLaunch &tl) {
        if (!n) return;
        const int ncode = kind == M2L ? NCODE_M2L : 8;
        const int *tab = kind == M2M ? t.m2m_tab : kind == M2L ? t.m2l_tab : t.l2l_tab;
        if (tc) {
            TcArgs a{};
            a.n_out = n; a.out0 = out0; a.ncode = ncode; a.tab = tab;
            a.op_img = kind == M2M ? t.img_m2m : kind == M2L ? t.img_m2l : t.img_l2l;
            a.in_hi = kind == L2L ? t.Fh : t.Mh;
            a.in_lo = kind == L2L ? t.Fl : t.Ml;
            a.out = (float *)(kind == M2M ? M : F);
            a.out_hi = kind == M2M ? t.Mh : t.Fh;
            a.out_lo = kind == M2M ? t.Ml : t.Fl;
            a.accumulate = kind == L2L;
            a.tile_code = t.tc_code; a.err = t.tc_err; a.terms = 7;
            a.units = t.tc_units + tl.unit0; a.nunits = tl.nunit;
            a.comb = t.tc_comb + tl.comb0; a.ncomb = tl.ncomb; a.scratch = t.tc_scratch;
            a.nset = nq; a.set_io = sstride; a.set_scratch = t.nslot_floats;
            const cudaError_t e = launch_translate_tc(c.stream, a);
            if (e != cudaSuccess && terr == cudaSuccess) terr = e;
        } else if (sizeof(T) == 8 && t.ds) {  // FP64 path: double-single, both sets per launch
            const double *ops = (const double *)(kind == M2M ? t.op_m2m : kind == M2L ? t.op_m2l : t.op_l2l);
            double *in = (double *)(kind == L2L ? F : M), *out = (double *)(kind == M2M ? M : F);
            k_translate_ds<<<(n + DS_TB - 1) / DS_TB, 160, tr_ds_smem(), c.stream>>>(n, out0, ncode, tab, ops, in, out,
                                                                                     kind == L2L, nq, sstride);
        } else {
            const void *ops = kind == M2M ? t.op_m2m : kind == M2L ? t.op_m2l : t.op_l2l;
            for (int q = 0; q < nq; q++) {
                T *in = (kind == L2L ? F : M) + q * sstride, *out = (kind == M2M ? M : F) + q * sstride;
                k_translate<T><<<(n + TB - 1) / TB, 160, tr_smem<T>(), c.stream>>>(n, out0, ncode, tab,
                                                                                (const T *)ops, in, out, kind == L2L);
            }
        }
    };
    const FmmTree::TcLaunch none;
    for (int l = L - 1; l >= 2; l--)
        translate(M2M, t.lev_begin[l + 1] - t.lev_begin[l], t.lev_begin[l], t.tc ? t.tc_m2m[l] : none);
    if (prof) cudaEventRecord(ev[2], c.stream);
    if (split) {  // the near field beside M2L and L2L
        cudaEventRecord(c.ev_fork, c.stream);
        cudaStreamWaitEvent(c.stream2, c.ev_fork, 0);
        ns.near_only = 1;
        if (prof) cudaEventRecord(t.evn[t.ev_next][0], c.stream2);
        near_field(c.stream2);
        if (prof) cudaEventRecord(t.evn[t.ev_next][1], c.stream2);
        cudaEventRecord(c.ev_join, c.stream2);
        ns.near_only = 0;
    }
    translate(M2L, t.ncell, 0, t.tc_m2l);
    if (prof) cudaEventRecord(ev[3], c.stream);
    for (int l = 3; l <= L; l++)
        translate(L2L, t.lev_begin[l + 1] - t.lev_begin[l], t.lev_begin[l], t.tc ? t.tc_l2l[l] : none);
    if (prof) cudaEventRecord(ev[4], c.stream);
    if (split) {
        cudaStreamWaitEvent(c.stream, c.ev_join, 0);
        auto k = nq == 2 ? k_l2p<T, 2> : k_l2p<T, 1>;
        k<<<nb, 128, 0, c.stream>>>(t.nleaf, t.leaf_tgt, t.tgt_node, (const T *)t.tloc, t.leaf0, t.leaf_scale, ns);
    } else {
        near_field(c.stream);
    }
    if (prof) {
        cudaEventRecord(ev[5], c.stream);
        t.ev_pending[t.ev_next] = true;
        t.ev_next ^= 1;
    }
    const cudaError_t e = cudaGetLastError();
    return terr != cudaSuccess ? terr : e;
}

cudaError_t fmm_eval(Ctx &c, int nq) {
    FmmTree *t = static_cast<FmmTree *>(c.fmm);
    if (!t) return cudaErrorNotSupported;
    return t->fp32 ? fmm_eval_t<float>(c, *t, nq) : fmm_eval_t<double>(c, *t, nq);
}

int fmm_eval_fp64(Ctx &c, int nq) {
    FmmTree *t32 = static_cast<FmmTree *>(c.fmm);
    if (!t32) {
        c.err = "fmm: no tree";
        return FG_EINVAL;
    }
    if (!t32->fp32) {
        FCK(fmm_eval_t<double>(c, *t32, nq));
        return FG_OK;
    }
    if (!c.fmm64) {
        // the same depth (and so the same source order, src_dst) as the FP32 tree
        FmmTree *t = new FmmTree();
        t->fp32 = false;
        c.fmm = t;
        const int s = fmm_build_forest(c, t32->L);
        if (s != FG_OK) {
            fmm_free(c);
            c.fmm = t32;
            return s;
        }
        c.fmm64 = t;
        c.fmm = t32;
    }
    FCK(fmm_eval_t<double>(c, *static_cast<FmmTree *>(c.fmm64), nq));
    return FG_OK;
}

void fmm64_free(Ctx &c) {
    if (!c.fmm64) return;
    void *keep = c.fmm;
    c.fmm = c.fmm64;
    fmm_free(c);
    c.fmm = keep;
    c.fmm64 = nullptr;
}

int fmm_stage_ms(const Ctx &c, double ms[5]) {
    FmmTree *t = static_cast<FmmTree *>(c.fmm);
    if (!t) return FG_EINVAL;
    harvest_set(*t, t->ev_next ^ 1);
    harvest_set(*t, t->ev_next);
    for (int k = 0; k < 5; k++) ms[k] = t->stage_n ? t->stage_sum[k] / t->stage_n : 0.0;
    for (double &x : t->stage_sum) x = 0.0;
    t->stage_n = 0;
    return FG_OK;
}

int fmm_launches_per_eval(const Ctx &c, int nq) {
    const FmmTree *t = static_cast<const FmmTree *>(c.fmm);
    if (!t) return 0;
    int n = 2;  // P2M, L2P + P2P (both sets in one launch each)
    if (c.opts.fmm_overlap != 0 && c.stream2) n += 1;  // L2P after the overlapped near field
    // tensor-core and double-single translations: both sets in one launch (the tensor-core
    // form adds one combine launch); the k_translate form launches once per set
    const int per = (t->tc || (!t->fp32 && t->ds)) ? 1 : nq;
    for (int l = 2; l <= t->L - 1; l++) n += per + (t->tc && t->tc_m2m[l].ncomb > 0);
    n += per + (t->tc && t->tc_m2l.ncomb > 0);
    for (int l = 3; l <= t->L; l++) n += per + (t->tc && t->tc_l2l[l].ncomb > 0);
    return n;
}

int *fmm_error_flag(const Ctx &c) {
    const FmmTree *t = static_cast<const FmmTree *>(c.fmm);
    return t ? t->tc_err : nullptr;
}

int fmm_info(const Ctx &c, int *L, int *nleaf, double *n_m2l, double *n_p2p) {
    const FmmTree *t = static_cast<const FmmTree *>(c.fmm);
    if (!t) return FG_EINVAL;
    *L = t->L;
    *nleaf = t->nleaf;
    *n_m2l = (double)t->n_m2l;
    *n_p2p = (double)t->n_p2p_pairs;
    return FG_OK;
}

}  // namespace fg
