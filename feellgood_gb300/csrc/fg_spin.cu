// Spin accumulation coupling (spin_accumulation.enable): the electrostatic potential V of
// the current flowing between two surfaces (electrostatSolver, src/electrostatSolver.cpp),
// solved once; the spin accumulation s (spinAcc, src/spinAccumulationSolver.cpp), solved in
// every compute_all (src/fem.h:203-224); its field Hst = D0 / (lsd^2 gamma0 Ms) s at the
// Gauss points enters the next step's element integrals (src/tetra.cpp:248-303).
//
// Both problems live on all tetrahedra and nodes (metals as well as magnets). The spin
// operator is factorised like the LLG one: a static scalar operator A on the node graph,
// A_ij = sum_t D0 sum_g w_g (da_i . da_j) + delta_ij sum_t (D0 / lsf^2) a_w,i, the same for
// the three components, plus the magnetic coupling c_i (x_i x m_i) with
// c_i = sum_(magnetic t) (D0 / lsd^2) a_w,i and m the CURRENT magnetisation
// (Tet::calcOffDiagBlock). The RHS is G_i m_i (m of NEXT, G_i = sum_t cst0 sum_g w_g
// (grad V . da_i), cst0 = muB P sigma / e) plus the static surface terms; Dirichlet values on
// the surface nodes. The per-step solve is the reference's bicg_dir with Dirichlet values
// (src/algebra/bicg.h:82-153) as one persistent cooperative kernel, FP64.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <type_traits>
#include <vector>

#include "fg_device.cuh"
#include "fg_internal.h"

namespace fg {

namespace {

constexpr double CHARGE_ELECTRON = 1.602176634e-19;
constexpr double PLANCKS_HBAR = 6.62607015e-34 / (2 * M_PI);
constexpr double MASS_ELECTRON = 9.1093837139e-31;
constexpr double BOHRS_MUB = CHARGE_ELECTRON * PLANCKS_HBAR / (2. * MASS_ELECTRON);

struct SpinArgs {
    int nn;
    const int *ptr, *col;
    const double *A, *dinv, *cc, *G, *L, *xd;
    const unsigned char *dir;
    const double *m0, *m1;  // CURRENT (operator) and NEXT (RHS) magnetisation
    double *x, *r, *rt, *p, *phat, *v, *s, *shat, *t, *out;
    double *partial;
    GridBar *bar;
    SolveResult *res;
    double tol;
    int maxiter;
    // FP32 body with FP64 refinement (FG_PREC_FP32_REFINE): the operator scaled by `scale`
    // in FP32, CURRENT m in FP32, FP64 b and refinement residual, FP32 Krylov vectors
    // (the FP32 vectors are padded to n4 float4 chunks; dinv3 is the Jacobi factor per
    // component, zero at Dirichlet nodes and in the padding)
    const float *A32, *cc32, *dinv3;
    float *m32;
    int n4;
    double *b64, *r64;
    float *fr, *frt, *fp, *fphat, *fv, *fs, *fshat, *ft, *fd;
    double scale, inner_tol;
    int refine_max;
};

// One row of y = A x + c (x x m), zero at Dirichlet nodes, on LPR lanes (the group's lanes
// split the row's entries and combine with shuffles; every lane of the warp takes part).
template <typename T, int LPR>
__device__ __forceinline__ void spin_row(bool valid, int i, int sub, const int *__restrict__ ptr,
                                         const int *__restrict__ col, const T *__restrict__ A,
                                         const T *__restrict__ cc, const T *m, const unsigned char *__restrict__ dir,
                                         const T *x, T y[3]) {
    T s0 = 0, s1 = 0, s2 = 0;
    if (valid) {
        const int k1 = ptr[i + 1];
        for (int k = ptr[i] + sub; k < k1; k += LPR) {
            const int j = col[k];
            const T w = A[k];
            s0 += w * __ldcg(x + 3 * j);
            s1 += w * __ldcg(x + 3 * j + 1);
            s2 += w * __ldcg(x + 3 * j + 2);
        }
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    y[0] = y[1] = y[2] = T(0);
    if (!valid || dir[i]) return;
    const T c = cc[i];
    if (c != T(0)) {
        const T x0 = __ldcg(x + 3 * i), x1 = __ldcg(x + 3 * i + 1), x2 = __ldcg(x + 3 * i + 2);
        const T m0 = __ldcg(m + 3 * i), m1 = __ldcg(m + 3 * i + 1), m2 = __ldcg(m + 3 * i + 2);
        s0 += c * (x1 * m2 - x2 * m1);
        s1 += c * (x2 * m0 - x0 * m2);
        s2 += c * (x0 * m1 - x1 * m0);
    }
    y[0] = s0;
    y[1] = s1;
    y[2] = s2;
}

constexpr int SPIN_LPR = 4;

// Rows in groups of SPIN_LPR lanes, the loop warp-uniform: body(i, valid, sub).
#define SPIN_ROWS(body)                                                                                 \
    for (int gb_ = (blockIdx.x * (int)blockDim.x + (int)(threadIdx.x & ~31)) / SPIN_LPR; gb_ < nn;      \
         gb_ += gstride) {                                                                              \
        const int i_ = gb_ + (int)(threadIdx.x & 31) / SPIN_LPR;                                        \
        body(i_, i_ < nn, (int)threadIdx.x % SPIN_LPR);                                                 \
    }

// bicg_dir with Dirichlet values (src/algebra/bicg.h:82-153), every dot product formed as in
// the reference (five grid barriers per iteration: forming rho and |r| from the iteration's
// other sums instead stalled at tight tolerances).
__global__ void __launch_bounds__(256) k_spin_bicg(SpinArgs a) {
    const int G = gridDim.x, nn = a.nn;
    const int stride = G * blockDim.x, i0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int gstride = G * (int)blockDim.x / SPIN_LPR;
    // b = rhs - K xd (masked); x = 0 (the reference starts from a zero vector), r = rt = p = b
    {
        double bb = 0.0;
        auto row = [&](int i, bool valid, int sub) {
            double y[3];
            spin_row<double, SPIN_LPR>(valid, i, sub, a.ptr, a.col, a.A, a.cc, a.m0, a.dir, a.xd, y);
            if (!valid || sub != 0) return;
            const bool d = a.dir[i];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int k = 3 * i + c;
                const double b = d ? 0.0 : a.G[i] * a.m1[k] + a.L[k] - y[c];
                a.x[k] = 0.0;
                a.r[k] = b;
                a.rt[k] = b;
                a.p[k] = b;
                bb += b * b;
            }
        };
        SPIN_ROWS(row)
        double v1[1] = {bb};
        block_store<1>(v1, a.partial, G);
    }
    if (!grid_sync(a.bar)) goto timeout;
    {
        double s1[1];
        grid_sum<1>(a.partial, G, s1);
        const double rhsn = sqrt(fabs(s1[0]));
        double rr = s1[0], rtr = s1[0];
        double rho1 = 0.0, rho2 = 0.0, alpha = 0.0, beta = 0.0, omega = 0.0;
        int status = -1, nit = 0;
        double res = sqrt(fabs(rr));
        const double res0 = res;
        auto finished = [&](double nr) {  // iteration::finished (src/algebra/iter.h:119-175)
            res = fabs(nr);
            if (isnan(res)) {
                status = 2;
                return false;
            }
            const bool cv = res <= rhsn * a.tol;
            if (cv) status = 0;
            return cv;
        };
        while (!finished(sqrt(fabs(rr)))) {
            rho1 = rtr;
            if (nit > 0) {
                if (rho2 == 0.0 || omega == 0.0) {
                    status = 2;
                    break;
                }
                beta = (rho1 / rho2) * (alpha / omega);
            }
            for (int i = i0; i < nn; i += stride) {
                const double di = a.dinv[i];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const int k = 3 * i + c;
                    double pv = a.p[k];
                    if (nit > 0) {
                        pv = (pv - omega * a.v[k]) * beta + a.r[k];
                        a.p[k] = pv;
                    }
                    a.phat[k] = di * pv;
                }
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double vr = 0.0;
                auto row = [&](int i, bool valid, int sub) {
                    double y[3];
                    spin_row<double, SPIN_LPR>(valid, i, sub, a.ptr, a.col, a.A, a.cc, a.m0, a.dir, a.phat, y);
                    if (!valid || sub != 0) return;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        a.v[3 * i + c] = y[c];
                        vr += y[c] * a.rt[3 * i + c];
                    }
                };
                SPIN_ROWS(row)
                double v1[1] = {vr};
                block_store<1>(v1, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s1b[1];
                grid_sum<1>(a.partial, G, s1b);
                alpha = rho1 / s1b[0];
            }
            {
                double ss = 0.0;
                for (int i = i0; i < nn; i += stride) {
                    const double di = a.dinv[i];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const int k = 3 * i + c;
                        const double sv = a.r[k] + (-alpha) * a.v[k];
                        a.s[k] = sv;
                        a.shat[k] = di * sv;
                        ss += sv * sv;
                    }
                }
                double v1[1] = {ss};
                block_store<1>(v1, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s1c[1];
                grid_sum<1>(a.partial, G, s1c);
                if (finished(sqrt(fabs(s1c[0])))) {
                    for (int i = i0; i < nn; i += stride)
#pragma unroll
                        for (int c = 0; c < 3; c++) a.x[3 * i + c] += alpha * a.phat[3 * i + c];
                    break;
                } else if (status == 1 || status == 2) {
                    break;
                }
            }
            {
                double ts = 0.0, tt = 0.0;
                auto row = [&](int i, bool valid, int sub) {
                    double y[3];
                    spin_row<double, SPIN_LPR>(valid, i, sub, a.ptr, a.col, a.A, a.cc, a.m0, a.dir, a.shat, y);
                    if (!valid || sub != 0) return;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        a.t[3 * i + c] = y[c];
                        ts += y[c] * a.s[3 * i + c];
                        tt += y[c] * y[c];
                    }
                };
                SPIN_ROWS(row)
                double v2[2] = {ts, tt};
                block_store<2>(v2, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s2[2];
                grid_sum<2>(a.partial, G, s2);
                omega = s2[0] / s2[1];
            }
            {
                double r2 = 0.0, rtr2 = 0.0;
                for (int i = i0; i < nn; i += stride)
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const int k = 3 * i + c;
                        double xv = a.x[k] + alpha * a.phat[k];
                        xv += omega * a.shat[k];
                        a.x[k] = xv;
                        const double rv = a.s[k] - omega * a.t[k];
                        a.r[k] = rv;
                        r2 += rv * rv;
                        rtr2 += a.rt[k] * rv;
                    }
                double v2[2] = {r2, rtr2};
                block_store<2>(v2, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s2c[2];
                grid_sum<2>(a.partial, G, s2c);
                rr = s2c[0];
                rtr = s2c[1];
            }
            rho2 = rho1;
            nit++;
            if (nit >= a.maxiter) status = 1;
        }
        // spinAcc::solve / compute: s = x + xd when converged, zero otherwise
        const bool ok = (status == 0);
        for (int k = i0; k < 3 * nn; k += stride) a.out[k] = ok ? a.x[k] + a.xd[k] : 0.0;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.res->status = status;
            a.res->nit = nit;
            a.res->fail = ok ? 0 : 1;
            a.res->res = res;
            a.res->rhsn = rhsn;
            a.res->res0 = res0;
        }
        return;
    }
timeout:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.res->timeout = 1;
        a.res->fail = 1;
    }
}

// The same problem with an FP32 Krylov body and FP64 iterative refinement (the arithmetic
// of the LLG solve in FG_PREC_FP32_REFINE):
//   outer (FP64): r = b - K x; stop when |r| <= tol |b|, the reference's test on the true
//                 residual; status 1 after refine_max sweeps or maxiter inner iterations;
//   inner (FP32): Jacobi BiCGSTAB on (scale K) d = r / |r| from d = 0, dot products summed
//                 in FP32 per warp and FP64 across warps and blocks, the recurrence scalars
//                 in FP64 once per block, to the relative target max(inner_tol,
//                 0.3 tol |b| / |r|);
//   x += scale |r| d in FP64.
// Launched as four blocks of 256 threads per SM or one of 1024 (the same 32 warps per SM, a
// quarter of the blocks meeting at each grid barrier); every reduction works for either size.
__global__ void __launch_bounds__(1024, 1) k_spin_mixed(SpinArgs a) {
    const int G = gridDim.x, nn = a.nn;
    const int stride = G * blockDim.x, i0 = blockIdx.x * blockDim.x + threadIdx.x;
    const int gstride = G * (int)blockDim.x / SPIN_LPR;
    // FP32 CURRENT m; b = rhs - K xd (FP64, masked) = the first refinement residual; x = 0
    for (int k = i0; k < 3 * nn; k += stride) {
        a.m32[k] = (float)a.m0[k];
        a.x[k] = 0.0;
    }
    {
        double bb = 0.0;
        auto row = [&](int i, bool valid, int sub) {
            double y[3];
            spin_row<double, SPIN_LPR>(valid, i, sub, a.ptr, a.col, a.A, a.cc, a.m0, a.dir, a.xd, y);
            if (!valid || sub != 0) return;
            const bool d = a.dir[i];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int k = 3 * i + c;
                const double b = d ? 0.0 : a.G[i] * a.m1[k] + a.L[k] - y[c];
                a.b64[k] = b;
                a.r64[k] = b;
                bb += b * b;
            }
        };
        SPIN_ROWS(row)
        double v1[1] = {bb};
        block_store<1>(v1, a.partial, G);
    }
    if (!grid_sync(a.bar)) goto timeout;
    {
        double s1[1];
        grid_sum<1>(a.partial, G, s1);
        const double rhsn = sqrt(fabs(s1[0]));
        double res = rhsn;
        const double res0 = res;
        int status = -1, nit = 0, nref = 0;
        for (;;) {
            if (nref > 0) {
                // refinement residual r64 = b - K x (FP64)
                double rr = 0.0;
                auto row = [&](int i, bool valid, int sub) {
                    double y[3];
                    spin_row<double, SPIN_LPR>(valid, i, sub, a.ptr, a.col, a.A, a.cc, a.m0, a.dir, a.x, y);
                    if (!valid || sub != 0) return;
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const double rv = a.b64[3 * i + c] - y[c];
                        a.r64[3 * i + c] = rv;
                        rr += rv * rv;
                    }
                };
                SPIN_ROWS(row)
                double v1[1] = {rr};
                block_store<1>(v1, a.partial, G);
                if (!grid_sync(a.bar)) goto timeout;
                double s1r[1];
                grid_sum<1>(a.partial, G, s1r);
                res = block_once([=] { return sqrt(fabs(s1r[0])); });
            }
            if (isnan(res)) { status = 2; break; }
            if (res <= rhsn * a.tol) { status = 0; break; }
            if (nref >= a.refine_max || nit >= a.maxiter) { status = 1; break; }
            const double target = block_once([=] { return fmax(a.inner_tol, 0.3 * a.tol * rhsn / res); });
            const double target2 = target * target;
            {
                float rr = 0.0f;
                const float inv = (float)block_once([=] { return 1.0 / res; });
                for (int k = i0; k < 3 * nn; k += stride) {
                    const float rv = (float)a.r64[k] * inv;
                    a.fr[k] = rv;
                    a.frt[k] = rv;
                    a.fp[k] = rv;
                    a.fd[k] = 0.0f;
                    rr += rv * rv;
                }
                float v1[1] = {rr};
                block_store_f<1>(v1, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s1i[1];
                grid_sum<1>(a.partial, G, s1i);
                double rr = s1i[0], rtr = s1i[0];
                double rho1 = 0.0, rho2 = 0.0, alpha = 0.0, beta = 0.0, omega = 0.0;
                // four grid barriers per iteration, as k_mixed: the update d += alpha phat +
                // omega shat, r = s - omega t of a full iteration is carried into the first phase
                // of the next pass, and |r|^2, rt . r come from the recurrence on the partial
                // sums of the t phase
                bool pending = false;
                for (int it = 0;; it++) {
                    bool cont = rr > target2 && nit < a.maxiter;
                    if (cont) {
                        rho1 = rtr;
                        if (it > 0) {
                            if (rho2 == 0.0 || omega == 0.0) cont = false;
                            else beta = block_once([=] { return (rho1 / rho2) * (alpha / omega); });
                        }
                    }
                    if (pending || cont) {
                        const float fa = (float)alpha, fb = (float)beta, fo = (float)omega;
                        const bool upd = pending, go = cont, later = it > 0;
                        float4 *__restrict__ P = reinterpret_cast<float4 *>(a.fp);
                        float4 *__restrict__ PH = reinterpret_cast<float4 *>(a.fphat);
                        float4 *__restrict__ R4 = reinterpret_cast<float4 *>(a.fr);
                        float4 *__restrict__ D4 = reinterpret_cast<float4 *>(a.fd);
                        const float4 *__restrict__ V = reinterpret_cast<const float4 *>(a.fv);
                        const float4 *__restrict__ SH = reinterpret_cast<const float4 *>(a.fshat);
                        const float4 *__restrict__ S4 = reinterpret_cast<const float4 *>(a.fs);
                        const float4 *__restrict__ T4 = reinterpret_cast<const float4 *>(a.ft);
                        const float4 *__restrict__ D = reinterpret_cast<const float4 *>(a.dinv3);
                        for (int q = i0; q < a.n4; q += stride) {
                            float4 rv = make_float4(0.f, 0.f, 0.f, 0.f);
                            if (upd) {
                                float4 d = D4[q];
                                const float4 h = PH[q], g = SH[q];
                                d.x += fa * h.x + fo * g.x; d.y += fa * h.y + fo * g.y;
                                d.z += fa * h.z + fo * g.z; d.w += fa * h.w + fo * g.w;
                                D4[q] = d;
                                if (go) {
                                    const float4 sv = S4[q], t = T4[q];
                                    rv = make_float4(sv.x - fo * t.x, sv.y - fo * t.y, sv.z - fo * t.z, sv.w - fo * t.w);
                                    R4[q] = rv;
                                }
                            } else if (go) {
                                rv = R4[q];
                            }
                            if (go) {
                                float4 pv = P[q];
                                if (later) {
                                    const float4 v = V[q];
                                    pv.x = rv.x + fb * (pv.x - fo * v.x);
                                    pv.y = rv.y + fb * (pv.y - fo * v.y);
                                    pv.z = rv.z + fb * (pv.z - fo * v.z);
                                    pv.w = rv.w + fb * (pv.w - fo * v.w);
                                    P[q] = pv;
                                }
                                const float4 d = D[q];
                                PH[q] = make_float4(d.x * pv.x, d.y * pv.y, d.z * pv.z, d.w * pv.w);
                            }
                        }
                    }
                    pending = false;
                    if (!cont) break;
                    if (!grid_sync(a.bar)) goto timeout;
                    {
                        float vr = 0.0f;
                        auto row = [&](int i, bool valid, int sub) {
                            float y[3];
                            spin_row<float, SPIN_LPR>(valid, i, sub, a.ptr, a.col, a.A32, a.cc32, a.m32, a.dir,
                                                      a.fphat, y);
                            if (!valid || sub != 0) return;
#pragma unroll
                            for (int c = 0; c < 3; c++) {
                                a.fv[3 * i + c] = y[c];
                                vr += y[c] * a.frt[3 * i + c];
                            }
                        };
                        SPIN_ROWS(row)
                        float v1[1] = {vr};
                        block_store_f<1>(v1, a.partial, G);
                    }
                    if (!grid_sync(a.bar)) goto timeout;
                    {
                        double s1b[1];
                        grid_sum<1>(a.partial, G, s1b);
                        alpha = block_once([=] { return rho1 / s1b[0]; });
                    }
                    double ssum = 0.0;
                    {
                        float ss = 0.0f;
                        const float fa = (float)alpha;
                        float4 *__restrict__ S4 = reinterpret_cast<float4 *>(a.fs);
                        float4 *__restrict__ SH = reinterpret_cast<float4 *>(a.fshat);
                        const float4 *__restrict__ R = reinterpret_cast<const float4 *>(a.fr);
                        const float4 *__restrict__ V = reinterpret_cast<const float4 *>(a.fv);
                        const float4 *__restrict__ D = reinterpret_cast<const float4 *>(a.dinv3);
                        for (int q = i0; q < a.n4; q += stride) {
                            const float4 r = R[q], v = V[q], d = D[q];
                            const float4 sv = make_float4(r.x - fa * v.x, r.y - fa * v.y, r.z - fa * v.z, r.w - fa * v.w);
                            S4[q] = sv;
                            SH[q] = make_float4(d.x * sv.x, d.y * sv.y, d.z * sv.z, d.w * sv.w);
                            ss += sv.x * sv.x + sv.y * sv.y + sv.z * sv.z + sv.w * sv.w;
                        }
                        float v1[1] = {ss};
                        block_store_f<1>(v1, a.partial, G);
                    }
                    if (!grid_sync(a.bar)) goto timeout;
                    {
                        double s1c[1];
                        grid_sum<1>(a.partial, G, s1c);
                        ssum = s1c[0];
                        if (ssum <= target2) {
                            const float fa = (float)alpha;
                            float4 *__restrict__ D4 = reinterpret_cast<float4 *>(a.fd);
                            const float4 *__restrict__ PH = reinterpret_cast<const float4 *>(a.fphat);
                            for (int q = i0; q < a.n4; q += stride) {
                                float4 d = D4[q];
                                const float4 h = PH[q];
                                d.x += fa * h.x; d.y += fa * h.y; d.z += fa * h.z; d.w += fa * h.w;
                                D4[q] = d;
                            }
                            nit++;
                            break;
                        }
                    }
                    {
                        float ts = 0.0f, tt = 0.0f, rts = 0.0f, rtt = 0.0f;
                        auto row = [&](int i, bool valid, int sub) {
                            float y[3];
                            spin_row<float, SPIN_LPR>(valid, i, sub, a.ptr, a.col, a.A32, a.cc32, a.m32, a.dir,
                                                      a.fshat, y);
                            if (!valid || sub != 0) return;
#pragma unroll
                            for (int c = 0; c < 3; c++) {
                                const float sv = a.fs[3 * i + c], rt = a.frt[3 * i + c];
                                a.ft[3 * i + c] = y[c];
                                ts += y[c] * sv;
                                tt += y[c] * y[c];
                                rts += rt * sv;
                                rtt += rt * y[c];
                            }
                        };
                        SPIN_ROWS(row)
                        float v4[4] = {ts, tt, rts, rtt};
                        block_store_f<4>(v4, a.partial, G);
                    }
                    if (!grid_sync(a.bar)) goto timeout;
                    {
                        double s4[4];
                        grid_sum<4>(a.partial, G, s4);
                        omega = block_once([=] { return s4[0] / s4[1]; });
                        rr = fmax(0.0, ssum - 2.0 * omega * s4[0] + omega * omega * s4[1]);
                        rtr = s4[2] - omega * s4[3];
                    }
                    rho2 = rho1;
                    nit++;
                    pending = true;
                }
            }
            // the last pass's updates of d (float4 elements) are read below per element by other
            // threads
            if (!grid_sync(a.bar)) goto timeout;
            // x += scale |r| d (FP64); the next residual gathers x across the grid
            {
                const double f = a.scale * res;
                for (int k = i0; k < 3 * nn; k += stride) a.x[k] += f * (double)a.fd[k];
            }
            nref++;
            if (!grid_sync(a.bar)) goto timeout;
        }
        const bool ok = (status == 0);
        for (int k = i0; k < 3 * nn; k += stride) a.out[k] = ok ? a.x[k] + a.xd[k] : 0.0;
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            a.res->status = status;
            a.res->nit = nit;
            a.res->fail = ok ? 0 : 1;
            a.res->res = res;
            a.res->rhsn = rhsn;
            a.res->res0 = res0;
        }
        return;
    }
timeout:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.res->timeout = 1;
        a.res->fail = 1;
    }
}

// CSR with diagonal over the node graph of the given tets.
void node_graph(int nn, const std::vector<int> &tets, const int32_t *tet4, std::vector<int> &ptr,
                std::vector<int> &col) {
    std::vector<std::vector<int>> nb(nn);
    for (int t : tets)
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) nb[tet4[4 * t + i]].push_back(tet4[4 * t + j]);
    ptr.assign(nn + 1, 0);
    for (int i = 0; i < nn; i++) {
        auto &v = nb[i];
        v.push_back(i);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        ptr[i + 1] = ptr[i] + (int)v.size();
    }
    col.resize(ptr[nn]);
    for (int i = 0; i < nn; i++) std::copy(nb[i].begin(), nb[i].end(), col.begin() + ptr[i]);
}

inline int find_col(const std::vector<int> &ptr, const std::vector<int> &col, int i, int j) {
    auto b = col.begin() + ptr[i], e = col.begin() + ptr[i + 1];
    return (int)(std::lower_bound(b, e, j) - col.begin());
}

// algebra::cg_dir (src/algebra/cg.h:67-121) on the host: the potential is solved once.
int cg_dir(const std::vector<int> &ptr, const std::vector<int> &col, const std::vector<double> &val,
           std::vector<double> &x, const std::vector<double> &rhs, const std::vector<double> &xd,
           const std::vector<unsigned char> &dir, double tol, int maxiter, int *nit_out) {
    const int n = (int)x.size();
    auto mult = [&](const std::vector<double> &in, std::vector<double> &out) {
        for (int i = 0; i < n; i++) {
            double s = 0;
            for (int k = ptr[i]; k < ptr[i + 1]; k++) s += val[k] * in[col[k]];
            out[i] = s;
        }
    };
    auto dot = [&](const std::vector<double> &a, const std::vector<double> &b) {
        double s = 0;
        for (int i = 0; i < n; i++) s += a[i] * b[i];
        return s;
    };
    std::vector<double> p(n), q(n), r(n), z(n), diag(n), b(rhs), tmp(n);
    for (int i = 0; i < n; i++) diag[i] = 1.0 / val[find_col(ptr, col, i, i)];
    mult(xd, z);
    for (int i = 0; i < n; i++) b[i] -= z[i];
    for (int i = 0; i < n; i++)
        if (dir[i]) b[i] = diag[i] = 0.0;
    const double rhsn = std::sqrt(dot(b, b));
    r = b;
    mult(x, tmp);
    for (int i = 0; i < n; i++) r[i] -= tmp[i];
    for (int i = 0; i < n; i++)
        if (dir[i]) r[i] = 0.0;
    for (int i = 0; i < n; i++) z[i] = diag[i] * r[i];
    double rho = dot(z, r), rho_1 = 0.0;
    p = z;
    int nit = 0, status = -1;
    auto finished = [&](double nr) {
        const double res = std::fabs(nr);
        if (std::isnan(res)) { status = 2; return false; }
        const bool cv = res <= rhsn * tol;
        if (cv) status = 0;
        return cv;
    };
    while (!finished(std::sqrt(dot(r, r))) && status != 1 && status != 2) {
        if (nit > 0) {
            for (int i = 0; i < n; i++) z[i] = diag[i] * r[i];
            rho = dot(z, r);
            for (int i = 0; i < n; i++) p[i] = z[i] + (rho / rho_1) * p[i];
        }
        mult(p, q);
        for (int i = 0; i < n; i++)
            if (dir[i]) q[i] = 0.0;
        const double qp = dot(q, p);
        if (qp == 0.0) { status = 2; break; }
        const double a = rho / qp;
        for (int i = 0; i < n; i++) x[i] += a * p[i];
        for (int i = 0; i < n; i++) r[i] += (-a) * q[i];
        rho_1 = rho;
        nit++;
        if (nit >= maxiter) status = 1;
    }
    for (int i = 0; i < n; i++) x[i] += xd[i];
    *nit_out = nit;
    return status;
}

struct SpinState {
    int nn = 0, grid = 0, threads = 256;  // persistent blocks and their threads
    int *ptr = nullptr, *col = nullptr;
    double *A = nullptr, *dinv = nullptr, *cc = nullptr, *G = nullptr, *L = nullptr, *xd = nullptr;
    unsigned char *dir = nullptr;
    double *work = nullptr;  // x, r, rt, p, phat, v, s, shat, t: 9 x 3nn
    double *out = nullptr;   // s (3nn)
    double *partial = nullptr;
    GridBar *bar = nullptr;
    SolveResult *res = nullptr, *hres = nullptr;
    // FG_PREC_FP32_REFINE: scaled FP32 operator, FP32 Krylov vectors and CURRENT m
    // (10 x 3nn floats), FP64 b and refinement residual (2 x 3nn)
    bool mixed = false;
    double scale = 1.0;
    float *A32 = nullptr, *cc32 = nullptr, *dinv3 = nullptr, *work32 = nullptr;
    size_t n3p = 0;  // 3nn rounded up to whole float4 chunks
    double *b64 = nullptr;
    std::vector<double> V;   // electrostatic potential (host, node order of the mesh)
    int v_iters = 0, v_status = 0;
};

}  // namespace

int spin_setup(Ctx &c, const fg_mesh *m, const fg_region *regs, int nreg, const fg_tri_region *tregs, int ntreg,
               std::vector<DevRegion> &hreg) {
    const Rules R = make_rules(c.opts.one_gauss_point != 0);
    const int nn = m->n_nodes;
    // boundary conditions (electrostatSolver::checkBoundaryConditions, spinAcc::checkBoundaryConditions)
    int nJ = 0, nV = 0, nS = 0;
    std::vector<char> treg_used(ntreg, 0), reg_used(nreg, 0);
    for (int f = 0; f < m->n_tris; f++) treg_used[m->tri_region[f]] = 1;
    for (int t = 0; t < m->n_tets; t++) reg_used[m->tet_region[t]] = 1;
    for (int r = 0; r < ntreg; r++) {
        if (!treg_used[r]) continue;
        const fg_tri_region &g = tregs[r];
        if (std::isfinite(g.jn)) nJ++;
        if (std::isfinite(g.V)) nV++;
        if (std::isfinite(g.s[0]) && std::isfinite(g.s[1]) && std::isfinite(g.s[2])) nS++;
    }
    if (nJ != 1 || nV != 1) {
        c.err = "fg_create: incorrect boundary conditions for the potential V solver (one surface region with jn, "
                "one with V)";
        return FG_EINVAL;
    }
    if (nS != 1) {
        c.err = "fg_create: incorrect boundary conditions for the spin diffusion solver (one surface region with s)";
        return FG_EINVAL;
    }
    for (int r = 0; r < nreg; r++) {
        if (!reg_used[r]) continue;
        const fg_region &g = regs[r];
        if (!(std::isfinite(g.dens_state) && g.dens_state != 0.0) || !(g.P >= 0.0 && g.P < 1.0)) {
            c.err = "fg_create: incorrect parameters for the spin diffusion solver (every region needs dens_state "
                    "!= 0 and 0 <= P < 1)";
            return FG_EINVAL;
        }
    }
    // geometry of all tets (Tet constructor, src/tetra.h:140-163): da and the Gauss weights
    const int nt = m->n_tets;
    std::vector<double> da(12 * (size_t)nt), w((size_t)nt * R.npi_t);
    for (int t = 0; t < nt; t++) {
        const int *ind = &m->tet4[4 * t];
        double P[4][3];
        for (int i = 0; i < 4; i++)
            for (int d = 0; d < 3; d++) P[i][d] = m->xyz[3 * ind[i] + d];
        double J[3][3];
        for (int d = 0; d < 3; d++)
            for (int e = 0; e < 3; e++) J[d][e] = P[e + 1][d] - P[0][d];
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        double inv[3][3];
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        const double dadu[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int i = 0; i < 4; i++)
            for (int q = 0; q < 3; q++) {
                double s = 0;
                for (int mm = 0; mm < 3; mm++) s += dadu[i][mm] * inv[mm][q];
                da[12 * (size_t)t + 3 * i + q] = s;
            }
        for (int g = 0; g < R.npi_t; g++) w[(size_t)t * R.npi_t + g] = det * R.tp[g];
    }
    auto dd = [&](int t, int i, int j) {
        const double *a = &da[12 * (size_t)t];
        return a[3 * i] * a[3 * j] + a[3 * i + 1] * a[3 * j + 1] + a[3 * i + 2] * a[3 * j + 2];
    };
    std::vector<int> all(nt);
    for (int t = 0; t < nt; t++) all[t] = t;
    std::vector<int> ptr, col;
    node_graph(nn, all, m->tet4, ptr, col);
    const size_t nnz = col.size();
    // triangle weights 2 surf pds (Tri constructor)
    auto tri_w = [&](int f, int g) {
        const int *ind = &m->tri3[3 * f];
        double a[3], b[3];
        for (int d = 0; d < 3; d++) {
            a[d] = m->xyz[3 * ind[1] + d] - m->xyz[3 * ind[0] + d];
            b[d] = m->xyz[3 * ind[2] + d] - m->xyz[3 * ind[0] + d];
        }
        const double cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
        const double surf = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
        return 2.0 * surf * R.fp[g];
    };
    // electrostatic problem (electrostatSolver::solve): K_V, L_V, Dirichlet V
    std::vector<double> KV(nnz, 0.0), LV(nn, 0.0), Vd(nn, 0.0);
    std::vector<unsigned char> vdir(nn, 0);
    for (int t = 0; t < nt; t++) {
        const double sigma = regs[m->tet_region[t]].sigma;
        const int *ind = &m->tet4[4 * t];
        double AE[4][4] = {};
        for (int g = 0; g < R.npi_t; g++) {
            const double sw = sigma * w[(size_t)t * R.npi_t + g];
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) AE[i][j] += sw * dd(t, i, j);
        }
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) KV[find_col(ptr, col, ind[i], ind[j])] += AE[i][j];
    }
    for (int f = 0; f < m->n_tris; f++) {
        const fg_tri_region &g = tregs[m->tri_region[f]];
        const double J = std::isfinite(g.jn) ? g.jn : 0.0;
        const int *ind = &m->tri3[3 * f];
        double BE[3] = {0, 0, 0};
        for (int q = 0; q < R.npi_f; q++) {
            const double Jw = J * tri_w(f, q);
            for (int i = 0; i < 3; i++) BE[i] -= R.fa[i][q] * Jw;
        }
        for (int i = 0; i < 3; i++) LV[ind[i]] += BE[i];
    }
    for (int f = 0; f < m->n_tris; f++) {
        const fg_tri_region &g = tregs[m->tri_region[f]];
        if (std::isnan(g.V)) continue;
        for (int i = 0; i < 3; i++) {
            Vd[m->tri3[3 * f + i]] = g.V;
            vdir[m->tri3[3 * f + i]] = 1;
        }
    }
    SpinState *S = new SpinState();
    c.spin = S;
    S->nn = nn;
    S->V.assign(nn, 0.0);
    S->v_status = cg_dir(ptr, col, KV, S->V, LV, Vd, vdir, c.opts.spin_tol, c.opts.spin_max_iter, &S->v_iters);
    if (S->v_status != 0) {
        c.err = "fg_create: the electrostatic potential solve did not converge";
        return FG_SOLVER_CANNOT_CONVERGE;
    }
    // spin diffusion operator (spinAcc::integrales), coupling weights and RHS coefficients
    std::vector<double> A(nnz, 0.0), cc(nn, 0.0), Gc(nn, 0.0), L(3 * (size_t)nn, 0.0), xd(3 * (size_t)nn, 0.0);
    std::vector<unsigned char> sdir(nn, 0);
    for (int t = 0; t < nt; t++) {
        const fg_region &p = regs[m->tet_region[t]];
        const int *ind = &m->tet4[4 * t];
        const double D0 = 2.0 * p.sigma / (CHARGE_ELECTRON * CHARGE_ELECTRON * p.dens_state);
        double aw[4] = {0, 0, 0, 0}, wsum = 0.0;
        for (int g = 0; g < R.npi_t; g++) {
            const double wg = w[(size_t)t * R.npi_t + g];
            wsum += wg;
            for (int i = 0; i < 4; i++) aw[i] += R.ta[i][g] * wg;
        }
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double v = dd(t, i, j) * (D0 * wsum);
                if (i == j) v += (D0 / (p.lsf * p.lsf)) * aw[i];
                A[find_col(ptr, col, ind[i], ind[j])] += v;
            }
        if (p.Ms > 0) {
            const double invTau_sd = D0 / (p.lsd * p.lsd);
            for (int i = 0; i < 4; i++) cc[ind[i]] += invTau_sd * aw[i];
            const double cst0 = BOHRS_MUB * p.P * p.sigma / CHARGE_ELECTRON;
            double gV[3] = {0, 0, 0};
            for (int i = 0; i < 4; i++)
                for (int d = 0; d < 3; d++) gV[d] += S->V[ind[i]] * da[12 * (size_t)t + 3 * i + d];
            for (int g = 0; g < R.npi_t; g++) {
                const double cw = cst0 * w[(size_t)t * R.npi_t + g];
                for (int i = 0; i < 4; i++) {
                    const double *a = &da[12 * (size_t)t + 3 * i];
                    Gc[ind[i]] += cw * gV[0] * a[0] + cw * gV[1] * a[1] + cw * gV[2] * a[2];
                }
            }
        }
    }
    auto s_value_of = [&](const fg_tri_region &g, double sv[3]) {
        for (int d = 0; d < 3; d++) sv[d] = g.s[d];
        if (std::isfinite(g.jn) && std::isfinite(g.uP[0]) && std::isfinite(g.uP[1]) && std::isfinite(g.uP[2]))
            for (int d = 0; d < 3; d++) sv[d] = -g.jn * (BOHRS_MUB / CHARGE_ELECTRON) * g.uP[d];
    };
    for (int f = 0; f < m->n_tris; f++) {
        const fg_tri_region &g = tregs[m->tri_region[f]];
        double sv[3];
        s_value_of(g, sv);
        if (!(std::isfinite(sv[0]) && std::isfinite(sv[1]) && std::isfinite(sv[2]))) continue;
        const int *ind = &m->tri3[3 * f];
        for (int q = 0; q < R.npi_f; q++) {
            const double wq = tri_w(f, q);
            for (int i = 0; i < 3; i++) {
                const double aiw = wq * R.fa[i][q];
                for (int d = 0; d < 3; d++) L[3 * (size_t)ind[i] + d] -= sv[d] * aiw;
            }
        }
    }
    // Dirichlet values (spinAcc::boundaryConditions), later triangles overwrite earlier ones
    for (int f = 0; f < m->n_tris; f++) {
        const fg_tri_region &g = tregs[m->tri_region[f]];
        const bool s_set = std::isfinite(g.s[0]) && std::isfinite(g.s[1]) && std::isfinite(g.s[2]);
        double sv[3];
        if (!s_set && std::isfinite(g.jn)) {
            for (int d = 0; d < 3; d++) sv[d] = -g.jn * (BOHRS_MUB / CHARGE_ELECTRON) * g.uP[d];
        } else if (s_set && std::isnan(g.jn)) {
            for (int d = 0; d < 3; d++) sv[d] = g.s[d];
        } else {
            continue;
        }
        for (int i = 0; i < 3; i++) {
            const int k = m->tri3[3 * f + i];
            sdir[k] = 1;
            for (int d = 0; d < 3; d++) xd[3 * (size_t)k + d] = sv[d];
        }
    }
    std::vector<double> dinv(nn);
    for (int i = 0; i < nn; i++) dinv[i] = sdir[i] ? 0.0 : 1.0 / A[find_col(ptr, col, i, i)];
    // Hst prefactor per magnetic region (spinAcc::prepareExtraField)
    for (int r = 0; r < nreg; r++) {
        const fg_region &p = regs[r];
        if (p.Ms > 0 && p.lsd != 0.0 && p.dens_state != 0.0) {
            const double D0 = 2.0 * p.sigma / (CHARGE_ELECTRON * CHARGE_ELECTRON * p.dens_state);
            hreg[r].hst = D0 / (p.lsd * p.lsd * FG_GAMMA0 * p.Ms);
            const float hh = (float)hreg[r].hst;
            hreg[r].hst_ds = make_float2(hh, (float)(hreg[r].hst - (double)hh));
        }
    }
    // device
    auto up = [](auto **d, const auto &h) {
        using T = typename std::remove_reference<decltype(h)>::type::value_type;
        cudaError_t e = cudaMalloc((void **)d, std::max<size_t>(1, h.size()) * sizeof(T));
        if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    };
    const size_t n3 = 3 * (size_t)nn;
    if (up(&S->ptr, ptr) || up(&S->col, col) || up(&S->A, A) || up(&S->dinv, dinv) || up(&S->cc, cc) ||
        up(&S->G, Gc) || up(&S->L, L) || up(&S->xd, xd) || up(&S->dir, sdir) ||
        cudaMalloc(&S->work, 9 * n3 * sizeof(double)) || cudaMalloc(&S->out, n3 * sizeof(double)) ||
        cudaMemset(S->out, 0, n3 * sizeof(double)) || cudaMalloc(&S->bar, sizeof(GridBar)) ||
        cudaMemset(S->bar, 0, sizeof(GridBar)) || cudaMalloc(&S->res, sizeof(SolveResult)) ||
        cudaMallocHost(&S->hres, sizeof(SolveResult))) {
        c.err = "fg_create: device allocation for the spin accumulation failed";
        return FG_ECUDA;
    }
    if (c.opts.precision == FG_PREC_FP32_REFINE) {
        // scale = 1 / mean diagonal of the free rows keeps the FP32 operator O(1)
        double dsum = 0.0;
        int nfree = 0;
        for (int i = 0; i < nn; i++)
            if (!sdir[i]) {
                dsum += A[find_col(ptr, col, i, i)];
                nfree++;
            }
        S->mixed = true;
        S->scale = (nfree > 0 && dsum > 0.0) ? nfree / dsum : 1.0;
        S->n3p = (n3 + 3) / 4 * 4;
        std::vector<float> A32(nnz), cc32(nn), dinv3(S->n3p, 0.0f);
        for (size_t k = 0; k < nnz; k++) A32[k] = (float)(S->scale * A[k]);
        for (int i = 0; i < nn; i++) {
            cc32[i] = (float)(S->scale * cc[i]);
            for (int d = 0; d < 3; d++) dinv3[3 * (size_t)i + d] = sdir[i] ? 0.0f : (float)(dinv[i] / S->scale);
        }
        // the Krylov vectors start (and their padding stays) zero
        if (up(&S->A32, A32) || up(&S->cc32, cc32) || up(&S->dinv3, dinv3) ||
            cudaMalloc(&S->work32, 10 * S->n3p * sizeof(float)) ||
            cudaMemset(S->work32, 0, 10 * S->n3p * sizeof(float)) || cudaMalloc(&S->b64, 2 * n3 * sizeof(double))) {
            c.err = "fg_create: device allocation for the spin accumulation failed";
            return FG_ECUDA;
        }
    }
    // block size: 256 threads for the FP64 kernel; the FP32 body one block of 1024 per SM, the
    // warps of four 256-thread blocks with a quarter of the blocks at each grid barrier
    // (measured on the 1.2M-tet film: 68 against 72 us per iteration); FG_SPIN_THREADS=256
    // selects four blocks of 256
    if (S->mixed) S->threads = 1024;
    if (const char *env = std::getenv("FG_SPIN_THREADS"))
        if (std::atoi(env) == 256) S->threads = 256;
    int per_sm = 0, per_sm_mixed = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spin_bicg, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_mixed, k_spin_mixed, S->threads, 0);
    if (S->mixed) per_sm = per_sm_mixed;
    if (per_sm < 1 && S->threads != 256) {  // a 1024-thread block does not fit: back to 256
        S->threads = 256;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spin_mixed, 256, 0);
    }
    // blocks per SM: the FP64 kernel runs best with two (fewer blocks make each grid barrier
    // cheaper), the FP32 body with four (its latency-bound sweeps want the warps; measured
    // 77 against 93 us per iteration on the 1.2M-tet film); FG_SPIN_BLOCKS_PER_SM overrides
    // it (up to the kernel's occupancy)
    int bps = S->mixed ? 4 : 2;
    if (const char *env = std::getenv("FG_SPIN_BLOCKS_PER_SM")) bps = std::max(1, std::atoi(env));
    S->grid = std::max(1, std::min(std::min(std::max(1, per_sm), bps) * c.nsm, (nn + S->threads - 1) / S->threads));
    if (cudaMalloc(&S->partial, 4 * sizeof(double) * std::max(1024, S->grid)) != cudaSuccess) return FG_ECUDA;
    c.spin_s = S->out;
    return FG_OK;
}

void spin_free(Ctx &c) {
    SpinState *S = static_cast<SpinState *>(c.spin);
    if (!S) return;
    void *p[] = {S->ptr, S->col, S->A, S->dinv, S->cc, S->G, S->L, S->xd, S->dir, S->work, S->out, S->partial,
                 S->bar, S->res, S->A32, S->cc32, S->dinv3, S->work32, S->b64};
    for (void *q : p)
        if (q) cudaFree(q);
    if (S->hres) cudaFreeHost(S->hres);
    delete S;
    c.spin = nullptr;
    c.spin_s = nullptr;
}

// spinAcc::compute: solve for s with m = CURRENT (operator) and NEXT (RHS); on failure s = 0.
cudaError_t launch_spin(Ctx &c) {
    SpinState *S = static_cast<SpinState *>(c.spin);
    if (!S) return cudaSuccess;
    const size_t n3 = 3 * (size_t)S->nn;
    SpinArgs a;
    a.nn = S->nn;
    a.ptr = S->ptr; a.col = S->col; a.A = S->A; a.dinv = S->dinv; a.cc = S->cc; a.G = S->G; a.L = S->L;
    a.xd = S->xd; a.dir = S->dir;
    a.m0 = c.u[0]; a.m1 = c.u[1];
    a.x = S->work; a.r = a.x + n3; a.rt = a.r + n3; a.p = a.rt + n3; a.phat = a.p + n3; a.v = a.phat + n3;
    a.s = a.v + n3; a.shat = a.s + n3; a.t = a.shat + n3;
    a.out = S->out;
    a.partial = S->partial; a.bar = S->bar; a.res = S->res;
    a.tol = c.opts.spin_tol; a.maxiter = c.opts.spin_max_iter;
    a.A32 = S->A32; a.cc32 = S->cc32; a.dinv3 = S->dinv3; a.n4 = (int)(S->n3p / 4);
    a.m32 = a.fr = a.frt = a.fp = a.fphat = a.fv = a.fs = a.fshat = a.ft = a.fd = nullptr;
    a.b64 = a.r64 = nullptr;
    if (S->mixed) {
        float *w = S->work32;
        const size_t q = S->n3p;
        a.fr = w; a.frt = w + q; a.fp = w + 2 * q; a.fphat = w + 3 * q; a.fv = w + 4 * q; a.fs = w + 5 * q;
        a.fshat = w + 6 * q; a.ft = w + 7 * q; a.fd = w + 8 * q; a.m32 = w + 9 * q;
        a.b64 = S->b64; a.r64 = S->b64 + n3;
    }
    a.scale = S->scale; a.inner_tol = c.opts.inner_tol; a.refine_max = c.opts.refine_max;
    cudaError_t e = cudaMemsetAsync(S->res, 0, sizeof(SolveResult), c.stream);
    if (e != cudaSuccess) return e;
    void *args[] = {&a};
    return cudaLaunchCooperativeKernel(S->mixed ? (void *)k_spin_mixed : (void *)k_spin_bicg, dim3(S->grid),
                                       dim3(S->mixed ? S->threads : 256), args, 0, c.stream);
}

int spin_info(const Ctx &c, int *status, int *iters, double *V, int *v_iters) {
    const SpinState *S = static_cast<const SpinState *>(c.spin);
    if (!S) return FG_EINVAL;
    if (status || iters) {
        cudaMemcpy(S->hres, S->res, sizeof(SolveResult), cudaMemcpyDeviceToHost);
        if (status) *status = S->hres->timeout ? FG_ETIMEDOUT : S->hres->status;
        if (iters) *iters = S->hres->nit;
    }
    if (V) std::memcpy(V, S->V.data(), S->V.size() * sizeof(double));
    if (v_iters) *v_iters = S->v_iters;
    return FG_OK;
}

}  // namespace fg
