// FP32 Krylov body with FP64 iterative refinement for the per-step system (the
// FG_PREC_FP32_REFINE path). Same operator, preconditioner and mask as the plain path
// (bicg_dir, src/algebra/bicg.h:163-234); what changes is the arithmetic:
//   outer loop (FP64):  r = b - K x with the FP64 operator; stop when |r| <= tol |b|,
//                       the reference's own test (src/algebra/iter.h:144-156) applied to
//                       the true residual;
//   inner loop (FP32):  BiCGSTAB on (scale K) d = r/|r| from d = 0 with FP32 vectors and
//                       operator; dot products summed in FP32 per warp and in FP64 across
//                       warps and blocks, the recurrence scalars (alpha, beta, omega) in
//                       FP64 once per block (GB300's FP64 pipe runs at 1/64 of the FP32
//                       rate); scale = 1/mean(A) keeps every FP32 quantity O(1) (raw
//                       entries are ~1e-27);
//   x += scale |r| d in FP64.
// One cooperative launch per solve; the node update (Node::make_evol) is fused at the end.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "fg_device.cuh"
#include "fg_internal.h"

namespace fg {

// Rows and blocks of this block's sample. One system: all nodes, all blocks.
struct SegView {
    int g, lo, hi, b0, b1;
};

__device__ __forceinline__ SegView seg_view(const MixedArgs &a) {
    SegView v{0, 0, a.nn, 0, (int)gridDim.x};
    if (a.nseg > 1) {
        int lo = 0, hi = a.nseg - 1;
        const int b = blockIdx.x;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.seg_blk[mid] <= b) lo = mid;
            else hi = mid - 1;
        }
        v.g = lo;
        v.lo = a.seg_node[lo];
        v.hi = a.seg_node[lo + 1];
        v.b0 = a.seg_blk[lo];
        v.b1 = a.seg_blk[lo + 1];
    }
    return v;
}

// Batched form (nseg > 1): every sample of a block-diagonal system runs the same
// iteration with its own scalars (rho, alpha, omega), its own |b| and its own stopping
// tests, exactly as if it were solved alone; a sample that has stopped idles through the
// remaining grid barriers. The loops end when no sample is active: an activity flag rides
// along the first reduction of each loop pass (slot 1, summed over the whole grid).
#define SAMPLE_ROWS(i) for (int i = sv.lo + (blockIdx.x - sv.b0) * (int)blockDim.x + (int)threadIdx.x; i < sv.hi; i += rstride)

// Rows of the operator applications: LPR lanes per row (LPR = 1: thread per row), the loop
// warp-uniform so that the group shuffles see every lane; body(i, valid, sub).
#define GROUP_ROWS(body)                                                                                \
    for (int gbase = sv.lo + ((blockIdx.x - sv.b0) * (int)blockDim.x + (int)(threadIdx.x & ~31)) / LPR; \
         gbase < sv.hi; gbase += gstride) {                                                             \
        const int i_ = gbase + (int)(threadIdx.x & 31) / LPR;                                           \
        body(i_, i_ < sv.hi, (int)threadIdx.x % LPR);                                                   \
    }

// Blocks of 256 threads (two per SM at 128 registers) or 512 (one per SM: twice the warps of
// a 256-thread block to hide the operator's gathers, with the same number of blocks meeting at
// each grid barrier); every block-level reduction works for either size.
template <int LPR>
__global__ void __launch_bounds__(512, 1) k_mixed(MixedArgs a) {
    const int G = gridDim.x;
    const SegView sv = seg_view(a);
    const int rstride = (sv.b1 - sv.b0) * blockDim.x;
    const int gstride = (sv.b1 - sv.b0) * (int)blockDim.x / LPR;
    const bool multi = a.nseg > 1;
    double c0 = a.c0, dt = a.dt;
    if (a.seg) {
        c0 = a.seg[sv.g].c0;
        dt = a.seg[sv.g].dt;
    }
    const float c32 = (float)(c0 * a.scale);
    // phase 0: FP32 copies of the per-step operator, FP64 tangent vectors of x, |b|^2, and
    // the learned guess's candidate when its network outputs are given
    {
        double bb = 0.0;
        if (a.cand_o) {
            SAMPLE_ROWS(i) {
                double xp = 0.0, xq = 0.0;
                if (a.mag[i]) {
                    // the correction's mean over the node and its magnetic neighbours (the row of
                    // S holds both): a low-pass filter on the network's per-node errors
                    float o0 = 0.f, o1 = 0.f, o2 = 0.f;
                    int cnt = 0;
                    for (int k = a.Sptr[i]; k < a.Sptr[i + 1]; k++) {
                        const int j = a.Scol[k];
                        if (!a.mag[j]) continue;
                        o0 += a.cand_o[3 * (size_t)j];
                        o1 += a.cand_o[3 * (size_t)j + 1];
                        o2 += a.cand_o[3 * (size_t)j + 2];
                        cnt++;
                    }
                    const double sc = a.cand_scale[0] / (double)max(cnt, 1);
                    const double oo[3] = {o0, o1, o2};
                    double v[3];
#pragma unroll
                    for (int c = 0; c < 3; c++)
                        v[c] = 2.0 * a.cand_vprev[3 * i + c] - a.cand_vprev2[3 * i + c] + sc * oo[c];
                    xp = (v[0] * a.ep[3 * i] + v[1] * a.ep[3 * i + 1] + v[2] * a.ep[3 * i + 2]) / FG_GAMMA0;
                    xq = (v[0] * a.eq[3 * i] + v[1] * a.eq[3 * i + 1] + v[2] * a.eq[3 * i + 2]) / FG_GAMMA0;
                }
                a.cand_x[2 * i] = xp;
                a.cand_x[2 * i + 1] = xq;
                tangent<double>(i, a.ep, a.eq, xp, xq, a.cand_W);
            }
        }
        SAMPLE_ROWS(i) {
            for (int c = 0; c < 3; c++) {
                a.ep32[3 * i + c] = (float)a.ep[3 * i + c];
                a.eq32[3 * i + c] = (float)a.eq[3 * i + c];
            }
            a.Dl32[i] = (float)(a.Dl[i] * a.scale);
            const bool m = a.mag[i];
            a.Minv32[2 * i] = m ? 1.0f / a.A32[i] : 0.0f;
            a.Minv32[2 * i + 1] = m ? -1.0f / a.A32[i] : 0.0f;
            tangent<double>(i, a.ep, a.eq, a.x[2 * i], a.x[2 * i + 1], a.W64);
            if (m) bb += a.b[2 * i] * a.b[2 * i] + a.b[2 * i + 1] * a.b[2 * i + 1];
        }
        double v1[1] = {bb};
        block_store<1>(v1, a.partial, G);
    }
    if (!grid_sync(a.bar)) goto timeout;
    {
        double s1[1];
        range_sum<1>(a.partial, G, sv.b0, sv.b1, s1);
        const double rhsn = sqrt(fabs(s1[0]));
        int status = -1, nit = 0, nref = 0;
        double res = 0.0, res0 = 0.0;
        bool done = false;  // this sample's solve has ended (status set)
        for (;;) {
            // refinement residual r64 = b - K x (FP64, masked); on the first pass with a
            // candidate guess, also the candidate's residual (the referee of the learned guess)
            const bool judge = nref == 0 && a.cand_x != nullptr;
            {
                double rr = 0.0, rc = 0.0, rx = 0.0;
                if (!done) {
                    auto row = [&](int i, bool valid, int sub) {
                        double y0 = 0, y1 = 0;
                        apply_row_g<double, LPR>(valid, i, sub, a.Sptr, a.Scol, a.Sval, a.W64, a.ep, a.eq, a.A, a.Dl,
                                                 c0, valid ? a.x[2 * i] : 0.0, valid ? a.x[2 * i + 1] : 0.0, y0, y1);
                        if (valid && sub == 0) {
                            const bool m = a.mag[i];
                            const double r0 = m ? a.b[2 * i] - y0 : 0.0, r1 = m ? a.b[2 * i + 1] - y1 : 0.0;
                            a.r64[2 * i] = r0;
                            a.r64[2 * i + 1] = r1;
                            rr += r0 * r0 + r1 * r1;
                        }
                        if (judge) {
                            double z0 = 0, z1 = 0;
                            apply_row_g<double, LPR>(valid, i, sub, a.Sptr, a.Scol, a.Sval, a.cand_W, a.ep, a.eq, a.A,
                                                     a.Dl, c0, valid ? a.cand_x[2 * i] : 0.0,
                                                     valid ? a.cand_x[2 * i + 1] : 0.0, z0, z1);
                            if (valid && sub == 0) {
                                const bool m = a.mag[i];
                                const double r0 = m ? a.b[2 * i] - z0 : 0.0, r1 = m ? a.b[2 * i + 1] - z1 : 0.0;
                                a.cand_r[2 * i] = r0;
                                a.cand_r[2 * i + 1] = r1;
                                rc += r0 * r0 + r1 * r1;
                                rx += r0 * a.r64[2 * i] + r1 * a.r64[2 * i + 1];
                            }
                        }
                    };
                    GROUP_ROWS(row)
                }
                double v3[3] = {rr, rc, rx};
                block_store<3>(v3, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s3[3];
                range_sum<3>(a.partial, G, sv.b0, sv.b1, s3);
                double s2 = s3[0];
                if (judge && !done) {
                    // x = x_prev + t (x_cand - x_prev) with the t in [0, 1] that minimises the
                    // FP64 residual norm |r_prev + t (r_cand - r_prev)| (the residual is affine in
                    // t: no further operator application); t > 0 counts as the guess accepted
                    const double dd = s3[0] + s3[1] - 2.0 * s3[2];
                    const double t = dd > 0.0 ? fmin(1.0, fmax(0.0, (s3[0] - s3[2]) / dd)) : 0.0;
                    if (blockIdx.x == sv.b0 && threadIdx.x == 0) {  // per sample in a batch
                        a.cand_flag[sv.g] = t > 0.0 ? 1 : 0;
                        a.cand_res2[2 * sv.g] = s3[1];
                        a.cand_res2[2 * sv.g + 1] = s3[0];
                    }
                    if (t > 0.0) {
                        SAMPLE_ROWS(i) {
#pragma unroll
                            for (int c = 0; c < 2; c++) {
                                const int k = 2 * i + c;
                                a.x[k] += t * (a.cand_x[k] - a.x[k]);
                                a.r64[k] += t * (a.cand_r[k] - a.r64[k]);
                            }
#pragma unroll
                            for (int c = 0; c < 3; c++) a.W64[3 * i + c] += t * (a.cand_W[3 * i + c] - a.W64[3 * i + c]);
                        }
                        s2 = s3[0] + 2.0 * t * (s3[2] - s3[0]) + t * t * dd;
                    }
                }
                if (!done) res = block_once([=] { return sqrt(fabs(s2)); });
            }
            if (!done) {
                if (nref == 0) res0 = res;
                if (isnan(res)) { status = 2; done = true; }
                else if (res <= rhsn * a.tol) { status = 0; done = true; }
                else if (nref >= a.refine_max || nit >= a.maxiter) { status = 1; done = true; }
            }
            if (!multi && done) break;
            // inner FP32 BiCGSTAB on (scale K) d = r64/res to the relative target the outer
            // test needs, with a margin of 0.7 for the FP32 recursion's drift from the true
            // residual (about 1e-7 of the inner system's unit residual, far below any target
            // above the floor inner_tol, 1e-5 by default)
            const double rho = res;
            const double target =
                done ? 0.0 : block_once([=] { return fmax(a.inner_tol, 0.7 * a.tol * rhsn / res); });
            const double target2 = target * target;
            {
                float rr = 0.0f;
                if (!done) {
                    const float inv = (float)block_once([=] { return 1.0 / rho; });
                    SAMPLE_ROWS(i) {
                        for (int c = 0; c < 2; c++) {
                            const int k = 2 * i + c;
                            const float rv = (float)a.r64[k] * inv;
                            a.r[k] = rv;
                            a.rt[k] = rv;
                            a.p[k] = rv;
                            a.d[k] = 0.0f;
                            rr += rv * rv;
                        }
                    }
                }
                float v2[2] = {rr, (threadIdx.x == 0 && !done) ? 1.0f : 0.0f};
                block_store_f<2>(v2, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s2[1];
                range_sum<1>(a.partial, G, sv.b0, sv.b1, s2);
                if (multi) {
                    double f[1];
                    grid_sum<1>(a.partial + G, G, f);
                    if (f[0] == 0.0) break;  // every sample has ended
                }
                double rr = s2[0], rtr = s2[0];
                double rho1 = 0.0, rho2 = 0.0, alpha = 0.0, beta = 0.0, omega = 0.0;
                int it = 0;
                bool act = !done;
                // Four grid barriers per iteration: the update x += alpha phat + omega shat,
                // r = s - omega t of a full iteration is carried into the first phase of the
                // next pass (pending), and its |r|^2 and (rt . r) come from the recurrence
                // |s - omega t|^2 = |s|^2 - 2 omega (t . s) + omega^2 |t|^2,
                // rt . (s - omega t) = rt . s - omega (rt . t) on the partial sums of the t phase.
                bool pending = false;
                for (;;) {
                    bool cont = act && rr > target2 && nit < a.maxiter;
                    if (cont) {
                        rho1 = rtr;
                        if (it > 0) {
                            if (rho2 == 0.0 || omega == 0.0) cont = false;
                            else beta = block_once([=] { return (rho1 / rho2) * (alpha / omega); });
                        }
                    }
                    if (pending || cont) {
                        const float fa = (float)alpha, fo = (float)omega, fb = (float)beta;
                        const bool upd = pending, go = cont, later = it > 0;
                        SAMPLE_ROWS(i) {
                            float rv[2];
#pragma unroll
                            for (int c = 0; c < 2; c++) {
                                const int k = 2 * i + c;
                                if (upd) {
                                    a.d[k] += fa * a.phat[k] + fo * a.shat[k];
                                    if (go) {
                                        rv[c] = a.s[k] - fo * a.t[k];
                                        a.r[k] = rv[c];
                                    }
                                } else if (go) {
                                    rv[c] = a.r[k];
                                }
                            }
                            if (go) {
                                float p0 = a.p[2 * i], p1 = a.p[2 * i + 1];
                                if (later) {
                                    p0 = rv[0] + fb * (p0 - fo * a.v[2 * i]);
                                    p1 = rv[1] + fb * (p1 - fo * a.v[2 * i + 1]);
                                    a.p[2 * i] = p0;
                                    a.p[2 * i + 1] = p1;
                                }
                                const float h0 = a.Minv32[2 * i] * p0, h1 = a.Minv32[2 * i + 1] * p1;
                                a.phat[2 * i] = h0;
                                a.phat[2 * i + 1] = h1;
                                tangent<float>(i, a.ep32, a.eq32, h0, h1, a.W32);
                            }
                        }
                    }
                    pending = false;
                    act = cont;
                    if (!multi && !act) break;
                    if (!grid_sync(a.bar)) goto timeout;
                    {
                        float vr = 0.0f;
                        if (act) {
                            auto row = [&](int i, bool valid, int sub) {
                                float y0 = 0, y1 = 0;
                                apply_row_g<float, LPR>(valid, i, sub, a.Sptr, a.Scol, a.Sval32, a.W32, a.ep32, a.eq32,
                                                        a.A32, a.Dl32, c32, valid ? a.phat[2 * i] : 0.f,
                                                        valid ? a.phat[2 * i + 1] : 0.f, y0, y1);
                                if (valid && sub == 0) {
                                    if (!a.mag[i]) y0 = y1 = 0.0f;
                                    a.v[2 * i] = y0;
                                    a.v[2 * i + 1] = y1;
                                    vr += y0 * a.rt[2 * i] + y1 * a.rt[2 * i + 1];
                                }
                            };
                            GROUP_ROWS(row)
                        }
                        float v2[2] = {vr, (threadIdx.x == 0 && act) ? 1.0f : 0.0f};
                        block_store_f<2>(v2, a.partial, G);
                    }
                    if (!grid_sync(a.bar)) goto timeout;
                    {
                        double s1b[1];
                        range_sum<1>(a.partial, G, sv.b0, sv.b1, s1b);
                        if (multi) {
                            double f[1];
                            grid_sum<1>(a.partial + G, G, f);
                            if (f[0] == 0.0) break;
                        }
                        if (act) alpha = block_once([=] { return rho1 / s1b[0]; });
                    }
                    {
                        float ss = 0.0f;
                        if (act) {
                            const float fa = (float)alpha;
                            SAMPLE_ROWS(i) {
                                const float s0 = a.r[2 * i] - fa * a.v[2 * i], s1 = a.r[2 * i + 1] - fa * a.v[2 * i + 1];
                                a.s[2 * i] = s0;
                                a.s[2 * i + 1] = s1;
                                const float h0 = a.Minv32[2 * i] * s0, h1 = a.Minv32[2 * i + 1] * s1;
                                a.shat[2 * i] = h0;
                                a.shat[2 * i + 1] = h1;
                                tangent<float>(i, a.ep32, a.eq32, h0, h1, a.W32);
                                ss += s0 * s0 + s1 * s1;
                            }
                        }
                        float v1[1] = {ss};
                        block_store_f<1>(v1, a.partial, G);
                    }
                    if (!grid_sync(a.bar)) goto timeout;
                    double ssum = 0.0;
                    {
                        double s1c[1];
                        range_sum<1>(a.partial, G, sv.b0, sv.b1, s1c);
                        ssum = s1c[0];
                        if (act && ssum <= target2) {
                            const float fa = (float)alpha;
                            SAMPLE_ROWS(i) {
                                a.d[2 * i] += fa * a.phat[2 * i];
                                a.d[2 * i + 1] += fa * a.phat[2 * i + 1];
                            }
                            // a solve that ends at the half step counts no iteration, as
                            // in the plain path and the reference's iteration counter
                            act = false;
                        }
                    }
                    if (!multi && !act) break;
                    {
                        float ts = 0.0f, tt = 0.0f, rts = 0.0f, rtt = 0.0f;
                        if (act) {
                            auto row = [&](int i, bool valid, int sub) {
                                float y0 = 0, y1 = 0;
                                apply_row_g<float, LPR>(valid, i, sub, a.Sptr, a.Scol, a.Sval32, a.W32, a.ep32, a.eq32,
                                                        a.A32, a.Dl32, c32, valid ? a.shat[2 * i] : 0.f,
                                                        valid ? a.shat[2 * i + 1] : 0.f, y0, y1);
                                if (valid && sub == 0) {
                                    if (!a.mag[i]) y0 = y1 = 0.0f;
                                    a.t[2 * i] = y0;
                                    a.t[2 * i + 1] = y1;
                                    const float s0 = a.s[2 * i], s1 = a.s[2 * i + 1];
                                    const float q0 = a.rt[2 * i], q1 = a.rt[2 * i + 1];
                                    ts += y0 * s0 + y1 * s1;
                                    tt += y0 * y0 + y1 * y1;
                                    rts += q0 * s0 + q1 * s1;
                                    rtt += q0 * y0 + q1 * y1;
                                }
                            };
                            GROUP_ROWS(row)
                        }
                        float v4[4] = {ts, tt, rts, rtt};
                        block_store_f<4>(v4, a.partial, G);
                    }
                    if (!grid_sync(a.bar)) goto timeout;
                    {
                        double s4[4];
                        range_sum<4>(a.partial, G, sv.b0, sv.b1, s4);
                        if (act) {
                            omega = block_once([=] { return s4[0] / s4[1]; });
                            rr = fmax(0.0, ssum - 2.0 * omega * s4[0] + omega * omega * s4[1]);
                            rtr = s4[2] - omega * s4[3];
                            rho2 = rho1;
                            it++;
                            nit++;
                            pending = true;
                        }
                    }
                }
            }
            // x += scale * rho * d (FP64) and the tangent vectors of the new x
            if (!done) {
                const double f = a.scale * rho;
                SAMPLE_ROWS(i) {
                    const double x0 = a.x[2 * i] + f * (double)a.d[2 * i];
                    const double x1 = a.x[2 * i + 1] + f * (double)a.d[2 * i + 1];
                    a.x[2 * i] = x0;
                    a.x[2 * i + 1] = x1;
                    tangent<double>(i, a.ep, a.eq, x0, x1, a.W64);
                }
                nref++;
            }
            if (!grid_sync(a.bar)) goto timeout;
        }
        const bool fail = (status != 0);
        if (!grid_sync(a.bar)) goto timeout;
        double v2max = 0.0;
        if (!fail) {
            SAMPLE_ROWS(i) {
                if (!a.mag[i]) continue;
                const double vp = a.x[2 * i], vq = a.x[2 * i + 1];
                v2max = fmax(v2max, vp * vp + vq * vq);
                const double pa = vp * FG_GAMMA0, qb = vq * FG_GAMMA0;
                double nv[3], nu[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    nv[c] = pa * a.ep[3 * i + c] + qb * a.eq[3 * i + c];
                    nu[c] = a.u0[3 * i + c] + dt * nv[c];
                }
                const double n = sqrt(nu[0] * nu[0] + nu[1] * nu[1] + nu[2] * nu[2]);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    a.v1[3 * i + c] = nv[c];
                    a.u1[3 * i + c] = nu[c] / n;
                }
            }
        }
        v2max = dmax_reduce_block(v2max);
        if (threadIdx.x == 0) {
            SolveResult *R = a.res + sv.g;
            atomicMax((unsigned long long *)&R->v2max, (unsigned long long)__double_as_longlong(v2max));
            if (blockIdx.x == sv.b0) {
                R->status = status;
                R->nit = nit;
                R->nref = nref;
                R->fail = fail ? 1 : 0;
                R->res = res;
                R->rhsn = rhsn;
                R->res0 = res0;
            }
            if (a.acc) {
                SegAcc *S = a.acc + sv.g;
                atomicMax((unsigned long long *)&S->v2max, (unsigned long long)__double_as_longlong(v2max));
                if (blockIdx.x == sv.b0) {
                    S->nit_sum += nit;
                    S->nref_sum += nref;
                    S->nit_max = max(S->nit_max, nit);
                    S->nref_max = max(S->nref_max, nref);
                    if (fail) {
                        if (S->fails == 0) S->first_fail = a.step_ctr ? *a.step_ctr : 0;
                        S->fails++;
                        S->worst = max(S->worst, status == 1 ? 1 : 2);
                    }
                }
            }
        }
        return;
    }
timeout:
    if (blockIdx.x == sv.b0 && threadIdx.x == 0) {
        a.res[sv.g].timeout = 1;
        a.res[sv.g].fail = 1;
        if (a.acc) {
            if (a.acc[sv.g].fails == 0) a.acc[sv.g].first_fail = a.step_ctr ? *a.step_ctr : 0;
            a.acc[sv.g].fails++;
            a.acc[sv.g].worst = 3;
        }
    }
}

#undef SAMPLE_ROWS
#undef GROUP_ROWS

int mixed_max_blocks(Ctx &c) {
    int per_sm = 0;
    int per_sm2 = 0, per_sm3 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mixed<1>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_mixed<4>, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm3, k_mixed<8>, 256, 0);
    per_sm = std::min(per_sm, std::min(per_sm2, per_sm3));
    return std::max(1, per_sm) * c.nsm;
}

int mixed_grid_size(Ctx &c) {
    int per_sm = 0;
    {
        int p1 = 0, p4 = 0, p8 = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p1, k_mixed<1>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p4, k_mixed<4>, 256, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p8, k_mixed<8>, 256, 0);
        per_sm = std::min(p1, std::min(p4, p8));
    }
    if (per_sm < 1) per_sm = 1;
    int g = per_sm * c.nsm;
    const int need = (c.nn + 255) / 256;
    if (need < g) g = need;
    return g < 1 ? 1 : g;
}

cudaError_t launch_mixed(Ctx &c, double dt, double prefactor) {
    const size_t n2 = 2 * (size_t)c.nn;
    MixedArgs a;
    a.nn = c.nn;
    a.Sptr = c.Sptr; a.Scol = c.Scol; a.Sval = c.Sval; a.A = c.A; a.Dl = c.Dl; a.ep = c.ep; a.eq = c.eq;
    a.Sval32 = c.Sval32; a.A32 = c.A32;
    a.ep32 = c.ep32; a.eq32 = c.eq32; a.Dl32 = c.Dl32;
    float *f = c.fv;
    a.r = f; a.rt = f + n2; a.p = f + 2 * n2; a.v = f + 3 * n2; a.s = f + 4 * n2; a.t = f + 5 * n2;
    a.phat = f + 6 * n2; a.shat = f + 7 * n2; a.d = f + 8 * n2; a.Minv32 = f + 9 * n2; a.W32 = f + 10 * n2;
    a.mag = c.mag;
    a.c0 = prefactor * FG_THETA * dt * FG_GAMMA0;
    a.b = c.rhs; a.x = c.x;
    a.r64 = c.bv; a.W64 = c.W;
    a.partial = c.partial; a.bar = c.bar; a.res = c.dres;
    a.tol = c.opts.tol; a.inner_tol = c.opts.inner_tol;
    a.maxiter = c.opts.max_iter; a.refine_max = c.opts.refine_max;
    a.dt = dt; a.u0 = c.u[0]; a.u1 = c.u[1]; a.v1 = c.v[1];
    a.scale = 1.0 / c.mean_A;
    a.cand_x = c.cand_x;
    a.cand_W = c.cand_W;
    a.cand_r = c.cand_r;
    a.cand_flag = c.cand_flag;
    a.cand_res2 = c.cand_res2;
    a.cand_o = c.cand_o;
    a.cand_vprev = c.cand_vprev;
    a.cand_vprev2 = c.cand_vprev2;
    a.cand_scale = c.cand_scale;
    a.nseg = 1;
    a.seg_node = a.seg_blk = nullptr;
    a.seg = nullptr;
    a.acc = nullptr;
    a.step_ctr = nullptr;
    int grid = c.mixed_grid, nres = 1;
    if (c.batch) {
        a.nseg = c.nseg;
        a.seg_node = c.d_seg_node;
        a.seg_blk = c.d_seg_blk;
        a.seg = c.seg_par;
        a.acc = c.acc_active;
        a.step_ctr = c.step_ctr;
        grid = c.seg_grid;
        nres = c.nseg;
    }
    cudaError_t e = cudaMemsetAsync(c.bar, 0, sizeof(GridBar), c.stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(c.dres, 0, sizeof(SolveResult) * nres, c.stream);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(c.batch ? 256 : c.mixed_threads);
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const int lpr = c.lpr > 0 ? c.lpr : 1;
    if (lpr == 8) return cudaLaunchKernelEx(&cfg, k_mixed<8>, a);
    if (lpr == 4) return cudaLaunchKernelEx(&cfg, k_mixed<4>, a);
    return cudaLaunchKernelEx(&cfg, k_mixed<1>, a);
}

// Failure-path probe: block 0 leaves without arriving at the grid barrier, so block 1's
// bounded wait must expire (about 2 s), set the barrier's error and return false.
__global__ void k_barrier_timeout_probe(GridBar *bar, int *out) {
    if (blockIdx.x == 0) return;
    const bool ok = grid_sync(bar);
    if (threadIdx.x == 0 && !ok) atomicExch(out, 1);
}

cudaError_t launch_barrier_timeout_probe(Ctx &c, int *out) {
    cudaError_t e = cudaMemsetAsync(c.bar, 0, sizeof(GridBar), c.stream);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2);
    cfg.blockDim = dim3(32);
    cfg.stream = c.stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_barrier_timeout_probe, c.bar, out);
}

// Co-resident blocks per SM of the variant with LPR lanes per row at the given block size.
static int mixed_blocks_per_sm(int lpr, int threads) {
    int n = 0;
    if (lpr == 8) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mixed<8>, threads, 0);
    else if (lpr == 4) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mixed<4>, threads, 0);
    else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mixed<1>, threads, 0);
    return n;
}

cudaError_t mixed_autotune(Ctx &c, double dt, double prefactor, double angle) {
    if (c.lpr > 0) return cudaSuccess;
    if (c.opts.solver_lpr == 1 || c.opts.solver_lpr == 4 || c.opts.solver_lpr == 8) {
        c.lpr = c.opts.solver_lpr;
        if (c.opts.solver_blocks > 0 && !c.batch) c.mixed_grid = std::min(c.opts.solver_blocks, c.mixed_grid);
        if (c.opts.solver_threads == 512 && !c.batch) {
            const int per_sm = mixed_blocks_per_sm(c.lpr, 512);
            if (per_sm < 1) {
                c.err = "solver_threads 512: a block of 512 threads does not fit on an SM";
                return cudaErrorInvalidConfiguration;
            }
            c.mixed_threads = 512;
            c.mixed_grid = std::min(c.mixed_grid, per_sm * c.nsm);  // all blocks co-resident
        }
        return cudaSuccess;
    }
    const int cand[3] = {1, 4, 8};
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (e != cudaSuccess) return e;
    e = cudaEventCreate(&e1);
    if (e != cudaSuccess) return e;
    SegAcc *acc = c.acc_active;
    c.acc_active = nullptr;
    // the timed solves write NEXT (u1, v1) and the next initial guess is read from v1: keep
    // both in spare FP64 vectors and put them back afterwards
    const size_t n3 = 3 * sizeof(double) * c.nn;
    double *keep_v = c.bv + 4 * (size_t)c.nn, *keep_u = keep_v + 3 * (size_t)c.nn;
    if ((e = cudaMemcpyAsync(keep_v, c.v[1], n3, cudaMemcpyDeviceToDevice, c.stream)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(keep_u, c.u[1], n3, cudaMemcpyDeviceToDevice, c.stream)) != cudaSuccess) return e;
    double best = 1e300;
    int bestv = 1, bestg = c.mixed_grid, bestt = 256;
    std::vector<SolveResult> res(c.batch ? c.nseg : 1);
    // launch shapes of the single-system solver: all co-resident blocks of 256 threads, or 2 or
    // 1 per SM (fewer blocks make each grid barrier cheaper), and one block of 512 threads per
    // SM (as few blocks, twice the warps); a batch keeps its per-sample block ranges
    std::vector<int2> shapes{make_int2(c.mixed_grid, 256)};
    if (!c.batch) {
        for (int g : {2 * c.nsm, c.nsm})
            if (g < c.mixed_grid) shapes.push_back(make_int2(g, 256));
        if (c.nsm <= c.mixed_grid) shapes.push_back(make_int2(c.nsm, 512));
    }
    const int gmax = c.mixed_grid;
    for (int vi = 0; vi < 3 * (int)shapes.size(); vi++) {
        const int v = cand[vi % 3];
        const int2 sh = shapes[vi / 3];
        if (sh.y == 512 && mixed_blocks_per_sm(v, 512) < 1) continue;  // does not fit: not a candidate
        c.lpr = v;
        c.mixed_grid = sh.x;
        c.mixed_threads = sh.y;
        for (int rep = 0; rep < 2; rep++) {  // the first run of each variant warms it up
            if ((e = launch_node(c, angle)) != cudaSuccess) break;
            cudaEventRecord(e0, c.stream);
            if ((e = launch_mixed(c, dt, prefactor)) != cudaSuccess) break;
            cudaEventRecord(e1, c.stream);
            cudaMemcpyAsync(res.data(), c.dres, sizeof(SolveResult) * res.size(), cudaMemcpyDeviceToHost, c.stream);
            if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            int it = 1;
            for (const SolveResult &r : res) it = std::max(it, r.nit + r.nref);
            if (rep == 1 && !res[0].timeout && ms / it < best) {
                best = ms / it;
                bestv = v;
                bestg = c.mixed_grid;
                bestt = c.mixed_threads;
            }
        }
        if (e != cudaSuccess) break;
        cudaMemsetAsync(c.bar, 0, sizeof(GridBar), c.stream);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaMemcpyAsync(c.v[1], keep_v, n3, cudaMemcpyDeviceToDevice, c.stream);
    cudaMemcpyAsync(c.u[1], keep_u, n3, cudaMemcpyDeviceToDevice, c.stream);
    c.acc_active = acc;
    c.lpr = bestv;
    c.mixed_grid = e == cudaSuccess ? bestg : gmax;
    c.mixed_threads = e == cudaSuccess ? bestt : 256;
    if (c.opts.verbose)
        fprintf(stderr, "mixed solver: %d lane(s) per row, %d blocks of %d threads\n", bestv, c.mixed_grid,
                c.mixed_threads);
    return e;
}

}  // namespace fg
