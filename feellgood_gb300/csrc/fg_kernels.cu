// Device kernels of the per-time-step LLG update (sm_103a).
//
// Formulation. In Tet::integrales (src/tetra.cpp:210-307) the 12x12 matrix AE has
// off-diagonal node couplings only through the exchange block c*vol*(da_i . da_j),
// identical in the three Cartesian components; the magnetisation cross terms and the
// lumped damping sit on the node diagonal. Projected with P and the row permutation
// Perm, the 2x2 block of K coupling nodes i != j is therefore
//     c0 * S_ij * [eq_i.ep_j  eq_i.eq_j ; ep_i.ep_j  ep_i.eq_j],
// with S_ij = sum_t Abis_t vol_t (da_i . da_j) a STATIC scalar stiffness matrix and
// c0 = prefactor * theta * dt * gamma0. The diagonal block of node i is
//     [A_i  D_i ; D_i  -A_i],  A_i = sum_t sum_g a_i(g) w_g (lumped mass, static),
//     D_i = c0 S_ii + sum_t sum_g a_i(g) w_g alpha_eff(g).
// (u x ep = eq and u x eq = -ep for the orthonormal basis of Node::setBasis.) So the
// per-step element work reduces to four scalars per (tet, vertex): the lumped damping
// and the 3-vector BE, and K x needs only S, the basis and two diagonals:
//     (K x)_i = [eq_i ; ep_i] . (c0 sum_j S_ij W_j) + diag block * x_i,
//     W_j = x_2j ep_j + x_2j+1 eq_j.
// The RHS is L_i = [eq_i . BE_i ; ep_i . BE_i] (Perm P BE, src/tetra.cpp:306).
#include <cooperative_groups.h>

#include <cmath>
#include <cstdio>

#include "fg_internal.h"
#include "fg_device.cuh"
#include "fg_ds.cuh"

namespace fg {

__constant__ double c_ta[4][5];   // tet shape functions at Gauss points (src/tetra.h:50-80)
__constant__ double c_tpds[5];
__constant__ float c_tpds32[5];  // the same weights in FP32 (charges of the incremental demag)
__constant__ double c_cw[4][5];   // c_ta[i][g] * c_tpds[g]: weight of vertex i at Gauss point g per unit detJ
__constant__ double c_cws[4];     // sum_g c_cw[i][g]
__constant__ double c_tps;        // sum_g c_tpds[g]
__constant__ float2 c_cws_dsp[4], c_tps_dsp;  // the same as double-single pairs (energies)
__constant__ double c_fa[3][4];   // triangle rule (src/triangle.h:42-64)
__constant__ float2 c_fa_ds[3][4];  // the same weights as double-single pairs
__constant__ float c_fa32[3][4];    // and in FP32 (charges of the incremental demag)
__constant__ double c_fpds[4];

// ---------------------------------------------------------------------------------
// Element kernel: one thread per magnetic tetrahedron. Restates the interpolation,
// calc_alpha_eff, anisotropy and BE parts of Tet::integrales (src/tetra.cpp:47-75,
// 171-307) and writes per vertex (lumped alpha_eff weight, BE_i) to its slot.

template <int NPI, bool DRIFT>
__global__ void __launch_bounds__(128) k_tet64(int nmt, const int4 *__restrict__ tet, const double *__restrict__ da,
                                               const double *__restrict__ detJ, const int *__restrict__ treg,
                                               const DevRegion *__restrict__ regs, const double *__restrict__ u0,
                                               const double *__restrict__ v0, const double *__restrict__ phi0,
                                               const double *__restrict__ phiv0, double dt, double Hx, double Hy,
                                               double Hz, double4 *__restrict__ slot,
                                               const int *__restrict__ tet_seg, const SegPar *__restrict__ seg,
                                               const double *__restrict__ hsp, double amp,
                                               const double *__restrict__ s_node, int ddir, double vdrift) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmt) return;
    if (seg) {  // batch: the tet's sample carries dt and the applied field
        const SegPar &P = seg[tet_seg[t]];
        dt = P.dt; Hx = P.H[0]; Hy = P.H[1]; Hz = P.H[2];
    }
    const int4 I = tet[t];
    const int ind[4] = {I.x, I.y, I.z, I.w};
    double d[4][3];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) d[i][k] = da[(3 * i + k) * (size_t)nmt + t];
    const double J = detJ[t];
    const DevRegion &R = regs[treg[t]];
    double un[4][3], vn[4][3], ph[4], phv[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const double *pu = u0 + 3 * (size_t)ind[i];
        const double *pv = v0 + 3 * (size_t)ind[i];
        un[i][0] = pu[0]; un[i][1] = pu[1]; un[i][2] = pu[2];
        vn[i][0] = pv[0]; vn[i][1] = pv[1]; vn[i][2] = pv[2];
        ph[i] = phi0[ind[i]];
        phv[i] = phiv0[ind[i]];
    }
    // constant gradients: dU[k][c] = d u_c / d x_k
    double dU[3][3], Hd[3], Hv[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double s = 0.0;
#pragma unroll
            for (int i = 0; i < 4; i++) s += d[i][k] * un[i][c];
            dU[k][c] = s;
        }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        double h = 0.0, hv = 0.0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            h -= ph[i] * d[i][c];
            hv -= phv[i] * d[i][c];
        }
        Hd[c] = h;
        Hv[c] = hv;
    }
    const double Abis = R.Abis, alpha = R.alpha;
    const double s_dt = FG_THETA * dt * FG_GAMMA0;
    const double gradsq = dU[0][0] * dU[0][0] + dU[0][1] * dU[0][1] + dU[0][2] * dU[0][2] +
                          dU[1][0] * dU[1][0] + dU[1][1] * dU[1][1] + dU[1][2] * dU[1][2] +
                          dU[2][0] * dU[2][0] + dU[2][1] * dU[2][1] + dU[2][2] * dU[2][2];
    const double He[3] = {Hd[0] + Hx, Hd[1] + Hy, Hd[2] + Hz};
    double w[NPI], aeff[NPI], H[NPI][3];
    // spin accumulation field Hst = hst s at the Gauss points (spinAcc::prepareExtraField,
    // Tetra::calc_Hst src/tetra.cpp:93-106), and the second-order term's (Hst . U) and V
    const bool spin = s_node && R.hst != 0.0;
    double Hst[NPI][3], sHu[NPI], Vg[NPI][3];
    const double reduced_dt = FG_GAMMA0 * dt;
    const double M = 2. * alpha * 0.1 / reduced_dt;
    // recentering drift (Tet::add_drift_BE, src/tetra.cpp:150-169, called at :277-288):
    // Dr(g) = alpha dU + U x dU + s_dt (alpha dV + U x dV + V x dU) with dU, dV the constant
    // derivatives of u and v along the direction; BE_i += vdrift w_g a_i(g) Dr(g)
    double dUr[3] = {0.0, 0.0, 0.0}, dVr[3] = {0.0, 0.0, 0.0}, Dr[DRIFT ? NPI : 1][3];
    if constexpr (DRIFT) {
#pragma unroll
        for (int k = 0; k < 3; k++) {  // selects the direction without indexing registers at run time
            if (k != ddir) continue;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                dUr[c] = dU[k][c];
#pragma unroll
                for (int i = 0; i < 4; i++) dVr[c] += d[i][k] * vn[i][c];
            }
        }
    }
#pragma unroll
    for (int g = 0; g < NPI; g++) {
        w[g] = J * c_tpds[g];
        double U[3], V[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            double su = 0.0, sv = 0.0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                su += c_ta[i][g] * un[i][c];
                sv += c_ta[i][g] * vn[i][c];
            }
            U[c] = su;
            V[c] = sv;
        }
        if constexpr (DRIFT) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
                Dr[g][c] = alpha * dUr[c] + (U[c1] * dUr[c2] - U[c2] * dUr[c1]) +
                           s_dt * (alpha * dVr[c] + (U[c1] * dVr[c2] - U[c2] * dVr[c1]) +
                                   (V[c1] * dUr[c2] - V[c2] * dUr[c1]));
            }
        }
        double uHeff = -Abis * gradsq;
        double Han[3] = {0.0, 0.0, 0.0};
        if (R.K != 0.0) {
            const double sdt = s_dt / FG_GAMMA0;
            const double kk = R.Kbis * (R.uk[0] * (U[0] + sdt * V[0]) + R.uk[1] * (U[1] + sdt * V[1]) +
                                        R.uk[2] * (U[2] + sdt * V[2]));
            Han[0] += kk * R.uk[0];
            Han[1] += kk * R.uk[1];
            Han[2] += kk * R.uk[2];
            const double uu = U[0] * R.uk[0] + U[1] * R.uk[1] + U[2] * R.uk[2];
            uHeff += R.Kbis * uu * uu;
        }
        if (R.K3 != 0.0) {
            const double sdt = s_dt / FG_GAMMA0;
            const double *e[3] = {R.ex, R.ey, R.ez};
            double ku[3], kv[3], uuu[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                ku[a] = e[a][0] * U[0] + e[a][1] * U[1] + e[a][2] * U[2];
                kv[a] = e[a][0] * V[0] + e[a][1] * V[1] + e[a][2] * V[2];
                uuu[a] = ku[a] * (1.0 - ku[a] * ku[a]);
            }
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const double tmp = kv[c] * R.ex[c];  // the reference multiplies by ex here
                const double h = uuu[0] * R.ex[c] + uuu[1] * R.ey[c] + uuu[2] * R.ez[c] +
                                 sdt * (tmp * (1.0 - 3.0 * ku[c] * ku[c]));
                Han[c] += -R.K3bis * h;
            }
            uHeff += -R.K3bis * (ku[0] * uuu[0] + ku[1] * uuu[1] + ku[2] * uuu[2]);
        }
        double Hg[3] = {He[0], He[1], He[2]};
        if (hsp) {  // space-dependent applied field at this Gauss point (R4toR3)
            const double *F = hsp + 3 * ((size_t)t * NPI + g);
            Hg[0] += amp * F[0]; Hg[1] += amp * F[1]; Hg[2] += amp * F[2];
        }
        if (spin) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                double h = 0.0;
#pragma unroll
                for (int i = 0; i < 4; i++) h += (R.hst * s_node[3 * (size_t)ind[i] + c]) * c_ta[i][g];
                Hst[g][c] = h;
                Vg[g][c] = V[c];
            }
            sHu[g] = Hst[g][0] * U[0] + Hst[g][1] * U[1] + Hst[g][2] * U[2];
            uHeff += U[0] * (Hg[0] + Hst[g][0]) + U[1] * (Hg[1] + Hst[g][1]) + U[2] * (Hg[2] + Hst[g][2]);
        } else {
            uHeff += U[0] * Hg[0] + U[1] * Hg[1] + U[2] * Hg[2];
        }
        // calc_alpha_eff (src/tetra.cpp:47-75)
        double a;
        if (uHeff > 0.0)
            a = (uHeff > M) ? alpha + reduced_dt / 2. * M : alpha + reduced_dt / 2. * uHeff;
        else
            a = (uHeff < -M) ? alpha / (1. + reduced_dt / (2. * alpha) * M)
                             : alpha / (1. - reduced_dt / (2. * alpha) * uHeff);
        aeff[g] = a;
        const double kv = s_dt / FG_GAMMA0;
#pragma unroll
        for (int c = 0; c < 3; c++) H[g][c] = Hg[c] + Han[c] + kv * Hv[c];
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        double contrib = 0.0;
#pragma unroll
        for (int g = 0; g < NPI; g++) contrib += c_ta[i][g] * w[g] * aeff[g];
        double ex[3];
#pragma unroll
        for (int c = 0; c < 3; c++) ex[c] = d[i][0] * dU[0][c] + d[i][1] * dU[1][c] + d[i][2] * dU[2][c];
        double BE[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int g = 0; g < NPI; g++) {
            const double ai_w = w[g] * c_ta[i][g];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                BE[c] -= w[g] * Abis * ex[c];
                if (spin) {  // Hst and the spin accumulation's second-order term (src/tetra.cpp:296-303)
                    BE[c] += ai_w * (H[g][c] + Hst[g][c]);
                    BE[c] -= ai_w * sHu[g] * (FG_THETA * dt * FG_GAMMA0) * Vg[g][c];
                } else {
                    BE[c] += ai_w * H[g][c];
                }
                if constexpr (DRIFT) BE[c] += vdrift * ai_w * Dr[g][c];
            }
        }
        slot[4 * (size_t)t + i] = make_double4(contrib, BE[0], BE[1], BE[2]);
    }
}

// Element kernel without anisotropy (all regions K = K3 = 0, the case of the benchmark
// configurations). The same quantities in closed form: with no anisotropy the Gauss-point
// fields of Tet::integrales reduce to constants per tet, so
//   uHeff(g) = -Abis |grad u|^2 + sum_i a_i(g) (u_i . He),            He = Hd + Hext
//   BE_i     = -Abis vol (da_i . grad) u + (sum_g w_g a_i(g)) (He + (s_dt/gamma0) Hv)
// and v is not read (it enters integrales only through the anisotropy terms).
template <int NPI>
__global__ void __launch_bounds__(128) k_tet64_iso(int nmt, const int4 *__restrict__ tet, const double *__restrict__ da,
                                                   const double *__restrict__ detJ, const int *__restrict__ treg,
                                                   const DevRegion *__restrict__ regs, const double *__restrict__ u0,
                                                   const double *__restrict__ phi0, const double *__restrict__ phiv0,
                                                   double dt, double Hx, double Hy, double Hz,
                                                   double4 *__restrict__ slot, const int *__restrict__ tet_seg,
                                                   const SegPar *__restrict__ seg, const double *__restrict__ hsp,
                                                   double amp, const double *__restrict__ s_node,
                                                   const double *__restrict__ v0) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmt) return;
    if (seg) {
        const SegPar &P = seg[tet_seg[t]];
        dt = P.dt; Hx = P.H[0]; Hy = P.H[1]; Hz = P.H[2];
    }
    const int4 I = tet[t];
    const int ind[4] = {I.x, I.y, I.z, I.w};
    double d[4][3];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) d[i][k] = da[(3 * i + k) * (size_t)nmt + t];
    const double J = detJ[t];
    const DevRegion &R = regs[treg[t]];
    double un[4][3], ph[4], phv[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const double *pu = u0 + 3 * (size_t)ind[i];
        un[i][0] = pu[0]; un[i][1] = pu[1]; un[i][2] = pu[2];
        ph[i] = phi0[ind[i]];
        phv[i] = phiv0[ind[i]];
    }
    double dU[3][3], Hd[3], Hv[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) dU[k][c] = d[0][k] * un[0][c] + d[1][k] * un[1][c] + d[2][k] * un[2][c] + d[3][k] * un[3][c];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        Hd[c] = -(ph[0] * d[0][c] + ph[1] * d[1][c] + ph[2] * d[2][c] + ph[3] * d[3][c]);
        Hv[c] = -(phv[0] * d[0][c] + phv[1] * d[1][c] + phv[2] * d[2][c] + phv[3] * d[3][c]);
    }
    const double Abis = R.Abis, alpha = R.alpha;
    double gradsq = 0.0;
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) gradsq += dU[k][c] * dU[k][c];
    const double He[3] = {Hd[0] + Hx, Hd[1] + Hy, Hd[2] + Hz};
    double uh[4];
#pragma unroll
    for (int i = 0; i < 4; i++) uh[i] = un[i][0] * He[0] + un[i][1] * He[1] + un[i][2] * He[2];
    const double reduced_dt = FG_GAMMA0 * dt;
    const double M = 2. * alpha * 0.1 / reduced_dt;
    const double kv = FG_THETA * dt;  // s_dt / gamma0
    // calc_alpha_eff (src/tetra.cpp:47-75): alpha + (reduced_dt / 2) min(h, M) for h > 0,
    // alpha / (1 - reduced_dt / (2 alpha) max(h, -M)) otherwise
    const double half_rdt = reduced_dt / 2., k2 = reduced_dt / (2. * alpha);
    const double hx = -Abis * gradsq;
    // sum_g w_g a_i(g) aeff(g) with w_g = J tpds_g: the vertex weights c_cw = a_i(g) tpds_g
    // are constants, so J multiplies once
    double contrib[4] = {0, 0, 0, 0};
    // space-dependent applied field (R4toR3): amp F(g) adds U(g) . amp F(g) to uHeff(g) and
    // sum_g w_g a_i(g) amp F(g) to BE_i
    double fw[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    // spin accumulation (src/tetra.cpp:248-303): Hst(g) = hst sum_i a_i(g) s_i adds U(g).Hst(g)
    // to uHeff(g) and sum_g w_g a_i(g) (Hst(g) - (Hst(g).U(g)) s_dt V(g)) to BE_i
    const bool spin = s_node && R.hst != 0.0;
    double sw[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    double sn[4][3], vn[4][3];
    if (spin) {
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                sn[i][c] = R.hst * s_node[3 * (size_t)ind[i] + c];
                vn[i][c] = v0[3 * (size_t)ind[i] + c];
            }
    }
    const double sdt = FG_THETA * dt * FG_GAMMA0;
#pragma unroll
    for (int g = 0; g < NPI; g++) {
        double h = hx + c_ta[0][g] * uh[0] + c_ta[1][g] * uh[1] + c_ta[2][g] * uh[2] + c_ta[3][g] * uh[3];
        double U[3] = {0, 0, 0};
        if (hsp || spin) {
#pragma unroll
            for (int c = 0; c < 3; c++)
                U[c] = c_ta[0][g] * un[0][c] + c_ta[1][g] * un[1][c] + c_ta[2][g] * un[2][c] + c_ta[3][g] * un[3][c];
        }
        if (spin) {
            double Hs[3], Vg[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                Hs[c] = sn[0][c] * c_ta[0][g] + sn[1][c] * c_ta[1][g] + sn[2][c] * c_ta[2][g] + sn[3][c] * c_ta[3][g];
                Vg[c] = c_ta[0][g] * vn[0][c] + c_ta[1][g] * vn[1][c] + c_ta[2][g] * vn[2][c] + c_ta[3][g] * vn[3][c];
            }
            const double hu = Hs[0] * U[0] + Hs[1] * U[1] + Hs[2] * U[2];
            h += U[0] * Hs[0] + U[1] * Hs[1] + U[2] * Hs[2];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int c = 0; c < 3; c++) sw[i][c] += c_cw[i][g] * (Hs[c] - hu * sdt * Vg[c]);
        }
        if (hsp) {
            const double *F = hsp + 3 * ((size_t)t * NPI + g);
            h += amp * (U[0] * F[0] + U[1] * F[1] + U[2] * F[2]);
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int c = 0; c < 3; c++) fw[i][c] += c_cw[i][g] * F[c];
        }
        const double a = (h > 0.0) ? alpha + half_rdt * fmin(h, M) : alpha / (1. - k2 * fmax(h, -M));
#pragma unroll
        for (int i = 0; i < 4; i++) contrib[i] += c_cw[i][g] * a;
    }
    const double vol = J * c_tps, nva = -vol * Abis;
    const double H[3] = {He[0] + kv * Hv[0], He[1] + kv * Hv[1], He[2] + kv * Hv[2]};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const double aw = J * c_cws[i];
        double BE[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const double ex = d[i][0] * dU[0][c] + d[i][1] * dU[1][c] + d[i][2] * dU[2][c];
            BE[c] = nva * ex + aw * H[c];
            if (hsp) BE[c] += (amp * J) * fw[i][c];
            if (spin) BE[c] += J * sw[i][c];
        }
        slot[4 * (size_t)t + i] = make_double4(J * contrib[i], BE[0], BE[1], BE[2]);
    }
}

// Surface anisotropy of the magnetic triangles, Tri::integrales (src/triangle.cpp:6-36):
// BE(k, i) = sum_g w_g Kbis (uk . u(g)) a_i(g) uk_k with Kbis = 2 Ks / dMs, u of CURRENT;
// written per (triangle, vertex) beside the tet slots and gathered by the node kernel
// (zero for triangles of regions with Ks = 0, which the reference skips).
template <int NPF>
__global__ void k_tri_aniso(int nft, const int4 *__restrict__ tri, const DevTri *__restrict__ tc,
                            const double *__restrict__ u0, double *__restrict__ tri_be) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nft) return;
    const DevTri &T = tc[f];
    double BE[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (T.Ks != 0.0) {
        const int4 I = tri[f];
        const int ind[3] = {I.x, I.y, I.z};
        const double Kbis = 2.0 * T.Ks / T.dMs;
#pragma unroll
        for (int g = 0; g < NPF; g++) {
            double U[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < 3; i++) s += c_fa[i][g] * u0[3 * (size_t)ind[i] + c];
                U[c] = s;
            }
            const double pre = T.w[g] * Kbis * (T.uk[0] * U[0] + T.uk[1] * U[1] + T.uk[2] * U[2]);
#pragma unroll
            for (int i = 0; i < 3; i++)
#pragma unroll
                for (int k = 0; k < 3; k++) BE[i][k] += pre * c_fa[i][g] * T.uk[k];
        }
    }
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) tri_be[9 * (size_t)f + 3 * i + k] = BE[i][k];
}

// ---------------------------------------------------------------------------------
// Node kernel: Node::setBasis with the step's angle (src/node.h:73-102), the gather of
// the per-vertex slots (assembly, src/solver.cpp:11-48), the RHS projection, the Jacobi
// preconditioner (src/algebra/sparseMat.h:174-183) and the initial guess
// (src/linear_algebra.cpp:13-24: previous v on the new basis / gamma0).

__global__ void k_node64(int nn, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                         const double4 *__restrict__ slot, int slot_ds, const int *__restrict__ tinc_ptr,
                         const int *__restrict__ tinc, const double *__restrict__ tri_be,
                         const unsigned char *__restrict__ mag,
                         const double *__restrict__ Ainv, const double *__restrict__ u0, const double *__restrict__ v1,
                         double cr, double sr, double *__restrict__ ep, double *__restrict__ eq,
                         double *__restrict__ Dl, double *__restrict__ rhs, double *__restrict__ x,
                         double *__restrict__ Minv, double *__restrict__ W,
                         const int *__restrict__ node_seg, const SegPar *__restrict__ seg, NodeFeat nf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    if (seg) {  // batch: the angle of the node's sample
        cr = seg[node_seg[i]].cr;
        sr = seg[node_seg[i]].sr;
    }
    const double u[3] = {u0[3 * i], u0[3 * i + 1], u0[3 * i + 2]};
    double e[3], q[3];
    if (mag[i]) {
        const double ax = fabs(u[0]), ay = fabs(u[1]), az = fabs(u[2]);
        int m = 0;
        double mv = ax;
        if (ay < mv) { mv = ay; m = 1; }
        if (az < mv) { m = 2; }
        e[0] = (m == 0) - u[m] * u[0];
        e[1] = (m == 1) - u[m] * u[1];
        e[2] = (m == 2) - u[m] * u[2];
        // one reciprocal square root instead of a square root and three divisions (GB300's
        // FP64 pipe is 1/64 rate); the norm is exact to a few ulp either way
        const double in = rsqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
        e[0] *= in; e[1] *= in; e[2] *= in;
        q[0] = u[1] * e[2] - u[2] * e[1];
        q[1] = u[2] * e[0] - u[0] * e[2];
        q[2] = u[0] * e[1] - u[1] * e[0];
        double ne[3];
        for (int c = 0; c < 3; c++) {
            ne[c] = cr * e[c] - sr * q[c];
            q[c] = sr * e[c] + cr * q[c];
        }
        e[0] = ne[0]; e[1] = ne[1]; e[2] = ne[2];
    } else {
        e[0] = e[1] = e[2] = q[0] = q[1] = q[2] = 0.0;
    }
    ep[3 * i] = e[0]; ep[3 * i + 1] = e[1]; ep[3 * i + 2] = e[2];
    eq[3 * i] = q[0]; eq[3 * i + 1] = q[1]; eq[3 * i + 2] = q[2];
    double dl = 0.0, be0 = 0.0, be1 = 0.0, be2 = 0.0;
    if (slot_ds) {  // double-single slots scaled by 2^DS_SLOT_SCALE: sum in double-single, convert once
        const float4 *sf = reinterpret_cast<const float4 *>(slot);
        dsf a0 = {0.f, 0.f}, a1 = a0, a2 = a0, a3 = a0;
        for (int k = inc_ptr[i]; k < inc_ptr[i + 1]; k++) {
            const float4 h = sf[2 * (size_t)inc[k]], l = sf[2 * (size_t)inc[k] + 1];
            a0 = ds_add(a0, {h.x, l.x});
            a1 = ds_add(a1, {h.y, l.y});
            a2 = ds_add(a2, {h.z, l.z});
            a3 = ds_add(a3, {h.w, l.w});
        }
        dl = ds_to(a0) * DS_SLOT_INV;  // exact: a product by a power of two
        be0 = ds_to(a1) * DS_SLOT_INV;
        be1 = ds_to(a2) * DS_SLOT_INV;
        be2 = ds_to(a3) * DS_SLOT_INV;
    } else {
        for (int k = inc_ptr[i]; k < inc_ptr[i + 1]; k++) {
            const double4 s = slot[inc[k]];
            dl += s.x; be0 += s.y; be1 += s.z; be2 += s.w;
        }
    }
    if (tri_be)  // surface anisotropy of the adjacent magnetic triangles (Tri::integrales)
        for (int k = tinc_ptr[i]; k < tinc_ptr[i + 1]; k++) {
            const double *b = tri_be + 3 * (size_t)tinc[k];
            be0 += b[0]; be1 += b[1]; be2 += b[2];
        }
    Dl[i] = dl;
    const double ia = Ainv[i];  // 1 / A_i (0 off the magnetic nodes), formed once per mesh
    if (nf.feat) {  // the learned guess's per-node features: m, H_eff / Ms, v_prev / V0 (the
                    // 1-ring mean of m, features 9..11, is formed in FP32 from these rows later)
        float *f = nf.feat + 12 * (size_t)i;
        if (!mag[i]) {
#pragma unroll
            for (int k = 0; k < 12; k++) f[k] = 0.f;
        } else {
            const double hb[3] = {be0 * ia, be1 * ia, be2 * ia};
#pragma unroll
            for (int c = 0; c < 3; c++) {
                f[c] = (float)u[c];
                f[3 + c] = (float)(hb[c] * nf.inv_ms);
                f[6 + c] = (float)(v1[3 * i + c] * nf.inv_v0);
            }
        }
    }
    if (mag[i]) {
        rhs[2 * i] = q[0] * be0 + q[1] * be1 + q[2] * be2;
        rhs[2 * i + 1] = e[0] * be0 + e[1] * be1 + e[2] * be2;
        Minv[2 * i] = ia;
        Minv[2 * i + 1] = -ia;
        // initial guess v / gamma0 in the new basis (a start vector: the product with the
        // reciprocal is as good as the quotient)
        constexpr double inv_gamma0 = 1.0 / FG_GAMMA0;
        const double vv[3] = {v1[3 * i], v1[3 * i + 1], v1[3 * i + 2]};
        const double xp = (vv[0] * e[0] + vv[1] * e[1] + vv[2] * e[2]) * inv_gamma0;
        const double xq = (vv[0] * q[0] + vv[1] * q[1] + vv[2] * q[2]) * inv_gamma0;
        x[2 * i] = xp;
        x[2 * i + 1] = xq;
        W[3 * i] = xp * e[0] + xq * q[0];
        W[3 * i + 1] = xp * e[1] + xq * q[1];
        W[3 * i + 2] = xp * e[2] + xq * q[2];
    } else {
        rhs[2 * i] = rhs[2 * i + 1] = 0.0;
        Minv[2 * i] = Minv[2 * i + 1] = 0.0;
        x[2 * i] = x[2 * i + 1] = 0.0;
        W[3 * i] = W[3 * i + 1] = W[3 * i + 2] = 0.0;
    }
}

// ---------------------------------------------------------------------------------
// Persistent FP64 BiCGSTAB, one cooperative launch per solve. Same iteration, masks
// and stopping logic as algebra::bicg_dir (src/algebra/bicg.h:163-234) with the
// iteration monitor of src/algebra/iter.h:119-175; vector phases are separated by
// bounded grid barriers and the dot products are deterministic two-level reductions.
// On success the node update of LinAlgebra::solve (src/solver.cpp:74-88) is fused.

__global__ void __launch_bounds__(256) k_bicg64(BicgArgs a) {
    const int G = gridDim.x;
    const int nn = a.nn;
    const int stride = G * blockDim.x;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    // phase 0: r = b - K x (masked), rt = r, p = r; |b|^2, |r|^2
    {
        double bb = 0.0, rr = 0.0;
        for (int i = i0; i < nn; i += stride) {
            double y0, y1;
            const double xp = a.x[2 * i], xq = a.x[2 * i + 1];
            apply_row(i, a.Sptr, a.Scol, a.Sval, a.W, a.ep, a.eq, a.A, a.Dl, a.c0, xp, xq, y0, y1);
            const bool m = a.mag[i];
            const double b0 = m ? a.b[2 * i] : 0.0, b1 = m ? a.b[2 * i + 1] : 0.0;
            const double r0 = m ? b0 - y0 : 0.0, r1 = m ? b1 - y1 : 0.0;
            a.r[2 * i] = r0; a.r[2 * i + 1] = r1;
            a.rt[2 * i] = r0; a.rt[2 * i + 1] = r1;
            a.p[2 * i] = r0; a.p[2 * i + 1] = r1;
            bb += b0 * b0 + b1 * b1;
            rr += r0 * r0 + r1 * r1;
        }
        double v2[2] = {bb, rr};
        block_store<2>(v2, a.partial, G);
    }
    if (!grid_sync(a.bar)) goto timeout;
    {
        double s2[2];
        grid_sum<2>(a.partial, G, s2);
        const double rhsn = sqrt(fabs(s2[0]));
        const double resmax = a.tol;
        double rr = s2[1], rtr = s2[1];
        double rho1 = 0.0, rho2 = 0.0, alpha = 0.0, beta = 0.0, omega = 0.0;
        int status = -1, nit = 0;
        double res = sqrt(fabs(rr));
        const double res0 = res;
        // iteration::finished
        auto finished = [&](double nr) {
            res = fabs(nr);
            if (isnan(res)) {
                status = 2;
                return false;
            }
            const bool cv = res <= rhsn * resmax;
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
            // phase 1: p = r + beta (p - omega v); phat = M p; W = tangent(phat)
            for (int i = i0; i < nn; i += stride) {
                double p0 = a.p[2 * i], p1 = a.p[2 * i + 1];
                if (nit > 0) {
                    p0 = (p0 - omega * a.v[2 * i]) * beta + a.r[2 * i];
                    p1 = (p1 - omega * a.v[2 * i + 1]) * beta + a.r[2 * i + 1];
                    a.p[2 * i] = p0; a.p[2 * i + 1] = p1;
                }
                const double h0 = a.Minv[2 * i] * p0, h1 = a.Minv[2 * i + 1] * p1;
                a.phat[2 * i] = h0; a.phat[2 * i + 1] = h1;
                tangent(i, a.ep, a.eq, h0, h1, a.W);
            }
            if (!grid_sync(a.bar)) goto timeout;
            // phase 2: v = K phat (masked); v . rt
            {
                double vr = 0.0;
                for (int i = i0; i < nn; i += stride) {
                    double y0, y1;
                    apply_row(i, a.Sptr, a.Scol, a.Sval, a.W, a.ep, a.eq, a.A, a.Dl, a.c0, a.phat[2 * i],
                              a.phat[2 * i + 1], y0, y1);
                    if (!a.mag[i]) y0 = y1 = 0.0;
                    a.v[2 * i] = y0; a.v[2 * i + 1] = y1;
                    vr += y0 * a.rt[2 * i] + y1 * a.rt[2 * i + 1];
                }
                double v1[1] = {vr};
                block_store<1>(v1, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s1[1];
                grid_sum<1>(a.partial, G, s1);
                alpha = rho1 / s1[0];
            }
            // phase 3: s = r - alpha v; shat = M s; |s|^2
            {
                double ss = 0.0;
                for (int i = i0; i < nn; i += stride) {
                    const double s0 = a.r[2 * i] + (-alpha) * a.v[2 * i];
                    const double s1 = a.r[2 * i + 1] + (-alpha) * a.v[2 * i + 1];
                    a.s[2 * i] = s0; a.s[2 * i + 1] = s1;
                    ss += s0 * s0 + s1 * s1;
                }
                double v1[1] = {ss};
                block_store<1>(v1, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s1[1];
                grid_sum<1>(a.partial, G, s1);
                if (finished(sqrt(fabs(s1[0])))) {
                    for (int i = i0; i < nn; i += stride) {
                        a.x[2 * i] += alpha * a.phat[2 * i];
                        a.x[2 * i + 1] += alpha * a.phat[2 * i + 1];
                    }
                    break;
                } else if (status == 1 || status == 2) {
                    break;
                }
            }
            // phase 4: shat = M s, W = tangent(shat) ... needs a barrier before the SpMV
            for (int i = i0; i < nn; i += stride) {
                const double h0 = a.Minv[2 * i] * a.s[2 * i], h1 = a.Minv[2 * i + 1] * a.s[2 * i + 1];
                a.shat[2 * i] = h0; a.shat[2 * i + 1] = h1;
                tangent(i, a.ep, a.eq, h0, h1, a.W);
            }
            if (!grid_sync(a.bar)) goto timeout;
            // phase 5: t = K shat (masked); t.s, t.t
            {
                double ts = 0.0, tt = 0.0;
                for (int i = i0; i < nn; i += stride) {
                    double y0, y1;
                    apply_row(i, a.Sptr, a.Scol, a.Sval, a.W, a.ep, a.eq, a.A, a.Dl, a.c0, a.shat[2 * i],
                              a.shat[2 * i + 1], y0, y1);
                    if (!a.mag[i]) y0 = y1 = 0.0;
                    a.t[2 * i] = y0; a.t[2 * i + 1] = y1;
                    ts += y0 * a.s[2 * i] + y1 * a.s[2 * i + 1];
                    tt += y0 * y0 + y1 * y1;
                }
                double v2[2] = {ts, tt};
                block_store<2>(v2, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s2b[2];
                grid_sum<2>(a.partial, G, s2b);
                omega = s2b[0] / s2b[1];
            }
            // phase 6: x += alpha phat + omega shat; r = s - omega t; |r|^2, rt.r
            {
                double r2 = 0.0, rtr2 = 0.0;
                for (int i = i0; i < nn; i += stride) {
#pragma unroll
                    for (int c = 0; c < 2; c++) {
                        const int k = 2 * i + c;
                        double xv = a.x[k] + alpha * a.phat[k];
                        xv += omega * a.shat[k];
                        a.x[k] = xv;
                        const double rv = a.s[k] - omega * a.t[k];
                        a.r[k] = rv;
                        r2 += rv * rv;
                        rtr2 += a.rt[k] * rv;
                    }
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
        // solve() epilogue: failure test, then the fused node update
        const bool fail = (status == 1 || status == 2 || res > resmax);
        if (!grid_sync(a.bar)) goto timeout;
        double v2max = 0.0;
        if (!fail) {
            for (int i = i0; i < nn; i += stride) {
                if (!a.mag[i]) continue;
                const double vp = a.x[2 * i], vq = a.x[2 * i + 1];
                const double v2 = vp * vp + vq * vq;
                v2max = fmax(v2max, v2);
                const double pa = vp * FG_GAMMA0, qb = vq * FG_GAMMA0;
                double nv[3], nu[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    nv[c] = pa * a.ep[3 * i + c] + qb * a.eq[3 * i + c];
                    nu[c] = a.u0[3 * i + c] + a.dt * nv[c];
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
            // v2 >= 0: the bit patterns of non-negative doubles order like the values
            atomicMax((unsigned long long *)&a.res->v2max, (unsigned long long)__double_as_longlong(v2max));
            if (blockIdx.x == 0) {
                a.res->status = status;
                a.res->nit = nit;
                a.res->fail = fail ? 1 : 0;
                a.res->res = res;
                a.res->rhsn = rhsn;
                a.res->res0 = res0;
            }
        }
        return;
    }
timeout:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.res->timeout = 1;
        a.res->fail = 1;
    }
}

// The same FP64 BiCGSTAB for a batch of independent samples (a block-diagonal system):
// every sample runs the iteration of k_bicg64 with its own scalars, |b|, stopping test and
// node update (its own dt and c0), exactly as if it were solved alone, on its own range of
// blocks; a sample that has stopped idles through the remaining grid barriers. The loop
// ends when no sample is active: an activity flag rides along the first reduction of each
// pass (slot 1, summed over the whole grid).
__global__ void __launch_bounds__(256) k_bicg64_seg(BicgArgs a) {
    const int G = gridDim.x;
    int g = 0;
    {
        int lo = 0, hi = a.nseg - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (a.seg_blk[mid] <= (int)blockIdx.x) lo = mid;
            else hi = mid - 1;
        }
        g = lo;
    }
    const int r_lo = a.seg_node[g], r_hi = a.seg_node[g + 1];
    const int b0 = a.seg_blk[g], b1 = a.seg_blk[g + 1];
    const int stride = (b1 - b0) * blockDim.x;
    const int i0 = r_lo + (blockIdx.x - b0) * blockDim.x + threadIdx.x;
    const double c0 = a.seg[g].c0, dt = a.seg[g].dt;
    {
        double bb = 0.0, rr = 0.0;
        for (int i = i0; i < r_hi; i += stride) {
            double y0, y1;
            const double xp = a.x[2 * i], xq = a.x[2 * i + 1];
            apply_row(i, a.Sptr, a.Scol, a.Sval, a.W, a.ep, a.eq, a.A, a.Dl, c0, xp, xq, y0, y1);
            const bool m = a.mag[i];
            const double bv0 = m ? a.b[2 * i] : 0.0, bv1 = m ? a.b[2 * i + 1] : 0.0;
            const double r0 = m ? bv0 - y0 : 0.0, r1 = m ? bv1 - y1 : 0.0;
            a.r[2 * i] = r0; a.r[2 * i + 1] = r1;
            a.rt[2 * i] = r0; a.rt[2 * i + 1] = r1;
            a.p[2 * i] = r0; a.p[2 * i + 1] = r1;
            bb += bv0 * bv0 + bv1 * bv1;
            rr += r0 * r0 + r1 * r1;
        }
        double v2[2] = {bb, rr};
        block_store<2>(v2, a.partial, G);
    }
    if (!grid_sync(a.bar)) goto timeout;
    {
        double s2[2];
        range_sum<2>(a.partial, G, b0, b1, s2);
        const double rhsn = sqrt(fabs(s2[0]));
        const double resmax = a.tol;
        double rr = s2[1], rtr = s2[1];
        double rho1 = 0.0, rho2 = 0.0, alpha = 0.0, beta = 0.0, omega = 0.0;
        int status = -1, nit = 0;
        double res = sqrt(fabs(rr));
        const double res0 = res;
        auto finished = [&](double nr) {
            res = fabs(nr);
            if (isnan(res)) {
                status = 2;
                return false;
            }
            const bool cv = res <= rhsn * resmax;
            if (cv) status = 0;
            return cv;
        };
        bool act = true;
        for (;;) {
            if (act && finished(sqrt(fabs(rr)))) act = false;
            if (act) {
                rho1 = rtr;
                if (nit > 0) {
                    if (rho2 == 0.0 || omega == 0.0) {
                        status = 2;
                        act = false;
                    } else {
                        beta = (rho1 / rho2) * (alpha / omega);
                    }
                }
            }
            if (act)
                for (int i = i0; i < r_hi; i += stride) {
                    double p0 = a.p[2 * i], p1 = a.p[2 * i + 1];
                    if (nit > 0) {
                        p0 = (p0 - omega * a.v[2 * i]) * beta + a.r[2 * i];
                        p1 = (p1 - omega * a.v[2 * i + 1]) * beta + a.r[2 * i + 1];
                        a.p[2 * i] = p0; a.p[2 * i + 1] = p1;
                    }
                    const double h0 = a.Minv[2 * i] * p0, h1 = a.Minv[2 * i + 1] * p1;
                    a.phat[2 * i] = h0; a.phat[2 * i + 1] = h1;
                    tangent(i, a.ep, a.eq, h0, h1, a.W);
                }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double vr = 0.0;
                if (act)
                    for (int i = i0; i < r_hi; i += stride) {
                        double y0, y1;
                        apply_row(i, a.Sptr, a.Scol, a.Sval, a.W, a.ep, a.eq, a.A, a.Dl, c0, a.phat[2 * i],
                                  a.phat[2 * i + 1], y0, y1);
                        if (!a.mag[i]) y0 = y1 = 0.0;
                        a.v[2 * i] = y0; a.v[2 * i + 1] = y1;
                        vr += y0 * a.rt[2 * i] + y1 * a.rt[2 * i + 1];
                    }
                double v2[2] = {vr, (threadIdx.x == 0 && act) ? 1.0 : 0.0};
                block_store<2>(v2, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s1[1], f[1];
                range_sum<1>(a.partial, G, b0, b1, s1);
                grid_sum<1>(a.partial + G, G, f);
                if (f[0] == 0.0) break;  // every sample has ended
                if (act) alpha = rho1 / s1[0];
            }
            {
                double ss = 0.0;
                if (act)
                    for (int i = i0; i < r_hi; i += stride) {
                        const double s0 = a.r[2 * i] + (-alpha) * a.v[2 * i];
                        const double s1 = a.r[2 * i + 1] + (-alpha) * a.v[2 * i + 1];
                        a.s[2 * i] = s0; a.s[2 * i + 1] = s1;
                        ss += s0 * s0 + s1 * s1;
                    }
                double v1[1] = {ss};
                block_store<1>(v1, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s1[1];
                range_sum<1>(a.partial, G, b0, b1, s1);
                if (act) {
                    if (finished(sqrt(fabs(s1[0])))) {
                        for (int i = i0; i < r_hi; i += stride) {
                            a.x[2 * i] += alpha * a.phat[2 * i];
                            a.x[2 * i + 1] += alpha * a.phat[2 * i + 1];
                        }
                        act = false;
                    } else if (status == 1 || status == 2) {
                        act = false;
                    }
                }
            }
            if (act)
                for (int i = i0; i < r_hi; i += stride) {
                    const double h0 = a.Minv[2 * i] * a.s[2 * i], h1 = a.Minv[2 * i + 1] * a.s[2 * i + 1];
                    a.shat[2 * i] = h0; a.shat[2 * i + 1] = h1;
                    tangent(i, a.ep, a.eq, h0, h1, a.W);
                }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double ts = 0.0, tt = 0.0;
                if (act)
                    for (int i = i0; i < r_hi; i += stride) {
                        double y0, y1;
                        apply_row(i, a.Sptr, a.Scol, a.Sval, a.W, a.ep, a.eq, a.A, a.Dl, c0, a.shat[2 * i],
                                  a.shat[2 * i + 1], y0, y1);
                        if (!a.mag[i]) y0 = y1 = 0.0;
                        a.t[2 * i] = y0; a.t[2 * i + 1] = y1;
                        ts += y0 * a.s[2 * i] + y1 * a.s[2 * i + 1];
                        tt += y0 * y0 + y1 * y1;
                    }
                double v2[2] = {ts, tt};
                block_store<2>(v2, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s2b[2];
                range_sum<2>(a.partial, G, b0, b1, s2b);
                if (act) omega = s2b[0] / s2b[1];
            }
            {
                double r2 = 0.0, rtr2 = 0.0;
                if (act)
                    for (int i = i0; i < r_hi; i += stride) {
#pragma unroll
                        for (int c = 0; c < 2; c++) {
                            const int k = 2 * i + c;
                            double xv = a.x[k] + alpha * a.phat[k];
                            xv += omega * a.shat[k];
                            a.x[k] = xv;
                            const double rv = a.s[k] - omega * a.t[k];
                            a.r[k] = rv;
                            r2 += rv * rv;
                            rtr2 += a.rt[k] * rv;
                        }
                    }
                double v2[2] = {r2, rtr2};
                block_store<2>(v2, a.partial, G);
            }
            if (!grid_sync(a.bar)) goto timeout;
            {
                double s2c[2];
                range_sum<2>(a.partial, G, b0, b1, s2c);
                if (act) {
                    rr = s2c[0];
                    rtr = s2c[1];
                    rho2 = rho1;
                    nit++;
                    if (nit >= a.maxiter) status = 1;
                }
            }
        }
        const bool fail = (status == 1 || status == 2 || res > resmax);
        if (!grid_sync(a.bar)) goto timeout;
        double v2max = 0.0;
        if (!fail) {
            for (int i = i0; i < r_hi; i += stride) {
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
            SolveResult *R = a.res + g;
            atomicMax((unsigned long long *)&R->v2max, (unsigned long long)__double_as_longlong(v2max));
            if ((int)blockIdx.x == b0) {
                R->status = status;
                R->nit = nit;
                R->fail = fail ? 1 : 0;
                R->res = res;
                R->rhsn = rhsn;
                R->res0 = res0;
            }
            if (a.acc) {
                SegAcc *S = a.acc + g;
                atomicMax((unsigned long long *)&S->v2max, (unsigned long long)__double_as_longlong(v2max));
                if ((int)blockIdx.x == b0) {
                    S->nit_sum += nit;
                    S->nit_max = max(S->nit_max, nit);
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
    if ((int)blockIdx.x == b0 && threadIdx.x == 0) {
        a.res[g].timeout = 1;
        a.res[g].fail = 1;
        if (a.acc) {
            if (a.acc[g].fails == 0) a.acc[g].first_fail = a.step_ctr ? *a.step_ctr : 0;
            a.acc[g].fails++;
            a.acc[g].worst = 3;
        }
    }
}

// y = K x for inspection (two launches: tangent vectors, then rows).
__global__ void k_tangent64(int nn, const double *x, const double *ep, const double *eq, double *W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nn) tangent(i, ep, eq, x[2 * i], x[2 * i + 1], W);
}
__global__ void k_apply64(int nn, const int *Sptr, const int *Scol, const double *Sval, const double *W,
                          const double *ep, const double *eq, const double *A, const double *Dl,
                          const unsigned char *mag, double c0, const double *x, double *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double y0, y1;
    apply_row(i, Sptr, Scol, Sval, W, ep, eq, A, Dl, c0, x[2 * i], x[2 * i + 1], y0, y1);
    if (!mag[i]) y0 = y1 = 0.0;
    y[2 * i] = y0;
    y[2 * i + 1] = y1;
}

// ---------------------------------------------------------------------------------
// Demag sources: Tet::charges (src/tetra.cpp:347-359), Tri::charges and the
// self-corrections of Tri::correctionCharges + Tri::potential (src/triangle.cpp:45-125),
// in the source order of fmm::calc_charges (src/fmm_demag.h:155-179).

template <int NPI, int NPF, int NQ>
__global__ void k_charges(int nmt, int nft, const int4 *__restrict__ tet, const double *__restrict__ da,
                          const double *__restrict__ detJ, const int *__restrict__ treg,
                          const DevRegion *__restrict__ regs, const int4 *__restrict__ tri,
                          const DevTri *__restrict__ tc, const double *__restrict__ m0, const double *__restrict__ m1,
                          const int *__restrict__ dst, double *__restrict__ q0, double *__restrict__ q1,
                          double *__restrict__ ts0, double *__restrict__ ts1) {
    // NQ = 2: the charges of two fields (m and v) from one pass over the geometry
    const double *mm[2] = {m0, m1};
    double *qq[2] = {q0, q1}, *ts[2] = {ts0, ts1};
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nmt) {
        const int4 I = tet[k];
        const int ind[4] = {I.x, I.y, I.z, I.w};
        double d[4][3];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int c = 0; c < 3; c++) d[i][c] = da[(3 * i + c) * (size_t)nmt + k];
        const double Ms = regs[treg[k]].Ms, J = detJ[k];
#pragma unroll
        for (int f = 0; f < NQ; f++) {
            double dud = 0.0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const double *pm = mm[f] + 3 * (size_t)ind[i];
                dud += pm[0] * d[i][0] + pm[1] * d[i][1] + pm[2] * d[i][2];
            }
#pragma unroll
            for (int g = 0; g < NPI; g++) {
                const size_t s = (size_t)k * NPI + g;
                qq[f][dst ? dst[s] : s] = -Ms * (J * c_tpds[g]) * dud;
            }
        }
    } else if (k < nmt + nft) {
        const int f = k - nmt;
        const int4 I = tri[f];
        const int ind[3] = {I.x, I.y, I.z};
        const DevTri &T = tc[f];
#pragma unroll
        for (int h = 0; h < NQ; h++) {
            double s[3];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const double *pm = mm[h] + 3 * (size_t)ind[i];
                s[i] = pm[0] * T.n[0] + pm[1] * T.n[1] + pm[2] * T.n[2];
            }
#pragma unroll
            for (int g = 0; g < NPF; g++) {
                double un = c_fa[0][g] * s[0] + c_fa[1][g] * s[1] + c_fa[2][g] * s[2];
                const size_t sidx = (size_t)nmt * NPI + (size_t)f * NPF + g;
                qq[h][dst ? dst[sidx] : sidx] = (T.dMs != 0.0) ? T.dMs * T.w[g] * un : 0.0;
            }
#pragma unroll
            for (int i = 0; i < 3; i++)
                ts[h][3 * (size_t)f + i] =
                    T.dMs * (T.beta[3 * i] * s[0] + T.beta[3 * i + 1] * s[1] + T.beta[3 * i + 2] * s[2]);
        }
    }
}

// The charges of the change of the field (incremental demag of the FP32 path) in FP32:
// the volume charges from FP32 copies of da and of -Ms detJ (k_charges' formula, FP32
// arithmetic: the FP32 FMM reads FP32 charges), written as FP32 in the FMM's leaf order;
// the triangles (few) in FP64 as in k_charges, their charges stored as FP32 and their
// self-correction terms as FP64 for k_phi_final.
template <int NPI, int NPF, int NQ>
__global__ void k_charges32(int nmt, int nft, const int4 *__restrict__ tet, const float *__restrict__ da32,
                            const float *__restrict__ cq32, const int4 *__restrict__ tri,
                            const float4 *__restrict__ tc32, const float *__restrict__ m0, const float *__restrict__ m1,
                            const int *__restrict__ dst, float *__restrict__ q0, float *__restrict__ q1,
                            double *__restrict__ ts0, double *__restrict__ ts1) {
    const float *mm[2] = {m0, m1};
    float *qq[2] = {q0, q1};
    double *ts[2] = {ts0, ts1};
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nmt) {
        const int4 I = tet[k];
        const int ind[4] = {I.x, I.y, I.z, I.w};
        float d[4][3];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int c = 0; c < 3; c++) d[i][c] = da32[(3 * i + c) * (size_t)nmt + k];
        const float cq = cq32[k];
#pragma unroll
        for (int f = 0; f < NQ; f++) {
            float dud = 0.f;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const float *pm = mm[f] + 3 * (size_t)ind[i];
                dud += pm[0] * d[i][0] + pm[1] * d[i][1] + pm[2] * d[i][2];
            }
#pragma unroll
            for (int g = 0; g < NPI; g++) {
                const size_t s = (size_t)k * NPI + g;
                qq[f][dst[s]] = cq * c_tpds32[g] * dud;
            }
        }
    } else if (k < nmt + nft) {
        // per triangle in FP32 from constants formed on the host: n, dMs w_g, dMs beta
        const int f = k - nmt;
        const int4 I = tri[f];
        const int ind[3] = {I.x, I.y, I.z};
        const float4 *T = tc32 + 4 * (size_t)f;
        const float4 t0 = T[0], t1 = T[1], t2 = T[2], t3 = T[3];
        const float n[3] = {t0.x, t0.y, t0.z};
        const float wq[4] = {t0.w, t1.x, t1.y, t1.z};
        const float be[9] = {t1.w, t2.x, t2.y, t2.z, t2.w, t3.x, t3.y, t3.z, t3.w};
#pragma unroll
        for (int h = 0; h < NQ; h++) {
            float sn[3];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                const float *pm = mm[h] + 3 * (size_t)ind[i];
                sn[i] = pm[0] * n[0] + pm[1] * n[1] + pm[2] * n[2];
            }
#pragma unroll
            for (int g = 0; g < NPF; g++) {
                const float un = c_fa32[0][g] * sn[0] + c_fa32[1][g] * sn[1] + c_fa32[2][g] * sn[2];
                const size_t sidx = (size_t)nmt * NPI + (size_t)f * NPF + g;
                qq[h][dst[sidx]] = wq[g] * un;
            }
#pragma unroll
            for (int i = 0; i < 3; i++)
                ts[h][3 * (size_t)f + i] = (double)(be[3 * i] * sn[0] + be[3 * i + 1] * sn[1] + be[3 * i + 2] * sn[2]);
        }
    }
}

// Exact FP64 direct sum pot_i = sum_s q_s / |x_i - y_s| over all sources, tiled through
// shared memory (one thread per magnetic node).
__global__ void __launch_bounds__(256) k_p2p_direct64(int nt, const int *__restrict__ tnode,
                                                      const double *__restrict__ xyz, int ns,
                                                      const double *__restrict__ sxyz,
                                                      const double *__restrict__ q, double *__restrict__ pot) {
    __shared__ double4 tile[256];
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double x = 0, y = 0, z = 0;
    int node = -1;
    if (k < nt) {
        node = tnode[k];
        x = xyz[3 * node];
        y = xyz[3 * node + 1];
        z = xyz[3 * node + 2];
    }
    double acc = 0.0;
    for (int base = 0; base < ns; base += 256) {
        const int s = base + threadIdx.x;
        if (s < ns) tile[threadIdx.x] = make_double4(sxyz[3 * s], sxyz[3 * s + 1], sxyz[3 * s + 2], q[s]);
        else tile[threadIdx.x] = make_double4(0, 0, 0, 0);
        __syncthreads();
        const int cnt = min(256, ns - base);
        for (int j = 0; j < cnt; j++) {
            const double4 t = tile[j];
            const double dx = x - t.x, dy = y - t.y, dz = z - t.z;
            acc += t.w * rsqrt(dx * dx + dy * dy + dz * dz);
        }
        __syncthreads();
    }
    if (node >= 0) pot[node] = acc;
}

// phi_i = (pot_i + corr_i) / (4 pi), src/fmm_demag.h:211-223; corr gathered per node.
__global__ void k_phi_final(int nt, const int *__restrict__ tnode, const int *__restrict__ tinc_ptr,
                            const int *__restrict__ tinc, const double *__restrict__ tri_slot,
                            const double *__restrict__ pot, const double *__restrict__ base,
                            double *__restrict__ phi) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nt) return;
    const int i = tnode[k];
    double corr = 0.0;
    for (int j = tinc_ptr[i]; j < tinc_ptr[i + 1]; j++) corr += tri_slot[tinc[j]];
    const double p = (pot[i] + corr) / (4 * M_PI);
    phi[i] = base ? base[i] + p : p;
}

// d = NEXT - CURRENT of u (first 3 nn) and of v (next 3 nn).
__global__ void k_state_diff(size_t n3, const double *__restrict__ u1, const double *__restrict__ u0,
                             const double *__restrict__ v1, const double *__restrict__ v0, float *__restrict__ d) {
    const size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (k >= n3) return;
    d[k] = (float)(u1[k] - u0[k]);
    d[n3 + k] = (float)(v1[k] - v0[k]);
}

// ---------------------------------------------------------------------------------
// Energies of the NEXT state and <m> (Fem::energy, src/energy.cpp:5-68; mesh::avg,
// src/mesh.cpp:89-106). partial layout: [7][G]: E_ex, E_aniso, E_demag, E_zeeman, <m>*V.

template <int NPI, int NPF, bool ISO>
__global__ void __launch_bounds__(256) k_energy(int nmt, int nft, const int4 *__restrict__ tet,
                                                const double *__restrict__ da, const double *__restrict__ detJ,
                                                const int *__restrict__ treg, const DevRegion *__restrict__ regs,
                                                const int4 *__restrict__ tri, const DevTri *__restrict__ tc,
                                                const double *__restrict__ u, const double *__restrict__ phi,
                                                double Hx, double Hy, double Hz, double *__restrict__ partial,
                                                const int4 *__restrict__ blk_rng, const int *__restrict__ blk_seg,
                                                const double *__restrict__ segH, const double *__restrict__ hsp,
                                                double amp, const float2 *__restrict__ da_ds,
                                                const float2 *__restrict__ J_ds, const float2 *__restrict__ st_ds,
                                                int nn_ds, const float4 *__restrict__ tri_ds) {
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    // isotropic form in double-single (FP32 + refinement path): state of NEXT and geometry as
    // double-single pairs, the Jacobian scaled by 2^DS_SLOT_SCALE; per-thread double-single sums
    dsf dacc[7] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    const bool dsp = ISO && da_ds;
    // default: grid-stride over all elements; batch: this block's ranges of one sample
    int stride = gridDim.x * blockDim.x, t0 = blockIdx.x * blockDim.x + threadIdx.x, t1 = nmt;
    int f0 = t0, f1 = nft;
    if (blk_rng) {
        const int4 r = blk_rng[blockIdx.x];
        stride = blockDim.x;
        t0 = r.x + threadIdx.x; t1 = r.y;
        f0 = r.z + threadIdx.x; f1 = r.w;
        const double *h = segH + 3 * blk_seg[blockIdx.x];
        Hx = h[0]; Hy = h[1]; Hz = h[2];
    }
    if (dsp) {
        // every constant as a double-single pair formed once (host, or one thread per block):
        // per-thread FP64 set-up and FP64 block sums would keep the 1/64-rate FP64 pipe busy
        // longer than the tets of a thread take on the FP32 pipes
        const float2 *uds = st_ds, *pds = st_ds + 3 * (size_t)nn_ds;
        __shared__ dsf Hsh[3];
        if (threadIdx.x == 0) {
            Hsh[0] = ds_from(Hx);
            Hsh[1] = ds_from(Hy);
            Hsh[2] = ds_from(Hz);
        }
        __syncthreads();
        dsf cw[4];
        const dsf tp = {c_tps_dsp.x, c_tps_dsp.y};
#pragma unroll
        for (int i = 0; i < 4; i++) cw[i] = {c_cws_dsp[i].x, c_cws_dsp[i].y};
        const dsf Hd[3] = {Hsh[0], Hsh[1], Hsh[2]};
        for (int k = t0; k < t1; k += stride) {
            const int4 I = tet[k];
            const int ind[4] = {I.x, I.y, I.z, I.w};
            // the region's constants as double-single pairs formed on the host (forming them
            // here would put FP64 conversions on the 1/64-rate FP64 pipe for every tet)
            const DevRegion &R = regs[treg[k]];
            const dsf rA = {R.A_ds.x, R.A_ds.y}, rD = {R.edm_ds.x, R.edm_ds.y}, rZ = {R.ez_ds.x, R.ez_ds.y};
            dsf un[4][3], ph[4], d[4][3];
#pragma unroll
            for (int i = 0; i < 4; i++) {
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const float2 a = uds[3 * (size_t)ind[i] + c], b = da_ds[(3 * i + c) * (size_t)nmt + k];
                    un[i][c] = {a.x, a.y};
                    d[i][c] = {b.x, b.y};
                }
                const float2 p = pds[ind[i]];
                ph[i] = {p.x, p.y};
            }
            dsf dU[3][3];
#pragma unroll
            for (int kk = 0; kk < 3; kk++)
#pragma unroll
                for (int c = 0; c < 3; c++)
                    dU[kk][c] = ds_fma(d[3][kk], un[3][c],
                                       ds_fma(d[2][kk], un[2][c], ds_fma(d[1][kk], un[1][c], ds_mul(d[0][kk], un[0][c]))));
            dsf dens = {0.f, 0.f};
#pragma unroll
            for (int kk = 0; kk < 3; kk++)
#pragma unroll
                for (int c = 0; c < 3; c++) dens = ds_fma(dU[kk][c], dU[kk][c], dens);
            const dsf div = ds_add(ds_add(dU[0][0], dU[1][1]), dU[2][2]);
            const float2 Jf = J_ds[k];
            const dsf J = {Jf.x, Jf.y};
            dsf su[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}}, sp = {0.f, 0.f};
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const dsf aw = ds_mul(J, cw[i]);
#pragma unroll
                for (int c = 0; c < 3; c++) su[c] = ds_fma(aw, un[i][c], su[c]);
                sp = ds_fma(aw, ph[i], sp);
            }
            dacc[0] = ds_fma(ds_mul(rA, ds_mul(J, tp)), dens, dacc[0]);
            dacc[2] = ds_fma(ds_mul(rD, div), sp, dacc[2]);
            dacc[3] = ds_fma(rZ, ds_fma(su[2], Hd[2], ds_fma(su[1], Hd[1], ds_mul(su[0], Hd[0]))), dacc[3]);
            dacc[4] = ds_add(dacc[4], su[0]);
            dacc[5] = ds_add(dacc[5], su[1]);
            dacc[6] = ds_add(dacc[6], su[2]);
        }
        t1 = t0;  // the FP64 tet loop below has nothing left to do
        dsf dtri = {0.f, 0.f};
        if (tri_ds) {
            // the surface demag term of the triangles (no surface anisotropy) in double-single:
            // per triangle the normal and the Gauss weights times 0.5 mu0 dMs as pairs
            for (int f = f0; f < f1; f += stride) {
                const int4 I = tri[f];
                const int ind[3] = {I.x, I.y, I.z};
                const float4 *q = tri_ds + 4 * (size_t)f;
                const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
                const dsf n[3] = {{q0.x, q0.y}, {q0.z, q0.w}, {q1.x, q1.y}};
                const dsf wq[4] = {{q1.z, q1.w}, {q2.x, q2.y}, {q2.z, q2.w}, {q3.x, q3.y}};
                dsf un[3][3], ph[3];
#pragma unroll
                for (int i = 0; i < 3; i++) {
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float2 a = uds[3 * (size_t)ind[i] + c];
                        un[i][c] = {a.x, a.y};
                    }
                    const float2 pp = pds[ind[i]];
                    ph[i] = {pp.x, pp.y};
                }
                dsf dm = {0.f, 0.f};
#pragma unroll
                for (int g = 0; g < NPF; g++) {
                    dsf U[3], pg = {0.f, 0.f};
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        U[c] = {0.f, 0.f};
#pragma unroll
                        for (int i = 0; i < 3; i++) U[c] = ds_fma(dsf{c_fa_ds[i][g].x, c_fa_ds[i][g].y}, un[i][c], U[c]);
                    }
#pragma unroll
                    for (int i = 0; i < 3; i++) pg = ds_fma(dsf{c_fa_ds[i][g].x, c_fa_ds[i][g].y}, ph[i], pg);
                    const dsf un_n = ds_fma(U[2], n[2], ds_fma(U[1], n[1], ds_mul(U[0], n[0])));
                    dm = ds_fma(ds_mul(un_n, pg), wq[g], dm);
                }
                dtri = ds_add(dtri, dm);
            }
            f1 = f0;  // the FP64 triangle loop below has nothing left to do
        }
        // block sums in double-single (warp shuffles of both words, then the warps' sums in a
        // fixed order), converted to FP64 once per block; the FP64 triangle loop's sums (with
        // surface anisotropy) follow in acc
        __shared__ dsf wsum[8][32];
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        dsf v8[8] = {dacc[0], dacc[1], dacc[2], dacc[3], dacc[4], dacc[5], dacc[6], dtri};
#pragma unroll
        for (int q = 0; q < 8; q++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
                v8[q] = ds_add(v8[q], dsf{__shfl_xor_sync(0xffffffffu, v8[q].h, o),
                                          __shfl_xor_sync(0xffffffffu, v8[q].l, o)});
            if (lane == 0) wsum[q][warp] = v8[q];
        }
        __syncthreads();
        if (threadIdx.x < 8) {
            dsf t = {0.f, 0.f};
            for (int w = 0; w < nw; w++) t = ds_add(t, wsum[threadIdx.x][w]);
            wsum[threadIdx.x][0] = t;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
#pragma unroll
            for (int q = 0; q < 7; q++) acc[q] += ds_to(wsum[q][0]) * DS_SLOT_INV;
            acc[2] += ds_to(wsum[7][0]);
        }
        if (tri_ds) {  // no FP64 triangle loop (uniform over the block): thread 0 holds the sums
            if (threadIdx.x == 0)
#pragma unroll
                for (int q = 0; q < 7; q++) partial[q * gridDim.x + blockIdx.x] = acc[q];
            return;
        }
    }
    for (int k = t0; k < t1; k += stride) {
        const int4 I = tet[k];
        const int ind[4] = {I.x, I.y, I.z, I.w};
        const DevRegion &R = regs[treg[k]];
        double un[4][3], ph[4], d[4][3];
#pragma unroll
        for (int i = 0; i < 4; i++) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                un[i][c] = u[3 * (size_t)ind[i] + c];
                d[i][c] = da[(3 * i + c) * (size_t)nmt + k];
            }
            ph[i] = phi[ind[i]];
        }
        double dU[3][3];
#pragma unroll
        for (int kk = 0; kk < 3; kk++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < 4; i++) s += d[i][kk] * un[i][c];
                dU[kk][c] = s;
            }
        const double dens = dU[0][0] * dU[0][0] + dU[0][1] * dU[0][1] + dU[0][2] * dU[0][2] + dU[1][0] * dU[1][0] +
                            dU[1][1] * dU[1][1] + dU[1][2] * dU[1][2] + dU[2][0] * dU[2][0] +
                            dU[2][1] * dU[2][1] + dU[2][2] * dU[2][2];
        const double div = dU[0][0] + dU[1][1] + dU[2][2];
        const double J = detJ[k];
        if constexpr (ISO) {
            // no anisotropy: every Gauss-point sum is a fixed combination of nodal values,
            // sum_g w_g a_i(g) = J sum_g pds_g a_i(g) (the same sums, reassociated)
            double aw[4], vol = 0.0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                double c = 0.0;
#pragma unroll
                for (int g = 0; g < NPI; g++) c += c_tpds[g] * c_ta[i][g];
                aw[i] = J * c;
            }
#pragma unroll
            for (int g = 0; g < NPI; g++) vol += J * c_tpds[g];
            double su[3] = {0, 0, 0}, sp = 0.0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
#pragma unroll
                for (int c = 0; c < 3; c++) su[c] += aw[i] * un[i][c];
                sp += aw[i] * ph[i];
            }
            acc[0] += R.A * vol * dens;
            acc[2] += -0.5 * FG_MU0 * R.Ms * div * sp;
            acc[3] += -FG_MU0 * R.Ms * (su[0] * Hx + su[1] * Hy + su[2] * Hz);
            acc[4] += su[0];
            acc[5] += su[1];
            acc[6] += su[2];
            continue;
        }
        double ex = 0.0, dm = 0.0, an = 0.0, ze = 0.0, cub = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
#pragma unroll
        for (int g = 0; g < NPI; g++) {
            const double w = J * c_tpds[g];
            double U[3], pg = 0.0;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < 4; i++) s += c_ta[i][g] * un[i][c];
                U[c] = s;
            }
#pragma unroll
            for (int i = 0; i < 4; i++) pg += c_ta[i][g] * ph[i];
            ex += w * dens;
            dm += w * div * pg;
            if (R.K != 0.0) {
                const double a = R.uk[0] * U[0] + R.uk[1] * U[1] + R.uk[2] * U[2];
                an += w * a * a;
            }
            if (R.K3 != 0.0) {
                const double a0 = U[0] * R.ex[0] + U[1] * R.ex[1] + U[2] * R.ex[2];
                const double a1 = U[0] * R.ey[0] + U[1] * R.ey[1] + U[2] * R.ey[2];
                const double a2 = U[0] * R.ez[0] + U[1] * R.ez[1] + U[2] * R.ez[2];
                cub += w * ((a0 * a1) * (a0 * a1) + (a1 * a2) * (a1 * a2) + (a2 * a0) * (a2 * a0));
            }
            if (hsp) {  // Tet::zeemanEnergy with the space field (src/tetra.cpp:381-390)
                const double *F = hsp + 3 * ((size_t)k * NPI + g);
                ze += w * (U[0] * (Hx + amp * F[0]) + U[1] * (Hy + amp * F[1]) + U[2] * (Hz + amp * F[2]));
            } else {
                ze += w * (U[0] * Hx + U[1] * Hy + U[2] * Hz);
            }
            mx += w * U[0];
            my += w * U[1];
            mz += w * U[2];
        }
        acc[0] += R.A * ex;
        acc[1] += -R.K * an + R.K3 * cub;
        acc[2] += -0.5 * FG_MU0 * R.Ms * dm;
        acc[3] += -FG_MU0 * R.Ms * ze;
        acc[4] += mx;
        acc[5] += my;
        acc[6] += mz;
    }
    for (int f = f0; f < f1; f += stride) {
        const int4 I = tri[f];
        const int ind[3] = {I.x, I.y, I.z};
        const DevTri &T = tc[f];
        double an = 0.0, dm = 0.0;
#pragma unroll
        for (int g = 0; g < NPF; g++) {
            double U[3], pg = 0.0;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < 3; i++) s += c_fa[i][g] * u[3 * (size_t)ind[i] + c];
                U[c] = s;
            }
#pragma unroll
            for (int i = 0; i < 3; i++) pg += c_fa[i][g] * phi[ind[i]];
            if (T.Ks != 0.0) {
                const double a = U[0] * T.uk[0] + U[1] * T.uk[1] + U[2] * T.uk[2];
                an += T.w[g] * a * a;
            }
            dm += (U[0] * T.n[0] + U[1] * T.n[1] + U[2] * T.n[2]) * pg * T.w[g];
        }
        acc[1] += -T.Ks * an;
        acc[2] += 0.5 * FG_MU0 * T.dMs * dm;
    }
    block_store<7>(acc, partial, gridDim.x);
}

// Per-sample sums of the energy partials: one block per sample adds its blocks' partials.
__global__ void k_seg_energy_sum(int G, const int *__restrict__ seg_blk, const double *__restrict__ partial,
                                 double *__restrict__ out) {
    const int g = blockIdx.x;
    if (threadIdx.x < 7) {
        double s = 0.0;
        for (int b = seg_blk[g]; b < seg_blk[g + 1]; b++) s += partial[threadIdx.x * G + b];
        out[7 * g + threadIdx.x] = s;
    }
}

// Step parameters of a run: copy step *ctr of the schedule to the current parameters.
__global__ void k_select_params(int nseg, const SegPar *__restrict__ sched, const int *__restrict__ ctr,
                                SegPar *__restrict__ cur) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < nseg) cur[g] = sched[(size_t)(*ctr) * nseg + g];
}

__global__ void k_advance(int *ctr) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *ctr += 1;
}

// ---------------------------------------------------------------------------------
// launch wrappers

static inline int nblocks(long n, int b) { return (int)((n + b - 1) / b); }

void upload_rules(bool one_point) {
    double ta[4][5] = {{0}}, tp[5] = {0}, fa[3][4] = {{0}}, fp[4] = {0};
    if (one_point) {
        for (int i = 0; i < 4; i++) ta[i][0] = 0.25;
        tp[0] = 1.0 / 6.0;
        for (int i = 0; i < 3; i++) fa[i][0] = 1.0 / 3.0;
        fp[0] = 0.5;
    } else {
        const double A = 1. / 4., B = 1. / 6., C = 1. / 2., D = -2. / 15., E = 3. / 40.;
        const double u[5] = {A, B, B, B, C}, v[5] = {A, B, B, C, B}, w[5] = {A, B, C, B, B};
        const double p[5] = {D, E, E, E, E};
        for (int j = 0; j < 5; j++) {
            ta[0][j] = 1. - u[j] - v[j] - w[j];
            ta[1][j] = u[j];
            ta[2][j] = v[j];
            ta[3][j] = w[j];
            tp[j] = p[j];
        }
        const double fu[4] = {1 / 3., 1 / 5., 3 / 5., 1 / 5.}, fv[4] = {1 / 3., 1 / 5., 1 / 5., 3 / 5.};
        const double fpds[4] = {-27 / 96., 25 / 96., 25 / 96., 25 / 96.};
        for (int j = 0; j < 4; j++) {
            fa[0][j] = 1. - fu[j] - fv[j];
            fa[1][j] = fu[j];
            fa[2][j] = fv[j];
            fp[j] = fpds[j];
        }
    }
    cudaMemcpyToSymbol(c_ta, ta, sizeof(ta));
    cudaMemcpyToSymbol(c_tpds, tp, sizeof(tp));
    {
        float tp32[5];
        for (int j = 0; j < 5; j++) tp32[j] = (float)tp[j];
        cudaMemcpyToSymbol(c_tpds32, tp32, sizeof(tp32));
    }
    double cw[4][5] = {}, cws[4] = {}, tps = 0.0;
    for (int j = 0; j < 5; j++) tps += tp[j];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 5; j++) {
            cw[i][j] = ta[i][j] * tp[j];
            cws[i] += cw[i][j];
        }
    cudaMemcpyToSymbol(c_cw, cw, sizeof(cw));
    cudaMemcpyToSymbol(c_cws, cws, sizeof(cws));
    cudaMemcpyToSymbol(c_tps, &tps, sizeof(tps));
    {
        auto pair = [](double x) {
            const float h = (float)x;
            return make_float2(h, (float)(x - (double)h));
        };
        float2 cwd[4];
        for (int i = 0; i < 4; i++) cwd[i] = pair(cws[i]);
        const float2 tpd = pair(tps);
        cudaMemcpyToSymbol(c_cws_dsp, cwd, sizeof(cwd));
        cudaMemcpyToSymbol(c_tps_dsp, &tpd, sizeof(tpd));
    }
    upload_rules_ds(ta, tp);
    cudaMemcpyToSymbol(c_fa, fa, sizeof(fa));
    {
        float2 fad[3][4];
        for (int i = 0; i < 3; i++)
            for (int g = 0; g < 4; g++) {
                const float h = (float)fa[i][g];
                fad[i][g] = make_float2(h, (float)(fa[i][g] - (double)h));
            }
        cudaMemcpyToSymbol(c_fa_ds, fad, sizeof(fad));
        float fa32[3][4];
        for (int i = 0; i < 3; i++)
            for (int g = 0; g < 4; g++) fa32[i][g] = (float)fa[i][g];
        cudaMemcpyToSymbol(c_fa32, fa32, sizeof(fa32));
    }
    cudaMemcpyToSymbol(c_fpds, fp, sizeof(fp));
}

cudaError_t launch_tet(Ctx &c, double dt, const double H[3]) {
    if (use_elem_ds(c)) {  // FP32 + refinement, isotropic, no space field or drift (spin coupling included)
        if (c.tri_be && c.nft > 0) {
            if (c.npi_f == 4) k_tri_aniso<4><<<nblocks(c.nft, 128), 128, 0, c.stream>>>(c.nft, c.tri, c.tri_c, c.u[0], c.tri_be);
            else k_tri_aniso<1><<<nblocks(c.nft, 128), 128, 0, c.stream>>>(c.nft, c.tri, c.tri_c, c.u[0], c.tri_be);
        }
        return launch_tet_ds(c, dt, H);
    }
    if (c.tri_be && c.nft > 0) {  // surface anisotropy (only when some region has Ks != 0)
        if (c.npi_f == 4) k_tri_aniso<4><<<nblocks(c.nft, 128), 128, 0, c.stream>>>(c.nft, c.tri, c.tri_c, c.u[0], c.tri_be);
        else k_tri_aniso<1><<<nblocks(c.nft, 128), 128, 0, c.stream>>>(c.nft, c.tri, c.tri_c, c.u[0], c.tri_be);
    }
    if (c.nmt == 0) return cudaGetLastError();
    const int b = 128;
    if (!c.aniso && !drift_on(c)) {
        if (c.npi_t == 5)
            k_tet64_iso<5><<<nblocks(c.nmt, b), b, 0, c.stream>>>(c.nmt, c.tet, c.da, c.detJ, c.treg, c.regs, c.u[0],
                                                                   c.phi[0], c.phiv[0], dt, H[0], H[1], H[2], c.slot,
                                                                   c.tet_seg, c.batch ? c.seg_par : nullptr, c.hsp,
                                                                   c.field_amp, c.spin_s, c.v[0]);
        else
            k_tet64_iso<1><<<nblocks(c.nmt, b), b, 0, c.stream>>>(c.nmt, c.tet, c.da, c.detJ, c.treg, c.regs, c.u[0],
                                                                   c.phi[0], c.phiv[0], dt, H[0], H[1], H[2], c.slot,
                                                                   c.tet_seg, c.batch ? c.seg_par : nullptr, c.hsp,
                                                                   c.field_amp, c.spin_s, c.v[0]);
        return cudaGetLastError();
    }
    if (c.npi_t == 5)
        (drift_on(c) ? k_tet64<5, true> : k_tet64<5, false>)<<<nblocks(c.nmt, b), b, 0, c.stream>>>(
            c.nmt, c.tet, c.da, c.detJ, c.treg, c.regs, c.u[0], c.v[0], c.phi[0], c.phiv[0], dt, H[0], H[1], H[2],
            c.slot, c.tet_seg, c.batch ? c.seg_par : nullptr, c.hsp, c.field_amp, c.spin_s, c.drift_dir, c.drift_v);
    else
        (drift_on(c) ? k_tet64<1, true> : k_tet64<1, false>)<<<nblocks(c.nmt, b), b, 0, c.stream>>>(
            c.nmt, c.tet, c.da, c.detJ, c.treg, c.regs, c.u[0], c.v[0], c.phi[0], c.phiv[0], dt, H[0], H[1], H[2],
            c.slot, c.tet_seg, c.batch ? c.seg_par : nullptr, c.hsp, c.field_amp, c.spin_s, c.drift_dir, c.drift_v);
    return cudaGetLastError();
}

cudaError_t launch_node(Ctx &c, double angle) {
    const double cr = std::cos(angle), sr = std::sin(angle);
    double *bv = c.bv;
    const long n2 = 2L * c.nn;
    double *Minv = bv + 8 * n2;
    k_node64<<<nblocks(c.nn, 256), 256, 0, c.stream>>>(c.nn, c.inc_ptr, c.inc, c.slot, use_elem_ds(c) ? 1 : 0,
                                                        c.tinc_ptr, c.tinc, c.tri_be,
                                                        c.mag, c.Ainv, c.u[0], c.v[1],
                                                        cr, sr, c.ep, c.eq, c.Dl, c.rhs, c.x, Minv, c.W,
                                                        c.node_seg,
                                                        c.batch ? c.seg_par : nullptr, c.node_feat);
    return cudaGetLastError();
}

int bicg_seg_max_blocks(Ctx &c) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bicg64_seg, 256, 0);
    return std::max(1, per_sm) * c.nsm;
}

int bicg_grid_size(Ctx &c, bool mixed) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bicg64, 256, 0);
    (void)mixed;
    if (per_sm < 1) per_sm = 1;
    int g = per_sm * c.nsm;
    const int need = nblocks(c.nn, 256);
    if (need < g) g = need;
    if (g < 1) g = 1;
    return g;
}

cudaError_t launch_bicg64(Ctx &c, double dt, double prefactor) {
    const long n2 = 2L * c.nn;
    BicgArgs a;
    a.nn = c.nn;
    a.Sptr = c.Sptr; a.Scol = c.Scol; a.Sval = c.Sval;
    a.A = c.A; a.Dl = c.Dl; a.ep = c.ep; a.eq = c.eq; a.mag = c.mag;
    a.c0 = prefactor * FG_THETA * dt * FG_GAMMA0;
    a.b = c.rhs; a.x = c.x;
    double *bv = c.bv;
    a.r = bv; a.rt = bv + n2; a.p = bv + 2 * n2; a.v = bv + 3 * n2; a.s = bv + 4 * n2; a.t = bv + 5 * n2;
    a.phat = bv + 6 * n2; a.shat = bv + 7 * n2; a.Minv = bv + 8 * n2; a.W = c.W;
    a.partial = c.partial; a.bar = c.bar; a.res = c.dres;
    a.tol = c.opts.tol; a.maxiter = c.opts.max_iter;
    a.dt = dt; a.u0 = c.u[0]; a.u1 = c.u[1]; a.v1 = c.v[1];
    a.nseg = 1;
    a.seg_node = a.seg_blk = nullptr;
    a.seg = nullptr;
    a.acc = nullptr;
    a.step_ctr = nullptr;
    const bool multi = c.batch;
    if (multi) {
        a.nseg = c.nseg;
        a.seg_node = c.d_seg_node;
        a.seg_blk = c.d_seg_blk;
        a.seg = c.seg_par;
        a.acc = c.acc_active;
        a.step_ctr = c.step_ctr;
    }
    cudaError_t e = cudaMemsetAsync(c.bar, 0, sizeof(GridBar), c.stream);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(c.dres, 0, sizeof(SolveResult) * a.nseg, c.stream);
    if (e != cudaSuccess) return e;
    void *args[] = {&a};
    if (multi)
        return cudaLaunchCooperativeKernel((void *)k_bicg64_seg, dim3(c.seg_grid), dim3(256), args, 0, c.stream);
    return cudaLaunchCooperativeKernel((void *)k_bicg64, dim3(c.bicg_grid), dim3(256), args, 0, c.stream);
}

cudaError_t launch_apply(Ctx &c, double c0, const double *x, double *y) {
    k_tangent64<<<nblocks(c.nn, 256), 256, 0, c.stream>>>(c.nn, x, c.ep, c.eq, c.W);
    k_apply64<<<nblocks(c.nn, 256), 256, 0, c.stream>>>(c.nn, c.Sptr, c.Scol, c.Sval, c.W, c.ep, c.eq, c.A, c.Dl,
                                                         c.mag, c0, x, y);
    return cudaGetLastError();
}

cudaError_t launch_charges(Ctx &c, const double *m, int set) {
    const int n = c.nmt + c.nft;
    if (n == 0) return cudaSuccess;
    double *q = set ? c.src_q2 : c.src_q, *ts = set ? c.tri_slot2 : c.tri_slot;
    if (!q || !ts) return cudaErrorInvalidValue;
    if (c.npi_t == 5)
        k_charges<5, 4, 1><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs,
                                                                   c.tri, c.tri_c, m, m, c.src_dst, q, q, ts, ts);
    else
        k_charges<1, 1, 1><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs,
                                                                   c.tri, c.tri_c, m, m, c.src_dst, q, q, ts, ts);
    return cudaGetLastError();
}

cudaError_t launch_charges_pair(Ctx &c, const double *m, const double *v) {
    const int n = c.nmt + c.nft;
    if (n == 0) return cudaSuccess;
    if (!c.src_q2 || !c.tri_slot2) return cudaErrorInvalidValue;
    if (c.npi_t == 5)
        k_charges<5, 4, 2><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs,
                                                                   c.tri, c.tri_c, m, v, c.src_dst, c.src_q, c.src_q2,
                                                                   c.tri_slot, c.tri_slot2);
    else
        k_charges<1, 1, 2><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs,
                                                                   c.tri, c.tri_c, m, v, c.src_dst, c.src_q, c.src_q2,
                                                                   c.tri_slot, c.tri_slot2);
    return cudaGetLastError();
}

cudaError_t launch_p2p_direct(Ctx &c) {
    if (c.n_mag_nodes == 0) return cudaSuccess;
    k_p2p_direct64<<<nblocks(c.n_mag_nodes, 256), 256, 0, c.stream>>>(c.n_mag_nodes, c.mag_nodes, c.xyz, c.nsrc,
                                                                        c.src_xyz, c.src_q, c.pot);
    return cudaGetLastError();
}

cudaError_t launch_phi_final(Ctx &c, double *phi_out, int set, const double *base) {
    if (c.n_mag_nodes == 0) return cudaSuccess;
    const double *ts = set ? c.tri_slot2 : c.tri_slot, *pot = set ? c.pot2 : c.pot;
    if (!ts || !pot) return cudaErrorInvalidValue;
    k_phi_final<<<nblocks(c.n_mag_nodes, 256), 256, 0, c.stream>>>(c.n_mag_nodes, c.mag_nodes, c.tinc_ptr, c.tinc,
                                                                     ts, pot, base, phi_out);
    return cudaGetLastError();
}

cudaError_t launch_state_diff(Ctx &c) {
    if (!c.dstate32) return cudaErrorInvalidValue;
    const size_t n3 = 3 * (size_t)c.nn;
    k_state_diff<<<(unsigned)((n3 + 255) / 256), 256, 0, c.stream>>>(n3, c.u[1], c.u[0], c.v[1], c.v[0], c.dstate32);
    return cudaGetLastError();
}

cudaError_t launch_charges32(Ctx &c, int nq) {
    const int n = c.nmt + c.nft;
    if (n == 0) return cudaSuccess;
    if (!c.dstate32 || !c.src_qf || !c.src_dst || (c.nft > 0 && !c.tri32) || (nq == 2 && (!c.src_q2f || !c.tri_slot2)))
        return cudaErrorInvalidValue;
    const float *du = c.dstate32, *dv = c.dstate32 + 3 * (size_t)c.nn;
    if (nq == 2) {
        if (c.npi_t == 5)
            k_charges32<5, 4, 2><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da32, c.cq32, c.tri,
                                                                         c.tri32, du, dv, c.src_dst, c.src_qf,
                                                                         c.src_q2f, c.tri_slot, c.tri_slot2);
        else
            k_charges32<1, 1, 2><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da32, c.cq32, c.tri,
                                                                         c.tri32, du, dv, c.src_dst, c.src_qf,
                                                                         c.src_q2f, c.tri_slot, c.tri_slot2);
    } else {
        if (c.npi_t == 5)
            k_charges32<5, 4, 1><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da32, c.cq32, c.tri,
                                                                         c.tri32, du, du, c.src_dst, c.src_qf,
                                                                         c.src_qf, c.tri_slot, c.tri_slot);
        else
            k_charges32<1, 1, 1><<<nblocks(n, 128), 128, 0, c.stream>>>(c.nmt, c.nft, c.tet, c.da32, c.cq32, c.tri,
                                                                         c.tri32, du, du, c.src_dst, c.src_qf,
                                                                         c.src_qf, c.tri_slot, c.tri_slot);
    }
    return cudaGetLastError();
}

// The closed isotropic form needs a uniform applied field: a space field takes the
// Gauss-point form.
static bool energy_iso(const Ctx &c) { return !c.aniso && !c.hsp; }

cudaError_t launch_energy(Ctx &c, const double H[3]) { return launch_energy_into(c, H, c.epart); }

// Same reduction as launch_energy with the per-block partial sums written to a caller-given
// device buffer of at least 7 * c.epart_blocks doubles (used by fg_energy_noalloc).
cudaError_t launch_energy_into(Ctx &c, const double H[3], double *partial) {
    const int G = c.epart_blocks;
    // the double-single form of the FP32 + refinement path reads NEXT as double-single pairs
    const bool dsp = energy_iso(c) && use_elem_ds(c);
    if (dsp) {
        const cudaError_t e = launch_state_ds(c, c.u[1], c.phi[1], c.phiv[1]);
        if (e != cudaSuccess) return e;
    }
    const float2 *dda = dsp ? c.da_ds : nullptr;
    if (c.npi_t == 5)
        (energy_iso(c) ? k_energy<5, 4, true> : k_energy<5, 4, false>)<<<G, 256, 0, c.stream>>>(
            c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs, c.tri, c.tri_c, c.u[1], c.phi[1], H[0], H[1], H[2],
            partial, nullptr, nullptr, nullptr, c.hsp, c.field_amp, dda, c.J_ds, c.state_ds, c.nn,
            dsp ? c.tri_ds : nullptr);
    else
        (energy_iso(c) ? k_energy<1, 1, true> : k_energy<1, 1, false>)<<<G, 256, 0, c.stream>>>(
            c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs, c.tri, c.tri_c, c.u[1], c.phi[1], H[0], H[1], H[2],
            partial, nullptr, nullptr, nullptr, c.hsp, c.field_amp, dda, c.J_ds, c.state_ds, c.nn,
            dsp ? c.tri_ds : nullptr);
    return cudaGetLastError();
}

// Per-sample energies of a batch: blocks aligned to samples, then one sum per sample.
cudaError_t launch_energy_seg(Ctx &c) {
    const int G = c.eblk_n;
    const double H0[3] = {0, 0, 0};
    if (c.npi_t == 5)
        (c.aniso ? k_energy<5, 4, false> : k_energy<5, 4, true>)<<<G, 256, 0, c.stream>>>(
            c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs, c.tri, c.tri_c,
                                                 c.u[1], c.phi[1], H0[0], H0[1], H0[2], c.seg_epart, c.eblk_rng,
                                                 c.eblk_seg, c.seg_H, nullptr, 0.0, nullptr, nullptr, nullptr, 0, nullptr);
    else
        (c.aniso ? k_energy<1, 1, false> : k_energy<1, 1, true>)<<<G, 256, 0, c.stream>>>(
            c.nmt, c.nft, c.tet, c.da, c.detJ, c.treg, c.regs, c.tri, c.tri_c,
                                                 c.u[1], c.phi[1], H0[0], H0[1], H0[2], c.seg_epart, c.eblk_rng,
                                                 c.eblk_seg, c.seg_H, nullptr, 0.0, nullptr, nullptr, nullptr, 0, nullptr);
    k_seg_energy_sum<<<c.nseg, 32, 0, c.stream>>>(G, c.d_seg_eblk, c.seg_epart, c.seg_energy);
    return cudaGetLastError();
}

cudaError_t launch_select_params(Ctx &c) {
    k_select_params<<<nblocks(c.nseg, 128), 128, 0, c.stream>>>(c.nseg, c.seg_sched, c.step_ctr, c.seg_par);
    return cudaGetLastError();
}

cudaError_t launch_advance(Ctx &c) {
    k_advance<<<1, 32, 0, c.stream>>>(c.step_ctr);
    return cudaGetLastError();
}

}  // namespace fg
