// Element integrals of the FP32 + refinement path in double-single arithmetic.
//
// The same closed isotropic form as k_tet64_iso (Tet::integrales without anisotropy,
// src/tetra.cpp:210-307), every quantity as a double-single value (about 48 bits): GB300's
// FP64 pipe runs at 1/64 of its FP32 rate and bounded the FP64 kernel. The slots come out as
// double-single pairs scaled by 2^70 (the Jacobian is scaled on the host, so that products of
// tet volumes ~1e-27 keep their low words normal in FP32); the node kernel sums them in
// double-single and converts each node's sums to FP64 once. The assembled system then
// agrees with the FP64 path's to ~1e-14 relative, far below the solver tolerance. Used when
// there is no anisotropy or space field (those keep the FP64 kernels), with the spin
// accumulation's Hst terms (src/tetra.cpp:248-303) in the same arithmetic when the coupling
// is on; batches read each tet's dt and field from its sample.
#include <cmath>

#include "fg_ds.cuh"
#include "fg_internal.h"

namespace fg {

__constant__ float2 c_ta_ds[4][5];  // shape functions at the Gauss points
__constant__ float2 c_cw_ds[4][5];  // a_i(g) pds_g
__constant__ float2 c_cws_ds[4];    // sum_g a_i(g) pds_g
__constant__ float2 c_tps_ds;       // sum_g pds_g

namespace {

__device__ __forceinline__ dsf ld2(const float2 *p, size_t k) {
    const float2 v = p[k];
    return {v.x, v.y};
}
__device__ __forceinline__ dsf cs(float2 v) { return {v.x, v.y}; }

// CURRENT u, phi, phiv of every node as double-single (read by ~24 tets each); with s0 set
// also the spin accumulation s and the velocity v of CURRENT (the spin coupling's terms)
__global__ void k_state_ds(int nn, const double *__restrict__ u0, const double *__restrict__ phi0,
                           const double *__restrict__ phiv0, float2 *__restrict__ uds, float2 *__restrict__ phids,
                           float2 *__restrict__ phivds, const double *__restrict__ s0, const double *__restrict__ v0,
                           float2 *__restrict__ sds, float2 *__restrict__ vds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const dsf v = ds_from(u0[3 * (size_t)i + c]);
        uds[3 * (size_t)i + c] = make_float2(v.h, v.l);
    }
    const dsf p = ds_from(phi0[i]), q = ds_from(phiv0[i]);
    phids[i] = make_float2(p.h, p.l);
    phivds[i] = make_float2(q.h, q.l);
    if (s0) {
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const dsf a = ds_from(s0[3 * (size_t)i + c]), b = ds_from(v0[3 * (size_t)i + c]);
            sds[3 * (size_t)i + c] = make_float2(a.h, a.l);
            vds[3 * (size_t)i + c] = make_float2(b.h, b.l);
        }
    }
}

// SPIN: the spin coupling (single contexts only): Hst(g) = hst sum_i a_i(g) s_i adds U(g).Hst(g)
// to uHeff(g) and sum_g w_g a_i(g) (Hst(g) - (Hst(g).U(g)) s_dt V(g)) to BE_i, s_dt = theta dt
// gamma0 (sdt2), from the double-single s and v of CURRENT (sds, vds).
template <int NPI, bool SPIN>
__global__ void __launch_bounds__(128) k_tet_ds(int nmt, const int4 *__restrict__ tet, const float2 *__restrict__ da,
                                                const float2 *__restrict__ Js, const int *__restrict__ treg,
                                                const DevRegion *__restrict__ regs, const float2 *__restrict__ uds,
                                                const float2 *__restrict__ phids, const float2 *__restrict__ phivds,
                                                float2 Hx2, float2 Hy2, float2 Hz2, float2 rdt2, float2 kv2,
                                                float4 *__restrict__ slot, const int *__restrict__ tet_seg,
                                                const SegPar *__restrict__ seg, const float2 *__restrict__ sds,
                                                const float2 *__restrict__ vds, float2 sdt2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nmt) return;
    if (seg) {  // batch: the tet's sample carries dt and the applied field (pairs formed on the host)
        const SegPar &P = seg[tet_seg[t]];
        Hx2 = P.H_ds[0];
        Hy2 = P.H_ds[1];
        Hz2 = P.H_ds[2];
        rdt2 = P.rdt_ds;
        kv2 = P.kv_ds;
    }
    const int4 I = tet[t];
    const int ind[4] = {I.x, I.y, I.z, I.w};
    dsf d[4][3];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) d[i][k] = ld2(da, (3 * i + k) * (size_t)nmt + t);
    const dsf J = ld2(Js, t);
    const DevRegion &R = regs[treg[t]];
    const dsf Abis = {R.Abis_ds.x, R.Abis_ds.y}, alpha = {R.alpha_ds.x, R.alpha_ds.y};
    dsf un[4][3], ph[4], phv[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
#pragma unroll
        for (int c = 0; c < 3; c++) un[i][c] = ld2(uds, 3 * (size_t)ind[i] + c);
        ph[i] = ld2(phids, ind[i]);
        phv[i] = ld2(phivds, ind[i]);
    }
    dsf dU[3][3], Hd[3], Hv[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int c = 0; c < 3; c++)
            dU[k][c] = ds_fma(d[3][k], un[3][c], ds_fma(d[2][k], un[2][c], ds_fma(d[1][k], un[1][c], ds_mul(d[0][k], un[0][c]))));
#pragma unroll
    for (int c = 0; c < 3; c++) {
        Hd[c] = ds_neg(ds_fma(ph[3], d[3][c], ds_fma(ph[2], d[2][c], ds_fma(ph[1], d[1][c], ds_mul(ph[0], d[0][c])))));
        Hv[c] = ds_neg(ds_fma(phv[3], d[3][c], ds_fma(phv[2], d[2][c], ds_fma(phv[1], d[1][c], ds_mul(phv[0], d[0][c])))));
    }
    dsf gradsq = {0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
        for (int c = 0; c < 3; c++) gradsq = ds_fma(dU[k][c], dU[k][c], gradsq);
    const dsf He[3] = {ds_add(Hd[0], {Hx2.x, Hx2.y}), ds_add(Hd[1], {Hy2.x, Hy2.y}), ds_add(Hd[2], {Hz2.x, Hz2.y})};
    dsf uh[4];
#pragma unroll
    for (int i = 0; i < 4; i++) uh[i] = ds_fma(un[i][2], He[2], ds_fma(un[i][1], He[1], ds_mul(un[i][0], He[0])));
    // calc_alpha_eff (src/tetra.cpp:47-75) with M = 2 alpha 0.1 / reduced_dt
    const dsf rdt = {rdt2.x, rdt2.y};
    const dsf two_alpha = {2.f * alpha.h, 2.f * alpha.l};
    const dsf M = ds_div(ds_mul(two_alpha, ds_make(0.1f, -1.4901161e-09f)), rdt);
    const dsf k2 = ds_div(rdt, two_alpha);
    const dsf half_rdt = {0.5f * rdt.h, 0.5f * rdt.l};
    const dsf hx = ds_neg(ds_mul(Abis, gradsq));
    const dsf one = {1.f, 0.f};
    dsf contrib[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    // spin coupling: hst s and v at the vertices, and the per-vertex sums of its BE term
    const bool spin = SPIN && (R.hst_ds.x != 0.f || R.hst_ds.y != 0.f);
    dsf sn[4][3], vn[4][3], sw[4][3];
    if constexpr (SPIN) {
        const dsf hst = cs(R.hst_ds);
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                sw[i][c] = {0.f, 0.f};
                sn[i][c] = spin ? ds_mul(hst, ld2(sds, 3 * (size_t)ind[i] + c)) : dsf{0.f, 0.f};
                vn[i][c] = spin ? ld2(vds, 3 * (size_t)ind[i] + c) : dsf{0.f, 0.f};
            }
    }
    const dsf sdt = {sdt2.x, sdt2.y};
#pragma unroll
    for (int g = 0; g < NPI; g++) {
        dsf h = hx;
#pragma unroll
        for (int i = 0; i < 4; i++) h = ds_fma(cs(c_ta_ds[i][g]), uh[i], h);
        if constexpr (SPIN) {
            if (spin) {
                const dsf t0 = cs(c_ta_ds[0][g]), t1 = cs(c_ta_ds[1][g]), t2 = cs(c_ta_ds[2][g]),
                          t3 = cs(c_ta_ds[3][g]);
                dsf U[3], Hs[3], Vg[3];
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    U[c] = ds_fma(t3, un[3][c], ds_fma(t2, un[2][c], ds_fma(t1, un[1][c], ds_mul(t0, un[0][c]))));
                    Hs[c] = ds_fma(sn[3][c], t3, ds_fma(sn[2][c], t2, ds_fma(sn[1][c], t1, ds_mul(sn[0][c], t0))));
                    Vg[c] = ds_fma(t3, vn[3][c], ds_fma(t2, vn[2][c], ds_fma(t1, vn[1][c], ds_mul(t0, vn[0][c]))));
                }
                const dsf hu = ds_fma(Hs[2], U[2], ds_fma(Hs[1], U[1], ds_mul(Hs[0], U[0])));
                h = ds_add(h, hu);
                const dsf hs = ds_mul(hu, sdt);
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    const dsf e = ds_sub(Hs[c], ds_mul(hs, Vg[c]));
#pragma unroll
                    for (int i = 0; i < 4; i++) sw[i][c] = ds_fma(cs(c_cw_ds[i][g]), e, sw[i][c]);
                }
            }
        }
        dsf a;
        if (h.h > 0.f) {
            a = ds_fma(half_rdt, ds_gt(h, M) ? M : h, alpha);
        } else {
            const dsf mM = ds_neg(M);
            a = ds_div(alpha, ds_sub(one, ds_mul(k2, ds_gt(mM, h) ? mM : h)));
        }
#pragma unroll
        for (int i = 0; i < 4; i++) contrib[i] = ds_fma(cs(c_cw_ds[i][g]), a, contrib[i]);
    }
    const dsf vol = ds_mul(J, cs(c_tps_ds)), nva = ds_neg(ds_mul(vol, Abis));
    const dsf kv = {kv2.x, kv2.y};
    const dsf H[3] = {ds_fma(kv, Hv[0], He[0]), ds_fma(kv, Hv[1], He[1]), ds_fma(kv, Hv[2], He[2])};
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const dsf aw = ds_mul(J, cs(c_cws_ds[i]));
        dsf BE[3];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const dsf ex = ds_fma(d[i][2], dU[2][c], ds_fma(d[i][1], dU[1][c], ds_mul(d[i][0], dU[0][c])));
            BE[c] = ds_fma(nva, ex, ds_mul(aw, H[c]));
            if constexpr (SPIN) {
                if (spin) BE[c] = ds_fma(J, sw[i][c], BE[c]);
            }
        }
        const dsf ct = ds_mul(J, contrib[i]);
        slot[2 * (4 * (size_t)t + i)] = make_float4(ct.h, BE[0].h, BE[1].h, BE[2].h);
        slot[2 * (4 * (size_t)t + i) + 1] = make_float4(ct.l, BE[0].l, BE[1].l, BE[2].l);
    }
}

inline float2 split(double x) {
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

}  // namespace

void upload_rules_ds(const double ta[4][5], const double tp[5]) {
    float2 t[4][5], w[4][5], ws[4], ps;
    double tps = 0.0;
    for (int j = 0; j < 5; j++) tps += tp[j];
    for (int i = 0; i < 4; i++) {
        double s = 0.0;
        for (int j = 0; j < 5; j++) {
            t[i][j] = split(ta[i][j]);
            w[i][j] = split(ta[i][j] * tp[j]);
            s += ta[i][j] * tp[j];
        }
        ws[i] = split(s);
    }
    ps = split(tps);
    cudaMemcpyToSymbol(c_ta_ds, t, sizeof(t));
    cudaMemcpyToSymbol(c_cw_ds, w, sizeof(w));
    cudaMemcpyToSymbol(c_cws_ds, ws, sizeof(ws));
    cudaMemcpyToSymbol(c_tps_ds, &ps, sizeof(ps));
}

// Host: double-single copies of the static geometry (da, and detJ scaled by 2^70).
int elem_ds_setup(Ctx &c, const std::vector<double> &da, const std::vector<double> &detJ) {
    const size_t n = detJ.size();
    std::vector<float2> dd(da.size()), jj(n);
    for (size_t k = 0; k < da.size(); k++) dd[k] = split(da[k]);
    for (size_t k = 0; k < n; k++) jj[k] = split(std::ldexp(detJ[k], DS_SLOT_SCALE));
    if (cudaMalloc(&c.da_ds, sizeof(float2) * std::max<size_t>(1, dd.size())) != cudaSuccess ||
        cudaMalloc(&c.J_ds, sizeof(float2) * std::max<size_t>(1, n)) != cudaSuccess ||
        cudaMalloc(&c.state_ds, sizeof(float2) * (c.opts.spin_acc ? 11 : 5) * std::max(1, c.nn)) != cudaSuccess)
        return FG_ECUDA;
    if (cudaMemcpy(c.da_ds, dd.data(), sizeof(float2) * dd.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(c.J_ds, jj.data(), sizeof(float2) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        return FG_ECUDA;
    return FG_OK;
}

cudaError_t launch_state_ds(Ctx &c, const double *u, const double *phi, const double *phiv) {
    float2 *uds = c.state_ds, *phids = uds + 3 * (size_t)c.nn, *phivds = phids + c.nn;
    k_state_ds<<<(c.nn + 255) / 256, 256, 0, c.stream>>>(c.nn, u, phi, phiv, uds, phids, phivds, nullptr, nullptr,
                                                          nullptr, nullptr);
    return cudaGetLastError();
}

cudaError_t launch_tet_ds(Ctx &c, double dt, const double H[3]) {
    if (c.nmt == 0) return cudaSuccess;
    float2 *uds = c.state_ds, *phids = uds + 3 * (size_t)c.nn, *phivds = phids + c.nn;
    // with the spin coupling the buffer also holds s and v of CURRENT (allocated for it)
    const bool spin = c.spin_s != nullptr;
    float2 *sds = phivds + c.nn, *vds = sds + 3 * (size_t)c.nn;
    cudaError_t e;
    if (spin) {
        k_state_ds<<<(c.nn + 255) / 256, 256, 0, c.stream>>>(c.nn, c.u[0], c.phi[0], c.phiv[0], uds, phids, phivds,
                                                              c.spin_s, c.v[0], sds, vds);
        e = cudaGetLastError();
    } else {
        e = launch_state_ds(c, c.u[0], c.phi[0], c.phiv[0]);
    }
    if (e != cudaSuccess) return e;
    const float2 hx = split(H[0]), hy = split(H[1]), hz = split(H[2]);
    const float2 rdt = split(FG_GAMMA0 * dt), kv = split(FG_THETA * dt), sdt = split(FG_THETA * dt * FG_GAMMA0);
    float4 *slot = reinterpret_cast<float4 *>(c.slot);
    const int b = 128, g = (c.nmt + b - 1) / b;
    auto k = c.npi_t == 5 ? (spin ? k_tet_ds<5, true> : k_tet_ds<5, false>)
                          : (spin ? k_tet_ds<1, true> : k_tet_ds<1, false>);
    k<<<g, b, 0, c.stream>>>(c.nmt, c.tet, c.da_ds, c.J_ds, c.treg, c.regs, uds, phids, phivds, hx, hy, hz, rdt, kv,
                             slot, c.tet_seg, c.batch ? c.seg_par : nullptr, spin ? sds : nullptr,
                             spin ? vds : nullptr, sdt);
    return cudaGetLastError();
}

}  // namespace fg
