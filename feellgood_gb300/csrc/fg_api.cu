// C ABI of the fggpu library: context construction (once per mesh), state transfer and
// the per-step orchestration of the device kernels. No function exits the process and
// no exception crosses the ABI.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "fg_internal.h"

namespace fg {
void upload_rules(bool one_point);
int fmm_build(Ctx &c);
void fmm_free(Ctx &c);
}  // namespace fg

using namespace fg;

static thread_local std::string g_create_error;

#define CK(call)                                                                      \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess) {                                                      \
            c.err = std::string(#call) + ": " + cudaGetErrorString(e_);               \
            return FG_ECUDA;                                                          \
        }                                                                             \
    } while (0)

template <typename T>
static cudaError_t dalloc(T **p, size_t n) {
    if (n == 0) n = 1;
    return cudaMalloc((void **)p, n * sizeof(T));
}
template <typename T>
static cudaError_t upload(T **p, const std::vector<T> &h) {
    cudaError_t e = dalloc(p, h.size());
    if (e != cudaSuccess) return e;
    if (!h.empty()) e = cudaMemcpy(*p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e;
}

namespace fg {
Rules make_rules(bool one) {
    Rules r{};
    if (one) {
        r.npi_t = 1;
        r.npi_f = 1;
        for (int i = 0; i < 4; i++) r.ta[i][0] = 0.25;
        r.tp[0] = 1.0 / 6.0;
        for (int i = 0; i < 3; i++) r.fa[i][0] = 1.0 / 3.0;
        r.fp[0] = 0.5;
    } else {
        r.npi_t = 5;
        r.npi_f = 4;
        const double A = 1. / 4., B = 1. / 6., C = 1. / 2., D = -2. / 15., E = 3. / 40.;
        const double u[5] = {A, B, B, B, C}, v[5] = {A, B, B, C, B}, w[5] = {A, B, C, B, B};
        const double p[5] = {D, E, E, E, E};
        for (int j = 0; j < 5; j++) {
            r.ta[0][j] = 1. - u[j] - v[j] - w[j];
            r.ta[1][j] = u[j];
            r.ta[2][j] = v[j];
            r.ta[3][j] = w[j];
            r.tp[j] = p[j];
        }
        const double fu[4] = {1 / 3., 1 / 5., 3 / 5., 1 / 5.}, fv[4] = {1 / 3., 1 / 5., 1 / 5., 3 / 5.};
        const double fpds[4] = {-27 / 96., 25 / 96., 25 / 96., 25 / 96.};
        for (int j = 0; j < 4; j++) {
            r.fa[0][j] = 1. - fu[j] - fv[j];
            r.fa[1][j] = fu[j];
            r.fa[2][j] = fv[j];
            r.fp[j] = fpds[j];
        }
    }
    return r;
}
}  // namespace fg

namespace {

struct P3 {
    double x, y, z;
};
inline P3 sub(P3 a, P3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot3(P3 a, P3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline P3 cross3(P3 a, P3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double nrm(P3 a) { return std::sqrt(dot3(a, a)); }

// Tri::potential geometry (src/triangle.cpp:87-125): coefficients of s_i, s_{i+1}, s_{i+2}.
void tri_potential_coeffs(P3 p1, P3 p2, P3 p3, double surf, double out[3]) {
    P3 p1p2 = sub(p2, p1), p1p3 = sub(p3, p1);
    auto f = [](double x) { return std::sqrt(1.0 + x * x); };
    double b = nrm(p1p2);
    double t = dot3(p1p2, p1p3) / b;
    double _2s = 2. * surf;
    double h = _2s / b;
    double c = (t - b) / h;
    double r = h * f(t / h);
    double log_1 = std::log((c * t + h + f(c) * r) / (b * (c + f(c))));
    double xi = b * log_1 / f(c);
    double den = b / (_2s * (1 + c * c));
    out[0] = xi;
    out[1] = (xi * (h + c * t) - b * (r - b)) * den;
    out[2] = b * (r - b - c * xi) * den;
}

}  // namespace

extern "C" {

void fg_opts_default(fg_opts *o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->tol = 1e-6;
    o->max_iter = 700;
    o->precision = FG_PREC_FP64;
    o->learned_guess = 0;
    o->demag = FG_DEMAG_AUTO;
    o->fmm_order = 0;
    o->fmm_leaf = 0;
    o->one_gauss_point = 0;
    o->first_order = 0;
    o->refine_max = 20;
    o->inner_tol = 1e-5;
    o->verbose = 0;
    o->mlp_train_steps = 20;
    o->mlp_batch = 16384;
    o->mlp_lr = 1e-3;
    o->fmm_tensor = 1;
    o->mlp_train_every = 1;
    o->spin_tol = 1e-8;        // spinAcc and electrostatSolver tolerance (src/main.cpp:252)
    o->spin_max_iter = 1000;
    o->demag_increment = 1;
    o->fmm_overlap = 0;
    o->fmm_tree_host = 0;
    o->solver_threads = 0;
}

const char *fg_strerror(int s) {
    switch (s) {
        case FG_OK: return "ok";
        case FG_SOLVER_ITER_OVERFLOW: return "solver: iteration overflow";
        case FG_SOLVER_CANNOT_CONVERGE: return "solver: cannot converge";
        case FG_ETIMEDOUT: return "bounded device wait timed out";
        case FG_EINVAL: return "invalid argument";
        case FG_ECUDA: return "CUDA error";
        case FG_ENOMEM: return "out of memory";
        case FG_EMESH: return "invalid mesh";
        case FG_EIO: return "I/O error";
        default: return "unknown status";
    }
}

const char *fg_last_error(const fg_ctx *ctx) { return ctx ? ctx->c.err.c_str() : g_create_error.c_str(); }

static int create_impl(fg_ctx *h, const fg_mesh *m, const fg_region *regs, int nreg, const fg_tri_region *tregs,
                       int ntreg, const fg_opts *opts) {
    Ctx &c = h->c;
    if (opts) c.opts = *opts; else fg_opts_default(&c.opts);
    if (c.batch) {
        // a batch runs the FP32 + refinement or the FP64 solver and a forest FMM (one tree
        // per sample); the learned guess (one network for all samples, judged per sample
        // inside the FP32 + refinement solver) with the FP32 + refinement solver only
        if ((c.opts.precision != FG_PREC_FP32_REFINE && c.opts.precision != FG_PREC_FP64) ||
            (c.opts.learned_guess && c.opts.precision != FG_PREC_FP32_REFINE) || c.opts.demag == FG_DEMAG_DIRECT) {
            c.err = "fg_batch_create: a batch needs precision FG_PREC_FP32_REFINE (with or without the learned guess) "
                    "or FG_PREC_FP64, and demag FMM";
            return FG_EINVAL;
        }
        if (c.opts.spin_acc) {
            c.err = "fg_batch_create: spin accumulation is not available for batches";
            return FG_EINVAL;
        }
        c.opts.demag = FG_DEMAG_FMM;
        c.opts.profile = 0;
    }
    if (c.opts.solver_threads != 0 && c.opts.solver_threads != 256 && c.opts.solver_threads != 512) {
        c.err = "fg_create: solver_threads must be 0, 256 or 512";
        return FG_EINVAL;
    }
    if (!m || !regs || nreg <= 0 || m->n_nodes <= 0 || m->n_tets <= 0 || !m->xyz || !m->tet4 || !m->tet_region) {
        c.err = "fg_create: missing mesh or region data";
        return FG_EINVAL;
    }
    if (m->n_tris > 0 && (!m->tri3 || !m->tri_region || !m->tri_dMs || !tregs || ntreg <= 0)) {
        c.err = "fg_create: triangles given without their regions";
        return FG_EINVAL;
    }
    const Rules R = make_rules(c.opts.one_gauss_point != 0);
    c.npi_t = R.npi_t;
    c.npi_f = R.npi_f;
    const int nn = m->n_nodes;
    c.nn = nn;
    c.n_tets_total = m->n_tets;
    CK(cudaGetDevice(&c.device));
    cudaDeviceProp prop;
    CK(cudaGetDeviceProperties(&prop, c.device));
    c.nsm = prop.multiProcessorCount;
    {
        // the near field of the FMM runs on a second stream of lower priority, so that the
        // far-field chain's blocks go first where both wait for an SM
        int least = 0, greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CK(cudaStreamCreateWithPriority(&c.stream, cudaStreamNonBlocking, greatest));
        CK(cudaStreamCreateWithPriority(&c.stream2, cudaStreamNonBlocking, least));
        CK(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming));
    }
    for (int k = 0; k < 8; k++) CK(cudaEventCreate(&c.ev[k]));
    upload_rules(c.opts.one_gauss_point != 0);

    // region table
    std::vector<DevRegion> hreg(nreg);
    for (int r = 0; r < nreg; r++) {
        const fg_region &g = regs[r];
        DevRegion &d = hreg[r];
        std::memset(&d, 0, sizeof(d));
        d.A = g.Ae; d.Ms = g.Ms; d.alpha = g.alpha; d.K = g.K; d.K3 = g.K3;
        if (g.Ms > 0) {
            if (g.K != 0.0 || g.K3 != 0.0) c.aniso = true;
            c.ms_ref = std::max(c.ms_ref == 1.0 ? 0.0 : c.ms_ref, g.Ms);
            d.Abis = 2.0 * g.Ae / (FG_MU0 * g.Ms);
            const float ah = (float)d.Abis, lh = (float)g.alpha;
            d.Abis_ds = make_float2(ah, (float)(d.Abis - (double)ah));
            d.alpha_ds = make_float2(lh, (float)(g.alpha - (double)lh));
            d.Kbis = 2.0 * g.K / (FG_MU0 * g.Ms);
            d.K3bis = 2.0 * g.K3 / (FG_MU0 * g.Ms);
        }
        for (int k = 0; k < 3; k++) {
            d.uk[k] = g.uk[k]; d.ex[k] = g.ex[k]; d.ey[k] = g.ey[k]; d.ez[k] = g.ez[k];
        }
        auto pair = [](double x) {
            const float h = (float)x;
            return make_float2(h, (float)(x - (double)h));
        };
        d.A_ds = pair(g.Ae);
        d.edm_ds = pair(-0.5 * FG_MU0 * g.Ms);
        d.ez_ds = pair(-FG_MU0 * g.Ms);
    }
    // magnetic tetrahedra and nodes (src/mesh.h:115-131)
    std::vector<unsigned char> mag(nn, 0);
    std::vector<int> mtets;
    for (int t = 0; t < m->n_tets; t++) {
        const int r = m->tet_region[t];
        if (r < 0 || r >= nreg) { c.err = "fg_create: tet region out of range"; return FG_EINVAL; }
        for (int i = 0; i < 4; i++) {
            const int v = m->tet4[4 * t + i];
            if (v < 0 || v >= nn) { c.err = "fg_create: tet node index out of range"; return FG_EMESH; }
        }
        if (regs[r].Ms > 0) {
            mtets.push_back(t);
            for (int i = 0; i < 4; i++) mag[m->tet4[4 * t + i]] = 1;
        }
    }
    c.h_mag = mag;
    c.h_xyz.assign(m->xyz, m->xyz + 3 * (size_t)nn);
    const int nmt = (int)mtets.size();
    c.nmt = nmt;
    auto P = [&](int i) { return P3{m->xyz[3 * i], m->xyz[3 * i + 1], m->xyz[3 * i + 2]}; };

    // per-tet geometry: da = dadu inv(J), detJ (src/tetra.h:140-163)
    std::vector<double> da(12 * (size_t)nmt), detJ(nmt);
    std::vector<int4> htet(nmt);
    std::vector<int> htreg(nmt);
    std::vector<double> A(nn, 0.0);
    for (int k = 0; k < nmt; k++) {
        const int t = mtets[k];
        const int *ind = &m->tet4[4 * t];
        htet[k] = make_int4(ind[0], ind[1], ind[2], ind[3]);
        htreg[k] = m->tet_region[t];
        P3 p0 = P(ind[0]);
        P3 a = sub(P(ind[1]), p0), b = sub(P(ind[2]), p0), cc = sub(P(ind[3]), p0);
        double J[3][3] = {{a.x, b.x, cc.x}, {a.y, b.y, cc.y}, {a.z, b.z, cc.z}};
        double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                     J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        if (!(det > 0)) {
            c.err = "fg_create: tetrahedron " + std::to_string(t) + " is flat or not positively oriented";
            return FG_EMESH;
        }
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
                da[(3 * i + q) * (size_t)nmt + k] = s;
            }
        detJ[k] = det;
        for (int i = 0; i < 4; i++) {
            double aw = 0;
            for (int g = 0; g < R.npi_t; g++) aw += R.ta[i][g] * (det * R.tp[g]);
            A[ind[i]] += aw;
        }
        for (int g = 0; g < R.npi_t; g++) c.total_mag_vol += det * R.tp[g];
    }
    // static stiffness S_ij = sum_t Abis vol (da_i . da_j) on the node graph (with diagonal)
    std::vector<std::vector<int>> nb(nn);
    for (int k = 0; k < nmt; k++) {
        const int4 I = htet[k];
        const int ind[4] = {I.x, I.y, I.z, I.w};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) nb[ind[i]].push_back(ind[j]);
    }
    std::vector<int> Sptr(nn + 1, 0);
    for (int i = 0; i < nn; i++) {
        auto &v = nb[i];
        v.push_back(i);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        Sptr[i + 1] = Sptr[i] + (int)v.size();
    }
    c.nnzS = Sptr[nn];
    std::vector<int> Scol(c.nnzS);
    for (int i = 0; i < nn; i++) std::copy(nb[i].begin(), nb[i].end(), Scol.begin() + Sptr[i]);
    nb.clear();
    nb.shrink_to_fit();
    std::vector<double> Sval(c.nnzS, 0.0);
    for (int k = 0; k < nmt; k++) {
        const int4 I = htet[k];
        const int ind[4] = {I.x, I.y, I.z, I.w};
        const double Abis = hreg[htreg[k]].Abis;
        double wsum = 0;
        for (int g = 0; g < R.npi_t; g++) wsum += detJ[k] * R.tp[g];
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double dd = 0;
                for (int q = 0; q < 3; q++)
                    dd += da[(3 * i + q) * (size_t)nmt + k] * da[(3 * j + q) * (size_t)nmt + k];
                auto b0 = Scol.begin() + Sptr[ind[i]], e0 = Scol.begin() + Sptr[ind[i] + 1];
                auto it = std::lower_bound(b0, e0, ind[j]);
                Sval[it - Scol.begin()] += dd * (Abis * wsum);
            }
    }
    // node -> tet-vertex slots
    std::vector<int> inc_ptr(nn + 1, 0), inc(4 * (size_t)nmt);
    for (int k = 0; k < nmt; k++) {
        inc_ptr[htet[k].x + 1]++; inc_ptr[htet[k].y + 1]++; inc_ptr[htet[k].z + 1]++; inc_ptr[htet[k].w + 1]++;
    }
    for (int i = 0; i < nn; i++) inc_ptr[i + 1] += inc_ptr[i];
    {
        std::vector<int> fill(inc_ptr.begin(), inc_ptr.end() - 1);
        for (int k = 0; k < nmt; k++) {
            const int ind[4] = {htet[k].x, htet[k].y, htet[k].z, htet[k].w};
            for (int i = 0; i < 4; i++) inc[fill[ind[i]]++] = 4 * k + i;
        }
    }
    // magnetic triangles (src/mesh.h:127-131) and their charge/correction constants
    std::vector<int4> htri;
    std::vector<DevTri> htc;
    for (int f = 0; f < m->n_tris; f++) {
        const int *ind = &m->tri3[3 * f];
        const int r = m->tri_region[f];
        if (r < 0 || r >= ntreg) { c.err = "fg_create: triangle region out of range"; return FG_EINVAL; }
        for (int i = 0; i < 3; i++)
            if (ind[i] < 0 || ind[i] >= nn) { c.err = "fg_create: triangle node out of range"; return FG_EMESH; }
        if (!(mag[ind[0]] && mag[ind[1]] && mag[ind[2]]) || tregs[r].suppress_charges) continue;
        P3 p[3] = {P(ind[0]), P(ind[1]), P(ind[2])};
        P3 nv = cross3(sub(p[1], p[0]), sub(p[2], p[0]));
        const double surf = 0.5 * nrm(nv);
        const double nn_ = nrm(nv);
        DevTri T;
        std::memset(&T, 0, sizeof(T));
        T.n[0] = nv.x / nn_; T.n[1] = nv.y / nn_; T.n[2] = nv.z / nn_;
        T.dMs = m->tri_dMs[f];
        for (int g = 0; g < R.npi_f; g++) T.w[g] = 2.0 * surf * R.fp[g];
        P3 gp[4];
        for (int g = 0; g < R.npi_f; g++) {
            gp[g] = {0, 0, 0};
            for (int i = 0; i < 3; i++) {
                gp[g].x += R.fa[i][g] * p[i].x; gp[g].y += R.fa[i][g] * p[i].y; gp[g].z += R.fa[i][g] * p[i].z;
            }
        }
        for (int i = 0; i < 3; i++) {
            double pc[3];
            tri_potential_coeffs(p[i], p[(i + 1) % 3], p[(i + 2) % 3], surf, pc);
            for (int k = 0; k < 3; k++) {
                double b = 0;
                for (int g = 0; g < R.npi_f; g++) b -= T.w[g] * R.fa[k][g] / nrm(sub(p[i], gp[g]));
                const int rel = (k - i + 3) % 3;
                b += 0.5 * pc[rel];
                T.beta[3 * i + k] = b;
            }
        }
        T.Ks = tregs[r].Ks;
        for (int k = 0; k < 3; k++) T.uk[k] = tregs[r].uk[k];
        htri.push_back(make_int4(ind[0], ind[1], ind[2], f));
        htc.push_back(T);
    }
    c.nft = (int)htri.size();
    c.nsrc = nmt * c.npi_t + c.nft * c.npi_f;
    std::vector<double> sxyz(3 * (size_t)c.nsrc);
    {
        size_t s = 0;
        for (int k = 0; k < nmt; k++) {
            const int ind[4] = {htet[k].x, htet[k].y, htet[k].z, htet[k].w};
            for (int g = 0; g < c.npi_t; g++, s++) {
                double x = 0, y = 0, z = 0;
                for (int i = 0; i < 4; i++) {
                    P3 q = P(ind[i]);
                    x += R.ta[i][g] * q.x; y += R.ta[i][g] * q.y; z += R.ta[i][g] * q.z;
                }
                sxyz[3 * s] = x; sxyz[3 * s + 1] = y; sxyz[3 * s + 2] = z;
            }
        }
        for (int f = 0; f < c.nft; f++) {
            const int ind[3] = {htri[f].x, htri[f].y, htri[f].z};
            for (int g = 0; g < c.npi_f; g++, s++) {
                double x = 0, y = 0, z = 0;
                for (int i = 0; i < 3; i++) {
                    P3 q = P(ind[i]);
                    x += R.fa[i][g] * q.x; y += R.fa[i][g] * q.y; z += R.fa[i][g] * q.z;
                }
                sxyz[3 * s] = x; sxyz[3 * s + 1] = y; sxyz[3 * s + 2] = z;
            }
        }
    }
    std::vector<int> tinc_ptr(nn + 1, 0), tinc(3 * (size_t)c.nft);
    for (int f = 0; f < c.nft; f++) { tinc_ptr[htri[f].x + 1]++; tinc_ptr[htri[f].y + 1]++; tinc_ptr[htri[f].z + 1]++; }
    for (int i = 0; i < nn; i++) tinc_ptr[i + 1] += tinc_ptr[i];
    {
        std::vector<int> fill(tinc_ptr.begin(), tinc_ptr.end() - 1);
        for (int f = 0; f < c.nft; f++) {
            const int ind[3] = {htri[f].x, htri[f].y, htri[f].z};
            for (int i = 0; i < 3; i++) tinc[fill[ind[i]]++] = 3 * f + i;
        }
    }
    std::vector<int> mnodes;
    double sumA = 0;
    for (int i = 0; i < nn; i++)
        if (mag[i]) { mnodes.push_back(i); sumA += A[i]; }
    c.n_mag_nodes = (int)mnodes.size();
    c.mean_A = c.n_mag_nodes ? sumA / c.n_mag_nodes : 1.0;

    // uploads
    std::vector<double> hxyz(m->xyz, m->xyz + 3 * (size_t)nn);
    CK(upload(&c.xyz, hxyz));
    CK(upload(&c.tet, htet));
    CK(upload(&c.da, da));
    CK(upload(&c.detJ, detJ));
    // double-single element integrals for the FP32 + refinement path without anisotropy, with
    // or without the spin coupling (FG_DS_ELEMENTS=0 in the environment keeps the FP64 kernel,
    // for comparisons)
    {
        const char *env = std::getenv("FG_DS_ELEMENTS");
        c.elem_ds = c.opts.precision == FG_PREC_FP32_REFINE && !c.aniso && !(env && env[0] == '0');
    }
    if (c.elem_ds) {
        const int s = elem_ds_setup(c, da, detJ);
        if (s != FG_OK) return s;
    }
    CK(upload(&c.treg, htreg));
    if (c.opts.spin_acc) {  // before the region table goes to the device: it adds the Hst prefactors
        const int s = spin_setup(c, m, regs, nreg, tregs, ntreg, hreg);
        if (s != FG_OK) return s;
    }
    CK(upload(&c.regs, hreg));
    c.nreg = nreg;
    CK(upload(&c.mag, mag));
    CK(upload(&c.inc_ptr, inc_ptr));
    CK(upload(&c.inc, inc));
    CK(upload(&c.Sptr, Sptr));
    CK(upload(&c.Scol, Scol));
    CK(upload(&c.Sval, Sval));
    CK(upload(&c.A, A));
    {
        std::vector<double> ainv(A.size(), 0.0);
        for (size_t i = 0; i < A.size(); i++)
            if (mag[i]) ainv[i] = 1.0 / A[i];
        CK(upload(&c.Ainv, ainv));
    }
    {
        std::vector<float> s32(Sval.begin(), Sval.end()), a32(A.size());
        const double sc = 1.0 / c.mean_A;
        for (size_t i = 0; i < A.size(); i++) a32[i] = (float)(A[i] * sc);
        CK(upload(&c.Sval32, s32));
        CK(upload(&c.A32, a32));
    }
    CK(upload(&c.tri, htri));
    CK(upload(&c.tri_c, htc));
    CK(upload(&c.tinc_ptr, tinc_ptr));
    CK(upload(&c.tinc, tinc));
    bool surf_aniso = false;
    for (const DevTri &T : htc) surf_aniso = surf_aniso || T.Ks != 0.0;
    if (c.elem_ds && !surf_aniso && c.nft > 0) {
        // the double-single energies' triangle constants: normal and 0.5 mu0 dMs times each
        // Gauss weight as (hi, lo) pairs, four float4 per triangle
        auto split = [](double x, float &h, float &l) {
            h = (float)x;
            l = (float)(x - (double)h);
        };
        std::vector<float4> tds(4 * (size_t)c.nft, make_float4(0.f, 0.f, 0.f, 0.f));
        for (int f = 0; f < c.nft; f++) {
            const DevTri &T = htc[f];
            float v[16] = {0};
            for (int k = 0; k < 3; k++) split(T.n[k], v[2 * k], v[2 * k + 1]);
            for (int g = 0; g < 4; g++) split(0.5 * FG_MU0 * T.dMs * T.w[g], v[6 + 2 * g], v[7 + 2 * g]);
            for (int q = 0; q < 4; q++) tds[4 * (size_t)f + q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        }
        CK(upload(&c.tri_ds, tds));
    }
    if (surf_aniso && c.nft > 0) {
        CK(dalloc(&c.tri_be, 9 * (size_t)c.nft));
        CK(cudaMemset(c.tri_be, 0, 9 * sizeof(double) * c.nft));
    }
    CK(upload(&c.src_xyz, sxyz));
    c.h_src_xyz = std::move(sxyz);
    CK(upload(&c.mag_nodes, mnodes));
    for (int k = 0; k < 2; k++) {
        CK(dalloc(&c.u[k], 3 * (size_t)nn));
        CK(dalloc(&c.v[k], 3 * (size_t)nn));
        CK(dalloc(&c.phi[k], nn));
        CK(dalloc(&c.phiv[k], nn));
        CK(cudaMemset(c.u[k], 0, 3 * sizeof(double) * nn));
        CK(cudaMemset(c.v[k], 0, 3 * sizeof(double) * nn));
        CK(cudaMemset(c.phi[k], 0, sizeof(double) * nn));
        CK(cudaMemset(c.phiv[k], 0, sizeof(double) * nn));
    }
    CK(dalloc(&c.ep, 3 * (size_t)nn));
    CK(dalloc(&c.eq, 3 * (size_t)nn));
    CK(dalloc(&c.slot, 4 * (size_t)nmt));
    CK(dalloc(&c.Dl, nn));
    CK(dalloc(&c.rhs, 2 * (size_t)nn));
    CK(dalloc(&c.x, 2 * (size_t)nn));
    CK(dalloc(&c.bv, 10 * 2 * (size_t)nn));
    CK(dalloc(&c.W, 3 * (size_t)nn));
    CK(dalloc(&c.ep32, 3 * (size_t)nn));
    CK(dalloc(&c.eq32, 3 * (size_t)nn));
    CK(dalloc(&c.Dl32, nn));
    CK(dalloc(&c.fv, 23 * (size_t)nn));
    c.bicg_grid = bicg_grid_size(c, false);
    c.mixed_grid = mixed_grid_size(c);
    c.partial_len = 8 * std::max(c.bicg_grid, 1024);
    CK(dalloc(&c.partial, c.partial_len));
    CK(dalloc(&c.bar, 1));
    CK(cudaMemset(c.bar, 0, sizeof(GridBar)));
    CK(dalloc(&c.dres, 1));
    CK(cudaMallocHost((void **)&c.hres, sizeof(SolveResult)));
    CK(cudaMallocHost((void **)&c.hflag, sizeof(int)));
    *c.hflag = 0;
    CK(dalloc(&c.src_q, c.nsrc));
    CK(dalloc(&c.tri_slot, 3 * (size_t)c.nft));
    CK(dalloc(&c.pot, nn));
    CK(cudaMemset(c.pot, 0, sizeof(double) * nn));
    if (!c.opts.first_order) {  // the demag of v is evaluated beside that of m
        CK(dalloc(&c.src_q2, c.nsrc));
        CK(dalloc(&c.tri_slot2, 3 * (size_t)c.nft));
        CK(dalloc(&c.pot2, nn));
        CK(cudaMemset(c.pot2, 0, sizeof(double) * nn));
    }
    c.epart_blocks = std::max(1, std::min(4 * c.nsm, (nmt + 255) / 256));
    CK(dalloc(&c.epart, 7 * (size_t)c.epart_blocks));
    CK(cudaMallocHost((void **)&c.hepart, 7 * sizeof(double) * c.epart_blocks));
    if (c.opts.learned_guess) {
        int sm = mlp_create(c);
        if (sm != FG_OK) {
            c.err = "fg_create: learned-guess buffers";
            return sm;
        }
    }
    if (c.batch) {
        int sb = batch_setup(c, htet, htri);
        if (sb != FG_OK) return sb;
    }
    int demag = c.opts.demag;
    if (demag == FG_DEMAG_AUTO) demag = ((double)c.nsrc * c.n_mag_nodes > 4e9) ? FG_DEMAG_FMM : FG_DEMAG_DIRECT;
    c.opts.demag = demag;
    if (demag == FG_DEMAG_FMM) {
        int s = fmm_build(c);
        if (s != FG_OK) return s;
    }
    c.dinc = demag == FG_DEMAG_FMM && c.opts.precision == FG_PREC_FP32_REFINE && c.opts.demag_increment != 0 &&
            !c.batch;
    if (c.dinc) {
        // the change of the field in FP32 and the FP32 charges of the incremental evaluation:
        // FP32 copies of da and of -Ms detJ per magnetic tet (the FP64 charge arithmetic would
        // keep GB300's 1/64-rate FP64 pipe busy for the whole charge pass)
        CK(dalloc(&c.dstate32, 6 * (size_t)c.nn));
        std::vector<float> da32(da.begin(), da.end()), cq32(c.nmt);
        for (int k = 0; k < c.nmt; k++) cq32[k] = (float)(-hreg[htreg[k]].Ms * detJ[k]);
        CK(upload(&c.da32, da32));
        CK(upload(&c.cq32, cq32));
        CK(dalloc(&c.src_qf, std::max(1, c.nsrc)));
        if (c.src_q2) CK(dalloc(&c.src_q2f, std::max(1, c.nsrc)));
        if (c.nft > 0) {
            std::vector<float4> t32(4 * (size_t)c.nft);
            for (int f = 0; f < c.nft; f++) {
                const DevTri &T = htc[f];
                float v[16];
                for (int k = 0; k < 3; k++) v[k] = (float)T.n[k];
                for (int g = 0; g < 4; g++) v[3 + g] = (float)(T.dMs * T.w[g]);
                for (int k = 0; k < 9; k++) v[7 + k] = (float)(T.dMs * T.beta[k]);
                for (int q = 0; q < 4; q++) t32[4 * (size_t)f + q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
            CK(upload(&c.tri32, t32));
        }
    }
    CK(cudaDeviceSynchronize());
    return FG_OK;
}

static int create_common(const fg_mesh *mesh, const fg_region *regions, int n_regions,
                         const fg_tri_region *tri_regions, int n_tri_regions, const fg_opts *opts,
                         std::vector<int> *node_seg, int nseg, fg_ctx **out) {
    if (!out) return FG_EINVAL;
    *out = nullptr;
    fg_ctx *h = new (std::nothrow) fg_ctx();
    if (!h) return FG_ENOMEM;
    if (node_seg) {
        h->c.batch = true;
        h->c.nseg = nseg;
        h->c.h_node_seg = std::move(*node_seg);
    }
    int s;
    try {
        s = create_impl(h, mesh, regions, n_regions, tri_regions, n_tri_regions, opts);
    } catch (const std::bad_alloc &) {
        h->c.err = "host allocation failed";
        s = FG_ENOMEM;
    } catch (...) {
        h->c.err = "unexpected exception";
        s = FG_EINVAL;
    }
    if (s != FG_OK) {
        g_create_error = h->c.err;
        fg_destroy(h);
        return s;
    }
    *out = h;
    return FG_OK;
}

int fg_create(const fg_mesh *mesh, const fg_region *regions, int n_regions, const fg_tri_region *tri_regions,
              int n_tri_regions, const fg_opts *opts, fg_ctx **out) {
    return create_common(mesh, regions, n_regions, tri_regions, n_tri_regions, opts, nullptr, 1, out);
}

int fg_batch_create(const fg_mesh *meshes, int n_samples, const fg_region *regions, int n_regions,
                    const fg_tri_region *tri_regions, int n_tri_regions, const fg_opts *opts, fg_ctx **out) {
    if (!out) return FG_EINVAL;
    *out = nullptr;
    if (!meshes || n_samples <= 0) {
        g_create_error = "fg_batch_create: no samples";
        return FG_EINVAL;
    }
    // the samples' meshes concatenated: a block-diagonal system over disjoint node sets
    std::vector<double> xyz, dMs;
    std::vector<int32_t> tet4, treg, tri3, freg;
    std::vector<int> node_seg;
    try {
        int off = 0;
        for (int g = 0; g < n_samples; g++) {
            const fg_mesh &m = meshes[g];
            if (m.n_nodes <= 0 || m.n_tets <= 0 || !m.xyz || !m.tet4 || !m.tet_region ||
                (m.n_tris > 0 && (!m.tri3 || !m.tri_region || !m.tri_dMs))) {
                g_create_error = "fg_batch_create: sample " + std::to_string(g) + " has incomplete mesh data";
                return FG_EINVAL;
            }
            xyz.insert(xyz.end(), m.xyz, m.xyz + 3 * (size_t)m.n_nodes);
            for (size_t k = 0; k < 4 * (size_t)m.n_tets; k++) {
                const int v = m.tet4[k];
                if (v < 0 || v >= m.n_nodes) {
                    g_create_error = "fg_batch_create: tet node index out of range in sample " + std::to_string(g);
                    return FG_EMESH;
                }
                tet4.push_back(v + off);
            }
            treg.insert(treg.end(), m.tet_region, m.tet_region + m.n_tets);
            for (size_t k = 0; k < 3 * (size_t)m.n_tris; k++) {
                const int v = m.tri3[k];
                if (v < 0 || v >= m.n_nodes) {
                    g_create_error = "fg_batch_create: triangle node out of range in sample " + std::to_string(g);
                    return FG_EMESH;
                }
                tri3.push_back(v + off);
            }
            if (m.n_tris > 0) {
                freg.insert(freg.end(), m.tri_region, m.tri_region + m.n_tris);
                dMs.insert(dMs.end(), m.tri_dMs, m.tri_dMs + m.n_tris);
            }
            node_seg.insert(node_seg.end(), m.n_nodes, g);
            off += m.n_nodes;
        }
    } catch (const std::bad_alloc &) {
        g_create_error = "host allocation failed";
        return FG_ENOMEM;
    }
    fg_mesh u;
    std::memset(&u, 0, sizeof(u));
    u.n_nodes = (int)node_seg.size();
    u.n_tets = (int)treg.size();
    u.n_tris = (int)freg.size();
    u.xyz = xyz.data();
    u.tet4 = tet4.data();
    u.tet_region = treg.data();
    u.tri3 = u.n_tris ? tri3.data() : nullptr;
    u.tri_region = u.n_tris ? freg.data() : nullptr;
    u.tri_dMs = u.n_tris ? dMs.data() : nullptr;
    return create_common(&u, regions, n_regions, tri_regions, n_tri_regions, opts, &node_seg, n_samples, out);
}

void fg_destroy(fg_ctx *h) {
    if (!h) return;
    Ctx &c = h->c;
    if (c.stream) cudaStreamSynchronize(c.stream);
    void *ptrs[] = {c.xyz, c.tet, c.da, c.detJ, c.treg, c.regs, c.mag, c.inc_ptr, c.inc, c.Sptr, c.Scol, c.Sval,
                    c.Sval32, c.A, c.Ainv, c.A32, c.tri, c.tri_c, c.tinc_ptr, c.tinc, c.src_xyz, c.mag_nodes, c.u[0], c.u[1],
                    c.v[0], c.v[1], c.phi[0], c.phi[1], c.phiv[0], c.phiv[1], c.ep, c.eq, c.ep32, c.eq32, c.Dl32,
                    c.slot, c.Dl, c.rhs, c.x, c.bv, c.W, c.fv, c.partial, c.bar, c.dres, c.src_q, c.tri_slot,
                    c.pot, c.epart, c.src_dst, c.src_q2, c.tri_slot2, c.pot2, c.tri_be, c.hsp, c.da_ds, c.J_ds, c.state_ds,
                    c.dstate32, c.da32, c.cq32, c.src_qf, c.src_q2f, c.tri_ds, c.tri32};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    fmm64_free(c);
    fmm_free(c);
    mlp_free(c);
    spin_free(c);
    recenter_free(c);
    batch_free(c);
    if (c.hres) cudaFreeHost(c.hres);
    if (c.hflag) cudaFreeHost(c.hflag);
    if (c.hepart) cudaFreeHost(c.hepart);
    for (int k = 0; k < 8; k++)
        if (c.ev[k]) cudaEventDestroy(c.ev[k]);
    if (c.stream2) cudaStreamSynchronize(c.stream2);
    if (c.ev_fork) cudaEventDestroy(c.ev_fork);
    if (c.ev_join) cudaEventDestroy(c.ev_join);
    if (c.stream2) cudaStreamDestroy(c.stream2);
    if (c.stream) cudaStreamDestroy(c.stream);
    delete h;
}

int fg_set_state(fg_ctx *h, const double *u, const double *v, const double *phi, const double *phiv) {
    if (!h || !u) return FG_EINVAL;
    Ctx &c = h->c;
    const size_t n3 = 3 * sizeof(double) * c.nn, n1 = sizeof(double) * c.nn;
    // the host data crosses the link once (into CURRENT); NEXT is a device-side copy
    CK(cudaMemcpyAsync(c.u[0], u, n3, cudaMemcpyHostToDevice, c.stream));
    if (v) CK(cudaMemcpyAsync(c.v[0], v, n3, cudaMemcpyHostToDevice, c.stream));
    else CK(cudaMemsetAsync(c.v[0], 0, n3, c.stream));
    if (phi) CK(cudaMemcpyAsync(c.phi[0], phi, n1, cudaMemcpyHostToDevice, c.stream));
    else CK(cudaMemsetAsync(c.phi[0], 0, n1, c.stream));
    if (phiv) CK(cudaMemcpyAsync(c.phiv[0], phiv, n1, cudaMemcpyHostToDevice, c.stream));
    else CK(cudaMemsetAsync(c.phiv[0], 0, n1, c.stream));
    CK(cudaMemcpyAsync(c.u[1], c.u[0], n3, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.v[1], c.v[0], n3, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.phi[1], c.phi[0], n1, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.phiv[1], c.phiv[0], n1, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    // given potentials are those of the given fields (v = 0 has phiv = 0)
    c.dinc_valid[0] = phi != nullptr;
    c.dinc_valid[1] = phiv != nullptr || v == nullptr;
    return FG_OK;
}

int fg_host_alloc(size_t bytes, void **ptr) {
    if (!ptr) return FG_EINVAL;
    *ptr = nullptr;
    if (cudaMallocHost(ptr, bytes > 0 ? bytes : 1) != cudaSuccess) {
        cudaGetLastError();
        *ptr = nullptr;
        return FG_ECUDA;
    }
    return FG_OK;
}

int fg_host_free(void *ptr) {
    if (ptr && cudaFreeHost(ptr) != cudaSuccess) {
        cudaGetLastError();
        return FG_ECUDA;
    }
    return FG_OK;
}

int fg_get_state(const fg_ctx *hc, int which, double *u, double *v, double *phi, double *phiv) {
    if (!hc || which < 0 || which > 1) return FG_EINVAL;
    fg_ctx *h = const_cast<fg_ctx *>(hc);
    Ctx &c = h->c;
    const size_t n3 = 3 * sizeof(double) * c.nn, n1 = sizeof(double) * c.nn;
    if (u) CK(cudaMemcpyAsync(u, c.u[which], n3, cudaMemcpyDeviceToHost, c.stream));
    if (v) CK(cudaMemcpyAsync(v, c.v[which], n3, cudaMemcpyDeviceToHost, c.stream));
    if (phi) CK(cudaMemcpyAsync(phi, c.phi[which], n1, cudaMemcpyDeviceToHost, c.stream));
    if (phiv) CK(cudaMemcpyAsync(phiv, c.phiv[which], n1, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return FG_OK;
}

int fg_step(fg_ctx *h, double dt, double prefactor, const double Hext[3], double basis_angle, fg_step_report *rep) {
    if (!h || !Hext || !(dt > 0)) return FG_EINVAL;
    Ctx &c = h->c;
    if (c.batch) {
        c.err = "fg_step: a batch context steps with fg_batch_step";
        return FG_EINVAL;
    }
    if (c.opts.precision == FG_PREC_FP32_REFINE && c.lpr == 0) {
        CK(launch_tet(c, dt, Hext));
        CK(mixed_autotune(c, dt, prefactor, basis_angle));
    }
    CK(cudaEventRecord(c.ev[0], c.stream));
    c.step_open = true;
    const bool use_mlp = c.mlp && mlp_steps(c) >= c.opts.mlp_train_steps;
    const int train_every = std::max(1, c.opts.mlp_train_every);
    // a successful solve of this step trains the guess (features kept from before the solve)
    const bool will_train = !use_mlp || h->solves_since_train + 1 >= train_every;
    CK(launch_tet(c, dt, Hext));
    // the node kernel forms the learned guess's features when this step uses or trains it
    if (c.mlp && (use_mlp || will_train)) c.node_feat = mlp_node_features(c);
    const cudaError_t en = launch_node(c, basis_angle);
    c.node_feat.feat = nullptr;
    CK(en);
    c.launches += 2;
    h->last_c0 = prefactor * FG_THETA * dt * FG_GAMMA0;
    if (c.mlp) CK(mlp_before_solve(c, h->last_c0, use_mlp, will_train));
    CK(cudaEventRecord(c.ev[1], c.stream));
    if (c.opts.precision == FG_PREC_FP32_REFINE) {
        const cudaError_t e = launch_mixed(c, dt, prefactor);
        c.cand_x = c.cand_W = nullptr;  // a candidate is judged by one solve only
        c.cand_o = nullptr;
        CK(e);
    } else {
        CK(launch_bicg64(c, dt, prefactor));
    }
    c.launches += 1;
    CK(cudaEventRecord(c.ev[2], c.stream));
    CK(cudaMemcpyAsync(c.hres, c.dres, sizeof(SolveResult), cudaMemcpyDeviceToHost, c.stream));
    if (c.mlp) CK(mlp_before_sync(c));
    CK(cudaStreamSynchronize(c.stream));
    cudaEventElapsedTime(&c.ms[0], c.ev[0], c.ev[1]);
    cudaEventElapsedTime(&c.ms[1], c.ev[1], c.ev[2]);
    const SolveResult &r = *c.hres;
    int status = FG_OK;
    if (r.timeout) status = FG_ETIMEDOUT;
    else if (r.status == 1) status = FG_SOLVER_ITER_OVERFLOW;
    else if (r.status == 2 || r.fail) status = FG_SOLVER_CANNOT_CONVERGE;
    int accepted = 0;
    double r0m = r.res0, r0p = r.res0;
    if (c.mlp) {
        mlp_after_sync(c, use_mlp ? &accepted : nullptr, &r0m, &r0p, nullptr);
        if (mlp_take_timeout(c)) {
            status = FG_ETIMEDOUT;
            c.err = "learned guess: a tensor-core pipeline wait timed out";
        }
        if (!use_mlp) { r0m = r.res0; r0p = r.res0; }
        // train on this step's solution (asynchronous; its loss is read at the next sync)
        if (status == FG_OK) {
            ++h->solves_since_train;
            if (will_train) {
                h->solves_since_train = 0;
                CK(mlp_train(c));
            }
        }
    }
    if (rep) {
        std::memset(rep, 0, sizeof(*rep));
        rep->status = status;
        rep->iters = r.nit;
        rep->refinements = r.nref;
        rep->guess_accepted = accepted;
        rep->vmax = FG_GAMMA0 * std::sqrt(r.v2max);
        rep->res = r.res;
        rep->rhsn = r.rhsn;
        rep->res0 = r.res0;
        rep->res0_fallback = use_mlp ? r0p : r.res0;
    }
    if (status == FG_ETIMEDOUT) {
        c.err = "persistent solver: grid barrier timed out";
        cudaMemsetAsync(c.bar, 0, sizeof(GridBar), c.stream);
    }
    return status;
}

static int demag_into(fg_ctx *h, const double *m, double *phi_out) {
    Ctx &c = h->c;
    CK(launch_charges(c, m));
    if (c.opts.demag == FG_DEMAG_FMM) {
        CK(fmm_eval(c));
        c.launches += fmm_launches_per_eval(c);
    } else {
        CK(launch_p2p_direct(c));
        c.launches += 1;
    }
    CK(launch_phi_final(c, phi_out));
    c.launches += 2;
    return FG_OK;
}

static int energy_impl(fg_ctx *h, const double Hext[3], double E[4], double avg[3]) {
    Ctx &c = h->c;
    CK(launch_energy(c, Hext));
    c.launches += 1;
    CK(cudaMemcpyAsync(c.hepart, c.epart, 7 * sizeof(double) * c.epart_blocks, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    double s[7] = {0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 7; k++)
        for (int b = 0; b < c.epart_blocks; b++) s[k] += c.hepart[k * c.epart_blocks + b];
    if (E)
        for (int k = 0; k < 4; k++) E[k] = s[k];
    if (avg)
        for (int k = 0; k < 3; k++) avg[k] = s[4 + k] / c.total_mag_vol;
    return FG_OK;
}

// Demag of m and of v (Fem::compute_all, src/fem.h): with the FMM one evaluation of both
// charge sets (shared tree passes, one near-field pass), else one after the other.
static int demag_pair(fg_ctx *h) {
    Ctx &c = h->c;
    if (c.opts.demag != FG_DEMAG_FMM || !c.src_q2) {
        int s = demag_into(h, c.u[1], c.phi[1]);
        if (s == FG_OK) s = demag_into(h, c.v[1], c.phiv[1]);
        return s;
    }
    CK(launch_charges_pair(c, c.u[1], c.v[1]));
    CK(fmm_eval(c, 2));
    CK(launch_phi_final(c, c.phi[1], 0));
    CK(launch_phi_final(c, c.phiv[1], 1));
    c.launches += 3 + fmm_launches_per_eval(c, 2);
    return FG_OK;
}

// Incremental demag (fg_opts.demag_increment): the potentials are linear in the field, so
// NEXT's = CURRENT's + those of d = NEXT - CURRENT; the FP32 FMM evaluates d only and the sum
// is formed in FP64, so the FP32 rounding scales with the step's change, not with the
// potential. Where CURRENT's potentials are not valid the FP64 FMM evaluates NEXT in full.
static int demag_increment(fg_ctx *h) {
    Ctx &c = h->c;
    const int nq = c.opts.first_order ? 1 : 2;
    const bool valid = c.dinc_valid[0] && (nq == 1 || c.dinc_valid[1]) && c.opts.demag_increment != 2;
    if (valid) {
        CK(launch_state_diff(c));
        CK(launch_charges32(c, nq));
        c.charges32 = true;  // the FP32 FMM reads the FP32 charges of the change
        const cudaError_t se = fmm_eval(c, nq);
        c.charges32 = false;
        CK(se);
        CK(launch_phi_final(c, c.phi[1], 0, c.phi[0]));
        if (nq == 2) CK(launch_phi_final(c, c.phiv[1], 1, c.phiv[0]));
        c.launches += 2 + nq + fmm_launches_per_eval(c, nq);
        return FG_OK;
    }
    if (nq == 2) CK(launch_charges_pair(c, c.u[1], c.v[1]));
    else CK(launch_charges(c, c.u[1]));
    const int s = fmm_eval_fp64(c, nq);
    if (s != FG_OK) return s;
    CK(launch_phi_final(c, c.phi[1], 0));
    if (nq == 2) CK(launch_phi_final(c, c.phiv[1], 1));
    c.launches += 1 + nq;
    return FG_OK;
}

int fg_compute_all(fg_ctx *h, const double Hext[3], double energies[4]) {
    if (!h || !Hext) return FG_EINVAL;
    Ctx &c = h->c;
    CK(cudaEventRecord(c.ev[3], c.stream));
    int s = c.dinc ? demag_increment(h) : c.opts.first_order ? demag_into(h, c.u[1], c.phi[1]) : demag_pair(h);
    if (s) return s;
    if (c.spin) {  // spinAcc::compute after the demag (src/fem.h:203-224)
        CK(cudaEventRecord(c.ev[6], c.stream));
        CK(launch_spin(c));
        CK(cudaEventRecord(c.ev[7], c.stream));
        c.spin_timed = true;
        c.launches += 1;
    }
    CK(cudaEventRecord(c.ev[4], c.stream));
    // energies of NEXT: the partial sums are read back with the evolution's copies queued
    // behind them, so the step has one host round trip here, at its end
    CK(launch_energy(c, Hext));
    c.launches += 1;
    CK(cudaMemcpyAsync(c.hepart, c.epart, 7 * sizeof(double) * c.epart_blocks, cudaMemcpyDeviceToHost, c.stream));
    // Fem::evolution: CURRENT <- NEXT
    if (c.mlp) CK(mlp_before_evolution(c));
    const size_t n3 = 3 * sizeof(double) * c.nn, n1 = sizeof(double) * c.nn;
    CK(cudaMemcpyAsync(c.u[0], c.u[1], n3, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.v[0], c.v[1], n3, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.phi[0], c.phi[1], n1, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaMemcpyAsync(c.phiv[0], c.phiv[1], n1, cudaMemcpyDeviceToDevice, c.stream));
    CK(cudaEventRecord(c.ev[5], c.stream));
    if (int *fl = fmm_error_flag(c)) CK(cudaMemcpyAsync(c.hflag, fl, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (energies) {
        double E[4] = {0, 0, 0, 0};
        for (int k = 0; k < 4; k++)
            for (int b = 0; b < c.epart_blocks; b++) E[k] += c.hepart[k * c.epart_blocks + b];
        for (int k = 0; k < 4; k++) energies[k] = E[k];
    }
    if (*c.hflag) {
        c.err = "fmm: a tensor-core pipeline wait timed out";
        *c.hflag = 0;
        cudaMemsetAsync(fmm_error_flag(c), 0, sizeof(int), c.stream);
        return FG_ETIMEDOUT;
    }
    cudaEventElapsedTime(&c.ms[2], c.ev[3], c.ev[4]);
    cudaEventElapsedTime(&c.ms[3], c.ev[4], c.ev[5]);
    // whole step on the stream's timeline: fg_step's first event to this call's last one
    // (includes the learned guess's training kernels and the host gap between the calls)
    c.ms[4] = c.ms[2] + c.ms[3];
    if (c.step_open) cudaEventElapsedTime(&c.ms[4], c.ev[0], c.ev[5]);
    c.step_open = false;
    c.dinc_valid[0] = c.dinc_valid[1] = true;  // CURRENT now holds NEXT and its potentials
    return FG_OK;
}

int fg_demag(fg_ctx *h, int which, double *out) {
    if (!h || !out || which < 0 || which > 1) return FG_EINVAL;
    Ctx &c = h->c;
    int s = demag_into(h, which ? c.v[1] : c.u[1], c.bv + 9 * 2 * (size_t)c.nn);
    if (s) return s;
    // non-magnetic nodes keep 0 in the scratch vector
    CK(cudaMemcpyAsync(out, c.bv + 9 * 2 * (size_t)c.nn, sizeof(double) * c.nn, cudaMemcpyDeviceToHost, c.stream));
    if (int *fl = fmm_error_flag(c)) CK(cudaMemcpyAsync(c.hflag, fl, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    if (*c.hflag) {
        c.err = "fmm: a tensor-core pipeline wait timed out";
        *c.hflag = 0;
        cudaMemsetAsync(fmm_error_flag(c), 0, sizeof(int), c.stream);
        return FG_ETIMEDOUT;
    }
    for (int i = 0; i < c.nn; i++)
        if (!c.h_mag[i]) out[i] = 0.0;
    return FG_OK;
}

int fg_energy(fg_ctx *h, const double Hext[3], double energies[4]) {
    if (!h || !Hext || !energies) return FG_EINVAL;
    return energy_impl(h, Hext, energies, nullptr);
}

int fg_average(fg_ctx *h, int which, double avg[3]) {
    if (!h || !avg || which < 0 || which > 1) return FG_EINVAL;
    Ctx &c = h->c;
    double zero[3] = {0, 0, 0};
    if (which == 0) return energy_impl(h, zero, nullptr, avg);
    // <v>: run the same reduction on the NEXT velocity field
    std::swap(c.u[1], c.v[1]);
    int s = energy_impl(h, zero, nullptr, avg);
    std::swap(c.u[1], c.v[1]);
    return s;
}

int fg_debug_system(fg_ctx *h, double *rhs, double *ep, double *eq) {
    if (!h) return FG_EINVAL;
    Ctx &c = h->c;
    if (rhs) CK(cudaMemcpy(rhs, c.rhs, 2 * sizeof(double) * c.nn, cudaMemcpyDeviceToHost));
    if (ep) CK(cudaMemcpy(ep, c.ep, 3 * sizeof(double) * c.nn, cudaMemcpyDeviceToHost));
    if (eq) CK(cudaMemcpy(eq, c.eq, 3 * sizeof(double) * c.nn, cudaMemcpyDeviceToHost));
    return FG_OK;
}

int fg_debug_apply(fg_ctx *h, const double *x, double *y) {
    if (!h || !x || !y) return FG_EINVAL;
    Ctx &c = h->c;
    const size_t n2 = 2 * (size_t)c.nn;
    double *dx = c.bv + 9 * n2, *dy = c.bv + 8 * n2;  // scratch: spare vector and Minv slot
    std::vector<double> keep(n2);
    CK(cudaMemcpy(keep.data(), dy, n2 * sizeof(double), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(dx, x, n2 * sizeof(double), cudaMemcpyHostToDevice));
    CK(launch_apply(c, h->last_c0, dx, dy));
    CK(cudaMemcpyAsync(y, dy, n2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    CK(cudaMemcpy(dy, keep.data(), n2 * sizeof(double), cudaMemcpyHostToDevice));
    return FG_OK;
}

int fg_counters(const fg_ctx *h, long long out[4]) {
    if (!h || !out) return FG_EINVAL;
    const Ctx &c = h->c;
    out[0] = c.launches;
    int L = 0, nl = 0;
    double a = 0, b = 0;
    if (c.fmm) fmm_info(c, &L, &nl, &a, &b);
    out[1] = L;
    out[2] = (long long)a;
    out[3] = (long long)b;
    return FG_OK;
}

int fg_mlp_info(const fg_ctx *h, long long *train_steps, double *last_loss) {
    if (!h) return FG_EINVAL;
    if (!h->c.mlp) return FG_EINVAL;
    if (train_steps) *train_steps = mlp_steps(h->c);
    if (last_loss) *last_loss = mlp_loss(h->c);
    return FG_OK;
}

int fg_mlp_debug_grad(fg_ctx *h, int nsamples, const float *feat, const float *target, float *weights,
                      float *grad, float *loss) {
    if (!h || !h->c.mlp || !feat || !target || !weights || !grad || !loss) return FG_EINVAL;
    return mlp_debug_grad(h->c, nsamples, feat, target, weights, grad, loss);
}

int fg_mlp_nparam(void) { return mlp_nparam(); }

int fg_mlp_debug_infer(fg_ctx *h, int n, const float *feat, float *out) {
    if (!h || !h->c.mlp || !feat || !out || n <= 0) return FG_EINVAL;
    return mlp_debug_infer(h->c, n, feat, out);
}

int fg_debug_wait_timeout(fg_ctx *h, int which) {
    if (!h || which < 0 || which > 1) return FG_EINVAL;
    Ctx &c = h->c;
    int *flag = nullptr;
    CK(cudaMalloc(&flag, sizeof(int)));
    int hv = 0;
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), c.stream);
    if (e == cudaSuccess)
        e = which == 0 ? launch_barrier_timeout_probe(c, flag) : launch_mbar_timeout_probe(c.stream, flag);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hv, flag, sizeof(int), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    cudaFree(flag);
    cudaMemsetAsync(c.bar, 0, sizeof(GridBar), c.stream);  // the context's barrier is reusable
    if (e != cudaSuccess) {
        c.err = std::string("fg_debug_wait_timeout: ") + cudaGetErrorString(e);
        return FG_ECUDA;
    }
    if (hv) {
        c.err = which == 0 ? "grid barrier: bounded wait expired" : "mbarrier: bounded wait expired";
        return FG_ETIMEDOUT;
    }
    return FG_OK;
}

int fg_recenter(fg_ctx *h, int direction, double threshold, int *shifted) {
    if (!h || !shifted || direction < 0 || direction > 2) return FG_EINVAL;
    Ctx &c = h->c;
    if (c.batch) {
        c.err = "fg_recenter: not available for batch contexts";
        return FG_EINVAL;
    }
    double avg[3];
    int s = fg_average(h, 0, avg);
    if (s != FG_OK) return s;
    const int st = recenter_apply(c, direction, threshold, avg[direction], shifted);
    if (st == FG_OK && *shifted) c.dinc_valid[0] = c.dinc_valid[1] = false;  // the potentials belong to the old field
    return st;
}

int fg_spin_info(const fg_ctx *h, int *status, int *iters, double *V, int *v_iters, double *ms) {
    if (!h || !h->c.spin) return FG_EINVAL;
    if (ms) {
        float f = 0.f;
        if (h->c.spin_timed && cudaEventSynchronize(h->c.ev[7]) == cudaSuccess)
            cudaEventElapsedTime(&f, h->c.ev[6], h->c.ev[7]);
        *ms = f;
    }
    return spin_info(h->c, status, iters, V, v_iters);
}

int fg_get_spin(const fg_ctx *hc, double *s) {
    if (!hc || !s || !hc->c.spin_s) return FG_EINVAL;
    Ctx &c = const_cast<fg_ctx *>(hc)->c;
    CK(cudaMemcpyAsync(s, c.spin_s, 3 * sizeof(double) * c.nn, cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    return FG_OK;
}

int fg_gauss_points(const fg_ctx *h, int *n_points, double *pts) {
    if (!h || !n_points) return FG_EINVAL;
    const Ctx &c = h->c;
    const size_t n = (size_t)c.nmt * c.npi_t;
    *n_points = (int)n;
    // the tet sources are the magnetic tets' Gauss points, in magnetic-tet order
    if (pts) std::memcpy(pts, c.h_src_xyz.data(), 3 * n * sizeof(double));
    return FG_OK;
}

int fg_set_space_field(fg_ctx *h, const double *field) {
    if (!h) return FG_EINVAL;
    Ctx &c = h->c;
    if (c.batch) {
        c.err = "fg_set_space_field: not available for batch contexts";
        return FG_EINVAL;
    }
    if (!field) {
        if (c.hsp) cudaFree(c.hsp);
        c.hsp = nullptr;
        return FG_OK;
    }
    const size_t n = 3 * (size_t)c.nmt * c.npi_t;
    if (!c.hsp) CK(dalloc(&c.hsp, std::max<size_t>(n, 1)));
    CK(cudaMemcpy(c.hsp, field, n * sizeof(double), cudaMemcpyHostToDevice));
    return FG_OK;
}

int fg_set_field_amplitude(fg_ctx *h, double amplitude) {
    if (!h || !std::isfinite(amplitude)) return FG_EINVAL;
    h->c.field_amp = amplitude;
    return FG_OK;
}

int fg_set_drift(fg_ctx *h, int direction, double vdrift) {
    if (!h || direction < -1 || direction > 2 || !std::isfinite(vdrift)) return FG_EINVAL;
    if (h->c.batch && direction >= 0 && vdrift != 0.0) {
        h->c.err = "fg_set_drift: not available for batch contexts";
        return FG_EINVAL;
    }
    h->c.drift_dir = direction;
    h->c.drift_v = vdrift;
    return FG_OK;
}

int fg_solver_info(const fg_ctx *h, int *lanes_per_row, int *blocks) {
    if (!h) return FG_EINVAL;
    if (lanes_per_row) *lanes_per_row = h->c.lpr;
    if (blocks) *blocks = h->c.batch ? h->c.seg_grid : h->c.mixed_grid;
    return FG_OK;
}

int fg_fmm_timings(const fg_ctx *h, double ms[5]) {
    if (!h || !ms) return FG_EINVAL;
    return fmm_stage_ms(h->c, ms);
}

int fg_fmm_tree_info(const fg_ctx *h, double out[5]) {
    if (!h || !out) return FG_EINVAL;
    const Ctx &c = h->c;
    int L = 0, nleaf = 0;
    double a = 0, b = 0;
    if (fmm_info(c, &L, &nleaf, &a, &b) != FG_OK) {
        const_cast<Ctx &>(c).err = "fg_fmm_tree_info: the context has no FMM";
        return FG_EINVAL;
    }
    out[0] = c.fmm_setup_ms;
    out[1] = c.tree_wall_ms;
    out[2] = c.tree_sort_ms;
    out[3] = L;
    out[4] = c.batch ? c.nseg : 1;
    return FG_OK;
}

int fg_timings(const fg_ctx *h, double ms[5]) {
    if (!h || !ms) return FG_EINVAL;
    for (int k = 0; k < 5; k++) ms[k] = h->c.ms[k];
    return FG_OK;
}

}  // extern "C"
