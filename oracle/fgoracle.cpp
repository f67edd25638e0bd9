// FP64 CPU oracle for the per-time-step LLG path of FeeLLGood.
//
// TEST INFRASTRUCTURE ONLY. This library is the reference against which the GPU path is
// tested: only the tests, the smoke check and the CPU-baseline leg of bench.py may load it. The
// product library never links, loads or calls it.
//
// It restates, step by step and in plain C++17 + OpenMP (no Eigen), the reference
// algorithm of the files cited beside each function (paths are relative to the
// FeeLLGood source tree). The element matrices are formed explicitly
// (Kp = Perm.P.AE.P^T, Lp = Perm.P.BE) and scattered into a 2x2-block scalar CSR,
// exactly as the reference does, so the factorised GPU formulation is checked
// against the literal one.
//
// The demagnetising potential is an FP64 direct sum over the same Gauss-point
// sources plus the same triangle self-corrections. The reference evaluates that sum
// with ScalFMM (rotation kernel, P=9, 6 levels), which is absent here; the direct
// sum is the exact value ScalFMM approximates.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// src/config.h.in:31-32, :59
constexpr double MU0 = 1.25663706127e-6;
constexpr double GAMMA0 = 1.76085962784e11 * MU0;
constexpr double THETA = 0.5;
constexpr double QE = 1.602176634e-19;  // src/config.h.in:31-37
constexpr double MUB = QE * (6.62607015e-34 / (2 * M_PI)) / (2. * 9.1093837139e-31);

inline double sq(double x) { return x * x; }

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(double s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalized(V3 a) { return (1.0 / norm(a)) * a; }
inline double comp(V3 a, int d) { return d == 0 ? a.x : (d == 1 ? a.y : a.z); }

// Gauss rules: src/tetra.h:27-81 and src/triangle.h:20-65.
struct TetRule {
    int npi;
    double a[4][5];
    double pds[5];
};
struct TriRule {
    int npi;
    double a[3][4];
    double pds[4];
};

TetRule make_tet_rule(bool one_point) {
    TetRule r{};
    if (one_point) {
        r.npi = 1;
        for (int i = 0; i < 4; i++) r.a[i][0] = 0.25;
        r.pds[0] = 1.0 / 6.0;
    } else {
        r.npi = 5;
        const double A = 1. / 4., B = 1. / 6., C = 1. / 2., D = -2. / 15., E = 3. / 40.;
        const double u[5] = {A, B, B, B, C}, v[5] = {A, B, B, C, B}, w[5] = {A, B, C, B, B};
        const double p[5] = {D, E, E, E, E};
        for (int j = 0; j < 5; j++) {
            r.a[0][j] = 1. - u[j] - v[j] - w[j];
            r.a[1][j] = u[j];
            r.a[2][j] = v[j];
            r.a[3][j] = w[j];
            r.pds[j] = p[j];
        }
    }
    return r;
}

TriRule make_tri_rule(bool one_point) {
    TriRule r{};
    if (one_point) {
        r.npi = 1;
        for (int i = 0; i < 3; i++) r.a[i][0] = 1. / 3.;
        r.pds[0] = 0.5;
    } else {
        r.npi = 4;
        const double u[4] = {1 / 3., 1 / 5., 3 / 5., 1 / 5.}, v[4] = {1 / 3., 1 / 5., 1 / 5., 3 / 5.};
        const double p[4] = {-27 / 96., 25 / 96., 25 / 96., 25 / 96.};
        for (int j = 0; j < 4; j++) {
            r.a[0][j] = 1. - u[j] - v[j];
            r.a[1][j] = u[j];
            r.a[2][j] = v[j];
            r.pds[j] = p[j];
        }
    }
    return r;
}

// Tetra::prm subset (src/tetra.h:86-112) and Triangle::prm subset (src/triangle.h:69-101).
struct Region {
    double A, Ms, K, uk[3], K3, ex[3], ey[3], ez[3], alpha;
    double sigma, N0, P, lsd, lsf;  // spin accumulation (src/tetra.h:86-112)
};
struct TriRegion {
    double Ks, uk[3];
    int suppress_charges;
    double jn, V, uP[3], s[3];  // NaN where not given (src/triangle.h:69-101)
};

struct Node {
    V3 p, ep, eq;
    V3 u[2], v[2];
    double phi[2], phiv[2];
};
enum { CUR = 0, NXT = 1 };

struct Oracle {
    TetRule tr;
    TriRule fr;
    int nn = 0, nt = 0, nf = 0;
    std::vector<Node> node;
    std::vector<int> tet, tet_reg, tri, tri_reg;
    std::vector<double> tri_dMs;
    std::vector<Region> reg;
    std::vector<TriRegion> treg;
    // per tet: da (4x3, row-major), weight[npi]; per tri: n, surf, weight
    std::vector<double> da, wt, tri_n, tri_surf, tri_w;
    std::vector<char> magNode;
    std::vector<int> magTet, magTri, lvd;
    // R4toR3 applied field (mesh::setExtSpaceField, src/mesh.cpp:377-389): f at the Gauss points
    // of every tet [nt][npi][3] (zero for non-magnetic tets), used as Hext + amp f(g)
    std::vector<double> hsp;
    double amp = 1.0;
    // recentering drift (LinAlgebra::idx_dir and DW_vz, src/linear_algebra.h:51-53,97-118):
    // direction 0/1/2 or -1 (IDX_UNDEF), speed in m/s
    int drift_dir = -1;
    double drift_v = 0.0;
    // spin accumulation (spinAcc, electrostatSolver): potential V, spin accumulation s
    bool spin = false;
    double spin_tol = 1e-8;
    int spin_maxiter = 1000, spin_status = -1, spin_nit = 0, V_status = -1, V_nit = 0;
    std::vector<double> Vpot;
    std::vector<V3> sacc;
    double totalMagVol = 0;
    // scalar CSR with 2x2 blocks per node and per edge (src/solver.h:75-104)
    std::vector<int> rowptr, col;
    std::vector<double> val, rhs, Xw;
    // element matrices (src/element.h:59-65)
    std::vector<double> Kp, Lp;
    // solver settings and last status
    double tol = 1e-6;
    int maxiter = 700;
    int status = -1, nit = 0;
    double res = 0, rhsn = 1, vmax = 0;
    double E[4] = {0, 0, 0, 0};
    int nthreads = 0;
    int fmm_levels = 0;  // 0: exact direct sum; > 0: CPU FMM with this tree depth
    void *fmm = nullptr;
};

V3 v3(const double *p) { return {p[0], p[1], p[2]}; }

// ---------------------------------------------------------------------------------
// Element geometry: src/tetra.h:140-163 (da = dadu.inv(J), weight = detJ.pds),
// src/tetra.cpp:393-408 (Jacobian), src/triangle.h:113-127, :200-233.
void build_geometry(Oracle &o) {
    o.da.assign((size_t)o.nt * 12, 0.0);
    o.wt.assign((size_t)o.nt * o.tr.npi, 0.0);
    for (int t = 0; t < o.nt; t++) {
        const int *ind = &o.tet[4 * t];
        V3 p0 = o.node[ind[0]].p;
        V3 a = o.node[ind[1]].p - p0, b = o.node[ind[2]].p - p0, c = o.node[ind[3]].p - p0;
        double J[3][3] = {{a.x, b.x, c.x}, {a.y, b.y, c.y}, {a.z, b.z, c.z}};
        double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
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
            for (int k = 0; k < 3; k++) {
                double s = 0;
                for (int m = 0; m < 3; m++) s += dadu[i][m] * inv[m][k];
                o.da[12 * t + 3 * i + k] = s;
            }
        for (int j = 0; j < o.tr.npi; j++) o.wt[(size_t)t * o.tr.npi + j] = det * o.tr.pds[j];
    }
    o.tri_n.assign((size_t)o.nf * 3, 0.0);
    o.tri_surf.assign(o.nf, 0.0);
    o.tri_w.assign((size_t)o.nf * o.fr.npi, 0.0);
    for (int f = 0; f < o.nf; f++) {
        const int *ind = &o.tri[3 * f];
        V3 p0 = o.node[ind[0]].p;
        V3 nv = cross(o.node[ind[1]].p - p0, o.node[ind[2]].p - p0);
        double surf = 0.5 * norm(nv);
        V3 n = normalized(nv);
        o.tri_n[3 * f] = n.x;
        o.tri_n[3 * f + 1] = n.y;
        o.tri_n[3 * f + 2] = n.z;
        o.tri_surf[f] = surf;
        for (int j = 0; j < o.fr.npi; j++) o.tri_w[(size_t)f * o.fr.npi + j] = 2.0 * surf * o.fr.pds[j];
    }
}

// src/mesh.h:100-131 (edges, magNode, magTet, magTri), src/linear_algebra.h:55-63 (lvd),
// src/solver.h:75-104 (matrix shape).
void build_pattern(Oracle &o) {
    o.magNode.assign(o.nn, 0);
    o.magTet.clear();
    for (int t = 0; t < o.nt; t++)
        if (o.reg[o.tet_reg[t]].Ms > 0) {
            o.magTet.push_back(t);
            for (int i = 0; i < 4; i++) o.magNode[o.tet[4 * t + i]] = 1;
        }
    o.magTri.clear();
    for (int f = 0; f < o.nf; f++) {
        const int *ind = &o.tri[3 * f];
        if (o.magNode[ind[0]] && o.magNode[ind[1]] && o.magNode[ind[2]] &&
            !o.treg[o.tri_reg[f]].suppress_charges)
            o.magTri.push_back(f);
    }
    o.totalMagVol = 0;
    for (int t : o.magTet)
        for (int j = 0; j < o.tr.npi; j++) o.totalMagVol += o.wt[(size_t)t * o.tr.npi + j];
    o.lvd.clear();
    for (int i = 0; i < o.nn; i++)
        if (!o.magNode[i]) {
            o.lvd.push_back(2 * i);
            o.lvd.push_back(2 * i + 1);
        }
    // unique sorted edges over all tets
    std::vector<std::pair<int, int>> edges;
    edges.reserve((size_t)o.nt * 6);
    for (int t = 0; t < o.nt; t++)
        for (int i = 0; i < 3; i++)
            for (int j = i + 1; j < 4; j++) edges.push_back(std::minmax(o.tet[4 * t + i], o.tet[4 * t + j]));
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    std::vector<std::vector<int>> nb(o.nn);
    for (int i = 0; i < o.nn; i++) nb[i].push_back(i);
    for (auto &e : edges)
        if (o.magNode[e.first] && o.magNode[e.second]) {
            nb[e.first].push_back(e.second);
            nb[e.second].push_back(e.first);
        }
    const int n = 2 * o.nn;
    o.rowptr.assign(n + 1, 0);
    for (int i = 0; i < o.nn; i++) {
        std::sort(nb[i].begin(), nb[i].end());
        o.rowptr[2 * i + 1] = 2 * (int)nb[i].size();
        o.rowptr[2 * i + 2] = 2 * (int)nb[i].size();
    }
    for (int r = 0; r < n; r++) o.rowptr[r + 1] += o.rowptr[r];
    o.col.assign(o.rowptr[n], 0);
    for (int i = 0; i < o.nn; i++)
        for (int k = 0; k < 2; k++) {
            int pos = o.rowptr[2 * i + k];
            for (int j : nb[i]) {
                o.col[pos++] = 2 * j;
                o.col[pos++] = 2 * j + 1;
            }
        }
    o.val.assign(o.rowptr[n], 0.0);
    o.rhs.assign(n, 0.0);
    o.Xw.assign(n, 0.0);
    o.Kp.assign((size_t)o.nt * 64, 0.0);
    o.Lp.assign((size_t)o.nt * 8, 0.0);
}

// src/node.h:73-102 (PARANOID_ORTHONORMALIZATION is false)
void set_basis(Node &nd, double r) {
    V3 u = nd.u[CUR];
    double ax = std::fabs(u.x), ay = std::fabs(u.y), az = std::fabs(u.z);
    int minIdx = 0;  // Eigen minCoeff returns the first minimum
    double m = ax;
    if (ay < m) { m = ay; minIdx = 1; }
    if (az < m) { minIdx = 2; }
    V3 ep = {minIdx == 0 ? 1.0 : 0.0, minIdx == 1 ? 1.0 : 0.0, minIdx == 2 ? 1.0 : 0.0};
    ep = ep - dot(ep, u) * u;
    ep = normalized(ep);
    V3 eq = cross(u, ep);
    V3 nep = std::cos(r) * ep - std::sin(r) * eq;
    eq = std::sin(r) * ep + std::cos(r) * eq;
    nd.ep = nep;
    nd.eq = eq;
}

// src/tetra.cpp:47-75
void alpha_eff(double dt, double alpha, const double *uHeff, int npi, double *a_eff) {
    double reduced_dt = GAMMA0 * dt;
    const double r = 0.1;
    const double M = 2. * alpha * r / reduced_dt;
    for (int g = 0; g < npi; g++) {
        double h = uHeff[g];
        if (h > 0.) {
            a_eff[g] = (h > M) ? alpha + reduced_dt / 2. * M : alpha + reduced_dt / 2. * h;
        } else {
            a_eff[g] = (h < -M) ? alpha / (1. + reduced_dt / (2. * alpha) * M)
                                : alpha / (1. - reduced_dt / (2. * alpha) * h);
        }
    }
}

// Tet::integrales, src/tetra.cpp:210-307, with lumping :108-131, calcDiagBlock :133-140,
// calc_aniso_uniax :171-181, calc_aniso_cub :183-208, buildMatP src/element.h:81-96.
// Hext is the constant applied field plus the R4toR3 field at the Gauss points; Hst of the
// spin accumulation; the recentering drift when a direction is set (Tet::add_drift_BE).
void integrales(Oracle &o, int t, double dt, double prefactor, const double Hext[3]) {
    const TetRule &R = o.tr;
    const int npi = R.npi;
    const Region &p = o.reg[o.tet_reg[t]];
    const double alpha = p.alpha, Ms = p.Ms;
    const double Abis = 2.0 * p.A / (MU0 * Ms);
    const double s_dt = THETA * dt * GAMMA0;
    const int *ind = &o.tet[4 * t];
    const double *da = &o.da[12 * t];
    const double *w = &o.wt[(size_t)t * npi];
    V3 un[4], vn[4];
    double phin[4], phivn[4];
    for (int i = 0; i < 4; i++) {
        const Node &nd = o.node[ind[i]];
        un[i] = nd.u[CUR];
        vn[i] = nd.v[CUR];
        phin[i] = nd.phi[CUR];
        phivn[i] = nd.phiv[CUR];
    }
    V3 U[5], V[5], dUd[3];
    for (int g = 0; g < npi; g++) {
        U[g] = {0, 0, 0};
        V[g] = {0, 0, 0};
        for (int i = 0; i < 4; i++) {
            U[g] = U[g] + R.a[i][g] * un[i];
            V[g] = V[g] + R.a[i][g] * vn[i];
        }
    }
    for (int k = 0; k < 3; k++) {
        dUd[k] = {0, 0, 0};
        for (int i = 0; i < 4; i++) dUd[k] = dUd[k] + da[3 * i + k] * un[i];
    }
    V3 Hd = {0, 0, 0}, Hv = {0, 0, 0};
    for (int i = 0; i < 4; i++) {
        V3 dai = v3(&da[3 * i]);
        Hd = Hd - phin[i] * dai;
        Hv = Hv - phivn[i] * dai;
    }
    double uHeff[5];
    V3 Han[5];
    for (int g = 0; g < npi; g++) {
        uHeff[g] = -Abis * (dot(dUd[0], dUd[0]) + dot(dUd[1], dUd[1]) + dot(dUd[2], dUd[2]));
        Han[g] = {0, 0, 0};
    }
    if (p.K != 0) {
        double Kbis = 2.0 * p.K / (MU0 * Ms);
        V3 uk = v3(p.uk);
        double sdt = s_dt / GAMMA0;
        for (int g = 0; g < npi; g++) {
            Han[g] = Han[g] + (Kbis * dot(uk, U[g] + sdt * V[g])) * uk;
            uHeff[g] += Kbis * sq(dot(U[g], uk));
        }
    }
    if (p.K3 != 0) {
        double K3bis = 2.0 * p.K3 / (MU0 * Ms);
        V3 ex = v3(p.ex), ey = v3(p.ey), ez = v3(p.ez);
        double sdt = s_dt / GAMMA0;
        for (int g = 0; g < npi; g++) {
            V3 uk_u = {dot(ex, U[g]), dot(ey, U[g]), dot(ez, U[g])};
            V3 uk_v = {dot(ex, V[g]), dot(ey, V[g]), dot(ez, V[g])};
            V3 uuu = {uk_u.x * (1 - uk_u.x * uk_u.x), uk_u.y * (1 - uk_u.y * uk_u.y),
                      uk_u.z * (1 - uk_u.z * uk_u.z)};
            V3 tmp = {uk_v.x * ex.x, uk_v.y * ex.y, uk_v.z * ex.z};
            V3 corr = {tmp.x * (1 - 3 * uk_u.x * uk_u.x), tmp.y * (1 - 3 * uk_u.y * uk_u.y),
                       tmp.z * (1 - 3 * uk_u.z * uk_u.z)};
            V3 h = uuu.x * ex + uuu.y * ey + uuu.z * ez + sdt * corr;
            Han[g] = Han[g] + (-K3bis) * h;
            uHeff[g] += -K3bis * dot(uk_u, uuu);
        }
    }
    V3 H[5];
    V3 He = v3(Hext);
    // spin accumulation field (spinAcc::prepareExtraField, Tetra::calc_Hst src/tetra.cpp:93-106)
    V3 Hst[5];
    const bool spin = o.spin && !o.sacc.empty();
    if (spin) {
        const double D0 = 2.0 * p.sigma / (QE * QE * p.N0);
        const double pref = D0 / (sq(p.lsd) * GAMMA0 * Ms);
        for (int g = 0; g < npi; g++) {
            Hst[g] = {0, 0, 0};
            for (int i = 0; i < 4; i++) Hst[g] = Hst[g] + R.a[i][g] * (pref * o.sacc[ind[i]]);
        }
    }
    for (int g = 0; g < npi; g++) {
        V3 Heff = Hd + He;
        if (!o.hsp.empty())  // calc_Hext of the R4toR3 prepareElements (src/linear_algebra.cpp:54-72)
            Heff = Heff + o.amp * v3(&o.hsp[3 * ((size_t)t * npi + g)]);
        H[g] = Heff;
        if (spin) Heff = Heff + Hst[g];
        uHeff[g] += dot(U[g], Heff);
    }
    double a_eff[5];
    alpha_eff(dt, alpha, uHeff, npi, a_eff);

    // AE (12x12), index d*4+i
    double AE[12][12];
    std::memset(AE, 0, sizeof(AE));
    const double c = prefactor * s_dt * Abis;
    double wsum = 0;
    for (int g = 0; g < npi; g++) wsum += w[g];
    double contrib[4], a_w[4];
    for (int i = 0; i < 4; i++) {
        contrib[i] = 0;
        a_w[i] = 0;
        for (int g = 0; g < npi; g++) {
            contrib[i] += R.a[i][g] * w[g] * a_eff[g];
            a_w[i] += R.a[i][g] * w[g];
        }
    }
    double Eb[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            double dd = da[3 * i] * da[3 * j] + da[3 * i + 1] * da[3 * j + 1] + da[3 * i + 2] * da[3 * j + 2];
            Eb[i][j] = dd * (c * wsum);
        }
    for (int i = 0; i < 4; i++) Eb[i][i] += contrib[i];
    for (int d = 0; d < 3; d++)
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) AE[d * 4 + i][d * 4 + j] += Eb[i][j];
    for (int i = 0; i < 4; i++) {
        double dx = a_w[i] * un[i].x, dy = a_w[i] * un[i].y, dz = a_w[i] * un[i].z;
        AE[4 + i][8 + i] -= dx;
        AE[8 + i][4 + i] += dx;
        AE[0 + i][8 + i] += dy;
        AE[8 + i][0 + i] -= dy;
        AE[0 + i][4 + i] -= dz;
        AE[4 + i][0 + i] += dz;
    }
    // P (8x12): rows 0..3 ep, 4..7 eq; column d*4+i holds component d of node i.
    double P[8][12];
    std::memset(P, 0, sizeof(P));
    for (int i = 0; i < 4; i++) {
        const Node &nd = o.node[ind[i]];
        for (int d = 0; d < 3; d++) {
            P[i][d * 4 + i] = comp(nd.ep, d);
            P[4 + i][d * 4 + i] = comp(nd.eq, d);
        }
    }
    // Perm swaps the two block lines: (Perm P).row(r) = P.row(perm^-1 r), perm = {4..7,0..3}.
    double PP[8][12];
    for (int r = 0; r < 8; r++)
        for (int k = 0; k < 12; k++) PP[r][k] = P[(r + 4) % 8][k];
    double PAE[8][12];
    for (int r = 0; r < 8; r++)
        for (int k = 0; k < 12; k++) {
            double s = 0;
            for (int m = 0; m < 12; m++) s += PP[r][m] * AE[m][k];
            PAE[r][k] = s;
        }
    double *Kp = &o.Kp[(size_t)t * 64];
    for (int r = 0; r < 8; r++)
        for (int q = 0; q < 8; q++) {
            double s = 0;
            for (int k = 0; k < 12; k++) s += PAE[r][k] * P[q][k];
            Kp[r * 8 + q] = s;
        }
    // BE (3x4) -> Lp
    double BE[3][4];
    std::memset(BE, 0, sizeof(BE));
    // recentering drift (Tet::add_drift_BE, src/tetra.cpp:150-169, called at :277-288):
    // BE_i += Vdrift w_g a_i(g) (alpha dU + U x dU + s_dt (alpha dV + U x dV + V x dU)),
    // dU and dV the derivatives of u and v along the direction
    if (o.drift_dir >= 0) {
        const V3 dUdir = dUd[o.drift_dir];
        V3 dVdir = {0, 0, 0};
        for (int i = 0; i < 4; i++) dVdir = dVdir + da[3 * i + o.drift_dir] * vn[i];
        for (int g = 0; g < npi; g++) {
            const V3 D = alpha * dUdir + cross(U[g], dUdir) +
                         s_dt * (alpha * dVdir + cross(U[g], dVdir) + cross(V[g], dUdir));
            for (int i = 0; i < 4; i++) {
                const double f = o.drift_v * w[g] * R.a[i][g];
                for (int d = 0; d < 3; d++) BE[d][i] += f * comp(D, d);
            }
        }
    }
    for (int g = 0; g < npi; g++) H[g] = H[g] + Han[g] + (s_dt / GAMMA0) * Hv;
    for (int g = 0; g < npi; g++) {
        const double wg = w[g];
        for (int i = 0; i < 4; i++) {
            const double ai_w = wg * R.a[i][g];
            V3 ex = da[3 * i] * dUd[0] + da[3 * i + 1] * dUd[1] + da[3 * i + 2] * dUd[2];
            for (int d = 0; d < 3; d++) {
                BE[d][i] -= wg * Abis * comp(ex, d);
                if (spin) {  // Hst and its second-order term (src/tetra.cpp:296-303)
                    BE[d][i] += ai_w * (comp(H[g], d) + comp(Hst[g], d));
                    BE[d][i] -= ai_w * dot(Hst[g], U[g]) * s_dt * comp(V[g], d);
                } else {
                    BE[d][i] += ai_w * comp(H[g], d);
                }
            }
        }
    }
    double *Lp = &o.Lp[(size_t)t * 8];
    for (int r = 0; r < 8; r++) {
        double s = 0;
        for (int d = 0; d < 3; d++)
            for (int i = 0; i < 4; i++) s += PP[r][d * 4 + i] * BE[d][i];
        Lp[r] = s;
    }
}

// SparseMatrix::add (src/algebra/sparseMat.h:114-124): binary search + guarded +=.
inline void mat_add(Oracle &o, int i, int j, double v) {
    auto b = o.col.begin() + o.rowptr[i], e = o.col.begin() + o.rowptr[i + 1];
    auto it = std::lower_bound(b, e, j);
    double &ref = o.val[it - o.col.begin()];
#pragma omp atomic
    ref += v;
}
inline void mat_set(Oracle &o, int i, int j, double v) {
    auto b = o.col.begin() + o.rowptr[i], e = o.col.begin() + o.rowptr[i + 1];
    auto it = std::lower_bound(b, e, j);
    o.val[it - o.col.begin()] = v;
}

void spmv(const Oracle &o, const std::vector<double> &x, std::vector<double> &y) {
    const int n = 2 * o.nn;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; r++) {
        double s = 0;
        for (int k = o.rowptr[r]; k < o.rowptr[r + 1]; k++) s += o.val[k] * x[o.col[k]];
        y[r] = s;
    }
}

double vdot(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
}
double vnorm(const std::vector<double> &a) { return std::sqrt(std::fabs(vdot(a, a))); }
void mask(const std::vector<int> &ld, std::vector<double> &x) {
    for (int i : ld) x[i] = 0;
}

// algebra::iteration (src/algebra/iter.h:119-175)
struct Iter {
    double rhsn = 1.0, res = std::numeric_limits<double>::max(), resmax;
    int maxiter, nit = 0, status = -1;
    bool finished(double nr) {
        res = std::fabs(nr);
        if (std::isnan(res)) {
            status = 2;
            return false;
        }
        bool cv = res <= rhsn * resmax;
        if (cv) status = 0;
        return cv;
    }
    void inc() {
        nit++;
        if (nit >= maxiter) status = 1;
    }
};

// algebra::bicg_dir (src/algebra/bicg.h:163-234)
void bicg_dir(Oracle &o, Iter &it) {
    const size_t n = o.Xw.size();
    double rho_1 = 0, rho_2 = 0, alpha = 0, beta = 0, omega = 0;
    std::vector<double> p(n), phat(n), shat(n), r(n), rt(n), s(n), t(n), v(n), diag(n), b(o.rhs);
    for (size_t i = 0; i < n; i++) {
        auto bb = o.col.begin() + o.rowptr[i], ee = o.col.begin() + o.rowptr[i + 1];
        auto q = std::lower_bound(bb, ee, (int)i);
        double cval = (q != ee && *q == (int)i) ? o.val[q - o.col.begin()] : 0.0;
        diag[i] = 1.0 / cval;
    }
    mask(o.lvd, b);
    mask(o.lvd, diag);
    it.rhsn = vnorm(b);
    std::vector<double> &x = o.Xw;
    r = b;
    spmv(o, x, v);
    for (size_t i = 0; i < n; i++) r[i] -= v[i];
    mask(o.lvd, r);
    rt = r;
    p = r;
    while (!it.finished(vnorm(r))) {
        rho_1 = vdot(rt, r);
        if (it.nit > 0) {
            if (rho_2 == 0 || omega == 0) {
                it.status = 2;
                break;
            }
            beta = (rho_1 / rho_2) * (alpha / omega);
            for (size_t i = 0; i < n; i++) v[i] *= omega;
            for (size_t i = 0; i < n; i++) p[i] -= v[i];
            for (size_t i = 0; i < n; i++) p[i] *= beta;
            for (size_t i = 0; i < n; i++) p[i] += r[i];
        }
        for (size_t i = 0; i < n; i++) phat[i] = diag[i] * p[i];
        spmv(o, phat, v);
        mask(o.lvd, v);
        alpha = rho_1 / vdot(v, rt);
        s = r;
        for (size_t i = 0; i < n; i++) s[i] += -alpha * v[i];
        if (it.finished(vnorm(s))) {
            for (size_t i = 0; i < n; i++) x[i] += alpha * phat[i];
            break;
        } else if (it.status == 1 || it.status == 2) {
            break;
        }
        for (size_t i = 0; i < n; i++) shat[i] = diag[i] * s[i];
        spmv(o, shat, t);
        mask(o.lvd, t);
        omega = vdot(t, s) / vdot(t, t);
        for (size_t i = 0; i < n; i++) x[i] += alpha * phat[i];
        for (size_t i = 0; i < n; i++) x[i] += omega * shat[i];
        for (size_t i = 0; i < n; i++) t[i] *= omega;
        r = s;
        for (size_t i = 0; i < n; i++) r[i] -= t[i];
        rho_2 = rho_1;
        it.inc();
    }
}

// LinAlgebra::prepareElements (src/linear_algebra.cpp:26-53), Ks = 0 only.
void prepare_elements(Oracle &o, double dt, double prefactor, const double Hext[3]) {
    const int m = (int)o.magTet.size();
#pragma omp parallel for schedule(static)
    for (int k = 0; k < m; k++) integrales(o, o.magTet[k], dt, prefactor, Hext);
}

// Tri::integrales (src/triangle.cpp:6-36): surface anisotropy contribution to Lp (6 values).
void tri_integrales(Oracle &o, int f, double *Lp6) {
    const TriRule &R = o.fr;
    const TriRegion &p = o.treg[o.tri_reg[f]];
    const int *ind = &o.tri[3 * f];
    const double *w = &o.tri_w[(size_t)f * R.npi];
    double Kbis = 2.0 * p.Ks / o.tri_dMs[f];
    V3 uk = v3(p.uk);
    double BE[3][3] = {{0}};
    for (int g = 0; g < R.npi; g++) {
        V3 u = {0, 0, 0};
        for (int i = 0; i < 3; i++) u = u + R.a[i][g] * o.node[ind[i]].u[CUR];
        double pre = w[g] * Kbis * dot(uk, u);
        for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++) BE[k][i] += pre * R.a[i][g] * comp(uk, k);
    }
    for (int r = 0; r < 6; r++) {
        int src = (r + 3) % 6;  // Perm {3,4,5,0,1,2}
        int i = src % 3;
        bool isq = src >= 3;
        V3 e = isq ? o.node[ind[i]].eq : o.node[ind[i]].ep;
        Lp6[r] = e.x * BE[0][i] + e.y * BE[1][i] + e.z * BE[2][i];
    }
}

// LinAlgebra::solve (src/solver.cpp:6-89). Returns true on failure.
bool solve(Oracle &o, double dt) {
    std::fill(o.val.begin(), o.val.end(), 0.0);
    const int m = (int)o.magTet.size();
#pragma omp parallel for schedule(static)
    for (int k = 0; k < m; k++) {
        int t = o.magTet[k];
        const int *ind = &o.tet[4 * t];
        const double *Kp = &o.Kp[(size_t)t * 64];
        for (int ie = 0; ie < 4; ie++)
            for (int je = 0; je < 4; je++)
                for (int di = 0; di < 2; di++)
                    for (int dj = 0; dj < 2; dj++)
                        mat_add(o, 2 * ind[ie] + di, 2 * ind[je] + dj, Kp[(di * 4 + ie) * 8 + dj * 4 + je]);
    }
    std::fill(o.rhs.begin(), o.rhs.end(), 0.0);
    for (int t : o.magTet) {
        const int *ind = &o.tet[4 * t];
        const double *Lp = &o.Lp[(size_t)t * 8];
        for (int ie = 0; ie < 4; ie++)
            for (int di = 0; di < 2; di++) o.rhs[2 * ind[ie] + di] += Lp[di * 4 + ie];
    }
    for (int f : o.magTri) {
        if (o.treg[o.tri_reg[f]].Ks == 0) continue;  // Lp stays zero (linear_algebra.cpp:48-50)
        double Lp6[6];
        tri_integrales(o, f, Lp6);
        const int *ind = &o.tri[3 * f];
        for (int ie = 0; ie < 3; ie++)
            for (int di = 0; di < 2; di++) o.rhs[2 * ind[ie] + di] += Lp6[di * 3 + ie];
    }
    mask(o.lvd, o.rhs);
    for (int i : o.lvd) mat_set(o, i, i, 1.0);
    // buildInitGuess (src/linear_algebra.cpp:13-24)
    std::fill(o.Xw.begin(), o.Xw.end(), 0.0);
    for (int i = 0; i < o.nn; i++)
        if (o.magNode[i]) {
            o.Xw[2 * i] = dot(o.node[i].v[NXT], o.node[i].ep) / GAMMA0;
            o.Xw[2 * i + 1] = dot(o.node[i].v[NXT], o.node[i].eq) / GAMMA0;
        }
    Iter it;
    it.resmax = o.tol;
    it.maxiter = o.maxiter;
    bicg_dir(o, it);
    o.status = it.status;
    o.nit = it.nit;
    o.res = it.res;
    o.rhsn = it.rhsn;
    if (it.status == 1 || it.status == 2 || it.res > it.resmax) return true;
    double v2max = 0;
    for (int i = 0; i < o.nn; i++)
        if (o.magNode[i]) {
            double vp = o.Xw[2 * i], vq = o.Xw[2 * i + 1];
            double v2 = sq(vp) + sq(vq);
            if (v2 > v2max) v2max = v2;
            // mesh::updateNode -> Node::make_evol (src/mesh.h:185-186, src/node.h:116-122)
            Node &nd = o.node[i];
            double a = vp * GAMMA0, b = vq * GAMMA0;
            nd.v[NXT] = a * nd.ep + b * nd.eq;
            nd.u[NXT] = normalized(nd.u[CUR] + dt * nd.v[NXT]);
        }
    o.vmax = GAMMA0 * std::sqrt(v2max);
    return false;
}

// Tri::potential (src/triangle.cpp:87-125)
double tri_potential(const Oracle &o, int f, int which, int i) {
    const int *ind = &o.tri[3 * f];
    int ii = (i + 1) % 3, iii = (i + 2) % 3;
    const Node &n1 = o.node[ind[i]], &n2 = o.node[ind[ii]], &n3 = o.node[ind[iii]];
    V3 p1p2 = n2.p - n1.p, p1p3 = n3.p - n1.p;
    auto fsq = [](double x) { return std::sqrt(1.0 + x * x); };
    double b = norm(p1p2);
    double t = dot(p1p2, p1p3) / b;
    double _2s = 2. * o.tri_surf[f];
    double h = _2s / b;
    double c = (t - b) / h;
    double r = h * fsq(t / h);
    double log_1 = std::log((c * t + h + fsq(c) * r) / (b * (c + fsq(c))));
    double xi = b * log_1 / fsq(c);
    V3 n = v3(&o.tri_n[3 * f]);
    double s1 = dot(which ? n1.v[NXT] : n1.u[NXT], n);
    double s2 = dot(which ? n2.v[NXT] : n2.u[NXT], n);
    double s3 = dot(which ? n3.v[NXT] : n3.u[NXT], n);
    double pot = xi * s1 + ((xi * (h + c * t) - b * (r - b)) * s2 + b * (r - b - c * xi) * s3) * b /
                               (_2s * (1 + c * c));
    return 0.5 * o.tri_dMs[f] * pot;
}

// Gauss points of the sources, magTet then magTri order (src/fmm_demag.h:74-88).
void source_points(const Oracle &o, std::vector<double> &pts) {
    const int nts = (int)o.magTet.size() * o.tr.npi, nfs = (int)o.magTri.size() * o.fr.npi;
    pts.assign((size_t)(nts + nfs) * 3, 0.0);
    size_t k = 0;
    for (int t : o.magTet) {
        const int *ind = &o.tet[4 * t];
        for (int g = 0; g < o.tr.npi; g++, k++) {
            V3 s = {0, 0, 0};
            for (int i = 0; i < 4; i++) s = s + o.tr.a[i][g] * o.node[ind[i]].p;
            pts[3 * k] = s.x;
            pts[3 * k + 1] = s.y;
            pts[3 * k + 2] = s.z;
        }
    }
    for (int f : o.magTri) {
        const int *ind = &o.tri[3 * f];
        for (int g = 0; g < o.fr.npi; g++, k++) {
            V3 s = {0, 0, 0};
            for (int i = 0; i < 3; i++) s = s + o.fr.a[i][g] * o.node[ind[i]].p;
            pts[3 * k] = s.x;
            pts[3 * k + 1] = s.y;
            pts[3 * k + 2] = s.z;
        }
    }
}

// fmm::calc_charges (src/fmm_demag.h:155-179), Tet::charges (src/tetra.cpp:347-359),
// Tri::charges (src/triangle.cpp:45-59), Tri::correctionCharges (src/triangle.cpp:61-78).
void charges(const Oracle &o, int which, const std::vector<double> &pts, std::vector<double> &q,
             std::vector<double> &corr) {
    const int nts = (int)o.magTet.size() * o.tr.npi;
    q.assign(pts.size() / 3, 0.0);
    corr.assign(o.nn, 0.0);
    size_t k = 0;
    for (int t : o.magTet) {
        const int *ind = &o.tet[4 * t];
        const double *da = &o.da[12 * t];
        double dud = 0;
        for (int i = 0; i < 4; i++) {
            V3 m = which ? o.node[ind[i]].v[NXT] : o.node[ind[i]].u[NXT];
            dud += m.x * da[3 * i] + m.y * da[3 * i + 1] + m.z * da[3 * i + 2];
        }
        const double Ms = o.reg[o.tet_reg[t]].Ms;
        for (int g = 0; g < o.tr.npi; g++) q[k++] = -Ms * o.wt[(size_t)t * o.tr.npi + g] * dud;
    }
    for (int f : o.magTri) {
        const int *ind = &o.tri[3 * f];
        double loc[4] = {0, 0, 0, 0};
        const double dMs = o.tri_dMs[f];
        if (dMs != 0.0) {
            V3 n = v3(&o.tri_n[3 * f]);
            for (int g = 0; g < o.fr.npi; g++) {
                V3 u = {0, 0, 0};
                for (int i = 0; i < 3; i++)
                    u = u + o.fr.a[i][g] * (which ? o.node[ind[i]].v[NXT] : o.node[ind[i]].u[NXT]);
                loc[g] = dMs * o.tri_w[(size_t)f * o.fr.npi + g] * dot(u, n);
            }
        }
        for (int g = 0; g < o.fr.npi; g++) q[nts + (k - nts) + g] = loc[g];
        for (int i = 0; i < 3; i++) {
            V3 pi = o.node[ind[i]].p;
            for (int g = 0; g < o.fr.npi; g++) {
                size_t s = k + g;
                V3 gp = {pts[3 * s], pts[3 * s + 1], pts[3 * s + 2]};
                corr[ind[i]] -= loc[g] / norm(pi - gp);
            }
            corr[ind[i]] += tri_potential(o, f, which, i);
        }
        k += o.fr.npi;
    }
}

}  // namespace
extern "C" void *fgo_fmm_create(int ns, const double *src, int nt, const double *tgt, int levels);
extern "C" void fgo_fmm_destroy(void *h);
extern "C" void fgo_fmm_eval(void *h, const double *q, double *pot);
namespace {

// fmm::demag (src/fmm_demag.h:184-224): an exact FP64 direct sum in place of ScalFMM, or
// the CPU FMM (fmm_cpu.cpp) when fmm_levels > 0 (used to time the CPU baseline).
void demag_direct(Oracle &o, int which) {
    std::vector<double> pts, q, corr;
    source_points(o, pts);
    charges(o, which, pts, q, corr);
    const long ns = (long)q.size();
    if (o.fmm_levels > 0) {
        std::vector<int> tn;
        std::vector<double> txyz;
        for (int i = 0; i < o.nn; i++)
            if (o.magNode[i]) {
                tn.push_back(i);
                txyz.push_back(o.node[i].p.x);
                txyz.push_back(o.node[i].p.y);
                txyz.push_back(o.node[i].p.z);
            }
        if (!o.fmm) o.fmm = fgo_fmm_create((int)ns, pts.data(), (int)tn.size(), txyz.data(), o.fmm_levels);
        std::vector<double> pot(tn.size());
        fgo_fmm_eval(o.fmm, q.data(), pot.data());
        for (size_t k = 0; k < tn.size(); k++) {
            const int i = tn[k];
            const double phi = (pot[k] + corr[i]) / (4 * M_PI);
            if (which) o.node[i].phiv[NXT] = phi; else o.node[i].phi[NXT] = phi;
        }
        return;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < o.nn; i++) {
        if (!o.magNode[i]) continue;
        V3 x = o.node[i].p;
        double pot = 0;
        for (long s = 0; s < ns; s++) {
            double dx = x.x - pts[3 * s], dy = x.y - pts[3 * s + 1], dz = x.z - pts[3 * s + 2];
            pot += q[s] / std::sqrt(dx * dx + dy * dy + dz * dz);
        }
        double phi = (pot + corr[i]) / (4 * M_PI);
        if (which) o.node[i].phiv[NXT] = phi; else o.node[i].phi[NXT] = phi;
    }
}

// Fem::energy (src/energy.cpp:5-68) for the constant applied field, NEXT state.
void energy(Oracle &o, const double Hext[3]) {
    double E[4] = {0, 0, 0, 0};
    const TetRule &R = o.tr;
    V3 He = v3(Hext);
    for (int t : o.magTet) {
        const Region &p = o.reg[o.tet_reg[t]];
        const int *ind = &o.tet[4 * t];
        const double *da = &o.da[12 * t];
        const double *w = &o.wt[(size_t)t * R.npi];
        V3 un[4];
        double ph[4];
        for (int i = 0; i < 4; i++) {
            un[i] = o.node[ind[i]].u[NXT];
            ph[i] = o.node[ind[i]].phi[NXT];
        }
        V3 dUd[3];
        for (int k = 0; k < 3; k++) {
            dUd[k] = {0, 0, 0};
            for (int i = 0; i < 4; i++) dUd[k] = dUd[k] + da[3 * i + k] * un[i];
        }
        double dens = dot(dUd[0], dUd[0]) + dot(dUd[1], dUd[1]) + dot(dUd[2], dUd[2]);
        double ex = 0, dm = 0, an = 0, ze = 0;
        for (int g = 0; g < R.npi; g++) {
            V3 U = {0, 0, 0};
            double phg = 0;
            for (int i = 0; i < 4; i++) {
                U = U + R.a[i][g] * un[i];
                phg += R.a[i][g] * ph[i];
            }
            ex += w[g] * dens;
            dm += w[g] * (dUd[0].x + dUd[1].y + dUd[2].z) * phg;
            if (p.K != 0.0) an += w[g] * sq(dot(v3(p.uk), U));
            V3 Hg = He;
            if (!o.hsp.empty()) Hg = Hg + o.amp * v3(&o.hsp[3 * ((size_t)t * R.npi + g)]);
            ze += w[g] * dot(U, Hg);
            if (p.K3 != 0.0) {
                double a0 = dot(U, v3(p.ex)), a1 = dot(U, v3(p.ey)), a2 = dot(U, v3(p.ez));
                E[1] += p.K3 * w[g] * (sq(a0 * a1) + sq(a1 * a2) + sq(a2 * a0));
            }
        }
        E[0] += p.A * ex;
        E[2] += -0.5 * MU0 * p.Ms * dm;
        if (p.K != 0.0) E[1] += -p.K * an;
        E[3] += -MU0 * p.Ms * ze;
    }
    const TriRule &F = o.fr;
    for (int f : o.magTri) {
        const TriRegion &p = o.treg[o.tri_reg[f]];
        const int *ind = &o.tri[3 * f];
        const double *w = &o.tri_w[(size_t)f * F.npi];
        V3 n = v3(&o.tri_n[3 * f]);
        double an = 0, dm = 0;
        for (int g = 0; g < F.npi; g++) {
            V3 U = {0, 0, 0};
            double phg = 0;
            for (int i = 0; i < 3; i++) {
                U = U + F.a[i][g] * o.node[ind[i]].u[NXT];
                phg += F.a[i][g] * o.node[ind[i]].phi[NXT];
            }
            if (p.Ks != 0.0) an += w[g] * sq(dot(U, v3(p.uk)));
            dm += dot(U, n) * phg * w[g];
        }
        if (p.Ks != 0.0) E[1] += -p.Ks * an;
        E[2] += 0.5 * MU0 * o.tri_dMs[f] * dm;
    }
    for (int k = 0; k < 4; k++) o.E[k] = E[k];
}

// ----- spin accumulation: electrostatSolver and spinAcc with explicit CSR assembly -----

// Sparse matrix with the reference's shape over all tets (solver::build_shape): rows of
// dim * node + component, every component pair of every node pair of a tet.
struct Csr {
    std::vector<int> ptr, col;
    std::vector<double> val;
    void add(int i, int j, double v) {
        auto b = col.begin() + ptr[i], e = col.begin() + ptr[i + 1];
        val[std::lower_bound(b, e, j) - col.begin()] += v;
    }
    double diag(int i) const {
        auto b = col.begin() + ptr[i], e = col.begin() + ptr[i + 1];
        auto q = std::lower_bound(b, e, i);
        return (q != e && *q == i) ? val[q - col.begin()] : 0.0;
    }
    void mult(const std::vector<double> &x, std::vector<double> &y) const {
        for (size_t r = 0; r + 1 < ptr.size(); r++) {
            double s = 0;
            for (int k = ptr[r]; k < ptr[r + 1]; k++) s += val[k] * x[col[k]];
            y[r] = s;
        }
    }
};

Csr shape(const Oracle &o, int dim) {
    std::vector<std::vector<int>> nb((size_t)o.nn * dim);
    for (int t = 0; t < o.nt; t++)
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++)
                for (int a = 0; a < dim; a++)
                    for (int b = 0; b < dim; b++) nb[dim * o.tet[4 * t + i] + a].push_back(dim * o.tet[4 * t + j] + b);
    Csr M;
    M.ptr.assign(nb.size() + 1, 0);
    for (size_t r = 0; r < nb.size(); r++) {
        auto &v = nb[r];
        v.push_back((int)r);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        M.ptr[r + 1] = M.ptr[r] + (int)v.size();
    }
    for (auto &v : nb) M.col.insert(M.col.end(), v.begin(), v.end());
    M.val.assign(M.col.size(), 0.0);
    return M;
}

// algebra::cg_dir (src/algebra/cg.h:67-121)
void cg_dir(const Csr &A, std::vector<double> &x, const std::vector<double> &rhs, const std::vector<double> &xd,
            const std::vector<int> &ld, Iter &it) {
    const size_t n = x.size();
    std::vector<double> p(n), q(n), r(n), z(n), diag(n), b(rhs), tmp(n);
    for (size_t i = 0; i < n; i++) diag[i] = 1.0 / A.diag((int)i);
    A.mult(xd, z);
    for (size_t i = 0; i < n; i++) b[i] -= z[i];
    mask(ld, b);
    mask(ld, diag);
    it.rhsn = vnorm(b);
    r = b;
    A.mult(x, tmp);
    for (size_t i = 0; i < n; i++) r[i] -= tmp[i];
    mask(ld, r);
    for (size_t i = 0; i < n; i++) z[i] = diag[i] * r[i];
    double rho = vdot(z, r), rho_1 = 0.0;
    p = z;
    while (!it.finished(vnorm(r)) && it.status != 1 && it.status != 2) {
        if (it.nit > 0) {
            for (size_t i = 0; i < n; i++) z[i] = diag[i] * r[i];
            rho = vdot(z, r);
            for (size_t i = 0; i < n; i++) p[i] *= rho / rho_1;
            for (size_t i = 0; i < n; i++) p[i] += z[i];
        }
        A.mult(p, q);
        mask(ld, q);
        const double qp = vdot(q, p);
        if (qp == 0.0) {
            it.status = 2;
            break;
        }
        const double a = rho / qp;
        for (size_t i = 0; i < n; i++) x[i] += a * p[i];
        for (size_t i = 0; i < n; i++) r[i] += (-a) * q[i];
        rho_1 = rho;
        it.inc();
    }
    for (size_t i = 0; i < n; i++) x[i] += xd[i];
}

// algebra::bicg_dir with Dirichlet values (src/algebra/bicg.h:82-153)
void bicg_dir_values(const Csr &A, std::vector<double> &x, const std::vector<double> &rhs,
                     const std::vector<double> &xd, const std::vector<int> &ld, Iter &it) {
    const size_t n = x.size();
    double rho_1 = 0, rho_2 = 0, alpha = 0, beta = 0, omega = 0;
    std::vector<double> p(n), phat(n), shat(n), r(n), rt(n), s(n), t(n), v(n), diag(n), b(rhs);
    for (size_t i = 0; i < n; i++) diag[i] = 1.0 / A.diag((int)i);
    A.mult(xd, v);
    for (size_t i = 0; i < n; i++) b[i] -= v[i];
    mask(ld, b);
    mask(ld, diag);
    it.rhsn = vnorm(b);
    r = b;
    A.mult(x, v);
    for (size_t i = 0; i < n; i++) r[i] -= v[i];
    mask(ld, r);
    rt = r;
    p = r;
    while (!it.finished(vnorm(r))) {
        rho_1 = vdot(rt, r);
        if (it.nit > 0) {
            if (rho_2 == 0 || omega == 0) {
                it.status = 2;
                break;
            }
            beta = (rho_1 / rho_2) * (alpha / omega);
            for (size_t i = 0; i < n; i++) p[i] = (p[i] - omega * v[i]) * beta + r[i];
        }
        for (size_t i = 0; i < n; i++) phat[i] = diag[i] * p[i];
        A.mult(phat, v);
        mask(ld, v);
        alpha = rho_1 / vdot(v, rt);
        for (size_t i = 0; i < n; i++) s[i] = r[i] + (-alpha) * v[i];
        if (it.finished(vnorm(s))) {
            for (size_t i = 0; i < n; i++) x[i] += alpha * phat[i];
            break;
        } else if (it.status == 1 || it.status == 2) {
            break;
        }
        for (size_t i = 0; i < n; i++) shat[i] = diag[i] * s[i];
        A.mult(shat, t);
        mask(ld, t);
        omega = vdot(t, s) / vdot(t, t);
        for (size_t i = 0; i < n; i++) {
            x[i] += alpha * phat[i];
            x[i] += omega * shat[i];
        }
        for (size_t i = 0; i < n; i++) r[i] = s[i] - omega * t[i];
        rho_2 = rho_1;
        it.inc();
    }
    for (size_t i = 0; i < n; i++) x[i] += xd[i];
}

inline bool finite3(const double *v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

// electrostatSolver::solve (src/electrostatSolver.cpp:94-131), all tets and triangles
void electrostat(Oracle &o) {
    const TetRule &R = o.tr;
    Csr K = shape(o, 1);
    std::vector<double> L(o.nn, 0.0), Vd(o.nn, 0.0);
    for (int t = 0; t < o.nt; t++) {
        const double sigma = o.reg[o.tet_reg[t]].sigma;
        const double *da = &o.da[12 * t];
        const int *ind = &o.tet[4 * t];
        double AE[4][4] = {};
        for (int g = 0; g < R.npi; g++) {
            const double sw = sigma * o.wt[(size_t)t * R.npi + g];
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++)
                    AE[i][j] += sw * (da[3 * i] * da[3 * j] + da[3 * i + 1] * da[3 * j + 1] + da[3 * i + 2] * da[3 * j + 2]);
        }
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) K.add(ind[i], ind[j], AE[i][j]);
    }
    for (int f = 0; f < o.nf; f++) {
        const TriRegion &g = o.treg[o.tri_reg[f]];
        const double J = std::isfinite(g.jn) ? g.jn : 0.0;
        double BE[3] = {0, 0, 0};
        for (int q = 0; q < o.fr.npi; q++) {
            const double Jw = J * o.tri_w[(size_t)f * o.fr.npi + q];
            for (int i = 0; i < 3; i++) BE[i] -= o.fr.a[i][q] * Jw;
        }
        for (int i = 0; i < 3; i++) L[o.tri[3 * f + i]] += BE[i];
    }
    std::vector<int> ld;
    for (int f = 0; f < o.nf; f++) {
        const double V = o.treg[o.tri_reg[f]].V;
        if (std::isnan(V)) continue;
        for (int i = 0; i < 3; i++) {
            Vd[o.tri[3 * f + i]] = V;
            ld.push_back(o.tri[3 * f + i]);
        }
    }
    std::sort(ld.begin(), ld.end());
    ld.erase(std::unique(ld.begin(), ld.end()), ld.end());
    o.Vpot.assign(o.nn, 0.0);
    Iter it;
    it.resmax = o.spin_tol;
    it.maxiter = o.spin_maxiter;
    cg_dir(K, o.Vpot, L, Vd, ld, it);
    o.V_status = it.status;
    o.V_nit = it.nit;
}

// spinAcc::solve / compute (src/spinAccumulationSolver.cpp:130-287): operator with m of
// CURRENT (calcOffDiagBlock), RHS with m of NEXT (getNode_u); s = 0 when it fails.
void spin_solve(Oracle &o) {
    const TetRule &R = o.tr;
    const int N = 4;
    Csr K = shape(o, 3);
    std::vector<double> L(3 * (size_t)o.nn, 0.0), xd(3 * (size_t)o.nn, 0.0);
    for (int t = 0; t < o.nt; t++) {
        const Region &p = o.reg[o.tet_reg[t]];
        const double *da = &o.da[12 * t];
        const double *w = &o.wt[(size_t)t * R.npi];
        const int *ind = &o.tet[4 * t];
        const double D0 = 2.0 * p.sigma / (sq(QE) * p.N0);
        double aw[4] = {0, 0, 0, 0}, wsum = 0;
        for (int i = 0; i < 4; i++)
            for (int g = 0; g < R.npi; g++) aw[i] += R.a[i][g] * w[g];
        for (int g = 0; g < R.npi; g++) wsum += w[g];
        double AE[12][12] = {};
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 4; j++) {
                double v = (da[3 * i] * da[3 * j] + da[3 * i + 1] * da[3 * j + 1] + da[3 * i + 2] * da[3 * j + 2]) *
                           (D0 * wsum);
                if (i == j) v += (D0 / sq(p.lsf)) * aw[i];
                for (int d = 0; d < 3; d++) AE[d * N + i][d * N + j] += v;
            }
        double BE[12] = {};
        if (p.Ms > 0) {
            const double itsd = D0 / sq(p.lsd);
            for (int i = 0; i < 4; i++) {
                const V3 m = o.node[ind[i]].u[CUR];
                const double dx = itsd * aw[i] * m.x, dy = itsd * aw[i] * m.y, dz = itsd * aw[i] * m.z;
                AE[N + i][2 * N + i] += dx;
                AE[2 * N + i][N + i] -= dx;
                AE[i][2 * N + i] -= dy;
                AE[2 * N + i][i] += dy;
                AE[i][N + i] += dz;
                AE[N + i][i] -= dz;
            }
            const double cst0 = MUB * p.P * p.sigma / QE;
            V3 gV = {0, 0, 0};
            for (int i = 0; i < 4; i++) gV = gV + o.Vpot[ind[i]] * v3(&da[3 * i]);
            for (int g = 0; g < R.npi; g++) {
                const V3 c = (cst0 * w[g]) * gV;
                for (int i = 0; i < 4; i++) {
                    const V3 m = o.node[ind[i]].u[NXT];
                    const double tmp = dot(c, v3(&da[3 * i]));
                    BE[i] += tmp * m.x;
                    BE[N + i] += tmp * m.y;
                    BE[2 * N + i] += tmp * m.z;
                }
            }
        }
        for (int a = 0; a < 12; a++) {
            for (int b = 0; b < 12; b++)
                if (AE[a][b] != 0.0) K.add(3 * ind[a % N] + a / N, 3 * ind[b % N] + b / N, AE[a][b]);
            L[3 * (size_t)ind[a % N] + a / N] += BE[a];
        }
    }
    for (int f = 0; f < o.nf; f++) {
        const TriRegion &g = o.treg[o.tri_reg[f]];
        double sv[3] = {g.s[0], g.s[1], g.s[2]};
        if (std::isfinite(g.jn) && finite3(g.uP))
            for (int d = 0; d < 3; d++) sv[d] = -g.jn * (MUB / QE) * g.uP[d];
        if (!finite3(sv)) continue;
        for (int q = 0; q < o.fr.npi; q++) {
            const double wq = o.tri_w[(size_t)f * o.fr.npi + q];
            for (int i = 0; i < 3; i++) {
                const double aiw = wq * o.fr.a[i][q];
                for (int d = 0; d < 3; d++) L[3 * (size_t)o.tri[3 * f + i] + d] -= sv[d] * aiw;
            }
        }
    }
    std::vector<int> ld;
    for (int f = 0; f < o.nf; f++) {
        const TriRegion &g = o.treg[o.tri_reg[f]];
        double sv[3];
        if (!finite3(g.s) && std::isfinite(g.jn)) {
            for (int d = 0; d < 3; d++) sv[d] = -g.jn * (MUB / QE) * g.uP[d];
        } else if (finite3(g.s) && std::isnan(g.jn)) {
            for (int d = 0; d < 3; d++) sv[d] = g.s[d];
        } else {
            continue;
        }
        for (int i = 0; i < 3; i++)
            for (int d = 0; d < 3; d++) {
                xd[3 * (size_t)o.tri[3 * f + i] + d] = sv[d];
                ld.push_back(3 * o.tri[3 * f + i] + d);
            }
    }
    std::sort(ld.begin(), ld.end());
    ld.erase(std::unique(ld.begin(), ld.end()), ld.end());
    std::vector<double> X(3 * (size_t)o.nn, 0.0);
    Iter it;
    it.resmax = o.spin_tol;
    it.maxiter = o.spin_maxiter;
    bicg_dir_values(K, X, L, xd, ld, it);
    o.spin_status = it.status;
    o.spin_nit = it.nit;
    o.sacc.assign(o.nn, {0, 0, 0});
    if (it.status == 0)
        for (int i = 0; i < o.nn; i++) o.sacc[i] = {X[3 * i], X[3 * i + 1], X[3 * i + 2]};
}

// Fem::compute_all (src/fem.h:203-224): demag of m and v, the spin accumulation when
// enabled, energies, CURRENT <- NEXT.
void compute_all(Oracle &o, const double Hext[3], bool first_order) {
    demag_direct(o, 0);
    if (!first_order) demag_direct(o, 1);
    if (o.spin) spin_solve(o);
    energy(o, Hext);
    for (auto &nd : o.node) {
        nd.u[CUR] = nd.u[NXT];
        nd.v[CUR] = nd.v[NXT];
        nd.phi[CUR] = nd.phi[NXT];
        nd.phiv[CUR] = nd.phiv[NXT];
    }
}

// mesh::avg (src/mesh.cpp:89-106), all magnetic regions, NEXT u (which=0) or v (which=1).
double avg(const Oracle &o, int which, int d) {
    double sum = 0;
    for (int t : o.magTet) {
        const int *ind = &o.tet[4 * t];
        for (int g = 0; g < o.tr.npi; g++) {
            double val = 0;
            for (int i = 0; i < 4; i++) {
                const Node &nd = o.node[ind[i]];
                val += o.tr.a[i][g] * comp(which ? nd.v[NXT] : nd.u[NXT], d);
            }
            sum += o.wt[(size_t)t * o.tr.npi + g] * val;
        }
    }
    return sum / o.totalMagVol;
}

// Fem::recenter (src/recentering.cpp:47-131) with a brute-force nearest node (the
// reference's ANN kd-tree; equal distances go to the lower node index). Returns 1 when the
// pattern was translated, 0 when |<u_dir>| < threshold, -1 when there is no domain wall.
int recenter(Oracle &o, int dir, double thres) {
    thres = std::fabs(thres);
    const double m_i = avg(o, 0, dir);
    if (std::fabs(m_i) < thres) return 0;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (const Node &nd : o.node)
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], comp(nd.p, a));
            hi[a] = std::max(hi[a], comp(nd.p, a));
        }
    double c[3], l[3];
    for (int a = 0; a < 3; a++) {
        l[a] = hi[a] - lo[a];
        c[a] = 0.5 * (hi[a] + lo[a]);
    }
    auto nearest = [&](const double q[3]) {
        int best = -1;
        double bd = 1e300;
        for (int j = 0; j < o.nn; j++) {
            const double dx = q[0] - o.node[j].p.x, dy = q[1] - o.node[j].p.y, dz = q[2] - o.node[j].p.z;
            const double d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < bd) {
                bd = d2;
                best = j;
            }
        }
        return best;
    };
    double qL[3] = {c[0], c[1], c[2]}, qR[3] = {c[0], c[1], c[2]};
    qL[dir] -= 0.5 * l[dir];
    qR[dir] += 0.5 * l[dir];
    const double u2L = comp(o.node[nearest(qL)].u[NXT], dir), u2R = comp(o.node[nearest(qR)].u[NXT], dir);
    if (u2L * u2R > 0) return -1;
    const double D = m_i * 0.5 * l[dir] * u2L;
    for (int i = 0; i < o.nn; i++) {
        double p[3] = {o.node[i].p.x, o.node[i].p.y, o.node[i].p.z};
        p[dir] += D;
        if (p[dir] - c[dir] > +0.5 * l[dir]) {
            for (int a = 0; a < 3; a++) p[a] = c[a];
            p[dir] += 0.5 * l[dir];
        }
        if (p[dir] - c[dir] < -0.5 * l[dir]) {
            for (int a = 0; a < 3; a++) p[a] = c[a];
            p[dir] -= 0.5 * l[dir];
        }
        o.node[i].u[CUR] = o.node[nearest(p)].u[NXT];
        o.node[i].v[NXT] = {0, 0, 0};
    }
    return 1;
}

// timing (src/time_integration.h:10-42)
struct Timing {
    double tf, DTMIN, DTMAX, TAUR, t = 0, dt = 0, prefactor = 1;
    void set_dt(double d) {
        dt = d;
        double tt = d / TAUR;
        prefactor = 1. + tt * std::fabs(std::log(tt));
    }
};

// TimeStepper (src/time_integration.cpp:11-38)
struct Stepper {
    double hard_min, hard_max, soft_max;
    void set_soft_limit(double m) { soft_max = std::min(soft_max, m); }
    double operator()(double stride) {
        double step = std::min(stride, soft_max);
        if (step > stride - 2 * hard_min && step < stride) step = stride - 2 * hard_min;
        soft_max = std::max(soft_max, std::min(step * 1.1, hard_max));
        return step;
    }
};

double draw_angle() {
    // LinAlgebra::base_projection (src/linear_algebra.cpp:3-11)
    std::mt19937 gen(rand());
    std::uniform_real_distribution<> distrib(0.0, 1.0);
    double r = distrib(gen);
    return M_2_PI * r;
}

void base_projection(Oracle &o, double angle) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < o.nn; i++) set_basis(o.node[i], angle);
}

}  // namespace

// ===================================================================================
// C API (ctypes). All arrays are host arrays; indices are 0-based and in the sorted
// node numbering produced by the mesh set-up.
extern "C" {

struct fgo_region {
    double A, Ms, K, uk[3], K3, ex[3], ey[3], ez[3], alpha;
    double sigma, N0, P, lsd, lsf;
};
struct fgo_tri_region {
    double Ks, uk[3];
    int suppress_charges;
    double jn, V, uP[3], s[3];
};

void *fgo_create(int nn, const double *xyz, int nt, const int *tet, const int *tet_reg, int nf, const int *tri,
                 const int *tri_reg, const double *tri_dMs, int nreg, const fgo_region *regs, int ntreg,
                 const fgo_tri_region *tregs, int one_gauss_point) {
    Oracle *o = new Oracle();
    o->tr = make_tet_rule(one_gauss_point != 0);
    o->fr = make_tri_rule(one_gauss_point != 0);
    o->nn = nn;
    o->nt = nt;
    o->nf = nf;
    o->node.resize(nn);
    for (int i = 0; i < nn; i++) {
        Node &nd = o->node[i];
        nd.p = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        nd.ep = nd.eq = {0, 0, 0};
        for (int k = 0; k < 2; k++) {
            nd.u[k] = nd.v[k] = {0, 0, 0};
            nd.phi[k] = nd.phiv[k] = 0;
        }
    }
    o->tet.assign(tet, tet + 4 * (size_t)nt);
    o->tet_reg.assign(tet_reg, tet_reg + nt);
    o->tri.assign(tri, tri + 3 * (size_t)nf);
    o->tri_reg.assign(tri_reg, tri_reg + nf);
    o->tri_dMs.assign(tri_dMs, tri_dMs + nf);
    for (int r = 0; r < nreg; r++) {
        Region g;
        std::memcpy(&g, &regs[r], sizeof(Region));
        o->reg.push_back(g);
    }
    for (int r = 0; r < ntreg; r++) {
        TriRegion g;
        g.Ks = tregs[r].Ks;
        for (int k = 0; k < 3; k++) g.uk[k] = tregs[r].uk[k];
        g.suppress_charges = tregs[r].suppress_charges;
        g.jn = tregs[r].jn;
        g.V = tregs[r].V;
        for (int k = 0; k < 3; k++) {
            g.uP[k] = tregs[r].uP[k];
            g.s[k] = tregs[r].s[k];
        }
        o->treg.push_back(g);
    }
    build_geometry(*o);
    build_pattern(*o);
    return o;
}

void fgo_destroy(void *h) {
    Oracle *o = static_cast<Oracle *>(h);
    if (o->fmm) fgo_fmm_destroy(o->fmm);
    delete o;
}

// Demag evaluator: levels 0 = exact direct sum, > 0 = CPU FMM with that tree depth
// (5 reproduces ScalFMM's NbLevels = 6 of the reference: 32^3 leaves).
void fgo_set_demag(void *h, int levels) {
    Oracle *o = static_cast<Oracle *>(h);
    if (o->fmm) { fgo_fmm_destroy(o->fmm); o->fmm = nullptr; }
    o->fmm_levels = levels;
}

void fgo_set_threads(void *h, int n) {
    static_cast<Oracle *>(h)->nthreads = n;
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}

int fgo_max_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int fgo_recenter(void *h, int dir, double threshold) { return recenter(*static_cast<Oracle *>(h), dir, threshold); }

// Spin accumulation on (the potential is solved here, once) or off; status and iterations of
// the potential solve are returned.
void fgo_set_spin(void *h, int enable, double tol, int maxiter, int *v_status, int *v_iters) {
    Oracle *o = static_cast<Oracle *>(h);
    o->spin = enable != 0;
    o->spin_tol = tol;
    o->spin_maxiter = maxiter;
    o->sacc.clear();
    if (o->spin) electrostat(*o);
    if (v_status) *v_status = o->V_status;
    if (v_iters) *v_iters = o->V_nit;
}

// V[nn], s[3 nn] (either may be NULL), last spin solve status and iterations.
void fgo_get_spin(void *h, double *V, double *s, int *status, int *iters) {
    Oracle *o = static_cast<Oracle *>(h);
    if (V && !o->Vpot.empty()) std::memcpy(V, o->Vpot.data(), sizeof(double) * o->nn);
    if (s)
        for (int i = 0; i < o->nn; i++) {
            const V3 v = o->sacc.empty() ? V3{0, 0, 0} : o->sacc[i];
            s[3 * i] = v.x;
            s[3 * i + 1] = v.y;
            s[3 * i + 2] = v.z;
        }
    if (status) *status = o->spin_status;
    if (iters) *iters = o->spin_nit;
}

// R4toR3 field: f at the Gauss points of the magnetic tets, [n_mag_tets][npi][3] in magTet
// order (NULL removes it), and its amplitude A(t).
void fgo_set_space_field(void *h, const double *field, double amp) {
    Oracle *o = static_cast<Oracle *>(h);
    o->amp = amp;
    if (!field) {
        o->hsp.clear();
        return;
    }
    const int npi = o->tr.npi;
    o->hsp.assign(3 * (size_t)o->nt * npi, 0.0);
    for (size_t k = 0; k < o->magTet.size(); k++)
        for (int q = 0; q < 3 * npi; q++) o->hsp[3 * (size_t)o->magTet[k] * npi + q] = field[3 * k * npi + q];
}

// LinAlgebra::set_DW_vz (src/linear_algebra.h:97-98) and the recentering direction
void fgo_set_drift(void *h, int dir, double vdrift) {
    Oracle *o = static_cast<Oracle *>(h);
    o->drift_dir = (dir >= 0 && dir < 3) ? dir : -1;
    o->drift_v = vdrift;
}

void fgo_set_solver(void *h, double tol, int maxiter) {
    Oracle *o = static_cast<Oracle *>(h);
    o->tol = tol;
    o->maxiter = maxiter;
}

// Sets both CURRENT and NEXT node data (u, v, phi, phiv; v/phi/phiv may be NULL = 0).
void fgo_set_state(void *h, const double *u, const double *v, const double *phi, const double *phiv) {
    Oracle *o = static_cast<Oracle *>(h);
    for (int i = 0; i < o->nn; i++) {
        Node &nd = o->node[i];
        V3 uu = v3(&u[3 * i]);
        V3 vv = v ? v3(&v[3 * i]) : V3{0, 0, 0};
        for (int k = 0; k < 2; k++) {
            nd.u[k] = uu;
            nd.v[k] = vv;
            nd.phi[k] = phi ? phi[i] : 0.0;
            nd.phiv[k] = phiv ? phiv[i] : 0.0;
        }
    }
}

// which: 0 = CURRENT, 1 = NEXT. Any output may be NULL.
void fgo_get_state(void *h, int which, double *u, double *v, double *phi, double *phiv) {
    Oracle *o = static_cast<Oracle *>(h);
    for (int i = 0; i < o->nn; i++) {
        const Node &nd = o->node[i];
        if (u) { u[3 * i] = nd.u[which].x; u[3 * i + 1] = nd.u[which].y; u[3 * i + 2] = nd.u[which].z; }
        if (v) { v[3 * i] = nd.v[which].x; v[3 * i + 1] = nd.v[which].y; v[3 * i + 2] = nd.v[which].z; }
        if (phi) phi[i] = nd.phi[which];
        if (phiv) phiv[i] = nd.phiv[which];
    }
}

void fgo_get_basis(void *h, double *ep, double *eq) {
    Oracle *o = static_cast<Oracle *>(h);
    for (int i = 0; i < o->nn; i++) {
        const Node &nd = o->node[i];
        ep[3 * i] = nd.ep.x; ep[3 * i + 1] = nd.ep.y; ep[3 * i + 2] = nd.ep.z;
        eq[3 * i] = nd.eq.x; eq[3 * i + 1] = nd.eq.y; eq[3 * i + 2] = nd.eq.z;
    }
}

void fgo_base_projection(void *h, double angle) { base_projection(*static_cast<Oracle *>(h), angle); }

// prepareElements + solve (+ update on success). Returns 1 on failure (solve returned true).
int fgo_step(void *h, double dt, double prefactor, const double *Hext, int *status, int *iters, double *vmax,
             double *res, double *rhsn) {
    Oracle *o = static_cast<Oracle *>(h);
    prepare_elements(*o, dt, prefactor, Hext);
    bool fail = solve(*o, dt);
    if (status) *status = o->status;
    if (iters) *iters = o->nit;
    if (vmax) *vmax = o->vmax;
    if (res) *res = o->res;
    if (rhsn) *rhsn = o->rhsn;
    return fail ? 1 : 0;
}

void fgo_compute_all(void *h, const double *Hext, int first_order, double *E4) {
    Oracle *o = static_cast<Oracle *>(h);
    compute_all(*o, Hext, first_order != 0);
    if (E4)
        for (int k = 0; k < 4; k++) E4[k] = o->E[k];
}

// Demag potential of the NEXT field (which: 0 = u -> phi, 1 = v -> phiv), written to out[nn].
void fgo_demag(void *h, int which, double *out) {
    Oracle *o = static_cast<Oracle *>(h);
    demag_direct(*o, which);
    for (int i = 0; i < o->nn; i++) out[i] = which ? o->node[i].phiv[NXT] : o->node[i].phi[NXT];
}

// Source points, charges and triangle corrections of the NEXT field.
int fgo_num_sources(void *h) {
    Oracle *o = static_cast<Oracle *>(h);
    return (int)(o->magTet.size() * o->tr.npi + o->magTri.size() * o->fr.npi);
}
void fgo_charges(void *h, int which, double *pts, double *q, double *corr) {
    Oracle *o = static_cast<Oracle *>(h);
    std::vector<double> P, Q, C;
    source_points(*o, P);
    charges(*o, which, P, Q, C);
    if (pts) std::memcpy(pts, P.data(), P.size() * sizeof(double));
    if (q) std::memcpy(q, Q.data(), Q.size() * sizeof(double));
    if (corr) std::memcpy(corr, C.data(), C.size() * sizeof(double));
}

void fgo_energy(void *h, const double *Hext, double *E4) {
    Oracle *o = static_cast<Oracle *>(h);
    energy(*o, Hext);
    for (int k = 0; k < 4; k++) E4[k] = o->E[k];
}

double fgo_avg(void *h, int which, int d) { return avg(*static_cast<Oracle *>(h), which, d); }

int fgo_nnz(void *h) { return (int)static_cast<Oracle *>(h)->col.size(); }

// Assembled system of the last fgo_step (after mask) and the element matrices.
void fgo_export_system(void *h, int *rowptr, int *col, double *val, double *rhs) {
    Oracle *o = static_cast<Oracle *>(h);
    if (rowptr) std::memcpy(rowptr, o->rowptr.data(), o->rowptr.size() * sizeof(int));
    if (col) std::memcpy(col, o->col.data(), o->col.size() * sizeof(int));
    if (val) std::memcpy(val, o->val.data(), o->val.size() * sizeof(double));
    if (rhs) std::memcpy(rhs, o->rhs.data(), o->rhs.size() * sizeof(double));
}
void fgo_export_elements(void *h, double *Kp, double *Lp) {
    Oracle *o = static_cast<Oracle *>(h);
    if (Kp) std::memcpy(Kp, o->Kp.data(), o->Kp.size() * sizeof(double));
    if (Lp) std::memcpy(Lp, o->Lp.data(), o->Lp.size() * sizeof(double));
}
void fgo_export_solution(void *h, double *Xw) {
    Oracle *o = static_cast<Oracle *>(h);
    std::memcpy(Xw, o->Xw.data(), o->Xw.size() * sizeof(double));
}

// glibc rand() stream (main.cpp:211 srand) and the per-step basis angle draw.
void fgo_srand(unsigned int seed) { srand(seed); }
double fgo_draw_angle() { return draw_angle(); }

// Fem::time_integration (src/time_integration.cpp:136-250) with a constant applied
// field and no recentering/spin accumulation. Writes one row per visible step into
// rows[max_rows][8] = t, <Mx>, <My>, <Mz>, E_ex, E_demag, E_zeeman, E_tot (the default
// evol columns, src/default-settings.yml:63-71). Returns the number of rows, or -1 if
// aborted (dt < DTMIN). Counts accepted steps in *nsteps.
int fgo_time_integration(void *h, unsigned int seed, double tf, double dtmin, double dtmax, double evol_step,
                         double dumax, const double *Hext, int first_order, double *rows, int max_rows,
                         int *nsteps, double *Eaniso_out) {
    Oracle *o = static_cast<Oracle *>(h);
    srand(seed);
    Timing tp{tf, dtmin, dtmax, 100. * dtmax};
    tp.set_dt(std::sqrt(dtmin * dtmax));
    // LinAlgebra constructor calls base_projection() once (src/linear_algebra.h:40-65)
    base_projection(*o, draw_angle());
    compute_all(*o, Hext, first_order != 0);
    const double t_initial = tp.t;
    const int step_count = (int)std::lround((tp.tf - t_initial) / evol_step);
    Stepper st{dtmin, dtmax * (1 + 1.1920928955078125e-07), tp.dt};
    int nrow = 0, nt = 0, status = 0;
    for (int step_nb = 0; step_nb <= step_count; step_nb++) {
        double t_target = t_initial + step_nb * evol_step;
        while (tp.t < t_target) {
            tp.set_dt(st(t_target - tp.t));
            bool last_step = (tp.dt == t_target - tp.t);
            if (tp.dt < tp.DTMIN) {
                status = 1;
                goto bailout;
            }
            base_projection(*o, draw_angle());
            prepare_elements(*o, tp.dt, tp.prefactor, Hext);
            bool err = solve(*o, tp.dt);
            double vmax = o->vmax;
            if (err) {
                st.set_soft_limit(tp.dt / 2);
                continue;
            }
            double dumaxv = tp.dt * vmax;
            st.set_soft_limit((dumax / vmax) * 0.95);
            if (dumaxv > dumax) continue;
            compute_all(*o, Hext, first_order != 0);
            nt++;
            if (last_step) tp.t = t_target; else tp.t += tp.dt;
        }
        if (nrow < max_rows) {
            double *r = &rows[8 * nrow];
            r[0] = tp.t;
            r[1] = avg(*o, 0, 0);
            r[2] = avg(*o, 0, 1);
            r[3] = avg(*o, 0, 2);
            r[4] = o->E[0];
            r[5] = o->E[2];
            r[6] = o->E[3];
            r[7] = o->E[0] + o->E[1] + o->E[2] + o->E[3];
            if (Eaniso_out) Eaniso_out[nrow] = o->E[1];
        }
        nrow++;
    }
bailout:
    if (nsteps) *nsteps = nt;
    return status ? -1 : nrow;
}

}  // extern "C"
