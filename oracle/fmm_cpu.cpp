// CPU FP64 fast multipole method for the oracle's timed CPU baseline. TEST
// INFRASTRUCTURE ONLY (loaded by tests and bench.py's CPU leg, never by the product).
//
// Stands in for ScalFMM (revision 22b9e4f6cf..., absent here), which fmm::demag calls
// with order P = 9 and NbLevels = 6, i.e. a uniform octree with 32^3 leaves over the
// normalised box (src/fmm_demag.h:26-28, 52-53, 184-224). Same potential: the sum over
// all Gauss-point sources of q / |x - y| at every magnetic node. Expansions in scaled
// solid harmonics of degree <= P (complex, m >= 0 stored), translations by the addition
// theorems, one-cell separation; P2P exact in FP64. Parallel over cells with OpenMP.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

using cd = std::complex<double>;
constexpr int P = 9;
constexpr int NC = (P + 1) * (P + 2) / 2;
constexpr int NC2 = (2 * P + 1) * (2 * P + 2) / 2;
inline int ci(int n, int m) { return n * (n + 1) / 2 + m; }

// regular harmonics Ups_n^m(r) = (-1)^m r^n P_n^m e^{im phi}/(n+m)! (P_n^m with Condon-Shortley phase)
void ups(double x, double y, double z, int p, cd *U) {
    const double r2 = x * x + y * y + z * z;
    const cd w(x, y);
    U[0] = 1.0;
    for (int m = 0; m <= p; m++) {
        if (m > 0) U[ci(m, m)] = w / (2.0 * m) * U[ci(m - 1, m - 1)];
        if (m + 1 <= p) U[ci(m + 1, m)] = z * U[ci(m, m)];
        for (int n = m + 2; n <= p; n++)
            U[ci(n, m)] = ((2.0 * n - 1) * z * U[ci(n - 1, m)] - r2 * U[ci(n - 2, m)]) / double((n + m) * (n - m));
    }
}
// irregular harmonics The_n^m(r) = (-1)^m (n-m)! P_n^m e^{im phi} / r^{n+1}
void the(double x, double y, double z, int p, cd *T) {
    const double r2 = x * x + y * y + z * z, ir2 = 1.0 / r2;
    const cd w(x, y);
    T[0] = 1.0 / std::sqrt(r2);
    for (int m = 0; m <= p; m++) {
        if (m > 0) T[ci(m, m)] = (2.0 * m - 1) * w * ir2 * T[ci(m - 1, m - 1)];
        if (m + 1 <= p) T[ci(m + 1, m)] = (2.0 * m + 1) * z * ir2 * T[ci(m, m)];
        for (int n = m + 2; n <= p; n++)
            T[ci(n, m)] = ((2.0 * n - 1) * z * T[ci(n - 1, m)] - double((n + m - 1) * (n - m - 1)) * T[ci(n - 2, m)]) * ir2;
    }
}
inline cd get(const cd *A, int n, int m) {
    if (m >= 0) return A[ci(n, m)];
    const cd v = std::conj(A[ci(n, -m)]);
    return (m & 1) ? -v : v;
}

inline uint64_t key3(int x, int y, int z) { return ((uint64_t)x << 42) | ((uint64_t)y << 21) | (uint64_t)z; }

struct Cell {
    int ijk[3];
    int level;
    int parent;
    std::vector<int> children;
    std::vector<int> m2l;  // source cells
    int src0 = 0, src1 = 0, tgt0 = 0, tgt1 = 0;  // leaves only
    int nsrc = 0, ntgt = 0;
    cd M[NC], F[NC];
};

}  // namespace

struct OracleFmm {
    int L;
    double c0[3], side;
    std::vector<Cell> cells;
    std::vector<std::vector<int>> level_cells;  // indices per level
    std::vector<int> src_perm, tgt_perm;         // sorted position -> original index
    std::vector<double> sxyz, txyz;              // sorted, normalised [0,1)
    std::vector<std::vector<int>> near;          // per leaf cell index: near leaf cells
};

extern "C" {

// Builds the tree for ns sources and nt targets (original coordinates, metres).
void *fgo_fmm_create(int ns, const double *src, int nt, const double *tgt, int levels) {
    OracleFmm *f = new OracleFmm();
    f->L = levels;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int s = 0; s < ns; s++)
        for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], src[3 * s + d]); hi[d] = std::max(hi[d], src[3 * s + d]); }
    for (int s = 0; s < nt; s++)
        for (int d = 0; d < 3; d++) { lo[d] = std::min(lo[d], tgt[3 * s + d]); hi[d] = std::max(hi[d], tgt[3 * s + d]); }
    // the reference normalises by 2/max(l) into a box of width 2.01 (src/fmm_demag.h:52-53, 72)
    double l = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
    f->side = l * 2.01 / 2.0;
    for (int d = 0; d < 3; d++) f->c0[d] = 0.5 * (lo[d] + hi[d]);
    const int n = 1 << levels;
    auto cell_of = [&](const double *p, int *ijk) {
        for (int d = 0; d < 3; d++)
            ijk[d] = std::min(n - 1, std::max(0, (int)(((p[d] - f->c0[d]) / f->side + 0.5) * n)));
    };
    std::vector<std::pair<uint64_t, int>> sk(ns), tk(nt);
    int ijk[3];
    for (int s = 0; s < ns; s++) { cell_of(&src[3 * s], ijk); sk[s] = {key3(ijk[0], ijk[1], ijk[2]), s}; }
    for (int s = 0; s < nt; s++) { cell_of(&tgt[3 * s], ijk); tk[s] = {key3(ijk[0], ijk[1], ijk[2]), s}; }
    std::sort(sk.begin(), sk.end());
    std::sort(tk.begin(), tk.end());
    f->src_perm.resize(ns);
    f->tgt_perm.resize(nt);
    f->sxyz.resize(3 * (size_t)ns);
    f->txyz.resize(3 * (size_t)nt);
    for (int k = 0; k < ns; k++) {
        f->src_perm[k] = sk[k].second;
        for (int d = 0; d < 3; d++) f->sxyz[3 * k + d] = (src[3 * sk[k].second + d] - f->c0[d]) / f->side + 0.5;
    }
    for (int k = 0; k < nt; k++) {
        f->tgt_perm[k] = tk[k].second;
        for (int d = 0; d < 3; d++) f->txyz[3 * k + d] = (tgt[3 * tk[k].second + d] - f->c0[d]) / f->side + 0.5;
    }
    // leaves
    f->level_cells.assign(levels + 1, {});
    std::vector<std::unordered_map<uint64_t, int>> where(levels + 1);
    auto get_cell = [&](int lev, int x, int y, int z) {
        auto it = where[lev].find(key3(x, y, z));
        if (it != where[lev].end()) return it->second;
        Cell c;
        c.ijk[0] = x; c.ijk[1] = y; c.ijk[2] = z;
        c.level = lev;
        c.parent = -1;
        f->cells.push_back(c);
        const int id = (int)f->cells.size() - 1;
        where[lev][key3(x, y, z)] = id;
        f->level_cells[lev].push_back(id);
        return id;
    };
    f->cells.reserve(2 * (ns / 64 + nt / 8 + 16));
    size_t a = 0, b = 0;
    while (a < sk.size() || b < tk.size()) {
        uint64_t k = ~0ull;
        if (a < sk.size()) k = std::min(k, sk[a].first);
        if (b < tk.size()) k = std::min(k, tk[b].first);
        const int x = (int)(k >> 42), y = (int)((k >> 21) & 0x1fffff), z = (int)(k & 0x1fffff);
        const int id = get_cell(levels, x, y, z);
        f->cells[id].src0 = (int)a;
        while (a < sk.size() && sk[a].first == k) a++;
        f->cells[id].src1 = (int)a;
        f->cells[id].tgt0 = (int)b;
        while (b < tk.size() && tk[b].first == k) b++;
        f->cells[id].tgt1 = (int)b;
        f->cells[id].nsrc = f->cells[id].src1 - f->cells[id].src0;
        f->cells[id].ntgt = f->cells[id].tgt1 - f->cells[id].tgt0;
    }
    for (int lev = levels; lev >= 3; lev--) {
        const std::vector<int> ids = f->level_cells[lev];
        for (int id : ids) {
            const int p = get_cell(lev - 1, f->cells[id].ijk[0] >> 1, f->cells[id].ijk[1] >> 1, f->cells[id].ijk[2] >> 1);
            f->cells[id].parent = p;
            f->cells[p].children.push_back(id);
            f->cells[p].nsrc += f->cells[id].nsrc;
            f->cells[p].ntgt += f->cells[id].ntgt;
        }
    }
    for (int lev = 2; lev <= levels; lev++) {
        const int nl = 1 << lev;
        for (int id : f->level_cells[lev]) {
            Cell &c = f->cells[id];
            if (c.ntgt == 0) continue;
            const int px = c.ijk[0] >> 1, py = c.ijk[1] >> 1, pz = c.ijk[2] >> 1;
            for (int x = 2 * (px - 1); x <= 2 * px + 3; x++)
                for (int y = 2 * (py - 1); y <= 2 * py + 3; y++)
                    for (int z = 2 * (pz - 1); z <= 2 * pz + 3; z++) {
                        if (x < 0 || y < 0 || z < 0 || x >= nl || y >= nl || z >= nl) continue;
                        if (std::abs(x - c.ijk[0]) <= 1 && std::abs(y - c.ijk[1]) <= 1 && std::abs(z - c.ijk[2]) <= 1) continue;
                        auto it = where[lev].find(key3(x, y, z));
                        if (it == where[lev].end() || f->cells[it->second].nsrc == 0) continue;
                        c.m2l.push_back(it->second);
                    }
        }
    }
    f->near.assign(f->cells.size(), {});
    for (int id : f->level_cells[levels]) {
        Cell &c = f->cells[id];
        if (c.ntgt == 0) continue;
        for (int dx = -1; dx <= 1; dx++)
            for (int dy = -1; dy <= 1; dy++)
                for (int dz = -1; dz <= 1; dz++) {
                    auto it = where[levels].find(key3(c.ijk[0] + dx, c.ijk[1] + dy, c.ijk[2] + dz));
                    if (c.ijk[0] + dx < 0 || c.ijk[1] + dy < 0 || c.ijk[2] + dz < 0) continue;
                    if (it == where[levels].end() || f->cells[it->second].nsrc == 0) continue;
                    f->near[id].push_back(it->second);
                }
    }
    return f;
}

void fgo_fmm_destroy(void *h) { delete static_cast<OracleFmm *>(h); }

// pot[target original index] = sum_s q[s] / |x_t - y_s| (metres).
void fgo_fmm_eval(void *h, const double *q, double *pot) {
    OracleFmm &f = *static_cast<OracleFmm *>(h);
    const int L = f.L;
    std::vector<int> &leaves = f.level_cells[L];
    const int nleaf = (int)leaves.size();
    const double wl = 1.0 / (1 << L);
    // P2M at leaves: M_n^m = sum q conj(Ups((y - c)/w))
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < nleaf; k++) {
        Cell &c = f.cells[leaves[k]];
        std::fill(c.M, c.M + NC, cd(0));
        const double cx = (c.ijk[0] + 0.5) * wl, cy = (c.ijk[1] + 0.5) * wl, cz = (c.ijk[2] + 0.5) * wl;
        cd U[NC];
        for (int s = c.src0; s < c.src1; s++) {
            ups((f.sxyz[3 * s] - cx) / wl, (f.sxyz[3 * s + 1] - cy) / wl, (f.sxyz[3 * s + 2] - cz) / wl, P, U);
            const double qq = q[f.src_perm[s]];
            for (int j = 0; j < NC; j++) c.M[j] += qq * std::conj(U[j]);
        }
    }
    // M2M: parent (width w) from children (w/2): sum conj(Ups_k^l(t/w)) 2^-(n-k) M_{n-k}^{m-l}
    for (int lev = L - 1; lev >= 2; lev--) {
        std::vector<int> &ids = f.level_cells[lev];
#pragma omp parallel for schedule(dynamic, 16)
        for (int k = 0; k < (int)ids.size(); k++) {
            Cell &p = f.cells[ids[k]];
            std::fill(p.M, p.M + NC, cd(0));
            for (int ch : p.children) {
                const Cell &c = f.cells[ch];
                if (c.nsrc == 0) continue;
                cd U[NC];
                ups((c.ijk[0] & 1) ? 0.25 : -0.25, (c.ijk[1] & 1) ? 0.25 : -0.25, (c.ijk[2] & 1) ? 0.25 : -0.25, P, U);
                for (int n = 0; n <= P; n++)
                    for (int m = 0; m <= n; m++) {
                        cd s = 0;
                        for (int kk = 0; kk <= n; kk++)
                            for (int l = -kk; l <= kk; l++)
                                if (std::abs(m - l) <= n - kk)
                                    s += std::conj(get(U, kk, l)) * std::ldexp(1.0, -(n - kk)) * get(c.M, n - kk, m - l);
                        p.M[ci(n, m)] += s;
                    }
            }
        }
    }
    // M2L: F_n^m = (-1)^n sum M_k^l The_{n+k}^{m+l}(target - source, cell units)
    for (int lev = 2; lev <= L; lev++) {
        std::vector<int> &ids = f.level_cells[lev];
#pragma omp parallel for schedule(dynamic, 8)
        for (int k = 0; k < (int)ids.size(); k++) {
            Cell &c = f.cells[ids[k]];
            std::fill(c.F, c.F + NC, cd(0));
            cd T[NC2];
            for (int sid : c.m2l) {
                const Cell &s = f.cells[sid];
                the(c.ijk[0] - s.ijk[0], c.ijk[1] - s.ijk[1], c.ijk[2] - s.ijk[2], 2 * P, T);
                for (int n = 0; n <= P; n++)
                    for (int m = 0; m <= n; m++) {
                        cd acc = 0;
                        for (int kk = 0; kk <= P; kk++)
                            for (int l = -kk; l <= kk; l++) acc += get(s.M, kk, l) * get(T, n + kk, m + l);
                        c.F[ci(n, m)] += (n & 1) ? -acc : acc;
                    }
            }
        }
    }
    // L2L: child (w/2) from parent (w): 2^-(k+1) sum_{n>=k} F_n^m conj(Ups_{n-k}^{m-l}(t/w))
    for (int lev = 3; lev <= L; lev++) {
        std::vector<int> &ids = f.level_cells[lev];
#pragma omp parallel for schedule(dynamic, 16)
        for (int k = 0; k < (int)ids.size(); k++) {
            Cell &c = f.cells[ids[k]];
            if (c.ntgt == 0) continue;
            const Cell &p = f.cells[c.parent];
            cd U[NC];
            ups((c.ijk[0] & 1) ? 0.25 : -0.25, (c.ijk[1] & 1) ? 0.25 : -0.25, (c.ijk[2] & 1) ? 0.25 : -0.25, P, U);
            for (int kk = 0; kk <= P; kk++)
                for (int l = 0; l <= kk; l++) {
                    cd s = 0;
                    for (int n = kk; n <= P; n++)
                        for (int m = -n; m <= n; m++)
                            if (std::abs(m - l) <= n - kk) s += get(p.F, n, m) * std::conj(get(U, n - kk, m - l));
                    c.F[ci(kk, l)] += s * std::ldexp(1.0, -(kk + 1));
                }
        }
    }
    // L2P + P2P at leaves
    const double scale = 1.0 / f.side;
#pragma omp parallel for schedule(dynamic, 8)
    for (int k = 0; k < nleaf; k++) {
        const int id = leaves[k];
        Cell &c = f.cells[id];
        const double cx = (c.ijk[0] + 0.5) * wl, cy = (c.ijk[1] + 0.5) * wl, cz = (c.ijk[2] + 0.5) * wl;
        cd U[NC];
        for (int t = c.tgt0; t < c.tgt1; t++) {
            const double x = f.txyz[3 * t], y = f.txyz[3 * t + 1], z = f.txyz[3 * t + 2];
            ups((x - cx) / wl, (y - cy) / wl, (z - cz) / wl, P, U);
            double far = 0;
            for (int n = 0; n <= P; n++) {
                far += (c.F[ci(n, 0)] * std::conj(U[ci(n, 0)])).real();
                for (int m = 1; m <= n; m++) far += 2.0 * (c.F[ci(n, m)] * std::conj(U[ci(n, m)])).real();
            }
            far /= wl;
            double near = 0;
            for (int nl : f.near[id]) {
                const Cell &s = f.cells[nl];
                for (int j = s.src0; j < s.src1; j++) {
                    const double dx = x - f.sxyz[3 * j], dy = y - f.sxyz[3 * j + 1], dz = z - f.sxyz[3 * j + 2];
                    near += q[f.src_perm[j]] / std::sqrt(dx * dx + dy * dy + dz * dz);
                }
            }
            pot[f.tgt_perm[t]] = (far + near) * scale;
        }
    }
}

}  // extern "C"
