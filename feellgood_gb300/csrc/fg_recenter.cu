// Recentering (Fem::recenter, src/recentering.cpp:47-131): when the average magnetisation
// along the direction exceeds a threshold, the whole pattern is translated by
// D = <m_dir> (l_dir / 2) u_dir(left frontier) so that the domain wall comes back to the
// centre: every node takes the magnetisation of the node nearest to its shifted position.
// The reference looks nodes up in an ANN kd-tree; here a uniform grid of cells over the
// mesh's bounding box (built once) answers all nearest-node queries in one kernel, exactly
// (shells of cells around the query until no unvisited cell can hold a closer node; equal
// distances go to the lower node index).
#include <algorithm>
#include <cmath>
#include <vector>

#include "fg_internal.h"

namespace fg {

namespace {

struct NnGrid {
    double lo[3], h[3];
    int n[3];
    int *start = nullptr;  // [ncell + 1]
    int *node = nullptr;   // nodes sorted by cell, then index
    double *xyz = nullptr; // copy of the node positions
};

__device__ int nearest_node(const NnGrid g, double px, double py, double pz) {
    const double p[3] = {px, py, pz};
    int ci[3];
#pragma unroll
    for (int a = 0; a < 3; a++) ci[a] = min(g.n[a] - 1, max(0, (int)floor((p[a] - g.lo[a]) / g.h[a])));
    double best = INFINITY;
    int bj = -1;
    const int rmax = max(g.n[0], max(g.n[1], g.n[2]));
    for (int r = 0; r <= rmax; r++) {
        // the cells at Chebyshev distance r from the query's cell
        for (int iz = ci[2] - r; iz <= ci[2] + r; iz++) {
            if (iz < 0 || iz >= g.n[2]) continue;
            for (int iy = ci[1] - r; iy <= ci[1] + r; iy++) {
                if (iy < 0 || iy >= g.n[1]) continue;
                for (int ix = ci[0] - r; ix <= ci[0] + r; ix++) {
                    if (ix < 0 || ix >= g.n[0]) continue;
                    if (max(abs(ix - ci[0]), max(abs(iy - ci[1]), abs(iz - ci[2]))) != r) continue;
                    const int cell = (iz * g.n[1] + iy) * g.n[0] + ix;
                    for (int k = g.start[cell]; k < g.start[cell + 1]; k++) {
                        const int j = g.node[k];
                        const double dx = px - g.xyz[3 * j], dy = py - g.xyz[3 * j + 1], dz = pz - g.xyz[3 * j + 2];
                        const double d2 = dx * dx + dy * dy + dz * dz;
                        if (d2 < best || (d2 == best && j < bj)) {
                            best = d2;
                            bj = j;
                        }
                    }
                }
            }
        }
        // distance from the query to the outside of the block of cells visited so far
        bool all = true;
        double bound = INFINITY;
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const int c0 = ci[a] - r, c1 = ci[a] + r;
            if (c0 > 0) bound = fmin(bound, p[a] - (g.lo[a] + c0 * g.h[a]));
            if (c1 < g.n[a] - 1) bound = fmin(bound, (g.lo[a] + (c1 + 1) * g.h[a]) - p[a]);
            all = all && c0 <= 0 && c1 >= g.n[a] - 1;
        }
        if (all || (bj >= 0 && bound > 0 && best <= bound * bound)) break;
    }
    return bj;
}

// Every node takes u (NEXT) of the node nearest to its position shifted by D along dir
// (clamped to the box as the reference does) into CURRENT; NEXT v is set to zero
// (mesh::set_node_u0, mesh::set_node_zero_v).
__global__ void k_recenter(int nn, NnGrid g, int dir, double D, double c0, double c1, double c2, double ldir,
                           const double *__restrict__ u1, double *__restrict__ u0, double *__restrict__ v1) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nn) return;
    double p[3] = {g.xyz[3 * i], g.xyz[3 * i + 1], g.xyz[3 * i + 2]};
    p[dir] += D;
    const double cc[3] = {c0, c1, c2};
    if (p[dir] - cc[dir] > 0.5 * ldir) {
        p[0] = cc[0]; p[1] = cc[1]; p[2] = cc[2];
        p[dir] += 0.5 * ldir;
    }
    if (p[dir] - cc[dir] < -0.5 * ldir) {
        p[0] = cc[0]; p[1] = cc[1]; p[2] = cc[2];
        p[dir] -= 0.5 * ldir;
    }
    const int ns = nearest_node(g, p[0], p[1], p[2]);
    for (int k = 0; k < 3; k++) {
        u0[3 * i + k] = u1[3 * (size_t)ns + k];
        v1[3 * i + k] = 0.0;
    }
}

struct RecenterState {
    NnGrid g;
    double c[3], l[3];
};

int nearest_host(const std::vector<double> &xyz, const double q[3]) {
    int best = -1;
    double bd = INFINITY;
    for (size_t j = 0; j < xyz.size() / 3; j++) {
        const double dx = q[0] - xyz[3 * j], dy = q[1] - xyz[3 * j + 1], dz = q[2] - xyz[3 * j + 2];
        const double d2 = dx * dx + dy * dy + dz * dz;
        if (d2 < bd) {
            bd = d2;
            best = (int)j;
        }
    }
    return best;
}

int recenter_setup(Ctx &c) {
    RecenterState *R = new RecenterState();
    c.recenter = R;
    const int nn = c.nn;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < nn; i++)
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], c.h_xyz[3 * (size_t)i + a]);
            hi[a] = std::max(hi[a], c.h_xyz[3 * (size_t)i + a]);
        }
    // the mesh's centre and extent (src/mesh.h:56-62)
    for (int a = 0; a < 3; a++) {
        R->l[a] = hi[a] - lo[a];
        R->c[a] = 0.5 * (hi[a] + lo[a]);
    }
    // about two nodes per cell
    double vol = 1.0;
    int flat = 0;
    for (int a = 0; a < 3; a++) {
        if (R->l[a] > 0) vol *= R->l[a];
        else flat++;
    }
    const double hc = std::pow(2.0 * vol / std::max(1, nn), 1.0 / (3 - std::min(flat, 2)));
    long ncell = 1;
    for (int a = 0; a < 3; a++) {
        R->g.lo[a] = lo[a];
        R->g.n[a] = std::max(1, std::min(1024, (int)std::ceil(R->l[a] / hc)));
        R->g.h[a] = R->l[a] > 0 ? R->l[a] / R->g.n[a] : 1.0;
        ncell *= R->g.n[a];
    }
    std::vector<std::pair<int, int>> cn(nn);
    for (int i = 0; i < nn; i++) {
        int ci[3];
        for (int a = 0; a < 3; a++)
            ci[a] = std::min(R->g.n[a] - 1,
                             std::max(0, (int)std::floor((c.h_xyz[3 * (size_t)i + a] - lo[a]) / R->g.h[a])));
        cn[i] = {(ci[2] * R->g.n[1] + ci[1]) * R->g.n[0] + ci[0], i};
    }
    std::sort(cn.begin(), cn.end());
    std::vector<int> start(ncell + 1, 0), node(nn);
    for (int i = 0; i < nn; i++) {
        start[cn[i].first + 1]++;
        node[i] = cn[i].second;
    }
    for (long k = 0; k < ncell; k++) start[k + 1] += start[k];
    if (cudaMalloc(&R->g.start, sizeof(int) * (ncell + 1)) != cudaSuccess ||
        cudaMalloc(&R->g.node, sizeof(int) * std::max(1, nn)) != cudaSuccess ||
        cudaMalloc(&R->g.xyz, sizeof(double) * 3 * std::max(1, nn)) != cudaSuccess)
        return FG_ECUDA;
    cudaMemcpy(R->g.start, start.data(), sizeof(int) * (ncell + 1), cudaMemcpyHostToDevice);
    cudaMemcpy(R->g.node, node.data(), sizeof(int) * nn, cudaMemcpyHostToDevice);
    cudaMemcpy(R->g.xyz, c.h_xyz.data(), sizeof(double) * 3 * nn, cudaMemcpyHostToDevice);
    return cudaGetLastError() == cudaSuccess ? FG_OK : FG_ECUDA;
}

}  // namespace

void recenter_free(Ctx &c) {
    RecenterState *R = static_cast<RecenterState *>(c.recenter);
    if (!R) return;
    if (R->g.start) cudaFree(R->g.start);
    if (R->g.node) cudaFree(R->g.node);
    if (R->g.xyz) cudaFree(R->g.xyz);
    delete R;
    c.recenter = nullptr;
}

// Fem::recenter; avg_dir is <u_dir> of NEXT over the magnetic volume (mesh::avg).
int recenter_apply(Ctx &c, int dir, double threshold, double avg_dir, int *shifted) {
    *shifted = 0;
    threshold = std::fabs(threshold);
    if (std::fabs(avg_dir) < threshold) return FG_OK;
    if (!c.recenter) {
        const int s = recenter_setup(c);
        if (s != FG_OK) return s;
    }
    RecenterState *R = static_cast<RecenterState *>(c.recenter);
    double qL[3] = {R->c[0], R->c[1], R->c[2]}, qR[3] = {R->c[0], R->c[1], R->c[2]};
    qL[dir] -= 0.5 * R->l[dir];
    qR[dir] += 0.5 * R->l[dir];
    const int nL = nearest_host(c.h_xyz, qL), nR = nearest_host(c.h_xyz, qR);
    double u2L = 0, u2R = 0;
    if (cudaMemcpy(&u2L, c.u[1] + 3 * (size_t)nL + dir, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&u2R, c.u[1] + 3 * (size_t)nR + dir, sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
        return FG_ECUDA;
    if (u2L * u2R > 0) {
        c.err = "recentering: no domain wall (the two ends have the same magnetisation sign)";
        return FG_EINVAL;
    }
    const double D = avg_dir * 0.5 * R->l[dir] * u2L;
    k_recenter<<<(c.nn + 127) / 128, 128, 0, c.stream>>>(c.nn, R->g, dir, D, R->c[0], R->c[1], R->c[2], R->l[dir],
                                                        c.u[1], c.u[0], c.v[1]);
    if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(c.stream) != cudaSuccess) return FG_ECUDA;
    *shifted = 1;
    return FG_OK;
}

}  // namespace fg
