// Host-side mesh ingest and set-up (once per mesh, before any time step).
//
// Restates what FeeLLGood does between opening a gmsh file and the first step:
//   gmsh 2.2 / 4.1 ASCII reading as the gmsh API exposes it to mesh::readNodes,
//   readTetraedrons and readTriangles (src/read.cpp:73-197; node index = tag - 1,
//   elements kept when their physical name is a settings region);
//   Tet::orientate (src/tetra.cpp:410-424);
//   mesh::controlTriangles / diffTriHandler / assertNoErrInTriangle (src/mesh.cpp:121-332):
//   creation of missing surface/interface triangles and regions, signed dMs;
//   mesh::sortNodes along the longest axis (src/mesh.cpp:334-367, src/mesh.h:51-79).
// sortNodes uses a stable sort here: the reference's std::sort leaves the order of equal
// coordinates unspecified, and ties only change floating-point summation order.
// Also a structured cuboid generator with the 6-tetrahedra split of
// python-modules/meshMaker.py:470-483 (Cuboid), which writes the same gmsh 2.2 file.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "fg_host.h"

namespace {

struct MeshError {
    int code;
    std::string msg;
};

struct RawMesh {
    std::vector<double> nodes;  // 3 per node (index = tag - 1)
    std::map<std::pair<int, int>, std::string> names;  // (dim, phys tag) -> name
    struct Block {
        int dim, entity, etype;
        std::vector<int> phys;
        std::vector<int> conn;  // node tags (1-based), npe per element
        int npe;
    };
    std::vector<Block> blocks;
};

int npe_of(int etype) {
    switch (etype) {
        case 15: return 1;
        case 1: return 2;
        case 2: return 3;
        case 4: return 4;
        case 3: return 4;
        case 5: return 8;
        case 6: return 6;
        case 7: return 5;
        default: return -1;
    }
}
int dim_of(int etype) {
    switch (etype) {
        case 15: return 0;
        case 1: return 1;
        case 2: case 3: return 2;
        default: return 3;
    }
}

bool seek(std::istream &in, const std::string &tag) {
    std::string line;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line == tag) return true;
    }
    return false;
}

RawMesh read_msh(const std::string &path) {
    std::ifstream in(path);
    if (!in) throw MeshError{FG_EIO, "cannot open mesh file " + path};
    RawMesh r;
    if (!seek(in, "$MeshFormat")) throw MeshError{FG_EMESH, "not a gmsh file: " + path};
    std::string ver;
    int ftype = 0, dsize = 0;
    in >> ver >> ftype >> dsize;
    if (ftype != 0) throw MeshError{FG_EMESH, "binary gmsh files are not supported: " + path};
    const bool v4 = ver[0] == '4';
    in.clear();
    in.seekg(0);
    if (seek(in, "$PhysicalNames")) {
        int n;
        in >> n;
        std::string rest;
        std::getline(in, rest);
        for (int k = 0; k < n; k++) {
            std::getline(in, rest);
            std::istringstream ss(rest);
            int d, t;
            ss >> d >> t;
            std::string name;
            std::getline(ss, name);
            size_t a = name.find('"'), b = name.rfind('"');
            if (a != std::string::npos && b > a) name = name.substr(a + 1, b - a - 1);
            else {
                size_t s = name.find_first_not_of(" \t");
                name = s == std::string::npos ? "" : name.substr(s);
            }
            r.names[{d, t}] = name;
        }
    }
    std::map<std::pair<int, int>, std::vector<int>> ent_phys;
    if (v4) {
        in.clear();
        in.seekg(0);
        if (seek(in, "$Entities")) {
            int cnt[4];
            in >> cnt[0] >> cnt[1] >> cnt[2] >> cnt[3];
            for (int d = 0; d < 4; d++)
                for (int k = 0; k < cnt[d]; k++) {
                    int tag;
                    double x;
                    in >> tag;
                    const int nb = d == 0 ? 3 : 6;
                    for (int q = 0; q < nb; q++) in >> x;
                    int nph;
                    in >> nph;
                    std::vector<int> ph(nph);
                    for (int q = 0; q < nph; q++) in >> ph[q];
                    if (d > 0) {
                        int nbd, b;
                        in >> nbd;
                        for (int q = 0; q < nbd; q++) in >> b;
                    }
                    ent_phys[{d, tag}] = ph;
                }
        }
        in.clear();
        in.seekg(0);
        if (!seek(in, "$Nodes")) throw MeshError{FG_EMESH, "no $Nodes section"};
        long nblk, nnode, mintag, maxtag;
        in >> nblk >> nnode >> mintag >> maxtag;
        r.nodes.assign(3 * (size_t)maxtag, 0.0);
        for (long b = 0; b < nblk; b++) {
            int ed, et, par;
            long m;
            in >> ed >> et >> par >> m;
            std::vector<long> tags(m);
            for (long k = 0; k < m; k++) in >> tags[k];
            for (long k = 0; k < m; k++) {
                double x, y, z;
                in >> x >> y >> z;
                if (par) {
                    double p;
                    for (int q = 0; q < ed; q++) in >> p;
                }
                if (tags[k] < 1 || tags[k] > maxtag) throw MeshError{FG_EMESH, "node tag out of range"};
                r.nodes[3 * (tags[k] - 1)] = x;
                r.nodes[3 * (tags[k] - 1) + 1] = y;
                r.nodes[3 * (tags[k] - 1) + 2] = z;
            }
        }
        in.clear();
        in.seekg(0);
        if (!seek(in, "$Elements")) throw MeshError{FG_EMESH, "no $Elements section"};
        long neb, ne, mn, mx;
        in >> neb >> ne >> mn >> mx;
        for (long b = 0; b < neb; b++) {
            RawMesh::Block B;
            long m;
            in >> B.dim >> B.entity >> B.etype >> m;
            B.npe = npe_of(B.etype);
            if (B.npe < 0) throw MeshError{FG_EMESH, "unsupported gmsh element type " + std::to_string(B.etype)};
            B.phys = ent_phys[{B.dim, B.entity}];
            B.conn.resize((size_t)m * B.npe);
            for (long k = 0; k < m; k++) {
                long tag;
                in >> tag;
                for (int q = 0; q < B.npe; q++) in >> B.conn[(size_t)k * B.npe + q];
            }
            r.blocks.push_back(std::move(B));
        }
        std::stable_sort(r.blocks.begin(), r.blocks.end(),
                         [](const RawMesh::Block &a, const RawMesh::Block &b) {
                             return a.dim != b.dim ? a.dim < b.dim : a.entity < b.entity;
                         });
    } else {
        in.clear();
        in.seekg(0);
        if (!seek(in, "$Nodes")) throw MeshError{FG_EMESH, "no $Nodes section"};
        long n;
        in >> n;
        std::vector<std::pair<long, std::array<double, 3>>> tmp(n);
        long maxtag = 0;
        for (long k = 0; k < n; k++) {
            in >> tmp[k].first >> tmp[k].second[0] >> tmp[k].second[1] >> tmp[k].second[2];
            maxtag = std::max(maxtag, tmp[k].first);
        }
        r.nodes.assign(3 * (size_t)maxtag, 0.0);
        for (auto &p : tmp) {
            if (p.first < 1) throw MeshError{FG_EMESH, "node tag out of range"};
            for (int d = 0; d < 3; d++) r.nodes[3 * (p.first - 1) + d] = p.second[d];
        }
        in.clear();
        in.seekg(0);
        if (!seek(in, "$Elements")) throw MeshError{FG_EMESH, "no $Elements section"};
        long ne;
        in >> ne;
        // gmsh builds one discrete entity per (elementary tag, type); visited by tag
        std::map<std::array<int, 3>, RawMesh::Block> groups;
        for (long k = 0; k < ne; k++) {
            long id;
            int etype, ntags;
            in >> id >> etype >> ntags;
            std::vector<int> tg(ntags);
            for (int q = 0; q < ntags; q++) in >> tg[q];
            const int npe = npe_of(etype);
            if (npe < 0) throw MeshError{FG_EMESH, "unsupported gmsh element type " + std::to_string(etype)};
            const int phys = ntags > 0 ? tg[0] : 0, elem = ntags > 1 ? tg[1] : 0;
            const std::array<int, 3> key = {dim_of(etype), elem, etype};
            RawMesh::Block &B = groups[key];
            B.dim = key[0];
            B.entity = elem;
            B.etype = etype;
            B.npe = npe;
            if (std::find(B.phys.begin(), B.phys.end(), phys) == B.phys.end()) B.phys.push_back(phys);
            for (int q = 0; q < npe; q++) {
                int v;
                in >> v;
                B.conn.push_back(v);
            }
        }
        for (auto &g : groups) {
            std::sort(g.second.phys.begin(), g.second.phys.end());
            r.blocks.push_back(std::move(g.second));
        }
    }
    return r;
}

struct Setup {
    std::vector<double> xyz;
    std::vector<int> tets, tet_reg, tris, tri_reg;
    std::vector<double> dMs;
    std::vector<int> node_index;  // file index -> sorted index
    std::vector<std::string> vol_names, surf_names;
};

void orient(const std::vector<double> &xyz, std::vector<int> &tets) {
    const size_t nt = tets.size() / 4;
    for (size_t t = 0; t < nt; t++) {
        int *ind = &tets[4 * t];
        const double *p0 = &xyz[3 * ind[0]], *p1 = &xyz[3 * ind[1]], *p2 = &xyz[3 * ind[2]], *p3 = &xyz[3 * ind[3]];
        const double a[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
        const double b[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
        const double c[3] = {p3[0] - p0[0], p3[1] - p0[1], p3[2] - p0[2]};
        const double mixed = a[0] * (b[1] * c[2] - b[2] * c[1]) + a[1] * (b[2] * c[0] - b[0] * c[2]) +
                             a[2] * (b[0] * c[1] - b[1] * c[0]);
        if (std::fabs(mixed) < 1e-40) throw MeshError{FG_EMESH, "Singular tetrahedron: mixed product= " + std::to_string(mixed)};
        if (mixed < 0) std::swap(ind[2], ind[3]);
    }
}

struct BasicTri {
    std::array<int, 3> n;
    int reg;
    bool surf, flip;
};
BasicTri basic(int a, int b, int c, int reg, bool surf) {
    BasicTri t{{a, b, c}, reg, surf, false};
    const int inv = (a > b) + (b > c) + (a > c);
    std::sort(t.n.begin(), t.n.end());
    t.flip = inv % 2;
    return t;
}

void control_triangles(Setup &S, const std::vector<double> &Ms) {
    if (S.tets.empty()) throw MeshError{FG_EMESH, "Error: not a single tetrahedron is present in the mesh"};
    const size_t nt = S.tets.size() / 4, nf = S.tris.size() / 3;
    std::vector<BasicTri> all;
    all.reserve(4 * nt + nf);
    for (size_t t = 0; t < nt; t++) {
        const int *i = &S.tets[4 * t];
        const int r = S.tet_reg[t];
        all.push_back(basic(i[0], i[2], i[1], r, false));
        all.push_back(basic(i[1], i[2], i[3], r, false));
        all.push_back(basic(i[2], i[0], i[3], r, false));
        all.push_back(basic(i[3], i[0], i[1], r, false));
    }
    for (size_t f = 0; f < nf; f++) all.push_back(basic(S.tris[3 * f], S.tris[3 * f + 1], S.tris[3 * f + 2], S.tri_reg[f], true));
    std::stable_sort(all.begin(), all.end(), [](const BasicTri &a, const BasicTri &b) { return a.n < b.n; });
    std::vector<std::array<int, 3>> add_nodes;
    std::vector<std::pair<int, int>> add_pairs;
    size_t lo = 0;
    for (size_t up = 1; up <= all.size(); up++) {
        if (up < all.size() && all[up].n == all[lo].n) continue;
        int id_surf = -1, n_faces = 0, n_surf = 0;
        std::pair<int, int> pair(-1, -1);
        for (size_t i = lo; i < up; i++) {
            if (all[i].surf) {
                id_surf = all[i].reg;
                n_surf++;
            } else {
                n_faces++;
                if (all[i].reg > pair.first) {
                    pair.second = pair.first;
                    pair.first = all[i].reg;
                } else pair.second = all[i].reg;
            }
        }
        if (n_surf == 0 && (n_faces == 1 || (n_faces == 2 && pair.first != pair.second))) {
            add_nodes.push_back(all[lo].n);
            add_pairs.push_back(pair);
        }
        if (n_surf > 1)
            throw MeshError{FG_EMESH, "Error: bad mesh. " + std::to_string(n_surf) +
                                          " instances of the same surface triangle have been found"};
        if (n_faces == 0)
            throw MeshError{FG_EMESH, "Error: bad mesh. A triangle which belongs to 1 surface region and no "
                                      "tetrahedron has been found"};
        if (n_faces > 2) {
            if (n_surf == 1)
                throw MeshError{FG_EMESH, "Error: bad mesh. A triangular face shared by " + std::to_string(n_faces) +
                                              " tetrahedrons has been found in the surface region " +
                                              std::to_string(id_surf)};
            throw MeshError{FG_EMESH, "Error: bad mesh. A triangular face shared by " + std::to_string(n_faces) +
                                          " tetrahedrons has been found"};
        }
        if (n_faces == 2 && n_surf == 1 && pair.first == pair.second)
            throw MeshError{FG_EMESH, "Error: bad mesh. An internal triangle has been found in the surface region " +
                                          std::to_string(id_surf)};
        lo = up;
    }
    std::map<std::pair<int, int>, int> pair_reg;
    for (auto &p : add_pairs) {
        if (pair_reg.count(p)) continue;
        std::string base = p.second == -1 ? "surface(" + S.vol_names[p.first] + ")"
                                          : "interface(" + S.vol_names[p.first] + ", " + S.vol_names[p.second] + ")";
        std::string name = base;
        for (int i = 0;; i++) {
            name = i == 0 ? base : base + "." + std::to_string(i);
            if (std::find(S.surf_names.begin(), S.surf_names.end(), name) == S.surf_names.end()) break;
        }
        S.surf_names.push_back(name);
        pair_reg[p] = (int)S.surf_names.size() - 1;
    }
    for (size_t k = 0; k < add_nodes.size(); k++) {
        for (int d = 0; d < 3; d++) S.tris.push_back(add_nodes[k][d]);
        S.tri_reg.push_back(pair_reg[add_pairs[k]]);
    }
    // dMs (src/mesh.cpp:218-232)
    const size_t nf2 = S.tris.size() / 3;
    S.dMs.assign(nf2, 0.0);
    for (size_t f = 0; f < nf2; f++) {
        const BasicTri tb = basic(S.tris[3 * f], S.tris[3 * f + 1], S.tris[3 * f + 2], S.tri_reg[f], true);
        auto it = std::lower_bound(all.begin(), all.end(), tb, [](const BasicTri &a, const BasicTri &b) { return a.n < b.n; });
        for (; it != all.end() && it->n == tb.n; ++it)
            if (!it->surf) {
                const double ms = Ms[it->reg];
                S.dMs[f] += (tb.flip ^ it->flip) ? -ms : ms;
            }
    }
}

void sort_nodes(Setup &S) {
    const size_t nn = S.xyz.size() / 3;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (size_t i = 0; i < nn; i++)
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], S.xyz[3 * i + d]);
            hi[d] = std::max(hi[d], S.xyz[3 * i + d]);
        }
    const double l[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    int axis;
    if (l[0] > l[1]) axis = l[0] > l[2] ? 0 : 2;
    else axis = l[1] > l[2] ? 1 : 2;
    std::vector<int> perm(nn);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(),
                     [&](int a, int b) { return S.xyz[3 * a + axis] < S.xyz[3 * b + axis]; });
    S.node_index.assign(nn, 0);
    for (size_t i = 0; i < nn; i++) S.node_index[perm[i]] = (int)i;
    std::vector<double> xs(3 * nn);
    for (size_t i = 0; i < nn; i++)
        for (int d = 0; d < 3; d++) xs[3 * i + d] = S.xyz[3 * perm[i] + d];
    S.xyz.swap(xs);
    for (int &v : S.tets) v = S.node_index[v];
    for (int &v : S.tris) v = S.node_index[v];
}

fg_mesh_data *publish(Setup &S) {
    fg_mesh_data *d = new fg_mesh_data();
    std::memset(d, 0, sizeof(*d));
    auto dup_d = [](const std::vector<double> &v) {
        double *p = (double *)malloc(sizeof(double) * std::max<size_t>(1, v.size()));
        if (!v.empty()) std::memcpy(p, v.data(), sizeof(double) * v.size());
        return p;
    };
    auto dup_i = [](const std::vector<int> &v) {
        int32_t *p = (int32_t *)malloc(sizeof(int32_t) * std::max<size_t>(1, v.size()));
        for (size_t i = 0; i < v.size(); i++) p[i] = v[i];
        return p;
    };
    d->n_nodes = (int)(S.xyz.size() / 3);
    d->n_tets = (int)(S.tets.size() / 4);
    d->n_tris = (int)(S.tris.size() / 3);
    d->xyz = dup_d(S.xyz);
    d->tet4 = dup_i(S.tets);
    d->tet_region = dup_i(S.tet_reg);
    d->tri3 = dup_i(S.tris);
    d->tri_region = dup_i(S.tri_reg);
    d->tri_dMs = dup_d(S.dMs);
    d->node_index = dup_i(S.node_index);
    d->n_vol_regions = (int)S.vol_names.size();
    d->n_surf_regions = (int)S.surf_names.size();
    d->vol_names = (char **)malloc(sizeof(char *) * d->n_vol_regions);
    d->surf_names = (char **)malloc(sizeof(char *) * std::max(1, d->n_surf_regions));
    for (int k = 0; k < d->n_vol_regions; k++) d->vol_names[k] = strdup(S.vol_names[k].c_str());
    for (int k = 0; k < d->n_surf_regions; k++) d->surf_names[k] = strdup(S.surf_names[k].c_str());
    return d;
}

thread_local std::string g_mesh_error;

int finish(Setup &S, const std::vector<double> &Ms, fg_mesh_data **out) {
    orient(S.xyz, S.tets);
    control_triangles(S, Ms);
    sort_nodes(S);
    *out = publish(S);
    return FG_OK;
}

}  // namespace

extern "C" {

const char *fg_mesh_last_error(void) { return g_mesh_error.c_str(); }

int fg_mesh_load_msh(const char *path, double length_unit, int n_vol, const char *const *vol_names,
                     const double *vol_Ms, int n_surf, const char *const *surf_names, fg_mesh_data **out) {
    if (!path || !out || n_vol < 0 || n_surf < 0 || (n_vol && (!vol_names || !vol_Ms)) || (n_surf && !surf_names) ||
        !(length_unit > 0))
        return FG_EINVAL;
    *out = nullptr;
    try {
        RawMesh r = read_msh(path);
        Setup S;
        S.vol_names.push_back("__default__");
        S.surf_names.push_back("__default__");
        std::vector<double> Ms(1, 0.0);
        for (int k = 0; k < n_vol; k++) {
            S.vol_names.push_back(vol_names[k]);
            Ms.push_back(vol_Ms[k]);
        }
        for (int k = 0; k < n_surf; k++) S.surf_names.push_back(surf_names[k]);
        S.xyz = r.nodes;
        for (double &x : S.xyz) x *= length_unit;
        const int nn = (int)(S.xyz.size() / 3);
        for (auto &B : r.blocks)
            for (int ph : B.phys) {
                auto it = r.names.find({B.dim, ph});
                if (it == r.names.end()) continue;
                const std::string &name = it->second;
                if (B.dim == 3) {
                    auto f = std::find(S.vol_names.begin(), S.vol_names.end(), name);
                    if (f == S.vol_names.end()) continue;
                    if (B.etype != 4)
                        throw MeshError{FG_EMESH, "Fatal error: a volume mesh entity contains other elements than tetraedrons."};
                    const int reg = (int)(f - S.vol_names.begin());
                    for (size_t k = 0; k < B.conn.size(); k++) {
                        if (B.conn[k] < 1 || B.conn[k] > nn) throw MeshError{FG_EMESH, "Error: Tet constructor has out of bound index"};
                        S.tets.push_back(B.conn[k] - 1);
                    }
                    for (size_t k = 0; k < B.conn.size() / 4; k++) S.tet_reg.push_back(reg);
                } else if (B.dim == 2) {
                    auto f = std::find(S.surf_names.begin(), S.surf_names.end(), name);
                    if (f == S.surf_names.end()) continue;
                    if (B.etype != 2)
                        throw MeshError{FG_EMESH, "Fatal error: a surface mesh entity contains other elements than triangles."};
                    const int reg = (int)(f - S.surf_names.begin());
                    for (size_t k = 0; k < B.conn.size(); k++) {
                        if (B.conn[k] < 1 || B.conn[k] > nn) throw MeshError{FG_EMESH, "Error: Tri constructor has out of bound index"};
                        S.tris.push_back(B.conn[k] - 1);
                    }
                    for (size_t k = 0; k < B.conn.size() / 3; k++) S.tri_reg.push_back(reg);
                }
            }
        return finish(S, Ms, out);
    } catch (const MeshError &e) {
        g_mesh_error = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        g_mesh_error = e.what();
        return FG_EMESH;
    }
}

int fg_mesh_cuboid(int nx, int ny, int nz, double lx, double ly, double lz, double length_unit, double Ms,
                   fg_mesh_data **out) {
    if (!out || nx < 1 || ny < 1 || nz < 1 || !(lx > 0) || !(ly > 0) || !(lz > 0) || !(length_unit > 0))
        return FG_EINVAL;
    *out = nullptr;
    try {
        Setup S;
        S.vol_names = {"__default__", "volume"};
        S.surf_names = {"__default__"};
        const double dx = lx / nx, dy = ly / ny, dz = lz / nz;
        auto idx = [&](int i, int j, int k) { return (nz + 1) * (ny + 1) * i + (nz + 1) * j + k; };
        S.xyz.resize(3 * (size_t)(nx + 1) * (ny + 1) * (nz + 1));
        for (int i = 0; i <= nx; i++)
            for (int j = 0; j <= ny; j++)
                for (int k = 0; k <= nz; k++) {
                    const size_t n = idx(i, j, k);
                    S.xyz[3 * n] = (i * dx) * length_unit;
                    S.xyz[3 * n + 1] = (j * dy) * length_unit;
                    S.xyz[3 * n + 2] = (k * dz) * length_unit;
                }
        S.tets.reserve(24 * (size_t)nx * ny * nz);
        for (int i = 0; i < nx; i++)
            for (int j = 0; j < ny; j++)
                for (int k = 0; k < nz; k++) {
                    const int A = idx(i, j, k), B = idx(i + 1, j, k), C = idx(i + 1, j + 1, k), D = idx(i, j + 1, k);
                    const int E = idx(i, j, k + 1), F = idx(i + 1, j, k + 1), G = idx(i + 1, j + 1, k + 1),
                              H = idx(i, j + 1, k + 1);
                    const int t6[6][4] = {{A, B, D, H}, {A, B, E, H}, {E, F, H, B}, {B, C, D, H}, {B, C, G, H}, {F, B, G, H}};
                    for (auto &t : t6)
                        for (int q = 0; q < 4; q++) S.tets.push_back(t[q]);
                }
        S.tet_reg.assign(S.tets.size() / 4, 1);
        return finish(S, std::vector<double>{0.0, Ms}, out);
    } catch (const MeshError &e) {
        g_mesh_error = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        g_mesh_error = e.what();
        return FG_EMESH;
    }
}

void fg_mesh_free(fg_mesh_data *d) {
    if (!d) return;
    free((void *)d->xyz);
    free((void *)d->tet4);
    free((void *)d->tet_region);
    free((void *)d->tri3);
    free((void *)d->tri_region);
    free((void *)d->tri_dMs);
    free((void *)d->node_index);
    for (int k = 0; k < d->n_vol_regions; k++) free(d->vol_names[k]);
    for (int k = 0; k < d->n_surf_regions; k++) free(d->surf_names[k]);
    free(d->vol_names);
    free(d->surf_names);
    delete d;
}

int fg_mesh_view(const fg_mesh_data *d, fg_mesh *m) {
    if (!d || !m) return FG_EINVAL;
    m->n_nodes = d->n_nodes;
    m->n_tets = d->n_tets;
    m->n_tris = d->n_tris;
    m->xyz = d->xyz;
    m->tet4 = d->tet4;
    m->tet_region = d->tet_region;
    m->tri3 = d->tri3;
    m->tri_region = d->tri_region;
    m->tri_dMs = d->tri_dMs;
    return FG_OK;
}

}  // extern "C"
