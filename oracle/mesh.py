"""Mesh reading and set-up, restated in numpy. TEST INFRASTRUCTURE ONLY.

This module is part of the oracle (the CPU restatement). Only tests, the smoke check and
bench.py's CPU-baseline leg may import it; the product never does.

It restates what FeeLLGood does between opening a gmsh file and the first time step
(paths relative to the FeeLLGood source tree):

* ``read_msh``      gmsh 2.2 / 4.1 ASCII reading as the gmsh API exposes it to
                    ``mesh::readNodes/readTetraedrons/readTriangles`` (src/read.cpp:73-197)
* ``orient_tets``   ``Tet::orientate`` (src/tetra.cpp:410-424)
* ``control_triangles``  ``mesh::controlTriangles`` / ``diffTriHandler`` /
                    ``assertNoErrInTriangle`` (src/mesh.cpp:121-332): missing surface and
                    interface triangles are created, and the signed ``dMs`` is computed
* ``sort_nodes``    ``mesh::sortNodes`` along the longest axis (src/mesh.cpp:334-367).
                    The reference uses ``std::sort``, whose order among equal coordinates
                    is unspecified; this restatement uses a stable sort. Ties only change
                    the order of floating-point summations.
"""
from __future__ import annotations

import numpy as np


class MeshError(RuntimeError):
    """A mesh the reference rejects; the message is the reference's stderr line."""


def read_msh(path):
    """Parse a gmsh ASCII file (format 2.2 or 4.1).

    Returns dict with ``nodes`` (N x 3, row = tag-1), ``names`` {(dim, phys_tag): name},
    and ``blocks``: list of (dim, entity_tag, phys_tags tuple, elem_type, node_tags (m x k)).
    """
    with open(path) as f:
        lines = f.read().split("\n")
    pos = 0

    def section(name):
        nonlocal pos
        for k in range(len(lines)):
            if lines[k].strip() == "$" + name:
                return k + 1
        return None

    k = section("MeshFormat")
    version = lines[k].split()[0]
    names = {}
    k = section("PhysicalNames")
    if k is not None:
        n = int(lines[k])
        for l in lines[k + 1 : k + 1 + n]:
            parts = l.split(None, 2)
            names[(int(parts[0]), int(parts[1]))] = parts[2].strip().strip('"')
    blocks = []
    if version.startswith("2"):
        k = section("Nodes")
        n = int(lines[k])
        arr = np.array([l.split() for l in lines[k + 1 : k + 1 + n]], dtype=float)
        tags = arr[:, 0].astype(np.int64)
        nodes = np.zeros((int(tags.max()), 3))
        nodes[tags - 1] = arr[:, 1:4]
        k = section("Elements")
        n = int(lines[k])
        groups = {}
        order = []
        for l in lines[k + 1 : k + 1 + n]:
            p = [int(x) for x in l.split()]
            etype, ntags = p[1], p[2]
            tg = p[3 : 3 + ntags]
            phys, elem = tg[0], (tg[1] if ntags > 1 else 0)
            dim = {2: 2, 4: 3, 1: 1, 15: 0}.get(etype, -1)
            key = (dim, elem, etype)
            if key not in groups:
                groups[key] = {"phys": [], "nodes": []}
                order.append(key)
            groups[key]["phys"].append(phys)
            groups[key]["nodes"].append(p[3 + ntags :])
        # gmsh builds one discrete entity per elementary tag, carrying the physical tags
        # of its elements; entities are visited in increasing tag order.
        for key in sorted(order, key=lambda t: (t[0], t[1], t[2])):
            dim, elem, etype = key
            g = groups[key]
            phys = tuple(sorted(set(g["phys"])))
            blocks.append((dim, elem, phys, etype, np.array(g["nodes"], dtype=np.int64)))
    else:
        ent_phys = {}
        k = section("Entities")
        if k is not None:
            counts = [int(x) for x in lines[k].split()[:4]]
            r = k + 1
            for dim in range(4):
                for _ in range(counts[dim]):
                    p = lines[r].split()
                    r += 1
                    tag = int(p[0])
                    if dim == 0:
                        nph = int(p[4])
                        ph = [int(x) for x in p[5 : 5 + nph]]
                    else:
                        nph = int(p[7])
                        ph = [int(x) for x in p[8 : 8 + nph]]
                    ent_phys[(dim, tag)] = tuple(ph)
        k = section("Nodes")
        nb, nnodes, mintag, maxtag = (int(x) for x in lines[k].split()[:4])
        nodes = np.zeros((maxtag, 3))
        r = k + 1
        for _ in range(nb):
            ed, et, par, m = (int(x) for x in lines[r].split()[:4])
            r += 1
            tags = np.array([int(lines[r + i]) for i in range(m)], dtype=np.int64)
            r += m
            xyz = np.array([lines[r + i].split()[:3] for i in range(m)], dtype=float).reshape(m, 3)
            r += m
            if m:
                nodes[tags - 1] = xyz
        k = section("Elements")
        nb = int(lines[k].split()[0])
        r = k + 1
        for _ in range(nb):
            ed, et, etype, m = (int(x) for x in lines[r].split()[:4])
            r += 1
            rows = np.array([lines[r + i].split() for i in range(m)], dtype=np.int64)
            r += m
            blocks.append((ed, et, ent_phys.get((ed, et), ()), etype, rows[:, 1:]))
        blocks.sort(key=lambda b: (b[0], b[1]))
    return {"nodes": nodes, "names": names, "blocks": blocks}


def orient_tets(xyz, tets):
    """Tet::orientate (src/tetra.cpp:410-424): swap ind[2], ind[3] when the mixed product < 0."""
    p0 = xyz[tets[:, 0]]
    a, b, c = xyz[tets[:, 1]] - p0, xyz[tets[:, 2]] - p0, xyz[tets[:, 3]] - p0
    mixed = np.einsum("ij,ij->i", a, np.cross(b, c))
    if np.any(np.abs(mixed) < 1e-40):
        raise MeshError("Singular tetrahedron")
    tets = tets.copy()
    neg = mixed < 0
    tets[neg, 2], tets[neg, 3] = tets[neg, 3].copy(), tets[neg, 2].copy()
    return tets


def _basic(inds):
    """BasicTri (src/mesh.cpp:13-50): sorted node triple and the parity of the sort."""
    inds = np.asarray(inds)
    inv = (inds[:, 0] > inds[:, 1]).astype(int) + (inds[:, 1] > inds[:, 2]) + (inds[:, 0] > inds[:, 2])
    return np.sort(inds, axis=1), (inv % 2).astype(bool)


def control_triangles(tets, tet_reg, tris, tri_reg, vol_names, surf_names, Ms):
    """mesh::controlTriangles (src/mesh.cpp:121-245). Returns (tris, tri_reg, dMs, surf_names).

    vol_names/surf_names are the settings' region lists (index 0 = ``__default__``); Ms is
    indexed like vol_names. Raises MeshError with the reference's message on a bad mesh.
    """
    if len(tets) == 0:
        raise MeshError("Error: not a single tetrahedron is present in the mesh")
    t = np.asarray(tets)
    faces = np.concatenate(
        [t[:, [0, 2, 1]], t[:, [1, 2, 3]], t[:, [2, 0, 3]], t[:, [3, 0, 1]]], axis=0
    ).reshape(4, -1, 3).transpose(1, 0, 2).reshape(-1, 3)
    freg = np.repeat(np.asarray(tet_reg), 4)
    fs, fflip = _basic(faces)
    tris = np.asarray(tris, dtype=np.int64).reshape(-1, 3)
    ss, sflip = _basic(tris) if len(tris) else (np.zeros((0, 3), np.int64), np.zeros(0, bool))
    all_nodes = np.concatenate([fs, ss])
    all_reg = np.concatenate([freg, np.asarray(tri_reg, dtype=np.int64)])
    all_surf = np.concatenate([np.zeros(len(fs), bool), np.ones(len(ss), bool)])
    all_flip = np.concatenate([fflip, sflip])
    order = np.lexsort((all_nodes[:, 2], all_nodes[:, 1], all_nodes[:, 0]))
    all_nodes, all_reg, all_surf, all_flip = all_nodes[order], all_reg[order], all_surf[order], all_flip[order]
    change = np.any(all_nodes[1:] != all_nodes[:-1], axis=1)
    starts = np.concatenate([[0], np.nonzero(change)[0] + 1])
    gid = np.cumsum(np.concatenate([[0], change.astype(np.int64)]))
    ng = len(starts)
    n_surf = np.bincount(gid, weights=all_surf, minlength=ng).astype(np.int64)
    n_faces = np.bincount(gid, weights=~all_surf, minlength=ng).astype(np.int64)
    # region pair of the (at most two) tetrahedron faces: (max, min), -1 when absent
    face_reg = np.where(all_surf, -1, all_reg)
    rmax = np.full(ng, -1, np.int64)
    np.maximum.at(rmax, gid, face_reg)
    big = np.iinfo(np.int64).max
    rmin = np.full(ng, big, np.int64)
    np.minimum.at(rmin, gid, np.where(all_surf, big, all_reg))
    rmin = np.where(n_faces >= 2, rmin, -1)
    surf_reg = np.full(ng, -1, np.int64)
    np.maximum.at(surf_reg, gid, np.where(all_surf, all_reg, -1))
    # assertNoErrInTriangle, in the reference's order of tests, first failing group wins
    bad = (n_surf > 1) | (n_faces == 0) | (n_faces > 2) | ((n_faces == 2) & (n_surf == 1) & (rmax == rmin))
    if np.any(bad):
        g = int(np.nonzero(bad)[0][0])
        ns_, nf_, sid = int(n_surf[g]), int(n_faces[g]), int(surf_reg[g])
        if ns_ > 1:
            raise MeshError(f"Error: bad mesh. {ns_} instances of the same surface triangle have been found")
        if nf_ == 0:
            raise MeshError(
                "Error: bad mesh. A triangle which belongs to 1 surface region and no tetrahedron has been found")
        if nf_ > 2:
            if ns_ == 1:
                raise MeshError(f"Error: bad mesh. A triangular face shared by {nf_} tetrahedrons has been found "
                                f"in the surface region {sid}")
            raise MeshError(f"Error: bad mesh. A triangular face shared by {nf_} tetrahedrons has been found")
        raise MeshError(f"Error: bad mesh. An internal triangle has been found in the surface region {sid}")
    add = (n_surf == 0) & ((n_faces == 1) | ((n_faces == 2) & (rmax != rmin)))
    to_add_nodes = all_nodes[starts[add]]
    to_add_pairs = [(int(a), int(b)) for a, b in zip(rmax[add], rmin[add])]
    # create the missing surface regions and triangles (src/mesh.cpp:155-203)
    surf_names = list(surf_names)
    pair_to_reg = {}
    for pair in to_add_pairs:
        if pair in pair_to_reg:
            continue
        if pair[1] == -1:
            base = f"surface({vol_names[pair[0]]})"
        else:
            base = f"interface({vol_names[pair[0]]}, {vol_names[pair[1]]})"
        i = 0
        while True:
            name = base if i == 0 else f"{base}.{i}"
            if name not in surf_names:
                break
            i += 1
        surf_names.append(name)
        pair_to_reg[pair] = len(surf_names) - 1
    new_tris = np.asarray(to_add_nodes, dtype=np.int64).reshape(-1, 3)
    new_reg = np.array([pair_to_reg[p] for p in to_add_pairs], dtype=np.int64)
    tris = np.concatenate([tris, new_tris]) if len(new_tris) else tris
    tri_reg = np.concatenate([np.asarray(tri_reg, dtype=np.int64), new_reg])
    # dMs (src/mesh.cpp:218-232): sum of +-Ms over the tetrahedron faces matching each triangle
    ts, tflip = _basic(tris) if len(tris) else (np.zeros((0, 3), np.int64), np.zeros(0, bool))
    face = ~all_surf
    fkeys = all_nodes[face]
    n = int(max(all_nodes.max(), ts.max() if len(ts) else 0)) + 1

    def key(a):
        return (a[:, 0].astype(np.int64) * n + a[:, 1]) * n + a[:, 2]
    fk = key(fkeys)  # already sorted (lexicographic order of the triples)
    fms = np.asarray(Ms)[all_reg[face]]
    fflp = all_flip[face]
    dMs = np.zeros(len(tris))
    if len(tris):
        tk = key(ts)
        lo = np.searchsorted(fk, tk, side="left")
        hi = np.searchsorted(fk, tk, side="right")
        for off in range(int((hi - lo).max()) if len(hi) else 0):
            sel = lo + off < hi
            j = lo[sel] + off
            sgn = np.where(tflip[sel] ^ fflp[j], -1.0, 1.0)
            dMs[sel] += sgn * fms[j]
    return tris, tri_reg, dMs, surf_names


def sort_nodes(xyz, tets, tris):
    """mesh::sortNodes (src/mesh.cpp:334-367) plus the longest-axis choice (src/mesh.h:51-79).

    Returns (xyz_sorted, tets, tris, node_index) with node_index[file_idx] = sorted index.
    """
    lo, hi = xyz.min(axis=0), xyz.max(axis=0)
    l = hi - lo
    if l[0] > l[1]:
        axis = 0 if l[0] > l[2] else 2
    else:
        axis = 1 if l[1] > l[2] else 2
    perm = np.argsort(xyz[:, axis], kind="stable")
    node_index = np.empty(len(perm), dtype=np.int64)
    node_index[perm] = np.arange(len(perm))
    return xyz[perm], node_index[tets], node_index[tris] if len(tris) else tris, node_index


def setup(msh, vol_regions, surf_regions=(), scale=1e-9, Ms=None):
    """The reference's mesh construction for a parsed file.

    vol_regions: names of the settings' volume regions (``__default__`` is prepended
    as index 0, like the reference's Settings). Ms: list of Ms per vol_regions entry.
    """
    vol_names = ["__default__"] + list(vol_regions)
    surf_names = ["__default__"] + list(surf_regions)
    nodes = msh["nodes"] * scale
    tets, treg, tris, freg = [], [], [], []
    for dim, ent, phys, etype, conn in msh["blocks"]:
        for ph in phys:
            name = msh["names"].get((dim, ph))
            if dim == 3 and name in vol_names:
                if etype != 4:
                    raise MeshError("Fatal error: a volume mesh entity contains other elements than tetraedrons.")
                tets.append(conn - 1)
                treg += [vol_names.index(name)] * len(conn)
            if dim == 2 and name in surf_names:
                if etype != 2:
                    raise MeshError("Fatal error: a surface mesh entity contains other elements than triangles.")
                tris.append(conn - 1)
                freg += [surf_names.index(name)] * len(conn)
    tets = np.concatenate(tets) if tets else np.zeros((0, 4), np.int64)
    tris = np.concatenate(tris) if tris else np.zeros((0, 3), np.int64)
    tets = orient_tets(nodes, tets)
    ms = np.array([0.0] + list(Ms if Ms is not None else [1.0] * len(vol_regions)))
    tris, freg, dMs, surf_names = control_triangles(tets, treg, tris, freg, vol_names, surf_names, ms)
    xyz, tets, tris, node_index = sort_nodes(nodes, tets, tris)
    return {
        "xyz": xyz,
        "tets": tets.astype(np.int32),
        "tet_reg": np.asarray(treg, dtype=np.int32),
        "tris": tris.astype(np.int32),
        "tri_reg": np.asarray(freg, dtype=np.int32),
        "dMs": dMs,
        "node_index": node_index,
        "vol_names": vol_names,
        "surf_names": surf_names,
    }
