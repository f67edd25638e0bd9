"""Shared test inputs: structured cuboid meshes set up by the oracle, seeded states."""
import numpy as np

from oracle import fgo
from oracle import mesh as om

MS = 8.0e5
AE = 1.3e-11


def cuboid_msh(nx, ny, nz, lx, ly, lz):
    """gmsh-like dict of a cuboid split into 6 tets per cell (python-modules/meshMaker.py:470-483)."""
    xs, ys, zs = np.linspace(0, lx, nx + 1), np.linspace(0, ly, ny + 1), np.linspace(0, lz, nz + 1)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    nodes = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)

    def idx(i, j, k):
        return (nz + 1) * (ny + 1) * i + (nz + 1) * j + k
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    A, B, Cc, D = idx(i, j, k), idx(i + 1, j, k), idx(i + 1, j + 1, k), idx(i, j + 1, k)
    E, F, G, H = idx(i, j, k + 1), idx(i + 1, j, k + 1), idx(i + 1, j + 1, k + 1), idx(i, j + 1, k + 1)
    tets = np.stack([np.stack(t, 1) for t in ([A, B, D, H], [A, B, E, H], [E, F, H, B], [B, Cc, D, H],
                                               [B, Cc, G, H], [F, B, G, H])], axis=1).reshape(-1, 4)
    return {"nodes": nodes, "names": {(3, 300): "volume"},
            "blocks": [(3, 1, (300,), 4, tets + 1)]}


def cuboid(nx, ny, nz, h=2.5):
    """Set-up mesh (oriented tets, boundary triangles with dMs, sorted nodes), lengths in nm * 1e-9."""
    msh = cuboid_msh(nx, ny, nz, nx * h, ny * h, nz * h)
    return om.setup(msh, ["volume"], [], 1e-9, Ms=[MS])


def regions(alpha=0.5, K=0.0, uk=(0, 0, 1), K3=0.0):
    return [dict(Ae=1e-11, Ms=795774.7, alpha=0.5),
            dict(Ae=AE, Ms=MS, alpha=alpha, K=K, uk=uk, K3=K3)]


def oracle_regions(alpha=0.5, K=0.0, uk=(0, 0, 1), K3=0.0):
    return [fgo.make_region(), fgo.make_region(A=AE, Ms=MS, alpha=alpha, K=K, uk=uk, K3=K3)]


def perturbed_state(xyz, seed=1, sigma=0.05, base=(1, 1, 0)):
    rng = np.random.default_rng(seed)
    u = np.asarray(base, float) / np.linalg.norm(base) + rng.normal(0, sigma, (len(xyz), 3))
    return u / np.linalg.norm(u, axis=1, keepdims=True)


def tangent_field(u, seed=2, scale=1e9):
    rng = np.random.default_rng(seed)
    v = rng.normal(0, 1, u.shape)
    v -= np.sum(v * u, axis=1, keepdims=True) * u
    return scale * v
