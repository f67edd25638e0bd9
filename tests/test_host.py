"""Host-side parts of the product (no GPU needed): C-ABI exports, mesh ingest and set-up.

The mesh set-up of libfggpu (C++) is compared array for array with the oracle's
restatement, and against the reference's own known answers (ellipsoid counts, the
controlTriangles error messages of unit-tests/ut_readMesh.cpp, meshMaker.Cuboid output).
"""
import json
import os
import re

import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import mesh as om
from tests import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "fggpu.h")).read()
    names = sorted(set(re.findall(r"\b(fg_[a-z_0-9]+)\s*\(", hdr)))
    lib = fg.fg_lib()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert len(names) >= 20


def test_opts_mirror_matches_the_c_layout():
    """The ctypes mirror of fg_opts has the C struct's size and field offsets: fg_opts_default
    (host code) writes every field of a buffer larger than the mirror, leaves the bytes after
    it alone, and the mirror reads the documented defaults at its field offsets, the last
    field included."""
    import ctypes as C
    n = C.sizeof(fg.api.fg_opts)
    raw = (C.c_ubyte * (n + 64))(*([0xA5] * (n + 64)))
    fg.fg_lib().fg_opts_default(C.cast(raw, C.POINTER(fg.api.fg_opts)))
    assert all(b == 0xA5 for b in raw[n:]), "fg_opts is larger in C than its mirror"
    o = fg.api.fg_opts.from_buffer(raw)
    assert (o.tol, o.max_iter, o.precision, o.refine_max, o.inner_tol) == (1e-6, 700, fg.FG_PREC_FP64, 20, 1e-5)
    assert (o.mlp_train_steps, o.mlp_batch, o.mlp_lr, o.fmm_tensor, o.mlp_train_every) == (20, 16384, 1e-3, 1, 1)
    assert (o.spin_tol, o.spin_max_iter, o.demag_increment) == (1e-8, 1000, 1)
    assert (o.fmm_overlap, o.fmm_tree_host, o.solver_threads) == (0, 0, 0)


def _same(a, b, keys=("xyz", "tets", "tet_reg", "tris", "tri_reg", "dMs")):
    for k in keys:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


@pytest.mark.parametrize("shape", [(3, 2, 2), (6, 5, 4), (4, 4, 1)])
def test_cuboid_setup_matches_oracle(shape):
    nx, ny, nz = shape
    a = fg.cuboid(nx, ny, nz, 2.5 * nx, 2.5 * ny, 2.5 * nz, 1e-9, cases.MS)
    b = cases.cuboid(nx, ny, nz)
    _same(a, b)
    assert a["surf_names"] == ["__default__", "surface(volume)"]


def test_cuboid_matches_meshmaker_fixture(golden_dir):
    """meshMaker.Cuboid((0,0,0),(7.5,5,5),3,2,2) written by the reference's generator."""
    path = os.path.join(golden_dir, "cuboid_3x2x2.msh")
    a = fg.load_msh(path, ["volume"], [cases.MS])       # boundary recreated by controlTriangles
    b = fg.cuboid(3, 2, 2, 7.5, 5, 5, 1e-9, cases.MS)
    _same(a, b)
    c = fg.load_msh(path, ["volume"], [cases.MS], ["surface"])  # the file's own triangles
    d = om.setup(om.read_msh(path), ["volume"], ["surface"], 1e-9, Ms=[cases.MS])
    _same(c, d)
    assert np.all(np.abs(c["dMs"]) == cases.MS)
    info = json.load(open(os.path.join(golden_dir, "cuboid_20.json")))
    e = fg.cuboid(20, 20, 20, 50, 50, 50, 1e-9, cases.MS)
    assert (len(e["xyz"]), len(e["tets"]), len(e["tris"])) == (info["nodes"], info["tets"], info["tris"])


def test_ellipsoid_setup_matches_oracle(golden_dir):
    path = os.path.join(golden_dir, "ellipsoid.msh")
    g = json.load(open(os.path.join(golden_dir, "golden.json")))["ellipsoid_counts"]
    a = fg.load_msh(path, ["ellipsoid_volume"], [795774.7])
    b = om.setup(om.read_msh(path), ["ellipsoid_volume"], [], 1e-9, Ms=[795774.7])
    _same(a, b, keys=("xyz", "tets", "tet_reg", "tris", "tri_reg", "dMs", "node_index"))
    assert (len(a["xyz"]), len(a["tets"]), len(a["tris"])) == (g["nodes"], g["tets"], g["tris"])


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_bad_meshes_rejected_with_reference_message(golden_dir, k):
    msg = json.load(open(os.path.join(golden_dir, "golden.json")))["bad_cuboid_errors"][k - 1]
    with pytest.raises(fg.FgError) as e:
        fg.load_msh(os.path.join(golden_dir, f"bad_cuboid_{k}.msh"), ["whole_volume"], [8e5], ["whole_surface"], 1.0)
    assert e.value.status == fg.api.FG_EMESH
    assert str(e.value).endswith(msg)


def test_missing_mesh_file():
    with pytest.raises(fg.FgError) as e:
        fg.load_msh("/nonexistent/file.msh", ["v"], [1.0])
    assert e.value.status == fg.api.FG_EIO


def _checkpoint_bytes(n=4, nmt=2, meta=None, version=1):
    """A checkpoint in the documented layout (fg_checkpoint.cu): header, meta, state, FNV-1a.
    Version 2 adds the solver's threads per block after the FMM depth."""
    import struct
    m = dict(t0=0.0, t=1.5e-12, dt=2e-14, dt_soft_max=3e-14, steps=75, output_index=4, rng_seed=9, rng_draws=80,
             E=[1.0, 2.0, -3.0, 4.0])
    m.update(meta or {})
    b = b"FGGPUCK1" + struct.pack("<I6i", version, n, nmt, 1, 4, 304, 6)
    if version >= 2:
        b += struct.pack("<i", 512)
    b += struct.pack("<4d", m["t0"], m["t"], m["dt"], m["dt_soft_max"])
    b += struct.pack("<qqIq", m["steps"], m["output_index"], m["rng_seed"], m["rng_draws"])
    b += struct.pack("<4d", *m["E"])
    b += np.arange(8 * n, dtype="<f8").tobytes()
    h = 1469598103934665603
    for x in b:
        h = ((h ^ x) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return b + struct.pack("<Q", h), m


def test_checkpoint_header_and_checksum(tmp_path):
    """fg_checkpoint_peek reads the documented layout and rejects a corrupted file."""
    raw, m = _checkpoint_bytes()
    p = tmp_path / "a.ckpt"
    p.write_bytes(raw)
    h = fg.checkpoint_peek(p)
    assert (h["n_nodes"], h["n_mag_tets"], h["precision"], h["solver_lpr"], h["solver_blocks"], h["fmm_depth"]) == \
        (4, 2, 1, 4, 304, 6)
    assert h["solver_threads"] == 0  # a version-1 file has no block size (256 threads)
    for k in ("t0", "t", "dt", "dt_soft_max", "steps", "output_index", "rng_seed", "rng_draws", "E"):
        assert h[k] == m[k], k
    bad = bytearray(raw)
    bad[100] ^= 1
    p.write_bytes(bytes(bad))
    with pytest.raises(fg.FgError):
        fg.checkpoint_peek(p)
    p.write_bytes(raw[:-9])
    with pytest.raises(fg.FgError):
        fg.checkpoint_peek(p)


def test_checkpoint_version2_header(tmp_path):
    """Version 2 of the layout carries the solver's threads per block after the FMM depth; a
    version the library does not know is rejected."""
    raw, m = _checkpoint_bytes(version=2)
    p = tmp_path / "b.ckpt"
    p.write_bytes(raw)
    h = fg.checkpoint_peek(p)
    assert (h["solver_lpr"], h["solver_blocks"], h["fmm_depth"], h["solver_threads"]) == (4, 304, 6, 512)
    for k in ("t", "steps", "rng_draws", "E"):
        assert h[k] == m[k], k
    raw3, _ = _checkpoint_bytes(version=3)
    p.write_bytes(raw3)
    with pytest.raises(fg.FgError):
        fg.checkpoint_peek(p)
