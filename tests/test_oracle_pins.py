"""Pins of the FP64 oracle against the reference's own known answers (no GPU).

* ci-tests/full_test.py: final <m> and E_tot on examples/ellipsoid.msh, seed 2, for the
  5-point and the 1-point Gauss builds, tolerance 1e-5 (the test's own threshold).
* unit-tests/ut_readMesh.cpp: ellipsoid node/tet/triangle counts and the four
  controlTriangles error messages on unit-tests/meshes/bad_cuboid_{1..4}.msh.
"""
import json
import os

import numpy as np
import pytest

from oracle import fgo
from oracle import mesh as om


def _gold(golden_dir):
    return json.load(open(os.path.join(golden_dir, "golden.json")))


@pytest.mark.parametrize("one_point", [False, True])
def test_full_test_golden(golden_dir, one_point):
    g = _gold(golden_dir)["full_test"]
    msh = om.read_msh(os.path.join(golden_dir, g["mesh"]))
    m = om.setup(msh, [g["volume_region"]], [], g["length_unit"], Ms=[795774.7])
    regs = [fgo.make_region(), fgo.make_region(K=g["K"], uk=g["uk"])]
    o = fgo.Oracle(m, regs, one_gauss_point=one_point)
    o.set_state(np.tile(g["initial_magnetization"], (len(m["xyz"]), 1)))
    Hext = np.array(g["Bext"]) / fgo.MU0
    rows, nsteps, _ = o.time_integration(g["seed"], g["final_time"], g["min_dt"], g["max_dt"],
                                         g["evol_time_step"], g["max_du"], Hext)
    exp = g["expected_1pt" if one_point else "expected_5pt"]
    last = rows[-1]
    assert abs(last[0] - g["final_time"]) < 1e-20
    m_err = np.linalg.norm(np.array(exp["m"]) - last[1:4])
    e_err = abs((last[7] - exp["E_tot"]) / exp["E_tot"])
    assert m_err < g["threshold"], (last[1:4], exp["m"])
    assert e_err < g["threshold"], (last[7], exp["E_tot"])
    assert len(rows) == round(g["final_time"] / g["evol_time_step"]) + 1


def test_ellipsoid_counts(golden_dir):
    g = _gold(golden_dir)
    msh = om.read_msh(os.path.join(golden_dir, "ellipsoid.msh"))
    c = g["ellipsoid_counts"]
    assert msh["nodes"].shape[0] == c["nodes"]
    ntet = sum(len(b[4]) for b in msh["blocks"] if b[3] == 4)
    ntri = sum(len(b[4]) for b in msh["blocks"] if b[3] == 2)
    assert (ntet, ntri) == (c["tets"], c["tris"])
    # with the surface declared in the settings, the file's triangles are used as they are
    m = om.setup(msh, ["ellipsoid_volume"], ["ellipsoid_surface"], 1e-9, Ms=[8e5])
    assert len(m["tris"]) == c["tris"] and len(m["surf_names"]) == 2
    # without it, controlTriangles recreates exactly the same boundary
    m2 = om.setup(msh, ["ellipsoid_volume"], [], 1e-9, Ms=[8e5])
    assert len(m2["tris"]) == c["tris"] and m2["surf_names"][1] == "surface(ellipsoid_volume)"
    assert np.all(np.abs(m2["dMs"]) == 8e5)


@pytest.mark.parametrize("k", [1, 2, 3, 4])
def test_bad_cuboid_messages(golden_dir, k):
    g = _gold(golden_dir)
    msh = om.read_msh(os.path.join(golden_dir, f"bad_cuboid_{k}.msh"))
    with pytest.raises(om.MeshError) as e:
        om.setup(msh, ["whole_volume"], ["whole_surface"], 1.0, Ms=[8e5])
    assert str(e.value) == g["bad_cuboid_errors"][k - 1]


def test_oracle_cpu_fmm_matches_direct_sum():
    """The CPU FMM that times the CPU baseline computes the same potential as the exact sum."""
    from tests import cases
    m = cases.cuboid(10, 10, 3)
    u = cases.perturbed_state(m["xyz"], seed=3, sigma=0.3)
    o = fgo.Oracle(m, cases.oracle_regions())
    o.set_state(u)
    d = o.demag(0)
    o.set_demag(3)
    f = o.demag(0)
    assert np.linalg.norm(f - d) / np.linalg.norm(d) < 1e-5


def test_oracle_drift_term_properties():
    """The oracle's recentering drift (Tet::add_drift_BE) is linear in the drift speed and
    vanishes for a uniform state with v = 0 (no derivative along the direction)."""
    from tests import cases
    m = cases.cuboid(5, 4, 3)
    H = np.array([1e4, 0.0, 2e4])

    def rhs(u, v, direction, vdrift):
        o = fgo.Oracle(m, cases.oracle_regions())
        o.set_state(u, v)
        o.set_drift(direction, vdrift)
        o.base_projection(0.3)
        o.step(1e-14, 1.0, H)
        return o.export_system()[3]

    u = cases.perturbed_state(m["xyz"], seed=5)
    v = cases.tangent_field(u, seed=6)
    r0, r1, r2 = (rhs(u, v, 1, s) for s in (0.0, 1e-3, 2e-3))
    assert np.linalg.norm(r1 - r0) > 1e-6 * np.linalg.norm(r0)
    assert np.linalg.norm((r2 - r0) - 2 * (r1 - r0)) <= 1e-9 * np.linalg.norm(r2 - r0)
    uni = np.tile(np.array([0.6, 0.0, 0.8]), (len(m["xyz"]), 1))
    assert np.array_equal(rhs(uni, None, 2, 1e-3), rhs(uni, None, -1, 0.0))
