"""The small cube configuration stepped on the GPU (plain FP64) and by the FP64 oracle side
by side: cube 50 x 50 x 50 nm on a 2.5 nm grid (20^3 cells x 6 = 48,000 tets, 9,261
nodes), permalloy (Ms 8e5 A/m, A 1.3e-11 J/m, alpha 0.5), m = (1,1,0)/sqrt(2) plus a
seeded Gaussian perturbation (sigma 0.05), zero field, dt 1e-14 s, BiCG tolerance 1e-6,
the same basis angle on both sides every step. Both sides use the exact FP64 direct sum
for the demag potential (the GPU FMM is checked against that sum in test_gpu_fmm.py), so
every difference is rounding: per step, v within rel-L2 1e-9, u within 1e-12, phi within
1e-11, along the whole trajectory.
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import fgo
from tests import cases

pytestmark = pytest.mark.gpu

NSTEPS = 25
DT = 1e-14


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_cube_trajectory_parity():
    m = cases.cuboid(20, 20, 20)
    assert len(m["tets"]) == 48000 and len(m["xyz"]) == 9261
    u0 = cases.perturbed_state(m["xyz"], seed=21, sigma=0.05)
    H = np.zeros(3)
    o = fgo.Oracle(m, cases.oracle_regions(alpha=0.5))
    o.set_solver(1e-6, 700)
    o.set_state(u0)
    o.compute_all(H)
    c = fg.Context(m, cases.regions(alpha=0.5), tol=1e-6, max_iter=700, precision=fg.FG_PREC_FP64,
                   demag=fg.FG_DEMAG_DIRECT)
    c.set_state(u0)
    c.compute_all(H)
    pref = 1.0
    rng = np.random.default_rng(5)
    worst = {"v": 0.0, "u": 0.0, "phi": 0.0}
    for k in range(NSTEPS):
        angle = float(rng.uniform(0, 2 * np.pi))
        o.base_projection(angle)
        ro = o.step(DT, pref, H)
        rg = c.step(DT, pref, H, angle)
        assert not ro["fail"] and rg["status"] == fg.FG_OK
        assert rg["iters"] == ro["iters"]
        so, sg = o.get_state(1), c.get_state(1)
        worst["v"] = max(worst["v"], _rel(sg["v"], so["v"]))
        worst["u"] = max(worst["u"], np.abs(sg["u"] - so["u"]).max())
        o.compute_all(H)
        c.compute_all(H)
        so, sg = o.get_state(0), c.get_state(0)
        worst["phi"] = max(worst["phi"], _rel(sg["phi"], so["phi"]))
    print("cube trajectory, worst over %d steps:" % NSTEPS, worst)
    assert worst["v"] < 1e-9
    assert worst["u"] < 1e-12
    assert worst["phi"] < 1e-11
