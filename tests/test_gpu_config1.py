"""The parity protocol on the small cube configuration, with the FMM at the reference's
settings: cube 50 x 50 x 50 nm on a 2.5 nm grid (20^3 cells x 6 = 48,000 tets, 9,261 nodes),
permalloy (Ms 8e5 A/m, A 1.3e-11 J/m, alpha 0.5), m = (1,1,0)/sqrt(2) plus a seeded Gaussian
perturbation (sigma 0.05), zero field, dt 1e-14 s, BiCG tolerance 1e-6, 200 steps.

The demag potential is the GPU FMM at the reference's expansion order and tree (P = 9,
NbLevels = 6: 32^3 leaves over the box of width 2.01 in the reference's normalised units,
src/fmm_demag.h:26-28, 52-53, 72), against the oracle's CPU FMM on the same tree (the oracle's
stand-in for ScalFMM, which is absent here), both in FP64, and both against the exact FP64
direct sum (the FMM's own error).

The trajectory runs on the GPU (plain FP64 path); every step the oracle is put in the GPU's
CURRENT state (u, v, phi, phiv), takes the same step (same basis angle) and is compared with
the GPU's NEXT state: v (rel-L2), u (max abs) and the iteration count; after every
fg_compute_all the energies of the new state. The oracle's CPU FMM (a few seconds per
evaluation at this depth) evaluates the potentials of the first and of the last state.
The reference's step is src/time_integration.cpp:193-231, its compute_all src/fem.h:203-224.
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import fgo
from tests import cases

pytestmark = pytest.mark.gpu

NSTEPS = 200
DT = 1e-14
LEVELS = 5  # leaves at depth 5: the reference's 6-level tree


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def cube():
    m = cases.cuboid(20, 20, 20)
    assert len(m["tets"]) == 48000 and len(m["xyz"]) == 9261
    u0 = cases.perturbed_state(m["xyz"], seed=21, sigma=0.05)
    return m, u0


def _fmm_vs_oracle(c, o, st):
    """GPU FMM (FP64) and the oracle's CPU FMM on the same state; both sets."""
    c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    o.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    out = {}
    for which, name in ((0, "phi"), (1, "phiv")):
        out[name] = (c.demag(which), o.demag(which))
    return out


def test_cube_fmm_at_reference_tree_matches_oracle_fmm(cube):
    m, u0 = cube
    H = np.zeros(3)
    v0 = cases.tangent_field(u0, seed=4)
    cf = fg.Context(m, cases.regions(alpha=0.5), precision=fg.FG_PREC_FP64, demag=fg.FG_DEMAG_FMM, fmm_leaf=-LEVELS)
    assert cf.counters()[1] == LEVELS
    cd = fg.Context(m, cases.regions(alpha=0.5), precision=fg.FG_PREC_FP64, demag=fg.FG_DEMAG_DIRECT)
    o = fgo.Oracle(m, cases.oracle_regions(alpha=0.5))
    o.set_demag(LEVELS)
    st = {"u": u0, "v": v0, "phi": None, "phiv": None}
    res = _fmm_vs_oracle(cf, o, st)
    cd.set_state(u0, v0)
    exact = {"phi": cd.demag(0), "phiv": cd.demag(1)}
    report = {}
    for k in ("phi", "phiv"):
        g, r = res[k]
        report[k] = {"gpu_vs_oracle_fmm": _rel(g, r), "gpu_fmm_vs_exact": _rel(g, exact[k]),
                     "oracle_fmm_vs_exact": _rel(r, exact[k])}
    print("cube FMM at the reference's tree (P=9, 32^3 leaves):", report)
    for k in report:
        # same tree, order and interaction lists: the two FMMs agree to FP64 rounding
        assert report[k]["gpu_vs_oracle_fmm"] < 1e-10, report
        # the FMM's own error against the exact sum, identical for both
        assert report[k]["gpu_fmm_vs_exact"] < 1e-4, report
    cf.close()
    cd.close()


def test_cube_200_steps_fmm_lockstep_with_oracle(cube):
    m, u0 = cube
    H = np.zeros(3)
    c = fg.Context(m, cases.regions(alpha=0.5), tol=1e-6, max_iter=700, precision=fg.FG_PREC_FP64,
                   demag=fg.FG_DEMAG_FMM, fmm_leaf=-LEVELS)
    o = fgo.Oracle(m, cases.oracle_regions(alpha=0.5))
    o.set_solver(1e-6, 700)
    c.set_state(u0)
    c.compute_all(H)
    first = c.get_state(0)
    rng = np.random.default_rng(5)
    worst = {"v": 0.0, "u": 0.0, "E": 0.0}
    iters_equal = 0
    for k in range(NSTEPS):
        cur = c.get_state(0)
        o.set_state(cur["u"], cur["v"], cur["phi"], cur["phiv"])
        angle = float(rng.uniform(0, 2 * np.pi))
        o.base_projection(angle)
        ro = o.step(DT, 1.0, H)
        rg = c.step(DT, 1.0, H, angle)
        assert not ro["fail"] and rg["status"] == fg.FG_OK
        iters_equal += int(rg["iters"] == ro["iters"])
        so, sg = o.get_state(1), c.get_state(1)
        worst["v"] = max(worst["v"], _rel(sg["v"], so["v"]))
        worst["u"] = max(worst["u"], float(np.abs(sg["u"] - so["u"]).max()))
        Eg = c.compute_all(H)
        new = c.get_state(0)
        o.set_state(new["u"], new["v"], new["phi"], new["phiv"])
        Eo = o.energy(H)
        worst["E"] = max(worst["E"], float(np.max(np.abs(Eg - Eo)) / np.max(np.abs(Eo))))
    last = c.get_state(0)
    # the potentials along the trajectory: GPU FMM against the oracle's CPU FMM (same tree)
    o.set_demag(LEVELS)
    phi_dev = {}
    for name, st in (("first", first), ("last", last)):
        o.set_state(st["u"], st["v"], st["phi"], st["phiv"])
        # the first state has v = 0 (set_state without v), so its phiv is 0 on both sides
        dv = _rel(st["phiv"], o.demag(1)) if np.any(st["v"]) else float(np.abs(st["phiv"]).max())
        phi_dev[name] = (_rel(st["phi"], o.demag(0)), dv)
    dm = float(np.linalg.norm(last["u"] - first["u"], axis=1).max())
    print(f"cube, {NSTEPS} steps with the FMM (P=9, 32^3 leaves), worst per-step deviation from the oracle's "
          f"step: {worst}; same iteration count on {iters_equal}/{NSTEPS} steps; phi/phiv vs the oracle's FMM: "
          f"{phi_dev}; max |m(200) - m(0)| = {dm:.3e}")
    assert worst["v"] < 1e-9
    assert worst["u"] < 1e-12
    assert worst["E"] < 1e-10
    assert iters_equal == NSTEPS
    for a, b in phi_dev.values():
        assert a < 1e-10 and b < 1e-10, phi_dev
    assert dm > 1e-3  # the state moved: the comparison is not of a frozen state
    c.close()
