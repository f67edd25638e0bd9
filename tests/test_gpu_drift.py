"""Trajectory accuracy of the FP32 + refinement path against the plain FP64 path.

Cube 30 x 30 x 30 nm on a 2.5 nm grid (12^3 cells x 6 = 10,368 tets, 2,197 nodes), permalloy
with alpha 0.1, a seeded perturbed state, an applied field of 40 kA/m, dt 1e-14 s, the FMM on
both sides at the same depth; 200 steps from the same state with the same basis angles.

Two pairs of runs:
  * control: the plain FP64 path with the learned initial guess against the plain FP64 path
    with the previous-step guess: the same arithmetic, another valid initial guess, so their
    difference is what the solver tolerance alone allows;
  * mixed: the FP32 Krylov body with FP64 refinement, the double-single element integrals and
    the FP32 FMM on the change of the field (fg_opts.demag_increment) against the plain FP64
    path.
At each tolerance the mixed pair's max |dm| must stay within twice the control's (or below
a floor of 1e-9, where both are at rounding level); at 1e-8 it must be below 1e-6.
The reference's loop is src/time_integration.cpp:166-247.
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from tests import cases

pytestmark = pytest.mark.gpu

NSTEPS = 200
DT = 1e-14


def _run(m, u0, H, tol, angles, **opts):
    c = fg.Context(m, cases.regions(alpha=0.1), tol=tol, max_iter=700, demag=fg.FG_DEMAG_FMM, fmm_leaf=-3,
                   mlp_train_steps=20, **opts)
    c.set_state(u0)
    c.compute_all(H)
    iters = []
    for k in range(NSTEPS):
        r = c.step(DT, 1.0, H, angles[k])
        assert r["status"] == fg.FG_OK, r
        iters.append(r["iters"])
        c.compute_all(H)
    st = c.get_state(0)
    c.close()
    return st["u"], float(np.mean(iters))


@pytest.mark.parametrize("tol", [1e-6, 1e-8])
def test_mixed_path_within_the_tolerance_spread(tol):
    m = cases.cuboid(12, 12, 12)
    u0 = cases.perturbed_state(m["xyz"], seed=31, sigma=0.1)
    H = np.array([0.0, 0.0, 4e4])
    rng = np.random.default_rng(3)
    angles = rng.uniform(0, 2 * np.pi, NSTEPS)
    plain, ip = _run(m, u0, H, tol, angles, precision=fg.FG_PREC_FP64)
    ctrl, ic = _run(m, u0, H, tol, angles, precision=fg.FG_PREC_FP64, learned_guess=1)
    mixed, im = _run(m, u0, H, tol, angles, precision=fg.FG_PREC_FP32_REFINE)
    d_ctrl = float(np.linalg.norm(ctrl - plain, axis=1).max())
    d_mixed = float(np.linalg.norm(mixed - plain, axis=1).max())
    moved = float(np.linalg.norm(plain - u0, axis=1).max())
    print(f"tol {tol:g}, {NSTEPS} steps: max |dm| mixed {d_mixed:.2e}, control {d_ctrl:.2e}; iterations per step "
          f"plain {ip:.2f}, control {ic:.2f}, mixed {im:.2f}; the state moved by {moved:.2e}")
    assert moved > 1e-2
    assert d_mixed <= max(2.0 * d_ctrl, 1e-9)
    if tol <= 1e-8:
        assert d_mixed < 1e-6
