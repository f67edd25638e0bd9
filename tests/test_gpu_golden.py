"""The reference's functional test (ci-tests/full_test.py) run through the GPU plain path.

The time loop here is the test harness (restating Fem::time_integration and TimeStepper,
src/time_integration.cpp:11-38, 136-250); every step and compute_all runs on the GPU.
The basis angles come from the same glibc rand() -> mt19937 stream as the reference
(seed 2). Pass criterion: the test's own 1e-5 on final <m> and E_tot.
"""
import json
import math
import os

import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import fgo
from oracle import mesh as om

pytestmark = pytest.mark.gpu


def run_time_integration(ctx, g, Hext):
    fgo.srand(g["seed"])
    tf, dtmin, dtmax, evol, dumax = g["final_time"], g["min_dt"], g["max_dt"], g["evol_time_step"], g["max_du"]
    taur = 100 * dtmax

    def prefactor(dt):
        tt = dt / taur
        return 1 + tt * abs(math.log(tt))
    fgo.draw_angle()  # the LinAlgebra constructor's base_projection
    ctx.compute_all(Hext)
    t, dt = 0.0, math.sqrt(dtmin * dtmax)
    hard_max = dtmax * (1 + 1.1920928955078125e-07)
    soft_max = dt
    rows = []
    step_count = round((tf - t) / evol)
    E = None
    for step_nb in range(step_count + 1):
        target = step_nb * evol
        while t < target:
            stride = target - t
            step = min(stride, soft_max)
            if stride - 2 * dtmin < step < stride:
                step = stride - 2 * dtmin
            soft_max = max(soft_max, min(step * 1.1, hard_max))
            dt = step
            last = dt == target - t
            assert dt >= dtmin
            angle = fgo.draw_angle()
            rep = ctx.step(dt, prefactor(dt), Hext, angle)
            if rep["status"] != fg.FG_OK:
                soft_max = min(soft_max, dt / 2)
                continue
            soft_max = min(soft_max, (dumax / rep["vmax"]) * 0.95)
            if dt * rep["vmax"] > dumax:
                continue
            E = ctx.compute_all(Hext)
            t = target if last else t + dt
        avg = ctx.average(0)
        Ev = E if E is not None else ctx.energy(Hext)
        rows.append([t, *avg, Ev.sum()])
    return np.array(rows)


@pytest.mark.parametrize("one_point", [False, True])
def test_full_test_golden_gpu(golden_dir, one_point):
    g = json.load(open(os.path.join(golden_dir, "golden.json")))["full_test"]
    msh = om.read_msh(os.path.join(golden_dir, g["mesh"]))
    m = om.setup(msh, [g["volume_region"]], [], g["length_unit"], Ms=[795774.7])
    regs = [dict(), dict(K=g["K"], uk=g["uk"])]
    ctx = fg.Context(m, regs, one_gauss_point=int(one_point))
    ctx.set_state(np.tile(g["initial_magnetization"], (len(m["xyz"]), 1)))
    rows = run_time_integration(ctx, g, np.array(g["Bext"]) / fg.MU0)
    exp = g["expected_1pt" if one_point else "expected_5pt"]
    last = rows[-1]
    assert np.linalg.norm(np.array(exp["m"]) - last[1:4]) < g["threshold"]
    assert abs((last[4] - exp["E_tot"]) / exp["E_tot"]) < g["threshold"]
