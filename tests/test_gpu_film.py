"""One step of the headline precision path at full size against the oracle's FP64 step.

Film 400 x 400 x 10 nm on a 2 nm grid (200 x 200 x 5 cells x 6 = 1,200,000 tets, 242,406
nodes), permalloy with alpha 0.02, a seeded smooth random state. The GPU context runs the FP32
Krylov body with FP64 refinement, the double-single element integrals and the FMM; its
potentials of the state (full FP64 FMM evaluation, no potentials given) are handed to the
oracle with the state, so that both sides step from the same CURRENT state: basis
(src/linear_algebra.cpp:3-11), element integrals (src/tetra.cpp:210-307), assembly and
bicg_dir (src/solver.cpp:11-88, src/algebra/bicg.h:163-234), node update. At a solver
tolerance of 1e-10 the refined FP32 solve must land on the oracle's FP64 solution: v within
rel-L2 1e-8 (measured on GB300: 1.3e-10), u within 1e-9 (max abs; dt v is up to 7e-2 per
step on this state; measured 8.1e-11).
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import fgo

pytestmark = pytest.mark.gpu

MS, AE = 8.0e5, 1.3e-11


def _smooth_state(mesh, seed=7):
    rng = np.random.default_rng(seed)
    x = mesh["xyz"] / 1e-9
    k = rng.normal(size=(3, 3)) / 60.0
    ph = rng.uniform(0, 2 * np.pi, 3)
    u = np.stack([np.sin(x @ k[i] + ph[i]) for i in range(3)], axis=1) + np.array([0.3, 0.2, 0.1])
    return u / np.linalg.norm(u, axis=1, keepdims=True)


def test_film_fp32_refine_step_matches_oracle_fp64_step():
    mesh = fg.cuboid(200, 200, 5, 400.0, 400.0, 10.0, 1e-9, MS)
    assert len(mesh["tets"]) == 1200000 and len(mesh["xyz"]) == 242406
    u0 = _smooth_state(mesh)
    H = np.array([0.0, 2e4, 0.0])
    regs = [dict(Ae=1e-11, Ms=795774.7, alpha=0.5), dict(Ae=AE, Ms=MS, alpha=0.02)]
    c = fg.Context(mesh, regs, tol=1e-10, max_iter=700, precision=fg.FG_PREC_FP32_REFINE,
                   demag=fg.FG_DEMAG_FMM)
    c.set_state(u0)
    c.compute_all(H)
    st = c.get_state(0)
    o = fgo.Oracle({k: mesh[k] for k in ("xyz", "tets", "tet_reg", "tris", "tri_reg", "dMs")},
                   [fgo.make_region(), fgo.make_region(A=AE, Ms=MS, alpha=0.02)])
    o.set_solver(1e-10, 700)
    o.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    dt, angle = 5e-14, 1.234
    o.base_projection(angle)
    ro = o.step(dt, 1.0, H)
    rg = c.step(dt, 1.0, H, angle)
    assert not ro["fail"] and rg["status"] == fg.FG_OK, (ro, rg)
    so, sg = o.get_state(1), c.get_state(1)
    dv = float(np.linalg.norm(sg["v"] - so["v"]) / np.linalg.norm(so["v"]))
    du = float(np.abs(sg["u"] - so["u"]).max())
    print(f"film FP32 + refinement step vs the oracle's FP64 step: v rel-L2 {dv:.2e}, u max {du:.2e}, "
          f"iterations {rg['iters']} (+{rg['refinements']} refinements) vs {ro['iters']}")
    assert dv < 1e-8
    assert du < 1e-9
    c.close()
