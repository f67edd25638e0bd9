"""Failure detection without a GPU fault: every device-side wait of the library is bounded.
A probe runs the persistent solvers' grid barrier with a block that never arrives, and an
mbarrier wait of the tensor-core pipeline with no arrival; each wait must expire, report
FG_ETIMEDOUT to the host, and leave the context usable for the next step."""
import numpy as np
import pytest

import feellgood_gb300 as fg
from tests import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_wait_expires_and_context_survives(which):
    m = cases.cuboid(6, 5, 4)
    u = cases.perturbed_state(m["xyz"], seed=3)
    c = fg.Context(m, cases.regions(), precision=fg.FG_PREC_FP32_REFINE, demag=fg.FG_DEMAG_FMM, fmm_leaf=-2)
    c.set_state(u)
    c.compute_all(np.zeros(3))
    assert c.debug_wait_timeout(which) == fg.FG_ETIMEDOUT
    r = c.step(1e-14, 1.0, np.zeros(3), 0.3)
    assert r["status"] == fg.FG_OK
    c.compute_all(np.zeros(3))
    st = c.get_state(0)
    assert np.all(np.isfinite(st["u"])) and np.allclose(np.linalg.norm(st["u"], axis=1), 1.0)
