"""fg_energy_noalloc: the energy reduction for callers that cannot allocate device memory.

Some callers (a host framework that owns all device memory after start-up, or a loop that
must not cause the device synchronisation an allocation can bring) cannot let a library
call cudaMalloc. fg_energy_noalloc computes the same energies as fg_energy with its
scratch in a static device array instead. Checked here through the C ABI against
fg_energy, on two calls in a row (the array keeps the previous call's contents, which
must not leak into the next), within the tests' energy tolerance of 1e-10 relative, for
both branches of the energy kernel: FP64 with anisotropy, and the isotropic FP32 +
refinement context whose energies are summed in double-single arithmetic.
This file is collected last on purpose.
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from tests import cases

pytestmark = pytest.mark.gpu

CASES = {
    "fp64_anisotropic": (dict(K=3e4, uk=(0.3, 0.2, 1.0), K3=1e4), dict(precision=fg.FG_PREC_FP64)),
    "fp32_refine_isotropic": (dict(), dict(precision=fg.FG_PREC_FP32_REFINE)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_energy_noalloc_matches_energy_twice(name):
    reg, opts = CASES[name]
    m = cases.cuboid(8, 6, 5)
    u = cases.perturbed_state(m["xyz"], seed=11, sigma=0.2)
    c = fg.Context(m, cases.regions(**reg), demag=fg.FG_DEMAG_DIRECT, **opts)
    c.set_state(u)
    H1 = np.array([2e4, -1e4, 3e4])
    c.compute_all(H1)  # potentials of the state, so every energy term is non-zero
    for H in (H1, np.array([-5e3, 7e4, 1e3])):
        ref = c.energy(H)
        got = c.energy_noalloc(H)
        scale = np.max(np.abs(ref))
        assert scale > 0
        assert np.all(np.abs(got - ref) <= 1e-10 * scale), (got, ref)
    c.close()
