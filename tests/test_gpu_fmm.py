"""GPU FMM demag potential against exact direct sums.

The reference evaluates the demag potential with ScalFMM (P=9, uniform octree, one-cell
separation); its error against the exact sum is not recorded anywhere in the reference,
so the bound here is the one measured for this FMM with the same order and separation:
relative L2 error below 1e-5 for the potential of a magnetisation field and below 1e-4
for a random (strongly cancelling) tangent field, in FP64 and in FP32.
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import fgo
from tests import cases

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("shape", [(12, 12, 12), (40, 40, 3)])
@pytest.mark.parametrize("precision", [fg.FG_PREC_FP64, fg.FG_PREC_FP32_REFINE])
@pytest.mark.parametrize("leaf", [40, 200])
def test_fmm_vs_direct(shape, precision, leaf):
    m = cases.cuboid(*shape)
    u = cases.perturbed_state(m["xyz"], seed=4, sigma=0.3)
    v = cases.tangent_field(u, seed=5)
    cd = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_DIRECT)
    cd.set_state(u, v)
    cf = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, precision=precision, fmm_leaf=leaf)
    cf.set_state(u, v)
    assert _rel(cf.demag(0), cd.demag(0)) < 1e-5
    assert _rel(cf.demag(1), cd.demag(1)) < 1e-4


def test_direct_matches_oracle():
    m = cases.cuboid(10, 8, 6)
    u = cases.perturbed_state(m["xyz"], seed=6, sigma=0.3)
    o = fgo.Oracle(m, cases.oracle_regions())
    o.set_state(u)
    cd = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_DIRECT)
    cd.set_state(u)
    assert _rel(cd.demag(0), o.demag(0)) < 1e-12
    cf = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, fmm_leaf=50)
    cf.set_state(u)
    assert _rel(cf.demag(0), o.demag(0)) < 1e-5
