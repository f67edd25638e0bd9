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


@pytest.mark.parametrize("shape,leaf", [((12, 12, 12), -3), ((40, 40, 3), -4), ((24, 20, 6), 60)])
def test_tensor_core_translations(shape, leaf):
    """FP32 FMM with the tcgen05 translations (3 x TF32) against the CUDA-core FP32
    translations and the exact sum: the same accuracy, agreement to FP32 rounding."""
    m = cases.cuboid(*shape)
    u = cases.perturbed_state(m["xyz"], seed=7, sigma=0.3)
    v = cases.tangent_field(u, seed=8)
    cd = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_DIRECT)
    cd.set_state(u, v)
    ct = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, precision=fg.FG_PREC_FP32_REFINE, fmm_leaf=leaf)
    ct.set_state(u, v)
    cc = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, precision=fg.FG_PREC_FP32_REFINE, fmm_leaf=leaf,
                    fmm_tensor=0)
    cc.set_state(u, v)
    for which, bound in ((0, 1e-5), (1, 1e-4)):
        pd, pt, pc = cd.demag(which), ct.demag(which), cc.demag(which)
        assert _rel(pt, pd) < bound
        assert _rel(pt, pc) < 3e-6


def test_tensor_core_split_precision():
    """The tcgen05 translation on random data against an FP64 product: the three-term TF32
    split (hi*hi + hi*lo + lo*hi) must give FP32-level accuracy, far below one TF32 term."""
    rng = np.random.default_rng(11)
    ncode, n_in, n_out = 7, 300, 200
    ops = rng.normal(size=(ncode, 100, 100)) * np.exp(rng.uniform(-3, 3, size=(ncode, 100, 1)))
    x = rng.normal(size=(n_in, 100))
    tab = rng.integers(-1, n_in, size=(n_out, ncode))
    tab[5] = -1  # a cell with no input
    ref = np.zeros((n_out, 100))
    for c in range(n_out):
        for k in range(ncode):
            if tab[c, k] >= 0:
                ref[c] += ops[k].astype(np.float32).astype(np.float64) @ x[tab[c, k]].astype(np.float32)
    err = {}
    for terms in (1, 7):
        out = fg.api.debug_translate_tc(ops, tab, x, terms)
        err[terms] = np.linalg.norm(out - ref) / np.linalg.norm(ref)
        assert np.all(out[5] == 0)
    print("tensor-core translation rel. error: 1 term %.2e, 3 terms %.2e" % (err[1], err[7]))
    assert err[7] < 1.5e-6
    assert err[7] < err[1] / 30


@pytest.mark.parametrize("shape,leaf", [((12, 12, 12), -3), ((40, 40, 3), -4)])
def test_double_single_near_field(shape, leaf):
    """The FP64 path's P2M, near field and translations in double-single arithmetic on the
    FP32 pipes against the same FMM on the FP64 pipe (same tree): FP64-level agreement."""
    m = cases.cuboid(*shape)
    u = cases.perturbed_state(m["xyz"], seed=9, sigma=0.3)
    v = cases.tangent_field(u, seed=10)
    cs = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, precision=fg.FG_PREC_FP64, fmm_leaf=leaf)
    cs.set_state(u, v)
    cn = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, precision=fg.FG_PREC_FP64, fmm_leaf=leaf,
                    fmm_native_fp64=1)
    cn.set_state(u, v)
    for which in (0, 1):
        ps, pn = cs.demag(which), cn.demag(which)
        print("double-single vs FP64 FMM, rel. difference %.2e" % _rel(ps, pn))
        assert _rel(ps, pn) < 1e-12


@pytest.mark.parametrize("precision,native", [(fg.FG_PREC_FP32_REFINE, 0), (fg.FG_PREC_FP64, 0),
                                              (fg.FG_PREC_FP64, 1)])
@pytest.mark.parametrize("shape,leaf", [((12, 12, 12), -3), ((40, 40, 3), 60)])
def test_pair_evaluation_matches_single(precision, native, shape, leaf):
    """compute_all evaluates the demag of m and of v in one FMM pass (both charge sets
    through the same launches, one near-field pass with shared pair geometry); each set
    follows the arithmetic of its own single evaluation, so the potentials agree with
    fg_demag(0) and fg_demag(1) to the last bits (a full evaluation per compute_all:
    demag_increment 0)."""
    m = cases.cuboid(*shape)
    u = cases.perturbed_state(m["xyz"], seed=11, sigma=0.3)
    v = cases.tangent_field(u, seed=12)
    c = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, precision=precision, fmm_leaf=leaf,
                   fmm_native_fp64=native, demag_increment=0)
    c.set_state(u, v)
    c.compute_all(np.zeros(3))
    st = c.get_state(0)
    for got, which in ((st["phi"], 0), (st["phiv"], 1)):
        single = c.demag(which)
        scale = np.abs(single).max()
        assert np.abs(got - single).max() <= 1e-13 * scale, (which, np.abs(got - single).max() / scale)


@pytest.mark.parametrize("precision", [fg.FG_PREC_FP32_REFINE, fg.FG_PREC_FP64])
def test_overlapped_evaluation_is_bit_identical(precision):
    """The near field on the second stream beside the far field, then L2P as its own launch,
    performs the same operations as the fused single-stream evaluation: the potentials of
    both charge sets agree bit for bit."""
    m = cases.cuboid(24, 20, 6)
    u = cases.perturbed_state(m["xyz"], seed=13, sigma=0.3)
    v = cases.tangent_field(u, seed=14)
    out = []
    for overlap in (0, 1):
        c = fg.Context(m, cases.regions(), demag=fg.FG_DEMAG_FMM, precision=precision, fmm_leaf=-4,
                       fmm_overlap=overlap, demag_increment=0)
        c.set_state(u, v)
        c.compute_all(np.zeros(3))
        st = c.get_state(0)
        out.append((st["phi"], st["phiv"], c.demag(0), c.demag(1)))
        c.close()
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_tc_translation_launch_resources():
    """The tensor-core translation kernel fits its own launch: the runtime's register and
    shared-memory view admits at least one resident block of 288 threads with the dynamic
    shared memory a launch asks for (a launch that does not fit fails with 'too many
    resources requested for launch')."""
    import ctypes as C
    L = fg.fg_lib()
    a = (C.c_int * 8)()
    assert L.fg_debug_tc_resources(a) == fg.FG_OK
    regs, max_threads, static_smem, max_dyn, local, dyn_req, threads, blocks = list(a)
    assert threads <= max_threads
    assert dyn_req <= max_dyn
    assert blocks >= 1, list(a)
