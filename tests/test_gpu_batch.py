"""Batches of independent samples (fg_batch_*): the block-diagonal system, the forest FMM
and the graph-replayed run against the same samples stepped one context at a time.

A batch sample must follow the iteration it would follow alone: its Krylov scalars, its
|b| and its stopping test are its own. What may differ is the order of the per-block
partial sums (a sample gets a different number of solver blocks in a batch), so the
per-sample solutions agree to the solver tolerance, not bit for bit. The demag potential is
a forest of the same octrees, but the tensor-core translations group the interaction codes
of a tile of 64 cells (which may hold cells of several samples) into work units, so sums
are grouped differently: it agrees to FP32 rounding. A graph replay of the stream-ordered
step agrees exactly.
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import fgo
from tests import cases

pytestmark = pytest.mark.gpu

SHAPES = [(4, 4, 4), (7, 5, 4), (5, 6, 8)]
H = np.array([[0.0, 0.0, 3e4], [2e4, 0.0, 0.0], [1e4, -1e4, 5e3]])
# fixed solver variant and tree depth: bitwise comparisons across contexts need the same kernels
OPTS = dict(precision=fg.FG_PREC_FP32_REFINE, demag=fg.FG_DEMAG_FMM, fmm_leaf=-3, tol=1e-9, refine_max=12,
            solver_lpr=1)


def _samples():
    ms = [cases.cuboid(*s) for s in SHAPES]
    us = [cases.perturbed_state(m["xyz"], seed=10 + g, sigma=0.2) for g, m in enumerate(ms)]
    return ms, us


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _singles(ms, us):
    cs = []
    for m, u in zip(ms, us):
        # a batch evaluates the full FP32 FMM every step: the single context does the same
        c = fg.Context(m, cases.regions(alpha=0.1), demag_increment=0, **OPTS)
        c.set_state(u)
        c.compute_all([0, 0, 0])
        cs.append(c)
    return cs


def _batch(ms, us, **over):
    b = fg.Context(ms, cases.regions(alpha=0.1), **dict(OPTS, **over))
    b.set_state(np.concatenate(us))
    b.batch_compute_all(None, energies=False)
    return b


def test_batch_layout_and_forest_demag():
    ms, us = _samples()
    b = _batch(ms, us)
    off = b.node_offsets
    assert list(np.diff(off)) == [len(m["xyz"]) for m in ms]
    singles = _singles(ms, us)
    phi_b = b.get_state(0)["phi"]
    for g, c in enumerate(singles):
        phi = c.get_state(0)["phi"]
        assert _rel(phi_b[off[g]:off[g + 1]], phi) < 1e-6
    # the forest potential is each sample's own: it matches the oracle's exact sum per sample
    for g, m in enumerate(ms):
        o = fgo.Oracle(m, cases.oracle_regions(alpha=0.1))
        o.set_state(us[g])
        assert _rel(phi_b[off[g]:off[g + 1]], o.demag(0)) < 1e-4


def test_batch_step_matches_single_contexts():
    ms, us = _samples()
    b = _batch(ms, us)
    singles = _singles(ms, us)
    off = b.node_offsets
    dt, pref = 1e-14, 1.0
    angles = np.array([0.3, 1.1, 2.0])
    for it in range(3):
        s, reps = b.batch_step(dt, pref, H, angles + it)
        assert s == fg.FG_OK
        vb = b.get_state(1)["v"]
        for g, c in enumerate(singles):
            r = c.step(dt, pref, H[g], angles[g] + it)
            assert r["status"] == fg.FG_OK
            v = c.get_state(1)["v"]
            assert _rel(vb[off[g]:off[g + 1]], v) < 1e-7
            assert abs(reps[g]["vmax"] - r["vmax"]) <= 1e-7 * r["vmax"]
            assert reps[g]["res"] <= 1e-9 * reps[g]["rhsn"]
        E = b.batch_compute_all(H)
        for g, c in enumerate(singles):
            e = c.compute_all(H[g])
            np.testing.assert_allclose(E[g], e, rtol=1e-6, atol=1e-30)


def test_batch_of_one_is_the_single_path():
    ms, us = _samples()
    b = fg.Context([ms[2]], cases.regions(alpha=0.1), **OPTS)
    b.set_state(us[2])
    b.batch_compute_all(None, energies=False)
    c = _singles(ms[2:], us[2:])[0]
    s, reps = b.batch_step(1e-14, 1.0, H[2:], [0.7])
    r = c.step(1e-14, 1.0, H[2], 0.7)
    assert s == fg.FG_OK and r["status"] == fg.FG_OK
    assert reps[0]["iters"] == r["iters"]
    np.testing.assert_array_equal(b.get_state(1)["v"], c.get_state(1)["v"])


@pytest.mark.parametrize("precision", [fg.FG_PREC_FP32_REFINE, fg.FG_PREC_FP64])
def test_batch_run_graph_equals_stepwise(precision):
    ms, us = _samples()
    nsteps = 5
    rng = np.random.default_rng(3)
    angles = rng.uniform(0, 2 * np.pi, (nsteps, len(ms)))
    a = _batch(ms, us, precision=precision)
    s, reps = a.batch_run(1e-14, 1.0, H, angles)
    assert s == fg.FG_OK
    graph, ms_dev = a.batch_run_info()
    print(f"batch run: graph replay {graph}, {ms_dev:.3f} ms for {nsteps} steps")
    assert ms_dev > 0
    b = _batch(ms, us, precision=precision)
    iters = np.zeros(len(ms), dtype=int)
    for k in range(nsteps):
        s, rr = b.batch_step(1e-14, 1.0, H, angles[k])
        assert s == fg.FG_OK
        iters += [r["iters"] for r in rr]
        b.batch_compute_all(None, energies=False)
    sa, sb = a.get_state(0), b.get_state(0)
    for k in ("u", "v", "phi", "phiv"):
        np.testing.assert_array_equal(sa[k], sb[k])
    assert [r["iters"] for r in reps] == list(iters)
    assert all(r["fails"] == 0 for r in reps)
    # a second run continues from the committed state and reuses the captured graph
    s, _ = a.batch_run(1e-14, 1.0, H, angles)
    assert s == fg.FG_OK
    assert a.batch_run_info()[0] == graph
    u = a.get_state(0)["u"]
    assert np.allclose(np.linalg.norm(u, axis=1), 1.0, atol=1e-12)


@pytest.mark.parametrize("lpr", [4, 8])
def test_batch_solver_lanes_per_row(lpr):
    """The group-per-row operator applications give the thread-per-row solution to the
    solver tolerance (only the order of the row sums differs)."""
    ms, us = _samples()
    ref = _batch(ms, us)
    opts = dict(OPTS, solver_lpr=lpr)
    b = fg.Context(ms, cases.regions(alpha=0.1), **opts)
    b.set_state(np.concatenate(us))
    b.batch_compute_all(None, energies=False)
    for k in range(2):
        s1, _ = ref.batch_step(1e-14, 1.0, H, [0.4 + k, 1.2, 2.3])
        s2, reps = b.batch_step(1e-14, 1.0, H, [0.4 + k, 1.2, 2.3])
        assert s1 == fg.FG_OK and s2 == fg.FG_OK
        assert _rel(b.get_state(1)["v"], ref.get_state(1)["v"]) < 1e-7
        assert b.solver_lanes_per_row() == lpr
        ref.batch_compute_all(None, energies=False)
        b.batch_compute_all(None, energies=False)



def test_fp64_batch_steps_like_single_fp64_contexts_and_the_oracle():
    """precision FG_PREC_FP64 in a batch: the plain FP64 BiCGSTAB per sample (k_bicg64_seg,
    the iteration of bicg_dir, src/algebra/bicg.h:163-234, with each sample's own scalars and
    stopping test) and the FP64 forest FMM. Three steps against single FP64 contexts (same
    iteration counts; v within 1e-9 relative: only the order of partial sums and of the
    translations' groups differs), and the first step of every sample against the oracle's
    FP64 step from the same state and potentials (v within 1e-8 relative at tolerance 1e-10)."""
    ms, us = _samples()
    opts = dict(precision=fg.FG_PREC_FP64, demag=fg.FG_DEMAG_FMM, fmm_leaf=-3, tol=1e-10)
    b = fg.Context(ms, cases.regions(alpha=0.1), **opts)
    b.set_state(np.concatenate(us))
    b.batch_compute_all(None, energies=False)
    off = b.node_offsets
    st0 = b.get_state(0)
    singles = []
    for g, (m, u) in enumerate(zip(ms, us)):
        c = fg.Context(m, cases.regions(alpha=0.1), **opts)
        c.set_state(u, st0["v"][off[g]:off[g + 1]], st0["phi"][off[g]:off[g + 1]], st0["phiv"][off[g]:off[g + 1]])
        singles.append(c)
    dt, pref = 1e-14, 1.0
    angles = np.array([0.3, 1.1, 2.0])
    for it in range(3):
        s, reps = b.batch_step(dt, pref, H, angles + it)
        assert s == fg.FG_OK
        vb = b.get_state(1)["v"]
        if it == 0:
            for g, m in enumerate(ms):
                o = fgo.Oracle(m, cases.oracle_regions(alpha=0.1))
                o.set_solver(1e-10, 500)
                sl = slice(off[g], off[g + 1])
                o.set_state(st0["u"][sl], st0["v"][sl], st0["phi"][sl], st0["phiv"][sl])
                o.base_projection(float(angles[g]))
                ro = o.step(dt, pref, H[g])
                assert not ro["fail"]
                assert _rel(vb[sl], o.get_state(1)["v"]) < 1e-8
        for g, c in enumerate(singles):
            r = c.step(dt, pref, H[g], angles[g] + it)
            assert r["status"] == fg.FG_OK
            assert reps[g]["iters"] == r["iters"], (g, reps[g], r)
            assert reps[g]["refinements"] == 0
            assert _rel(vb[off[g]:off[g + 1]], c.get_state(1)["v"]) < 1e-9
            assert reps[g]["res"] <= 1e-10 * reps[g]["rhsn"]
        b.batch_compute_all(None, energies=False)
        for c in singles:
            c.compute_all(np.zeros(3))
    for c in singles:
        c.close()
    b.close()


@pytest.mark.parametrize("batch", [False, True])
def test_device_tree_build_equals_host_tree_build(batch):
    """The octree from the device Morton-key radix sort (fg_opts.fmm_tree_host 0) is the
    octree of the host's comparison sort: the same depth from the occupancy count (the depth
    whose mean sources per leaf is closest to 300), and bit-identical potentials (the same
    tables in the same order)."""
    ms, us = _samples()
    mesh = ms if batch else cases.cuboid(24, 20, 10)
    u = np.concatenate(us) if batch else cases.perturbed_state(mesh["xyz"], seed=5, sigma=0.2)
    phi, info = [], []
    for host in (1, 0):
        opts = dict(OPTS, fmm_leaf=300, fmm_tree_host=host)  # depth from the occupancy count
        c = fg.Context(mesh, cases.regions(alpha=0.1), **opts)
        c.set_state(u)
        if batch:
            c.batch_compute_all(None, energies=False)
        else:
            c.compute_all(np.zeros(3))
        st = c.get_state(0)
        phi.append((st["phi"], st["phiv"]))
        info.append(c.fmm_tree_info())
        c.close()
    print(f"octree set-up, host sort: {info[0]}; device sort: {info[1]}")
    assert info[0]["depth"] == info[1]["depth"]
    assert info[0]["trees"] == info[1]["trees"] == (len(ms) if batch else 1)
    assert info[0]["sort_device_ms"] == 0.0 and info[1]["sort_device_ms"] > 0.0
    for a, b in zip(phi[0], phi[1]):
        np.testing.assert_array_equal(a, b)


def test_batch_learned_guess():
    """The learned guess inside a batch (FP32 + refinement): one network for all samples,
    trained by fg_batch_step on the batch's solutions (src/linear_algebra.cpp:13-24 is the
    fallback), its candidate formed and judged per sample inside the solver. After the
    training solves: every sample converges to the tolerance, the judged initial residual is
    never above the fallback's, the candidate is taken, and the states agree with the same
    batch stepped with the previous-step guess to the solver's tolerance; a graph-replayed
    run with the frozen network does the same."""
    ms, us = _samples()
    ntrain, nuse = 30, 4
    b = _batch(ms, us, learned_guess=1, mlp_train_steps=ntrain, mlp_train_every=1)
    p = _batch(ms, us)
    rng = np.random.default_rng(21)
    accepted = 0
    for k in range(ntrain + nuse):
        angles = rng.uniform(0, 2 * np.pi, len(ms))
        s1, rb = b.batch_step(1e-14, 1.0, H, angles)
        s2, rp = p.batch_step(1e-14, 1.0, H, angles)
        assert s1 == fg.FG_OK and s2 == fg.FG_OK
        if k >= ntrain:
            for r in rb:
                assert r["res"] <= 1e-9 * r["rhsn"]
                assert r["res0"] <= r["res0_fallback"] * (1 + 1e-12)
                accepted += r["guess_accepted"]
            assert _rel(b.get_state(1)["v"], p.get_state(1)["v"]) < 1e-6
        b.batch_compute_all(None, energies=False)
        p.batch_compute_all(None, energies=False)
    assert accepted > 0
    angles = rng.uniform(0, 2 * np.pi, (3, len(ms)))
    s1, rb = b.batch_run(1e-14, 1.0, H, angles)
    s2, rp = p.batch_run(1e-14, 1.0, H, angles)
    assert s1 == fg.FG_OK and s2 == fg.FG_OK
    assert all(r["fails"] == 0 for r in rb)
    assert b.batch_run_info()[0]
    assert _rel(b.get_state(0)["u"], p.get_state(0)["u"]) < 1e-6
    b.close()
    p.close()
