"""GPU parity of the plain FP64 path against the FP64 oracle.

Both sides start from the same state (u, v, phi, phiv) and the same basis angle. The
GPU assembles the factorised system (static stiffness + per-step diagonals); the oracle
assembles the reference's explicit 2x2-block CSR. Tolerances: basis 1e-14 absolute,
RHS and K x within 1e-12 relative (same algebra, different rounding order); v within
rel-L2 1e-9 when both solve to a relative residual of 1e-12; demag potential within
1e-11 relative (both exact direct sums); energies within 1e-10 relative.
"""
import numpy as np
import pytest

import feellgood_gb300 as fg
from oracle import fgo
from tests import cases

pytestmark = pytest.mark.gpu

DT = 1e-14
DTMAX = 1e-13
UK = (0.3, 0.2, 1.0)


def _setup(nx=6, ny=5, nz=4, K=0.0, K3=0.0, alpha=0.5, seed=1, tol=1e-12, one_point=False, **opts):
    m = cases.cuboid(nx, ny, nz)
    u = cases.perturbed_state(m["xyz"], seed=seed)
    v = cases.tangent_field(u, seed=seed + 1)
    o = fgo.Oracle(m, cases.oracle_regions(alpha=alpha, K=K, uk=UK, K3=K3), one_gauss_point=one_point)
    o.set_solver(tol, 5000)
    o.set_state(u, v)
    H = np.array([2e4, -1e4, 3e4])
    o.compute_all(H)  # phi, phiv of (u, v), then CURRENT <- NEXT
    st = o.get_state(0)
    c = fg.Context(m, cases.regions(alpha=alpha, K=K, uk=UK, K3=K3), tol=tol, max_iter=5000,
                   one_gauss_point=int(one_point), **opts)
    c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    return m, st, H, o, c


def _csr_apply(rowptr, col, val, x):
    y = np.zeros_like(x)
    for r in range(len(x)):
        y[r] = val[rowptr[r]:rowptr[r + 1]] @ x[col[rowptr[r]:rowptr[r + 1]]]
    return y


def _rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


@pytest.mark.parametrize("aniso", [(0.0, 0.0), (4e4, 0.0), (0.0, 2e4)])
@pytest.mark.parametrize("one_point", [False, True])
def test_rhs_and_operator(aniso, one_point):
    K, K3 = aniso
    m, st, H, o, c = _setup(K=K, K3=K3, one_point=one_point)
    angle = 0.41
    pref = fgo.prefactor(DT, DTMAX)
    o.base_projection(angle)
    o.step(DT, pref, H)
    rowptr, col, val, rhs_o = o.export_system()
    rep = c.step(DT, pref, H, angle)
    assert rep["status"] == fg.FG_OK
    rhs_g, ep, eq = c.debug_system()
    ep_o, eq_o = o.basis()
    assert np.max(np.abs(ep - ep_o)) < 1e-14 and np.max(np.abs(eq - eq_o)) < 1e-14
    assert _rel(rhs_g, rhs_o) <= 1e-12
    rng = np.random.default_rng(5)
    for _ in range(3):
        x = rng.normal(size=2 * len(m["xyz"]))
        assert _rel(c.debug_apply(x), _csr_apply(rowptr, col, val, x)) <= 1e-12


@pytest.mark.parametrize("nodes", [(6, 5, 4), (10, 10, 3)])
def test_solve_and_update(nodes):
    m, st, H, o, c = _setup(*nodes)
    angle = 1.1 * 0.5
    pref = fgo.prefactor(DT, DTMAX)
    o.base_projection(angle)
    ro = o.step(DT, pref, H)
    rg = c.step(DT, pref, H, angle)
    assert not ro["fail"] and rg["status"] == fg.FG_OK
    so, sg = o.get_state(1), c.get_state(1)
    assert _rel(sg["v"], so["v"]) <= 1e-9
    assert np.max(np.abs(sg["u"] - so["u"])) <= 1e-12
    assert abs(rg["vmax"] - ro["vmax"]) <= 1e-9 * ro["vmax"]
    assert abs(rg["iters"] - ro["iters"]) <= 2
    assert abs(rg["rhsn"] - ro["rhsn"]) <= 1e-12 * ro["rhsn"]


def test_solver_failure_is_reported():
    """max(iter)=1 forces ITER_OVERFLOW on both sides (iter.h:119-125); NEXT is not written."""
    m, st, H, o, c = _setup(tol=1e-14)
    o.set_solver(1e-14, 1)
    c2 = fg.Context(m, cases.regions(), tol=1e-14, max_iter=1)
    c2.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    pref = fgo.prefactor(DT, DTMAX)
    o.base_projection(0.2)
    ro = o.step(DT, pref, H)
    rg = c2.step(DT, pref, H, 0.2)
    assert ro["fail"] and ro["status"] == 1
    assert rg["status"] == fg.FG_SOLVER_ITER_OVERFLOW
    assert np.array_equal(c2.get_state(1)["u"], st["u"])


@pytest.mark.parametrize("one_point", [False, True])
def test_compute_all(one_point):
    m, st, H, o, c = _setup(8, 6, 5, K=3e4, one_point=one_point)
    pref = fgo.prefactor(DT, DTMAX)
    o.base_projection(0.3)
    o.step(DT, pref, H)
    c.step(DT, pref, H, 0.3)
    Eo = o.compute_all(H)
    Eg = c.compute_all(H)
    so, sg = o.get_state(0), c.get_state(0)
    assert _rel(sg["phi"], so["phi"]) <= 1e-11
    assert _rel(sg["phiv"], so["phiv"]) <= 1e-11
    for k in range(4):
        assert abs(Eg[k] - Eo[k]) <= 1e-10 * np.max(np.abs(Eo)), (k, Eg, Eo)
    avg = c.average(0)
    for d in range(3):
        assert abs(avg[d] - o.avg(0, d)) <= 1e-12


def test_state_round_trip_pinned():
    """fg_set_state fills CURRENT and NEXT (one host upload, NEXT copied on the device);
    fg_get_state writes into caller buffers, pinned (fg_host_alloc) or pageable, bit for bit;
    malformed output buffers are refused before any copy."""
    m, st, H, o, c = _setup()
    nn = len(m["xyz"])
    host = {"u": fg.pinned_empty((nn, 3)), "v": fg.pinned_empty((nn, 3)), "phi": fg.pinned_empty(nn),
            "phiv": fg.pinned_empty(nn)}
    for k in host:
        host[k][...] = st[k]
    c.set_state(host["u"], host["v"], host["phi"], host["phiv"])
    for which in (0, 1):
        out = {k: fg.pinned_empty(a.shape) for k, a in host.items()}
        assert c.get_state(which, out=out) is out
        for k in host:
            assert np.array_equal(out[k], st[k])
        pageable = c.get_state(which)
        for k in host:
            assert np.array_equal(pageable[k], st[k])
    with pytest.raises(ValueError):
        c.get_state(0, out={"u": np.zeros((nn, 3), np.float32), "v": host["v"], "phi": host["phi"],
                            "phiv": host["phiv"]})


def test_bad_mesh_is_rejected():
    m = cases.cuboid(2, 2, 2)
    bad = dict(m)
    t = m["tets"].copy()
    t[0, 2], t[0, 3] = t[0, 3], t[0, 2]  # negative Jacobian
    bad["tets"] = t
    with pytest.raises(fg.FgError) as e:
        fg.Context(bad, cases.regions())
    assert e.value.status == 7
    bad2 = dict(m)
    t2 = m["tets"].copy()
    t2[1, 0] = len(m["xyz"]) + 5
    bad2["tets"] = t2
    with pytest.raises(fg.FgError):
        fg.Context(bad2, cases.regions())


@pytest.mark.parametrize("tol", [1e-6, 1e-10])
def test_mixed_precision_solve(tol):
    """FP32 Krylov body + FP64 refinement stops on the true FP64 residual at the same
    tolerance; its v agrees with the FP64 oracle to within the tolerance's reach."""
    m, st, H, o, c = _setup(10, 10, 4, tol=tol)
    cm = fg.Context(m, cases.regions(), tol=tol, max_iter=5000, precision=fg.FG_PREC_FP32_REFINE)
    cm.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    pref = fgo.prefactor(DT, DTMAX)
    o.set_solver(1e-13, 5000)
    o.base_projection(0.9)
    ro = o.step(DT, pref, H)
    rg = cm.step(DT, pref, H, 0.9)
    assert rg["status"] == fg.FG_OK and not ro["fail"]
    assert rg["res"] <= tol * rg["rhsn"]
    assert rg["refinements"] >= 1
    so, sg = o.get_state(1), cm.get_state(1)
    assert _rel(sg["v"], so["v"]) <= 50 * tol
    assert np.max(np.abs(np.linalg.norm(sg["u"], axis=1) - 1.0)) < 1e-14


@pytest.mark.parametrize("lpr,threads", [(1, 256), (1, 512), (4, 512), (8, 512)])
def test_mixed_solver_block_shapes(lpr, threads):
    """The FP32 + refinement solver with 256- or 512-thread persistent blocks (one of 512 per
    SM: the same kernel, its reductions over 16 warps) on a mesh that spreads over many blocks:
    the same FP64 stopping test, and v within the tolerance's reach of the FP64 solver's."""
    tol = 1e-10
    m = cases.cuboid(40, 40, 10)
    u = cases.perturbed_state(m["xyz"], seed=21, sigma=0.3)
    v = cases.tangent_field(u, seed=22)
    H = np.array([0.0, 0.0, 0.02])
    phi0 = np.zeros(len(u))
    out = {}
    for prec, kw in ((fg.FG_PREC_FP64, {}), (fg.FG_PREC_FP32_REFINE, dict(solver_lpr=lpr, solver_threads=threads))):
        c = fg.Context(m, cases.regions(), tol=tol, max_iter=5000, precision=prec, demag=fg.FG_DEMAG_DIRECT, **kw)
        c.set_state(u, v, phi0, phi0)  # the same (zero) potentials for both solvers
        r = c.step(DT, 1.0, H, 0.3)
        assert r["status"] == fg.FG_OK and r["res"] <= tol * r["rhsn"]
        out[prec] = c.get_state(1)["v"]
        c.close()
    assert _rel(out[fg.FG_PREC_FP32_REFINE], out[fg.FG_PREC_FP64]) <= 50 * tol


@pytest.mark.parametrize("one_point", [False, True])
def test_surface_anisotropy(one_point):
    """Tri::integrales (src/triangle.cpp:6-36): the surface anisotropy of the magnetic
    triangles enters the RHS of their nodes; RHS within 1e-12 of the oracle's explicit
    assembly, the solution within 1e-9. Kbis = 2 Ks / dMs carries the sign of the
    triangle's dMs (+-Ms by orientation, src/mesh.cpp:239); the structured test mesh
    alternates orientations, which would cancel the term at shared nodes, so the test
    gives every triangle dMs = +Ms (both sides get the same mesh)."""
    m = cases.cuboid(6, 5, 4)
    m["dMs"] = np.abs(m["dMs"])
    u = cases.perturbed_state(m["xyz"], seed=21)
    v = cases.tangent_field(u, seed=22)
    ks, uks = 500.0, (0.2, -0.4, 1.0)
    # the cuboid's boundary triangles are in surface region 1
    o = fgo.Oracle(m, cases.oracle_regions(alpha=0.5), [fgo.make_tri_region(), fgo.make_tri_region(Ks=ks, uk=uks)],
                   one_gauss_point=one_point)
    o.set_solver(1e-12, 5000)
    o.set_state(u, v)
    H = np.array([2e4, -1e4, 3e4])
    o.compute_all(H)
    st = o.get_state(0)
    c = fg.Context(m, cases.regions(alpha=0.5), [dict(), dict(Ks=ks, uk=uks)], tol=1e-12, max_iter=5000,
                   one_gauss_point=int(one_point))
    c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    angle, pref = 0.73, fgo.prefactor(DT, DTMAX)
    o.base_projection(angle)
    ro = o.step(DT, pref, H)
    rowptr, col, val, rhs_o = o.export_system()
    rg = c.step(DT, pref, H, angle)
    assert not ro["fail"] and rg["status"] == fg.FG_OK
    rhs_g, _, _ = c.debug_system()
    assert _rel(rhs_g, rhs_o) <= 1e-12
    # the surface term is a visible part of the RHS
    o2 = fgo.Oracle(m, cases.oracle_regions(alpha=0.5), one_gauss_point=one_point)
    o2.set_solver(1e-12, 5000)
    o2.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    o2.base_projection(angle)
    o2.step(DT, pref, H)
    assert _rel(o2.export_system()[3], rhs_o) > 1e-2
    assert _rel(c.get_state(1)["v"], o.get_state(1)["v"]) <= 1e-9


@pytest.mark.parametrize("K", [0.0, 4e4])
def test_space_field(K):
    """R4toR3 applied field B(x, t) = A(t) f(x): f at the magnetic tets' Gauss points
    (mesh::setExtSpaceField, src/mesh.cpp:377-389), A per step; the applied field is
    Hext + A f(g). RHS within 1e-12 of the oracle, v within 1e-9, energies within 1e-10
    (both the isotropic element kernel and the general one with anisotropy)."""
    m = cases.cuboid(6, 5, 4)
    u = cases.perturbed_state(m["xyz"], seed=31)
    v = cases.tangent_field(u, seed=32)
    regs_o, regs_g = cases.oracle_regions(alpha=0.5, K=K, uk=UK), cases.regions(alpha=0.5, K=K, uk=UK)
    c = fg.Context(m, regs_g, tol=1e-12, max_iter=5000)
    pts = c.gauss_points()
    assert pts.shape == (len(m["tets"]) * 5, 3)
    s = pts / 3e-9
    f = 4e4 * np.stack([np.sin(s[:, 0]), np.cos(s[:, 1]), np.sin(s[:, 2] + s[:, 0])], axis=1)
    amp, H = 0.7, np.array([1e4, 0.0, -2e4])
    o = fgo.Oracle(m, regs_o)
    o.set_solver(1e-12, 5000)
    o.set_space_field(f, amp)
    o.set_state(u, v)
    o.compute_all(H)
    st = o.get_state(0)
    c.set_space_field(f)
    c.set_field_amplitude(amp)
    c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    angle, pref = 0.37, fgo.prefactor(DT, DTMAX)
    o.base_projection(angle)
    ro = o.step(DT, pref, H)
    rowptr, col, val, rhs_o = o.export_system()
    rg = c.step(DT, pref, H, angle)
    assert not ro["fail"] and rg["status"] == fg.FG_OK
    assert _rel(c.debug_system()[0], rhs_o) <= 1e-12
    assert _rel(c.get_state(1)["v"], o.get_state(1)["v"]) <= 1e-9
    Eo, Eg = o.compute_all(H), c.compute_all(H)
    for k in range(4):
        assert abs(Eg[k] - Eo[k]) <= 1e-10 * np.max(np.abs(Eo)), (k, Eg, Eo)
    # the space field is a visible part of the RHS and of the Zeeman energy
    c.set_space_field(None)
    c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    c.step(DT, pref, H, angle)
    assert _rel(c.debug_system()[0], rhs_o) > 1e-3


def _spin_case():
    """Cuboid with the bottom face (V = 0, s = 0) and the top face (jn, uP) as the two
    boundary surfaces of the electrostatic and spin-diffusion problems."""
    m = cases.cuboid(6, 5, 4)
    z = m["xyz"][:, 2]
    reg = np.ones(len(m["tris"]), np.int32)
    for f, t in enumerate(m["tris"]):
        if np.all(np.abs(z[t] - z.min()) < 1e-15):
            reg[f] = 2
        if np.all(np.abs(z[t] - z.max()) < 1e-15):
            reg[f] = 3
    m["tri_reg"] = reg
    sp = dict(sigma=5e6, P=0.5, lsd=1e-9, lsf=5e-9)
    regs_o = [fgo.make_region(N0=1e47, **sp), fgo.make_region(A=cases.AE, Ms=cases.MS, alpha=0.5, N0=1e47, **sp)]
    regs_g = [dict(Ae=1e-11, Ms=795774.7, alpha=0.5, dens_state=1e47, **sp),
              dict(Ae=cases.AE, Ms=cases.MS, alpha=0.5, dens_state=1e47, **sp)]
    bc = [dict(), dict(), dict(V=0.0, s=(0, 0, 0)), dict(jn=1e6, uP=(0, 1, 0))]
    tregs_o = [fgo.make_tri_region(**b) for b in bc]
    return m, regs_o, regs_g, tregs_o, bc


def test_spin_accumulation():
    """Spin accumulation coupling (spinAcc, electrostatSolver): the potential V (CG, once),
    the spin accumulation s (BiCGSTAB with Dirichlet values, every compute_all, operator with
    the CURRENT and RHS with the NEXT magnetisation) and its field Hst in the next step's
    element integrals, against the oracle's explicit assembly: V within 1e-10, s within
    1e-8 (both solved to 1e-12), the step's RHS within 1e-9 and v within 1e-8."""
    m, regs_o, regs_g, tregs_o, bc = _spin_case()
    u = cases.perturbed_state(m["xyz"], seed=41)
    v = cases.tangent_field(u, seed=42)
    H = np.array([2e4, -1e4, 3e4])
    o = fgo.Oracle(m, regs_o, tregs_o)
    assert o.set_spin(True, 1e-12, 5000)[0] == 0
    o.set_solver(1e-12, 5000)
    o.set_state(u, v)
    o.compute_all(H)
    st = o.get_state(0)
    Vo, so, sst, _ = o.spin()
    assert sst == 0 and np.abs(so).max() > 0
    c = fg.Context(m, regs_g, bc, tol=1e-12, max_iter=5000, spin_acc=1, spin_tol=1e-12, spin_max_iter=5000)
    c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    c.compute_all(H)
    info = c.spin_info()
    assert info["status"] == fg.FG_OK
    assert _rel(info["V"], Vo) <= 1e-10
    assert _rel(c.get_spin(), so) <= 1e-8
    angle, pref = 0.5, fgo.prefactor(DT, DTMAX)
    o.base_projection(angle)
    ro = o.step(DT, pref, H)
    rhs_o = o.export_system()[3]
    rg = c.step(DT, pref, H, angle)
    assert not ro["fail"] and rg["status"] == fg.FG_OK
    assert _rel(c.debug_system()[0], rhs_o) <= 1e-9
    assert _rel(c.get_state(1)["v"], o.get_state(1)["v"]) <= 1e-8
    # Hst is a visible part of the RHS
    o2 = fgo.Oracle(m, regs_o, tregs_o)
    o2.set_solver(1e-12, 5000)
    o2.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    o2.base_projection(angle)
    o2.step(DT, pref, H)
    assert _rel(o2.export_system()[3], rhs_o) > 1e-2


@pytest.mark.parametrize("spin_tol", [1e-12, 1e-8])
def test_spin_accumulation_fp32_refine(spin_tol):
    """In FG_PREC_FP32_REFINE the spin problem is solved with an FP32 BiCGSTAB body and FP64
    refinement: the same stopping test on the true FP64 residual, so s agrees with the
    oracle's FP64 bicg_dir solution to the level the tolerance allows (1e-8 at a solve
    tolerance of 1e-12, 1e-5 at 1e-8), and the step's RHS carries the same Hst."""
    m, regs_o, regs_g, tregs_o, bc = _spin_case()
    u = cases.perturbed_state(m["xyz"], seed=43)
    v = cases.tangent_field(u, seed=44)
    H = np.array([1e4, 2e4, -3e4])
    o = fgo.Oracle(m, regs_o, tregs_o)
    assert o.set_spin(True, 1e-12, 5000)[0] == 0
    o.set_solver(1e-12, 5000)
    o.set_state(u, v)
    o.compute_all(H)
    st = o.get_state(0)
    _, so, sst, _ = o.spin()
    assert sst == 0
    c = fg.Context(m, regs_g, bc, tol=1e-12, max_iter=5000, spin_acc=1, spin_tol=spin_tol, spin_max_iter=5000,
                   precision=fg.FG_PREC_FP32_REFINE)
    c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    c.compute_all(H)
    info = c.spin_info()
    assert info["status"] == fg.FG_OK and info["iters"] > 0
    assert _rel(c.get_spin(), so) <= (1e-8 if spin_tol < 1e-10 else 1e-5)
    if spin_tol < 1e-10:
        angle, pref = 0.3, fgo.prefactor(DT, DTMAX)
        o.base_projection(angle)
        o.step(DT, pref, H)
        c.step(DT, pref, H, angle)
        assert _rel(c.debug_system()[0], o.export_system()[3]) <= 1e-9


def test_double_single_elements_with_spin(monkeypatch):
    """With the spin coupling the FP32 + refinement path keeps its double-single element
    integrals, the Hst terms of Tet::integrales (src/tetra.cpp:248-303) included: on the same
    state, potentials and s, the assembled RHS and operator agree with those of the FP64
    element kernel (FG_DS_ELEMENTS=0) to 1e-12, while the coupling moves the RHS by far
    more than that."""
    m, regs_o, regs_g, tregs_o, bc = _spin_case()
    u = cases.perturbed_state(m["xyz"], seed=45)
    v = cases.tangent_field(u, seed=46)
    H = np.array([1e4, 2e4, -3e4])
    angle, pref = 0.3, fgo.prefactor(DT, DTMAX)
    xs = np.random.default_rng(47).normal(size=(2, 2 * len(m["xyz"])))
    out = {}
    for name, env, spin in (("ds", None, 1), ("fp64", "0", 1), ("no_spin", None, 0)):
        if env is None:
            monkeypatch.delenv("FG_DS_ELEMENTS", raising=False)
        else:
            monkeypatch.setenv("FG_DS_ELEMENTS", env)
        c = fg.Context(m, regs_g, bc, tol=1e-6, max_iter=5000, spin_acc=spin, spin_tol=1e-12, spin_max_iter=5000,
                       precision=fg.FG_PREC_FP32_REFINE)
        c.set_state(u, v)
        c.compute_all(H)
        if spin:
            assert c.spin_info()["status"] == fg.FG_OK
        c.step(DT, pref, H, angle)
        out[name] = (c.debug_system()[0], [c.debug_apply(x) for x in xs])
        c.close()
    monkeypatch.delenv("FG_DS_ELEMENTS", raising=False)
    rd, ad = out["ds"]
    r64, a64 = out["fp64"]
    print("ds vs FP64 elements with spin: rhs %.2e, operator %.2e; spin's share of the rhs %.2e"
          % (_rel(rd, r64), max(_rel(a, b) for a, b in zip(ad, a64)), _rel(r64, out["no_spin"][0])))
    assert _rel(rd, r64) <= 1e-12
    for a, b in zip(ad, a64):
        assert _rel(a, b) <= 1e-12
    assert _rel(r64, out["no_spin"][0]) >= 1e-6


def test_spin_boundary_conditions_checked():
    """A spin-accumulation context without exactly one jn surface, one V surface and one s
    surface is refused (the reference's checkBoundaryConditions exit)."""
    m, regs_o, regs_g, tregs_o, bc = _spin_case()
    bad = [dict(), dict(), dict(V=0.0), dict(jn=1e6)]
    with pytest.raises(fg.FgError):
        fg.Context(m, regs_g, bad, spin_acc=1)


def _wall(m, z0, width=5.0, seed=51):
    z = m["xyz"][:, 2] / 1e-9
    mz = np.tanh((z0 - z) / width)
    u = np.stack([np.sqrt(np.clip(1 - mz * mz, 0, 1)), np.zeros_like(mz), mz], axis=1)
    u[:, :2] += np.random.default_rng(seed).uniform(-0.02, 0.02, (len(z), 2))
    return u / np.linalg.norm(u, axis=1, keepdims=True)


@pytest.mark.parametrize("z0,expect", [(30.0, 1), (50.0, 0), (-1e3, -1)])
def test_recentering(z0, expect):
    """Fem::recenter (src/recentering.cpp:47-131): a head-to-head wall at z0 in a 10 x 10 x 100 nm
    wire. Off centre the pattern is translated: CURRENT u of every node is NEXT u of the node
    nearest to its shifted position (the oracle searches all nodes, the GPU a grid of cells;
    both exact, so the result is bitwise equal) and NEXT v is zero; at the centre |<m_z>| is
    below the threshold; without a wall (uniform m_z) both report the reference's error."""
    m = cases.cuboid(4, 4, 40)
    u = _wall(m, z0)
    v = cases.tangent_field(u, seed=52)
    H = np.zeros(3)
    o = fgo.Oracle(m, cases.oracle_regions(alpha=0.5))
    o.set_state(u, v)
    o.compute_all(H)
    c = fg.Context(m, cases.regions(alpha=0.5))
    c.set_state(u, v)
    c.compute_all(H)
    r = o.recenter(2, 0.1)
    assert r == expect
    if expect < 0:
        with pytest.raises(fg.FgError):
            c.recenter("Z", 0.1)
        return
    assert c.recenter("Z", 0.1) == bool(expect)
    so, sg = o.get_state(0), c.get_state(0)
    assert np.array_equal(sg["u"], so["u"])
    if expect:
        assert not np.array_equal(sg["u"], u)
        assert np.array_equal(c.get_state(1)["v"], np.zeros_like(v))
        assert np.array_equal(o.get_state(1)["v"], np.zeros_like(v))


@pytest.mark.parametrize("direction,K,precision", [(0, 0.0, fg.FG_PREC_FP64), (2, 0.0, fg.FG_PREC_FP32_REFINE),
                                                   (1, 3e4, fg.FG_PREC_FP64)])
def test_recentering_drift(direction, K, precision):
    """Tet::add_drift_BE (src/tetra.cpp:150-169): with a drift direction and speed the
    element integrals gain vdrift w_g a_i(g) (alpha dU + U x dU + s_dt (alpha dV + U x dV +
    V x dU)). The assembled RHS matches the oracle's to 1e-12 (the operator is unchanged),
    the term is a visible part of the RHS, and a zero speed or no direction leaves the
    step as it was."""
    m, st, H, o, c = _setup(K=K, precision=precision)
    angle, pref = 0.37, fgo.prefactor(DT, DTMAX)
    vdrift = 5e-3
    o.set_drift(direction, vdrift)
    o.base_projection(angle)
    o.step(DT, pref, H)
    rowptr, col, val, rhs_o = o.export_system()
    c.set_drift(direction, vdrift)
    assert c.step(DT, pref, H, angle)["status"] == fg.FG_OK
    rhs_g = c.debug_system()[0]
    assert _rel(rhs_g, rhs_o) <= 1e-12
    x = np.random.default_rng(3).normal(size=2 * len(m["xyz"]))
    assert _rel(c.debug_apply(x), _csr_apply(rowptr, col, val, x)) <= 1e-12
    # without the drift (speed 0, then no direction) the RHS differs visibly and matches the
    # oracle's drift-free system
    o2 = fgo.Oracle(m, cases.oracle_regions(alpha=0.5, K=K, uk=UK))
    o2.set_solver(1e-12, 5000)
    o2.set_state(st["u"], st["v"], st["phi"], st["phiv"])
    o2.base_projection(angle)
    o2.step(DT, pref, H)
    rhs_0 = o2.export_system()[3]
    assert _rel(rhs_0, rhs_o) > 1e-3
    for d, vd in ((direction, 0.0), (-1, vdrift)):
        c.set_state(st["u"], st["v"], st["phi"], st["phiv"])
        c.set_drift(d, vd)
        assert c.step(DT, pref, H, angle)["status"] == fg.FG_OK
        assert _rel(c.debug_system()[0], rhs_0) <= 1e-12
    with pytest.raises(fg.FgError):
        c.set_drift(3, 1.0)


@pytest.mark.parametrize("one_point", [False, True])
def test_double_single_elements(one_point):
    """The FP32 + refinement path computes the isotropic element integrals in double-single
    arithmetic (slots summed in double-single per node, then FP64): its assembled RHS and
    operator agree with the oracle's FP64 assembly to 1e-12 like the FP64 path's."""
    m, st, H, o, c = _setup(one_point=one_point, precision=fg.FG_PREC_FP32_REFINE)
    angle = 0.41
    pref = fgo.prefactor(DT, DTMAX)
    o.base_projection(angle)
    o.step(DT, pref, H)
    rowptr, col, val, rhs_o = o.export_system()
    rep = c.step(DT, pref, H, angle)
    assert rep["status"] == fg.FG_OK
    rhs_g, _, _ = c.debug_system()
    assert _rel(rhs_g, rhs_o) <= 1e-12
    rng = np.random.default_rng(7)
    for _ in range(3):
        x = rng.normal(size=2 * len(m["xyz"]))
        assert _rel(c.debug_apply(x), _csr_apply(rowptr, col, val, x)) <= 1e-12
    # energies of the new state: the isotropic energy kernel of this path is double-single too
    c.set_state(o.get_state(1)["u"], o.get_state(1)["v"])
    Eg = c.compute_all(H)
    Eo = o.compute_all(H)
    for k in range(4):
        assert abs(Eg[k] - Eo[k]) <= 1e-10 * np.max(np.abs(Eo)), (k, Eg, Eo)
