"""ctypes wrapper of the oracle's C++ restatement (oracle/fgoracle.cpp). TEST INFRASTRUCTURE ONLY."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

MU0 = 1.25663706127e-6
GAMMA0 = 1.76085962784e11 * MU0

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class Region(C.Structure):
    _fields_ = [("A", C.c_double), ("Ms", C.c_double), ("K", C.c_double), ("uk", C.c_double * 3),
                ("K3", C.c_double), ("ex", C.c_double * 3), ("ey", C.c_double * 3), ("ez", C.c_double * 3),
                ("alpha", C.c_double), ("sigma", C.c_double), ("N0", C.c_double), ("P", C.c_double),
                ("lsd", C.c_double), ("lsf", C.c_double)]


class TriRegion(C.Structure):
    _fields_ = [("Ks", C.c_double), ("uk", C.c_double * 3), ("suppress_charges", C.c_int), ("jn", C.c_double),
                ("V", C.c_double), ("uP", C.c_double * 3), ("s", C.c_double * 3)]


def make_region(A=1e-11, Ms=795774.7, K=0.0, uk=(0, 0, 1), K3=0.0, ex=(1, 0, 0), ey=(0, 1, 0), ez=(0, 0, 1),
                alpha=0.5, sigma=0.0, N0=0.0, P=0.0, lsd=0.0, lsf=0.0):
    def unit(v):
        v = np.asarray(v, float)
        return v / np.linalg.norm(v)
    r = Region()
    r.A, r.Ms, r.K, r.K3, r.alpha = A, Ms, K, K3, alpha
    r.sigma, r.N0, r.P, r.lsd, r.lsf = sigma, N0, P, lsd, lsf
    for name, v in (("uk", uk), ("ex", ex), ("ey", ey), ("ez", ez)):
        getattr(r, name)[:] = list(unit(v))
    return r


def make_tri_region(Ks=0.0, uk=(0, 0, 1), suppress_charges=False, jn=None, V=None, uP=(0, 0, 1), s=None):
    r = TriRegion()
    r.Ks = Ks
    u = np.asarray(uk, float)
    r.uk[:] = list(u / np.linalg.norm(u))
    r.suppress_charges = int(bool(suppress_charges))
    r.jn = float("nan") if jn is None else jn
    r.V = float("nan") if V is None else V
    p = np.asarray(uP, float)
    r.uP[:] = list(p / np.linalg.norm(p))
    r.s[:] = [float("nan")] * 3 if s is None else list(np.asarray(s, float))
    return r


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.fgo_create.restype = C.c_void_p
        L.fgo_create.argtypes = [C.c_int, _dp, C.c_int, _ip, _ip, C.c_int, _ip, _ip, _dp, C.c_int,
                                 C.POINTER(Region), C.c_int, C.POINTER(TriRegion), C.c_int]
        L.fgo_destroy.argtypes = [C.c_void_p]
        L.fgo_set_demag.argtypes = [C.c_void_p, C.c_int]
        L.fgo_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.fgo_max_threads.restype = C.c_int
        L.fgo_set_solver.argtypes = [C.c_void_p, C.c_double, C.c_int]
        L.fgo_set_space_field.argtypes = [C.c_void_p, C.c_void_p, C.c_double]
        L.fgo_set_drift.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.fgo_recenter.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.fgo_recenter.restype = C.c_int
        L.fgo_set_spin.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_int),
                                   C.POINTER(C.c_int)]
        L.fgo_get_spin.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.fgo_set_state.argtypes = [C.c_void_p, _dp, C.c_void_p, C.c_void_p, C.c_void_p]
        L.fgo_get_state.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]
        L.fgo_get_basis.argtypes = [C.c_void_p, _dp, _dp]
        L.fgo_base_projection.argtypes = [C.c_void_p, C.c_double]
        L.fgo_step.restype = C.c_int
        L.fgo_step.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp, C.POINTER(C.c_int), C.POINTER(C.c_int),
                               C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.fgo_compute_all.argtypes = [C.c_void_p, _dp, C.c_int, _dp]
        L.fgo_demag.argtypes = [C.c_void_p, C.c_int, _dp]
        L.fgo_num_sources.restype = C.c_int
        L.fgo_num_sources.argtypes = [C.c_void_p]
        L.fgo_charges.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.fgo_energy.argtypes = [C.c_void_p, _dp, _dp]
        L.fgo_avg.restype = C.c_double
        L.fgo_avg.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.fgo_nnz.restype = C.c_int
        L.fgo_nnz.argtypes = [C.c_void_p]
        L.fgo_export_system.argtypes = [C.c_void_p, _ip, _ip, _dp, _dp]
        L.fgo_export_elements.argtypes = [C.c_void_p, _dp, _dp]
        L.fgo_export_solution.argtypes = [C.c_void_p, _dp]
        L.fgo_srand.argtypes = [C.c_uint]
        L.fgo_draw_angle.restype = C.c_double
        L.fgo_time_integration.restype = C.c_int
        L.fgo_time_integration.argtypes = [C.c_void_p, C.c_uint, C.c_double, C.c_double, C.c_double, C.c_double,
                                           C.c_double, _dp, C.c_int, _dp, C.c_int, C.POINTER(C.c_int), _dp]
        _lib = L
    return _lib


def prefactor(dt, dtmax):
    """timing::set_dt (src/time_integration.h:37-42)."""
    tt = dt / (100.0 * dtmax)
    return 1.0 + tt * abs(np.log(tt))


class Oracle:
    """FP64 restatement of the reference per-step path on one set-up mesh."""

    def __init__(self, mesh, regions, tri_regions=None, one_gauss_point=False, threads=0):
        L = lib()
        self.L = L
        xyz = np.ascontiguousarray(mesh["xyz"], dtype=np.float64)
        tets = np.ascontiguousarray(mesh["tets"], dtype=np.int32)
        treg = np.ascontiguousarray(mesh["tet_reg"], dtype=np.int32)
        tris = np.ascontiguousarray(mesh["tris"], dtype=np.int32).reshape(-1, 3)
        freg = np.ascontiguousarray(mesh["tri_reg"], dtype=np.int32)
        dms = np.ascontiguousarray(mesh["dMs"], dtype=np.float64)
        if tri_regions is None:
            tri_regions = [make_tri_region() for _ in range(int(freg.max()) + 1 if len(freg) else 1)]
        R = (Region * len(regions))(*regions)
        T = (TriRegion * len(tri_regions))(*tri_regions)
        self.nn, self.nt, self.nf = len(xyz), len(tets), len(tris)
        if len(tris) == 0:
            tris = np.zeros((1, 3), np.int32)
            freg = np.zeros(1, np.int32)
            dms = np.zeros(1)
        self.h = L.fgo_create(self.nn, xyz.ravel(), self.nt, tets.ravel(), treg, self.nf, tris.ravel(), freg, dms,
                              len(regions), R, len(tri_regions), T, int(one_gauss_point))
        if threads:
            L.fgo_set_threads(self.h, threads)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.fgo_destroy(self.h)
            self.h = None

    def set_demag(self, levels):
        """0: exact direct sum; > 0: CPU FMM of that depth (5 = the reference's ScalFMM tree)."""
        self.L.fgo_set_demag(self.h, levels)

    def set_solver(self, tol=1e-6, maxiter=700):
        self.L.fgo_set_solver(self.h, tol, maxiter)

    def recenter(self, direction, threshold):
        """Fem::recenter: 1 translated, 0 below the threshold, -1 no domain wall."""
        return self.L.fgo_recenter(self.h, int(direction), float(threshold))

    def set_spin(self, enable=True, tol=1e-8, maxiter=1000):
        """Spin accumulation on: solves the electrostatic potential now; returns its (status, iters)."""
        st, it = C.c_int(), C.c_int()
        self.L.fgo_set_spin(self.h, int(enable), tol, maxiter, C.byref(st), C.byref(it))
        return st.value, it.value

    def spin(self):
        """(V [nn], s [nn, 3], last spin solve status, iterations)."""
        V, s = np.zeros(self.nn), np.zeros((self.nn, 3))
        st, it = C.c_int(), C.c_int()
        self.L.fgo_get_spin(self.h, V.ctypes.data_as(C.c_void_p), s.ctypes.data_as(C.c_void_p), C.byref(st),
                            C.byref(it))
        return V, s, st.value, it.value

    def set_space_field(self, field, amp=1.0):
        """R4toR3 applied field: f at the magnetic tets' Gauss points ([n_mag_tets * npi, 3],
        magTet order) or None, and its amplitude; the applied field is Hext + amp f(g)."""
        if field is None:
            self.L.fgo_set_space_field(self.h, None, float(amp))
            return
        f = np.ascontiguousarray(field, dtype=np.float64)
        self.L.fgo_set_space_field(self.h, f.ctypes.data_as(C.c_void_p), float(amp))

    def set_drift(self, direction, vdrift):
        """Recentering drift of the element integrals: direction 0/1/2 (x/y/z) or -1, speed m/s."""
        self.L.fgo_set_drift(self.h, int(direction), float(vdrift))

    def set_state(self, u, v=None, phi=None, phiv=None):
        u = np.ascontiguousarray(u, dtype=np.float64).ravel()
        keep = []

        def ptr(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64).ravel()
            keep.append(a)
            return a.ctypes.data_as(C.c_void_p)
        self.L.fgo_set_state(self.h, u, ptr(v), ptr(phi), ptr(phiv))

    def get_state(self, which=1):
        u, v = np.zeros(3 * self.nn), np.zeros(3 * self.nn)
        phi, phiv = np.zeros(self.nn), np.zeros(self.nn)
        self.L.fgo_get_state(self.h, which, u, v, phi, phiv)
        return {"u": u.reshape(-1, 3), "v": v.reshape(-1, 3), "phi": phi, "phiv": phiv}

    def basis(self):
        ep, eq = np.zeros(3 * self.nn), np.zeros(3 * self.nn)
        self.L.fgo_get_basis(self.h, ep, eq)
        return ep.reshape(-1, 3), eq.reshape(-1, 3)

    def base_projection(self, angle):
        self.L.fgo_base_projection(self.h, angle)

    def step(self, dt, pref, Hext):
        st, it = C.c_int(), C.c_int()
        vmax, res, rhsn = C.c_double(), C.c_double(), C.c_double()
        fail = self.L.fgo_step(self.h, dt, pref, np.asarray(Hext, dtype=np.float64), C.byref(st), C.byref(it),
                               C.byref(vmax), C.byref(res), C.byref(rhsn))
        return {"fail": bool(fail), "status": st.value, "iters": it.value, "vmax": vmax.value, "res": res.value,
                "rhsn": rhsn.value}

    def compute_all(self, Hext, first_order=False):
        E = np.zeros(4)
        self.L.fgo_compute_all(self.h, np.asarray(Hext, dtype=np.float64), int(first_order), E)
        return E

    def demag(self, which=0):
        out = np.zeros(self.nn)
        self.L.fgo_demag(self.h, which, out)
        return out

    def charges(self, which=0):
        ns = self.L.fgo_num_sources(self.h)
        pts, q, corr = np.zeros(3 * ns), np.zeros(ns), np.zeros(self.nn)
        self.L.fgo_charges(self.h, which, pts, q, corr)
        return pts.reshape(-1, 3), q, corr

    def energy(self, Hext):
        E = np.zeros(4)
        self.L.fgo_energy(self.h, np.asarray(Hext, dtype=np.float64), E)
        return E

    def avg(self, which, d):
        return self.L.fgo_avg(self.h, which, d)

    def export_system(self):
        nnz = self.L.fgo_nnz(self.h)
        n = 2 * self.nn
        rowptr, col = np.zeros(n + 1, np.int32), np.zeros(nnz, np.int32)
        val, rhs = np.zeros(nnz), np.zeros(n)
        self.L.fgo_export_system(self.h, rowptr, col, val, rhs)
        return rowptr, col, val, rhs

    def export_elements(self):
        Kp, Lp = np.zeros(64 * self.nt), np.zeros(8 * self.nt)
        self.L.fgo_export_elements(self.h, Kp, Lp)
        return Kp.reshape(-1, 8, 8), Lp.reshape(-1, 8)

    def export_solution(self):
        x = np.zeros(2 * self.nn)
        self.L.fgo_export_solution(self.h, x)
        return x

    def time_integration(self, seed, tf, dtmin, dtmax, evol_step, dumax, Hext, first_order=False, max_rows=100000):
        rows = np.zeros(8 * max_rows)
        eaniso = np.zeros(max_rows)
        ns = C.c_int()
        n = self.L.fgo_time_integration(self.h, seed, tf, dtmin, dtmax, evol_step, dumax,
                                        np.asarray(Hext, dtype=np.float64), int(first_order), rows, max_rows,
                                        C.byref(ns), eaniso)
        if n < 0:
            raise RuntimeError("time integration aborted: dt < DTMIN")
        return rows.reshape(-1, 8)[:n], ns.value, eaniso[:n]


def srand(seed):
    lib().fgo_srand(seed)


def draw_angle():
    """The basis angle of one base_projection() call: M_2_PI * U(0,1) from mt19937(rand())."""
    return lib().fgo_draw_angle()
