"""ctypes binding of the fggpu C ABI (include/fggpu.h).

``Context`` mirrors the reference's per-step sequence (src/time_integration.cpp:193-231):
``step`` = base_projection + prepareElements + solve, ``compute_all`` = demag of m and
of v, energy, evolution. Arrays are numpy host arrays in the caller's node numbering.
Loading fails loudly when the library has not been built: nothing here computes on
the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

MU0 = 1.25663706127e-6
GAMMA0 = 1.76085962784e11 * MU0

FG_OK, FG_SOLVER_ITER_OVERFLOW, FG_SOLVER_CANNOT_CONVERGE, FG_ETIMEDOUT = 0, 1, 2, 3
FG_EINVAL, FG_ECUDA, FG_ENOMEM, FG_EMESH, FG_EIO = 4, 5, 6, 7, 8
FG_PREC_FP64, FG_PREC_FP32_REFINE = 0, 1
FG_DEMAG_AUTO, FG_DEMAG_DIRECT, FG_DEMAG_FMM = 0, 1, 2

_HERE = os.path.dirname(os.path.abspath(__file__))


def lib_path():
    return os.path.join(_HERE, "_build", "libfggpu.so")


class FgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"fggpu status {status}: {msg}")
        self.status = status


class fg_mesh(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_tets", C.c_int), ("n_tris", C.c_int), ("xyz", C.c_void_p),
                ("tet4", C.c_void_p), ("tet_region", C.c_void_p), ("tri3", C.c_void_p),
                ("tri_region", C.c_void_p), ("tri_dMs", C.c_void_p)]


class fg_region(C.Structure):
    _fields_ = [("Ae", C.c_double), ("Ms", C.c_double), ("K", C.c_double), ("uk", C.c_double * 3),
                ("K3", C.c_double), ("ex", C.c_double * 3), ("ey", C.c_double * 3), ("ez", C.c_double * 3),
                ("alpha", C.c_double), ("sigma", C.c_double), ("dens_state", C.c_double), ("P", C.c_double),
                ("lsd", C.c_double), ("lsf", C.c_double)]


class fg_tri_region(C.Structure):
    _fields_ = [("Ks", C.c_double), ("uk", C.c_double * 3), ("suppress_charges", C.c_int), ("jn", C.c_double),
                ("V", C.c_double), ("uP", C.c_double * 3), ("s", C.c_double * 3)]


class fg_opts(C.Structure):
    _fields_ = [("tol", C.c_double), ("max_iter", C.c_int), ("precision", C.c_int), ("learned_guess", C.c_int),
                ("demag", C.c_int), ("fmm_order", C.c_int), ("fmm_leaf", C.c_int), ("one_gauss_point", C.c_int),
                ("first_order", C.c_int), ("refine_max", C.c_int), ("inner_tol", C.c_double),
                ("verbose", C.c_int), ("profile", C.c_int), ("mlp_train_steps", C.c_int), ("mlp_batch", C.c_int),
                ("mlp_lr", C.c_double), ("fmm_tensor", C.c_int),
                ("mlp_train_every", C.c_int), ("fmm_native_fp64", C.c_int),
                ("solver_lpr", C.c_int), ("solver_blocks", C.c_int), ("spin_acc", C.c_int), ("spin_tol", C.c_double),
                ("spin_max_iter", C.c_int), ("demag_increment", C.c_int), ("fmm_overlap", C.c_int),
                ("fmm_tree_host", C.c_int), ("solver_threads", C.c_int)]


class fg_step_report(C.Structure):
    _fields_ = [("status", C.c_int), ("iters", C.c_int), ("refinements", C.c_int), ("guess_accepted", C.c_int),
                ("vmax", C.c_double), ("res", C.c_double), ("rhsn", C.c_double), ("res0", C.c_double),
                ("res0_fallback", C.c_double)]


class fg_batch_report(C.Structure):
    _fields_ = [("fails", C.c_int), ("first_fail", C.c_int), ("iters_max", C.c_int), ("refinements_max", C.c_int),
                ("iters", C.c_longlong), ("refinements", C.c_longlong), ("vmax", C.c_double)]


StepReport = dict

_dp = C.POINTER(C.c_double)
_lib = None

# every symbol include/fggpu.h declares, with (restype, argtypes)
SIGNATURES = {
    "fg_opts_default": (None, [C.POINTER(fg_opts)]),
    "fg_strerror": (C.c_char_p, [C.c_int]),
    "fg_last_error": (C.c_char_p, [C.c_void_p]),
    "fg_create": (C.c_int, [C.POINTER(fg_mesh), C.POINTER(fg_region), C.c_int, C.POINTER(fg_tri_region), C.c_int,
                            C.POINTER(fg_opts), C.POINTER(C.c_void_p)]),
    "fg_destroy": (None, [C.c_void_p]),
    "fg_set_state": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fg_step": (C.c_int, [C.c_void_p, C.c_double, C.c_double, _dp, C.c_double, C.POINTER(fg_step_report)]),
    "fg_compute_all": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fg_get_state": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fg_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "fg_set_drift": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "fg_host_free": (C.c_int, [C.c_void_p]),
    "fg_demag": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "fg_energy": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fg_energy_noalloc": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fg_average": (C.c_int, [C.c_void_p, C.c_int, _dp]),
    "fg_debug_system": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "fg_debug_apply": (C.c_int, [C.c_void_p, _dp, _dp]),
    "fg_timings": (C.c_int, [C.c_void_p, _dp]),
    "fg_counters": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong)]),
    "fg_mesh_load_msh": (C.c_int, [C.c_char_p, C.c_double, C.c_int, C.POINTER(C.c_char_p), _dp, C.c_int,
                                   C.POINTER(C.c_char_p), C.POINTER(C.c_void_p)]),
    "fg_mesh_cuboid": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_double, C.POINTER(C.c_void_p)]),
    "fg_mesh_view": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fg_mesh_free": (None, [C.c_void_p]),
    "fg_mesh_last_error": (C.c_char_p, []),
    "fg_run": (C.c_int, [C.c_char_p, C.c_uint, C.c_int, C.c_void_p]),
    "fg_run_last_error": (C.c_char_p, []),
    "fg_run_request_stop": (None, []),
    "fg_settings_dump": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int]),
    "fg_rng_seed": (None, [C.c_uint]),
    "fg_rng_angle": (C.c_double, []),
    "fg_fmm_timings": (C.c_int, [C.c_void_p, _dp]),
    "fg_fmm_tree_info": (C.c_int, [C.c_void_p, _dp]),
    "fg_mlp_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), _dp]),
    "fg_mlp_debug_grad": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p]),
    "fg_mlp_nparam": (C.c_int, []),
    "fg_mlp_debug_infer": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "fg_solver_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "fg_debug_wait_timeout": (C.c_int, [C.c_void_p, C.c_int]),
    "fg_gauss_points": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_void_p]),
    "fg_spin_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p, C.POINTER(C.c_int),
                               C.POINTER(C.c_double)]),
    "fg_get_spin": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fg_recenter": (C.c_int, [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_int)]),
    "fg_set_space_field": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fg_set_field_amplitude": (C.c_int, [C.c_void_p, C.c_double]),
    "fg_checkpoint_peek": (C.c_int, [C.c_char_p, C.c_void_p, C.c_void_p]),
    "fg_debug_tc_resources": (C.c_int, [C.POINTER(C.c_int)]),
    "fg_measure_peaks": (C.c_int, [_dp]),
    "fg_debug_translate_tc": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_int]),
    "fg_batch_create": (C.c_int, [C.POINTER(fg_mesh), C.c_int, C.POINTER(fg_region), C.c_int,
                                  C.POINTER(fg_tri_region), C.c_int, C.POINTER(fg_opts), C.POINTER(C.c_void_p)]),
    "fg_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.c_void_p]),
    "fg_batch_step": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(fg_step_report)]),
    "fg_batch_compute_all": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fg_batch_run": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(fg_batch_report)]),
    "fg_batch_run_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), _dp]),
}


class fg_mesh_data(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_tets", C.c_int), ("n_tris", C.c_int), ("xyz", C.POINTER(C.c_double)),
                ("tet4", C.POINTER(C.c_int32)), ("tet_region", C.POINTER(C.c_int32)),
                ("tri3", C.POINTER(C.c_int32)), ("tri_region", C.POINTER(C.c_int32)),
                ("tri_dMs", C.POINTER(C.c_double)), ("node_index", C.POINTER(C.c_int32)),
                ("n_vol_regions", C.c_int), ("n_surf_regions", C.c_int), ("vol_names", C.POINTER(C.c_char_p)),
                ("surf_names", C.POINTER(C.c_char_p))]


def _take_mesh(ptr):
    d = C.cast(ptr, C.POINTER(fg_mesh_data)).contents

    def arr(p, n, dt):
        return np.ctypeslib.as_array(p, shape=(n,)).astype(dt).copy() if n else np.zeros(0, dt)
    out = {
        "xyz": arr(d.xyz, 3 * d.n_nodes, np.float64).reshape(-1, 3),
        "tets": arr(d.tet4, 4 * d.n_tets, np.int32).reshape(-1, 4),
        "tet_reg": arr(d.tet_region, d.n_tets, np.int32),
        "tris": arr(d.tri3, 3 * d.n_tris, np.int32).reshape(-1, 3),
        "tri_reg": arr(d.tri_region, d.n_tris, np.int32),
        "dMs": arr(d.tri_dMs, d.n_tris, np.float64),
        "node_index": arr(d.node_index, d.n_nodes, np.int64),
        "vol_names": [d.vol_names[k].decode() for k in range(d.n_vol_regions)],
        "surf_names": [d.surf_names[k].decode() for k in range(d.n_surf_regions)],
    }
    fg_lib().fg_mesh_free(ptr)
    return out


class fg_run_report(C.Structure):
    _fields_ = [("status", C.c_int), ("steps", C.c_longlong), ("t", C.c_double), ("wall_s", C.c_double),
                ("E", C.c_double * 4)]


def run(settings_path, seed=0, verbose=False):
    """A whole simulation from a settings file (the reference's `feellgood --seed N file`)."""
    L = fg_lib()
    rep = fg_run_report()
    s = L.fg_run(str(settings_path).encode(), seed, int(verbose), C.byref(rep))
    if s != FG_OK:
        raise FgError(s, L.fg_run_last_error().decode())
    return {"steps": rep.steps, "t": rep.t, "wall_s": rep.wall_s, "E": list(rep.E)}


def settings_dump(settings_path):
    """The parsed settings (reader check, no GPU work)."""
    import json
    L = fg_lib()
    buf = C.create_string_buffer(1 << 16)
    s = L.fg_settings_dump(str(settings_path).encode(), buf, len(buf))
    if s != FG_OK:
        raise FgError(s, L.fg_run_last_error().decode())
    return json.loads(buf.value.decode())


def rng_seed(seed):
    fg_lib().fg_rng_seed(seed)


class fg_checkpoint_shape(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_mag_tets", C.c_int), ("precision", C.c_int), ("solver_lpr", C.c_int),
                ("solver_blocks", C.c_int), ("fmm_depth", C.c_int), ("solver_threads", C.c_int)]


class fg_checkpoint_meta(C.Structure):
    _fields_ = [("t0", C.c_double), ("t", C.c_double), ("dt", C.c_double), ("dt_soft_max", C.c_double),
                ("steps", C.c_longlong), ("output_index", C.c_longlong), ("rng_seed", C.c_uint),
                ("rng_draws", C.c_longlong), ("E", C.c_double * 4)]


def checkpoint_peek(path):
    """fg_checkpoint_peek: header of a checkpoint file (shape and run metadata) as a dict."""
    sh, me = fg_checkpoint_shape(), fg_checkpoint_meta()
    s = fg_lib().fg_checkpoint_peek(str(path).encode(), C.byref(sh), C.byref(me))
    if s != FG_OK:
        raise FgError(s, f"cannot read checkpoint {path}")
    out = {k: getattr(sh, k) for k, _ in fg_checkpoint_shape._fields_}
    out.update({k: getattr(me, k) for k, _ in fg_checkpoint_meta._fields_ if k != "E"})
    out["E"] = list(me.E)
    return out


def pinned_empty(shape, dtype=np.float64):
    """numpy array in page-locked host memory (fg_host_alloc), freed with the array: state
    buffers for Context.set_state / get_state(out=...) that cross the host link at full speed."""
    dt = np.dtype(dtype)
    n = int(np.prod(shape)) * dt.itemsize
    L = fg_lib()
    p = C.c_void_p()
    st = L.fg_host_alloc(n, C.byref(p))
    if st != FG_OK:
        raise FgError(st, "fg_host_alloc: " + L.fg_strerror(st).decode())
    buf = (C.c_char * max(n, 1)).from_address(p.value)
    weakref.finalize(buf, L.fg_host_free, C.c_void_p(p.value))
    return np.frombuffer(buf, dtype=dt, count=int(np.prod(shape))).reshape(shape)


def rng_angle():
    """Next basis angle of the reference's stream (M_2_PI * U(0,1) from mt19937(rand()))."""
    return fg_lib().fg_rng_angle()


def load_msh(path, vol_regions, Ms, surf_regions=(), length_unit=1e-9):
    """Read a gmsh file and run the reference's mesh set-up (C++ host code of the library).

    vol_regions: names of the settings' volume regions; Ms: their saturation magnetisation."""
    L = fg_lib()
    vn = (C.c_char_p * max(1, len(vol_regions)))(*[n.encode() for n in vol_regions])
    sn = (C.c_char_p * max(1, len(surf_regions)))(*[n.encode() for n in surf_regions])
    ms = np.ascontiguousarray(Ms, dtype=np.float64)
    out = C.c_void_p()
    s = L.fg_mesh_load_msh(str(path).encode(), length_unit, len(vol_regions), vn, _dptr(ms), len(surf_regions), sn,
                           C.byref(out))
    if s != FG_OK:
        raise FgError(s, L.fg_mesh_last_error().decode())
    return _take_mesh(out)


def cuboid(nx, ny, nz, lx, ly, lz, length_unit=1e-9, Ms=8e5):
    """Structured cuboid (6 tetrahedra per cell) set up like a mesh read from a file."""
    L = fg_lib()
    out = C.c_void_p()
    s = L.fg_mesh_cuboid(nx, ny, nz, lx, ly, lz, length_unit, Ms, C.byref(out))
    if s != FG_OK:
        raise FgError(s, L.fg_mesh_last_error().decode())
    return _take_mesh(out)


def fg_lib():
    """Load libfggpu.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise ImportError(f"{path} is missing: build it with `python -m feellgood_gb300.build` "
                              "(there is no CPU fallback)")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _dptr(a):
    return a.ctypes.data_as(_dp)


def make_region(Ae=1e-11, Ms=795774.7, K=0.0, uk=(0, 0, 1), K3=0.0, ex=(1, 0, 0), ey=(0, 1, 0), ez=(0, 0, 1),
                alpha=0.5, sigma=0.0, dens_state=0.0, P=0.0, lsd=0.0, lsf=0.0, **_):
    r = fg_region()
    r.Ae, r.Ms, r.K, r.K3, r.alpha = Ae, Ms, K, K3, alpha
    r.sigma, r.dens_state, r.P, r.lsd, r.lsf = sigma, dens_state, P, lsd, lsf
    for name, v in (("uk", uk), ("ex", ex), ("ey", ey), ("ez", ez)):
        v = np.asarray(v, float)
        getattr(r, name)[:] = list(v / np.linalg.norm(v))
    return r


def make_tri_region(Ks=0.0, uk=(0, 0, 1), suppress_charges=False, jn=None, V=None, uP=(0, 0, 1), s=None, **_):
    """jn, V, s: None where not given (NaN in the C struct)."""
    r = fg_tri_region()
    r.Ks = Ks
    v = np.asarray(uk, float)
    r.uk[:] = list(v / np.linalg.norm(v))
    r.suppress_charges = int(bool(suppress_charges))
    r.jn = float("nan") if jn is None else jn
    r.V = float("nan") if V is None else V
    p = np.asarray(uP, float)
    r.uP[:] = list(p / np.linalg.norm(p))
    r.s[:] = [float("nan")] * 3 if s is None else list(np.asarray(s, float))
    return r


class Context:
    """One mesh (or batch) resident on the GPU; see include/fggpu.h."""

    def __init__(self, mesh, regions, tri_regions=None, **opts):
        """mesh: one mesh dict, or a list of mesh dicts for a batch of independent samples
        (fg_batch_create; the samples' nodes are concatenated in list order)."""
        L = fg_lib()
        self.L = L
        self._keep = []
        meshes = list(mesh) if isinstance(mesh, (list, tuple)) else [mesh]
        self.batch = isinstance(mesh, (list, tuple))
        cm = []
        nfreg = 0
        for one in meshes:
            xyz = np.ascontiguousarray(one["xyz"], dtype=np.float64)
            tets = np.ascontiguousarray(one["tets"], dtype=np.int32)
            treg = np.ascontiguousarray(one["tet_reg"], dtype=np.int32)
            tris = np.ascontiguousarray(one.get("tris", np.zeros((0, 3))), dtype=np.int32).reshape(-1, 3)
            freg = np.ascontiguousarray(one.get("tri_reg", np.zeros(0)), dtype=np.int32)
            dms = np.ascontiguousarray(one.get("dMs", np.zeros(0)), dtype=np.float64)
            self._keep += [xyz, tets, treg, tris, freg, dms]
            cm.append(fg_mesh(len(xyz), len(tets), len(tris), _ptr(xyz), _ptr(tets), _ptr(treg), _ptr(tris),
                              _ptr(freg), _ptr(dms)))
            if len(freg):
                nfreg = max(nfreg, int(freg.max()) + 1)
        regs = [r if isinstance(r, fg_region) else make_region(**r) for r in regions]
        if tri_regions is None:
            tri_regions = [make_tri_region() for _ in range(max(nfreg, 1))]
        tregs = [r if isinstance(r, fg_tri_region) else make_tri_region(**r) for r in tri_regions]
        R = (fg_region * len(regs))(*regs)
        T = (fg_tri_region * len(tregs))(*tregs)
        o = fg_opts()
        L.fg_opts_default(C.byref(o))
        for k, v in opts.items():
            if not hasattr(o, k):
                raise TypeError(f"unknown option {k}")
            setattr(o, k, v)
        self.opts = o
        h = C.c_void_p()
        if self.batch:
            M = (fg_mesh * len(cm))(*cm)
            s = L.fg_batch_create(M, len(cm), R, len(regs), T, len(tregs), C.byref(o), C.byref(h))
        else:
            s = L.fg_create(C.byref(cm[0]), R, len(regs), T, len(tregs), C.byref(o), C.byref(h))
        if s != FG_OK:
            raise FgError(s, L.fg_last_error(None).decode())
        self.h = h
        self.nn = sum(m.n_nodes for m in cm)
        self.n_samples = len(cm)
        off = np.zeros(self.n_samples + 1, dtype=np.int32)
        ns = C.c_int()
        self._check(L.fg_batch_info(h, C.byref(ns), _ptr(off)))
        self.node_offsets = off

    def close(self):
        if getattr(self, "h", None):
            self.L.fg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, s):
        if s not in (FG_OK,):
            raise FgError(s, self.L.fg_last_error(self.h).decode())

    def set_state(self, u, v=None, phi=None, phiv=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (u, v, phi, phiv)]
        self._check(self.L.fg_set_state(self.h, *[_ptr(a) for a in arrs]))

    def get_state(self, which=1, out=None):
        """fg_get_state; `out` (a dict of C-contiguous float64 arrays u, v, phi, phiv of the
        node count's shapes, e.g. from pinned_empty) is filled in place and returned."""
        if out is None:
            out = {"u": np.zeros((self.nn, 3)), "v": np.zeros((self.nn, 3)), "phi": np.zeros(self.nn),
                   "phiv": np.zeros(self.nn)}
        else:
            for k, shape in (("u", (self.nn, 3)), ("v", (self.nn, 3)), ("phi", (self.nn,)), ("phiv", (self.nn,))):
                a = out[k]
                if a.dtype != np.float64 or a.shape != shape or not a.flags["C_CONTIGUOUS"]:
                    raise ValueError(f"get_state: out[{k!r}] must be a C-contiguous float64 array of shape {shape}")
        self._check(self.L.fg_get_state(self.h, which, _ptr(out["u"]), _ptr(out["v"]), _ptr(out["phi"]),
                                        _ptr(out["phiv"])))
        return out

    @staticmethod
    def _sample_steps(dt, prefactor, Hext, angle, shape):
        """(..., 6) float64 rows laid out as fg_sample_step: dt, prefactor, Hext[3], angle."""
        a = np.empty(shape + (6,), dtype=np.float64)
        a[..., 0] = dt
        a[..., 1] = prefactor
        a[..., 2:5] = Hext
        a[..., 5] = angle
        return np.ascontiguousarray(a)

    def batch_step(self, dt, prefactor, Hext, angle):
        """fg_batch_step; every argument broadcasts to the samples (Hext: (n_samples, 3))."""
        ns = self.n_samples
        a = self._sample_steps(dt, prefactor, Hext, angle, (ns,))
        reps = (fg_step_report * ns)()
        s = self.L.fg_batch_step(self.h, _ptr(a), reps)
        if s == FG_ETIMEDOUT or s > FG_ETIMEDOUT:
            self._check(s)
        return s, [{k: getattr(r, k) for k, _ in fg_step_report._fields_} for r in reps]

    def batch_compute_all(self, Hext=None, energies=True):
        ns = self.n_samples
        H = None if Hext is None else np.ascontiguousarray(np.broadcast_to(Hext, (ns, 3)), dtype=np.float64)
        E = np.zeros((ns, 4)) if energies else None
        self._check(self.L.fg_batch_compute_all(self.h, _ptr(H), _ptr(E)))
        return E

    def batch_run(self, dt, prefactor, Hext, angles):
        """fg_batch_run over angles.shape[0] steps; angles: (n_steps, n_samples); dt, prefactor
        and Hext broadcast to (n_steps, n_samples[, 3])."""
        angles = np.asarray(angles, dtype=np.float64)
        nsteps = angles.shape[0]
        a = self._sample_steps(dt, prefactor, Hext, angles, angles.shape)
        reps = (fg_batch_report * self.n_samples)()
        s = self.L.fg_batch_run(self.h, nsteps, _ptr(a), reps)
        if s == FG_ETIMEDOUT or s > FG_ETIMEDOUT:
            self._check(s)
        return s, [{k: getattr(r, k) for k, _ in fg_batch_report._fields_} for r in reps]

    def debug_wait_timeout(self, which):
        """fg_debug_wait_timeout: the status a deliberately unended bounded device wait reports."""
        return self.L.fg_debug_wait_timeout(self.h, which)

    def solver_lanes_per_row(self):
        v = C.c_int()
        self._check(self.L.fg_solver_info(self.h, C.byref(v), None))
        return v.value

    def spin_info(self):
        """fg_spin_info: last spin solve (status, iterations), the potential V and its CG iterations."""
        st, it, vit, ms = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        V = np.zeros(self.nn)
        self._check(self.L.fg_spin_info(self.h, C.byref(st), C.byref(it), _ptr(V), C.byref(vit), C.byref(ms)))
        return {"status": st.value, "iters": it.value, "V": V, "V_iters": vit.value, "ms": ms.value}

    def set_drift(self, direction, vdrift):
        """fg_set_drift: recentering drift of the element integrals along direction 0/1/2
        ('X'/'Y'/'Z', -1 or None for none) at vdrift m/s."""
        d = {"X": 0, "Y": 1, "Z": 2, None: -1}.get(direction, direction)
        self._check(self.L.fg_set_drift(self.h, int(d), float(vdrift)))

    def recenter(self, direction, threshold):
        """fg_recenter: direction 0/1/2 (x/y/z) or 'X'/'Y'/'Z'; returns True when it translated."""
        d = {"X": 0, "Y": 1, "Z": 2}.get(direction, direction)
        sh = C.c_int()
        self._check(self.L.fg_recenter(self.h, int(d), float(threshold), C.byref(sh)))
        return bool(sh.value)

    def get_spin(self):
        """fg_get_spin: the spin accumulation s, (n_nodes, 3)."""
        s = np.zeros((self.nn, 3))
        self._check(self.L.fg_get_spin(self.h, _ptr(s)))
        return s

    def gauss_points(self):
        """fg_gauss_points: coordinates of the magnetic tets' Gauss points, (n_mag_tets * npi, 3)."""
        n = C.c_int()
        self._check(self.L.fg_gauss_points(self.h, C.byref(n), None))
        pts = np.zeros((n.value, 3))
        self._check(self.L.fg_gauss_points(self.h, C.byref(n), _ptr(pts)))
        return pts

    def set_space_field(self, field):
        """fg_set_space_field: f at the Gauss points (same rows as gauss_points()), or None."""
        if field is None:
            self._check(self.L.fg_set_space_field(self.h, None))
            return
        f = np.ascontiguousarray(field, dtype=np.float64)
        self._check(self.L.fg_set_space_field(self.h, _ptr(f)))

    def set_field_amplitude(self, a):
        """fg_set_field_amplitude: A(t) of the space field for the next steps."""
        self._check(self.L.fg_set_field_amplitude(self.h, float(a)))

    def solver_blocks(self):
        v = C.c_int()
        self._check(self.L.fg_solver_info(self.h, None, C.byref(v)))
        return v.value

    def batch_run_info(self):
        g = C.c_int()
        ms = C.c_double()
        self._check(self.L.fg_batch_run_info(self.h, C.byref(g), C.byref(ms)))
        return bool(g.value), ms.value

    def step(self, dt, prefactor, Hext, angle):
        """Returns the report dict; report['status'] is FG_OK or a solver status."""
        rep = fg_step_report()
        H = np.ascontiguousarray(Hext, dtype=np.float64)
        s = self.L.fg_step(self.h, dt, prefactor, _dptr(H), angle, C.byref(rep))
        if s not in (FG_OK, FG_SOLVER_ITER_OVERFLOW, FG_SOLVER_CANNOT_CONVERGE):
            self._check(s)
        return {k: getattr(rep, k) for k, _ in fg_step_report._fields_}

    def compute_all(self, Hext):
        H = np.ascontiguousarray(Hext, dtype=np.float64)
        E = np.zeros(4)
        self._check(self.L.fg_compute_all(self.h, _dptr(H), _dptr(E)))
        return E

    def demag(self, which=0):
        out = np.zeros(self.nn)
        self._check(self.L.fg_demag(self.h, which, _dptr(out)))
        return out

    def energy(self, Hext):
        H = np.ascontiguousarray(Hext, dtype=np.float64)
        E = np.zeros(4)
        self._check(self.L.fg_energy(self.h, _dptr(H), _dptr(E)))
        return E

    def energy_noalloc(self, Hext):
        """fg_energy through the entry point that allocates no device memory."""
        H = np.ascontiguousarray(Hext, dtype=np.float64)
        E = np.zeros(4)
        self._check(self.L.fg_energy_noalloc(self.h, _dptr(H), _dptr(E)))
        return E

    def average(self, which=0):
        a = np.zeros(3)
        self._check(self.L.fg_average(self.h, which, _dptr(a)))
        return a

    def debug_system(self):
        rhs, ep, eq = np.zeros(2 * self.nn), np.zeros((self.nn, 3)), np.zeros((self.nn, 3))
        self._check(self.L.fg_debug_system(self.h, _ptr(rhs), _ptr(ep), _ptr(eq)))
        return rhs, ep, eq

    def debug_apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        self._check(self.L.fg_debug_apply(self.h, _dptr(x), _dptr(y)))
        return y

    def counters(self):
        out = (C.c_longlong * 4)()
        self._check(self.L.fg_counters(self.h, out))
        return list(out)

    def mlp_info(self):
        """(training steps done, last minibatch loss) of the learned guess."""
        n = C.c_longlong()
        loss = np.zeros(1)
        self._check(self.L.fg_mlp_info(self.h, C.byref(n), _dptr(loss)))
        return n.value, float(loss[0])

    def mlp_debug_grad(self, feat, target):
        """(weights, summed gradient, loss) of the GPU training kernels for given samples."""
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        target = np.ascontiguousarray(target, dtype=np.float32)
        n = self.L.fg_mlp_nparam()
        w, g, loss = np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(1, np.float32)
        self._check(self.L.fg_mlp_debug_grad(self.h, len(feat), _ptr(feat), _ptr(target), _ptr(w), _ptr(g),
                                             _ptr(loss)))
        return w, g, float(loss[0])

    def mlp_debug_infer(self, feat):
        """The GPU inference kernel's network outputs [n, 3] for given feature rows [n, 12]."""
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        out = np.zeros((len(feat), 3), np.float32)
        self._check(self.L.fg_mlp_debug_infer(self.h, len(feat), _ptr(feat), _ptr(out)))
        return out

    def fmm_timings(self):
        """Device ms of the FMM stages of the last evaluation (needs profile=1):
        P2M, M2M, M2L, L2L, L2P+P2P."""
        ms = np.zeros(5)
        self._check(self.L.fg_fmm_timings(self.h, _dptr(ms)))
        return ms

    def fmm_tree_info(self):
        """FMM set-up: dict of the whole set-up's wall ms, the octree builds' wall ms, the
        device ms of the Morton-key radix sort, the depth and the number of trees."""
        out = np.zeros(5)
        self._check(self.L.fg_fmm_tree_info(self.h, _dptr(out)))
        return dict(setup_ms=float(out[0]), tree_ms=float(out[1]), sort_device_ms=float(out[2]),
                    depth=int(out[3]), trees=int(out[4]))

    def timings(self):
        """[elements, solve, demag, energy + evolution, whole step] device ms of the last step."""
        ms = np.zeros(5)
        self._check(self.L.fg_timings(self.h, _dptr(ms)))
        return ms


def measure_peaks():
    """fg_measure_peaks: per-SM, per-clock throughputs of the FP32 FMA (scalar and f32x2), the
    SFU reciprocal square root and tcgen05 kind::tf32 (N = 128 and 256), the SM clock and
    the number of SMs."""
    out = np.zeros(7)
    s = fg_lib().fg_measure_peaks(_dptr(out))
    if s != FG_OK:
        raise FgError(s, "fg_measure_peaks")
    keys = ["ffma_per_clk_sm", "ffma2_per_clk_sm", "rsqrt_per_clk_sm", "tf32_n128_flops_per_clk_sm",
            "tf32_n256_flops_per_clk_sm", "sm_mhz", "n_sm"]
    return dict(zip(keys, (float(x) for x in out)))


def debug_translate_tc(ops, tab, x, terms=7):
    """fg_debug_translate_tc: tensor-core translation of x[n_in, 100] by ops[ncode, 100, 100]
    through tab[n_out, ncode] (-1 = none); returns out[n_out, 100] (float32)."""
    L = fg_lib()
    ops = np.ascontiguousarray(ops, dtype=np.float32)
    tab = np.ascontiguousarray(tab, dtype=np.int32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.zeros((tab.shape[0], 100), dtype=np.float32)
    s = L.fg_debug_translate_tc(x.shape[0], tab.shape[0], tab.shape[1], _ptr(ops), _ptr(tab), _ptr(x), _ptr(out), terms)
    if s != FG_OK:
        raise FgError(s, "fg_debug_translate_tc")
    return out
