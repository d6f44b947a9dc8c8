"""CPU oracle of the RK4 residual path (TEST INFRASTRUCTURE ONLY).

ctypes bridge to oracle/_build/libminiaero_oracle.so, a plain-C restatement of
the reference's Kokkos functors (see miniaero_oracle.c). Used by tests/, by
__graft_entry__.smoke() as the checker, and by bench.py's CPU baseline; the
product never imports it.
"""
import ctypes
import os

import numpy as np

_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_DIR, "_build", "libminiaero_oracle.so")
# The same source at -O3 with the compiler's default multiply-add contraction
# (the reference Makefile's flags): CPU timing only, never a parity check.
TIMING_LIB_PATH = os.path.join(_DIR, "_build", "libminiaero_oracle_timing.so")

P_i32 = ctypes.POINTER(ctypes.c_int)
P_f64 = ctypes.POINTER(ctypes.c_double)


class oracle_faces(ctypes.Structure):
    _fields_ = [("nfaces", ctypes.c_int), ("type", ctypes.c_int), ("conn", P_i32), ("coords", P_f64),
                ("normal", P_f64), ("tangent", P_f64), ("binormal", P_f64), ("permutation", P_i32),
                ("flux_index", P_i32)]


class oracle_mesh(ctypes.Structure):
    _fields_ = [("ncells", ctypes.c_int), ("cell_coords", P_f64), ("cell_volumes", P_f64),
                ("internal", oracle_faces), ("nbc", ctypes.c_int), ("bc", ctypes.POINTER(oracle_faces))]


class oracle_options(ctypes.Structure):
    _fields_ = [("second_order", ctypes.c_int), ("viscous", ctypes.c_int), ("limiter", ctypes.c_int),
                ("viscosity_model", ctypes.c_int), ("mu", ctypes.c_double), ("prandtl", ctypes.c_double),
                ("dt", ctypes.c_double), ("nsteps", ctypes.c_int), ("inflow_state", ctypes.c_double * 5),
                ("cell_flux", ctypes.c_int)]


_libs = {}


def lib(timing=False):
    """The parity build (default) or, with timing=True, the -O3 timing build."""
    path = TIMING_LIB_PATH if timing else LIB_PATH
    if path not in _libs:
        if not os.path.exists(path):
            raise ImportError("oracle library not built: %s" % path)
        L = ctypes.CDLL(path)
        L.oracle_solve.restype = ctypes.c_int
        L.oracle_solve.argtypes = [ctypes.POINTER(oracle_mesh), ctypes.POINTER(oracle_options), P_f64, P_f64,
                                   ctypes.c_int]
        L.oracle_roe_flux.argtypes = [P_f64] * 6
        L.oracle_viscous_flux.argtypes = [P_f64, P_f64, P_f64, ctypes.c_int, ctypes.c_double, ctypes.c_double, P_f64]
        L.oracle_venkat.restype = ctypes.c_double
        L.oracle_venkat.argtypes = [ctypes.c_double] * 4
        L.oracle_vanalbada.restype = ctypes.c_double
        L.oracle_vanalbada.argtypes = [ctypes.c_double] * 3
        L.oracle_primitives.argtypes = [P_f64, P_f64]
        L.oracle_create.restype = ctypes.c_void_p
        L.oracle_create.argtypes = [ctypes.POINTER(oracle_mesh), ctypes.POINTER(oracle_options), P_f64, ctypes.c_int]
        L.oracle_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.oracle_get_state.argtypes = [ctypes.c_void_p, P_f64, P_f64]
        L.oracle_free.argtypes = [ctypes.c_void_p]
        for name in ("oracle_field_gradients", "oracle_field_limiter", "oracle_field_bc_flux"):
            getattr(L, name).argtypes = [ctypes.POINTER(oracle_mesh), ctypes.POINTER(oracle_options), P_f64, P_f64]
            getattr(L, name).restype = ctypes.c_int
        _libs[path] = L
    return _libs[path]


def _p(a, t):
    return a.ctypes.data_as(t)


class OracleMesh:
    """oracle_mesh over the arrays of a miniaero_gb300.MeshData (kept alive)."""

    def __init__(self, md):
        self.md = md

        def faces(fs):
            f = oracle_faces()
            f.nfaces = fs.nfaces
            f.type = fs.type
            f.conn = _p(fs.conn, P_i32)
            f.coords = _p(fs.coords, P_f64)
            f.normal = _p(fs.normal, P_f64)
            f.tangent = _p(fs.tangent, P_f64)
            f.binormal = _p(fs.binormal, P_f64)
            f.permutation = _p(fs.permutation, P_i32)
            fi = getattr(fs, "flux_index", None)
            f.flux_index = _p(fi, P_i32) if fi is not None else ctypes.cast(None, P_i32)
            return f

        self.bc = (oracle_faces * max(1, len(md.bc)))()
        for i, b in enumerate(md.bc):
            self.bc[i] = faces(b)
        m = oracle_mesh()
        m.ncells = md.ncells
        m.cell_coords = _p(md.cell_coords, P_f64)
        m.cell_volumes = _p(md.cell_volumes, P_f64)
        m.internal = faces(md.internal)
        m.nbc = len(md.bc)
        m.bc = ctypes.cast(self.bc, ctypes.POINTER(oracle_faces))
        self.c = m


def _c_options(options, nsteps=None, dt=None):
    o = oracle_options()
    o.second_order = int(options.second_order_space)
    o.viscous = int(options.viscous)
    o.limiter = int(options.limiter)
    o.viscosity_model = int(options.viscosity_model)
    o.mu = float(options.mu)
    o.prandtl = float(options.prandtl)
    o.dt = float(options.dt if dt is None else dt)
    o.nsteps = int(options.ntimesteps if nsteps is None else nsteps)
    for k in range(5):
        o.inflow_state[k] = options.inflow_state[k]
    o.cell_flux = int(options.gather == 1)  # MA_GATHER_CELL_FLUX
    return o


class Stepper:
    """Persistent oracle state advanced step by step (CPU baseline timing)."""

    def __init__(self, md, options, U0, dt=None, nthreads=1, timing=False):
        self.mesh = OracleMesh(md)
        self.opts = _c_options(options, 0, dt)
        self.ncells = md.ncells
        self.L = lib(timing)
        U0 = np.ascontiguousarray(U0, dtype=np.float64)
        self.h = self.L.oracle_create(ctypes.byref(self.mesh.c), ctypes.byref(self.opts), _p(U0, P_f64),
                                      int(nthreads))
        if not self.h:
            raise RuntimeError("oracle_create failed")

    def step(self, n=1):
        self.L.oracle_step(self.h, int(n))

    def state(self):
        U = np.empty((self.ncells, 5))
        self.L.oracle_get_state(self.h, _p(U, P_f64), ctypes.cast(None, P_f64))
        return U

    def close(self):
        if self.h:
            self.L.oracle_free(self.h)
            self.h = None

    def __del__(self):
        self.close()


def solve(md, options, U0, nsteps=None, dt=None, nthreads=1, return_residual=False):
    """Advances U0 ((ncells, 5) conserved) with the reference semantics.

    options: a miniaero_gb300.Options (second_order_space, viscous, limiter,
    viscosity_model, mu, prandtl, dt, ntimesteps, inflow_state).
    """
    om = OracleMesh(md)
    o = _c_options(options, nsteps, dt)
    U = np.ascontiguousarray(U0, dtype=np.float64).copy()
    res = np.zeros_like(U) if return_residual else None
    rc = lib().oracle_solve(ctypes.byref(om.c), ctypes.byref(o), _p(U, P_f64),
                            _p(res, P_f64) if res is not None else ctypes.cast(None, P_f64), int(nthreads))
    if rc != 0:
        raise RuntimeError("oracle_solve failed (%d)" % rc)
    return (U, res) if return_residual else U


def roe_flux(pl, pr, n, t, b):
    L = lib()
    pl = np.ascontiguousarray(pl, np.float64).reshape(-1, 5)
    N = pl.shape[0]
    pr = np.ascontiguousarray(pr, np.float64).reshape(N, 5)
    n = np.ascontiguousarray(n, np.float64).reshape(N, 3)
    t = np.ascontiguousarray(t, np.float64).reshape(N, 3)
    b = np.ascontiguousarray(b, np.float64).reshape(N, 3)
    out = np.empty((N, 5))
    for i in range(N):
        L.oracle_roe_flux(_p(pl[i], P_f64), _p(pr[i], P_f64), _p(n[i], P_f64), _p(t[i], P_f64), _p(b[i], P_f64),
                          _p(out[i], P_f64))
    return out


def viscous_flux(grad, prim, area, model=0, mu=0.0, prandtl=0.72):
    L = lib()
    grad = np.ascontiguousarray(grad, np.float64).reshape(-1, 5, 3)
    N = grad.shape[0]
    prim = np.ascontiguousarray(prim, np.float64).reshape(N, 5)
    area = np.ascontiguousarray(area, np.float64).reshape(N, 3)
    out = np.empty((N, 5))
    for i in range(N):
        L.oracle_viscous_flux(_p(grad[i], P_f64), _p(prim[i], P_f64), _p(area[i], P_f64), model, mu, prandtl,
                              _p(out[i], P_f64))
    return out


def venkat(dumax, dumin, du, d2):
    L = lib()
    return np.array([L.oracle_venkat(a, b, c, d) for a, b, c, d in zip(dumax, dumin, du, d2)])


def vanalbada(dumax, dumin, du):
    L = lib()
    return np.array([L.oracle_vanalbada(a, b, c) for a, b, c in zip(dumax, dumin, du)])


def primitives(U):
    L = lib()
    U = np.ascontiguousarray(U, np.float64).reshape(-1, 5)
    out = np.empty_like(U)
    for i in range(U.shape[0]):
        L.oracle_primitives(_p(U[i], P_f64), _p(out[i], P_f64))
    return out


def _field(fn, md, options, U, width):
    om = OracleMesh(md)
    o = _c_options(options)
    U = np.ascontiguousarray(U, dtype=np.float64).reshape(md.ncells, 5)
    out = np.empty((md.ncells, width))
    if getattr(lib(), fn)(ctypes.byref(om.c), ctypes.byref(o), _p(U, P_f64), _p(out, P_f64)) != 0:
        raise RuntimeError(fn + " failed")
    return out


def field_gradients(md, options, U):
    """GreenGauss::compute_gradients on state U: (ncells, 5, 3)."""
    return _field("oracle_field_gradients", md, options, U, 15).reshape(md.ncells, 5, 3)


def field_limiter(md, options, U):
    """compute_min_max + compute_limiter (options.limiter) on U: (ncells, 5)."""
    return _field("oracle_field_limiter", md, options, U, 5)


def field_bc_flux(md, options, U):
    """The BC functors in Solve's order on U: boundary part of cell_flux, (ncells, 5)."""
    return _field("oracle_field_bc_flux", md, options, U, 5)
