"""miniaero_gb300: GB300-native miniAero explicit RK4 residual path.

Python host-side mirror of the reference's interface for this path, over the
C ABI of libminiaero_gpu.so (include/miniaero_gpu.h):

  Options                   kokkos/Options.h:47-102 (miniaero.inp + extensions)
  Parallel3DMesh            kokkos/Parallel3DMesh.h:56-520 (single rank)
  MeshData                  kokkos/MeshData.h:42-58 (host copy)
  TimeSolverExplicitRK4     kokkos/TimeSolverExplicitRK4.h:160-539
  roe_flux, viscous_flux, venkat_limit, vanalbada_limit, compute_primitives
                            operator-level entry points (Roe_Flux.h:50,
                            Viscous_Flux.h:66, VenkatLimiter.h:45,
                            VanAlbadaLimiter.h:45, GasModel.h:69)

All numerical work runs on the GPU through the library; a missing library or
GPU raises MiniaeroError instead of falling back to the CPU.
"""
import ctypes
import os

import numpy as np

from . import _lib
from ._lib import (MA_BC_EXTRAPOLATE, MA_BC_INFLOW, MA_BC_NOSLIP, MA_BC_TANGENT, MA_IC_CONSTANT,
                   MA_IC_REFERENCE, MA_IC_SOD, MA_LAYOUT_AOS, MA_LAYOUT_SOA, MA_LIMITER_VANALBADA,
                   MA_LIMITER_VENKAT, MA_PREC_FP64, MA_PREC_FP64_FMA, MA_PREC_MIXED, MA_VISC_CONSTANT, MA_VISC_SUTHERLAND,
                   MiniaeroError, check, f64p, i32p, lib)

__all__ = [
    "Options", "Parallel3DMesh", "MeshData", "FaceSet", "DeviceMesh", "TimeSolverExplicitRK4",
    "initial_state", "mesh_hash", "checkpoint_write", "checkpoint_read", "run_options_read",
    "roe_flux", "viscous_flux", "venkat_limit", "vanalbada_limit", "compute_primitives",
    "device_count", "MiniaeroError", "BC_NAMES",
    "MA_BC_EXTRAPOLATE", "MA_BC_TANGENT", "MA_BC_INFLOW", "MA_BC_NOSLIP",
    "MA_LIMITER_VENKAT", "MA_LIMITER_VANALBADA", "MA_VISC_SUTHERLAND", "MA_VISC_CONSTANT",
    "MA_PREC_FP64", "MA_PREC_MIXED", "MA_PREC_FP64_FMA", "MA_IC_REFERENCE", "MA_IC_SOD", "MA_IC_CONSTANT",
    "MA_LAYOUT_AOS", "MA_LAYOUT_SOA",
]

BC_NAMES = {MA_BC_EXTRAPOLATE: "Extrapolate", MA_BC_TANGENT: "Tangent", MA_BC_INFLOW: "Inflow",
            MA_BC_NOSLIP: "NoSlip"}


def device_count():
    return int(lib().ma_device_count())


class Options:
    """Run options: the nine miniaero.inp values plus extension keys."""

    def __init__(self, **kw):
        object.__setattr__(self, "_o", _lib.ma_options())
        lib().ma_options_default(ctypes.byref(self._o))
        for k, v in kw.items():
            setattr(self, k, v)

    @classmethod
    def read_options_file(cls, path="miniaero.inp"):
        """Options::read_options_file; raises on a missing or malformed file."""
        o = cls()
        check(lib().ma_options_read(str(path).encode(), ctypes.byref(o._o)))
        return o

    def __getattr__(self, name):
        o = object.__getattribute__(self, "_o")
        v = getattr(o, name)
        if isinstance(v, ctypes.Array):
            return list(v)
        return v

    def __setattr__(self, name, value):
        o = self._o
        cur = getattr(o, name)
        if isinstance(cur, ctypes.Array):
            if len(value) != len(cur):
                raise ValueError("%s needs %d values" % (name, len(cur)))
            for i, x in enumerate(value):
                cur[i] = x
        else:
            setattr(o, name, value)

    def copy(self):
        c = Options()
        ctypes.memmove(ctypes.byref(c._o), ctypes.byref(self._o), ctypes.sizeof(self._o))
        return c

    @property
    def c(self):
        return self._o

    def __repr__(self):
        fields = ", ".join("%s=%r" % (n, getattr(self, n)) for n, _ in _lib.ma_options._fields_)
        return "Options(%s)" % fields


class FaceSet:
    """Host copy of one Faces<Device> list (kokkos/Faces.h:42-71)."""

    def __init__(self, fs, name):
        n = fs.nfaces
        self.name = name
        self.type = fs.type
        self.nfaces = n

        def arr(p, shape, dtype):
            if n == 0:
                return np.zeros(shape, dtype)
            return np.ctypeslib.as_array(p, shape=shape).astype(dtype, copy=True)

        self.conn = arr(fs.conn, (n, 2), np.int32)
        self.coords = arr(fs.coords, (n, 3), np.float64)
        self.normal = arr(fs.normal, (n, 3), np.float64)
        self.tangent = arr(fs.tangent, (n, 3), np.float64)
        self.binormal = arr(fs.binormal, (n, 3), np.float64)
        self.permutation = arr(fs.permutation, (n,), np.int32)
        # Element-local face slots of (left, right) (Faces.h:109-110), when given.
        self.flux_index = arr(fs.flux_index, (n, 2), np.int32) if (n == 0 or fs.flux_index) else None

    def to_c(self):
        fs = _lib.ma_face_set()
        fs.nfaces = self.nfaces
        fs.type = self.type
        fs.conn = i32p(self.conn)
        fi = getattr(self, "flux_index", None)
        fs.flux_index = i32p(fi) if fi is not None else ctypes.cast(None, _lib.P_i32)
        fs.coords = f64p(self.coords)
        fs.normal = f64p(self.normal)
        fs.tangent = f64p(self.tangent)
        fs.binormal = f64p(self.binormal)
        fs.permutation = i32p(self.permutation)
        return fs


class MeshData:
    """Mesh as the reference's MeshData holds it, in host numpy arrays."""

    def __init__(self, ncells, cell_coords, cell_volumes, internal, bc, handle=None):
        self.ncells = ncells
        self.cell_coords = cell_coords
        self.cell_volumes = cell_volumes
        self.internal = internal
        self.bc = bc
        self._handle = handle

    def view(self):
        """ma_mesh_view pointing into this object's arrays (keep self alive)."""
        v = _lib.ma_mesh_view()
        v.ncells = self.ncells
        v.cell_coords = f64p(self.cell_coords)
        v.cell_volumes = f64p(self.cell_volumes)
        v.internal = self.internal.to_c()
        v.nbc = len(self.bc)
        for i, b in enumerate(self.bc):
            v.bc[i] = b.to_c()
        return v

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h:
            try:
                lib().ma_host_mesh_free(h)
            except Exception:
                pass
            self._handle = None


class Parallel3DMesh:
    """Structured box (or ramp) Hexa8 mesh in unstructured form, one rank."""

    def __init__(self, nx, ny, nz, lx, ly, lz, problem_type, angle=0.0, bc_override=None):
        self.options = Options(nx=nx, ny=ny, nz=nz, lx=lx, ly=ly, lz=lz, problem_type=problem_type, angle=angle)
        if bc_override is not None:
            self.options.bc_override = bc_override

    @classmethod
    def from_options(cls, options):
        m = cls.__new__(cls)
        m.options = options.copy()
        return m

    def fill_mesh_data(self, device_geometry=False):
        """fillMeshData on the host; device_geometry=True computes the face
        and cell geometry on the current CUDA device (same bits)."""
        L = lib()
        h = ctypes.c_void_p()
        flags = _lib.MA_HOST_MESH_DEVICE_GEOMETRY if device_geometry else 0
        check(L.ma_host_mesh_build_ex(ctypes.byref(self.options.c), flags, ctypes.byref(h)))
        v = _lib.ma_mesh_view()
        check(L.ma_host_mesh_view(h, ctypes.byref(v)))
        C = v.ncells
        coords = np.ctypeslib.as_array(v.cell_coords, shape=(C, 3)).copy()
        vols = np.ctypeslib.as_array(v.cell_volumes, shape=(C,)).copy()
        internal = FaceSet(v.internal, "internal")
        bc = [FaceSet(v.bc[i], BC_NAMES[v.bc[i].type]) for i in range(v.nbc)]
        return MeshData(C, coords, vols, internal, bc, handle=h)


def initial_state(mesh_data, options):
    """Initial conserved state (kokkos/Initial_Conditions.h), shape (ncells, 5)."""
    if mesh_data._handle is None:
        raise ValueError("initial_state needs a MeshData built by Parallel3DMesh")
    U = np.empty((mesh_data.ncells, 5), np.float64)
    check(lib().ma_host_initial_state(mesh_data._handle, ctypes.byref(options.c), f64p(U)))
    return U


def mesh_hash(mesh_data):
    """ma_mesh_hash: 64-bit hash of the mesh a checkpoint belongs to."""
    v = mesh_data.view()
    return int(lib().ma_mesh_hash(ctypes.byref(v)))


def checkpoint_write(path, U, steps_done, time, dt, mesh_hash_value):
    """Writes the conserved state U (ncells, 5) as a checkpoint file."""
    U = np.ascontiguousarray(U, dtype=np.float64)
    info = _lib.ma_checkpoint_info(U.shape[0], int(steps_done), float(time), float(dt), int(mesh_hash_value))
    check(lib().ma_checkpoint_write(os.fsencode(path), ctypes.byref(info), f64p(U), MA_LAYOUT_AOS))


def checkpoint_read(path):
    """Reads a checkpoint: (info dict, U of shape (ncells, 5))."""
    info = _lib.ma_checkpoint_info()
    check(lib().ma_checkpoint_read(os.fsencode(path), ctypes.byref(info), ctypes.cast(None, _lib.P_f64), 0,
                                   MA_LAYOUT_AOS))
    U = np.empty((info.ncells, 5), np.float64)
    check(lib().ma_checkpoint_read(os.fsencode(path), ctypes.byref(info), f64p(U), info.ncells, MA_LAYOUT_AOS))
    return {"ncells": info.ncells, "steps_done": info.steps_done, "time": info.time, "dt": info.dt,
            "mesh_hash": info.mesh_hash}, U


def run_options_read(path):
    """ma_run_options_read: the checkpoint / restart lines of an input file."""
    r = _lib.ma_run_options()
    check(lib().ma_run_options_read(os.fsencode(path), ctypes.byref(r)))
    return {"checkpoint_path": r.checkpoint_path.decode(), "checkpoint_frequency": r.checkpoint_frequency,
            "restart_path": r.restart_path.decode()}


class DeviceMesh:
    """Device copy of a MeshData (ma_mesh_upload); shareable by solvers."""

    def __init__(self, mesh_data, cell_flux=False):
        """cell_flux: also build the slot-order lists of gather = MA_GATHER_CELL_FLUX."""
        self._mesh_data = mesh_data
        self._view = mesh_data.view()
        self._h = ctypes.c_void_p()
        flags = _lib.MA_MESH_CELL_FLUX if cell_flux else 0
        check(lib().ma_mesh_upload_ex(ctypes.byref(self._view), flags, ctypes.byref(self._h)))
        self.ncells = mesh_data.ncells

    @property
    def device_bytes(self):
        return int(lib().ma_mesh_device_bytes(self._h))

    def close(self):
        if self._h:
            lib().ma_mesh_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TimeSolverExplicitRK4:
    """RK4 solver on the GPU (kokkos/TimeSolverExplicitRK4.h:160-539)."""

    def __init__(self, mesh_data, options, device_mesh=None):
        self.options = options.copy()
        self.mesh_data = mesh_data
        self.device_mesh = device_mesh if device_mesh is not None else DeviceMesh(
            mesh_data, cell_flux=self.options.gather == _lib.MA_GATHER_CELL_FLUX)
        self._h = ctypes.c_void_p()
        check(lib().ma_solver_create(self.device_mesh._h, ctypes.byref(self.options.c), ctypes.byref(self._h)))
        self.ncells = mesh_data.ncells

    # -- state ---------------------------------------------------------------
    def set_state(self, U, layout=MA_LAYOUT_AOS):
        """U is (ncells, 5) for MA_LAYOUT_AOS, (5, ncells) for MA_LAYOUT_SOA."""
        shape = (self.ncells, 5) if layout == MA_LAYOUT_AOS else (5, self.ncells)
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(shape)
        check(lib().ma_solver_set_state(self._h, f64p(U), int(layout)))

    def init_state(self):
        check(lib().ma_solver_init_state(self._h, self.mesh_data._handle))

    def get_state(self, layout=MA_LAYOUT_AOS):
        U = np.empty((self.ncells, 5) if layout == MA_LAYOUT_AOS else (5, self.ncells), np.float64)
        check(lib().ma_solver_get_state(self._h, f64p(U), int(layout)))
        return U

    def get_residual(self):
        R = np.empty((self.ncells, 5), np.float64)
        check(lib().ma_solver_get_residual(self._h, f64p(R), MA_LAYOUT_AOS))
        return R

    # -- time stepping ---------------------------------------------------------
    def step(self, nsteps=1):
        check(lib().ma_solver_step(self._h, int(nsteps)))

    def synchronize(self):
        check(lib().ma_solver_synchronize(self._h))

    def solve(self):
        """Solve(): initial state then options.ntimesteps steps; returns U."""
        self.init_state()
        self.step(self.options.ntimesteps)
        self.synchronize()
        return self.get_state()

    def save_checkpoint(self, path):
        """Writes the current state, step count and dt to a checkpoint file."""
        self.synchronize()
        n = self.steps_done
        checkpoint_write(path, self.get_state(), n, n * self.dt, self.dt, mesh_hash(self.mesh_data))

    def restore_checkpoint(self, path):
        """Continues from a checkpoint of this mesh: state and dt; returns the
        checkpoint's step count (steps_done restarts from 0)."""
        info, U = checkpoint_read(path)
        if info["ncells"] != self.ncells or info["mesh_hash"] != mesh_hash(self.mesh_data):
            raise MiniaeroError(_lib.MA_EINVAL, "%s was written for a different mesh" % path)
        self.set_state(U)
        self.dt = info["dt"]
        return info["steps_done"]

    def profile_steps(self, nsteps):
        """Steps with CUDA events around each kernel; {kind: (ms_total, launches)}."""
        ms = np.zeros(_lib.MA_PROFILE_KINDS, np.float64)
        n = np.zeros(_lib.MA_PROFILE_KINDS, np.int32)
        check(lib().ma_solver_profile_steps(self._h, int(nsteps), f64p(ms), i32p(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(_lib.KERNEL_KINDS) if n[i] > 0}

    def check_state(self):
        bad = ctypes.c_int64(-1)
        st = lib().ma_solver_check_state(self._h, ctypes.byref(bad))
        return st, bad.value

    @property
    def dt(self):
        return float(lib().ma_solver_dt(self._h))

    @dt.setter
    def dt(self, value):
        check(lib().ma_solver_set_dt(self._h, float(value)))

    @property
    def stream(self):
        return lib().ma_solver_stream(self._h)

    @property
    def steps_done(self):
        return int(lib().ma_solver_steps_done(self._h))

    @property
    def launches_per_step(self):
        return int(lib().ma_solver_launches_per_step(self._h))

    def close(self):
        if self._h:
            lib().ma_solver_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Many independent meshes advanced together (ma_batch_*)."""

    def __init__(self, physics, capacity=256, budget_bytes=150 << 30):
        self.physics = physics.copy()
        self._h = ctypes.c_void_p()
        check(lib().ma_batch_create(ctypes.byref(self.physics.c), int(capacity), int(budget_bytes),
                                    ctypes.byref(self._h)))
        self._meshes = {}

    def member_bytes(self, device_mesh):
        return int(lib().ma_batch_member_bytes(self._h, device_mesh._h))

    def add(self, device_mesh, U0, dt=0.0, inflow_state=None):
        U0 = np.ascontiguousarray(U0, dtype=np.float64).reshape(device_mesh.ncells, 5)
        mid = ctypes.c_int32(-1)
        inflow = None
        if inflow_state is not None:
            inflow = np.ascontiguousarray(inflow_state, dtype=np.float64).reshape(5)
        check(lib().ma_batch_add(self._h, device_mesh._h, f64p(U0), MA_LAYOUT_AOS, float(dt),
                                 f64p(inflow) if inflow is not None else ctypes.cast(None, _lib.P_f64),
                                 ctypes.byref(mid)))
        self._meshes[mid.value] = device_mesh  # keep the mesh alive
        return mid.value

    def remove(self, member_id):
        check(lib().ma_batch_remove(self._h, int(member_id)))
        self._meshes.pop(member_id, None)

    def get_state(self, member_id):
        dm = self._meshes.get(member_id)
        if dm is None:
            raise MiniaeroError(_lib.MA_ENOTFOUND, "unknown batch member %r" % member_id)
        U = np.empty((dm.ncells, 5), np.float64)
        check(lib().ma_batch_get_state(self._h, int(member_id), f64p(U), MA_LAYOUT_AOS))
        return U

    def step(self, nsteps=1):
        check(lib().ma_batch_step(self._h, int(nsteps)))

    def set_single_launch(self, block=256):
        """block > 0: each step() call runs as one cooperative launch (all
        steps, all members); 0: per-kind launches in a CUDA graph. Returns
        the launch's grid (0 when off)."""
        grid = ctypes.c_int32(0)
        check(lib().ma_batch_set_single_launch(self._h, int(block), ctypes.byref(grid)))
        return grid.value

    def synchronize(self):
        check(lib().ma_batch_synchronize(self._h))

    def autotune(self, reps=3):
        best = np.zeros(4)
        check(lib().ma_batch_autotune(self._h, int(reps), f64p(best)))
        return best

    def profile_steps(self, nsteps):
        """Steps with CUDA events around each kernel; {kind: (ms_total, launches)}."""
        ms = np.zeros(_lib.MA_PROFILE_KINDS, np.float64)
        n = np.zeros(_lib.MA_PROFILE_KINDS, np.int32)
        check(lib().ma_batch_profile_steps(self._h, int(nsteps), f64p(ms), i32p(n)))
        return {k: (float(ms[i]), int(n[i])) for i, k in enumerate(_lib.KERNEL_KINDS) if n[i] > 0}

    @property
    def launch(self):
        b = np.zeros(4, np.int32)
        g = np.zeros(4, np.int32)
        check(lib().ma_batch_get_launch(self._h, i32p(b), i32p(g)))
        return b.tolist(), g.tolist()

    def set_launch(self, block, grid):
        b = np.ascontiguousarray(block, np.int32)
        g = np.ascontiguousarray(grid, np.int32)
        check(lib().ma_batch_set_launch(self._h, i32p(b), i32p(g)))

    def member_dt(self, member_id):
        return float(lib().ma_batch_member_dt(self._h, int(member_id)))

    def member_steps(self, member_id):
        return int(lib().ma_batch_member_steps(self._h, int(member_id)))

    @property
    def stream(self):
        return lib().ma_batch_stream(self._h)

    @property
    def cells(self):
        return int(lib().ma_batch_cells(self._h))

    @property
    def size(self):
        return int(lib().ma_batch_size(self._h))

    @property
    def device_bytes(self):
        return int(lib().ma_batch_device_bytes(self._h))

    def close(self):
        if self._h:
            lib().ma_batch_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Serving loop with continuous batching (ma_server_*)."""

    QUEUED, RUNNING, DONE, CANCELLED, FAILED = range(5)

    def __init__(self, physics, budget_bytes=150 << 30, tick_steps=10, capacity=512, thread=True, dry_run=False):
        self.physics = physics.copy()
        flags = (_lib.MA_SERVER_THREAD if thread else 0) | (_lib.MA_SERVER_DRYRUN if dry_run else 0)
        self._h = ctypes.c_void_p()
        check(lib().ma_server_create(ctypes.byref(self.physics.c), int(budget_bytes), int(tick_steps), int(capacity),
                                     flags, ctypes.byref(self._h)))
        self._cells = {}

    @staticmethod
    def request(nx, ny, nz, lx, ly, lz, inflow_state, nsteps, problem_type=1, dt=0.0, keep_result=False, angle=0.0):
        r = _lib.ma_request()
        r.nx, r.ny, r.nz, r.problem_type = int(nx), int(ny), int(nz), int(problem_type)
        r.lx, r.ly, r.lz, r.angle = float(lx), float(ly), float(lz), float(angle)
        for k in range(5):
            r.inflow_state[k] = float(inflow_state[k])
        r.nsteps = int(nsteps)
        r.dt = float(dt)
        r.keep_result = 1 if keep_result else 0
        return r

    def submit(self, req):
        rid = ctypes.c_int64(-1)
        check(lib().ma_server_submit(self._h, ctypes.byref(req), ctypes.byref(rid)))
        self._cells[rid.value] = req.nx * req.ny * req.nz
        return rid.value

    def set_max_running_cells(self, cells):
        check(lib().ma_server_set_max_running_cells(self._h, int(cells)))

    def set_launch(self, block, grid):
        """Launch shapes of the server's batch (e.g. from Batch.autotune); only while idle."""
        b = np.ascontiguousarray(block, dtype=np.int32)
        g = np.ascontiguousarray(grid, dtype=np.int32)
        check(lib().ma_server_set_launch(self._h, i32p(b), i32p(g)))

    def preload(self, req):
        check(lib().ma_server_preload_mesh(self._h, ctypes.byref(req)))

    def poll(self):
        p = ctypes.c_int32(0)
        check(lib().ma_server_poll(self._h, ctypes.byref(p)))
        return bool(p.value)

    def cancel(self, rid):
        check(lib().ma_server_cancel(self._h, int(rid)))

    def query(self, rid):
        info = _lib.ma_request_info()
        check(lib().ma_server_query(self._h, int(rid), ctypes.byref(info)))
        return info

    def wait(self, rid, timeout=60.0):
        check(lib().ma_server_wait(self._h, int(rid), float(timeout)))
        return self.query(rid)

    def result(self, rid):
        U = np.empty((self._cells[rid], 5), np.float64)
        check(lib().ma_server_result(self._h, int(rid), f64p(U)))
        return U

    def stats(self):
        st = _lib.ma_server_stats()
        check(lib().ma_server_get_stats(self._h, ctypes.byref(st)))
        return {n: getattr(st, n) for n, _ in st._fields_}

    def close(self):
        if self._h:
            lib().ma_server_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- operator-level entry points -------------------------------------------------
def _a(x, shape):
    return np.ascontiguousarray(x, dtype=np.float64).reshape(shape)


def roe_flux(pl, pr, normal, tangent, binormal):
    """roe_flux::compute_flux on n faces; primitives (n,5), vectors (n,3)."""
    pl = _a(pl, (-1, 5))
    n = pl.shape[0]
    pr, nm, tg, bn = _a(pr, (n, 5)), _a(normal, (n, 3)), _a(tangent, (n, 3)), _a(binormal, (n, 3))
    out = np.empty((n, 5), np.float64)
    check(lib().ma_op_roe_flux(n, f64p(pl), f64p(pr), f64p(nm), f64p(tg), f64p(bn), f64p(out)))
    return out


def viscous_flux(grad, prim, area, viscosity_model=MA_VISC_SUTHERLAND, mu=0.0, prandtl=0.72):
    """newtonian_viscous_flux::compute_flux; grad (n,5,3), prim (n,5), area (n,3)."""
    grad = _a(grad, (-1, 5, 3))
    n = grad.shape[0]
    prim, area = _a(prim, (n, 5)), _a(area, (n, 3))
    out = np.empty((n, 5), np.float64)
    check(lib().ma_op_viscous_flux(n, f64p(grad), f64p(prim), f64p(area), viscosity_model, mu, prandtl,
                                   f64p(out)))
    return out


def venkat_limit(dumax, dumin, du, d2):
    dumax = _a(dumax, (-1,))
    n = dumax.shape[0]
    dumin, du, d2 = _a(dumin, (n,)), _a(du, (n,)), _a(d2, (n,))
    out = np.empty(n, np.float64)
    check(lib().ma_op_limiter(n, MA_LIMITER_VENKAT, f64p(dumax), f64p(dumin), f64p(du), f64p(d2), f64p(out)))
    return out


def vanalbada_limit(dumax, dumin, du):
    dumax = _a(dumax, (-1,))
    n = dumax.shape[0]
    dumin, du = _a(dumin, (n,)), _a(du, (n,))
    out = np.empty(n, np.float64)
    check(lib().ma_op_limiter(n, MA_LIMITER_VANALBADA, f64p(dumax), f64p(dumin), f64p(du),
                              ctypes.cast(None, _lib.P_f64), f64p(out)))
    return out


def compute_primitives(U):
    U = _a(U, (-1, 5))
    out = np.empty_like(U)
    check(lib().ma_op_primitives(U.shape[0], f64p(U), f64p(out)))
    return out


def fp64_rate(op):
    """Measured FP64 thread-instruction rate of the current device for
    additions ("add"), multiplications ("mul") or fused multiply-adds ("fma")."""
    code = {"add": 0, "mul": 1, "fma": 2}[op]
    r = ctypes.c_double()
    check(lib().ma_debug_fp64_rate(code, ctypes.byref(r)))
    return r.value


# ---- one RK stage's drivers on a DeviceMesh and a state (n cells x 5) ----
def green_gauss(mesh, U):
    """GreenGauss::compute_gradients: gradients of the primitives of U, (ncells, 5, 3)."""
    U = _a(U, (mesh.ncells, 5))
    out = np.empty((mesh.ncells, 5, 3), np.float64)
    check(lib().ma_op_green_gauss(mesh._h, f64p(U), MA_LAYOUT_AOS, f64p(out)))
    return out


def stencil_limiter(mesh, U, limiter=MA_LIMITER_VENKAT):
    """StencilLimiter::compute_min_max + compute_limiter with U's Green-Gauss
    gradient: (ncells, 5)."""
    U = _a(U, (mesh.ncells, 5))
    out = np.empty((mesh.ncells, 5), np.float64)
    check(lib().ma_op_stencil_limiter(mesh._h, int(limiter), f64p(U), MA_LAYOUT_AOS, f64p(out)))
    return out


def bc_flux(mesh, options, U):
    """The boundary functors as Solve applies them: each cell's boundary
    contributions to cell_flux, (ncells, 5); options supply the viscosity
    model and the inflow state."""
    U = _a(U, (mesh.ncells, 5))
    out = np.empty((mesh.ncells, 5), np.float64)
    check(lib().ma_op_bc_flux(mesh._h, ctypes.byref(options._o), f64p(U), MA_LAYOUT_AOS, f64p(out)))
    return out


def apply_cell_flux(dt, volumes, cell_flux):
    """apply_cell_flux: res = 0 + (dt / V) * cell_flux, (ncells, 5)."""
    v = _a(volumes, (-1,))
    f = _a(cell_flux, (v.shape[0], 5))
    out = np.empty_like(f)
    check(lib().ma_op_apply_cell_flux(v.shape[0], float(dt), f64p(v), f64p(f), f64p(out)))
    return out


def rk_update(alpha, res, src):
    """update: src + alpha * res, elementwise."""
    src = np.ascontiguousarray(src, dtype=np.float64)
    res = _a(res, src.shape)
    out = np.empty_like(src)
    check(lib().ma_op_rk_update(src.size, float(alpha), f64p(res), f64p(src), f64p(out)))
    return out
