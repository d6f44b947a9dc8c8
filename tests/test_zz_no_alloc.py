"""Allocation-free CFL time step (ma_cfl_dt_noalloc, C-ABI) against the
solver's own CFL evaluation (ma_solver_set_state, which reduces in its arena):
the same dt bit for bit on consecutive calls, across meshes whose block counts
differ (a call runs over partial minima the previous call left behind), at the
largest accepted mesh, and a clear error one cell beyond it; repeated calls
leave the device's free memory unchanged. The file name
sorts last so that the suite also runs it after every other GPU test."""
import copy
import ctypes

import numpy as np
import pytest

import miniaero_gb300 as ma
from miniaero_gb300._lib import MA_EINVAL, check, lib

MAX_CELLS = 65536 * 256


def noalloc_dt(dmesh, U, cfl):
    """dt from the allocation-free entry point for host state U (C, 5)."""
    import torch
    d = torch.from_numpy(np.ascontiguousarray(U.T)).to("cuda")  # [5][C] on the device
    torch.cuda.synchronize()
    dt = ctypes.c_double(0.0)
    check(lib().ma_cfl_dt_noalloc(dmesh._h, ctypes.c_void_p(d.data_ptr()), cfl, ctypes.byref(dt), None))
    return dt.value


def box_case(problem_type, n, cfl=0.5):
    o = ma.Options(problem_type=problem_type, nx=n[0], ny=n[1], nz=n[2], lx=n[0] * 0.01, ly=n[1] * 0.01,
                   lz=n[2] * 0.01, ntimesteps=1, second_order_space=1, viscous=1, cfl=cfl)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    dm = ma.DeviceMesh(md)
    s = ma.TimeSolverExplicitRK4(md, o, device_mesh=dm)
    s.init_state()
    return md, dm, s


@pytest.mark.gpu
def test_matches_solver_on_consecutive_calls(has_gpu):
    mdA, dmA, sA = box_case(0, (64, 32, 32))  # Sod, 65,536 cells: 256 blocks
    mdB, dmB, sB = box_case(1, (20, 12, 6))  # flat plate, 1,440 cells: 6 blocks
    UA, UB = sA.get_state(), sB.get_state()
    assert noalloc_dt(dmA, UA, 0.5) == sA.dt
    assert noalloc_dt(dmB, UB, 0.5) == sB.dt
    assert noalloc_dt(dmA, UA, 0.5) == sA.dt
    # A moving state: the velocity term of the CFL sum is no longer zero.
    sA.step(3)
    UA3 = sA.get_state()
    sA.set_state(UA3)
    first = noalloc_dt(dmA, UA3, 0.5)
    second = noalloc_dt(dmA, UA3, 0.5)
    assert first == sA.dt and second == sA.dt
    assert noalloc_dt(dmB, UB, 0.25) == 0.25 * (sB.dt / 0.5)
    for s, d in ((sA, dmA), (sB, dmB)):
        s.close()
        d.close()


def faceless_mesh(ncells, template):
    """ncells unit cells with no faces but one boundary face on the last cell,
    so that only the last cell has a finite CFL quotient."""
    fs = copy.copy(template.bc[0])
    fs.nfaces = 1
    fs.conn = np.array([[ncells - 1, fs.conn[0, 1]]], np.int32)
    fs.coords, fs.normal = fs.coords[:1].copy(), fs.normal[:1].copy()
    fs.tangent, fs.binormal = fs.tangent[:1].copy(), fs.binormal[:1].copy()
    fs.permutation = np.zeros(1, np.int32)
    internal = copy.copy(template.internal)
    internal.nfaces = 0
    coords = np.zeros((ncells, 3), np.float64)
    vols = np.full(ncells, 1e-6, np.float64)
    return ma.MeshData(ncells, coords, vols, internal, [fs])


def uniform_state(ncells):
    U = np.empty((ncells, 5), np.float64)
    U[:, 0] = 1.2
    U[:, 1] = 1.2 * 100.0
    U[:, 2] = 1.2 * -30.0
    U[:, 3] = 0.0
    U[:, 4] = 1e5 / 0.4 + 0.5 * 1.2 * (100.0 ** 2 + 30.0 ** 2)
    return U


@pytest.mark.gpu
def test_calls_leave_device_memory_unchanged(has_gpu):
    """The property the entry point exists for: after a first call (which may
    load the module on the device), further calls on the largest accepted mesh
    change the device's free memory by nothing."""
    import torch
    o = ma.Options(problem_type=1, nx=4, ny=4, nz=2, ntimesteps=1, cfl=0.5)
    template = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    md = faceless_mesh(MAX_CELLS, template)
    dm = ma.DeviceMesh(md)
    U = uniform_state(MAX_CELLS)
    d = torch.from_numpy(np.ascontiguousarray(U.T)).to("cuda")
    torch.cuda.synchronize()
    dt = ctypes.c_double(0.0)

    def call():
        check(lib().ma_cfl_dt_noalloc(dm._h, ctypes.c_void_p(d.data_ptr()), 0.5, ctypes.byref(dt), None))
        return dt.value

    first = call()
    free_before, _ = torch.cuda.mem_get_info()
    values = [call() for _ in range(10)]
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert values == [first] * 10 and np.isfinite(first) and first > 0.0
    del d
    dm.close()


@pytest.mark.gpu
def test_largest_mesh_and_one_beyond(has_gpu):
    o = ma.Options(problem_type=1, nx=4, ny=4, nz=2, ntimesteps=1, cfl=0.5)
    template = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    md = faceless_mesh(MAX_CELLS, template)
    dm = ma.DeviceMesh(md)
    U = uniform_state(MAX_CELLS)
    s = ma.TimeSolverExplicitRK4(md, o, device_mesh=dm)
    s.set_state(U)
    assert np.isfinite(s.dt) and s.dt > 0.0
    assert noalloc_dt(dm, U, 0.5) == s.dt
    assert noalloc_dt(dm, U, 0.5) == s.dt
    s.close()
    dm.close()
    del U

    md = faceless_mesh(MAX_CELLS + 1, template)
    dm = ma.DeviceMesh(md)
    with pytest.raises(ma.MiniaeroError) as e:
        noalloc_dt(dm, uniform_state(MAX_CELLS + 1), 0.5)
    assert e.value.status == MA_EINVAL and "at most 16777216" in str(e.value)
    dm.close()
