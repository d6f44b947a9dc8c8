"""Size-independent properties at the benchmark sizes, where the oracle is too
slow to compare against: Sod 256x128x128 on 1.0x0.5x0.5 (4,194,304 cells,
2nd order, Venkatakrishnan, viscous) and the flat-plate box 512x128x128 on
2.0x0.5x0.5 (8,388,608 cells). Checked: mass and energy conservation with
closed (Tangent) walls, agreement of the ATOMICS_FLUX and CELL_FLUX reduction
orders, the mixed form's error against FP64, preservation of a uniform flow,
and the symmetries of the Sod problem (one-dimensional when inviscid, mirror
symmetric about the mid-planes when viscous)."""
import math

import numpy as np
import pytest

import miniaero_gb300 as ma

pytestmark = pytest.mark.gpu

STEPS = 10


def sod_options(**kw):
    o = ma.Options(problem_type=0, lx=1.0, ly=0.5, lz=0.5, nx=256, ny=128, nz=128, second_order_space=1, viscous=1,
                   ic=ma.MA_IC_SOD, viscosity_model=ma.MA_VISC_CONSTANT, mu=1.8e-5, prandtl=0.72, cfl=0.5)
    for k, v in kw.items():
        setattr(o, k, v)
    return o


@pytest.fixture(scope="module")
def sod_mesh():
    o = sod_options()
    return ma.Parallel3DMesh.from_options(o).fill_mesh_data()


def run(md, o, steps=STEPS, device_mesh=None):
    with ma.TimeSolverExplicitRK4(md, o, device_mesh=device_mesh) as s:
        s.set_state(ma.initial_state(md, o))
        s.step(steps)
        s.synchronize()
        return s.get_state()


def total(md, U, k):
    return math.fsum((U[:, k] * md.cell_volumes).tolist())


def test_closed_box_conserves_mass_and_energy(has_gpu, sod_mesh):
    o = sod_options(bc_override=[1, 1, 1, 1, 1, 1])
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    U = run(md, o)
    assert not np.array_equal(U, U0)
    for k in (0, 4):
        m0, m1 = total(md, U0, k), total(md, U, k)
        assert abs(m1 - m0) <= 1e-12 * abs(m0), (k, m0, m1)


def test_reduction_orders_agree(has_gpu, sod_mesh):
    o = sod_options()
    a = run(sod_mesh, o)
    oc = o.copy()
    oc.gather = ma._lib.MA_GATHER_CELL_FLUX
    dm = ma.DeviceMesh(sod_mesh, cell_flux=True)
    b = run(sod_mesh, oc, device_mesh=dm)
    dm.close()
    scale = np.abs(a).max(axis=0)
    scale[1:4] = scale[1:4].max()
    assert np.max(np.abs(a - b) / scale) <= 1e-12


def test_mixed_form_within_tolerance(has_gpu, sod_mesh):
    """The mixed form's stated bound: relative L2 error of density (and of
    energy) at most 1e-5 against FP64; momentum against the momentum norm."""
    o = sod_options()
    a = run(sod_mesh, o)
    om = o.copy()
    om.precision = ma.MA_PREC_MIXED
    b = run(sod_mesh, om)
    for k in (0, 4):
        assert np.linalg.norm(b[:, k] - a[:, k]) <= 1e-5 * np.linalg.norm(a[:, k]), k
    assert np.linalg.norm(b[:, 1:4] - a[:, 1:4]) <= 1e-5 * np.linalg.norm(a[:, 1:4])


def test_inviscid_sod_stays_one_dimensional(has_gpu, sod_mesh):
    """Without viscous terms the Sod problem varies along x only: the
    transverse momentum stays at round-off level against the x-momentum."""
    U = run(sod_mesh, sod_options(viscous=0))
    mx = np.abs(U[:, 1]).max()
    assert mx > 0.0
    assert np.abs(U[:, 2:4]).max() <= 1e-12 * mx


def test_viscous_sod_is_mirror_symmetric(has_gpu, sod_mesh):
    """With viscous terms the Tangent walls carry no viscous stress, so the
    reference's discretisation drives a transverse flow in the wall cells
    (about 1e-3 of the x-momentum here); the solution stays mirror-symmetric
    about the box's mid-planes in y and z: density, x-momentum and energy
    even, the normal momentum odd."""
    U = run(sod_mesh, sod_options())
    n = np.array([256, 128, 128])
    ijk = np.floor(sod_mesh.cell_coords / (np.array([1.0, 0.5, 0.5]) / n)).astype(np.int64)
    key = lambda a: a[:, 0] + n[0] * (a[:, 1] + n[1] * a[:, 2])
    pos = np.empty(sod_mesh.ncells, np.int64)
    pos[key(ijk)] = np.arange(sod_mesh.ncells)
    scale = np.abs(U).max(axis=0)
    assert scale[2] > 0.0 and scale[3] > 0.0
    for axis, comp in ((1, 2), (2, 3)):
        m = ijk.copy()
        m[:, axis] = n[axis] - 1 - m[:, axis]
        j = pos[key(m)]
        for k in range(5):
            err = U[:, k] + U[j, k] if k == comp else U[:, k] - U[j, k]
            assert np.max(np.abs(err)) <= 1e-10 * scale[k], (axis, k)


def test_uniform_flow_is_preserved_at_eight_million_cells(has_gpu):
    """Mach 0.3 inflow state everywhere, inflow on the left and extrapolation
    elsewhere (no wall): the state stays uniform."""
    R, g, T, p = 287.05, 1.4, 300.0, 1e5
    rho = p / (R * T)
    u = 0.3 * math.sqrt(g * R * T)
    state = [rho, rho * u, 0.0, 0.0, rho * (R / (g - 1.0) * T + 0.5 * u * u)]
    o = ma.Options(problem_type=1, lx=2.0, ly=0.5, lz=0.5, nx=512, ny=128, nz=128, second_order_space=1, viscous=1,
                   limiter=ma.MA_LIMITER_VANALBADA, ic=ma.MA_IC_CONSTANT, inflow_state=state, inflow_given=1,
                   bc_override=[0, 0, 0, 0, 0, 2], cfl=0.5)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    assert md.ncells == 8388608
    U0 = ma.initial_state(md, o)
    U = run(md, o, steps=5)
    scale = np.abs(U0).max(axis=0)
    scale[1:4] = scale[1:4].max()
    assert np.max(np.abs(U - U0) / scale) <= 1e-12


@pytest.mark.parametrize("name,steps", [("sod_2nd_viscous_256x128x128", 100),
                                        ("flat_plate_vanalbada_512x128x128", 50)])
def test_mixed_form_error_at_the_configured_step_count(has_gpu, name, steps):
    """The benchmark configurations at their own step counts (100 RK4 steps
    for the Sod mesh, 50 for the flat plate) and CFL 0.5 dt: the mixed form's
    relative L2 density error against the GPU's FP64 result (which equals the
    reference's bits) stays within 1e-5. All five variables are reported;
    momentum components relative to the momentum norm."""
    import json
    import os
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "full_size.json")) as f:
        case = json.load(f)["cases"][name]
    o = ma.Options(**case["options"])
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    dm = ma.DeviceMesh(md)
    a = run(md, o, steps=steps, device_mesh=dm)
    om = o.copy()
    om.precision = ma.MA_PREC_MIXED
    b = run(md, om, steps=steps, device_mesh=dm)
    dm.close()
    mom = np.linalg.norm(a[:, 1:4])
    err = [float(np.linalg.norm(b[:, k] - a[:, k]) / (mom if k in (1, 2, 3) else np.linalg.norm(a[:, k])))
           for k in range(5)]
    print("%s after %d steps: rel L2 error rho %.3e, rho u/v/w %.3e %.3e %.3e (of |rho u|), rho E %.3e"
          % (name, steps, *err))
    assert err[0] <= 1e-5, err
