"""CELL_FLUX gather order on the GPU (gather = MA_GATHER_CELL_FLUX, the
reference's -DCELL_FLUX build): bit-identical to the oracle's restatement on
the reference's serial cases and the extensions, the same bits in a batch as
alone, the mixed form within its tolerance, and a clear error for a mesh
uploaded without the slot-order lists."""
import numpy as np
import pytest

import miniaero_gb300 as ma
import oracle
from tests.golden.make_golden import CASES, options
from tests.test_gpu_parity import assert_bitexact

pytestmark = pytest.mark.gpu


def cf(o, **kw):
    c = o.copy()
    c.gather = ma._lib.MA_GATHER_CELL_FLUX
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def gpu_solve(md, o, U0):
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.set_state(U0)
        s.step(o.ntimesteps)
        s.synchronize()
        return s.get_state()


@pytest.mark.parametrize("case", sorted(CASES))
def test_reference_cases_bitexact(has_gpu, case):
    o = cf(options(case))
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    assert_bitexact(gpu_solve(md, o, U0), oracle.solve(md, o, U0))


@pytest.mark.parametrize("limiter,visc_model", [(ma.MA_LIMITER_VANALBADA, ma.MA_VISC_SUTHERLAND),
                                                (ma.MA_LIMITER_VENKAT, ma.MA_VISC_CONSTANT)])
def test_extensions_bitexact(has_gpu, limiter, visc_model):
    o = cf(options("flatplate_serial"), limiter=limiter, viscosity_model=visc_model, mu=1.8e-5, prandtl=0.72,
           ntimesteps=60)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    assert_bitexact(gpu_solve(md, o, U0), oracle.solve(md, o, U0))


def test_batch_member_equals_solve_alone(has_gpu):
    o = cf(options("ramp_serial"), ntimesteps=20)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    alone = gpu_solve(md, o, U0)
    dm = ma.DeviceMesh(md, cell_flux=True)
    b = ma.Batch(o, capacity=4)
    ids = [b.add(dm, U0, dt=o.dt) for _ in range(2)]
    b.step(20)
    b.synchronize()
    for i in ids:
        assert_bitexact(b.get_state(i), alone)
    b.close()
    dm.close()


def test_mixed_within_tolerance(has_gpu):
    o = cf(options("flatplate_serial"), ntimesteps=60)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    ref = gpu_solve(md, o, U0)
    m = cf(o, precision=ma.MA_PREC_MIXED)
    U = gpu_solve(md, m, U0)
    assert np.linalg.norm(U[:, 0] - ref[:, 0]) / np.linalg.norm(ref[:, 0]) < 1e-5


def test_cli_gather_cell_flux(has_gpu, tmp_path):
    """The CLI's `gather cell_flux` line: results.0 of the oracle's CELL_FLUX solve."""
    from tests.test_gpu_checkpoint import run_cli, write_inp
    from tests.test_oracle_gold import results_lines
    case = "flatplate_serial"
    write_inp(tmp_path / "miniaero.inp", case, steps=40, extra=["gather cell_flux"])
    run_cli(tmp_path)
    o = cf(options(case), ntimesteps=40)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    expected = results_lines(md, oracle.solve(md, o, ma.initial_state(md, o)))
    assert (tmp_path / "results.0").read_text().splitlines() == expected


def test_bad_slots_are_rejected(has_gpu):
    o = options("sod_serial")
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    # Every hex cell uses all six slots, so moving one face to another slot
    # makes that slot appear twice within its left cell.
    md.internal.flux_index[0, 0] = (md.internal.flux_index[0, 0] + 1) % 6
    with pytest.raises(ma.MiniaeroError, match="flux_index") as e:
        ma.DeviceMesh(md, cell_flux=True)
    assert e.value.status == ma._lib.MA_EINVAL
    md.internal.flux_index = None
    with pytest.raises(ma.MiniaeroError, match="flux_index"):
        ma.DeviceMesh(md, cell_flux=True)
    ma.DeviceMesh(md).close()  # the default lists need no slots


def test_mesh_without_slot_lists_is_rejected(has_gpu):
    o = cf(options("sod_serial"))
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    dm = ma.DeviceMesh(md)  # no MA_MESH_CELL_FLUX
    with pytest.raises(ma.MiniaeroError, match="MA_MESH_CELL_FLUX") as e:
        ma.TimeSolverExplicitRK4(md, o, device_mesh=dm)
    assert e.value.status == ma._lib.MA_EINVAL
    b = ma.Batch(o, capacity=2)
    with pytest.raises(ma.MiniaeroError, match="MA_MESH_CELL_FLUX"):
        b.add(dm, ma.initial_state(md, o), dt=o.dt)
    b.close()
    dm.close()
