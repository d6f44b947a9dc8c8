"""The reference's -DCELL_FLUX build as the oracle restates it (per-slot
storage, gathers in element-local slot order): it stays within rounding of
the default -DATOMICS_FLUX order on the reference's serial cases, threads do
not change its bits, and the input file selects it. There is no golden output
of a CELL_FLUX build in the reference tree, so this mode's parity rests on
the oracle's restatement (tests/test_gpu_cell_flux.py compares the GPU path
with it bit for bit)."""
import numpy as np
import pytest

import miniaero_gb300 as ma
import oracle
from tests.golden.make_golden import CASES, options


def cell_flux(o):
    c = o.copy()
    c.gather = ma._lib.MA_GATHER_CELL_FLUX
    return c


@pytest.mark.parametrize("case", sorted(CASES))
def test_cell_flux_order_within_rounding_of_atomics_order(case):
    o = options(case)
    o.ntimesteps = 60
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    a = oracle.solve(md, o, U0)
    b = oracle.solve(md, cell_flux(o), U0)
    assert not np.array_equal(a, b) or case == "sod_serial"  # another summation order
    for k in (0, 4):
        assert np.max(np.abs(a[:, k] - b[:, k])) <= 1e-12 * np.max(np.abs(a[:, k]))
    mom = np.max(np.abs(a[:, 1:4]))
    assert np.max(np.abs(a[:, 1:4] - b[:, 1:4])) <= 1e-12 * mom


def test_cell_flux_threads_do_not_change_bits():
    o = cell_flux(options("flatplate_serial"))
    o.ntimesteps = 20
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    st = oracle.Stepper(md, o, U0, nthreads=4)
    st.step(20)
    U4 = st.state()
    st.close()
    assert np.array_equal(U4, oracle.solve(md, o, U0))


def test_input_file_selects_gather(tmp_path):
    p = tmp_path / "miniaero.inp"
    p.write_text("1\n2.0 0.002 1.0 0\n16 32 2\n10\n3e-8\n0\n2\n1\n1\ngather cell_flux\n")
    assert ma.Options.read_options_file(p).gather == ma._lib.MA_GATHER_CELL_FLUX
    p.write_text("1\n2.0 0.002 1.0 0\n16 32 2\n10\n3e-8\n0\n2\n1\n1\ngather sideways\n")
    with pytest.raises(ma.MiniaeroError):
        ma.Options.read_options_file(p)
    assert ma.Options().gather == ma._lib.MA_GATHER_ATOMICS


def test_host_mesh_carries_slots():
    o = options("ramp_serial")
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    fi = md.internal.flux_index
    assert fi.shape == (md.internal.nfaces, 2) and fi.min() >= 0 and fi.max() <= 5
    # Every cell's six slots are taken exactly once over all face sets.
    seen = np.zeros((md.ncells, 6), np.int32)
    np.add.at(seen, (md.internal.conn[:, 0], fi[:, 0]), 1)
    np.add.at(seen, (md.internal.conn[:, 1], fi[:, 1]), 1)
    for b in md.bc:
        np.add.at(seen, (b.conn[:, 0], b.flux_index[:, 0]), 1)
    assert np.all(seen == 1)
