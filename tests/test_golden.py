"""Committed golden fixtures (tests/golden/reference_cases.npz, made by
tests/golden/make_golden.py): the host mesh digests and the final states of
the reference's three serial cases. CPU tests re-derive them with the host
mesh generator and the oracle; the GPU test compares the CUDA path to them
bit for bit (no reference tree needed)."""
import os

import numpy as np
import pytest

import miniaero_gb300 as ma
import oracle
from tests.golden.make_golden import CASES, mesh_digest, options

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_cases.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(FIXTURE)


@pytest.mark.parametrize("case", sorted(CASES))
def test_host_mesh_matches_fixture(golden, case):
    md = ma.Parallel3DMesh.from_options(options(case)).fill_mesh_data()
    assert mesh_digest(md) == str(golden[case + "_mesh_sha256"])


@pytest.mark.parametrize("case", ["sod_serial", "flatplate_serial"])
def test_oracle_matches_fixture(golden, case):
    o = options(case)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U = oracle.solve(md, o, ma.initial_state(md, o))
    assert np.array_equal(U, golden[case + "_U"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_matches_fixture(has_gpu, golden, case):
    o = options(case)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    with ma.TimeSolverExplicitRK4(md, o) as s:
        U = s.solve()
    ref = golden[case + "_U"]
    assert np.array_equal(U, ref), "max |diff| %g" % float(np.max(np.abs(U - ref)))
