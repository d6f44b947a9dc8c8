"""The CUDA path against the reference's own bits.

tests/golden/reference_build.json holds digests of what the reference
computes (its unmodified sources compiled against the project's Kokkos
stand-in, oracle/_ref) on its serial test inputs and its 32x64x2 flat-plate
input, in both of its reduction builds (-DATOMICS_FLUX, -DCELL_FLUX): the
final conserved state and the last RK stage's residual. The GPU's FP64 path
must give the same SHA-256 for both.

tests/golden/full_size.json holds digests of the state after 2 RK4 steps at
dt from CFL 0.5 on the full benchmark meshes: the reference's own Sod and
flat-plate problems on the 256x128x128 and 512x128x128 meshes (from the
reference build) and the two benchmark configurations exactly (from the
serial oracle, which equals the reference build bit for bit wherever the
reference can express the input).
"""
import json
import os

import numpy as np
import pytest

import miniaero_gb300 as ma
from oracle.ref import state_digest
from tests.golden.make_golden import CASES, options

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
with open(os.path.join(GOLDEN, "reference_build.json")) as _f:
    SMALL = json.load(_f)["cases"]
with open(os.path.join(GOLDEN, "full_size.json")) as _f:
    FULL = json.load(_f)["cases"]


@pytest.mark.parametrize("build", ["atomics", "cell_flux"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_state_and_residual_are_the_reference_bits(has_gpu, case, build):
    o = options(case)
    o.keep_residual = 1
    if build == "cell_flux":
        o.gather = ma._lib.MA_GATHER_CELL_FLUX
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    with ma.TimeSolverExplicitRK4(md, o) as s:
        U = s.solve()
        R = s.get_residual()
    want = SMALL[case][build]
    assert state_digest(U) == want["state_sha256"], "state l2 %s vs %s" % (
        [float(np.linalg.norm(U[:, k])) for k in range(5)], want["state_l2"])
    assert state_digest(R) == want["residual_sha256"]


@pytest.mark.parametrize("name", sorted(FULL))
def test_full_size_state_is_bit_identical(has_gpu, name):
    case = FULL[name]
    o = ma.Options(**case["options"])
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    assert md.ncells == case["cells"]
    assert o.cfl == 0.0 and o.dt == case["dt"]
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.set_state(ma.initial_state(md, o))
        s.step(case["steps"])
        s.synchronize()
        U = s.get_state()
    l2 = [float(np.linalg.norm(U[:, k])) for k in range(5)]
    assert state_digest(U) == case["sha256"], "%s (%s): l2 %s vs %s" % (name, case["source"], l2, case["l2"])
