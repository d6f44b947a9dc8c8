"""The oracle against the reference itself, bit for bit.

oracle/_ref holds the reference's own sources, unmodified, compiled against
the project's Kokkos stand-in (oracle/build_ref.py) in its two reduction
builds: -DATOMICS_FLUX (kokkos/Makefile:17) and -DCELL_FLUX
(kokkos/Flux.h:172-178). tests/golden/reference_build.json holds that build's
digests of the final state and last-stage residual on the reference's test
inputs (tests/golden/make_reference_digests.py).

Without the reference tree these tests tie the committed oracle fixtures and a
fresh oracle run to the reference build's digests; with it (the development
container) they also rebuild and rerun the reference and compare every array
it kept: final state, residual, cell centroids and volumes, and each face
set's connectivity, permutation and geometry.
"""
import json
import os

import numpy as np
import pytest

import miniaero_gb300 as ma
import oracle
from oracle import ref
from tests.golden.make_golden import CASES, options

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASE_DIRS = {"sod_serial": "3D_Sod_Serial", "ramp_serial": "Ramp_Serial", "flatplate_serial": "FlatPlate_Serial"}


@pytest.fixture(scope="module")
def digests():
    with open(os.path.join(GOLDEN, "reference_build.json")) as f:
        return json.load(f)["cases"]


@pytest.fixture(scope="module")
def fixtures():
    return np.load(os.path.join(GOLDEN, "reference_cases.npz"))


def oracle_run(case, cell_flux=False):
    o = options(case)
    if cell_flux:
        o.gather = ma._lib.MA_GATHER_CELL_FLUX
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U, R = oracle.solve(md, o, ma.initial_state(md, o), return_residual=True)
    return md, U, R


@pytest.mark.parametrize("case", sorted(CASES))
def test_committed_oracle_states_are_the_reference_bits(digests, fixtures, case):
    """The fixtures the GPU tests compare against hold the reference's bits."""
    assert ref.state_digest(fixtures[case + "_U"]) == digests[case]["atomics"]["state_sha256"]


@pytest.mark.parametrize("case", ["sod_serial", "flatplate_serial", "ramp_serial"])
@pytest.mark.parametrize("build", ["atomics", "cell_flux"])
def test_oracle_state_and_residual_match_reference_digests(digests, case, build):
    _, U, R = oracle_run(case, cell_flux=(build == "cell_flux"))
    assert ref.state_digest(U) == digests[case][build]["state_sha256"]
    assert ref.state_digest(R) == digests[case][build]["residual_sha256"]


def _face_sets(md):
    return [md.internal] + list(md.bc)


@pytest.mark.parametrize("case", ["sod_serial", "flatplate_serial", "ramp_serial"])
@pytest.mark.parametrize("build,variant", [("atomics", "miniaero_ref_serial"),
                                           ("cell_flux", "miniaero_ref_serial_cellflux")])
def test_reference_build_live(reference_dir, case, build, variant):
    """Rebuilds and reruns the reference; every array it kept equals ours."""
    with open(os.path.join(reference_dir, "tests", CASE_DIRS[case], "miniaero.inp")) as f:
        arrays, _, _ = ref.run(f.read(), variant=variant)
    md, U, R = oracle_run(case, cell_flux=(build == "cell_flux"))
    assert np.array_equal(arrays["solution_n"][0].view(np.uint64), U.view(np.uint64))
    assert np.array_equal(arrays["residual"][0].view(np.uint64), R.view(np.uint64))
    assert np.array_equal(arrays["cell_coordinates"][0], md.cell_coords)
    assert np.array_equal(arrays["cell_volumes"][0], md.cell_volumes)
    # Face sets: the reference allocates the internal set first, then its
    # boundary sets; each of ours equals one of the reference's (same size,
    # same bits), and every one is matched once.
    theirs = list(zip(arrays["face_cell_conn"], arrays["cell_permute_vector"], arrays["coordinates"],
                      arrays["face_normal"], arrays["face_tangent"], arrays["face_binormal"]))
    assert len(theirs) == len(_face_sets(md))
    used = set()
    for fs in _face_sets(md):
        mine = (fs.conn, fs.permutation, fs.coords, fs.normal, fs.tangent, fs.binormal)
        hit = [i for i, t in enumerate(theirs) if i not in used and all(
            a.shape == b.shape and np.array_equal(a, b) for a, b in zip(t, mine))]
        assert hit, "face set %s has no bit-identical counterpart in the reference" % fs.name
        used.add(hit[0])


def test_reference_build_openmp_threads(reference_dir):
    """The timed OpenMP build (-O3, compiler-default contraction): on one
    thread it gives the serial bits; on four its atomics sum in thread order
    and the flat plate's 400 steps amplify that round-off to about 1e-8 of
    each variable's scale (the reference's own golden files carry 6 digits)."""
    with open(os.path.join(reference_dir, "tests", "FlatPlate_Serial", "miniaero.inp")) as f:
        text = f.read()
    a, _, _ = ref.run(text, variant="miniaero_ref_serial")
    A = a["solution_n"][0]
    scale = np.abs(A).max(axis=0)
    scale[1:4] = scale[1:4].max()
    one, _, _ = ref.run(text, variant="miniaero_ref_openmp", env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert np.array_equal(one["solution_n"][0], A)
    four, _, _ = ref.run(text, variant="miniaero_ref_openmp", env=dict(os.environ, OMP_NUM_THREADS="4"))
    assert np.max(np.abs(four["solution_n"][0] - A) / scale) < 1e-7
