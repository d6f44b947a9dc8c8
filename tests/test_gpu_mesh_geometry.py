"""Mesh geometry computed on the device (ma_host_mesh_build_ex with
MA_HOST_MESH_DEVICE_GEOMETRY): face centroids, area vectors, tangents and
binormals, cell volumes and centroids must be bit-identical to the host
generator's, on axis-aligned boxes, the ramp (non-orthogonal faces) and odd
sizes; the reference cases' mesh digests must be the committed ones."""
import numpy as np
import pytest

import miniaero_gb300 as ma
from tests.golden.make_golden import CASES, mesh_digest, options

pytestmark = pytest.mark.gpu


def both(o):
    pm = ma.Parallel3DMesh.from_options(o)
    return pm.fill_mesh_data(), pm.fill_mesh_data(device_geometry=True)


def assert_same(h, d):
    assert h.ncells == d.ncells
    assert np.array_equal(h.cell_volumes.view(np.uint64), d.cell_volumes.view(np.uint64))
    assert np.array_equal(h.cell_coords.view(np.uint64), d.cell_coords.view(np.uint64))
    for a, b in zip([h.internal] + list(h.bc), [d.internal] + list(d.bc)):
        for name in ("coords", "normal", "tangent", "binormal"):
            assert np.array_equal(getattr(a, name).view(np.uint64), getattr(b, name).view(np.uint64)), name
        for name in ("conn", "permutation", "flux_index"):
            assert np.array_equal(getattr(a, name), getattr(b, name)), name
    assert mesh_digest(h) == mesh_digest(d)


@pytest.mark.parametrize("case", sorted(CASES))
def test_reference_cases_geometry_bit_identical(has_gpu, case):
    import os
    h, d = both(options(case))
    assert_same(h, d)
    golden = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_cases.npz"))
    assert mesh_digest(d) == str(golden[case + "_mesh_sha256"])


@pytest.mark.parametrize("pt,dims,lens,angle", [
    (0, (1, 1, 1), (1.0, 1.0, 1.0), 0.0),
    (1, (5, 3, 7), (2.0, 0.5, 0.5), 0.0),
    (2, (33, 17, 5), (2.0, 2.0, 1.0), 30.0),
    (2, (24, 40, 3), (2.0, 2.0, 1.0), 12.5),
    (0, (96, 64, 64), (1.0, 0.5, 0.5), 0.0),
])
def test_boxes_and_ramps_geometry_bit_identical(has_gpu, pt, dims, lens, angle):
    o = ma.Options(problem_type=pt, nx=dims[0], ny=dims[1], nz=dims[2], lx=lens[0], ly=lens[1], lz=lens[2],
                   angle=angle)
    h, d = both(o)
    assert_same(h, d)
