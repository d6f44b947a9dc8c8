"""Host mesh generation: ordering primitives and geometric invariants (CPU)."""
import ctypes
import subprocess
import sys

import numpy as np
import pytest

import miniaero_gb300 as ma
from miniaero_gb300 import _lib


def glibc_rand(seed, n):
    out = np.empty(n, np.int32)
    _lib.check(_lib.lib().ma_debug_glibc_rand(seed, n, _lib.i32p(out)))
    return out


def binsort(keys):
    keys = np.ascontiguousarray(keys, np.int32)
    out = np.empty_like(keys)
    _lib.check(_lib.lib().ma_debug_binsort(_lib.i32p(keys), len(keys), _lib.i32p(out)))
    return out


@pytest.mark.parametrize("seed", [1, 0, 12345])
def test_glibc_rand_matches_libc(seed):
    """The restated generator equals the C library's rand() in a fresh process."""
    if not sys.platform.startswith("linux"):
        pytest.skip("glibc only")
    code = ("import ctypes; c = ctypes.CDLL('libc.so.6'); c.srand(%d); "
            "print(' '.join(str(c.rand()) for _ in range(2000)))" % seed)
    libc = [int(x) for x in subprocess.check_output([sys.executable, "-c", code], text=True).split()]
    assert glibc_rand(seed, 2000).tolist() == libc


def test_glibc_rand_default_seed_is_one():
    code = ("import ctypes; c = ctypes.CDLL('libc.so.6'); "
            "print(' '.join(str(c.rand()) for _ in range(50)))")
    libc = [int(x) for x in subprocess.check_output([sys.executable, "-c", code], text=True).split()]
    assert glibc_rand(1, 50).tolist() == libc


def test_binsort_sorts_by_key_and_is_permutation():
    rng = np.random.default_rng(0)
    for n in (1, 2, 3, 10, 1000, 5001):
        keys = rng.integers(0, max(1, n // 3), n).astype(np.int32)
        p = binsort(keys)
        assert sorted(p.tolist()) == list(range(n))
        assert np.all(np.diff(keys[p]) >= 0)


def test_binsort_tie_order_bubble_semantics():
    """Within a bin, the bubble pass swaps equal keys: a run of equal keys ends reversed."""
    p = binsort(np.array([5, 5, 5, 5], np.int32))
    assert p.tolist() == [3, 2, 1, 0]
    # two bins (n/2 = 2 bins of width 1.5 over [0, 3]); keys in each bin reordered
    keys = np.array([0, 3, 0, 3], np.int32)
    p = binsort(keys)
    assert np.all(np.diff(keys[p]) >= 0)


def build(nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, pt=0, angle=0.0):
    return ma.Parallel3DMesh(nx, ny, nz, lx, ly, lz, pt, angle).fill_mesh_data()


@pytest.mark.parametrize("dims", [(1, 1, 1), (4, 3, 2), (8, 8, 8), (16, 4, 4)])
def test_face_counts_and_connectivity(dims):
    nx, ny, nz = dims
    md = build(nx, ny, nz, 2.0, 1.0, 0.5)
    C = nx * ny * nz
    assert md.ncells == C
    assert md.internal.nfaces == (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1)
    sides = [b.nfaces for b in md.bc]
    assert sides == [nx * nz, nx * nz, nx * ny, nx * ny, ny * nz, ny * nz]
    counts = np.zeros(C, int)
    np.add.at(counts, md.internal.conn.ravel(), 1)
    for b in md.bc:
        np.add.at(counts, b.conn[:, 0], 1)
        assert np.all(b.conn[:, 1] == -1)
    assert np.all(counts == 6)
    assert sorted(md.internal.permutation.tolist()) == list(range(md.internal.nfaces))
    keys = md.internal.conn[md.internal.permutation, 0]
    assert np.all(np.diff(keys) >= 0)


def test_volumes_normals_and_closure():
    md = build(6, 5, 4, 2.0, 1.0, 0.5, pt=2, angle=20.0)
    assert np.all(md.cell_volumes > 0)
    # Ramp domain volume: lx*ly*lz minus the wedge under the ramp
    wedge = 0.5 * 1.0 * np.tan(np.radians(20.0)) * 1.0 * 0.5
    assert abs(md.cell_volumes.sum() - (2.0 * 1.0 * 0.5 - wedge)) < 1e-2
    # Area vectors point out of elem1; the sum over each closed cell vanishes.
    closure = np.zeros((md.ncells, 3))
    fi = md.internal
    d = fi.coords - md.cell_coords[fi.conn[:, 0]]
    assert np.all((d * fi.normal).sum(1) > 0)
    np.add.at(closure, fi.conn[:, 0], fi.normal)
    np.add.at(closure, fi.conn[:, 1], -fi.normal)
    for b in md.bc:
        d = b.coords - md.cell_coords[b.conn[:, 0]]
        assert np.all((d * b.normal).sum(1) > 0)
        np.add.at(closure, b.conn[:, 0], b.normal)
    assert np.max(np.abs(closure)) < 1e-12
    # Orthonormal-ish frames: t and b orthogonal to n.
    for fs in [fi] + md.bc:
        assert np.max(np.abs((fs.normal * fs.tangent).sum(1))) < 1e-12
        assert np.max(np.abs((fs.normal * fs.binormal).sum(1))) < 1e-12


def test_bc_map_per_problem_type():
    names = {pt: [b.name for b in build(4, 4, 2, pt=pt).bc] for pt in (0, 1, 2)}
    assert names[0] == ["Tangent", "Tangent", "Tangent", "Tangent", "Extrapolate", "Extrapolate"]
    assert names[1] == ["NoSlip", "Extrapolate", "Tangent", "Tangent", "Extrapolate", "Inflow"]
    assert names[2] == ["Tangent", "Tangent", "Tangent", "Tangent", "Extrapolate", "Inflow"]


def test_bc_override():
    md = ma.Parallel3DMesh(4, 4, 2, 1.0, 1.0, 1.0, 0, 0.0,
                           bc_override=[ma.MA_BC_NOSLIP, -1, -1, -1, ma.MA_BC_INFLOW, -1]).fill_mesh_data()
    assert [b.name for b in md.bc] == ["NoSlip", "Tangent", "Tangent", "Tangent", "Inflow", "Extrapolate"]


def test_mesh_is_deterministic():
    a = build(10, 6, 4)
    b = build(10, 6, 4)
    assert np.array_equal(a.internal.conn, b.internal.conn)
    assert np.array_equal(a.internal.permutation, b.internal.permutation)
    assert a.internal.normal.tobytes() == b.internal.normal.tobytes()


def test_invalid_mesh_sizes_raise():
    with pytest.raises(ma.MiniaeroError):
        build(0, 4, 4)
    with pytest.raises(ma.MiniaeroError):
        ma.Parallel3DMesh(4, 4, 4, -1.0, 1.0, 1.0, 0).fill_mesh_data()


def test_initial_states():
    o = ma.Options(nx=8, ny=2, nz=2, lx=1.0, ly=0.1, lz=0.1, problem_type=0)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U = ma.initial_state(md, o)
    left = md.cell_coords[:, 0] < 0.5
    assert np.allclose(U[left, 0], 68947.57 / (287.05 * 288.889))
    o.ic = ma.MA_IC_SOD
    U = ma.initial_state(md, o)
    assert np.allclose(U[left, 0], 1.0) and np.allclose(U[~left, 0], 0.125)
    assert np.allclose(U[left, 4], 1.0 / 0.4) and np.allclose(U[~left, 4], 0.1 / 0.4)
    o.ic = ma.MA_IC_CONSTANT
    U = ma.initial_state(md, o)
    assert np.allclose(U, np.array(o.inflow_state)[None, :])
