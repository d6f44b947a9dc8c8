"""Checkpoint files and run controls on the host (no GPU): round trips in both
layouts, the header, detection of corrupt, truncated and foreign files,
atomic replacement, the mesh hash, and the run-control lines of an input
file (which ma_options_read skips)."""
import os

import numpy as np
import pytest

import miniaero_gb300 as ma
from miniaero_gb300 import _lib


def small_mesh(nx=8, lx=1.0):
    o = ma.Options(problem_type=0, nx=nx, ny=4, nz=4, lx=lx)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    return o, md


def state(md, seed=0):
    return np.random.default_rng(seed).standard_normal((md.ncells, 5))


def test_round_trip_and_header(tmp_path):
    o, md = small_mesh()
    U = state(md)
    p = tmp_path / "a.ckpt"
    h = ma.mesh_hash(md)
    ma.checkpoint_write(p, U, 17, 1.7e-4, 1e-5, h)
    info, V = ma.checkpoint_read(p)
    assert np.array_equal(U, V)
    assert info == {"ncells": md.ncells, "steps_done": 17, "time": 1.7e-4, "dt": 1e-5, "mesh_hash": h}
    assert os.path.getsize(p) == 64 + 5 * 8 * md.ncells
    assert sorted(os.listdir(tmp_path)) == ["a.ckpt"]  # no temporary left behind


def test_component_major_layout(tmp_path):
    import ctypes
    _, md = small_mesh()
    U = state(md, 1)
    p = str(tmp_path / "s.ckpt").encode()
    info = _lib.ma_checkpoint_info(md.ncells, 3, 0.0, 1.0, 5)
    soa = np.ascontiguousarray(U.T)
    _lib.check(_lib.lib().ma_checkpoint_write(p, ctypes.byref(info), _lib.f64p(soa), ma.MA_LAYOUT_SOA))
    _, V = ma.checkpoint_read(p.decode())
    assert np.array_equal(V, U)
    out = np.empty((5, md.ncells))
    _lib.check(_lib.lib().ma_checkpoint_read(p, ctypes.byref(info), _lib.f64p(out), md.ncells, ma.MA_LAYOUT_SOA))
    assert np.array_equal(out, soa)


def test_overwrite_replaces_file(tmp_path):
    _, md = small_mesh()
    p = tmp_path / "a.ckpt"
    ma.checkpoint_write(p, state(md, 1), 1, 0.1, 0.1, 1)
    ma.checkpoint_write(p, state(md, 2), 2, 0.2, 0.1, 1)
    info, V = ma.checkpoint_read(p)
    assert info["steps_done"] == 2 and np.array_equal(V, state(md, 2))


def test_corrupt_truncated_and_foreign_files(tmp_path):
    _, md = small_mesh()
    p = tmp_path / "a.ckpt"
    ma.checkpoint_write(p, state(md), 1, 0.0, 1.0, 9)
    raw = bytearray(p.read_bytes())
    bad = tmp_path / "bad.ckpt"
    raw2 = bytearray(raw)
    raw2[64 + 123] ^= 0x10  # one bit of the state
    bad.write_bytes(bytes(raw2))
    with pytest.raises(ma.MiniaeroError, match="checksum") as e:
        ma.checkpoint_read(bad)
    assert e.value.status == _lib.MA_EIO
    bad.write_bytes(bytes(raw[:-8]))
    with pytest.raises(ma.MiniaeroError, match="truncated") as e:
        ma.checkpoint_read(bad)
    assert e.value.status == _lib.MA_EIO
    bad.write_bytes(b"not a checkpoint at all, just text" * 4)
    with pytest.raises(ma.MiniaeroError, match="not a checkpoint") as e:
        ma.checkpoint_read(bad)
    assert e.value.status == _lib.MA_EINVAL
    with pytest.raises(ma.MiniaeroError) as e:
        ma.checkpoint_read(tmp_path / "missing.ckpt")
    assert e.value.status == _lib.MA_EIO


def test_buffer_too_small(tmp_path):
    import ctypes
    _, md = small_mesh()
    p = tmp_path / "a.ckpt"
    ma.checkpoint_write(p, state(md), 1, 0.0, 1.0, 9)
    info = _lib.ma_checkpoint_info()
    out = np.empty((md.ncells - 1, 5))
    st = _lib.lib().ma_checkpoint_read(str(p).encode(), ctypes.byref(info), _lib.f64p(out), md.ncells - 1,
                                       ma.MA_LAYOUT_AOS)
    assert st == _lib.MA_EINVAL and info.ncells == md.ncells


def test_mesh_hash_identifies_the_mesh():
    _, a = small_mesh()
    _, b = small_mesh()
    _, c = small_mesh(nx=9)
    _, d = small_mesh(lx=1.5)
    assert ma.mesh_hash(a) == ma.mesh_hash(b)
    assert len({ma.mesh_hash(a), ma.mesh_hash(c), ma.mesh_hash(d)}) == 3


def test_run_controls_in_the_input_file(tmp_path):
    p = tmp_path / "miniaero.inp"
    p.write_text("0\n1.0 0.5 0.5 0\n8 4 4\n10\n1e-5\n0\n2\n1\n0\n"
                 "precision mixed\ncheckpoint run.ckpt\ncheckpoint_frequency 5\nrestart old.ckpt\ncfl 0.5\n")
    r = ma.run_options_read(p)
    assert r == {"checkpoint_path": "run.ckpt", "checkpoint_frequency": 5, "restart_path": "old.ckpt"}
    o = ma.Options.read_options_file(p)  # skips the run controls
    assert o.precision == ma.MA_PREC_MIXED and o.cfl == 0.5 and o.ntimesteps == 10
    q = tmp_path / "plain.inp"
    q.write_text("0\n1.0 0.5 0.5 0\n8 4 4\n10\n1e-5\n0\n2\n1\n0\n")
    assert ma.run_options_read(q) == {"checkpoint_path": "", "checkpoint_frequency": 0, "restart_path": ""}
    bad = tmp_path / "bad.inp"
    bad.write_text("0\n1.0 0.5 0.5 0\n8 4 4\n10\n1e-5\n0\n2\n1\n0\ncheckpoint_frequency -3\n")
    with pytest.raises(ma.MiniaeroError):
        ma.run_options_read(bad)
