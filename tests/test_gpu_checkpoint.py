"""Checkpoint and restart on the GPU, and the command-line driver: a run
restarted from a checkpoint gives the bits of the uninterrupted run (both
precision forms, through the Python API and through the CLI), and the CLI's
results.0 equals the committed golden fixtures of the reference's three
serial cases, line for line in the reference's text format."""
import subprocess

import numpy as np
import pytest

import miniaero_gb300 as ma
from tests.golden.make_golden import CASES, options
from tests.test_golden import FIXTURE
from tests.test_oracle_gold import results_lines


def flat_plate(precision):
    o = ma.Options(problem_type=1, lx=2.0, ly=0.002, lz=1.0, nx=16, ny=32, nz=2, ntimesteps=8, dt=3e-8,
                   second_order_space=1, viscous=1, precision=precision)
    return o, ma.Parallel3DMesh.from_options(o).fill_mesh_data()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [ma.MA_PREC_FP64, ma.MA_PREC_MIXED])
def test_restart_equals_uninterrupted_run(has_gpu, tmp_path, precision):
    o, md = flat_plate(precision)
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.init_state()
        s.step(8)
        s.synchronize()
        straight = s.get_state()
    ck = tmp_path / "mid.ckpt"
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.init_state()
        s.step(3)
        s.save_checkpoint(ck)
    with ma.TimeSolverExplicitRK4(md, o) as s:
        assert s.restore_checkpoint(ck) == 3
        s.step(5)
        s.synchronize()
        restarted = s.get_state()
    assert np.array_equal(restarted, straight)


@pytest.mark.gpu
def test_restore_rejects_another_mesh(has_gpu, tmp_path):
    o, md = flat_plate(ma.MA_PREC_FP64)
    ck = tmp_path / "a.ckpt"
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.init_state()
        s.save_checkpoint(ck)
    o2 = o.copy()
    o2.lx = 2.5
    md2 = ma.Parallel3DMesh.from_options(o2).fill_mesh_data()
    with ma.TimeSolverExplicitRK4(md2, o2) as s:
        with pytest.raises(ma.MiniaeroError, match="different mesh"):
            s.restore_checkpoint(ck)


def write_inp(path, case, steps=None, extra=()):
    pt, lx, ly, lz, angle, nx, ny, nz, nsteps, dt, second, visc = CASES[case]
    steps = nsteps if steps is None else steps
    lines = [str(pt), "%r %r %r %r" % (lx, ly, lz, angle), "%d %d %d" % (nx, ny, nz), str(steps), repr(dt),
             "1", "50", str(second), str(visc), *extra]
    path.write_text("\n".join(lines) + "\n")


def run_cli(cwd):
    from miniaero_gb300 import build as b
    r = subprocess.run([b.CLI], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_cli_results_match_fixture(has_gpu, tmp_path, case):
    write_inp(tmp_path / "miniaero.inp", case)
    run_cli(tmp_path)
    got = (tmp_path / "results.0").read_text().splitlines()
    md = ma.Parallel3DMesh.from_options(options(case)).fill_mesh_data()
    golden = np.load(FIXTURE)
    assert got == results_lines(md, golden[case + "_U"])


@pytest.mark.gpu
def test_cli_restart_equals_uninterrupted_run(has_gpu, tmp_path):
    case = "flatplate_serial"
    a, b, c = (tmp_path / d for d in ("a", "b", "c"))
    for d in (a, b, c):
        d.mkdir()
    # Periodic checkpoints every 15 steps, then one at the end (same file).
    write_inp(a / "miniaero.inp", case, steps=40, extra=["checkpoint run.ckpt", "checkpoint_frequency 15"])
    r = run_cli(a)
    assert [ln for ln in r.stdout.splitlines() if "Checkpoint" in ln] == [
        " ... Checkpoint run.ckpt at step %d ..." % n for n in (15, 30, 40)]
    assert ma.checkpoint_read(a / "run.ckpt")[0]["steps_done"] == 40
    # Stop at step 30, restart from there to the case's 400 steps.
    write_inp(b / "miniaero.inp", case, steps=30, extra=["checkpoint mid.ckpt"])
    run_cli(b)
    write_inp(c / "miniaero.inp", case, extra=["restart ../b/mid.ckpt"])
    r = run_cli(c)
    assert "Restarted from ../b/mid.ckpt at step 30" in r.stdout
    straight = tmp_path / "d"
    straight.mkdir()
    write_inp(straight / "miniaero.inp", case)
    run_cli(straight)
    assert (c / "results.0").read_text() == (straight / "results.0").read_text()
