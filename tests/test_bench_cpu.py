"""bench.py's CPU baseline sample on the host: the oracle port timed on
whole-mesh steps. On a small mesh it takes as many steps as fill its time
budget (not a fixed handful), after re-estimating the step time over 10
untimed steps past the first, whose time includes the thread pool's start-up."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
import miniaero_gb300 as ma  # noqa: E402
import oracle  # noqa: E402


def test_cpu_baseline_sample_fills_its_budget_on_a_small_mesh():
    o = ma.Options(problem_type=0, lx=1.0, ly=0.1, lz=0.1, nx=16, ny=4, nz=4, second_order_space=0, viscous=0,
                   ic=1, sod_left=[1.0, 1.0], sod_right=[0.125, 0.1], dt=1e-5, ntimesteps=10)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    r = bench.cpu_baseline_sample(ma, oracle, md, o, U0, 1e-5, seconds=0.5, nthreads=2)
    assert r["kind"] == "port" and r["cores"] == 2 and r["unit"] == "Mcell-stage/s"
    assert r["value"] > 0.0
    words = r["sample"].split()
    assert int(words[0]) > 20, r["sample"]
    assert "of the full %d-cell mesh after 11 untimed steps" % md.ncells in r["sample"]
