"""Serving loop on the GPU: requests that arrive while others run are batched
with them (continuous batching), and every result equals the same solve run
alone (bit for bit in both precisions; the FP64 form also equals the oracle)."""
import numpy as np
import pytest

import miniaero_gb300 as ma
import oracle

pytestmark = pytest.mark.gpu


def inflow(mach, T=300.0, p=1e5):
    R, g = 287.05, 1.4
    rho = p / (R * T)
    u = mach * (g * R * T) ** 0.5
    return [rho, rho * u, 0.0, 0.0, rho * (R / (g - 1.0) * T + 0.5 * u * u)]


def physics(precision):
    return ma.Options(problem_type=1, second_order_space=1, viscous=1, limiter=ma.MA_LIMITER_VANALBADA,
                      viscosity_model=ma.MA_VISC_CONSTANT, mu=1.8e-5, prandtl=0.72, precision=precision, cfl=0.5)


def alone(phys, n, mach, steps):
    o = phys.copy()
    o.nx = o.ny = o.nz = n
    o.lx, o.ly, o.lz = 2.0, 0.5, 0.5
    o.ic = ma.MA_IC_CONSTANT
    o.inflow_state = inflow(mach)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    s = ma.TimeSolverExplicitRK4(md, o)
    s.set_state(U0)
    s.step(steps)
    s.synchronize()
    U, dt = s.get_state(), s.dt
    s.close()
    return U, dt, md, o, U0


@pytest.mark.parametrize("precision", [ma.MA_PREC_MIXED, ma.MA_PREC_FP64])
def test_continuous_batching_results_equal_alone(has_gpu, precision):
    phys = physics(precision)
    srv = ma.Server(phys, budget_bytes=4 << 30, tick_steps=5, capacity=16, thread=False)
    jobs = [(8, 0.1, 20), (12, 0.35, 15), (16, 0.6, 25), (8, 0.5, 10), (12, 0.2, 30)]
    ids = {}
    # Two arrive first; the rest arrive while those are running.
    for j in jobs[:2]:
        ids[j] = srv.submit(ma.Server.request(j[0], j[0], j[0], 2.0, 0.5, 0.5, inflow(j[1]), j[2], keep_result=True))
    assert srv.poll()
    for j in jobs[2:]:
        ids[j] = srv.submit(ma.Server.request(j[0], j[0], j[0], 2.0, 0.5, 0.5, inflow(j[1]), j[2], keep_result=True))
    while srv.poll():
        pass
    st = srv.stats()
    assert st["completed"] == len(jobs) and st["peak_running"] >= 3
    for j, rid in ids.items():
        info = srv.query(rid)
        assert info.state == srv.DONE and info.steps_done == j[2]
        U = srv.result(rid)
        ref, dt, md, o, U0 = alone(phys, j[0], j[1], j[2])
        assert np.array_equal(U, ref), j
        if precision == ma.MA_PREC_FP64 and j[0] <= 12:
            assert np.array_equal(U, oracle.solve(md, o, U0, nsteps=j[2], dt=dt))
    srv.close()


def test_threaded_server_with_budget_pressure(has_gpu):
    phys = physics(ma.MA_PREC_MIXED)
    probe = ma.Server(phys, budget_bytes=4 << 30, tick_steps=5, capacity=16, thread=False)
    probe.close()
    srv = ma.Server(phys, budget_bytes=8 << 20, tick_steps=5, capacity=16, thread=True)
    rids = [srv.submit(ma.Server.request(16, 16, 16, 2.0, 0.5, 0.5, inflow(0.3), 20, keep_result=True))
            for _ in range(6)]
    for r in rids:
        assert srv.wait(r, timeout=120.0).state == srv.DONE
    st = srv.stats()
    assert st["peak_bytes"] <= 8 << 20 and st["completed"] == 6
    ref = alone(phys, 16, 0.3, 20)[0]
    for r in rids:
        assert np.array_equal(srv.result(r), ref)
    srv.close()


def test_threaded_server_builds_new_meshes_beside_running_requests(has_gpu):
    """With its scheduler thread the server builds each new mesh shape on a
    mesh thread of its own: requests of five different sizes, submitted while
    a first one runs, all finish with the bits of their solves alone."""
    phys = physics(ma.MA_PREC_FP64)
    srv = ma.Server(phys, budget_bytes=2 << 30, tick_steps=5, capacity=16, thread=True)
    jobs = [(16, 0.3, 40), (10, 0.2, 15), (14, 0.45, 20), (18, 0.55, 10), (9, 0.1, 25), (12, 0.35, 5)]
    rids = {jobs[0]: srv.submit(ma.Server.request(16, 16, 16, 2.0, 0.5, 0.5, inflow(0.3), 40, keep_result=True))}
    for j in jobs[1:]:
        rids[j] = srv.submit(ma.Server.request(j[0], j[0], j[0], 2.0, 0.5, 0.5, inflow(j[1]), j[2], keep_result=True))
    for r in rids.values():
        assert srv.wait(r, timeout=300.0).state == srv.DONE
    st = srv.stats()
    assert st["completed"] == len(jobs) and st["cached_meshes"] == len(jobs)
    for j, r in rids.items():
        assert np.array_equal(srv.result(r), alone(phys, j[0], j[1], j[2])[0]), j
    srv.close()
