"""Batched multi-mesh solver on the GPU: each member must equal the same
solve run alone (bit for bit, both precisions), through membership changes,
launch-shape changes and the autotuner."""
import numpy as np
import pytest

import miniaero_gb300 as ma
import oracle

pytestmark = pytest.mark.gpu


def sod_options(precision=ma.MA_PREC_FP64, second=1, viscous=1):
    return ma.Options(problem_type=0, lx=1.0, ly=0.5, lz=0.5, second_order_space=second, viscous=viscous,
                      viscosity_model=ma.MA_VISC_CONSTANT, mu=1.8e-5, prandtl=0.72, ic=ma.MA_IC_SOD, cfl=0.5,
                      precision=precision)


def member(o, dims, ratio_rho, ratio_p):
    m = o.copy()
    m.nx, m.ny, m.nz = dims
    m.sod_left = [0.125 * ratio_rho, 0.1 * ratio_p]
    md = ma.Parallel3DMesh.from_options(m).fill_mesh_data()
    return m, md, ma.initial_state(md, m)


def single(md, m, U0, steps, dt):
    s = ma.TimeSolverExplicitRK4(md, m)
    s.set_state(U0)
    s.dt = dt
    s.step(steps)
    s.synchronize()
    U = s.get_state()
    s.close()
    return U


@pytest.mark.parametrize("precision", [ma.MA_PREC_FP64, ma.MA_PREC_MIXED])
def test_batch_members_equal_single_solves(has_gpu, precision):
    o = sod_options(precision)
    dims = [(12, 6, 4), (20, 3, 5), (7, 7, 7), (16, 8, 2), (1, 1, 1)]
    rng = np.random.default_rng(0)
    cases = [member(o, d, rng.uniform(2, 20), rng.uniform(2, 20)) for d in dims]
    b = ma.Batch(o, capacity=16, budget_bytes=1 << 30)
    ids = []
    meshes = []
    for m, md, U0 in cases:
        dm = ma.DeviceMesh(md)
        meshes.append(dm)
        ids.append(b.add(dm, U0))
    b.step(6)
    b.synchronize()
    for (m, md, U0), i in zip(cases, ids):
        ref = single(md, m, U0, 6, b.member_dt(i))
        assert np.array_equal(b.get_state(i), ref)
        if precision == ma.MA_PREC_FP64:
            assert np.array_equal(ref, oracle.solve(md, m, U0, nsteps=6, dt=b.member_dt(i)))
    b.close()


def test_batch_membership_changes_and_launch_shapes(has_gpu):
    o = sod_options()
    rng = np.random.default_rng(1)
    cases = [member(o, d, rng.uniform(2, 20), rng.uniform(2, 20)) for d in [(10, 4, 4), (6, 6, 6), (14, 2, 3)]]
    b = ma.Batch(o, capacity=8, budget_bytes=1 << 30)
    dms = [ma.DeviceMesh(md) for _, md, _ in cases]
    a = b.add(dms[0], cases[0][2])
    c = b.add(dms[1], cases[1][2])
    b.step(3)
    b.remove(c)                         # leaves mid-run
    d = b.add(dms[2], cases[2][2])      # joins mid-run
    b.set_launch([64, 256, 32, 128], [152, 304, 7, 1000])
    b.step(4)
    b.synchronize()
    assert b.member_steps(a) == 7 and b.member_steps(d) == 4
    m0, md0, U00 = cases[0]
    assert np.array_equal(b.get_state(a), single(md0, m0, U00, 7, b.member_dt(a)))
    m2, md2, U02 = cases[2]
    assert np.array_equal(b.get_state(d), single(md2, m2, U02, 4, b.member_dt(d)))
    with pytest.raises(ma.MiniaeroError):
        b.get_state(c)
    b.close()


def test_batch_autotune_preserves_results(has_gpu):
    o = sod_options()
    rng = np.random.default_rng(2)
    cases = [member(o, d, rng.uniform(2, 20), rng.uniform(2, 20)) for d in [(24, 12, 8), (16, 16, 16)]]
    b = ma.Batch(o, capacity=4, budget_bytes=1 << 30)
    ids = [b.add(ma.DeviceMesh(md), U0) for _, md, U0 in cases]
    best = b.autotune(reps=2)
    assert np.all(best > 0)
    b.step(5)
    b.synchronize()
    for (m, md, U0), i in zip(cases, ids):
        assert np.array_equal(b.get_state(i), single(md, m, U0, 5, b.member_dt(i)))
    b.close()


def test_batch_budget_is_enforced(has_gpu):
    o = sod_options()
    m, md, U0 = member(o, (16, 16, 16), 8.0, 10.0)
    dm = ma.DeviceMesh(md)
    probe = ma.Batch(o, capacity=4, budget_bytes=1 << 30)
    need = probe.member_bytes(dm)
    probe.close()
    b = ma.Batch(o, capacity=4, budget_bytes=2 * need + need // 2)
    b.add(dm, U0)
    b.add(dm, U0)
    with pytest.raises(ma.MiniaeroError) as e:
        b.add(dm, U0)
    assert e.value.status == 4  # MA_EBUDGET
    assert b.size == 2 and b.device_bytes == 2 * need
    b.close()


def test_batch_profile_steps_equal_graph_steps(has_gpu):
    """Kernel-by-kernel profiled steps advance members to the same bits as
    the graph-launched step, and count one launch per kind per stage."""
    o = sod_options()
    cases = [member(o, d, 4.0, 6.0) for d in [(10, 6, 4), (6, 5, 7)]]
    out = []
    for profiled in (False, True):
        b = ma.Batch(o, capacity=4, budget_bytes=1 << 30)
        ids = [b.add(ma.DeviceMesh(md), U0) for (m, md, U0) in cases]
        if profiled:
            prof = b.profile_steps(3)
            assert set(prof) == {"sweep_gradient_limiter", "internal_face_flux", "boundary_face_flux",
                                 "residual_rk_update"}
            assert all(n == 12 and ms > 0.0 for ms, n in prof.values())
        else:
            b.step(3)
        b.synchronize()
        assert all(b.member_steps(i) == 3 for i in ids)
        out.append([b.get_state(i) for i in ids])
        b.close()
    for a, c in zip(*out):
        assert np.array_equal(a, c)


@pytest.mark.parametrize("precision,second,viscous,limiter", [
    (ma.MA_PREC_FP64, 1, 1, ma.MA_LIMITER_VENKAT), (ma.MA_PREC_MIXED, 1, 1, ma.MA_LIMITER_VENKAT),
    (ma.MA_PREC_FP64, 1, 1, ma.MA_LIMITER_VANALBADA), (ma.MA_PREC_FP64, 0, 0, ma.MA_LIMITER_VENKAT),
    (ma.MA_PREC_FP64_FMA, 1, 1, ma.MA_LIMITER_VENKAT)])
def test_single_launch_steps_equal_single_solves(has_gpu, precision, second, viscous, limiter):
    """ma_batch_set_single_launch: a whole ma_batch_step (several RK4 steps,
    every member) as one cooperative launch gives each member the bits of
    its solve alone, for uneven members, across calls and after membership
    changes."""
    o = sod_options(precision, second, viscous)
    o.limiter = limiter

    def same(a, ref):
        if precision != ma.MA_PREC_FP64_FMA:
            return np.array_equal(a, ref)
        # The contracted form is compiled per kernel; fused operations may be
        # chosen differently in the one-launch kernel than in the per-kind ones.
        scale = np.abs(ref).max(axis=0)
        scale[1:4] = scale[1:4].max()
        return bool(np.all(np.abs(a - ref).max(axis=0) <= 1e-11 * scale))

    dims = [(12, 6, 4), (20, 3, 5), (7, 7, 7), (33, 9, 5), (1, 1, 1), (48, 16, 16)]
    rng = np.random.default_rng(1)
    cases = [member(o, d, rng.uniform(2, 20), rng.uniform(2, 20)) for d in dims]
    b = ma.Batch(o, capacity=16, budget_bytes=1 << 30)
    grid = b.set_single_launch(256)
    assert grid >= 152
    meshes = [ma.DeviceMesh(md) for _, md, _ in cases]
    ids = [b.add(dm, U0) for dm, (_, _, U0) in zip(meshes, cases)]
    b.step(5)
    b.step(2)
    b.synchronize()
    for (m, md, U0), i in zip(cases, ids):
        assert same(b.get_state(i), single(md, m, U0, 7, b.member_dt(i)))
    # A member leaves and another joins: the next single launch covers the new set.
    b.remove(ids[2])
    extra = member(o, (9, 11, 3), 5.0, 7.0)
    dx = ma.DeviceMesh(extra[1])
    ix = b.add(dx, extra[2])
    b.step(3)
    b.synchronize()
    assert same(b.get_state(ix), single(extra[1], extra[0], extra[2], 3, b.member_dt(ix)))
    assert same(b.get_state(ids[0]), single(cases[0][1], cases[0][0], cases[0][2], 10, b.member_dt(ids[0])))
    # Back to per-kind launches: same bits.
    b.set_single_launch(0)
    b.step(1)
    b.synchronize()
    assert same(b.get_state(ix), single(extra[1], extra[0], extra[2], 4, b.member_dt(ix)))
    b.close()
    for dm in meshes + [dx]:
        dm.close()


def test_grid_barrier_wait_runs_out_and_reports(has_gpu):
    """The single-launch step's grid barrier bounds every wait: a launch in
    which one block never reaches the barrier makes the other give up after
    the limit, leave the error word set and return; the device stays usable
    (a batch steps afterwards with the bits of its solves alone)."""
    import ctypes
    from miniaero_gb300._lib import check, lib
    passed, err, waited = ctypes.c_int32(-1), ctypes.c_int32(-1), ctypes.c_double(0.0)
    check(lib().ma_debug_barrier_timeout(0.05, ctypes.byref(passed), ctypes.byref(err), ctypes.byref(waited)))
    assert passed.value == 0 and err.value == 1
    assert 0.05 <= waited.value < 5.0
    o = sod_options(ma.MA_PREC_FP64)
    m, md, U0 = member(o, (10, 6, 4), 4.0, 3.0)
    dm = ma.DeviceMesh(md)
    b = ma.Batch(o, capacity=2)
    b.set_single_launch(128)
    i = b.add(dm, U0)
    b.step(3)
    b.synchronize()
    assert np.array_equal(b.get_state(i), single(md, m, U0, 3, b.member_dt(i)))
    b.close()
    dm.close()
