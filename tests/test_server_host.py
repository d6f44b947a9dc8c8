"""Serving loop scheduling on the host (dry-run mode: sizes and ticks only,
no device work): FIFO admission under the device-memory budget, mesh cache
sharing and eviction, exact step counts, cancellation, bounded waits."""
import time

import pytest

import miniaero_gb300 as ma

PHYS = dict(problem_type=1, second_order_space=1, viscous=1, precision=ma.MA_PREC_MIXED, cfl=0.5)


def server(budget, tick=10, capacity=64, thread=False):
    return ma.Server(ma.Options(**PHYS), budget_bytes=budget, tick_steps=tick, capacity=capacity, thread=thread,
                     dry_run=True)


def req(n, steps=50):
    return ma.Server.request(n, n, n, 2.0, 0.5, 0.5, [1.16, 120.0, 0.0, 0.0, 2.6e5], steps)


def sizes(n, mixed=True):
    C = n ** 3
    F = 3 * (n + 1) * n * n
    w = 4 if mixed else 8
    return C * (80 + 25 * w) + F * 5 * w + 6 * 256, C * 100 + F * 237 + 19 * 256  # member, mesh


def test_fifo_admission_under_budget():
    member, mesh = sizes(32)
    s = server(budget=mesh + 3 * member + member // 2)  # room for 3 members of 32^3
    ids = [s.submit(req(32)) for _ in range(5)]
    assert s.poll()
    st = [s.query(i).state for i in ids]
    assert st == [s.RUNNING] * 3 + [s.QUEUED] * 2
    for _ in range(5):
        s.poll()
    st = [s.query(i).state for i in ids]
    assert st[:3] == [s.DONE] * 3 and st[3:] == [s.RUNNING] * 2
    while s.poll():
        pass
    infos = [s.query(i) for i in ids]
    assert all(i.state == s.DONE and i.steps_done == 50 for i in infos)
    assert all(i.t_submit_ns <= i.t_admit_ns <= i.t_finish_ns for i in infos)
    stats = s.stats()
    assert stats["completed"] == 5 and stats["peak_running"] == 3 and stats["cached_meshes"] == 1
    assert stats["cell_stages"] == 5 * 32 ** 3 * 4 * 50
    s.close()


def test_exact_step_counts_with_uneven_requests():
    s = server(budget=1 << 40, tick=8)
    a = s.submit(req(16, steps=13))
    b = s.submit(req(16, steps=30))
    while s.poll():
        pass
    assert s.query(a).steps_done == 13 and s.query(b).steps_done == 30
    assert s.stats()["ticks"] >= 5
    s.close()


def test_request_larger_than_budget_fails_at_submit():
    member, mesh = sizes(64)
    s = server(budget=member)
    rid = s.submit(req(64))
    info = s.query(rid)
    assert info.state == s.FAILED and info.error == 4  # MA_EBUDGET
    s.close()


def test_mesh_cache_shared_and_evicted():
    m32, mesh32 = sizes(32)
    m48, mesh48 = sizes(48)
    s = server(budget=max(mesh32 + 2 * m32, mesh48 + m48) + 1000)
    a = s.submit(req(32))
    b = s.submit(req(32))
    s.poll()
    assert s.stats()["cached_meshes"] == 1 and s.stats()["running"] == 2
    c = s.submit(req(48))  # needs the 32^3 mesh evicted once both finish
    while s.poll():
        pass
    assert s.query(c).state == s.DONE
    assert s.stats()["cached_meshes"] == 1
    assert s.query(a).state == s.DONE and s.query(b).state == s.DONE
    s.close()


def test_cancel_queued_and_running():
    member, mesh = sizes(32)
    s = server(budget=mesh + member + 100)
    a = s.submit(req(32, steps=100))
    b = s.submit(req(32, steps=100))
    s.poll()
    assert s.query(a).state == s.RUNNING and s.query(b).state == s.QUEUED
    s.cancel(b)
    s.cancel(a)
    assert s.query(a).state == s.CANCELLED and s.query(b).state == s.CANCELLED
    assert s.stats()["bytes_in_use"] == mesh  # member freed, mesh cached
    with pytest.raises(ma.MiniaeroError):
        s.cancel(a)
    c = s.submit(req(32, steps=20))
    while s.poll():
        pass
    assert s.query(c).state == s.DONE
    s.close()


def test_capacity_limits_running_requests():
    s = server(budget=1 << 40, capacity=2)
    ids = [s.submit(req(8, steps=30)) for _ in range(5)]
    s.poll()
    assert sum(s.query(i).state == s.RUNNING for i in ids) == 2
    while s.poll():
        pass
    assert all(s.query(i).state == s.DONE for i in ids)
    s.close()


def test_running_cell_cap_orders_completion():
    s = server(budget=1 << 40)
    s.set_max_running_cells(2 * 16 ** 3)
    ids = [s.submit(req(16, steps=20)) for _ in range(5)]
    s.poll()
    assert [s.query(i).state for i in ids] == [s.RUNNING] * 2 + [s.QUEUED] * 3
    while s.poll():
        pass
    fin = [s.query(i).t_finish_ns for i in ids]
    assert fin[0] <= fin[2] and fin[1] <= fin[3] and fin[3] <= fin[4]
    big = s.submit(req(32, steps=10))  # larger than the cap: runs alone
    while s.poll():
        pass
    assert s.query(big).state == s.DONE
    s.close()


def test_wait_drives_manual_loop_and_times_out():
    s = server(budget=1 << 40)
    a = s.submit(req(8, steps=40))
    assert s.wait(a, timeout=10.0).state == s.DONE
    s.close()
    member, mesh = sizes(32)
    s = server(budget=mesh + member + 10)
    x = s.submit(req(32, steps=10))
    y = s.submit(req(32, steps=10))
    assert s.wait(y, timeout=10.0).state == s.DONE  # runs x to completion first
    assert s.query(x).state == s.DONE
    s.close()


def test_thread_mode_serves_and_bounded_wait():
    s = server(budget=1 << 40, thread=True)
    ids = [s.submit(req(12, steps=30)) for _ in range(8)]
    for i in ids:
        assert s.wait(i, timeout=10.0).state == s.DONE
    st = s.stats()
    assert st["completed"] == 8
    s.close()
    # A request that can never be admitted (budget taken by a running one)
    # makes a short wait time out instead of blocking.
    member, mesh = sizes(32)
    s = server(budget=mesh + member + 10, thread=True)
    a = s.submit(req(32, steps=10 ** 8))
    b = s.submit(req(32, steps=10))
    t0 = time.time()
    with pytest.raises(ma.MiniaeroError) as e:
        s.wait(b, timeout=0.3)
    assert e.value.status == 5 and time.time() - t0 < 5.0  # MA_ETIMEDOUT
    s.cancel(a)
    assert s.wait(b, timeout=10.0).state == s.DONE
    s.close()


def test_launch_shapes_change_only_while_idle():
    s = server(budget=1 << 30)
    s.set_launch([256, 64, 128, 64], [1216, 2432, 2432, 2432])
    with pytest.raises(ma.MiniaeroError):
        s.set_launch([300, 64, 128, 64], [1216, 2432, 2432, 2432])
    rid = s.submit(req(16, steps=30))
    with pytest.raises(ma.MiniaeroError) as e:
        s.set_launch([128] * 4, [1216] * 4)
    assert e.value.status == ma._lib.MA_ESTATE
    while s.poll():
        pass
    assert s.query(rid).state == s.DONE
    s.set_launch([128] * 4, [1216] * 4)
    s.close()


def test_request_beyond_the_index_limit_fails_at_submit():
    """A box with more cells than the device arrays' 32-bit indexing allows
    fails at once (MA_EINVAL), without building its mesh, even when the
    budget would hold it."""
    s = server(budget=1 << 50)
    rid = s.submit(req(524))  # 524^3 = 143,877,824 cells > 143,165,576
    info = s.query(rid)
    assert info.state == s.FAILED and info.error == ma._lib.MA_EINVAL
    ok = s.submit(req(16))
    while s.poll():
        pass
    assert s.query(ok).state == s.DONE
    s.close()
