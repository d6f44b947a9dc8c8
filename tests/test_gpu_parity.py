"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

The plain FP64 form must be bit-identical to the oracle (the reference's
serial arithmetic): the per-cell contribution lists replay the serial
summation order and the FP64 kernels are built without contracted FMAs.
The mixed form is checked against the FP64 oracle with a stated tolerance.
"""
import numpy as np
import pytest

import miniaero_gb300 as ma
import oracle

pytestmark = pytest.mark.gpu

REF_TESTS = {
    # name: (problem_type, (lx, ly, lz, angle), (nx, ny, nz), steps, dt, second, viscous)
    "3D_Sod_Serial": (0, (0.3048, 1.0, 1.0, 0.0), (128, 4, 4), 100, 2e-6, 0, 0),
    "Ramp_Serial": (2, (2.0, 2.0, 1.0, 30.0), (64, 32, 2), 400, 1e-5, 1, 0),
    "FlatPlate_Serial": (1, (2.0, 0.002, 1.0, 0.0), (16, 32, 2), 400, 3e-8, 1, 1),
}


def make_options(pt, lens, dims, steps, dt, second, viscous, **kw):
    lx, ly, lz, angle = lens
    nx, ny, nz = dims
    return ma.Options(problem_type=pt, lx=lx, ly=ly, lz=lz, angle=angle, nx=nx, ny=ny, nz=nz, ntimesteps=steps,
                      dt=dt, second_order_space=second, viscous=viscous, **kw)


def run_gpu(md, o, U0, steps=None):
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.set_state(U0)
        s.step(o.ntimesteps if steps is None else steps)
        s.synchronize()
        return s.get_state()


def assert_bitexact(U, ref):
    bad = np.argwhere(U.view(np.int64) != ref.view(np.int64))
    if bad.size:
        i, k = bad[0]
        raise AssertionError("%d values differ; first at cell %d comp %d: %r vs %r (max |diff| %g)"
                             % (len(bad), i, k, U[i, k], ref[i, k], float(np.max(np.abs(U - ref)))))


def test_device_present(has_gpu):
    assert ma.device_count() >= 1


# ---- operator level ------------------------------------------------------------
def _random_states(rng, n):
    rho = rng.uniform(0.1, 2.0, n)
    vel = rng.normal(0.0, 100.0, (n, 3))
    T = rng.uniform(200.0, 400.0, n)
    return np.column_stack([rho, vel, T])


def _random_frame(rng, n):
    a = rng.normal(size=(n, 3)) * rng.uniform(1e-4, 1.0, (n, 1))
    t = np.cross(a, rng.normal(size=(n, 3)))
    b = np.cross(a, t)
    return a, t, b


def test_op_roe_flux_bitexact(has_gpu):
    rng = np.random.default_rng(1)
    n = 4000
    pl, pr = _random_states(rng, n), _random_states(rng, n)
    pr[: n // 4] = pl[: n // 4]  # equal states: extrapolate boundary case
    a, t, b = _random_frame(rng, n)
    assert_bitexact(ma.roe_flux(pl, pr, a, t, b), oracle.roe_flux(pl, pr, a, t, b))


@pytest.mark.parametrize("model", [ma.MA_VISC_SUTHERLAND, ma.MA_VISC_CONSTANT])
def test_op_viscous_flux_bitexact(has_gpu, model):
    rng = np.random.default_rng(2)
    n = 3000
    g = rng.normal(size=(n, 5, 3)) * 1e3
    p = _random_states(rng, n)
    a = rng.normal(size=(n, 3))
    assert_bitexact(ma.viscous_flux(g, p, a, model, 1.8e-5, 0.72), oracle.viscous_flux(g, p, a, model, 1.8e-5, 0.72))


def test_op_limiters_bitexact(has_gpu):
    rng = np.random.default_rng(3)
    n = 20000
    dumax = np.abs(rng.normal(size=n)) * 10 ** rng.uniform(-8, 2, n)
    dumin = -np.abs(rng.normal(size=n)) * 10 ** rng.uniform(-8, 2, n)
    du = rng.normal(size=n) * 10 ** rng.uniform(-45, 2, n)
    du[:100] = 0.0
    d2 = 10 ** rng.uniform(-8, 0, n)
    assert_bitexact(ma.venkat_limit(dumax, dumin, du, d2)[:, None], oracle.venkat(dumax, dumin, du, d2)[:, None])
    assert_bitexact(ma.vanalbada_limit(dumax, dumin, du)[:, None], oracle.vanalbada(dumax, dumin, du)[:, None])


def test_op_primitives_bitexact(has_gpu):
    rng = np.random.default_rng(4)
    p = _random_states(rng, 5000)
    U = np.column_stack([p[:, 0], p[:, 0] * p[:, 1], p[:, 0] * p[:, 2], p[:, 0] * p[:, 3],
                         p[:, 0] * (717.625 * p[:, 4] + 0.5 * (p[:, 1:4] ** 2).sum(1))])
    assert_bitexact(ma.compute_primitives(U), oracle.primitives(U))


# ---- full solves ------------------------------------------------------------------
@pytest.mark.parametrize("name", sorted(REF_TESTS))
def test_reference_cases_bitexact(has_gpu, name):
    o = make_options(*REF_TESTS[name])
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    assert_bitexact(run_gpu(md, o, U0), oracle.solve(md, o, U0))


def test_sod_baseline_config_bitexact(has_gpu):
    """Sod 128x16x16 on 1.0x0.1x0.1, rho/p 1/1 | 0.125/0.1, first order, dt 1e-5, 200 steps."""
    o = make_options(0, (1.0, 0.1, 0.1, 0.0), (128, 16, 16), 200, 1e-5, 0, 0, ic=ma.MA_IC_SOD)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    assert_bitexact(run_gpu(md, o, U0), oracle.solve(md, o, U0))


@pytest.mark.parametrize("limiter,visc_model", [(ma.MA_LIMITER_VANALBADA, ma.MA_VISC_SUTHERLAND),
                                                (ma.MA_LIMITER_VENKAT, ma.MA_VISC_CONSTANT),
                                                (ma.MA_LIMITER_VANALBADA, ma.MA_VISC_CONSTANT)])
def test_extensions_bitexact(has_gpu, limiter, visc_model):
    o = make_options(1, (2.0, 0.5, 0.5, 0.0), (24, 12, 6), 30, 1e-6, 1, 1, limiter=limiter,
                     viscosity_model=visc_model, mu=1.8e-5, prandtl=0.72)
    o.inflow_state = [1.16, 1.16 * 104.0, 0.0, 0.0, 1.16 * (717.625 * 300.0 + 0.5 * 104.0 ** 2)]
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    assert_bitexact(run_gpu(md, o, U0), oracle.solve(md, o, U0))


@pytest.mark.parametrize("dims", [(1, 1, 1), (2, 1, 1), (1, 3, 2), (5, 1, 4), (3, 3, 3)])
@pytest.mark.parametrize("second,viscous", [(0, 0), (1, 1)])
def test_small_and_degenerate_meshes(has_gpu, dims, second, viscous):
    o = make_options(1, (1.0, 0.5, 0.25, 0.0), dims, 7, 1e-7, second, viscous)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    rng = np.random.default_rng(sum(dims))
    U0 = U0 * (1.0 + 0.01 * rng.standard_normal(U0.shape))
    assert_bitexact(run_gpu(md, o, U0), oracle.solve(md, o, U0))


def test_stepping_in_chunks_equals_one_call(has_gpu):
    o = make_options(*REF_TESTS["FlatPlate_Serial"])
    o.ntimesteps = 20
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.set_state(U0)
        for n in (3, 0, 7, 10):
            s.step(n)
        s.synchronize()
        U = s.get_state()
        assert s.steps_done == 20
    assert_bitexact(U, run_gpu(md, o, U0))


def test_component_major_state_layout(has_gpu):
    """MA_LAYOUT_SOA ((5, C) host arrays, the layout the end-to-end bench
    copies) carries the same bits as the cell-major layout."""
    o = make_options(*REF_TESTS["Ramp_Serial"])
    o.ntimesteps = 5
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.set_state(np.ascontiguousarray(U0.T), layout=ma.MA_LAYOUT_SOA)
        s.step(5)
        U_soa = s.get_state(layout=ma.MA_LAYOUT_SOA)
        assert U_soa.shape == (5, md.ncells)
        assert_bitexact(s.get_state(), U_soa.T)
    assert_bitexact(U_soa.T, run_gpu(md, o, U0))


def test_deterministic_repeat(has_gpu):
    o = make_options(*REF_TESTS["Ramp_Serial"])
    o.ntimesteps = 50
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    assert_bitexact(run_gpu(md, o, U0), run_gpu(md, o, U0))


def test_residual_matches_oracle(has_gpu):
    o = make_options(*REF_TESTS["FlatPlate_Serial"], keep_residual=1)
    o.ntimesteps = 3
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.set_state(U0)
        s.step(3)
        s.synchronize()
        U, R = s.get_state(), s.get_residual()
    Uo, Ro = oracle.solve(md, o, U0, return_residual=True)
    assert_bitexact(U, Uo)
    assert_bitexact(R, Ro)


# ---- mixed form -----------------------------------------------------------------------
def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_mixed_sod_density_error(has_gpu):
    """Mixed form within 1e-5 relative L2 density error of FP64 (Sod, 2nd order viscous)."""
    o = make_options(0, (1.0, 0.5, 0.5, 0.0), (64, 16, 16), 50, 1e-5, 1, 1, ic=ma.MA_IC_SOD,
                     viscosity_model=ma.MA_VISC_CONSTANT, mu=1.8e-5, prandtl=0.72)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    ref = oracle.solve(md, o, U0)
    om = o.copy()
    om.precision = ma.MA_PREC_MIXED
    Um = run_gpu(md, om, U0)
    assert rel_l2(Um[:, 0], ref[:, 0]) < 1e-5
    for k in range(5):
        if np.linalg.norm(ref[:, k]) > 0:
            assert rel_l2(Um[:, k], ref[:, k]) < 1e-3


def test_mixed_flat_plate_density_error(has_gpu):
    o = make_options(1, (2.0, 0.5, 0.5, 0.0), (32, 16, 8), 40, 2e-6, 1, 1, limiter=ma.MA_LIMITER_VANALBADA,
                     viscosity_model=ma.MA_VISC_CONSTANT, mu=1.8e-5, prandtl=0.72)
    rho = 1e5 / (287.05 * 300.0)
    u = 0.3 * np.sqrt(1.4 * 287.05 * 300.0)
    o.inflow_state = [rho, rho * u, 0.0, 0.0, rho * (717.625 * 300.0 + 0.5 * u * u)]
    o.ic = ma.MA_IC_CONSTANT
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    ref = oracle.solve(md, o, U0)
    om = o.copy()
    om.precision = ma.MA_PREC_MIXED
    Um = run_gpu(md, om, U0)
    assert rel_l2(Um[:, 0], ref[:, 0]) < 1e-5


# ---- exact division used by the gradient ------------------------------------------------
@pytest.mark.parametrize("mode", [0, 1, 2, 3, 4, 5, 6])
def test_reciprocal_division_is_correctly_rounded(has_gpu, mode):
    """div_by_recip(a, b, RN(1/b)) equals the IEEE quotient a/b bit for bit
    (2^28 pairs per mode; mode 5: numerators from the subnormal range to
    2^-880 and signed zeros, where the reciprocal method hands over to the
    IEEE division); mode 3: widen_exact equals the float->double conversion
    on 2^28 random bit patterns (subnormals: signed zero); mode 4: narrow_rn
    equals the double->float conversion (random patterns, both edges of the
    float range, exact midpoints and their neighbours); mode 6: the integer
    forms of 0.5*x, 2*x, 0+x, |x| and x < y (x >= 0) equal the FP64
    instructions on 2^28 patterns of every exponent class."""
    import ctypes
    from miniaero_gb300 import _lib
    mism = ctypes.c_uint64(0)
    ex = np.zeros(2)
    _lib.check(_lib.lib().ma_debug_check_division(mode, 1 << 28, 12345 + mode, ctypes.byref(mism), _lib.f64p(ex)))
    assert mism.value == 0, "first mismatch a=%r b=%r" % (ex[0], ex[1])


def test_fp64_rate_is_measured(has_gpu):
    """The FP64 ceiling the bench reports against: three positive, finite
    rates of at least one instruction per SM per 100 clocks."""
    for op in ("add", "mul", "fma"):
        r = ma.fp64_rate(op)
        assert np.isfinite(r) and r > 152 * 1e9 / 100, (op, r)
    import ctypes
    from miniaero_gb300 import _lib
    with pytest.raises(ma.MiniaeroError):
        _lib.check(_lib.lib().ma_debug_fp64_rate(3, ctypes.byref(ctypes.c_double())))


# ---- one stage's drivers taken one at a time (ma_op_green_gauss, ...) ---------------
@pytest.mark.parametrize("name", sorted(REF_TESTS))
def test_stage_drivers_one_at_a_time_bitexact(has_gpu, name):
    """Green-Gauss gradients, both limiters, the boundary functors,
    apply_cell_flux and update on an evolved state of each reference case,
    bit for bit against the oracle's drivers (and IEEE numpy for the two
    elementwise ones)."""
    import ctypes
    from miniaero_gb300 import _lib
    o = make_options(*REF_TESTS[name])
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U = oracle.solve(md, o, ma.initial_state(md, o), nsteps=5)
    dm = ma.DeviceMesh(md)
    assert_bitexact(ma.green_gauss(dm, U).reshape(-1, 5), oracle.field_gradients(md, o, U).reshape(-1, 5))
    soa = np.ascontiguousarray(U.T)
    g = np.empty((md.ncells, 5, 3))
    _lib.check(_lib.lib().ma_op_green_gauss(dm._h, _lib.f64p(soa), ma.MA_LAYOUT_SOA, _lib.f64p(g)))
    assert_bitexact(g.reshape(-1, 5), oracle.field_gradients(md, o, U).reshape(-1, 5))
    for lim in (ma.MA_LIMITER_VENKAT, ma.MA_LIMITER_VANALBADA):
        ol = o.copy()
        ol.limiter = lim
        assert_bitexact(ma.stencil_limiter(dm, U, lim), oracle.field_limiter(md, ol, U))
    flux = ma.bc_flux(dm, o, U)
    assert_bitexact(flux, oracle.field_bc_flux(md, o, U))
    res = ma.apply_cell_flux(o.dt, md.cell_volumes, flux)
    assert_bitexact(res, 0.0 + (o.dt / md.cell_volumes)[:, None] * flux)
    assert_bitexact(ma.rk_update(0.5, res, U), U + 0.5 * res)
    dm.close()


def test_stage_drivers_reject_bad_arguments(has_gpu):
    import ctypes
    from miniaero_gb300 import _lib
    o = make_options(0, (1.0, 0.5, 0.5, 0.0), (4, 2, 2), 1, 1e-6, 1, 1)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    dm = ma.DeviceMesh(md)
    U = ma.initial_state(md, o)
    with pytest.raises(ma.MiniaeroError):
        ma.stencil_limiter(dm, U, 7)
    g = np.empty((md.ncells, 5, 3))
    with pytest.raises(ma.MiniaeroError):
        _lib.check(_lib.lib().ma_op_green_gauss(dm._h, _lib.f64p(np.ascontiguousarray(U)), 9, _lib.f64p(g)))
    with pytest.raises(ma.MiniaeroError):
        _lib.check(_lib.lib().ma_op_rk_update(-1, 1.0, _lib.f64p(g), _lib.f64p(g), _lib.f64p(g)))
    dm.close()


# ---- failure detection: bad states found by a device reduction (no trap) -----------
def test_state_check_reports_the_first_bad_cell(has_gpu):
    """Host-prepared states with a NaN, an infinity, a negative density or a
    zero energy are reported as MA_ENUMERIC with the first bad cell; the
    solver stays usable afterwards."""
    o = make_options(0, (1.0, 0.5, 0.5, 0.0), (8, 4, 4), 2, 1e-6, 1, 1)
    md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
    U0 = ma.initial_state(md, o)
    with ma.TimeSolverExplicitRK4(md, o) as s:
        s.set_state(U0)
        assert s.check_state() == (0, -1)
        for cells, k, v in (([37], 2, np.nan), ([91, 12], 3, np.inf), ([60, 5], 0, -1.0), ([100], 4, 0.0)):
            U = U0.copy()
            for c in cells:
                U[c, k] = v
            s.set_state(U)
            st, bad = s.check_state()
            assert st == ma._lib.MA_ENUMERIC and bad == min(cells), (cells, k, v, st, bad)
        s.set_state(U0)
        s.step(2)
        s.synchronize()
        assert s.check_state() == (0, -1)
        assert np.array_equal(s.get_state(), oracle.solve(md, o, U0, nsteps=2))


def test_solvers_in_separate_threads_equal_sequential(has_gpu):
    """Separate solvers driven from separate host threads (each capturing
    and replaying its own step graph on its own stream) give the same bits as
    the same solves run one after another."""
    import threading
    cases = []
    for dims, prec in (((12, 6, 4), ma.MA_PREC_FP64), ((10, 8, 3), ma.MA_PREC_FP64), ((16, 4, 4), ma.MA_PREC_MIXED),
                       ((9, 9, 2), ma.MA_PREC_MIXED)):
        o = make_options(1, (1.0, 0.5, 0.25, 0.0), dims, 12, 2e-7, 1, 1, precision=prec)
        md = ma.Parallel3DMesh.from_options(o).fill_mesh_data()
        cases.append((md, o, ma.initial_state(md, o)))

    def solve(md, o, U0):
        with ma.TimeSolverExplicitRK4(md, o) as s:
            s.set_state(U0)
            for _ in range(3):
                s.step(4)
            s.synchronize()
            return s.get_state()

    expected = [solve(*c) for c in cases]
    got = [None] * len(cases)
    errors = []

    def worker(i):
        try:
            got[i] = solve(*cases[i])
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(cases))]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for a, b in zip(got, expected):
        assert_bitexact(a, b)
