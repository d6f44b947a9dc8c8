"""The oracle's one-driver-at-a-time functions (oracle_field_*), the checkers
of the device operator entry points ma_op_green_gauss / ma_op_stencil_limiter /
ma_op_bc_flux: properties the reference's drivers have on simple states."""
import numpy as np

import miniaero_gb300 as ma
import oracle

CV = 287.05 / 0.4  # R / (gamma - 1)


def box(nx=8, ny=6, nz=4, bc=None):
    o = ma.Options(problem_type=0, lx=1.0, ly=0.75, lz=0.5, nx=nx, ny=ny, nz=nz, second_order_space=1, viscous=1,
                   ic=ma.MA_IC_SOD, viscosity_model=ma.MA_VISC_CONSTANT, mu=1.8e-5, prandtl=0.72)
    if bc is not None:
        o.bc_override = bc
    return o, ma.Parallel3DMesh.from_options(o).fill_mesh_data()


def state_from_primitives(rho, u, T):
    U = np.empty((rho.shape[0], 5))
    U[:, 0] = rho
    U[:, 1:4] = rho[:, None] * u
    U[:, 4] = rho * (CV * T + 0.5 * (u ** 2).sum(1))
    return U


def test_gradients_of_a_linear_field_are_exact_inside():
    o, md = box()
    x = md.cell_coords
    rho = 1.0 + 0.1 * x[:, 0] - 0.05 * x[:, 2]
    T = 300.0 + 10.0 * x[:, 1]
    u = np.zeros((md.ncells, 3))
    g = oracle.field_gradients(md, o, state_from_primitives(rho, u, T))
    lo, hi = x.min(0), x.max(0)
    inside = np.all((x > lo + 1e-9) & (x < hi - 1e-9), axis=1)
    assert inside.sum() > 0
    np.testing.assert_allclose(g[inside, 0], np.tile([0.1, 0.0, -0.05], (inside.sum(), 1)), atol=1e-12)
    np.testing.assert_allclose(g[inside, 4], np.tile([0.0, 10.0, 0.0], (inside.sum(), 1)), atol=1e-9)
    assert np.all(g[inside, 1:4] == 0.0)


def test_limiter_is_one_on_a_uniform_state_and_within_bounds():
    o, md = box()
    U = state_from_primitives(np.full(md.ncells, 1.2), np.zeros((md.ncells, 3)), np.full(md.ncells, 300.0))
    for lim in (ma.MA_LIMITER_VENKAT, ma.MA_LIMITER_VANALBADA):
        o.limiter = lim
        assert np.all(oracle.field_limiter(md, o, U) == 1.0)
    rng = np.random.default_rng(3)
    U = state_from_primitives(1.0 + 0.2 * rng.random(md.ncells), 10 * rng.standard_normal((md.ncells, 3)),
                              300.0 + 20 * rng.random(md.ncells))
    for lim in (ma.MA_LIMITER_VENKAT, ma.MA_LIMITER_VANALBADA):
        o.limiter = lim
        phi = oracle.field_limiter(md, o, U)
        assert np.all(phi >= 0.0) and np.all(phi <= 1.0) and np.any(phi < 1.0)


def test_closed_box_at_rest_feels_no_net_boundary_force():
    """Tangent walls on every side, uniform gas at rest: no mass or energy
    crosses the boundary and the wall pressure forces cancel."""
    o, md = box(bc=[1, 1, 1, 1, 1, 1])
    U = state_from_primitives(np.full(md.ncells, 1.2), np.zeros((md.ncells, 3)), np.full(md.ncells, 300.0))
    f = oracle.field_bc_flux(md, o, U)
    assert np.all(f[:, 0] == 0.0) and np.all(f[:, 4] == 0.0)
    p = 1.2 * 287.05 * 300.0
    assert np.max(np.abs(f[:, 1:4].sum(0))) < 1e-9 * p
    assert np.max(np.abs(f[:, 1:4])) > 0.0
