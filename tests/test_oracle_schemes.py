"""Oracle: the predictor's time schemes and convective variants
(src/module_navier_stokes.f90:380-1101, 2386-2498) on CPU.

Known answers that follow from the formulas themselves:
* Superbee's limiter on a constant field (dq = 0) is psi = 0, so TVD equals
  UPWIND bit for bit;
* Adams-Bashforth without history advects with u_old, which equals u here,
  so it equals PICARD bit for bit; with u_nm1 = u_old the extrapolation
  2 u - u is exact, so it still does;
* Gear without history (the first step) is Euler bit for bit; with history
  its unsteady coefficient is 1.5 rho / dt and its inertial term
  rho (2 u^n - u^(n-1)/2) / dt.
"""
from __future__ import annotations

import numpy as np
import pytest


def _state(pkg, orc, nx=24, ny=32, seed=5, vel=1e-1):
    p, C0, dt = pkg.cases.bubble_case(nx=nx, ny=ny, nsub=4)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    f.u[...], f.v[...] = pkg.cases.random_velocity(p, vel, seed)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    return p, f, dt


def _apply(orc, p, dt, f, xu, xv, **hist):
    return orc.momentum_apply(p, dt, xu, xv, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, **hist)


def _rows(p, y):
    yu, yv = y
    return yu[1:p.ny + 1, 1:p.nx + 2], yv[1:p.ny + 2, 1:p.nx + 1]


def test_tvd_on_constant_field_is_upwind(pkg, orc):
    p, f, dt = _state(pkg, orc)
    f.u[...] = 0.3
    f.v[...] = -0.2
    rng = np.random.default_rng(1)
    xu, xv = rng.standard_normal(f.u.shape), rng.standard_normal(f.v.shape)
    p.convective_scheme = pkg.capi.CONV_UPWIND
    y_up = _apply(orc, p, dt, f, xu, xv)
    p.convective_scheme = pkg.capi.CONV_TVD_SUPERBEE
    y_tvd = _apply(orc, p, dt, f, xu, xv)
    for a, b in zip(_rows(p, y_up), _rows(p, y_tvd)):
        assert np.array_equal(a, b)


def test_tvd_differs_from_both_on_a_varying_field(pkg, orc):
    p, f, dt = _state(pkg, orc)
    rng = np.random.default_rng(2)
    xu, xv = rng.standard_normal(f.u.shape), rng.standard_normal(f.v.shape)
    ys = {}
    for name in ("UPWIND", "CENTERED", "TVD_SUPERBEE"):
        p.convective_scheme = getattr(pkg.capi, "CONV_" + name)
        ys[name] = _rows(p, _apply(orc, p, dt, f, xu, xv))
    for other in ("UPWIND", "CENTERED"):
        assert not np.array_equal(ys["TVD_SUPERBEE"][0], ys[other][0])


def test_tvd_operator_is_linear_in_the_operand(pkg, orc):
    """The limiter reads fields_old only, so A(x) stays linear."""
    p, f, dt = _state(pkg, orc)
    p.convective_scheme = pkg.capi.CONV_TVD_SUPERBEE
    rng = np.random.default_rng(3)
    x1 = rng.standard_normal(f.u.shape), rng.standard_normal(f.v.shape)
    x2 = rng.standard_normal(f.u.shape), rng.standard_normal(f.v.shape)
    y1 = _rows(p, _apply(orc, p, dt, f, *x1))
    y2 = _rows(p, _apply(orc, p, dt, f, *x2))
    y12 = _rows(p, _apply(orc, p, dt, f, x1[0] + 2.0 * x2[0], x1[1] + 2.0 * x2[1]))
    for a, b, c in zip(y1, y2, y12):
        assert np.allclose(c, a + 2.0 * b, rtol=1e-12, atol=1e-12 * np.abs(c).max())


def test_ab2_without_history_and_with_flat_history_is_picard(pkg, orc):
    p, f, dt = _state(pkg, orc)
    rng = np.random.default_rng(4)
    xu, xv = rng.standard_normal(f.u.shape), rng.standard_normal(f.v.shape)
    p.convective_scheme = pkg.capi.CONV_CENTERED
    p.convective_linearization = pkg.capi.CONV_LIN_PICARD
    y_pic = _rows(p, _apply(orc, p, dt, f, xu, xv))
    p.convective_linearization = pkg.capi.CONV_LIN_AB2
    y0 = _rows(p, _apply(orc, p, dt, f, xu, xv, u_old=f.u_old, v_old=f.v_old))
    y1 = _rows(p, _apply(orc, p, dt, f, xu, xv, u_old=f.u_old, v_old=f.v_old, u_nm1=f.u_old.copy(),
                         v_nm1=f.v_old.copy(), has_nm1=1))
    for a, b, c in zip(y_pic, y0, y1):
        assert np.array_equal(a, b) and np.array_equal(a, c)
    # a real history changes the advecting velocity
    u_nm1, v_nm1 = pkg.cases.random_velocity(p, 1e-1, 9)
    y2 = _rows(p, _apply(orc, p, dt, f, xu, xv, u_old=f.u_old, v_old=f.v_old, u_nm1=u_nm1, v_nm1=v_nm1,
                         has_nm1=1))
    assert not np.array_equal(y2[0], y_pic[0])


def test_gear_first_step_is_euler_then_bdf2(pkg, orc):
    p, f, dt = _state(pkg, orc)
    p.enable_convection = 0
    rng = np.random.default_rng(6)
    xu, xv = rng.standard_normal(f.u.shape), rng.standard_normal(f.v.shape)
    u_nm1, v_nm1 = pkg.cases.random_velocity(p, 1e-1, 11)
    hist = dict(u_old=f.u_old, v_old=f.v_old, u_nm1=u_nm1, v_nm1=v_nm1)
    p.time_scheme = pkg.capi.TIME_EULER
    y_e = _rows(p, _apply(orc, p, dt, f, xu, xv))
    r_e = orc.momentum_rhs(p, dt, f.u, f.v, f.rho_u, f.rho_v, f.mu_node, f.fx_sigma, f.fy_sigma, f.u_old, f.v_old)
    p.time_scheme = pkg.capi.TIME_GEAR
    y_g0 = _rows(p, _apply(orc, p, dt, f, xu, xv, **hist, has_nm1=0))
    r_g0 = orc.momentum_rhs(p, dt, f.u, f.v, f.rho_u, f.rho_v, f.mu_node, f.fx_sigma, f.fy_sigma, f.u_old,
                            f.v_old, u_nm1, v_nm1, 0)
    for a, b in zip(y_e, y_g0):
        assert np.array_equal(a, b)
    for a, b in zip(r_e, r_g0):
        assert np.array_equal(a, b)
    # with history: A_gear - A_euler = 0.5 rho/dt dvol x on interior rows
    y_g1 = _rows(p, _apply(orc, p, dt, f, xu, xv, **hist, has_nm1=1))
    dvol = p.dx * p.dy
    nx, ny = p.nx, p.ny
    du = (y_g1[0] - y_e[0])[:, 1:nx]          # u faces i = 2..nx
    want = (0.5 * f.rho_u / dt * dvol * xu)[1:ny + 1, 2:nx + 1]
    assert np.allclose(du, want, rtol=1e-9, atol=1e-12 * np.abs(want).max())
    # inertial term rho (2 u_old - u_nm1 / 2) / dt dvol on interior u rows
    r_g1 = orc.momentum_rhs(p, dt, f.u, f.v, f.rho_u, f.rho_v, f.mu_node, f.fx_sigma, f.fy_sigma, f.u_old,
                            f.v_old, u_nm1, v_nm1, 1)
    d = (r_g1[0] - r_e[0])[1:ny + 1, 2:nx + 1]
    want = (f.rho_u * (2.0 * f.u_old - 0.5 * u_nm1) / dt * dvol - f.rho_u / dt * f.u_old * dvol)[1:ny + 1, 2:nx + 1]
    assert np.allclose(d, want, rtol=1e-9, atol=1e-12 * np.abs(want).max())


def test_newton_is_unsupported(pkg, orc):
    p, f, dt = _state(pkg, orc)
    p.convective_linearization = pkg.capi.CONV_LIN_NEWTON
    with pytest.raises(AssertionError):
        _apply(orc, p, dt, f, f.u, f.v)


@pytest.mark.parametrize("combo", ["gear_ab2_centered", "gear_picard_tvd"])
def test_time_loop_with_history_runs(pkg, orc, combo):
    """Four oracle time steps of the two-phase bubble with history schemes:
    converged solves, bounded velocities."""
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=16, ny=32, nsub=4)
    p.time_scheme = cap.TIME_GEAR
    if combo == "gear_ab2_centered":
        p.convective_linearization = cap.CONV_LIN_AB2
        p.convective_scheme = cap.CONV_CENTERED
    else:
        p.convective_scheme = cap.CONV_TVD_SUPERBEE
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    for k in range(4):
        iu, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0 and rr <= p.p_tol
    assert np.isfinite(f.u).all() and np.abs(f.u).max() < 1.0
    # the history rotated: u_nm1 is the velocity at the start of step 3
    assert not np.array_equal(f.u_nm1, f.u_old)
