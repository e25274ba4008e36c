"""Oracle: the MONOLITHIC velocity-pressure coupling on CPU
(src/module_simulation.f90:552-583; operator src/module_navier_stokes.f90:
380-780 with the pressure block, preconditioner diagonal :1541-1590).

Known answers: the continuity rows are div u dvol (+ 1e-10 p(1,1) dvol in
cell (1,1)); the momentum rows are the predictor operator plus B^T p; the
Schur diagonal follows its formula; a fluid at rest under gravity solves to
u = 0 and the hydrostatic pressure gradient rho g; the Krylov solution of a
small coupled system equals a dense direct solve of the assembled matrix.
"""
from __future__ import annotations

import numpy as np
import pytest


def _cavity(pkg, orc, n=12, seed=3):
    p, dt = pkg.cases.cavity_case(n)
    f = pkg.Fields.allocate(p)
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    f.u[...], f.v[...] = pkg.cases.random_velocity(p, 0.3, seed)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    return p, f, dt


def _operands(p, seed=5):
    rng = np.random.default_rng(seed)
    shape = (p.ny + 2, p.nx + 2)
    return rng.standard_normal(shape), rng.standard_normal(shape), rng.standard_normal(shape)


def test_rows_are_momentum_plus_gradient_and_divergence(pkg, orc):
    p, f, dt = _cavity(pkg, orc)
    xu, xv, xp = _operands(p)
    yu, yv, yp = orc.mono_apply(p, dt, xu, xv, xp, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u, f.v)
    mu_, mv_ = orc.momentum_apply(p, dt, xu, xv, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u, f.v)
    nx, ny, dx, dy = p.nx, p.ny, p.dx, p.dy
    # interior u faces i = 2..nx, interior v faces j = 2..ny: + B^T p
    assert np.array_equal(yu[1:ny + 1, 2:nx + 1], mu_[1:ny + 1, 2:nx + 1] + (xp[1:ny + 1, 2:nx + 1] - xp[1:ny + 1, 1:nx]) * dy)
    assert np.array_equal(yv[2:ny + 1, 1:nx + 1], mv_[2:ny + 1, 1:nx + 1] + (xp[2:ny + 1, 1:nx + 1] - xp[1:ny, 1:nx + 1]) * dx)
    # wall rows carry no pressure
    assert np.array_equal(yu[1:ny + 1, 1], mu_[1:ny + 1, 1]) and np.array_equal(yu[1:ny + 1, nx + 1], mu_[1:ny + 1, nx + 1])
    assert np.array_equal(yv[1, 1:nx + 1], mv_[1, 1:nx + 1]) and np.array_equal(yv[ny + 1, 1:nx + 1], mv_[ny + 1, 1:nx + 1])
    # continuity rows
    div = (xu[1:ny + 1, 2:nx + 2] - xu[1:ny + 1, 1:nx + 1]) / dx + (xv[2:ny + 2, 1:nx + 1] - xv[1:ny + 1, 1:nx + 1]) / dy
    want = div * (dx * dy)
    want[0, 0] = div[0, 0] * (dx * dy) + 1.0e-10 * xp[1, 1] * (dx * dy)
    assert np.array_equal(yp[1:ny + 1, 1:nx + 1], want)


def test_operator_ignores_pressure_ghosts(pkg, orc):
    p, f, dt = _cavity(pkg, orc)
    xu, xv, xp = _operands(p)
    a = orc.mono_apply(p, dt, xu, xv, xp, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u, f.v)
    xq = xp.copy()
    xq[0, :] = 7.0; xq[-1, :] = -3.0; xq[:, 0] = 11.0; xq[:, -1] = 5.0
    b = orc.mono_apply(p, dt, xu, xv, xq, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u, f.v)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_schur_diagonal_formula(pkg, orc):
    p, f, dt = _cavity(pkg, orc)
    du, dv = orc.momentum_diag(p, dt, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u, f.v)
    dp = orc.schur_diag(p, dt, du, dv)
    nx, ny, dx, dy = p.nx, p.ny, p.dx, p.dy
    aW = (dy * dy) / np.maximum(1e-30, du[1:ny + 1, 1:nx + 1]); aW[:, 0] = 0.0
    aE = (dy * dy) / np.maximum(1e-30, du[1:ny + 1, 2:nx + 2]); aE[:, -1] = 0.0
    aS = (dx * dx) / np.maximum(1e-30, dv[1:ny + 1, 1:nx + 1]); aS[0, :] = 0.0
    aN = (dx * dx) / np.maximum(1e-30, dv[2:ny + 2, 1:nx + 1]); aN[-1, :] = 0.0
    reg = np.full((ny, nx), 1.0e-12 * dx * dy)
    reg[0, 0] = 1.0e-10 * dx * dy
    assert np.array_equal(dp[1:ny + 1, 1:nx + 1], aW + aE + aS + aN + 0.0 + reg)


def test_hydrostatic_rest(pkg, orc):
    """Uniform fluid at rest under gravity: u = v = 0 and dp/dy = rho g."""
    p, C0, dt = pkg.cases.bubble_case(nx=12, ny=24, nsub=4)
    p.solver_type = pkg.capi.SOLVER_MONOLITHIC
    p.linear_solver = pkg.capi.LINEAR_BICGSTAB2
    p.max_iter = 5000
    f = pkg.Fields.allocate(p)
    f.C[...] = 1.0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    for k in range(2):
        it, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    assert np.abs(f.u).max() < 1e-12 and np.abs(f.v).max() < 1e-12
    gp = (f.p[2:p.ny + 1, 1:-1] - f.p[1:p.ny, 1:-1]) / p.dy
    assert np.allclose(gp, p.rho1 * p.gy, rtol=1e-8, atol=0)


def test_krylov_matches_a_dense_solve(pkg, orc):
    """One step's Krylov solution (BiCGSTAB2, tol 1e-12) equals the dense
    solve of the coupled matrix assembled column by column (the pressure up
    to its level)."""
    p, f, dt = _cavity(pkg, orc, n=6)
    p.tol = 1e-12
    nx, ny = p.nx, p.ny
    dofs = ([("u", i, j) for j in range(1, ny + 1) for i in range(1, nx + 2)]
            + [("v", i, j) for j in range(1, ny + 2) for i in range(1, nx + 1)]
            + [("p", i, j) for j in range(1, ny + 1) for i in range(1, nx + 1)])
    z = np.zeros_like(f.u)

    def flat(yu, yv, yp):
        return np.array([{"u": yu, "v": yv, "p": yp}[t][j, i] for t, i, j in dofs])

    A = np.zeros((len(dofs), len(dofs)))
    for c, (t, i, j) in enumerate(dofs):
        x = {"u": z.copy(), "v": z.copy(), "p": z.copy()}
        x[t][j, i] = 1.0
        A[:, c] = flat(*orc.mono_apply(p, dt, x["u"], x["v"], x["p"], f.u, f.v, f.rho_u, f.rho_v, f.mu,
                                       f.mu_node, f.u, f.v))
    ru, rv = orc.momentum_rhs(p, dt, f.u, f.v, f.rho_u, f.rho_v, f.mu_node, f.fx_sigma, f.fy_sigma, f.u_old,
                              f.v_old)
    xd = np.linalg.solve(A, flat(ru, rv, z))
    g = f.copy()
    it, st = orc.mono_step(p, dt, g, 0)
    assert st == 0
    xk = flat(g.u, g.v, g.p)
    nvel = len(dofs) - nx * ny
    assert np.abs(xk[:nvel] - xd[:nvel]).max() < 1e-8 * np.abs(xd[:nvel]).max()
    # the pressure level is held only by the 1e-10 dvol regularisation of
    # cell (1,1): the Krylov tolerance leaves it loose, so compare the
    # pressure up to a constant
    pk_, pd_ = xk[nvel:] - xk[nvel:].mean(), xd[nvel:] - xd[nvel:].mean()
    assert np.abs(pk_ - pd_).max() < 1e-6 * np.abs(pd_).max()


def test_cavity_time_loop(pkg, orc):
    """Three coupled steps of the driven cavity converge; the lid drags the
    top row forward and the flow stays discretely divergence-free to the
    Krylov tolerance."""
    p, dt = pkg.cases.cavity_case(16)
    f = pkg.Fields.allocate(p)
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    for k in range(3):
        it, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0 and it > 0
    nx, ny, dx, dy = p.nx, p.ny, p.dx, p.dy
    div = (f.u[1:ny + 1, 2:nx + 2] - f.u[1:ny + 1, 1:nx + 1]) / dx + (f.v[2:ny + 2, 1:nx + 1] - f.v[1:ny + 1, 1:nx + 1]) / dy
    assert np.abs(div).max() < 1e-6
    assert f.u[ny, 1:nx + 1].mean() > 0.1
