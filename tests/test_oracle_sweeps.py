"""Oracle: the sweep preconditioners of the momentum / coupled Krylov solves
(SSOR and BLOCK_TRIANGULAR, src/module_linear_solvers.f90:137-278 with the
lexicographic solves :1278-1401 and the stencils of
ns_assemble_preconditioner_blocks, src/module_navier_stokes.f90:1268-1595).

Known answers: the stencil centres are the Jacobi diagonals (and the Schur
centre diag_p); the SSOR application equals a plain-Python restatement of
the serial sweeps on the exported stencils, bit for bit; the
block-triangular pressure output has zero mean; both are linear; and a
coupled solve preconditioned by either reaches the same solution as with
Jacobi in far fewer iterations.
"""
from __future__ import annotations

import numpy as np
import pytest


def _cavity(pkg, orc, n=10, m=None, seed=3):
    p, dt = pkg.cases.cavity_case(n)
    if m is not None:
        p.ny = m
        p.dy = 1.0 / m
    f = pkg.Fields.allocate(p)
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    f.u[...], f.v[...] = pkg.cases.random_velocity(p, 0.3, seed)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    return p, f, dt


def _z(p, seed=9):
    rng = np.random.default_rng(seed)
    shape = (p.ny + 2, p.nx + 2)
    zu, zv, zp = rng.standard_normal(shape), rng.standard_normal(shape), rng.standard_normal(shape)
    # only DOF entries are packed; zero the rest so comparisons see DOFs only
    zu[0, :] = zu[-1, :] = 0.0; zu[:, 0] = 0.0
    zv[0, :] = 0.0; zv[:, 0] = zv[:, -1] = 0.0
    zp[0, :] = zp[-1, :] = 0.0; zp[:, 0] = zp[:, -1] = 0.0
    return zu, zv, zp


def _args(f):
    return (f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u_old, f.v_old)


def test_stencil_centres_are_the_diagonals(pkg, orc):
    p, f, dt = _cavity(pkg, orc, 9, 13)
    blk = orc.prec_blocks(p, dt, *_args(f))
    du, dv = orc.momentum_diag(p, dt, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u_old, f.v_old)
    nx, ny = p.nx, p.ny
    assert np.array_equal(blk["u"]["P"][1:ny + 1, 1:nx + 2], du[1:ny + 1, 1:nx + 2])
    assert np.array_equal(blk["v"]["P"][1:ny + 2, 1:nx + 1], dv[1:ny + 2, 1:nx + 1])
    dp = orc.schur_diag(p, dt, du, dv)
    assert np.array_equal(blk["s"]["P"][1:ny + 1, 1:nx + 1], dp[1:ny + 1, 1:nx + 1])
    # M-matrix form: every neighbour coefficient is non-negative
    for b in "uvs":
        for c in "WESN":
            assert blk[b][c].min() >= 0.0


def _ssor_py(aW, aE, aS, aN, aP, z, ni, nj, sweeps, omega):
    r = np.zeros_like(z)

    def cell(i, j):
        d = aP[j, i]
        if abs(d) < 1e-30:
            d = 1.0
        val = z[j, i]
        if aW[j, i] != 0.0:
            val = val + aW[j, i] * r[j, i - 1]
        if aE[j, i] != 0.0:
            val = val + aE[j, i] * r[j, i + 1]
        if aS[j, i] != 0.0:
            val = val + aS[j, i] * r[j - 1, i]
        if aN[j, i] != 0.0:
            val = val + aN[j, i] * r[j + 1, i]
        r[j, i] = (1.0 - omega) * r[j, i] + omega * (val / d)

    for _ in range(sweeps):
        for j in range(1, nj + 1):
            for i in range(1, ni + 1):
                cell(i, j)
        for j in range(nj, 0, -1):
            for i in range(ni, 0, -1):
                cell(i, j)
    return r


@pytest.mark.parametrize("mono", [False, True])
def test_ssor_matches_serial_restatement(pkg, orc, mono):
    p, f, dt = _cavity(pkg, orc, 7, 9)
    p.precond = pkg.capi.PRECOND_SSOR
    if not mono:
        p.solver_type = pkg.capi.SOLVER_STANDARD_PROJECTION
    zu, zv, zp = _z(p)
    yu, yv, yp = orc.precond_apply(p, dt, zu, zv, zp, *_args(f))
    blk = orc.prec_blocks(p, dt, *_args(f))
    nx, ny = p.nx, p.ny
    # pad a row so the v block's north neighbour of its top row exists
    def pad(a):
        return np.vstack([a, np.zeros((1, a.shape[1]))])
    B = {b: {c: pad(blk[b][c]) for c in "WESNP"} for b in "uvs"}
    ru = _ssor_py(*(B["u"][c] for c in "WESNP"), pad(zu), nx + 1, ny, 2, 1.0)
    rv = _ssor_py(*(B["v"][c] for c in "WESNP"), pad(zv), nx, ny + 1, 2, 1.0)
    assert np.array_equal(yu[1:ny + 1, 1:nx + 2], ru[1:ny + 1, 1:nx + 2])
    assert np.array_equal(yv[1:ny + 2, 1:nx + 1], rv[1:ny + 2, 1:nx + 1])
    if mono:
        rp = _ssor_py(*(B["s"][c] for c in "WESNP"), pad(zp), nx, ny, 2, 1.0)
        assert np.array_equal(yp[1:ny + 1, 1:nx + 1], rp[1:ny + 1, 1:nx + 1])


def test_block_triangular_structure(pkg, orc):
    """BLOCK_TRIANGULAR: the pressure block is 12 over-relaxed Schur sweeps
    with the mean removed; the velocity blocks solve z - B^T r_p with four
    sweeps each."""
    p, f, dt = _cavity(pkg, orc, 7, 9)
    p.precond = pkg.capi.PRECOND_BLOCK_TRIANGULAR
    zu, zv, zp = _z(p)
    yu, yv, yp = orc.precond_apply(p, dt, zu, zv, zp, *_args(f))
    blk = orc.prec_blocks(p, dt, *_args(f))
    nx, ny, dx, dy = p.nx, p.ny, p.dx, p.dy

    def pad(a):
        return np.vstack([a, np.zeros((1, a.shape[1]))])
    B = {b: {c: pad(blk[b][c]) for c in "WESNP"} for b in "uvs"}
    rp = _ssor_py(*(B["s"][c] for c in "WESNP"), pad(zp), nx, ny, 12, 1.25)[:-1]
    s = 0.0
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            s += rp[j, i]
    rp[1:ny + 1, 1:nx + 1] -= s / (nx * ny)
    assert np.array_equal(yp[1:ny + 1, 1:nx + 1], rp[1:ny + 1, 1:nx + 1])
    hu = zu.copy()
    hu[1:ny + 1, 2:nx + 1] = zu[1:ny + 1, 2:nx + 1] - (rp[1:ny + 1, 2:nx + 1] - rp[1:ny + 1, 1:nx]) * dy
    hv = zv.copy()
    hv[2:ny + 1, 1:nx + 1] = zv[2:ny + 1, 1:nx + 1] - (rp[2:ny + 1, 1:nx + 1] - rp[1:ny, 1:nx + 1]) * dx
    ru = _ssor_py(*(B["u"][c] for c in "WESNP"), pad(hu), nx + 1, ny, 4, 1.0)
    rv = _ssor_py(*(B["v"][c] for c in "WESNP"), pad(hv), nx, ny + 1, 4, 1.0)
    assert np.array_equal(yu[1:ny + 1, 1:nx + 2], ru[1:ny + 1, 1:nx + 2])
    assert np.array_equal(yv[1:ny + 2, 1:nx + 1], rv[1:ny + 2, 1:nx + 1])


@pytest.mark.parametrize("prec", ["PRECOND_SSOR", "PRECOND_BLOCK_TRIANGULAR"])
def test_preconditioners_are_linear(pkg, orc, prec):
    p, f, dt = _cavity(pkg, orc, 8, 8)
    p.precond = getattr(pkg.capi, prec)
    z1, z2 = _z(p, 1), _z(p, 2)
    y1 = orc.precond_apply(p, dt, *z1, *_args(f))
    y2 = orc.precond_apply(p, dt, *z2, *_args(f))
    y3 = orc.precond_apply(p, dt, *(2.0 * a + b for a, b in zip(z1, z2)), *_args(f))
    for a, b, c in zip(y1, y2, y3):
        assert np.allclose(c, 2.0 * a + b, rtol=0, atol=1e-12 * np.abs(c).max())


@pytest.mark.parametrize("prec", ["PRECOND_SSOR", "PRECOND_BLOCK_TRIANGULAR"])
def test_coupled_solve_same_answer_fewer_iterations(pkg, orc, prec):
    p, f, dt = _cavity(pkg, orc, 16)
    g = f.copy()
    it_j, st_j = orc.mono_step(p, dt, f, 0)
    p.precond = getattr(pkg.capi, prec)
    it_s, st_s = orc.mono_step(p, dt, g, 0)
    assert st_j == st_s == 0
    assert it_s < it_j / 2, (it_s, it_j)
    for a, b in ((g.u, f.u), (g.v, f.v)):
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-7
    nx, ny = p.nx, p.ny
    pg, pf = g.p[1:ny + 1, 1:nx + 1], f.p[1:ny + 1, 1:nx + 1]
    pg, pf = pg - pg.mean(), pf - pf.mean()
    assert np.linalg.norm(pg - pf) / np.linalg.norm(pf) < 1e-5


@pytest.mark.parametrize("prec", ["PRECOND_SSOR", "PRECOND_BLOCK_TRIANGULAR"])
def test_predictor_with_sweeps_converges(pkg, orc, prec):
    """The projection predictor with the sweep preconditioners (velocity
    blocks only) reaches the Jacobi-preconditioned solution."""
    p, C0, dt = pkg.cases.bubble_case(nx=24, ny=40, nsub=4)
    p.linear_solver = pkg.capi.LINEAR_BICGSTAB2
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    f.u[...], f.v[...] = pkg.cases.random_velocity(p, 0.05, 4)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    g = f.copy()
    it_j, st_j = orc.predictor(p, dt, f, has_nm1=0)
    p.precond = getattr(pkg.capi, prec)
    it_s, st_s = orc.predictor(p, dt, g, has_nm1=0)
    assert st_j == st_s == 0
    for a, b in ((g.u, f.u), (g.v, f.v)):
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-9
