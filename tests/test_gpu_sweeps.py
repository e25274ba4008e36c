"""GPU sweep preconditioners (SSOR, BLOCK_TRIANGULAR) against the oracle,
through the C ABI (src/module_linear_solvers.f90:137-278, 1278-1401;
stencils src/module_navier_stokes.f90:1268-1595).

* the preconditioner application: SSOR bit for bit (the wavefront runs the
  serial sweeps' operations in the serial order), BLOCK_TRIANGULAR to the
  rounding of its pressure mean (a parallel sum against a serial one),
  JACOBI to one rounding (a multiply by the inverse against a division);
* coupled (MONOLITHIC), projection-predictor and augmented-Lagrangian solves
  preconditioned by the sweeps: iteration counts within 2 (coupled solves:
  within 10 %), solutions within the solve tolerance; resident steps (run
  eagerly) against the oracle's time loop.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cavity(pkg, orc, nx, ny, seed=3, solver=None):
    p, dt = pkg.cases.cavity_case(nx)
    p.ny, p.dy = ny, 1.0 / ny
    if solver is not None:
        p.solver_type = solver
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
    zu[0, :] = zu[-1, :] = 0.0; zu[:, 0] = 0.0
    zv[0, :] = 0.0; zv[:, 0] = zv[:, -1] = 0.0
    zp[0, :] = zp[-1, :] = 0.0; zp[:, 0] = zp[:, -1] = 0.0
    return zu, zv, zp


def _dofs(p, yu, yv, yp, mono):
    nx, ny = p.nx, p.ny
    out = [yu[1:ny + 1, 1:nx + 2], yv[1:ny + 2, 1:nx + 1]]
    if mono:
        out.append(yp[1:ny + 1, 1:nx + 1])
    return out


# sizes: one band, ragged bands, several bands per job, more bands than one
# chunk row
SIZES = [(7, 9), (20, 37), (45, 70), (40, 100), (97, 131)]


@pytest.mark.parametrize("nx,ny", SIZES)
@pytest.mark.parametrize("mono", [False, True])
def test_ssor_apply_bit_exact(gpu_pkg, orc, nx, ny, mono):
    pkg = gpu_pkg
    cap = pkg.capi
    p, f, dt = _cavity(pkg, orc, nx, ny, solver=None if mono else cap.SOLVER_STANDARD_PROJECTION)
    p.precond = cap.PRECOND_SSOR
    z = _z(p)
    yo = orc.precond_apply(p, dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u_old, f.v_old)
    with pkg.Solver(p) as s:
        s.state_set(f)
        yg = s.precond_apply(dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node)
    for a, b in zip(_dofs(p, *yg, mono), _dofs(p, *yo, mono)):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("nx,ny", SIZES)
def test_block_triangular_apply(gpu_pkg, orc, nx, ny):
    pkg = gpu_pkg
    p, f, dt = _cavity(pkg, orc, nx, ny)
    p.precond = pkg.capi.PRECOND_BLOCK_TRIANGULAR
    z = _z(p)
    yo = orc.precond_apply(p, dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u_old, f.v_old)
    with pkg.Solver(p) as s:
        s.state_set(f)
        yg = s.precond_apply(dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node)
    for a, b in zip(_dofs(p, *yg, True), _dofs(p, *yo, True)):
        assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()


def test_al_penalty_stencils(gpu_pkg, orc):
    """SSOR with the augmented-Lagrangian penalty in the velocity stencils."""
    pkg = gpu_pkg
    cap = pkg.capi
    p, f, dt = _cavity(pkg, orc, 33, 41, solver=cap.SOLVER_AUGMENTED_LAGRANGIAN)
    p.precond = cap.PRECOND_SSOR
    r = np.random.default_rng(5).uniform(1.0, 50.0, f.u.shape)
    z = _z(p)
    yo = orc.precond_apply(p, dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u_old, f.v_old, r_al=r)
    with pkg.Solver(p) as s:
        s.state_set(f)
        yg = s.precond_apply(dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, r_al=r)
    for a, b in zip(_dofs(p, *yg, False), _dofs(p, *yo, False)):
        assert np.array_equal(a, b)


def test_jacobi_apply(gpu_pkg, orc):
    pkg = gpu_pkg
    p, f, dt = _cavity(pkg, orc, 30, 26)
    z = _z(p)
    yo = orc.precond_apply(p, dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, f.u_old, f.v_old)
    with pkg.Solver(p) as s:
        s.state_set(f)
        yg = s.precond_apply(dt, *z, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node)
    for a, b in zip(_dofs(p, *yg, True), _dofs(p, *yo, True)):
        assert np.allclose(a, b, rtol=4e-16, atol=0)


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _close(g, f, nx, ny, tol_u=1e-8, tol_p=1e-6):
    assert _rel(g.u, f.u) < tol_u, _rel(g.u, f.u)
    assert _rel(g.v, f.v) < tol_u, _rel(g.v, f.v)
    pg, pf = g.p[1:ny + 1, 1:nx + 1], f.p[1:ny + 1, 1:nx + 1]
    pg, pf = pg - pg.mean(), pf - pf.mean()
    assert _rel(pg, pf) < tol_p, _rel(pg, pf)


@pytest.mark.parametrize("solver", ["LINEAR_BICGSTAB2", "LINEAR_BICGSTAB"])
@pytest.mark.parametrize("prec", ["PRECOND_SSOR", "PRECOND_BLOCK_TRIANGULAR"])
def test_monolithic_step(gpu_pkg, orc, prec, solver):
    pkg = gpu_pkg
    cap = pkg.capi
    p, f, dt = _cavity(pkg, orc, 40, 40)
    p.precond = getattr(cap, prec)
    p.linear_solver = getattr(cap, solver)
    g = f.copy()
    it_o, st_o = orc.mono_step(p, dt, f, 0)
    with pkg.Solver(p) as s:
        it, st = s.monolithic_step(dt, g, has_nm1=0)
    assert st == st_o == 0
    # BiCGSTAB(2) counts in pairs; the coupled system is ill-conditioned
    # enough (the pressure level) that rounding moves the exit a little
    assert abs(it - it_o) <= max(4, 0.1 * it_o), (it, it_o)
    _close(g, f, p.nx, p.ny)


@pytest.mark.parametrize("prec", ["PRECOND_SSOR", "PRECOND_BLOCK_TRIANGULAR"])
def test_predictor(gpu_pkg, orc, prec):
    pkg = gpu_pkg
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=40, ny=72, nsub=4)
    p.linear_solver = cap.LINEAR_BICGSTAB2
    p.precond = getattr(cap, prec)
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
    it_o, st_o = orc.predictor(p, dt, f, has_nm1=0)
    with pkg.Solver(p) as s:
        it, st = s.predictor(dt, g, has_nm1=0)
    assert st == st_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    for a, b in ((g.u, f.u), (g.v, f.v)):
        assert _rel(a, b) < 1e-10


def test_al_step_with_ssor(gpu_pkg, orc):
    pkg = gpu_pkg
    cap = pkg.capi
    p, f, dt = _cavity(pkg, orc, 32, 32, solver=cap.SOLVER_AUGMENTED_LAGRANGIAN)
    p.precond = cap.PRECOND_SSOR
    p.r_al = 10.0
    f.rho[...] = 1.0
    g = f.copy()
    it_o, ud_o, st_o = orc.al_step(p, dt, f, 0)
    with pkg.Solver(p) as s:
        it, ud, st = s.al_step(dt, g, has_nm1=0)
    assert st == st_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    for a, b in ((g.u, f.u), (g.v, f.v), (g.p, f.p)):
        assert _rel(a, b) < 1e-8


def test_resident_monolithic_block_triangular(gpu_pkg, orc):
    """run_steps with a sweep preconditioner runs eagerly (graph refused by
    design) and tracks the oracle's time loop."""
    pkg = gpu_pkg
    cap = pkg.capi
    p, dt = pkg.cases.cavity_case(32)
    p.precond = cap.PRECOND_BLOCK_TRIANGULAR
    p.time_scheme = cap.TIME_GEAR
    f = pkg.Fields.allocate(p)
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    g = f.copy()
    nsteps = 4
    for k in range(nsteps):
        it, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    with pkg.Solver(p) as s:
        s.state_set(g)
        st, stats = s.run_steps(dt, nsteps, graph=True)
        assert st == 0, stats
        assert stats["graph"] == 0
        s.state_get(g)
    _close(g, f, p.nx, p.ny)


@pytest.mark.parametrize("gauge", ["pinned", "reference"])
@pytest.mark.parametrize("n", [48, 130])
def test_poisson_gauss_seidel_pcg(gpu_pkg, orc, n, gauge):
    """The pressure Poisson with p_precond SSOR (the reference's symmetric
    Gauss-Seidel pair, src/module_simulation.f90:2709-2758): the GPU's
    wavefront sweeps inside a host-driven FP64 PCG against the oracle."""
    pkg = gpu_pkg
    cap = pkg.capi
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=n, n_incl=12)
    p.p_gauge = cap.GAUGE_PINNED if gauge == "pinned" else cap.GAUGE_REFERENCE
    p.p_tol = 1e-12
    p.p_precond = cap.PRECOND_SSOR
    p.p_precision = cap.PREC_FP64
    ref = np.zeros_like(b)
    it_o, rr_o, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
    assert st_o == 0
    x = np.zeros_like(b)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
    assert st == cap.OK and rr <= 1e-12
    assert abs(it - it_o) <= max(2, it_o // 50), (it, it_o)
    err = np.linalg.norm(x[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
    assert err < 1e-10, err


def test_sp_steps_with_gauss_seidel_poisson(gpu_pkg, orc):
    pkg = gpu_pkg
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=32, ny=64, nsub=4)
    p.p_precond = cap.PRECOND_SSOR
    p.p_tol = 1e-12
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    g = f.copy()
    nsteps = 3
    for k in range(nsteps):
        it, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    with pkg.Solver(p) as s:
        s.state_set(g)
        st, stats = s.run_steps(dt, nsteps, graph=True)
        assert st == 0, stats
        assert stats["graph"] == 0
        s.state_get(g)
    for name in ("u", "v", "p"):
        a, b = getattr(g, name), getattr(f, name)
        assert _rel(a, b) < (1e-8 if name == "p" else 1e-9), name
