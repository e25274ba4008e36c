"""GPU MONOLITHIC coupling against the oracle, through the C ABI: one
coupled (u, v, p) Krylov solve per step with the Schur diagonal as the
pressure block's Jacobi preconditioner (src/module_simulation.f90:552-583,
src/module_navier_stokes.f90:380-780, 1541-1590).

The GPU and the oracle run the same Krylov recurrences with different
rounding (assembled rows, parallel reductions), so converged results agree
to the solve tolerance, not bit for bit: velocities within 1e-7 relative,
the pressure within 1e-5 relative up to its level (held only by a 1e-10 dvol
regularisation of cell (1,1), which the Krylov tolerance leaves loose), the
iteration counts within 15 %.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cavity(pkg, orc, n, seed=3, vel=0.3):
    p, dt = pkg.cases.cavity_case(n)
    f = pkg.Fields.allocate(p)
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    if vel > 0:
        f.u[...], f.v[...] = pkg.cases.random_velocity(p, vel, seed)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    f.u_nm1[...] = f.u
    f.v_nm1[...] = f.v
    return p, f, dt


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def _close(g, f, nx, ny):
    assert _rel(g.u, f.u) < 1e-7, _rel(g.u, f.u)
    assert _rel(g.v, f.v) < 1e-7, _rel(g.v, f.v)
    pg, pf = g.p[1:ny + 1, 1:nx + 1], f.p[1:ny + 1, 1:nx + 1]
    pg, pf = pg - pg.mean(), pf - pf.mean()
    assert _rel(pg, pf) < 1e-5, _rel(pg, pf)


@pytest.mark.parametrize("n", [16, 40])
def test_single_step_matches_oracle(gpu_pkg, orc, n):
    pkg = gpu_pkg
    p, f, dt = _cavity(pkg, orc, n)
    g = f.copy()
    it_o, st_o = orc.mono_step(p, dt, f, 0)
    with pkg.Solver(p) as s:
        it, st = s.monolithic_step(dt, g, has_nm1=0)
    assert st == st_o == 0
    assert abs(it - it_o) <= max(4, 0.15 * it_o), (it, it_o)
    _close(g, f, p.nx, p.ny)


def test_hydrostatic_rest(gpu_pkg, orc):
    pkg = gpu_pkg
    p, C0, dt = pkg.cases.bubble_case(nx=16, ny=32, nsub=4)
    p.solver_type = pkg.capi.SOLVER_MONOLITHIC
    p.linear_solver = pkg.capi.LINEAR_BICGSTAB2
    p.max_iter = 5000
    f = pkg.Fields.allocate(p)
    f.C[...] = 1.0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    with pkg.Solver(p) as s:
        it, st = s.monolithic_step(dt, f, has_nm1=0)
    assert st == 0
    assert np.abs(f.u).max() < 1e-12 and np.abs(f.v).max() < 1e-12
    gp = (f.p[2:p.ny + 1, 1:-1] - f.p[1:p.ny, 1:-1]) / p.dy
    assert np.allclose(gp, p.rho1 * p.gy, rtol=1e-8, atol=0)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("scheme", ["euler_picard_upwind", "gear_ab2_centered"])
def test_resident_steps_match_oracle(gpu_pkg, orc, graph, scheme):
    pkg = gpu_pkg
    cap = pkg.capi
    p, f, dt = _cavity(pkg, orc, 24, vel=0.0)
    if scheme == "gear_ab2_centered":
        p.time_scheme = cap.TIME_GEAR
        p.convective_linearization = cap.CONV_LIN_AB2
        p.convective_scheme = cap.CONV_CENTERED
    g = f.copy()
    nsteps = 4
    for k in range(nsteps):
        it, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    with pkg.Solver(p) as s:
        s.state_set(g)
        st, stats = s.run_steps(dt, nsteps, graph=graph)
        assert st == 0, stats
        s.state_get(g)
    _close(g, f, p.nx, p.ny)


def test_batch_rejects_monolithic(gpu_pkg):
    pkg = gpu_pkg
    cases = pkg.cases.droplet_batch(n_cases=2, seed=3, sizes=(32,), nsub=4)
    ps = [c[0] for c in cases]
    ps[1].solver_type = pkg.capi.SOLVER_MONOLITHIC
    with pytest.raises(pkg.CovofError):
        pkg.Batch(ps)
