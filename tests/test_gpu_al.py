"""GPU augmented-Lagrangian coupling (solver_type AUGMENTED_LAGRANGIAN / AAL)
against the oracle, through the C ABI: single steps (covof_al_step) with one
and several Uzawa iterations, the divergence exit test, the adaptive penalty,
and resident time stepping (graph-replayed, and eager with the exit test)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(pkg, orc, solver="AUGMENTED_LAGRANGIAN", nx=40, ny=64, uzawa=1, tol=1e-12, adaptive=0):
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=nx, ny=ny, nsub=4)
    p.solver_type = getattr(cap, "SOLVER_" + solver)
    p.uzawa_iter = uzawa
    p.uzawa_tol = tol
    p.adaptative_al = adaptive
    if adaptive:
        p.t0_ref = 1.0  # keeps r near r_al (see tests/test_oracle_al.py)
        p.k_aal = 1.0
    p.tol = 1e-12
    p.max_iter = 2000
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.prepare_interface(p, f)
    f.u[...], f.v[...] = pkg.cases.random_velocity(p, 1e-2, 5)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    return p, f, dt


def _close(g, f, tol=1e-9):
    for name in ("u", "v", "p"):
        a, b = getattr(g, name), getattr(f, name)
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < tol, (name, np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("uzawa,solver,adaptive", [(1, "AUGMENTED_LAGRANGIAN", 0), (3, "AUGMENTED_LAGRANGIAN", 0),
                                                    (1, "AAL", 1), (2, "AAL", 1)])
def test_al_step_matches_oracle(gpu_pkg, orc, uzawa, solver, adaptive):
    pkg = gpu_pkg
    p, f, dt = _state(pkg, orc, solver=solver, uzawa=uzawa, tol=0.0, adaptive=adaptive)
    g = f.copy()
    it_o, ud_o, st_o = orc.al_step(p, dt, f)
    with pkg.Solver(p) as s:
        it, ud, st = s.al_step(dt, g)
    assert st == st_o == 0 and ud == ud_o == uzawa
    # later Uzawa iterations start from round-off-different states (the
    # assembled vs matrix-free operator), so their Krylov counts drift a little
    assert abs(it - it_o) <= 2 * uzawa + 0.1 * it_o, (it, it_o)
    _close(g, f)


def test_uzawa_exit_test_matches_oracle(gpu_pkg, orc):
    pkg = gpu_pkg
    p, f, dt = _state(pkg, orc, uzawa=40, tol=0.0)
    g = f.copy()
    orc.al_step(p, dt, g)
    d = (g.u[1:-1, 2:] - g.u[1:-1, 1:-1]) / p.dx + (g.v[2:, 1:-1] - g.v[1:-1, 1:-1]) / p.dy
    p.uzawa_tol = 30.0 * np.abs(d).max()
    h = f.copy()
    it_o, ud_o, st_o = orc.al_step(p, dt, f)
    with pkg.Solver(p) as s:
        it, ud, st = s.al_step(dt, h)
    assert st == st_o == 0 and 1 <= ud_o < 40 and ud == ud_o
    _close(h, f)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("uzawa,tol", [(1, 1e-12), (4, 1e-3)])
def test_resident_al_steps(gpu_pkg, orc, graph, uzawa, tol):
    pkg = gpu_pkg
    p, f, dt = _state(pkg, orc, uzawa=uzawa, tol=tol)
    f.u[...] = 0.0
    f.v[...] = 0.0
    g = f.copy()
    for k in range(3):
        iu, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    with pkg.Solver(p) as s:
        s.state_set(g)
        st, stats = s.run_steps(dt, 3, graph=graph)
        assert st == 0
        # with the Uzawa exit test on, the steps run eagerly
        assert stats["graph"] == int(graph and not (uzawa > 1 and tol > 0))
        s.state_get(g)
    _close(g, f, 1e-8)
    assert np.abs(g.C - f.C).max() <= 1e-12


def test_batch_rejects_al(gpu_pkg):
    pkg = gpu_pkg
    cases = pkg.cases.droplet_batch(n_cases=2, seed=3, sizes=(32,), nsub=4)
    ps = [c[0] for c in cases]
    ps[0].solver_type = pkg.capi.SOLVER_AUGMENTED_LAGRANGIAN
    with pytest.raises(pkg.CovofError):
        pkg.Batch(ps)


def test_caal_is_unsupported(gpu_pkg, orc):
    pkg = gpu_pkg
    p, f, dt = _state(pkg, orc)
    p.solver_type = pkg.capi.SOLVER_CAAL
    with pkg.Solver(p) as s:
        s.state_set(f)
        with pytest.raises(pkg.CovofError):
            s.run_steps(dt, 1)
