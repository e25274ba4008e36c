"""GPU predictor time schemes and convective variants against the oracle:
Gear / BDF2, Adams-Bashforth (AB2) and TVD-Superbee, through the C ABI.

* operator: bit-exact for every scheme, with and without the n-1 history;
* predictor solves: within 1e-10 of the oracle;
* resident time stepping (the first step without history runs eagerly, the
  rest replay CUDA graphs) and the batch engine against the oracle's time
  loop, u, v within 1e-9, p within 1e-8, C within 1e-12.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COMBOS = {
    "gear_ab2_centered": ("TIME_GEAR", "CONV_LIN_AB2", "CONV_CENTERED"),
    "gear_picard_tvd": ("TIME_GEAR", "CONV_LIN_PICARD", "CONV_TVD_SUPERBEE"),
    "euler_ab2_upwind": ("TIME_EULER", "CONV_LIN_AB2", "CONV_UPWIND"),
    "euler_picard_tvd": ("TIME_EULER", "CONV_LIN_PICARD", "CONV_TVD_SUPERBEE"),
}


def _set(pkg, p, combo):
    t, lin, sch = COMBOS[combo]
    p.time_scheme = getattr(pkg.capi, t)
    p.convective_linearization = getattr(pkg.capi, lin)
    p.convective_scheme = getattr(pkg.capi, sch)


def _state(pkg, orc, nx=40, ny=72, seed=31, vel=5e-2):
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
    f.u_nm1[...], f.v_nm1[...] = pkg.cases.random_velocity(p, vel, seed + 1)
    orc.apply_velocity_bc(p, f.u_nm1, f.v_nm1, False)
    return p, f, dt


@pytest.mark.parametrize("has_nm1", [0, 1])
@pytest.mark.parametrize("combo", list(COMBOS))
def test_operator_bit_exact(gpu_pkg, orc, combo, has_nm1):
    pkg = gpu_pkg
    p, f, dt = _state(pkg, orc)
    _set(pkg, p, combo)
    # u_old differs from u so that AB2 visibly advects with u_old
    f.u_old[...] = 0.5 * f.u + 0.5 * f.u_nm1
    f.v_old[...] = 0.5 * f.v + 0.5 * f.v_nm1
    rng = np.random.default_rng(7)
    xu, xv = rng.standard_normal(f.u.shape), rng.standard_normal(f.v.shape)
    hist = dict(u_old=f.u_old, v_old=f.v_old, u_nm1=f.u_nm1, v_nm1=f.v_nm1, has_nm1=has_nm1)
    yo = orc.momentum_apply(p, dt, xu, xv, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, **hist)
    with pkg.Solver(p) as s:
        yg = s.momentum_apply(dt, xu, xv, f.u, f.v, f.rho_u, f.rho_v, f.mu, f.mu_node, **hist)
    nx, ny = p.nx, p.ny
    assert np.array_equal(yg[0][1:ny + 1, 1:nx + 2], yo[0][1:ny + 1, 1:nx + 2])
    assert np.array_equal(yg[1][1:ny + 2, 1:nx + 1], yo[1][1:ny + 2, 1:nx + 1])


@pytest.mark.parametrize("combo", list(COMBOS))
def test_predictor_matches_oracle(gpu_pkg, orc, combo):
    pkg = gpu_pkg
    p, f, dt = _state(pkg, orc)
    _set(pkg, p, combo)
    p.linear_solver = pkg.capi.LINEAR_BICGSTAB
    p.tol = 1e-10
    g = f.copy()
    it_o, st_o = orc.predictor(p, dt, f, has_nm1=1)
    with pkg.Solver(p) as s:
        it, st = s.predictor(dt, g, has_nm1=1)
    assert st == st_o == 0
    assert abs(it - it_o) <= 2, (it, it_o)
    for a, b in ((g.u, f.u), (g.v, f.v)):
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-10


def _close(g, f):
    for name in ("u", "v", "p"):
        a, b = getattr(g, name), getattr(f, name)
        tol = 1e-8 if name == "p" else 1e-9
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < tol, name
    assert np.abs(g.C - f.C).max() <= 1e-12


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("combo", ["gear_ab2_centered", "gear_picard_tvd"])
def test_resident_steps_match_oracle(gpu_pkg, orc, combo, graph):
    pkg = gpu_pkg
    p, C0, dt = pkg.cases.bubble_case(nx=32, ny=64, nsub=4)
    _set(pkg, p, combo)
    p.p_tol = 1e-12
    p.tol = 1e-10
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    g = f.copy()
    nsteps = 5
    for k in range(nsteps):
        iu, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    with pkg.Solver(p) as s:
        assert s.has_nm1 == 0
        s.state_set(g)
        st, stats = s.run_steps(dt, 2, graph=graph)      # first step eager, then graphs
        assert st == 0 and s.has_nm1 == 1
        st, stats = s.run_steps(dt, nsteps - 2, graph=graph)
        assert st == 0 and stats["graph"] == int(graph)
        s.state_get(g)
    _close(g, f)
    # the history was rotated on the device
    assert np.linalg.norm(g.u_nm1 - f.u_nm1) / np.linalg.norm(f.u_nm1) < 1e-9


def test_host_sp_step_with_history_matches_oracle(gpu_pkg, orc):
    """covof_sp_step reads the handle's u_nm1 / v_nm1 and has_nm1."""
    pkg = gpu_pkg
    p, f, dt = _state(pkg, orc)
    _set(pkg, p, "gear_ab2_centered")
    p.p_tol = 1e-12
    p.tol = 1e-10
    g = f.copy()
    iu, ip, rr_o, st_o = orc.sp_step(p, dt, f, has_nm1=1)
    with pkg.Solver(p) as s:
        it, rr, st = s.sim_solve_standard_projection(dt, g, has_nm1=1)
    assert st == st_o == 0
    for name in ("u", "v", "p"):
        a, b = getattr(g, name), getattr(f, name)
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < (1e-9 if name == "p" else 1e-10), name


@pytest.mark.parametrize("mixed", [False, True])
def test_batch_with_history_matches_oracle(gpu_pkg, orc, mixed):
    pkg = gpu_pkg
    cases = []
    for q, (p, C0, dt) in enumerate(pkg.cases.droplet_batch(n_cases=4, seed=13, sizes=(32, 48), nsub=4,
                                                             mixed=mixed)):
        _set(pkg, p, ("gear_ab2_centered", "gear_picard_tvd")[q % 2])
        f = pkg.Fields.allocate(p)
        f.C[...] = C0
        orc.apply_vof_bc(p, f.C)
        orc.update_physical_properties(p, f)
        orc.compute_curvature_and_csf(p, f)
        cases.append((p, f, dt))
    nsteps = 4
    ref = []
    for p, f, dt in cases:
        g = f.copy()
        for k in range(nsteps):
            iu, ip, rr, st = orc.time_step(p, dt, k, g)
            assert st == 0
        ref.append(g)
    with pkg.Batch([c[0] for c in cases]) as b:
        for i, (p, f, dt) in enumerate(cases):
            b.state_set(i, f)
        st, stats, ms = b.run_steps([c[2] for c in cases], nsteps, graph=True)
        assert st == 0, stats
        out = []
        for i, (p, f, dt) in enumerate(cases):
            g = f.copy()
            b.state_get(i, g)
            out.append(g)
    for g, r in zip(out, ref):
        _close(g, r)
