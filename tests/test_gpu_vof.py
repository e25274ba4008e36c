"""GPU geometric VOF parity: bit-exact against the oracle (the VOF kernels
evaluate every expression in reference order without FMA contraction)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bubble(pkg, orc, nx=64, ny=128):
    p, C0, dt = pkg.cases.bubble_case(nx=nx, ny=ny, nsub=8)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    return p, f, dt


def _random_C(n, seed):
    rng = np.random.default_rng(seed)
    C = rng.uniform(0, 1, (n + 2, n + 2))
    C[C < 0.3] = 0.0
    C[C > 0.7] = 1.0
    return C


@pytest.mark.parametrize("recon", ["PLIC", "ELVIRA"])
def test_reconstruct_bit_exact(gpu_pkg, orc, recon):
    pkg = gpu_pkg
    p, f, _ = _bubble(pkg, orc)
    p.recon = getattr(pkg.capi, "RECON_" + recon)
    for Cf in (f.C, np.ascontiguousarray(_random_C(p.nx, 1)[:p.ny + 2, :] if p.nx == p.ny else f.C)):
        s_o = orc.reconstruct(p, Cf)
        with pkg.Solver(p) as s:
            s_g = s.reconstruct_interface(Cf)
        assert np.array_equal(s_g, s_o)
    # ragged random fields (many pure/mixed transitions, ghost-ring cases):
    # 37^2 (about 500 interface cells: ELVIRA's block-per-cell form on a
    # 152-SM part) and 80^2 (about 2500: the warp-per-cell form)
    for nr in (37, 80):
        q = pkg.cases.make_params(nr, nr, 1.0, 1.0)
        q.recon = p.recon
        Cr = _random_C(nr, 2)
        with pkg.Solver(q) as s:
            assert np.array_equal(s.reconstruct_interface(Cr), orc.reconstruct(q, Cr))


@pytest.mark.parametrize("recon", ["PLIC", "ELVIRA"])
def test_reconstruct_thread_per_cell_form_bit_exact(gpu_pkg, orc, recon):
    """The thread-per-cell reconstruction (long interface lists) forced on
    small cases through covof_launch.vof_cell_min = 1: bit-identical to the
    oracle, bubble and ragged random fields (ghost-ring cells in the list);
    the handle reports the threshold it uses, the built-in 16384 by default."""
    import ctypes
    pkg = gpu_pkg
    cap = pkg.capi
    p, f, _ = _bubble(pkg, orc)
    p.recon = getattr(cap, "RECON_" + recon)
    q = pkg.cases.make_params(37, 37, 1.0, 1.0)
    q.recon = p.recon
    for prm, Cf in ((p, f.C), (q, _random_C(37, 2)), (q, _random_C(37, 5))):
        with pkg.Solver(prm) as s:
            G = cap.Launch()
            assert s.lib.covof_get_launch(s.h, ctypes.byref(G)) == cap.OK and G.vof_cell_min == 16384
            L = cap.Launch(p_threads=0, p_blocks=0, p_inner_form=0, vof_cell_min=1)
            assert s.lib.covof_set_launch(s.h, ctypes.byref(L)) == cap.OK
            assert np.array_equal(s.reconstruct_interface(Cf), orc.reconstruct(prm, Cf))
    with pkg.Solver(q) as s:
        bad = cap.Launch(p_threads=0, p_blocks=0, p_inner_form=0, vof_cell_min=-1)
        assert s.lib.covof_set_launch(s.h, ctypes.byref(bad)) == cap.INVALID


@pytest.mark.parametrize("recon", ["PLIC", "ELVIRA"])
@pytest.mark.parametrize("x_first", [True, False])
def test_wy_step_bit_exact(gpu_pkg, orc, recon, x_first):
    pkg = gpu_pkg
    p, f, _ = _bubble(pkg, orc)
    p.recon = getattr(pkg.capi, "RECON_" + recon)
    u, v = pkg.cases.random_velocity(p, 0.5, 7)
    dt = 0.2 * p.dx
    Co = f.C.copy()
    orc.wy_step(p, dt, x_first, u, v, Co)
    Cg = f.C.copy()
    with pkg.Solver(p) as s:
        s.advect_vof_weymouth_yue(dt, u, v, Cg, x_first)
    assert np.array_equal(Cg, Co)


def test_advect_with_properties_and_csf_bit_exact(gpu_pkg, orc):
    pkg = gpu_pkg
    p, f, dt = _bubble(pkg, orc)
    u, v = pkg.cases.random_velocity(p, 0.5, 9)
    f.u[...] = u
    f.v[...] = v
    g = f.copy()
    with pkg.Solver(p) as s:
        for k in range(4):
            orc.vof_advect(p, 0.2 * p.dx, k, f)
            s.advect_vof(0.2 * p.dx, g)
        assert s.vof_step_count == 4
    for name in ("C", "rho", "rho_u", "rho_v", "mu", "mu_node", "fx_sigma", "fy_sigma", "curvature"):
        assert np.array_equal(getattr(g, name), getattr(f, name)), name


def test_properties_single_phase_and_no_tension(gpu_pkg, orc):
    pkg = gpu_pkg
    p, f, _ = _bubble(pkg, orc, 32, 32)
    p.enable_two_phase = 0
    p.enable_surface_tension = 0
    g = f.copy()
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    with pkg.Solver(p) as s:
        s.update_physical_properties(g)
        s.compute_curvature_and_csf(g)
    for name in ("rho", "rho_u", "mu_node", "fx_sigma", "curvature"):
        assert np.array_equal(getattr(g, name), getattr(f, name)), name


def test_vortex_period_parity_and_conservation(gpu_pkg, orc):
    """Whole reversal period of the single-vortex case on the GPU: bit-equal
    to the oracle at every 100th step; volume conserved per step."""
    pkg = gpu_pkg
    cases = pkg.cases
    p, C0, dt, T = cases.vortex_case(64, recon=pkg.capi.RECON_ELVIRA)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    g = f.copy()
    v0 = f.C[1:-1, 1:-1].sum()
    t, k, worst, vprev = 0.0, 0, 0.0, v0
    with pkg.Solver(p) as s:
        while t < T - 1e-12:
            u, v = cases.vortex_velocity(p, t, dt, T)
            for F in (f, g):
                F.u[...] = u
                F.v[...] = v
                orc.apply_velocity_bc(p, F.u, F.v, False)
            orc.vof_advect(p, dt, k, f)
            s.advect_vof(dt, g)
            vk = g.C[1:-1, 1:-1].sum()
            worst = max(worst, abs(vk - vprev) / v0)
            vprev = vk
            if k % 100 == 0:
                assert np.array_equal(g.C, f.C), k
            t += dt
            k += 1
    assert np.array_equal(g.C, f.C)
    assert worst < 1e-12


@pytest.mark.parametrize("walls", ["noslip", "lid_freeslip"])
def test_boundary_condition_entries_bit_exact(gpu_pkg, orc, walls):
    """covof_apply_velocity_bc / covof_apply_vof_bc against the oracle's
    apply_velocity_bc / apply_vof_bc on random interior values."""
    pkg = gpu_pkg
    cap = pkg.capi
    p = pkg.cases.make_params(37, 29, 1.0, 0.8)
    if walls == "lid_freeslip":
        p.bc_type[0] = cap.BC_FREESLIP
        p.bc_u[3] = 1.0
        p.bc_v[1] = -0.25
    rng = np.random.default_rng(9)
    f = pkg.Fields.allocate(p)
    f.u[...] = rng.standard_normal(f.u.shape)
    f.v[...] = rng.standard_normal(f.v.shape)
    f.C[...] = rng.random(f.C.shape)
    g = f.copy()
    orc.apply_velocity_bc(p, f.u, f.v, False)
    orc.apply_vof_bc(p, f.C)
    with pkg.Solver(p) as s:
        s.apply_velocity_bc(g)
        s.apply_vof_bc(g)
    assert np.array_equal(g.u, f.u) and np.array_equal(g.v, f.v)
    assert np.array_equal(g.C, f.C)
