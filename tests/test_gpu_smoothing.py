"""GPU interface smoothing against the oracle, through the C ABI:
SVOF Helmholtz smoothing (the wavefront Gauss-Seidel is bit-exact), explicit
diffusion smoothing, the properties and CSF forces that read them, and whole
time steps with smoothing on (resident, graph-replayed, and batched)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bubble(pkg, orc, nx, ny, svof=True, diffusion=False, width=1.0, steps=3):
    p, C0, dt = pkg.cases.bubble_case(nx=nx, ny=ny, nsub=4)
    p.enable_svof_smoothing = int(svof)
    p.svof_filter_width = width
    p.enable_diffusion_smoothing = int(diffusion)
    p.diffusion_smoothing_steps = steps
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    return p, f, dt


# sizes: below one band / one chunk, ragged bands and chunks, several of each
@pytest.mark.parametrize("nx,ny", [(8, 12), (20, 40), (64, 64), (97, 131), (200, 70)])
@pytest.mark.parametrize("width", [1.0, 2.5])
def test_svof_bit_exact(gpu_pkg, orc, nx, ny, width):
    pkg = gpu_pkg
    p, f, dt = _bubble(pkg, orc, nx, ny, width=width)
    g = f.copy()
    orc.svof_smooth(p, f)
    with pkg.Solver(p) as s:
        s.svof_smooth(g)
    assert np.array_equal(g.C_s, f.C_s)


@pytest.mark.parametrize("steps", [1, 3, 4])
def test_diffusion_bit_exact(gpu_pkg, orc, steps):
    pkg = gpu_pkg
    p, f, dt = _bubble(pkg, orc, 45, 70, svof=False, diffusion=True, steps=steps)
    g = f.copy()
    orc.diffusion_smooth(p, f)
    with pkg.Solver(p) as s:
        s.diffusion_smooth(g)
    assert np.array_equal(g.C_tilde, f.C_tilde)


@pytest.mark.parametrize("svof,diffusion", [(True, False), (False, True), (True, True)])
def test_properties_and_csf_bit_exact(gpu_pkg, orc, svof, diffusion):
    pkg = gpu_pkg
    p, f, dt = _bubble(pkg, orc, 48, 80, svof=svof, diffusion=diffusion)
    g = f.copy()
    orc.prepare_interface(p, f)
    with pkg.Solver(p) as s:
        if svof:
            s.svof_smooth(g)
        s.update_physical_properties(g)
        if diffusion:
            s.diffusion_smooth(g)
        s.compute_curvature_and_csf(g)
    for name in ("C_s", "C_tilde", "rho", "rho_u", "rho_v", "mu", "mu_node", "fx_sigma", "fy_sigma",
                 "curvature"):
        assert np.array_equal(getattr(g, name), getattr(f, name)), name


def test_vof_advect_with_smoothing_bit_exact(gpu_pkg, orc):
    pkg = gpu_pkg
    p, f, dt = _bubble(pkg, orc, 40, 72, svof=True, diffusion=True)
    orc.prepare_interface(p, f)
    f.u[...], f.v[...] = pkg.cases.random_velocity(p, 2e-1, 3)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    g = f.copy()
    with pkg.Solver(p) as s:
        for k in range(3):
            orc.vof_advect(p, 1e-2, k, f)
            s.advect_vof(1e-2, g)
    for name in ("C", "C_s", "C_tilde", "rho", "mu", "mu_node", "fx_sigma", "fy_sigma", "curvature"):
        assert np.array_equal(getattr(g, name), getattr(f, name)), name


def _close(g, f):
    for name in ("u", "v", "p"):
        a, b = getattr(g, name), getattr(f, name)
        tol = 1e-8 if name == "p" else 1e-9
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < tol, name
    assert np.abs(g.C - f.C).max() <= 1e-12
    assert np.abs(g.C_s - f.C_s).max() <= 1e-12


@pytest.mark.parametrize("graph", [False, True])
def test_resident_steps_with_smoothing(gpu_pkg, orc, graph):
    pkg = gpu_pkg
    p, f, dt = _bubble(pkg, orc, 32, 64, svof=True, diffusion=True)
    p.p_tol = 1e-12
    p.tol = 1e-10
    orc.prepare_interface(p, f)
    g = f.copy()
    for k in range(4):
        iu, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    with pkg.Solver(p) as s:
        s.state_set(g)
        st, stats = s.run_steps(dt, 4, graph=graph)
        assert st == 0 and stats["graph"] == int(graph)
        s.state_get(g)
    _close(g, f)


def test_batch_with_smoothing(gpu_pkg, orc):
    pkg = gpu_pkg
    cases = []
    for q, (p, C0, dt) in enumerate(pkg.cases.droplet_batch(n_cases=4, seed=17, sizes=(32, 48), nsub=4)):
        p.enable_svof_smoothing = 1 if q % 2 == 0 else 0
        p.enable_diffusion_smoothing = 1 if q % 3 == 0 else 0
        f = pkg.Fields.allocate(p)
        f.C[...] = C0
        orc.apply_vof_bc(p, f.C)
        orc.prepare_interface(p, f)
        cases.append((p, f, dt))
    nsteps = 3
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
