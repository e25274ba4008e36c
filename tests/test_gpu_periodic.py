"""Periodic boundaries on the GPU (one rank: the ghost ring holds the wrapped
interior), against the oracle's restatement of the reference's periodic
branches, for x-periodic, y-periodic and doubly periodic meshes:

* the Poisson operator's wrap (src/module_simulation.f90:2679-2701), bit for
  bit, and the plain FP64 Jacobi-PCG solve in both gauges;
* the projection correction's wrapped first face (:2602-2654), bit for bit;
* apply_velocity_bc's periodic ghosts and apply_vof_bc's (src/module_mpi_comm.f90:
  332-351, 636-683), bit for bit;
* reconstruct_interface's ghost ring after the normals' halo exchange, and
  the Weymouth-Yue step's periodic fluxes (src/module_interface_vof.f90:
  1223-1231, 1268-1276) with a blob crossing the boundaries, bit for bit
  over several steps, with advect_vof's properties and CSF;
* what stays closed: the momentum predictor, the multigrid and sweep
  Poisson solvers and the batch engine refuse periodic boundaries, and a
  periodic side without its partner is invalid.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIRS = [(True, False), (False, True), (True, True)]


def _periodic(pkg, nx, ny, lx, ly, x, y):
    cap = pkg.capi
    p = pkg.cases.make_params(nx, ny, lx, ly)
    if x:
        p.bc_type[0] = p.bc_type[1] = cap.BC_PERIODIC
    if y:
        p.bc_type[2] = p.bc_type[3] = cap.BC_PERIODIC
    return p


def _density(p, x, y, seed=1):
    rng = np.random.default_rng(seed)
    r = np.exp(2.0 * rng.standard_normal((p.ny + 2, p.nx + 2)))
    if x:
        r[:, 0] = r[:, -2]
        r[:, -1] = r[:, 1]
    if y:
        r[0, :] = r[-2, :]
        r[-1, :] = r[1, :]
    ru = np.ones_like(r)
    rv = np.ones_like(r)
    ru[1:-1, 1:] = 0.5 * (r[1:-1, :-1] + r[1:-1, 1:])
    rv[1:, 1:-1] = 0.5 * (r[:-1, 1:-1] + r[1:, 1:-1])
    return ru, rv


@pytest.mark.parametrize("x,y", DIRS)
def test_periodic_poisson_operator_bit_exact(gpu_pkg, orc, x, y):
    pkg = gpu_pkg
    p = _periodic(pkg, 45, 38, 1.0, 0.9, x, y)
    ru, rv = _density(p, x, y)
    xv = np.random.default_rng(3).standard_normal(ru.shape)
    y_o = orc.poisson_matvec(p, 0.7, ru, rv, xv)
    with pkg.Solver(p) as s:
        y_g = s.poisson_apply(0.7, ru, rv, xv)
    assert np.array_equal(y_g[1:-1, 1:-1], y_o[1:-1, 1:-1])


@pytest.mark.parametrize("gauge", ["reference", "pinned"])
@pytest.mark.parametrize("x,y", DIRS)
def test_periodic_fp64_pcg_matches_oracle(gpu_pkg, orc, x, y, gauge):
    pkg = gpu_pkg
    cap = pkg.capi
    p = _periodic(pkg, 96, 80, 1.0, 0.8, x, y)
    p.p_gauge = cap.GAUGE_PINNED if gauge == "pinned" else cap.GAUGE_REFERENCE
    p.p_tol = 1e-12
    p.p_max_iter = 100000
    ru, rv = _density(p, x, y, seed=5)
    b = np.zeros_like(ru)
    b[1:-1, 1:-1] = np.random.default_rng(6).standard_normal((p.ny, p.nx))
    b[1:-1, 1:-1] -= b[1:-1, 1:-1].mean()
    ref = np.zeros_like(b)
    it_o, rr_o, st_o = orc.poisson_solve_rhs(p, 1.0, b, ru, rv, ref)
    assert st_o == 0
    sol = np.zeros_like(b)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve_rhs(1.0, b, ru, rv, sol)
    assert st == cap.OK and rr <= 1e-12
    err = np.linalg.norm(sol[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
    assert err < 1e-10, err
    assert abs(it - it_o) <= max(3, it_o // 50), (it, it_o)


@pytest.mark.parametrize("x,y", DIRS)
def test_periodic_correction_and_ghosts_bit_exact(gpu_pkg, orc, x, y):
    pkg = gpu_pkg
    p = _periodic(pkg, 33, 27, 1.0, 0.8, x, y)
    ru, rv = _density(p, x, y, seed=7)
    rng = np.random.default_rng(8)
    f = pkg.Fields.allocate(p)
    f.u[...] = rng.standard_normal(f.u.shape)
    f.v[...] = rng.standard_normal(f.v.shape)
    f.p[...] = rng.standard_normal(f.p.shape)
    f.C[...] = rng.random(f.C.shape)
    g = f.copy()
    orc.project_correct(p, 1e-2, f.u, f.v, f.p, ru, rv)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    orc.apply_vof_bc(p, f.C)
    with pkg.Solver(p) as s:
        s.project_correct(1e-2, g.u, g.v, g.p, ru, rv)
        s.apply_velocity_bc(g)
        s.apply_vof_bc(g)
    assert np.array_equal(g.u, f.u) and np.array_equal(g.v, f.v)
    assert np.array_equal(g.C, f.C)


def _blob(pkg, p):
    return pkg.cases.subsample_fraction(p.nx, p.ny, p.dx, p.dy,
                                        lambda X, Y: np.hypot(X - 0.88, Y - 0.1) < 0.16, 8)


@pytest.mark.parametrize("recon", ["PLIC", "ELVIRA"])
@pytest.mark.parametrize("x,y", DIRS)
def test_periodic_reconstruct_and_wy_steps_bit_exact(gpu_pkg, orc, x, y, recon):
    """A blob at the east / south edges moving across both: the segments
    (ghost ring included) and C after each of eight Weymouth-Yue steps, both
    pass orders, equal the oracle's."""
    pkg = gpu_pkg
    cap = pkg.capi
    p = _periodic(pkg, 48, 40, 1.0, 0.8, x, y)
    p.recon = getattr(cap, "RECON_" + recon)
    p.enable_two_phase = 1
    C = _blob(pkg, p)
    orc.apply_vof_bc(p, C)
    Cg = C.copy()
    u = np.full_like(C, 0.7)
    v = np.full_like(C, -0.55)
    dt = 0.35 * p.dx
    with pkg.Solver(p) as s:
        assert np.array_equal(s.reconstruct_interface(Cg), orc.reconstruct(p, C))
        for k in range(8):
            orc.wy_step(p, dt, k % 2 == 0, u, v, C)
            orc.apply_vof_bc(p, C)
            s.advect_vof_weymouth_yue(dt, u, v, Cg, k % 2 == 0)
            f_tmp = pkg.Fields.allocate(p)
            f_tmp.C[...] = Cg
            s.apply_vof_bc(f_tmp)
            Cg[...] = f_tmp.C
            assert np.array_equal(Cg, C), k


@pytest.mark.parametrize("x,y", DIRS)
def test_periodic_advect_vof_bit_exact(gpu_pkg, orc, x, y):
    """advect_vof (Weymouth-Yue, the halo exchange and VOF BC, properties,
    curvature and CSF) on a periodic mesh, several steps."""
    pkg = gpu_pkg
    cap = pkg.capi
    p = _periodic(pkg, 40, 48, 0.8, 1.0, x, y)
    p.recon = cap.RECON_ELVIRA
    p.enable_two_phase = 1
    p.enable_surface_tension = 1
    p.rho1, p.rho2, p.mu1, p.mu2, p.sigma = 1000.0, 1.0, 1e-2, 1e-4, 0.07
    f = pkg.Fields.allocate(p)
    f.C[...] = _blob(pkg, p)
    orc.apply_vof_bc(p, f.C)
    rng = np.random.default_rng(9)
    f.u[...] = 0.5 + 0.1 * rng.standard_normal(f.u.shape)
    f.v[...] = 0.3 + 0.1 * rng.standard_normal(f.v.shape)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    g = f.copy()
    dt = 0.3 * p.dx
    with pkg.Solver(p) as s:
        for k in range(5):
            orc.vof_advect(p, dt, k, f)
            s.advect_vof(dt, g)
            for name in ("C", "rho", "rho_u", "rho_v", "mu", "mu_node", "fx_sigma", "fy_sigma", "curvature"):
                assert np.array_equal(getattr(g, name), getattr(f, name)), (k, name)


def test_periodic_refusals(gpu_pkg):
    pkg = gpu_pkg
    cap = pkg.capi
    p = _periodic(pkg, 32, 32, 1.0, 1.0, True, False)
    # multigrid / mixed / sweep Poisson solvers
    ru, rv = _density(p, True, False)
    b = np.zeros_like(ru)
    b[1:-1, 1:-1] = 1.0
    b[1:-1, 1:-1] -= b[1:-1, 1:-1].mean()
    for field, value in (("p_precision", cap.PREC_MIXED), ("p_precision", cap.PREC_FP64_MG),
                         ("p_precond", cap.PRECOND_SSOR)):
        q = p.copy()
        setattr(q, field, value)
        with pkg.Solver(q) as s:
            with pytest.raises(pkg.CovofError) as e:
                s.poisson_solve_rhs(1.0, b, ru, rv, np.zeros_like(b))
            assert e.value.status == cap.UNSUPPORTED
    # the momentum predictor and the batch engine
    with pkg.Solver(p) as s:
        with pytest.raises(pkg.CovofError) as e:
            s.predictor(1e-3, pkg.Fields.allocate(p))
        assert e.value.status == cap.UNSUPPORTED
    with pytest.raises(pkg.CovofError) as e:
        pkg.Batch([p])
    assert e.value.status == cap.UNSUPPORTED
    # one periodic side without its partner
    q = pkg.cases.make_params(16, 16, 1.0, 1.0)
    q.bc_type[0] = cap.BC_PERIODIC
    with pytest.raises(pkg.CovofError) as e:
        pkg.Solver(q)
    assert e.value.status == cap.INVALID
