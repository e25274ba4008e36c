"""The oracle's periodic branches (np = 1), pinned by the mathematics they
must satisfy: the wrapped Poisson operator is symmetric with every row
summing to the diagonal shift, converges at second order to a periodic
manufactured solution, and the Weymouth-Yue step on a periodic domain moves
the total volume only by round-off per step while a blob crosses the
boundary; the periodic ghost values are the wrapped interior values."""
from __future__ import annotations

import math

import numpy as np
import pytest


def _periodic(pkg, nx, ny, lx=1.0, ly=1.0, x=True, y=True):
    cap = pkg.capi
    p = pkg.cases.make_params(nx, ny, lx, ly)
    if x:
        p.bc_type[0] = p.bc_type[1] = cap.BC_PERIODIC
    if y:
        p.bc_type[2] = p.bc_type[3] = cap.BC_PERIODIC
    return p


def _faces_from_cells(rho, x, y):
    """Face densities of a periodic cell density (the ghost ring wrapped)."""
    r = rho.copy()
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


@pytest.mark.parametrize("x,y", [(True, False), (False, True), (True, True)])
def test_periodic_poisson_operator_symmetric_rows_sum_to_shift(pkg, orc, x, y):
    p = _periodic(pkg, 23, 17, 1.0, 0.7, x, y)
    rng = np.random.default_rng(2)
    rho = np.exp(rng.standard_normal((p.ny + 2, p.nx + 2)))
    ru, rv = _faces_from_cells(rho, x, y)
    dt = 0.3
    a = rng.standard_normal(rho.shape)
    b = rng.standard_normal(rho.shape)
    Aa = orc.poisson_matvec(p, dt, ru, rv, a)
    Ab = orc.poisson_matvec(p, dt, ru, rv, b)
    s1 = float((b[1:-1, 1:-1] * Aa[1:-1, 1:-1]).sum())
    s2 = float((a[1:-1, 1:-1] * Ab[1:-1, 1:-1]).sum())
    assert abs(s1 - s2) <= 1e-12 * (abs(s1) + abs(s2))
    if x and y:
        # no wall: every row of A 1 is the diagonal shift 1e-12 dvol, up to the
        # rounding of a_P (which sums the four faces and the shift)
        ones = np.zeros_like(a)
        ones[1:-1, 1:-1] = 1.0
        A1 = orc.poisson_matvec(p, dt, ru, rv, ones)[1:-1, 1:-1]
        e = np.zeros_like(a)
        e[1, 1] = 1.0
        scale = np.abs(orc.poisson_matvec(p, dt, ru, rv, e)).max()
        shift = 1e-12 * p.dx * p.dy
        assert np.abs(A1 - shift).max() <= 1e-14 * scale


def test_periodic_manufactured_solution_second_order(pkg, orc):
    errs = []
    for n in (32, 64, 128):
        p = _periodic(pkg, n, n)
        p.p_tol = 1e-13
        p.p_max_iter = 100000
        ru = np.ones((n + 2, n + 2))
        rv = np.ones((n + 2, n + 2))
        xc = (np.arange(n) + 0.5) / n
        X, Y = np.meshgrid(xc, xc)
        pe = np.zeros((n + 2, n + 2))
        pe[1:-1, 1:-1] = np.sin(2 * math.pi * X) * np.cos(4 * math.pi * Y)
        dt = 1.0
        # A p = -dt lap(p) dvol for unit density: b from the exact Laplacian
        b = np.zeros_like(pe)
        b[1:-1, 1:-1] = dt * (20.0 * math.pi ** 2) * pe[1:-1, 1:-1] * p.dx * p.dy
        b[1:-1, 1:-1] -= b[1:-1, 1:-1].mean()
        x = np.zeros_like(b)
        it, rr, st = orc.poisson_solve_rhs(p, dt, b, ru, rv, x)
        assert st == 0
        errs.append(np.abs(x[1:-1, 1:-1] - pe[1:-1, 1:-1]).max())
    assert errs[1] < errs[0] / 3.5 and errs[2] < errs[1] / 3.5, errs


def test_periodic_velocity_and_vof_ghosts_wrap(pkg, orc):
    p = _periodic(pkg, 9, 7)
    rng = np.random.default_rng(4)
    u = rng.standard_normal((p.ny + 2, p.nx + 2))
    v = rng.standard_normal(u.shape)
    C = rng.random(u.shape)
    orc.apply_velocity_bc(p, u, v, False)
    orc.apply_vof_bc(p, C)
    for f in (u, v):
        assert np.array_equal(f[1:-1, 0], f[1:-1, -2]) and np.array_equal(f[1:-1, -1], f[1:-1, 1])
        assert np.array_equal(f[0, 1:-1], f[-2, 1:-1]) and np.array_equal(f[-1, 1:-1], f[1, 1:-1])
    assert np.array_equal(C[1:-1, 0], C[1:-1, -2]) and np.array_equal(C[0, 1:-1], C[-2, 1:-1])


def test_periodic_refused_where_not_restated(pkg, orc):
    """One side periodic without its partner is invalid; the momentum path
    refuses periodic boundaries."""
    cap = pkg.capi
    p = pkg.cases.make_params(8, 8, 1.0, 1.0)
    p.bc_type[0] = cap.BC_PERIODIC
    z = np.zeros((10, 10))
    assert orc.lib().orc_apply_vof_bc(orc._params(p), orc._p(z)) == cap.INVALID
    q = _periodic(pkg, 8, 8)
    f = pkg.Fields.allocate(q)
    it, st = orc.predictor(q, 1e-3, f)
    assert st == cap.UNSUPPORTED


@pytest.mark.parametrize("recon", ["plic", "elvira"])
def test_periodic_wy_blob_crosses_boundary(pkg, orc, recon):
    cap = pkg.capi
    n = 48
    p = _periodic(pkg, n, n)
    p.recon = cap.RECON_PLIC if recon == "plic" else cap.RECON_ELVIRA
    p.enable_two_phase = 1
    # a disc near the north-east corner, moving diagonally across both
    # periodic boundaries
    C = pkg.cases.subsample_fraction(n, n, p.dx, p.dy,
                                     lambda X, Y: np.hypot(X - 0.85, Y - 0.8) < 0.12, 8)
    orc.apply_vof_bc(p, C)
    u = np.full_like(C, 0.6)
    v = np.full_like(C, 0.45)
    dt = 0.4 * p.dx
    v0 = C[1:-1, 1:-1].sum()
    prev = v0
    for k in range(60):
        orc.wy_step(p, dt, k % 2 == 0, u, v, C)
        orc.apply_vof_bc(p, C)
        # the fluxes through the periodic faces cancel; what moves the total
        # is the clamp to [0, 1] after the second pass (the reference's own
        # behaviour, as on an open domain): round-off per step
        vol = C[1:-1, 1:-1].sum()
        assert abs(vol - prev) <= 1e-12 * v0, k
        prev = vol
    assert abs(prev - v0) <= 2e-11 * v0
    # the blob moved across both boundaries: mass on the west / south sides now
    assert C[1:-1, 1:n // 4].sum() > 0.1 * v0 and C[1:n // 4, 1:-1].sum() > 0.1 * v0
