"""The pinned gauge solved through the reference gauge, restated on the
oracle (CPU): the identity the mixed multigrid path relies on.

Both gauges share the operator A (rows summing to e = A 1, the 1e-12 dvol
shift of the diagonal).  With F = b + kappa e off the pinned cell (1,1) and
F(1,1) = -(the sum of the others), the reference-gauge solution x of F,
shifted by -x(1,1), leaves the pinned residual (x(1,1) - kappa) e plus its
own residual; kappa = x(1,1) of that solution makes the first term vanish."""
from __future__ import annotations

import numpy as np
import pytest


def _route(orc, p, dt, b, ru, rv, kappa, cap):
    ones = np.zeros_like(b)
    ones[1:-1, 1:-1] = 1.0
    e = orc.poisson_matvec(p, dt, ru, rv, ones)
    F = b.copy()
    F[1:-1, 1:-1] += kappa * e[1:-1, 1:-1]
    F[1, 1] = 0.0
    F[1, 1] = -F[1:-1, 1:-1].sum()
    q = p.copy()
    q.p_gauge = cap.GAUGE_REFERENCE
    xr = np.zeros_like(b)
    _, _, st = orc.poisson_solve_rhs(q, dt, F, ru, rv, xr)
    assert st == 0
    c = xr[1, 1]
    x = xr.copy()
    x[1:-1, 1:-1] -= c
    return x, c, e


def _pinned_rel(orc, p, dt, b, ru, rv, x):
    r = (b - orc.poisson_matvec(p, dt, ru, rv, x))[1:-1, 1:-1].copy()
    r[0, 0] = 0.0
    bb = b[1:-1, 1:-1].copy()
    bb[0, 0] = 0.0
    return np.linalg.norm(r) / np.linalg.norm(bb)


def test_route_solves_the_pinned_system(pkg, orc):
    cap = pkg.capi
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=64, n_incl=8)
    p.p_tol = 1e-12
    b[1, 1] = 0.0
    xp = np.zeros_like(b)
    _, _, st = orc.poisson_solve_rhs(p, dt, b, ru, rv, xp)
    assert st == 0
    x, _, _ = _route(orc, p, dt, b, ru, rv, 0.0, cap)
    assert x[1, 1] == 0.0
    assert _pinned_rel(orc, p, dt, b, ru, rv, x) < 1e-11
    err = np.linalg.norm((x - xp)[1:-1, 1:-1]) / np.linalg.norm(xp[1:-1, 1:-1])
    assert err < 1e-9, err


@pytest.mark.parametrize("n", [48])
def test_route_level_mismatch_and_its_prediction(pkg, orc, n):
    """A large pressure level against its right-hand side (a ramp, dt 1e-8):
    with kappa = 0 the pinned residual is the predicted |x(1,1)| ||e||
    relative to ||b||.  kappa = x(1,1) of that run cuts it by the small
    response of the level to kappa (a contracting fixed point), and
    kappa = -mean(x0) of the converged pinned solution x0 -- a warm start
    from the previous solve of the same system -- brings it to the solves'
    own tolerance."""
    cap = pkg.capi
    p, _, ru, rv, _ = pkg.cases.poisson_inclusions(n=n, n_incl=4)
    dt = 1.0e-8
    p.p_gauge = cap.GAUGE_PINNED
    p.p_tol = 1e-12
    ramp = np.zeros((p.ny + 2, p.nx + 2))
    ramp[1:-1, 1:-1] = (np.arange(p.ny, dtype=np.float64) + 0.5)[:, None] * 10.0
    b = orc.poisson_matvec(p, dt, ru, rv, ramp)
    b[1, 1] = 0.0
    x0, c0, e = _route(orc, p, dt, b, ru, rv, 0.0, cap)
    rel0 = _pinned_rel(orc, p, dt, b, ru, rv, x0)
    ee = e[1:-1, 1:-1].copy()
    ee[0, 0] = 0.0
    bb = b[1:-1, 1:-1].copy()
    pred = abs(c0) * np.linalg.norm(ee) / np.linalg.norm(bb)
    assert rel0 > 1e-9
    assert abs(rel0 - pred) <= 0.05 * pred, (rel0, pred)
    x1, _, _ = _route(orc, p, dt, b, ru, rv, c0, cap)
    rel1 = _pinned_rel(orc, p, dt, b, ru, rv, x1)
    assert rel1 < 1e-3 * rel0, (rel1, rel0)
    xp = np.zeros_like(b)
    _, _, st = orc.poisson_solve_rhs(p, dt, b, ru, rv, xp)
    assert st == 0
    x2, _, _ = _route(orc, p, dt, b, ru, rv, -xp[1:-1, 1:-1].mean(), cap)
    rel2 = _pinned_rel(orc, p, dt, b, ru, rv, x2)
    assert rel2 < 1e-11, rel2
    err = np.linalg.norm((x2 - xp)[1:-1, 1:-1]) / np.linalg.norm(xp[1:-1, 1:-1])
    assert err < 1e-9, err
