"""Hand-written adjoint of the projection (GPU, through the C ABI and the
torch binding) against an explicit transposed-matrix reference gradient and
central finite differences."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def droplet_case(pkg, n, seed, nd=8, ratio=100.0):
    """Seeded two-phase density (random droplets, ratio 100), MAC velocity u*
    (std 1e-2) and target (std 1e-4); dt = 1e-3."""
    cases = pkg.cases
    p = cases.make_params(n, n, 1.0, 1.0)
    rng = np.random.default_rng(seed)
    cx, cy, rr = rng.uniform(0.2, 0.8, nd), rng.uniform(0.2, 0.8, nd), rng.uniform(0.05, 0.15, nd)

    def inside(X, Y):
        m = np.zeros_like(X, dtype=bool)
        for a, b, r in zip(cx, cy, rr):
            m |= (X - a) ** 2 + (Y - b) ** 2 <= r * r
        return m

    C = cases.subsample_fraction(n, n, p.dx, p.dy, inside, 4)
    rho = ratio * C + (1.0 - C)
    rho_u = np.ones_like(rho)
    rho_v = np.ones_like(rho)
    rho_u[1:-1, 1:] = 0.5 * (rho[1:-1, :-1] + rho[1:-1, 1:])
    rho_v[1:, 1:-1] = 0.5 * (rho[:-1, 1:-1] + rho[1:, 1:-1])
    us, vs = cases.random_velocity(p, 1e-2, seed + 1)
    ut, vt = cases.random_velocity(p, 1e-4, seed + 2)
    p.p_tol = 1e-13
    p.p_max_iter = 200000
    return p, rho_u, rho_v, us, vs, ut, vt, 1e-3


@pytest.mark.parametrize("gauge", ["pinned", "reference"])
def test_vjp_matches_transposed_matrix_reference(gpu_pkg, orc, gauge):
    import adjoint_reference as ar
    pkg = gpu_pkg
    p, ru, rv, us, vs, ut, vt, dt = droplet_case(pkg, 24, 31)
    p.p_gauge = pkg.capi.GAUGE_PINNED if gauge == "pinned" else pkg.capi.GAUGE_REFERENCE
    x = np.zeros_like(us)
    with pkg.Solver(p) as s:
        u, v, it, rr, st = s.projection(dt, us, vs, ru, rv, x)
        assert st == 0
        gu, gv = u - ut, v - vt
        gxu, gxv, gbu, gbv, it, rr, st = s.projection_vjp(dt, ru, rv, x, gu, gv)
        assert st == 0
    ref = ar.vjp(orc, p, dt, ru, rv, us, vs, gu, gv, gauge == "pinned")
    for a, b, name in zip((gxu, gxv, gbu, gbv), ref, ("du", "dv", "dbeta_u", "dbeta_v")):
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(b), name


def _J(s, dt, us, vs, ru, rv, ut, vt):
    x = np.zeros_like(us)
    u, v, it, rr, st = s.projection(dt, us, vs, ru, rv, x)
    assert st == 0
    return 0.5 * (np.sum((u - ut) ** 2) + np.sum((v - vt) ** 2)), u, v, x


def test_gradients_match_central_finite_differences_512(gpu_pkg):
    """512^2 droplets (ratio 100): dJ/du* and dJ/d(1/rho_face) against central
    differences (eps = 1e-6) along 16 seeded random directions each; relative
    error <= 1e-6."""
    pkg = gpu_pkg
    p, ru, rv, us, vs, ut, vt, dt = droplet_case(pkg, 512, 41)
    p.p_gauge = pkg.capi.GAUGE_PINNED
    rng = np.random.default_rng(43)
    eps = 1e-6
    with pkg.Solver(p) as s:
        J0, u, v, x = _J(s, dt, us, vs, ru, rv, ut, vt)
        gxu, gxv, gbu, gbv, it, rr, st = s.projection_vjp(dt, ru, rv, x, u - ut, v - vt)
        assert st == 0
        worst = 0.0
        for k in range(16):
            du = rng.standard_normal(us.shape)
            dv = rng.standard_normal(vs.shape)
            Jp = _J(s, dt, us + eps * du, vs + eps * dv, ru, rv, ut, vt)[0]
            Jm = _J(s, dt, us - eps * du, vs - eps * dv, ru, rv, ut, vt)[0]
            fd = (Jp - Jm) / (2 * eps)
            ad = np.sum(gxu * du) + np.sum(gxv * dv)
            worst = max(worst, abs(fd - ad) / abs(ad))
        assert worst <= 1e-6, ("u*", worst)
        bu, bv = 1.0 / ru, 1.0 / rv
        worst = 0.0
        for k in range(16):
            db_u = bu * rng.standard_normal(ru.shape)
            db_v = bv * rng.standard_normal(rv.shape)
            Jp = _J(s, dt, us, vs, 1.0 / (bu + eps * db_u), 1.0 / (bv + eps * db_v), ut, vt)[0]
            Jm = _J(s, dt, us, vs, 1.0 / (bu - eps * db_u), 1.0 / (bv - eps * db_v), ut, vt)[0]
            fd = (Jp - Jm) / (2 * eps)
            ad = np.sum(gbu * db_u) + np.sum(gbv * db_v)
            worst = max(worst, abs(fd - ad) / abs(ad))
        assert worst <= 1e-6, ("beta", worst)


def test_torch_autograd_function(gpu_pkg):
    import importlib
    import torch
    pkg = gpu_pkg
    tb = importlib.import_module("covof_gb300.torch_binding")
    p, ru, rv, us, vs, ut, vt, dt = droplet_case(pkg, 32, 51)
    p.p_gauge = pkg.capi.GAUGE_PINNED
    dev = torch.device("cuda")
    T = lambda a: torch.from_numpy(a).to(dev)  # noqa: E731
    with pkg.Solver(p) as s:
        tus, tvs = T(us).requires_grad_(), T(vs).requires_grad_()
        tbu, tbv = (1.0 / T(ru)).requires_grad_(), (1.0 / T(rv)).requires_grad_()
        u, v, pr = tb.project(tus, tvs, tbu, tbv, s, dt)
        J = 0.5 * (((u - T(ut)) ** 2).sum() + ((v - T(vt)) ** 2).sum())
        J.backward()
        x = np.zeros_like(us)
        uu, vv, *_ = s.projection(dt, us, vs, ru, rv, x)
        ref = s.projection_vjp(dt, ru, rv, x, uu - ut, vv - vt)
    for t, r in zip((tus.grad, tvs.grad, tbu.grad, tbv.grad), ref[:4]):
        assert np.linalg.norm(t.cpu().numpy() - r) <= 1e-10 * max(np.linalg.norm(r), 1e-300)
    # gradcheck on a tiny grid (u* and beta), including a pressure term in the loss
    q = pkg.cases.make_params(6, 6, 1.0, 1.0)
    # solves driven to round-off (the tolerance is not reachable; the status
    # is MAXITER after 300 iterations on 36 unknowns): a stop anywhere in
    # [1e-15, 1e-14] would put 1e-5 of noise into the finite differences
    q.p_tol = 1e-16
    q.p_max_iter = 300
    q.p_gauge = pkg.capi.GAUGE_PINNED
    rng = np.random.default_rng(5)
    with pkg.Solver(q) as s2:
        u0 = T(rng.standard_normal((8, 8))).requires_grad_()
        v0 = T(rng.standard_normal((8, 8))).requires_grad_()
        b0 = T(rng.uniform(0.5, 2.0, (8, 8))).requires_grad_()
        c0 = T(rng.uniform(0.5, 2.0, (8, 8))).requires_grad_()

        def f(a, b, c, d):
            u, v, pr = tb.project(a, b, c, d, s2, 0.1)
            return (u[1:7, 2:7] ** 2).sum() + (v[2:7, 1:7] * v[2:7, 1:7]).sum() + (pr[1:7, 1:7] ** 3).sum()

        # rtol 1e-4: with eps = 1e-6 the finite differences carry the forward
        # solves' round-off (about cond * 1e-16 relative in p) divided by eps,
        # about 1e-5 of the cubic pressure term; the 1e-6 finite-difference
        # bar is checked on the 512^2 case with directional derivatives
        assert torch.autograd.gradcheck(f, (u0, v0, b0, c0), eps=1e-6, atol=1e-6, rtol=1e-4)
