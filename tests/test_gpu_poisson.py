"""GPU Poisson parity (through the C ABI) against the oracle."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inclusions(pkg, n, k):
    return pkg.cases.poisson_inclusions(n=n, n_incl=k)


def test_operator_is_bit_identical(gpu_pkg, orc):
    pkg = gpu_pkg
    p, b, ru, rv, dt = _inclusions(pkg, 96, 8)
    x = np.random.default_rng(5).standard_normal(b.shape)
    y_o = orc.poisson_matvec(p, dt, ru, rv, x)
    with pkg.Solver(p) as s:
        y_g = s.poisson_apply(dt, ru, rv, x)
    assert np.array_equal(y_g[1:-1, 1:-1], y_o[1:-1, 1:-1])


@pytest.mark.parametrize("gauge", ["pinned", "reference"])
@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_strips", "mixed_cluster16", "mixed_cluster4", "mixed_stream", "mixed_cg", "mixed_mg",
                                  "mixed_mg_plain", "mixed_mg_gridtail", "mixed_mg_nuc32", "fp64_mg", "fp64_mg_gridtail"])
@pytest.mark.parametrize("n", [64, 128])
def test_solve_matches_oracle(gpu_pkg, orc, n, prec, gauge):
    pkg = gpu_pkg
    cap = pkg.capi
    p, b, ru, rv, dt = _inclusions(pkg, n, 12)
    p.p_gauge = cap.GAUGE_PINNED if gauge == "pinned" else cap.GAUGE_REFERENCE
    p.p_tol = 1e-12
    ref = np.zeros_like(b)
    it_o, rr_o, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
    assert st_o == 0
    q = p.copy()
    q.p_precision = cap.PREC_FP64 if prec == "fp64" else cap.PREC_MIXED
    q.p_inner_kind = cap.INNER_CHEBYSHEV
    if prec.startswith("fp64_mg"):
        # the multigrid flexible CG with the V-cycle in FP64
        q.p_precision = cap.PREC_FP64_MG
        q.p_inner_kind = cap.INNER_MG
        if prec == "fp64_mg_gridtail":
            q.p_mg_tail = 1
    if prec == "mixed_stream":
        q.p_inner_kind = cap.INNER_CHEBYSHEV_STREAM
    elif prec == "mixed_cg":
        q.p_inner_kind = cap.INNER_CG
    elif prec == "mixed_mg":
        q.p_inner_kind = cap.INNER_MG
    elif prec == "mixed_mg_plain":
        # plain coarse correction, one smoothing sweep each way
        q.p_inner_kind = cap.INNER_MG
        q.p_mg_nu = 1
        q.p_mg_cw = 1.0
    elif prec == "mixed_mg_gridtail":
        # no shared-memory tail: every level over the grid
        q.p_inner_kind = cap.INNER_MG
        q.p_mg_tail = 1
    elif prec == "mixed_mg_nuc32":
        # the coarsest level by 32 sweeps instead of its exact inverse: the
        # tail's W-cycle visits it twice
        q.p_inner_kind = cap.INNER_MG
        q.p_mg_nuc = 32
    x = np.zeros_like(b)
    with pkg.Solver(q) as s:
        # "mixed" on these meshes is the strip form on every SM; the strip form
        # and clusters of 16 and 4 CTAs are also selected explicitly
        form = {"mixed_strips": (1, 0), "mixed_cluster16": (3, 16), "mixed_cluster4": (3, 4)}.get(prec)
        if form:
            import ctypes
            L = cap.Launch(p_threads=0, p_blocks=form[1], p_inner_form=form[0])
            assert s.lib.covof_set_launch(s.h, ctypes.byref(L)) == cap.OK
            G = cap.Launch()
            s.lib.covof_get_launch(s.h, ctypes.byref(G))
            assert G.p_inner_form == form[0]
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
    assert st == cap.OK
    assert rr <= 1e-12
    err = np.linalg.norm(x[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
    # the parity bar for p is 1e-10 relative L2
    assert err < 1e-10, err
    if prec == "fp64":
        assert abs(it - it_o) <= max(3, it_o // 50), (it, it_o)


def test_reference_settings_from_velocity(gpu_pkg, orc):
    """Reference-literal tolerance (1e-7, reference gauge) from a predicted
    velocity: same iterations within a few, same pressure within the tolerance."""
    pkg = gpu_pkg
    p, C0, _ = pkg.cases.bubble_case(nx=48, ny=96, nsub=4)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    u, v = pkg.cases.random_velocity(p, 1e-2, 3)
    p.p_tol = 1e-7
    p.p_max_iter = 1000
    ref = np.zeros_like(u)
    it_o, rr_o, st_o = orc.poisson_solve(p, 1e-4, u, v, f.rho_u, f.rho_v, ref)
    x = np.zeros_like(u)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve(1e-4, u, v, f.rho_u, f.rho_v, x)
    assert st == st_o
    assert abs(it - it_o) <= 3
    d = np.linalg.norm(x - ref) / np.linalg.norm(ref)
    assert d < 1e-5, d


def test_maxiter_status_and_iterate_returned(gpu_pkg, orc):
    pkg = gpu_pkg
    p, b, ru, rv, dt = _inclusions(pkg, 64, 6)
    p.p_tol = 1e-12
    p.p_max_iter = 7
    x = np.zeros_like(b)
    ref = np.zeros_like(b)
    _, _, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
    assert st == pkg.capi.MAXITER == st_o and it == 7
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-8


def test_zero_rhs_returns_immediately(gpu_pkg):
    pkg = gpu_pkg
    p, b, ru, rv, dt = _inclusions(pkg, 32, 2)
    b[...] = 0.0
    x = np.zeros_like(b)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
    assert st == 0 and it == 0 and np.all(x == 0)


def test_full_size_1024_converges_fp64_and_mixed(gpu_pkg, orc):
    """Full 1024^2 workload: both arithmetics reach ||r||/||b|| <= 1e-10; the
    true residual is re-checked with the oracle's operator; both solutions
    agree to 1e-8 (size-independent properties at the benchmark size)."""
    pkg = gpu_pkg
    cap = pkg.capi
    p, b, ru, rv, dt = _inclusions(pkg, 1024, 200)
    sols = {}
    for prec, kind in ((cap.PREC_FP64, 0), (cap.PREC_MIXED, cap.INNER_CHEBYSHEV),
                       (cap.PREC_MIXED, cap.INNER_CHEBYSHEV_STREAM), (cap.PREC_MIXED, cap.INNER_MG)):
        q = p.copy()
        q.p_precision = prec
        q.p_inner_kind = kind
        x = np.zeros_like(b)
        with pkg.Solver(q) as s:
            it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
        assert st == cap.OK, (prec, st, it, rr)
        Ax = orc.poisson_matvec(q, dt, ru, rv, x)
        r = (b - Ax)[1:-1, 1:-1].copy()
        r[0, 0] = 0.0  # pinned cell
        true_rel = np.linalg.norm(r) / np.linalg.norm(b[1:-1, 1:-1])
        # mixed: the stopping test is the true FP64 residual itself; plain
        # FP64: the recursive residual (as the reference) -- its gap to the
        # true residual grows with the condition number (~1e7 here).
        assert true_rel < (2e-10 if prec == cap.PREC_MIXED else 1e-9), (prec, true_rel)
        assert x[1, 1] == 0.0
        sols[(prec, kind)] = x
    ref = sols[(cap.PREC_FP64, 0)]
    for key, x in sols.items():
        d = np.linalg.norm(x - ref) / np.linalg.norm(ref)
        assert d < 1e-7, (key, d)


def test_pinned_mixed_mg_route_with_large_level(gpu_pkg, orc):
    """Pinned gauge, mixed multigrid: a pressure with a large level against
    its right-hand side (a hydrostatic-like ramp, dt 1e-8) makes the
    reference-gauge route miss the pinned tolerance, so the pinned solve
    reruns and the next solves go to it directly before the route is tried
    again.  Every one of eleven solves on the same handle, cold and warm
    started, matches the oracle's pinned solution."""
    pkg = gpu_pkg
    cap = pkg.capi
    p, _, ru, rv, _ = _inclusions(pkg, 128, 12)
    dt = 1.0e-8
    p.p_gauge = cap.GAUGE_PINNED
    p.p_tol = 1e-12
    ny = p.ny
    ramp = np.zeros((ny + 2, p.nx + 2))
    ramp[1:-1, 1:-1] = (np.arange(ny, dtype=np.float64) + 0.5)[:, None] * 10.0
    b0 = orc.poisson_matvec(p, dt, ru, rv, ramp)
    rng = np.random.default_rng(11)
    q = p.copy()
    q.p_precision = cap.PREC_MIXED
    q.p_inner_kind = cap.INNER_MG
    x = np.zeros_like(b0)
    with pkg.Solver(q) as s:
        for k in range(11):
            b = b0.copy()
            b[1:-1, 1:-1] *= 1.0 + 1e-3 * k
            b[1:-1, 1:-1] += 1e-3 * np.abs(b0).max() * rng.standard_normal((ny, p.nx))
            ref = np.zeros_like(b)
            _, _, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
            assert st_o == 0
            if k % 2 == 0:
                x[...] = 0.0  # cold start; odd solves start from the last solution
            it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
            assert st == cap.OK, (k, st, it, rr)
            assert rr <= 1e-12, (k, rr)
            assert x[1, 1] == 0.0
            err = np.linalg.norm(x[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
            assert err < 1e-10, (k, err)


@pytest.mark.parametrize("prec", ["mixed_mg", "fp64_mg"])
@pytest.mark.parametrize("gauge", ["pinned", "reference"])
@pytest.mark.parametrize("nx,ny,lx,ly", [(64, 256, 1.0, 1.0), (256, 48, 1.0, 1.0), (96, 96, 1.0, 4.0)])
def test_multigrid_on_anisotropic_cells(gpu_pkg, orc, nx, ny, lx, ly, prec, gauge):
    """Cells of aspect 4:1 to 1:5 (the hierarchy halves only the strongly
    coupled direction until the cells are near square, 2 x 1 and 1 x 2
    aggregates), log-normal random density: the solution matches the
    oracle's converged Jacobi-PCG to 1e-10."""
    pkg = gpu_pkg
    cap = pkg.capi
    p = pkg.cases.make_params(nx, ny, lx, ly)
    rng = np.random.default_rng(nx + 7 * ny)
    rho = np.exp(2.0 * rng.standard_normal((ny + 2, nx + 2)))
    ru = np.ones_like(rho)
    rv = np.ones_like(rho)
    ru[1:-1, 1:] = 0.5 * (rho[1:-1, :-1] + rho[1:-1, 1:])
    rv[1:, 1:-1] = 0.5 * (rho[:-1, 1:-1] + rho[1:, 1:-1])
    b = np.zeros_like(rho)
    b[1:-1, 1:-1] = rng.standard_normal((ny, nx))
    b[1:-1, 1:-1] -= b[1:-1, 1:-1].mean()
    p.p_gauge = cap.GAUGE_PINNED if gauge == "pinned" else cap.GAUGE_REFERENCE
    p.p_tol = 1e-12
    p.p_max_iter = 1000000
    ref = np.zeros_like(b)
    _, _, st_o = orc.poisson_solve_rhs(p, 1e-3, b, ru, rv, ref)
    assert st_o == 0
    q = p.copy()
    q.p_precision = cap.PREC_MIXED if prec == "mixed_mg" else cap.PREC_FP64_MG
    q.p_inner_kind = cap.INNER_MG
    x = np.zeros_like(b)
    with pkg.Solver(q) as s:
        it, rr, st = s.poisson_solve_rhs(1e-3, b, ru, rv, x)
        outer = s.last_refine_steps()
    err = np.linalg.norm(x[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
    print(f"anisotropic {nx}x{ny} on {lx}x{ly} {prec} {gauge}: {outer} V-cycles, err {err:.2e}")
    assert st == cap.OK and rr <= 1e-12
    assert err < 1e-10, err


def test_semicoarsening_keeps_the_v_cycle_count(gpu_pkg):
    """A two-layer density (3 over 1, the Rayleigh-Taylor set-up) on 256^2
    cells of a [0,1] x [0,4] domain (cells 4:1): with the direction of the
    strong couplings halved first, the flexible CG needs about as many
    V-cycles as on square cells (full 2 x 2 aggregation needs several times
    more on this mesh)."""
    import math
    pkg = gpu_pkg
    cap = pkg.capi
    n = 256
    p = pkg.cases.make_params(n, n, 1.0, 4.0)
    xc = (np.arange(n) + 0.5) * p.dx
    yc = (np.arange(n) + 0.5) * p.dy
    X, Y = np.meshgrid(xc, yc)
    rho = np.ones((n + 2, n + 2))
    rho[1:-1, 1:-1] = np.where(Y > 2.0 + 0.05 * np.cos(2 * math.pi * X), 3.0, 1.0)
    rho[0, :], rho[-1, :], rho[:, 0], rho[:, -1] = rho[1, :], rho[-2, :], rho[:, 1], rho[:, -2]
    ru = np.ones_like(rho)
    rv = np.ones_like(rho)
    ru[1:-1, 1:] = 0.5 * (rho[1:-1, :-1] + rho[1:-1, 1:])
    rv[1:, 1:-1] = 0.5 * (rho[:-1, 1:-1] + rho[1:, 1:-1])
    b = np.zeros_like(rho)
    b[1:-1, 1:-1] = np.random.default_rng(4).standard_normal((n, n))
    b[1:-1, 1:-1] -= b[1:-1, 1:-1].mean()
    p.p_precision = cap.PREC_MIXED
    p.p_inner_kind = cap.INNER_MG
    p.p_tol = 1e-10
    p.p_max_iter = 1000000
    x = np.zeros_like(b)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve_rhs(2e-5, b, ru, rv, x)
        outer = s.last_refine_steps()
    print(f"two-layer 256^2 on 1x4: {outer} V-cycles")
    assert st == cap.OK and rr <= 1e-10
    assert outer <= 60, outer
