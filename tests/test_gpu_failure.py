"""Failure detection without a GPU fault.

* Bounded waits that run out: covof_set_wait_budget lowers the poll budget of
  every device-side wait to a handful of polls, so the blocks of a
  persistent solve give up at their barriers; the call returns COVOF_TIMEOUT
  (the kernel returns normally, nothing hangs or traps), and after the
  budget is restored the same handle solves correctly.
* Poisoned inputs: a NaN in the Poisson right-hand side gives COVOF_NAN on
  every arithmetic, as on the oracle; a NaN in the momentum right-hand side
  gives COVOF_NAN from the predictor.
* Zero-density faces: the assembly's rho < 1e-12 -> 1 guard
  (src/module_simulation.f90:2496) keeps the operator finite, bit for bit
  the oracle's, and the solve converges.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def wait_budget(gpu_pkg):
    lib = gpu_pkg.capi.load_library()
    yield lambda polls: lib.covof_set_wait_budget(polls)
    assert lib.covof_set_wait_budget(0) == gpu_pkg.capi.OK


@pytest.mark.parametrize("prec", ["fp64", "mixed_mg", "fp64_mg", "mixed_chebyshev"])
def test_waits_that_run_out_return_timeout_and_handle_recovers(gpu_pkg, orc, wait_budget, prec):
    pkg = gpu_pkg
    cap = pkg.capi
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=256, n_incl=12)
    p.p_tol = 1e-12
    p.p_precision = {"fp64": cap.PREC_FP64, "mixed_mg": cap.PREC_MIXED, "fp64_mg": cap.PREC_FP64_MG,
                     "mixed_chebyshev": cap.PREC_MIXED}[prec]
    p.p_inner_kind = cap.INNER_CHEBYSHEV if prec == "mixed_chebyshev" else cap.INNER_MG
    ref = np.zeros_like(b)
    _, _, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
    assert st_o == 0
    with pkg.Solver(p) as s:
        assert wait_budget(1) == cap.OK
        x = np.zeros_like(b)
        with pytest.raises(pkg.CovofError) as e:
            s.poisson_solve_rhs(dt, b, ru, rv, x)
        assert e.value.status == cap.TIMEOUT
        assert wait_budget(0) == cap.OK
        x[...] = 0.0
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
        assert st == cap.OK and rr <= 1e-12
    err = np.linalg.norm(x[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
    assert err < 1e-10, err


def test_resident_steps_report_timeout_then_continue(gpu_pkg, orc, wait_budget):
    """covof_run_steps folds a step's TIMEOUT into its statistics (the run
    does not stop, as the reference's silent Krylov exits); after the budget
    is restored the next steps on the same handle are clean."""
    pkg = gpu_pkg
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=64, ny=128, nsub=4)
    p.p_precision = cap.PREC_MIXED
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    import ctypes
    with pkg.Solver(p) as s:
        s.state_set(f)
        assert wait_budget(1) == cap.OK
        raw = cap.RunStats()
        st = s.lib.covof_run_steps(s.h, dt, 2, 0, ctypes.byref(raw))
        stats = raw.as_dict()
        # the call returns the first failing step's status, and both steps ran
        assert st == cap.TIMEOUT and stats["steps"] == 2, (st, stats)
        assert stats["first_bad_step"] == 0 and stats["first_bad_status"] == cap.TIMEOUT, stats
        assert wait_budget(0) == cap.OK
        s.state_set(f)
        st, stats = s.run_steps(dt, 2, graph=False)
        assert st == cap.OK and stats["first_bad_step"] == -1, stats


@pytest.mark.parametrize("prec", ["fp64", "mixed_mg", "fp64_mg", "sgs"])
def test_nan_rhs_returns_nan_status(gpu_pkg, orc, prec):
    pkg = gpu_pkg
    cap = pkg.capi
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=64, n_incl=4)
    b[20, 30] = np.nan
    p.p_gauge = cap.GAUGE_REFERENCE
    if prec == "sgs":
        p.p_precond = cap.PRECOND_SSOR
    else:
        p.p_precision = {"fp64": cap.PREC_FP64, "mixed_mg": cap.PREC_MIXED, "fp64_mg": cap.PREC_FP64_MG}[prec]
    ref = np.zeros_like(b)
    _, _, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
    assert st_o == cap.NAN
    x = np.zeros_like(b)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
    assert st == cap.NAN, cap.STATUS_NAMES.get(st)


def test_nan_momentum_source_returns_nan_status(gpu_pkg, orc):
    pkg = gpu_pkg
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=32, ny=64, nsub=4)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    f.fx_sigma[10, 10] = np.nan
    g = f.copy()
    it_o = orc.predictor(p, dt, g)
    with pkg.Solver(p) as s:
        it, st = s.predictor(dt, f)
    assert st == cap.NAN
    assert it_o[-1] == cap.NAN


def test_zero_density_faces_are_guarded(gpu_pkg, orc):
    pkg = gpu_pkg
    cap = pkg.capi
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=96, n_incl=6)
    rng = np.random.default_rng(3)
    for a in (ru, rv):
        mask = rng.random(a.shape) < 0.02
        a[mask] = 0.0
    x = rng.standard_normal(b.shape)
    y_o = orc.poisson_matvec(p, dt, ru, rv, x)
    assert np.all(np.isfinite(y_o))
    p.p_tol = 1e-12
    ref = np.zeros_like(b)
    _, _, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
    assert st_o == 0
    for prec in (cap.PREC_FP64, cap.PREC_MIXED):
        q = p.copy()
        q.p_precision = prec
        sol = np.zeros_like(b)
        with pkg.Solver(q) as s:
            y_g = s.poisson_apply(dt, ru, rv, x)
            it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, sol)
        assert np.array_equal(y_g[1:-1, 1:-1], y_o[1:-1, 1:-1])
        assert st == cap.OK and rr <= 1e-12
        err = np.linalg.norm(sol[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
        assert err < 1e-10, (prec, err)
