"""Parity at the benchmark workloads' own sizes, against the oracle converged
far below the GPU's stopping test.

* The standalone variable-density Poisson at 1024^2 (200 inclusions, ratio
  1000, the headline workload), both gauges: every arithmetic the benchmark
  reports (plain FP64 Jacobi-PCG, FP64 flexible CG with the FP64 V-cycle,
  the mixed multigrid path, the mixed path with the FP32 Jacobi-CG inner
  iteration) against an oracle Jacobi-PCG solve to ||r||/||b|| <= 1e-14.
* The batch workload's size classes: one droplet / bubble case per mesh
  size 64 .. 512 in each direction (512^2 included), two batch steps.
* The Rayleigh-Taylor workload at 512^2 (its 4:1 domain), two resident steps.

Two solves stopped at ||r||/||b|| <= 1e-10 along different Krylov paths
differ by their truncation errors, which the condition number (about 1e7
at 1024^2 with a 1000:1 density contrast) can amplify; the tests therefore
check each arithmetic twice: at the workload's own 1e-10 (error against the
converged oracle stated and bounded), and at a tighter stopping test (1e-13
on the Poisson solves), where the parity bar of
1e-10 relative L2 on p applies.  Each test prints the errors it measured.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NTH = os.cpu_count() or 1


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def c2(gpu_pkg, orc):
    cap = gpu_pkg.capi
    p, b, ru, rv, dt = gpu_pkg.cases.poisson_inclusions(n=1024, n_incl=200)
    refs = {}
    for gauge in (cap.GAUGE_PINNED, cap.GAUGE_REFERENCE):
        q = p.copy()
        q.p_gauge = gauge
        q.p_tol = 1e-14
        q.p_max_iter = 1_000_000
        x = np.zeros_like(b)
        it, rr, st = orc.poisson_solve_rhs(q, dt, b, ru, rv, x, NTH)
        assert st == 0 and rr <= 1e-14, (gauge, it, rr, st)
        refs[gauge] = x
    return p, b, ru, rv, dt, refs


def _arm(cap, name):
    return {"fp64_jacobi": (cap.PREC_FP64, cap.INNER_MG),
            "fp64_mg": (cap.PREC_FP64_MG, cap.INNER_MG),
            "mixed_mg": (cap.PREC_MIXED, cap.INNER_MG),
            "mixed_jacobi_cg": (cap.PREC_MIXED, cap.INNER_CG)}[name]


# Errors measured at the workload's own stopping test (1e-10) against the
# converged oracle, pinned gauge: plain FP64 Jacobi-PCG 1.0e-11 (it follows the
# oracle's own Krylov path), FP64 / mixed multigrid 1.0e-9, the mixed
# Jacobi-CG inner 1.4e-8 (a weak inner iteration: the outer stops with more
# of the error left in the smooth modes, which the residual hardly sees).
# The bars below are about ten times those.  At 1e-13 the reference gauge is
# held to the parity bar of 1e-10 (measured <= 1.4e-12 for every arithmetic).
# The pinned gauge anchors the whole 1000:1 system at one cell and is far
# worse conditioned: the oracle's own pinned solution to 1e-14 and its
# reference-gauge solution to 1e-14 shifted to p(1,1) = 0 differ by 1.0e-9,
# so no pinned solve can be checked closer than that; there the bar is 1e-9
# (measured: Jacobi-PCG 8e-12 along the oracle's own path, the multigrid
# arms 1.7e-10 and 2.1e-10).
BAR_AT_1E10 = {"fp64_jacobi": 1e-10, "fp64_mg": 1e-8, "mixed_mg": 1e-8, "mixed_jacobi_cg": 1e-7}


@pytest.mark.parametrize("tol", [1e-10, 1e-13])
@pytest.mark.parametrize("arm", ["fp64_jacobi", "fp64_mg", "mixed_mg", "mixed_jacobi_cg"])
@pytest.mark.parametrize("gauge", ["pinned", "reference"])
def test_c2_poisson_matches_converged_oracle(c2, gpu_pkg, orc, arm, gauge, tol):
    pkg = gpu_pkg
    cap = pkg.capi
    p, b, ru, rv, dt, refs = c2
    q = p.copy()
    q.p_gauge = cap.GAUGE_PINNED if gauge == "pinned" else cap.GAUGE_REFERENCE
    q.p_precision, q.p_inner_kind = _arm(cap, arm)
    q.p_tol = tol
    q.p_max_iter = 10_000_000
    x = np.zeros_like(b)
    with pkg.Solver(q) as s:
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
    assert st == cap.OK, (arm, cap.STATUS_NAMES.get(st), it, rr)
    assert rr <= tol
    ref = refs[q.p_gauge]
    err = _rel(x[1:-1, 1:-1], ref[1:-1, 1:-1])
    print(f"C2 1024^2 {gauge} {arm} tol {tol:g}: {it} iterations, err_vs_oracle {err:.3e}")
    if q.p_gauge == cap.GAUGE_PINNED:
        assert x[1, 1] == 0.0
    if tol < 1e-12:
        bar = 1e-9 if gauge == "pinned" else 1e-10
    else:
        bar = BAR_AT_1E10[arm]
    assert err < bar, (arm, gauge, tol, err)


def _step_fields(pkg, orc, p, C0):
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    return f


def _oracle_steps(orc, p, f, dt, nsteps):
    q = p.copy()
    q.p_precision = 0
    q.p_tol = 1e-14
    q.p_max_iter = 10_000_000
    g = f.copy()
    orc.set_step_threads(NTH)
    try:
        for k in range(nsteps):
            iu, ip, rr, st = orc.time_step(q, dt, k, g)
            assert st == 0, (k, st)
    finally:
        orc.set_step_threads(1)
    return g


def _check_step_parity(label, g, r, tol):
    errs = {name: _rel(getattr(g, name), getattr(r, name)) for name in ("u", "v", "p")}
    cerr = float(np.abs(g.C - r.C).max())
    print(f"{label} tol {tol:g}: " + ", ".join(f"{k} {v:.3e}" for k, v in errs.items()) + f", C max-abs {cerr:.1e}")
    # Measured (mixed multigrid Poisson, BiCGSTAB predictor): at the
    # workloads' own 1e-10 u, v, p within 2.5e-9 (the Rayleigh-Taylor v, small
    # after two steps from rest, is the largest relative error); at 1e-13
    # within 1e-10.  The bars: 1e-8 at 1e-10, 2e-10 at 1e-13.  C: the VOF
    # step is bit-exact for a given velocity (test_gpu_vof); over whole steps
    # C inherits the velocity's round-off difference through the donor
    # regions' geometry (measured up to 2.9e-11): bar 1e-10.
    for name, e in errs.items():
        bar = 2e-10 if tol < 1e-12 else 1e-8
        assert e < bar, (label, name, e)
    assert cerr <= 1e-10, (label, cerr)


# every size class of the batch workload in each direction, 512^2 included
C4_SHAPES = [(64, 128), (128, 512), (256, 64), (512, 512), (512, 256)]


@pytest.mark.parametrize("tol", [1e-10, 1e-13])
def test_c4_size_classes_batch_steps_match_oracle(gpu_pkg, orc, tol):
    pkg = gpu_pkg
    cap = pkg.capi
    cases = pkg.cases.droplet_batch(shapes=C4_SHAPES, mixed=True)
    nsteps = 2
    ps, fs, dts = [], [], []
    for p, C0, dt in cases:
        p.p_inner_kind = cap.INNER_MG
        p.p_tol = tol
        p.tol = tol
        ps.append(p)
        fs.append(_step_fields(pkg, orc, p, C0))
        dts.append(dt)
    with pkg.Batch(ps) as bt:
        for i, f in enumerate(fs):
            bt.state_set(i, f)
        st, stats, ms = bt.run_steps(dts, nsteps, graph=True)
        assert st == cap.OK, stats
        out = []
        for i, f in enumerate(fs):
            g = f.copy()
            bt.state_get(i, g)
            out.append(g)
    for i, (p, f, dt) in enumerate(zip(ps, fs, dts)):
        assert stats[i]["first_bad_step"] == -1 and stats[i]["last_relres"] <= tol
        q = p.copy()
        q.tol = min(tol, 1e-12)
        r = _oracle_steps(orc, q, f, dt, nsteps)
        _check_step_parity(f"C4 case {p.nx}x{p.ny}", out[i], r, tol)


@pytest.mark.parametrize("tol", [1e-10, 1e-13])
def test_rt_512_resident_steps_match_oracle(gpu_pkg, orc, tol):
    pkg = gpu_pkg
    cap = pkg.capi
    p, C0, dt = pkg.cases.rt_case(nx=512, ny=512, mixed=True)
    p.p_inner_kind = cap.INNER_MG
    p.p_tol = tol
    p.tol = tol
    f = _step_fields(pkg, orc, p, C0)
    nsteps = 2
    g = f.copy()
    with pkg.Solver(p) as s:
        s.state_set(g)
        st, stats = s.run_steps(dt, nsteps, graph=True)
        assert st == cap.OK and stats["first_bad_step"] == -1, stats
        s.state_get(g)
    q = p.copy()
    q.tol = min(tol, 1e-12)
    r = _oracle_steps(orc, q, f, dt, nsteps)
    _check_step_parity("Rayleigh-Taylor 512^2", g, r, tol)
