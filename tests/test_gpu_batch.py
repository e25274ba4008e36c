"""Batch engine (covof_batch_*): many independent cases of uneven sizes in
one persistent launch per Krylov solve, against the oracle's time loop case
by case; graph replay against eager execution; FP64 and mixed batches."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases(pkg, orc, mixed, n=6, sizes=(32, 48, 64), seed=7):
    out = []
    for p, C0, dt in pkg.cases.droplet_batch(n_cases=n, seed=seed, sizes=sizes, nsub=4, mixed=mixed):
        f = pkg.Fields.allocate(p)
        f.C[...] = C0
        orc.apply_vof_bc(p, f.C)
        orc.update_physical_properties(p, f)
        orc.compute_curvature_and_csf(p, f)
        out.append((p, f, dt))
    return out


@pytest.mark.parametrize("mode", ["fp64", "mixed", "mixed_stream", "mixed_mg", "fp64_mg"])
def test_batch_matches_oracle_per_case(gpu_pkg, orc, mode):
    pkg = gpu_pkg
    mixed = mode not in ("fp64", "fp64_mg")
    cases = _cases(pkg, orc, mixed)
    if mode == "fp64_mg":
        for p, f, dt in cases:
            p.p_precision = pkg.capi.PREC_FP64_MG
    kind = {"mixed": pkg.capi.INNER_CHEBYSHEV, "mixed_stream": pkg.capi.INNER_CHEBYSHEV_STREAM,
            "mixed_mg": pkg.capi.INNER_MG}.get(mode)
    if kind is not None:
        for p, f, dt in cases:
            p.p_inner_kind = kind
    nsteps = 3
    ref = []
    for p, f, dt in cases:
        g = f.copy()
        for k in range(nsteps):
            iu, ip, rr, st = orc.time_step(p, dt, k, g)
            assert st == 0
        ref.append(g)
    with pkg.Batch([c[0] for c in cases]) as b:
        info = b.info()
        assert info["poisson_teams"] >= 1 and info["poisson_blocks"] >= 1
        for i, (p, f, dt) in enumerate(cases):
            b.state_set(i, f)
        st, stats, ms = b.run_steps([c[2] for c in cases], nsteps, graph=True)
        assert st == 0, stats
        out = []
        for i, (p, f, dt) in enumerate(cases):
            g = f.copy()
            b.state_get(i, g)
            out.append(g)
    for i, (g, r) in enumerate(zip(out, ref)):
        assert stats[i]["steps"] == nsteps and stats[i]["first_bad_step"] == -1
        assert stats[i]["last_relres"] <= 1e-10
        for name in ("u", "v", "p"):
            a, e = getattr(g, name), getattr(r, name)
            # u, v 1e-9; p 1e-8 -- Krylov paths stopped at 1e-10 that are not
            # the oracle's bit for bit (mixed Poisson; assembled predictor
            # operator) differ by up to cond * 1e-10, and div(u*) amplifies
            # predictor differences into p (measured up to 1.7e-9)
            tol = 1e-8 if name == "p" else 1e-9
            assert np.linalg.norm(a - e) / np.linalg.norm(e) < tol, (i, name)
        assert np.abs(g.C - r.C).max() <= 1e-12, i


def test_batch_graph_equals_eager_bitwise(gpu_pkg, orc):
    pkg = gpu_pkg
    cases = _cases(pkg, orc, True, n=5, seed=11)
    res = []
    for graph in (False, True):
        with pkg.Batch([c[0] for c in cases]) as b:
            for i, (p, f, dt) in enumerate(cases):
                b.state_set(i, f)
            for n in (2, 3):
                st, stats, _ = b.run_steps([c[2] for c in cases], n, graph=graph)
                assert st == 0 and all(s["graph"] == int(graph) for s in stats)
            gs = []
            for i, (p, f, dt) in enumerate(cases):
                g = f.copy()
                b.state_get(i, g)
                gs.append(g)
        res.append(gs)
    for ge, gg in zip(*res):
        for name in pkg.capi.FIELD_NAMES:
            assert np.array_equal(getattr(ge, name), getattr(gg, name)), name


def test_batch_rejects_mixed_arithmetic(gpu_pkg, orc):
    pkg = gpu_pkg
    cases = _cases(pkg, orc, True, n=2)
    ps = [c[0] for c in cases]
    ps[1].p_precision = pkg.capi.PREC_FP64
    with pytest.raises(pkg.CovofError):
        pkg.Batch(ps)


def test_batch_rejects_mixed_inner_kinds(gpu_pkg, orc):
    pkg = gpu_pkg
    cases = _cases(pkg, orc, True, n=2)
    ps = [c[0] for c in cases]
    ps[0].p_inner_kind = pkg.capi.INNER_MG
    ps[1].p_inner_kind = pkg.capi.INNER_CHEBYSHEV
    with pytest.raises(pkg.CovofError):
        pkg.Batch(ps)


def test_sharded_sub_batches_match_the_whole_batch(gpu_pkg, orc):
    """The multi-GPU split (shard.plan) run as its two sub-batches one after
    the other on this GPU: every case is stepped exactly once, and each
    case's fields match those of the single batch holding all cases within
    the Krylov bars (the sub-batches' team sizes differ from the whole
    batch's, so their reductions associate differently)."""
    import importlib
    pkg = gpu_pkg
    shard = importlib.import_module(pkg.__name__ + ".shard")
    cases = _cases(pkg, orc, True, n=7, seed=13)
    for p, f, dt in cases:
        p.p_inner_kind = pkg.capi.INNER_MG
    nsteps = 2

    def run(idx):
        out = {}
        with pkg.Batch([cases[c][0] for c in idx]) as b:
            for i, c in enumerate(idx):
                b.state_set(i, cases[c][1])
            st, stats, _ = b.run_steps([cases[c][2] for c in idx], nsteps, graph=True)
            assert st == 0, stats
            for i, c in enumerate(idx):
                g = cases[c][1].copy()
                b.state_get(i, g)
                out[c] = (g, stats[i])
        return out

    whole = run(list(range(len(cases))))
    parts = shard.plan_params([c[0] for c in cases], 2)
    assert all(len(x) > 0 for x in parts)
    merged = {}
    for part in parts:
        merged.update(run(part))
    assert sorted(merged) == list(range(len(cases)))
    for c, (g, st) in merged.items():
        assert st["steps"] == nsteps and st["first_bad_step"] == -1
        r = whole[c][0]
        for name in ("u", "v", "p"):
            a, e = getattr(g, name), getattr(r, name)
            tol = 1e-8 if name == "p" else 1e-9
            assert np.linalg.norm(a - e) / np.linalg.norm(e) < tol, (c, name)
        assert np.abs(g.C - r.C).max() <= 1e-12, c


@pytest.mark.parametrize("mode", ["mixed_mg", "fp64_mg"])
def test_batch_with_anisotropic_cases(gpu_pkg, orc, mode):
    """Cases whose cells are stretched 2.5:1 or 1:3 beside square ones: the
    batch runs the semi-coarsening Poisson kernel for all of them and every
    case still matches the oracle's steps."""
    pkg = gpu_pkg
    cap = pkg.capi
    cases = []
    for q, (p, C0, dt) in enumerate(pkg.cases.droplet_batch(n_cases=4, seed=11, sizes=(32, 48, 64), nsub=4,
                                                            mixed=True)):
        if q == 1:
            p.dy = 2.5 * p.dx
        elif q == 2:
            p.dx = 3.0 * p.dy
        p.p_precision = cap.PREC_MIXED if mode == "mixed_mg" else cap.PREC_FP64_MG
        p.p_inner_kind = cap.INNER_MG
        f = pkg.Fields.allocate(p)
        f.C[...] = C0
        orc.apply_vof_bc(p, f.C)
        orc.update_physical_properties(p, f)
        orc.compute_curvature_and_csf(p, f)
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
    for i, (g, r) in enumerate(zip(out, ref)):
        assert stats[i]["last_relres"] <= 1e-10
        for name in ("u", "v", "p"):
            a, e = getattr(g, name), getattr(r, name)
            tol = 1e-8 if name == "p" else 1e-9
            assert np.linalg.norm(a - e) / np.linalg.norm(e) < tol, (i, name)
        assert np.abs(g.C - r.C).max() <= 1e-12, i
