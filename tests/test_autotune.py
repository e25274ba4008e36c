"""Autotuner: candidate lists, cache round trip (CPU); launch overrides and a
small tuning run whose choice still solves to tolerance (GPU)."""
from __future__ import annotations

import ctypes as C
import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def at(pkg):
    return importlib.import_module("covof_gb300.autotune")


def test_candidates_cover_shapes(pkg, at):
    p = pkg.cases.make_params(256, 256, 1.0, 1.0)
    c64 = at.candidates(p, 152)
    assert {d["p_threads"] for d, _ in c64} == {128, 256, 512, 1024}
    p.p_precision = pkg.capi.PREC_MIXED
    p.p_inner_kind = pkg.capi.INNER_CHEBYSHEV
    cm = at.candidates(p, 152)
    assert {d["p_inner_form"] for d, _ in cm} == {1, 2, 3}
    assert {o["p_inner_max_iter"] for _, o in cm} == {16, 24, 32, 48, 64, 96}
    assert all(1 <= d["p_blocks"] <= 152 for d, _ in cm)
    assert at.tuned_fields(p) == ("p_inner_max_iter", "p_cheb_lo")
    p.p_inner_kind = pkg.capi.INNER_MG
    cg = at.candidates(p, 152)
    assert {o["p_mg_nu"] for _, o in cg} == {2, 3, 4}
    assert {o["p_mg_cw"] for _, o in cg} == {1.8, 1.9, 2.0}
    assert {d["p_blocks"] for d, _ in cg} == {152, 76}
    assert {o["p_mg_nuc"] for _, o in cg} == {-1, 32, 64}
    assert at.tuned_fields(p) == ("p_mg_nu", "p_mg_cw", "p_mg_nuc")


def test_cache_round_trip(pkg, at, tmp_path):
    p = pkg.cases.make_params(64, 32, 1.0, 0.5)
    p.p_precision = pkg.capi.PREC_MIXED
    path = tmp_path / "tune.json"
    q, launch = at.apply(p, path)
    assert launch is None and q.p_inner_max_iter == p.p_inner_max_iter
    at.save_cache({at.key_of(p): {"ms": 1.0, "params": {"p_inner_max_iter": 24, "p_cheb_lo": 2e-3},
                                  "launch": {"p_threads": 1024, "p_blocks": 16, "p_inner_form": 1}}}, path)
    q, launch = at.apply(p, path)
    assert q.p_inner_max_iter == 24 and q.p_cheb_lo == 2e-3
    assert (launch.p_blocks, launch.p_inner_form) == (16, 1)


@pytest.mark.gpu
def test_launch_overrides_validate(gpu_pkg):
    pkg = gpu_pkg
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=64, n_incl=12)
    p.p_gauge = pkg.capi.GAUGE_PINNED
    with pkg.Solver(p) as s:
        L = pkg.capi.Launch(p_threads=100, p_blocks=0, p_inner_form=0)
        assert s.lib.covof_set_launch(s.h, C.byref(L)) == pkg.capi.INVALID
        L = pkg.capi.Launch(p_threads=256, p_blocks=8, p_inner_form=0)
        assert s.lib.covof_set_launch(s.h, C.byref(L)) == pkg.capi.OK
        G = pkg.capi.Launch()
        assert s.lib.covof_get_launch(s.h, C.byref(G)) == pkg.capi.OK
        assert (G.p_threads, G.p_blocks) == (256, 8)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_mg"])
def test_tuned_choice_solves_to_tolerance(gpu_pkg, orc, at, tmp_path, prec):
    import torch
    pkg = gpu_pkg
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=128, n_incl=20)
    p.p_gauge = pkg.capi.GAUGE_PINNED
    p.p_tol = 1e-10
    p.p_precision = pkg.capi.PREC_FP64 if prec == "fp64" else pkg.capi.PREC_MIXED
    p.p_inner_kind = pkg.capi.INNER_MG if prec == "mixed_mg" else pkg.capi.INNER_CHEBYSHEV
    T = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    path = tmp_path / "tune.json"
    best = at.tune(p, dt, T(b), T(ru), T(rv), repeats=1, cache_path=path, budget_s=60.0)
    assert best["ms"] > 0 and best["candidates"] >= 1
    ref = np.zeros_like(b)
    q = p.copy()
    q.p_tol = 1e-12
    orc.poisson_solve_rhs(q, dt, b, ru, rv, ref)
    x = np.zeros_like(b)
    with at.open_tuned(p, path) as s:
        it, rr, st = s.poisson_solve_rhs(dt, b, ru, rv, x)
    assert st == pkg.capi.OK and rr <= 1e-10
    err = np.linalg.norm(x[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
    assert err < 1e-8, err
