"""Autotuner for the pressure Poisson solve.

For one mesh and parameter set, times candidate launch shapes
(covof_set_launch: FP64 block size, block count, shared-memory vs streamed
Chebyshev state) and, on the mixed path, candidate inner settings (Chebyshev
degree and interval end; multigrid smoothing sweeps and coarse-correction
weight), on the case's own Poisson system; keeps the fastest candidate that
reaches the tolerance; caches the choice in a JSON file keyed by device,
mesh, arithmetic and inner kind.  The tuned inner settings change the inner
iteration, not the answer: the outer FP64 iteration still stops on the true
residual at p_tol.

    best = tune(params, dt, b, rho_u, rho_v)         # torch CUDA tensors
    params2, launch = apply(params)                  # from the cache
"""
from __future__ import annotations

import ctypes as C
import json
import os
import time
from pathlib import Path

from . import capi
from .capi import Launch, Params
from .solver import Solver

DEFAULT_CACHE = Path(os.environ.get("COVOF_TUNE_CACHE", Path.home() / ".cache" / "covof_gb300" / "tune.json"))


def _device_name() -> str:
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return "cuda"


def key_of(p: Params) -> str:
    walls = "".join(str(int(t)) for t in p.bc_type)
    return (f"{_device_name()}|{p.nx}x{p.ny}|prec{p.p_precision}|inner{p.p_inner_kind}|gauge{p.p_gauge}|"
            f"walls{walls}")


def load_cache(path: Path = DEFAULT_CACHE) -> dict:
    try:
        return json.loads(Path(path).read_text())
    except Exception:
        return {}


def save_cache(cache: dict, path: Path = DEFAULT_CACHE):
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    tmp = path.with_suffix(".tmp")
    tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
    tmp.replace(path)


def candidates(p: Params, sm_count: int) -> list[tuple[dict, dict]]:
    """(launch overrides, parameter overrides) pairs to time."""
    out = []
    if p.p_precision == capi.PREC_FP64:
        for t in (128, 256, 512, 1024):
            out.append(({"p_threads": t, "p_blocks": 0, "p_inner_form": 0}, {}))
        return out
    # most promising first (a time budget may cut the list): shared-memory
    # strips on every SM, then higher degrees and narrower intervals, which
    # trade FP64 outer iterations for cheap FP32 inner steps
    blocks = sorted({min(sm_count, p.ny), max(1, min(sm_count, p.ny) // 2)}, reverse=True)
    if p.p_inner_kind == capi.INNER_MG or p.p_precision == capi.PREC_FP64_MG:
        # the over-correction weight matters most (aggregation coarse
        # operators are about twice too stiff), then the smoothing sweeps
        # (a coarse solve that leaves less error behind also counts: the
        # coarsest level's sweeps)
        mg_blocks = sorted({sm_count, max(1, sm_count // 2)}, reverse=True)
        for nb in mg_blocks:
            for nuc in (-1, 64, 32):
                for nu in (3, 2, 4):
                    for cw in (2.0, 1.9, 1.8):
                        out.append(({"p_threads": 0, "p_blocks": nb, "p_inner_form": 0},
                                    {"p_mg_nu": nu, "p_mg_cw": cw, "p_mg_nuc": nuc}))
        return out
    shapes = []
    if p.p_inner_kind == capi.INNER_CHEBYSHEV:
        # one thread-block cluster (small meshes; covof_set_launch refuses
        # the sizes that do not fit)
        shapes += [(3, g) for g in (16, 8, 4) if g <= p.ny]
    if p.p_inner_kind != capi.INNER_CG:
        shapes += [(1, nb) for nb in blocks] + [(2, nb) for nb in blocks]
    else:
        shapes += [(0, nb) for nb in blocks]
    for form, nb in shapes:
        for m in (48, 64, 32, 96, 24, 16):
            for lo in (5.0e-4, 2.5e-4, 1.0e-3, 2.0e-3):
                out.append(({"p_threads": 0, "p_blocks": nb, "p_inner_form": form},
                            {"p_inner_max_iter": m, "p_cheb_lo": lo}))
    return out


def _set_launch(s: Solver, d: dict) -> int:
    L = Launch(**d)
    return s.lib.covof_set_launch(s.h, C.byref(L))


def _get_launch(s: Solver) -> dict:
    L = Launch()
    s.lib.covof_get_launch(s.h, C.byref(L))
    return L.as_dict()


def tune(p: Params, dt: float, b, rho_u, rho_v, repeats: int = 2, cache_path: Path | None = DEFAULT_CACHE,
         budget_s: float = 120.0, verbose: bool = False) -> dict:
    """Time every candidate (best of `repeats` solves from a zero guess) on
    A x = b with the given face densities; return and cache the fastest."""
    import torch
    x = torch.zeros_like(b)
    sm = torch.cuda.get_device_properties(b.device).multi_processor_count
    results = []
    t_start = time.perf_counter()
    by_params: dict[tuple, list] = {}
    for launch, over in candidates(p, sm):
        by_params.setdefault(tuple(sorted(over.items())), []).append(launch)
    # the rule's own settings are always timed (the reference point)
    rule_key = tuple(sorted({k: getattr(p, k) for k in tuned_fields(p)}.items()))
    if p.p_precision != capi.PREC_FP64 and rule_key in by_params:
        by_params = {rule_key: by_params.pop(rule_key), **by_params}
    for over_t, launches in by_params.items():
        q = p.copy()
        for k, v in over_t:
            setattr(q, k, v)
        with Solver(q) as s:
            rule_launch = _get_launch(s) if over_t == rule_key else None
            if rule_launch is not None:
                launches = [dict(rule_launch, rule=True)] + launches
            for launch in launches:
                is_rule = bool(launch.pop("rule", False)) if isinstance(launch, dict) else False
                if time.perf_counter() - t_start > budget_s:
                    break
                if _set_launch(s, launch) != capi.OK:
                    continue
                best = None
                for _ in range(repeats):
                    x.zero_()
                    it, rr, st = s.poisson_solve_rhs_dev(dt, b, rho_u, rho_v, x)
                    if st != capi.OK or not rr <= q.p_tol:
                        best = None
                        break
                    ms = s.last_solve_ms()
                    best = ms if best is None else min(best, ms)
                if best is None:
                    continue
                rec = {"ms": best, "launch": _get_launch(s), "params": dict(over_t), "iters": it,
                       "outer": s.last_refine_steps(), "t": round(time.perf_counter() - t_start, 2),
                       "rule": is_rule}
                results.append(rec)
                if verbose:
                    print(json.dumps(rec), flush=True)
    if not results:
        raise RuntimeError("autotune: no candidate reached the tolerance")
    results.sort(key=lambda r: r["ms"])
    best = dict(results[0])
    best["candidates"] = len(results)
    best["rule_ms"] = next((r["ms"] for r in results if _is_rule(r, p, sm)), None)
    if cache_path is not None:
        cache = load_cache(cache_path)
        cache[key_of(p)] = best
        save_cache(cache, cache_path)
    return best


def tuned_fields(p: Params) -> tuple[str, ...]:
    """The parameters the tuner varies for p's arithmetic and inner kind."""
    if p.p_precision == capi.PREC_FP64:
        return ()
    if p.p_inner_kind == capi.INNER_MG or p.p_precision == capi.PREC_FP64_MG:
        return ("p_mg_nu", "p_mg_cw", "p_mg_nuc")
    return ("p_inner_max_iter", "p_cheb_lo")


def _is_rule(r: dict, p: Params, sm: int) -> bool:
    """Whether a timed record is what the built-in rules would have chosen."""
    if p.p_precision == capi.PREC_FP64:
        return False
    return all(r["params"].get(k) == getattr(p, k) for k in tuned_fields(p)) and r.get("rule", False)


def apply(p: Params, cache_path: Path = DEFAULT_CACHE):
    """Cached choice for p: (params with the tuned inner settings, launch
    overrides as a Launch, or None when nothing is cached)."""
    rec = load_cache(cache_path).get(key_of(p))
    if not rec:
        return p.copy(), None
    q = p.copy()
    for k, v in rec.get("params", {}).items():
        setattr(q, k, v)
    return q, Launch(**rec["launch"])


def open_tuned(p: Params, cache_path: Path = DEFAULT_CACHE) -> Solver:
    """A Solver with the cached choice applied (rules when nothing is cached)."""
    q, launch = apply(p, cache_path)
    s = Solver(q)
    if launch is not None and s.lib.covof_set_launch(s.h, C.byref(launch)) != capi.OK:
        s.close()
        s = Solver(p)
    return s
