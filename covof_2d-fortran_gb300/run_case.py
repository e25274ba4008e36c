"""Run one workload of the hot path a few times, for profiling one kernel.

    python covof_2d-fortran_gb300/run_case.py poisson --n 1024 --prec mixed_mg --reps 3
    python covof_2d-fortran_gb300/run_case.py apply --n 4096 --reps 5
    python covof_2d-fortran_gb300/run_case.py bubble --nx 128 --ny 256 --steps 4
    python covof_2d-fortran_gb300/run_case.py batch --ncases 64 --steps 2
    python covof_2d-fortran_gb300/run_case.py droplets --n 4096 --reps 3

Each case runs `reps` (or `steps`) calls of the library on device-resident
seeded inputs (cases.py) and prints one JSON line with the CUDA-event time of
each call.  A profiler restricted to one kernel (`ncu -k`) captures that
kernel's launches in these calls; the launch count per call is fixed, so
`-s` / `-c` select which calls are captured.

* poisson: the standalone variable-density Poisson (n^2, inclusions of
  density 1000 in 1), pinned cell, from a zero guess, in one arithmetic:
  fp64 (k_pcg_fp64), fp64_mg (k_pcg_fp64_mg), mixed_mg (k_pcg_mixed_mg),
  mixed_cg (k_pcg_mixed_smem / k_pcg_mixed), mixed_cheb (k_pcg_mixed_cheb);
  --max-iter caps the iterations of a call (COVOF_MAXITER then), which bounds
  a capture of the slow arithmetics on large meshes.
* apply: the Poisson operator y = A x (k_poisson_apply), n^2.
* bubble: whole time steps (VOF + SP) of the rising bubble, eager (every
  kernel of the step as its own launch: k_vof_classify, k_vof_mixed,
  k_vof_ring_warp, k_vof_pass, k_props_*, k_csf_*, k_mom_*, k_bicgstab,
  the Poisson kernel).
* batch: batch steps of droplet / bubble cases of uneven sizes
  (k_mom_bicgstab_batch, k_pcg_mixed_mg_batch).
* droplets: ELVIRA reconstructions of an array of 64 x 64 droplets on n^2
  cells (0.5 M interface cells at 4096^2: k_vof_classify, k_vof_mixed_cell,
  k_vof_ring_warp).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def _pkg():
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    ge._load_build_module().build()
    return ge.load_package(), None


def _events(torch, stream):
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    return e0, e1


def run_poisson(args):
    import torch
    pkg, _ = _pkg()
    cap = pkg.capi
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=args.n, n_incl=200 if args.n >= 512 else 20)
    prec = {"fp64": (cap.PREC_FP64, cap.INNER_MG), "fp64_mg": (cap.PREC_FP64_MG, cap.INNER_MG),
            "mixed_mg": (cap.PREC_MIXED, cap.INNER_MG), "mixed_cg": (cap.PREC_MIXED, cap.INNER_CG),
            "mixed_cheb": (cap.PREC_MIXED, cap.INNER_CHEBYSHEV)}[args.prec]
    p.p_precision, p.p_inner_kind = prec
    p.p_gauge = cap.GAUGE_PINNED if args.gauge == "pinned" else cap.GAUGE_REFERENCE
    p.p_max_iter = args.max_iter if args.max_iter > 0 else 10_000_000
    dev = torch.device("cuda")
    tb, tru, trv = (torch.from_numpy(a).to(dev) for a in (b, ru, rv))
    tp = torch.zeros_like(tb)
    out = []
    with pkg.Solver(p) as s:
        stream = torch.cuda.ExternalStream(s.stream_ptr, device=dev)
        for _ in range(args.reps):
            tp.zero_()
            torch.cuda.synchronize()
            e0, e1 = _events(torch, stream)
            it, rr, st = s.poisson_solve_rhs_dev(dt, tb, tru, trv, tp)
            e1.record(stream)
            e1.synchronize()
            assert st in (cap.OK, cap.MAXITER), cap.STATUS_NAMES.get(st)
            out.append({"ms": e0.elapsed_time(e1), "kernel_ms": s.last_solve_ms(), "iters": it,
                        "outer": s.last_refine_steps(), "relres": rr, "status": cap.STATUS_NAMES.get(st)})
    return out


def run_apply(args):
    import torch
    pkg, _ = _pkg()
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=args.n, n_incl=200 if args.n >= 512 else 20)
    dev = torch.device("cuda")
    tru, trv = (torch.from_numpy(a).to(dev) for a in (ru, rv))
    x = torch.from_numpy(np.random.default_rng(1).standard_normal(b.shape)).to(dev)
    y = torch.zeros_like(x)
    out = []
    lib = pkg.capi.load_library()
    with pkg.Solver(p) as s:
        stream = torch.cuda.ExternalStream(s.stream_ptr, device=dev)
        for _ in range(args.reps):
            torch.cuda.synchronize()
            e0, e1 = _events(torch, stream)
            st = lib.covof_poisson_apply_dev(s.h, dt, ctypes.c_void_p(tru.data_ptr()), ctypes.c_void_p(trv.data_ptr()),
                                             ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()))
            e1.record(stream)
            e1.synchronize()
            assert st == pkg.capi.OK, st
            out.append({"ms": e0.elapsed_time(e1)})
    return out


def _state(pkg, p, C0):
    """Fields at t = 0 through the library: ghosts, properties, CSF force."""
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    with pkg.Solver(p) as s:
        s.apply_vof_bc(f)
        s.apply_velocity_bc(f)
        s.update_physical_properties(f)
        s.compute_curvature_and_csf(f)
    return f


def run_bubble(args):
    pkg, _ = _pkg()
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=args.nx, ny=args.ny, nsub=4)
    p.p_precision = cap.PREC_MIXED if args.prec == "mixed_mg" else cap.PREC_FP64
    f = _state(pkg, p, C0)
    out = []
    with pkg.Solver(p) as s:
        s.state_set(f)
        for _ in range(args.steps):
            st, r = s.run_steps(dt, 1, graph=False)
            assert st == cap.OK, st
            out.append({"ms": r["ms"], "poisson_iters": r["poisson_iters"], "mom_iters": r["mom_iters"]})
    return out


def run_batch(args):
    pkg, _ = _pkg()
    cap = pkg.capi
    cases = pkg.cases.droplet_batch(n_cases=args.ncases, mixed=True)
    out = []
    with pkg.Batch([c[0] for c in cases]) as bt:
        for i, (p, C0, dt) in enumerate(cases):
            bt.state_set(i, _state(pkg, p, C0))
        for _ in range(args.steps):
            st, stats, ms = bt.run_steps([c[2] for c in cases], 1, graph=False)
            assert st == cap.OK, st
            out.append({"ms": ms})
    return out


def run_droplets(args):
    import torch
    pkg, _ = _pkg()
    cap = pkg.capi
    p, C0 = pkg.cases.droplet_array(args.n, 64, 20.0 * args.n / 4096)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    with pkg.Solver(p) as s0:
        s0.apply_vof_bc(f)
    tC = torch.from_numpy(f.C).cuda()
    seg = torch.zeros(3 * tC.numel(), dtype=torch.float64, device=tC.device)
    out = []
    with pkg.Solver(p) as s:
        stream = torch.cuda.ExternalStream(s.stream_ptr, device=tC.device)
        for _ in range(args.reps):
            torch.cuda.synchronize()
            e0, e1 = _events(torch, stream)
            st = s.lib.covof_vof_reconstruct_dev(s.h, ctypes.c_void_p(tC.data_ptr()), ctypes.c_void_p(seg.data_ptr()))
            e1.record(stream)
            e1.synchronize()
            assert st == cap.OK, st
            out.append({"ms": e0.elapsed_time(e1)})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["poisson", "apply", "bubble", "batch", "droplets"])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--nx", type=int, default=128)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--prec", default="mixed_mg")
    ap.add_argument("--gauge", default="pinned", choices=["pinned", "reference"])
    ap.add_argument("--max-iter", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--ncases", type=int, default=64)
    args = ap.parse_args()
    fn = {"poisson": run_poisson, "apply": run_apply, "bubble": run_bubble, "batch": run_batch,
          "droplets": run_droplets}[args.case]
    print(json.dumps({"case": args.case, "args": vars(args), "calls": fn(args)}), flush=True)


if __name__ == "__main__":
    main()
