"""Generates the committed golden fixtures (tests/golden/*.npz).

Source of truth: the FP64 oracle (oracle/covof_oracle.cpp), a restatement of
the reference -- the Fortran reference itself cannot be built on these
machines (no Fortran compiler, no MPI), and it ships no golden vectors.  The
fixtures store their inputs as well as the outputs, so they do not depend on
the platform's libm when replayed.  Regenerate with:

    python tests/golden/gen_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as ge  # noqa: E402
import oracle.oracle as orc  # noqa: E402


def params_array(p):
    return np.frombuffer(bytes(p), dtype=np.uint8).copy()


def main():
    pkg = ge.load_package()
    cases, cap = pkg.cases, pkg.capi
    out = {}

    # 1. geometric kernels: cut_box_area / compute_alpha / hypot tables
    rng = np.random.default_rng(101)
    geo_in = np.column_stack([rng.uniform(0, 2, 200), rng.uniform(0, 2, 200)])
    th = rng.uniform(0, 2 * np.pi, 200)
    c = rng.uniform(0.0, 1.0, 200)
    c[:10] = [0.0, 1.0, 1e-7, 1 - 1e-7, 0.5, 1e-6, 1 - 1e-6, 0.25, 0.75, 0.999]
    h = 1.0 / 64
    alpha = np.array([orc.compute_alpha(x0, x0 + h, y0, y0 + h, np.cos(t), np.sin(t), cc)
                      for (x0, y0), t, cc in zip(geo_in, th, c)])
    area = np.array([orc.cut_box_area(x0, x0 + h, y0, y0 + h, np.cos(t), np.sin(t), a)
                     for (x0, y0), t, a in zip(geo_in, th, alpha)])
    hx = rng.uniform(-3, 3, 200) * 10.0 ** rng.uniform(-3, 3, 200)
    hy = rng.uniform(-3, 3, 200) * 10.0 ** rng.uniform(-3, 3, 200)
    hyp = np.array([orc.hypot(a, b) for a, b in zip(hx, hy)])
    np.savez_compressed(HERE / "geometry.npz", xy=geo_in, theta=th, c=c, h=h, alpha=alpha, area=area,
                        hx=hx, hy=hy, hypot=hyp)

    # 2. VOF: reconstruction (PLIC, ELVIRA) and one WY step each order, 16x32 bubble
    p, C0, dt = cases.bubble_case(nx=16, ny=32, nsub=16)
    orc.apply_vof_bc(p, C0)
    u, v = cases.random_velocity(p, 0.5, 102)
    d = {"C": C0, "u": u, "v": v, "dt": 0.2 * p.dx}
    for name, rc in (("plic", cap.RECON_PLIC), ("elvira", cap.RECON_ELVIRA)):
        q = p.copy()
        q.recon = rc
        d[f"params_{name}"] = params_array(q)
        d[f"seg_{name}"] = orc.reconstruct(q, C0)
        for xf in (0, 1):
            Cw = C0.copy()
            orc.wy_step(q, 0.2 * p.dx, xf, u, v, Cw)
            d[f"wy_{name}_x{xf}"] = Cw
    np.savez_compressed(HERE / "vof_bubble16x32.npz", **d)

    # 3. SP step, 16x32 bubble after one VOF step (ELVIRA)
    p.p_tol = 1e-12
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.update_physical_properties(p, f)
    orc.compute_curvature_and_csf(p, f)
    f.u[...], f.v[...] = cases.random_velocity(p, 1e-2, 103)
    orc.apply_velocity_bc(p, f.u, f.v, False)
    f.u_old[...] = f.u
    f.v_old[...] = f.v
    inp = {k: getattr(f, k).copy() for k in ("u", "v", "p", "rho_u", "rho_v", "mu", "mu_node",
                                              "fx_sigma", "fy_sigma", "u_old", "v_old")}
    iu, ip, rr, st = orc.sp_step(p, 1e-4, f)
    assert st == 0
    np.savez_compressed(HERE / "sp_bubble16x32.npz", params=params_array(p), dt=1e-4,
                        **{"in_" + k: a for k, a in inp.items()},
                        out_u=f.u, out_v=f.v, out_p=f.p, iters_u=iu, iters_p=ip)

    # 4. Poisson, 32^2 inclusions, pinned and reference gauge
    p, b, ru, rv, dt = cases.poisson_inclusions(n=32, n_incl=4)
    p.p_tol = 1e-12
    dd = {"b": b, "rho_u": ru, "rho_v": rv, "dt": dt}
    for g, name in ((cap.GAUGE_PINNED, "pinned"), (cap.GAUGE_REFERENCE, "reference")):
        q = p.copy()
        q.p_gauge = g
        x = np.zeros_like(b)
        it, r, st = orc.poisson_solve_rhs(q, dt, b, ru, rv, x)
        assert st == 0
        dd[f"params_{name}"] = params_array(q)
        dd[f"p_{name}"] = x
        dd[f"iters_{name}"] = it
    np.savez_compressed(HERE / "poisson32.npz", **dd)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
