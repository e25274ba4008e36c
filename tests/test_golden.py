"""Replay of the committed golden fixtures (tests/golden/gen_golden.py):
the oracle must reproduce them bit for bit on any platform (CPU), and the GPU
library must reproduce the VOF fixtures bit for bit and the solver fixtures
within 1e-10 relative L2 (gpu)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

G = Path(__file__).resolve().parent / "golden"


def _params(pkg, arr):
    # fixtures hold the parameter block as packed when they were made; fields
    # appended since (multigrid settings) are zero-filled, unused by the oracle
    import ctypes
    buf = arr.tobytes()
    buf += bytes(max(0, ctypes.sizeof(pkg.capi.Params) - len(buf)))
    return pkg.capi.Params.from_buffer_copy(buf)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_oracle_reproduces_geometry(orc):
    z = np.load(G / "geometry.npz")
    h = float(z["h"])
    for (x0, y0), t, c, a, ar in zip(z["xy"], z["theta"], z["c"], z["alpha"], z["area"]):
        assert orc.compute_alpha(x0, x0 + h, y0, y0 + h, np.cos(t), np.sin(t), c) == a
        assert orc.cut_box_area(x0, x0 + h, y0, y0 + h, np.cos(t), np.sin(t), a) == ar
    for x, y, r in zip(z["hx"], z["hy"], z["hypot"]):
        assert orc.hypot(x, y) == r


def test_oracle_reproduces_vof(pkg, orc):
    z = np.load(G / "vof_bubble16x32.npz")
    for name in ("plic", "elvira"):
        p = _params(pkg, z[f"params_{name}"])
        assert np.array_equal(orc.reconstruct(p, z["C"].copy()), z[f"seg_{name}"])
        for xf in (0, 1):
            C = z["C"].copy()
            orc.wy_step(p, float(z["dt"]), xf, z["u"], z["v"], C)
            assert np.array_equal(C, z[f"wy_{name}_x{xf}"])


def _sp_fields(pkg, z):
    p = _params(pkg, z["params"])
    f = pkg.Fields.allocate(p)
    for k in ("u", "v", "p", "rho_u", "rho_v", "mu", "mu_node", "fx_sigma", "fy_sigma", "u_old", "v_old"):
        getattr(f, k)[...] = z["in_" + k]
    return p, f


def test_oracle_reproduces_sp_and_poisson(pkg, orc):
    z = np.load(G / "sp_bubble16x32.npz")
    p, f = _sp_fields(pkg, z)
    iu, ip, rr, st = orc.sp_step(p, float(z["dt"]), f)
    assert st == 0 and iu == int(z["iters_u"]) and ip == int(z["iters_p"])
    for k in ("u", "v", "p"):
        assert np.array_equal(getattr(f, k), z["out_" + k]), k
    z = np.load(G / "poisson32.npz")
    for name in ("pinned", "reference"):
        p = _params(pkg, z[f"params_{name}"])
        x = np.zeros_like(z["b"])
        it, rr, st = orc.poisson_solve_rhs(p, float(z["dt"]), z["b"], z["rho_u"], z["rho_v"], x)
        assert st == 0 and it == int(z[f"iters_{name}"])
        assert np.array_equal(x, z[f"p_{name}"])


@pytest.mark.gpu
def test_gpu_reproduces_golden(gpu_pkg):
    pkg = gpu_pkg
    z = np.load(G / "vof_bubble16x32.npz")
    for name in ("plic", "elvira"):
        p = _params(pkg, z[f"params_{name}"])
        with pkg.Solver(p) as s:
            assert np.array_equal(s.reconstruct_interface(z["C"].copy()), z[f"seg_{name}"])
            for xf in (0, 1):
                C = z["C"].copy()
                s.advect_vof_weymouth_yue(float(z["dt"]), z["u"], z["v"], C, bool(xf))
                assert np.array_equal(C, z[f"wy_{name}_x{xf}"])
    z = np.load(G / "sp_bubble16x32.npz")
    p, f = _sp_fields(pkg, z)
    with pkg.Solver(p) as s:
        it, rr, st = s.sim_solve_standard_projection(float(z["dt"]), f)
    assert st == 0
    for k in ("u", "v", "p"):
        assert _rel(getattr(f, k), z["out_" + k]) < 1e-10, k
    z = np.load(G / "poisson32.npz")
    for name in ("pinned", "reference"):
        for prec in (pkg.capi.PREC_FP64, pkg.capi.PREC_MIXED):
            p = _params(pkg, z[f"params_{name}"])
            p.p_precision = prec
            x = np.zeros_like(z["b"])
            with pkg.Solver(p) as s:
                it, rr, st = s.poisson_solve_rhs(float(z["dt"]), z["b"], z["rho_u"], z["rho_v"], x)
            assert st == 0
            assert _rel(x, z[f"p_{name}"]) < 1e-10, (name, prec)
