"""GPU VOF transport variants against the oracle, through the C ABI:
CIAM (geometric, Lagrangian remap; src/module_interface_vof.f90:938-1159)
and the algebraic TVD scheme with each limiter (:828-935,
src/module_interface_reconstruction.f90:686-725).  Bit-exact, one pass order
each way, and whole time steps."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _state(pkg, orc, nx=48, ny=64, vel=0.8, seed=41):
    p, C0, dt = pkg.cases.bubble_case(nx=nx, ny=ny, nsub=4)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    f.u[...], f.v[...] = pkg.cases.random_velocity(p, vel, seed)
    return p, f, 0.4 * min(p.dx, p.dy) / vel


@pytest.mark.parametrize("x_first", [True, False])
@pytest.mark.parametrize("method,limiter", [("CIAM", "SUPERBEE"), ("TVD", "SUPERBEE"), ("TVD", "VAN_LEER"),
                                            ("TVD", "MUSCL"), ("TVD", "HRIC")])
@pytest.mark.parametrize("recon", ["PLIC", "ELVIRA"])
def test_transport_bit_exact(gpu_pkg, orc, method, limiter, recon, x_first):
    pkg = gpu_pkg
    cap = pkg.capi
    p, f, dt = _state(pkg, orc)
    p.advection_method = getattr(cap, "ADVECT_" + method)
    p.tvd_limiter = getattr(cap, "LIMITER_" + limiter)
    p.recon = getattr(cap, "RECON_" + recon)
    Cg = f.C.copy()
    orc.vof_transport(p, dt, x_first, f.u, f.v, f.C)
    with pkg.Solver(p) as s:
        s.advect_vof_weymouth_yue(dt, f.u, f.v, Cg, x_first)
    assert np.array_equal(Cg, f.C)
    assert not np.array_equal(f.C, _state(pkg, orc)[1].C)  # the interface moved


@pytest.mark.parametrize("method", ["CIAM", "TVD"])
def test_steps_with_transport_match_oracle(gpu_pkg, orc, method):
    pkg = gpu_pkg
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=32, ny=64, nsub=4)
    p.advection_method = getattr(cap, "ADVECT_" + method)
    p.p_tol = 1e-12
    p.tol = 1e-10
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.prepare_interface(p, f)
    g = f.copy()
    for k in range(4):
        iu, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0
    with pkg.Solver(p) as s:
        s.state_set(g)
        st, stats = s.run_steps(dt, 4, graph=True)
        assert st == 0
        s.state_get(g)
    for name in ("u", "v", "p"):
        a, b = getattr(g, name), getattr(f, name)
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < (1e-8 if name == "p" else 1e-9), name
    assert np.abs(g.C - f.C).max() <= 1e-12
