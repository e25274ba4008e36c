"""The reference's documented Young-Laplace acceptance check
(Guides_Tutos/volume3_tutorials/06_tuto_goutte_laplace.md, section 6.1) on
the GPU's resident time steps (CUDA-graph replay): the static droplet of the
oracle test, N = 32, 64 and 128 with the tutorial's time steps, SVOF-smoothed
curvature.  The pressure jump matches the oracle's, its error against
sigma / R0 = 4 Pa falls under refinement, the parasitic currents stay small
and the volume is kept."""
from __future__ import annotations

import numpy as np
import pytest

from test_oracle_acceptance import laplace_case, pressure_jump, run_oracle

pytestmark = pytest.mark.gpu


def run_gpu(pkg, orc, N, svof):
    p, f, dt, nst = laplace_case(pkg, N, svof)
    orc.apply_vof_bc(p, f.C)
    orc.prepare_interface(p, f)
    v0 = f.C[1:-1, 1:-1].sum()
    with pkg.Solver(p) as s:
        s.state_set(f)
        st, stats = s.run_steps(dt, nst, graph=True)
        assert st == pkg.capi.OK and stats["graph"] == 1, (st, stats)
        s.state_get(f)
    dp = pressure_jump(p, f)
    ca = max(np.abs(f.u).max(), np.abs(f.v).max()) * p.mu1 / p.sigma
    dv = abs(f.C[1:-1, 1:-1].sum() - v0) / v0
    return dp, ca, dv, f


def test_young_laplace_on_the_gpu(gpu_pkg, orc):
    pkg = gpu_pkg
    g = {N: run_gpu(pkg, orc, N, True) for N in (32, 64, 128)}
    err = {N: abs(g[N][0] - 4.0) / 4.0 for N in g}
    print("Young-Laplace (SVOF): " + ", ".join(f"N {N}: dP {g[N][0]:.6f} Erel {err[N]:.3e} Ca {g[N][1]:.2e}"
                                             for N in g))
    assert err[64] < err[32] and err[128] < err[64], err
    assert err[128] < 0.01, err
    for N in g:
        # parasitic currents small; the volume moves by round-off per step
        # (the reference's 1e-12 V0 criterion, accumulated over the steps)
        nst = int(round(0.02 / {32: 1e-3, 64: 3e-4, 128: 1e-4}[N]))
        assert g[N][1] < 0.1 and g[N][2] < 1e-12 * nst, (N, g[N][1], g[N][2])
    for N in (32, 64):
        dp_o, _, _, fo = run_oracle(pkg, orc, N, True)
        rel = abs(g[N][0] - dp_o) / abs(dp_o)
        perr = np.linalg.norm(g[N][3].p[1:-1, 1:-1] - fo.p[1:-1, 1:-1]) / np.linalg.norm(fo.p[1:-1, 1:-1])
        print(f"  N {N}: GPU vs oracle dP rel {rel:.2e}, p rel L2 {perr:.2e}")
        assert rel < 1e-8 and perr < 1e-8, (N, rel, perr)


def _vortex_l1(pkg, orc, n, recon):
    """Rider-Kothe single vortex over one period T = 6 s (the reference's
    tutorial 07 set-up and time steps), Weymouth-Yue advection on the GPU;
    L1 distance of C(T) from C(0) and the relative volume change."""
    cases = pkg.cases
    p, C0, dt, T = cases.vortex_case(n, recon=getattr(pkg.capi, "RECON_" + recon))
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    c_init = f.C[1:-1, 1:-1].copy()
    nst = int(round(T / dt))
    with pkg.Solver(p) as s:
        for k in range(nst):
            f.u[...], f.v[...] = cases.vortex_velocity(p, k * dt, dt, T)
            s.apply_velocity_bc(f)
            s.advect_vof(dt, f)
    return (np.abs(f.C[1:-1, 1:-1] - c_init).mean(),
            abs(f.C[1:-1, 1:-1].sum() - c_init.sum()) / c_init.sum())


@pytest.mark.parametrize("recon", ["PLIC", "ELVIRA"])
def test_vortex_shape_error_converges(gpu_pkg, orc, recon):
    """Tutorial 07's acceptance check (Guides_Tutos/volume3_tutorials/
    07_tuto_vortex_shear.md, section 6.1): the return error E_L1 after one
    period falls under refinement (64^2, 128^2, 256^2 with dt 0.005, 0.0025,
    0.00125) at an order p = log2(E(2h) / E(h)) the tutorial expects in
    [1, 2] once the filament's tail is resolved, with the volume kept to
    round-off (the reference's vortex criterion, README.md:219)."""
    import math
    pkg = gpu_pkg
    res = {n: _vortex_l1(pkg, orc, n, recon) for n in (64, 128, 256)}
    order = {n: math.log(res[n // 2][0] / res[n][0], 2) for n in (128, 256)}
    print(f"vortex {recon}: " + ", ".join(f"N {n}: E_L1 {res[n][0]:.4e} dV {res[n][1]:.1e}" for n in res)
          + ", orders " + ", ".join(f"{order[n]:.2f}" for n in order))
    assert res[128][0] < res[64][0] and res[256][0] < res[128][0]
    assert 1.0 <= order[256] <= 2.0, order
    for n in res:
        assert res[n][1] < 1e-12 * int(round(6.0 / {64: 0.005, 128: 0.0025, 256: 0.00125}[n])), (n, res[n][1])
