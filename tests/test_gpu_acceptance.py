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


def _rt_tutorial(pkg, orc, nx, ny, sigma):
    """Tutorial 19's single-mode Rayleigh-Taylor set-up (Guides_Tutos/
    volume3_tutorials/19_tuto_rayleigh_taylor_instabilite.md, sections 2-3):
    [0,1] x [0,4], heavy fluid (rho 3, C = 1) above y = 2 + 0.05 cos(2 pi x),
    light (rho 1) below, mu 1e-3, g -9.81, free-slip sides, no-slip top and
    bottom, TVD-Superbee convection, surface tension with diffusion smoothing
    when sigma > 0; the STANDARD_PROJECTION step with the mixed Poisson."""
    import math
    cap = pkg.capi
    p = pkg.cases.make_params(nx, ny, 1.0, 4.0)
    p.bc_type[0] = p.bc_type[1] = cap.BC_FREESLIP
    p.enable_two_phase = 1
    p.enable_surface_tension = int(sigma > 0)
    p.enable_diffusion_smoothing = int(sigma > 0)
    p.rho1, p.rho2, p.mu1, p.mu2 = 3.0, 1.0, 1e-3, 1e-3
    p.sigma, p.gx, p.gy = sigma, 0.0, -9.81
    p.convective_scheme = cap.CONV_TVD_SUPERBEE
    p.recon = cap.RECON_PLIC
    p.linear_solver = cap.LINEAR_BICGSTAB
    p.tol = 1e-10
    p.max_iter = 1000
    p.p_tol = 1e-10
    p.p_max_iter = 100000
    p.p_precision = cap.PREC_MIXED
    nsub = 16
    xs = (np.arange(nx)[:, None] + (np.arange(nsub) + 0.5)[None, :] / nsub) * p.dx
    eta = 2.0 + 0.05 * np.cos(2.0 * math.pi * xs)
    ylo = (np.arange(ny) * p.dy)[:, None, None]
    f = pkg.Fields.allocate(p)
    f.C[1:-1, 1:-1] = np.clip((ylo + p.dy - eta[None]) / p.dy, 0.0, 1.0).mean(axis=2)
    f.C[f.C <= 1e-6] = 0.0
    f.C[f.C >= 1.0 - 1e-6] = 1.0
    orc.apply_vof_bc(p, f.C)
    orc.prepare_interface(p, f)
    return p, f


@pytest.mark.parametrize("nx,ny,sigma", [(64, 256, 0.0), (128, 512, 0.0), (64, 256, 0.2), (64, 256, 0.6)])
def test_rayleigh_taylor_linear_growth(gpu_pkg, orc, nx, ny, sigma):
    """Tutorial 19's acceptance checks (section 6.1) over its linear window
    t in [0.05, 0.30] s (dt 1e-3): the half peak-to-trough amplitude A(t) of
    the interface (the column heights of the heavy fluid) fitted to
    A0 cosh(omega t) gives omega within 10 % of the inviscid linear rate
    omega_th^2 = ((rho1 - rho2) g k - sigma k^3) / (rho1 + rho2) (5.55 and
    4.29 1/s; the finite amplitude k A0 = 0.31 and the viscosity lower it);
    sigma = 0.6 > sigma_c: the interface does not grow; the mirror symmetry
    C(1 - x, y) = C(x, y) holds to round-off, the volume to 1e-4."""
    import math
    pkg = gpu_pkg
    cap = pkg.capi
    p, f = _rt_tutorial(pkg, orc, nx, ny, sigma)
    v0 = f.C[1:-1, 1:-1].sum()

    def amplitude():
        h = p.ny * p.dy - f.C[1:-1, 1:-1].sum(axis=0) * p.dy
        return 0.5 * (h.max() - h.min())

    amps, times = [amplitude()], [0.0]
    with pkg.Solver(p) as s:
        s.state_set(f)
        for k in range(30):
            st, _ = s.run_steps(1e-3, 10, graph=True)
            assert st == cap.OK, st
            s.state_get(f)
            amps.append(amplitude())
            times.append(0.01 * (k + 1))
    A, T = np.array(amps), np.array(times)
    win = (T >= 0.05) & (T <= 0.30)
    kk = 2.0 * math.pi
    w2 = ((p.rho1 - p.rho2) * 9.81 * kk - sigma * kk ** 3) / (p.rho1 + p.rho2)
    sym = np.abs(f.C[1:-1, 1:-1] - f.C[1:-1, 1:-1][:, ::-1]).max()
    dv = abs(f.C[1:-1, 1:-1].sum() - v0) / v0
    if w2 > 0:
        y = np.arccosh(np.maximum(A[win] / A[0], 1.0))
        w = float(T[win] @ y / (T[win] @ T[win]))
        print(f"RT {nx}x{ny} sigma {sigma}: omega {w:.4f} against {math.sqrt(w2):.4f}, symmetry {sym:.1e}, dV {dv:.1e}")
        assert abs(w - math.sqrt(w2)) <= 0.10 * math.sqrt(w2), (w, math.sqrt(w2))
    else:
        print(f"RT {nx}x{ny} sigma {sigma}: max A/A0 {A.max() / A[0]:.4f}, symmetry {sym:.1e}, dV {dv:.1e}")
        assert A.max() <= 1.05 * A[0], A
    assert sym < 1e-6 and dv < 1e-4, (sym, dv)
