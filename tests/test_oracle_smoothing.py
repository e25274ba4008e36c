"""Oracle: interface smoothing on CPU -- SVOF Helmholtz smoothing
(src/module_interface_vof.f90:387-476), diffusion smoothing (:1416-1461) and
the property / CSF variants that read them (:541-545, 596-601, 682-690).

Known answers from the mathematics: a constant indicator is a fixed point of
(I - D lap) with Neumann walls; 25 symmetric Gauss-Seidel pairs land close to
the exact Helmholtz solution (solved here with a sparse direct solver); the
explicit diffusion step is restated with numpy in the same operation order
and must agree bit for bit; the properties follow the stated formulas.
"""
from __future__ import annotations

import numpy as np
import pytest


def _bubble(pkg, nx=40, ny=56, svof=True, diffusion=False, width=1.0, steps=3):
    p, C0, dt = pkg.cases.bubble_case(nx=nx, ny=ny, nsub=4)
    p.enable_svof_smoothing = int(svof)
    p.svof_filter_width = width
    p.enable_diffusion_smoothing = int(diffusion)
    p.diffusion_smoothing_steps = steps
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    return p, f, dt


def test_constant_is_a_fixed_point(pkg, orc):
    p, f, dt = _bubble(pkg)
    f.C[...] = 0.37
    orc.svof_smooth(p, f)
    assert np.allclose(f.C_s, 0.37, rtol=0, atol=1e-15)


@pytest.mark.parametrize("width", [1.0, 2.5])
def test_close_to_the_helmholtz_solution(pkg, orc, width):
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    p, f, dt = _bubble(pkg, nx=24, ny=32, width=width)
    orc.apply_vof_bc(p, f.C)
    orc.svof_smooth(p, f)
    nx, ny, dx, dy = p.nx, p.ny, p.dx, p.dy
    D = width * dx * dy
    wx, wy = D / dx ** 2, D / dy ** 2
    idx = lambda i, j: (j - 1) * nx + (i - 1)  # noqa: E731
    rows, cols, vals = [], [], []
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            k = idx(i, j)
            aP = 1.0
            for (ii, jj, w, on) in ((i + 1, j, wx, i < nx), (i - 1, j, wx, i > 1),
                                    (i, j + 1, wy, j < ny), (i, j - 1, wy, j > 1)):
                if on:
                    rows.append(k); cols.append(idx(ii, jj)); vals.append(-w)
                    aP += w
            rows.append(k); cols.append(k); vals.append(aP)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(nx * ny, nx * ny))
    x = spla.spsolve(A.tocsc(), f.C[1:-1, 1:-1].ravel())
    exact = np.clip(x.reshape(ny, nx), 0.0, 1.0)
    err = np.abs(f.C_s[1:-1, 1:-1] - exact).max()
    assert err < 2e-3, err
    # and the smoothing did smooth: far from the raw indicator
    assert np.abs(f.C_s[1:-1, 1:-1] - f.C[1:-1, 1:-1]).max() > 0.05


def test_svof_clamp_and_ghosts(pkg, orc):
    p, f, dt = _bubble(pkg, nx=20, ny=28)
    orc.svof_smooth(p, f)
    Cs = f.C_s
    assert Cs.min() >= 0.0 and Cs.max() <= 1.0
    assert np.array_equal(Cs[1:-1, 0], Cs[1:-1, 1]) and np.array_equal(Cs[1:-1, -1], Cs[1:-1, -2])
    assert np.array_equal(Cs[0, 1:-1], Cs[1, 1:-1]) and np.array_equal(Cs[-1, 1:-1], Cs[-2, 1:-1])
    assert Cs[0, 0] == Cs[1, 1] and Cs[-1, -1] == Cs[-2, -2]


@pytest.mark.parametrize("steps", [1, 3, 4])
def test_diffusion_matches_numpy_restatement(pkg, orc, steps):
    p, f, dt = _bubble(pkg, nx=18, ny=26, svof=False, diffusion=True, steps=steps)
    orc.diffusion_smooth(p, f)
    ct = f.C.copy()
    dtau = 0.2 * min(p.dx * p.dx, p.dy * p.dy)

    def ghosts(a):
        a[1:-1, 0] = a[1:-1, 1]
        a[1:-1, -1] = a[1:-1, -2]
        a[0, :] = a[1, :]
        a[-1, :] = a[-2, :]

    for _ in range(steps):
        ghosts(ct)
        nxt = ct.copy()
        c = ct[1:-1, 1:-1]
        lx = (ct[1:-1, 2:] - 2.0 * c + ct[1:-1, :-2]) / (p.dx * p.dx)
        ly = (ct[2:, 1:-1] - 2.0 * c + ct[:-2, 1:-1]) / (p.dy * p.dy)
        nxt[1:-1, 1:-1] = c + dtau * (lx + ly)
        ct = nxt
    ghosts(ct)
    assert np.array_equal(f.C_tilde, ct)


def test_properties_follow_the_smoothed_indicator(pkg, orc):
    p, f, dt = _bubble(pkg, nx=20, ny=24)
    orc.apply_vof_bc(p, f.C)
    orc.svof_smooth(p, f)
    orc.update_physical_properties(p, f)
    c = np.clip(f.C_s, 0.0, 1.0)
    assert np.array_equal(f.rho[1:-1, 1:-1], (c * p.rho1 + (1.0 - c) * p.rho2)[1:-1, 1:-1])
    Cs = f.C_s
    cn = np.clip(0.25 * (Cs[:-1, :-1] + Cs[:-1, 1:] + Cs[1:, :-1] + Cs[1:, 1:]), 0.0, 1.0)
    mn = (p.mu1 * p.mu2) / np.maximum(1e-30, p.mu2 * cn + p.mu1 * (1.0 - cn))
    assert np.array_equal(f.mu_node[1:, 1:], mn)


def test_csf_normals_follow_the_smoothing(pkg, orc):
    """The same C with SVOF, diffusion smoothing or neither gives three
    different curvatures; the face gradient stays the raw C's."""
    out = {}
    for name, svof, diff in (("plain", False, False), ("svof", True, False), ("diff", False, True)):
        p, f, dt = _bubble(pkg, nx=32, ny=48, svof=svof, diffusion=diff)
        orc.apply_vof_bc(p, f.C)
        orc.prepare_interface(p, f)
        out[name] = f.curvature.copy()
    assert not np.array_equal(out["plain"], out["svof"])
    assert not np.array_equal(out["plain"], out["diff"])
    assert not np.array_equal(out["svof"], out["diff"])


def test_time_loop_with_smoothing_runs(pkg, orc):
    p, f, dt = _bubble(pkg, nx=16, ny=32, svof=True, diffusion=True)
    orc.apply_vof_bc(p, f.C)
    orc.prepare_interface(p, f)
    for k in range(3):
        iu, ip, rr, st = orc.time_step(p, dt, k, f)
        assert st == 0 and rr <= p.p_tol
    assert np.isfinite(f.u).all()


def _div_rcp(x: float, b: float, y: float) -> float:
    """The device's SVOF quotient restated exactly: q0 = RN(x y),
    r = RN(x - b q0) (one FMA), q = RN(q0 + r y) (one FMA); Fractions give
    the exact values that each FMA rounds once."""
    from fractions import Fraction as F
    q0 = x * y
    r = float(F(x) - F(b) * F(q0))
    return float(F(r) * F(y) + F(q0))


@pytest.mark.parametrize("width,aspect", [(1.0, 1.0), (2.5, 1.0), (1.0, 4.0), (0.5, 0.25), (10.0, 1.0)])
def test_reciprocal_division_is_correctly_rounded(width, aspect):
    """The SVOF kernel divides by 1 + aE + aW + aN + aS through a
    precomputed reciprocal and one FMA correction (Markstein); on every wall
    pattern and operands across the range C_s takes it equals IEEE x / b."""
    dx, dy = 1.0 / 64, aspect / 64
    D = width * dx * dy
    wx, wy = D / (dx * dx), D / (dy * dy)
    rng = np.random.default_rng(int(width * 10 + aspect * 100))
    for f in range(16):
        aE = 0.0 if f & 1 else wx
        aW = 0.0 if f & 2 else wx
        aN = 0.0 if f & 4 else wy
        aS = 0.0 if f & 8 else wy
        b = 1.0 + aE + aW + aN + aS
        y = 1.0 / b
        xs = list(rng.uniform(0.0, b, 300)) + list(rng.uniform(0.0, 1.0, 100)) + [0.0, 1.0, b, 1e-300]
        for x in xs:
            assert _div_rcp(float(x), b, y) == float(x) / b, (x, b)


@pytest.mark.parametrize("method", ["CIAM", "TVD"])
def test_transport_conserves_and_bounds(pkg, orc, method):
    """CIAM and TVD keep C in [0, 1]; with a divergence-free uniform flow
    along x through periodic-free interior (the bubble far from walls) the
    volume is kept to round-off (TVD is conservative; CIAM's remap is exact
    for du = 0)."""
    cap = pkg.capi
    p, C0, dt = pkg.cases.bubble_case(nx=32, ny=48, nsub=4)
    p.advection_method = getattr(cap, "ADVECT_" + method)
    f = pkg.Fields.allocate(p)
    f.C[...] = 1.0 - C0          # the bubble as the tracked phase, zero at the walls
    orc.apply_vof_bc(p, f.C)
    f.u[1:-1, 1:-1] = 0.3
    v0 = f.C[1:-1, 1:-1].sum()
    for k in range(5):
        orc.vof_transport(p, 0.2 * p.dx / 0.3, k % 2 == 0, f.u, f.v, f.C)
        orc.apply_vof_bc(p, f.C)
    assert f.C.min() >= 0.0 and f.C.max() <= 1.0
    assert abs(f.C[1:-1, 1:-1].sum() - v0) <= 1e-10 * v0
