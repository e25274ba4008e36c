"""Seeded synthetic inputs for the hot-path workloads.

No dataset or case file ships with the reference, so every workload is a
seeded synthetic stand-in with the shapes, sizes and value ranges of the
configurations it represents.  Seeds: base 20261203, workload k uses
base + k with numpy's PCG64.  Arrays use the reference layout (ny+2, nx+2).

* ``bubble_case``      -- rising bubble, 128x256 on [0,1]x[0,2] (the small
  STANDARD_PROJECTION + ELVIRA + Weymouth-Yue case).
* ``poisson_inclusions`` -- standalone variable-density Poisson on 1024^2
  with 200 heavy circular inclusions (rho 1000 in, 1 out), zero-mean
  Gaussian RHS, homogeneous Neumann walls.
* ``vortex_case``      -- Rider-Kothe single-vortex VOF transport
  (src/module_simulation.f90:2175-2416).
* ``droplet_batch``    -- many independent droplet / bubble cases of uneven
  sizes (64..512 cells per direction) for the batch engine.
* ``rt_case``          -- Rayleigh-Taylor instability, 4096^2 cells on
  [0,1] x [0,4], heavy fluid over light.
"""
from __future__ import annotations

import math

import numpy as np

from . import capi
from .capi import Params

SEED = 20261203


def make_params(nx: int, ny: int, lx: float, ly: float) -> Params:
    """Pure-Python twin of covof_params_default (checked against it in tests)."""
    p = Params()
    p.nx, p.ny = nx, ny
    p.dx, p.dy = lx / nx, ly / ny
    for s in range(4):
        p.bc_type[s] = capi.BC_DIRICHLET
        p.bc_u[s] = 0.0
        p.bc_v[s] = 0.0
    p.linear_solver = capi.LINEAR_BICGSTAB2
    p.precond = capi.PRECOND_JACOBI
    p.use_precond = 1
    p.max_iter = 300
    p.tol = 1.0e-5
    p.enable_convection = 1
    p.convective_scheme = capi.CONV_UPWIND
    p.p_precond = capi.PRECOND_JACOBI
    p.p_max_iter = 1000
    p.p_gauge = capi.GAUGE_REFERENCE
    p.p_precision = capi.PREC_FP64
    p.p_tol = 1.0e-7
    p.p_inner_tol = 1.0e-4
    p.p_inner_max_iter = 32
    p.p_max_refine = 1000000
    p.enable_two_phase = 0
    p.enable_surface_tension = 0
    p.rho1, p.rho2, p.mu1, p.mu2 = 1.0, 1.0, 1.0e-3, 1.0e-3
    p.sigma, p.gx, p.gy = 0.0, 0.0, 0.0
    p.recon = capi.RECON_PLIC
    p.p_inner_kind = capi.INNER_MG
    p.p_cheb_lo = 1.0e-3
    p.p_mg_nu = 2
    p.p_mg_cw = 2.0
    p.p_mg_tail = 2048
    p.time_scheme = capi.TIME_EULER
    p.convective_linearization = capi.CONV_LIN_PICARD
    p.enable_svof_smoothing = 0
    p.svof_filter_width = 1.0
    p.enable_diffusion_smoothing = 0
    p.diffusion_smoothing_steps = 3
    p.advection_method = capi.ADVECT_WEYMOUTH_YUE
    p.tvd_limiter = capi.LIMITER_SUPERBEE
    p.solver_type = capi.SOLVER_STANDARD_PROJECTION
    p.r_al = 100.0
    p.adaptative_al = 0
    p.k_aal = 100.0
    p.l0_ref = p.t0_ref = p.u0_ref = p.p0_ref = 0.0
    p.ic_radius = 0.25
    p.uzawa_iter = 1
    p.uzawa_tol = 1.0e-12
    p.p_mg_nuc = -1
    return p


def field(p: Params, value: float = 0.0) -> np.ndarray:
    return np.full((p.ny + 2, p.nx + 2), value, dtype=np.float64)


def subsample_fraction(nx, ny, dx, dy, inside, nsub: int) -> np.ndarray:
    """Fraction of nsub x nsub cell sub-samples where inside(x, y) holds, for
    every cell of (0:nx+1, 0:ny+1) (sample points as in
    src/module_interface_vof.f90:128-152)."""
    i = np.arange(0, nx + 2)
    j = np.arange(0, ny + 2)
    s = (np.arange(nsub) + 0.5) / nsub
    xs = ((i[:, None] - 1) + s[None, :]).reshape(-1) * dx   # (nx+2)*nsub
    ys = ((j[:, None] - 1) + s[None, :]).reshape(-1) * dy
    X, Y = np.meshgrid(xs, ys)                              # (ny+2)*nsub, (nx+2)*nsub
    ins = inside(X, Y)
    frac = ins.reshape(ny + 2, nsub, nx + 2, nsub).mean(axis=(1, 3))
    return np.ascontiguousarray(frac, dtype=np.float64)


# ---------------------------------------------------------------------------
def bubble_case(nx: int = 128, ny: int = 256, seed: int = SEED + 0, nsub: int = 16):
    """Rising gas bubble in liquid: params + initial C (liquid = fluid 1,
    C = fraction of sub-samples outside the bubble)."""
    lx, ly = 1.0, 2.0
    p = make_params(nx, ny, lx, ly)
    rng = np.random.default_rng(seed)
    phases = rng.uniform(0.0, 2.0 * math.pi, size=7)
    ks = np.arange(2, 9)

    def outside(X, Y):
        dxp, dyp = X - 0.5, Y - 0.5
        th = np.arctan2(dyp, dxp)
        r = 0.25 * (1.0 + 1.0e-3 * np.cos(ks[None, None, :] * th[..., None] + phases).sum(-1))
        return np.hypot(dxp, dyp) > r

    C = subsample_fraction(nx, ny, p.dx, p.dy, outside, nsub)
    p.enable_two_phase = 1
    p.enable_surface_tension = 1
    p.rho1, p.mu1, p.rho2, p.mu2 = 1000.0, 10.0, 1.0, 0.1
    p.sigma, p.gx, p.gy = 24.5, 0.0, -0.98
    p.linear_solver = capi.LINEAR_BICGSTAB
    p.tol = 1.0e-10
    p.p_tol = 1.0e-10
    p.p_max_iter = 100000
    p.recon = capi.RECON_ELVIRA
    dt = 1.0e-4
    return p, C, dt


def cavity_case(n: int = 32, re: float = 100.0, solver_type: int = capi.SOLVER_MONOLITHIC):
    """Lid-driven cavity (the reference's tutorial 08 set-up): unit square,
    one fluid (rho 1, mu 1/Re), no-slip walls and a lid moving at u = 1,
    coupled solve with BiCGSTAB2 + Jacobi.  Returns (params, dt)."""
    p = make_params(n, n, 1.0, 1.0)
    p.bc_u[3] = 1.0
    p.rho1 = p.rho2 = 1.0
    p.mu1 = p.mu2 = 1.0 / re
    p.solver_type = solver_type
    p.linear_solver = capi.LINEAR_BICGSTAB2
    p.tol = 1.0e-10
    p.max_iter = 20000
    dt = 0.25 * p.dx
    return p, dt


def poisson_inclusions(n: int = 1024, n_incl: int = 200, seed: int = SEED + 1, nsub: int = 4):
    """Standalone variable-density Poisson: returns (params, b, rho_u, rho_v, dt).
    rho = 1000 C + (1 - C) with C the sub-sampled inclusion fraction; face
    densities arithmetic (src/module_interface_vof.f90:576-591); RHS N(0,1)
    per cell minus its mean; walls => homogeneous Neumann for p."""
    p = make_params(n, n, 1.0, 1.0)
    rng = np.random.default_rng(seed)
    cx = rng.uniform(0.0, 1.0, n_incl)
    cy = rng.uniform(0.0, 1.0, n_incl)
    rr = rng.uniform(0.01, 0.05, n_incl)
    # sub-sample mask, built inclusion by inclusion on its bounding box
    ns = nsub
    h = 1.0 / (n * ns)
    ins = np.zeros((n * ns, n * ns), dtype=bool)
    for x0, y0, r in zip(cx, cy, rr):
        i0 = max(0, int((x0 - r) / h) - 1); i1 = min(n * ns, int((x0 + r) / h) + 2)
        j0 = max(0, int((y0 - r) / h) - 1); j1 = min(n * ns, int((y0 + r) / h) + 2)
        xs = (np.arange(i0, i1) + 0.5) * h
        ys = (np.arange(j0, j1) + 0.5) * h
        ins[j0:j1, i0:i1] |= ((xs[None, :] - x0) ** 2 + (ys[:, None] - y0) ** 2) <= r * r
    Cin = ins.reshape(n, ns, n, ns).mean(axis=(1, 3))
    C = np.zeros((n + 2, n + 2))
    C[1:-1, 1:-1] = Cin
    C[0, :] = C[1, :]; C[-1, :] = C[-2, :]; C[:, 0] = C[:, 1]; C[:, -1] = C[:, -2]
    rho = 1000.0 * C + 1.0 * (1.0 - C)
    rho_u = np.ones_like(rho)
    rho_v = np.ones_like(rho)
    rho_u[1:-1, 1:] = 0.5 * (rho[1:-1, :-1] + rho[1:-1, 1:])
    rho_v[1:, 1:-1] = 0.5 * (rho[:-1, 1:-1] + rho[1:, 1:-1])
    b = np.zeros_like(rho)
    g = rng.standard_normal((n, n))
    b[1:-1, 1:-1] = g - g.mean()
    p.p_tol = 1.0e-10
    p.p_max_iter = 200000
    p.p_gauge = capi.GAUGE_PINNED
    dt = 1.0
    return p, b, rho_u, rho_v, dt


def vortex_case(n: int = 64, recon: int = capi.RECON_PLIC, nsub: int = 16):
    """Single-vortex VOF case (Rider & Kothe): disk R=0.125 at (0.5, 0.75), T=6."""
    p = make_params(n, n, 1.0, 1.0)
    p.enable_two_phase = 1
    p.rho1, p.mu1, p.rho2, p.mu2 = 1000.0, 1.0e-3, 1.0, 1.0e-5
    p.recon = recon
    C = subsample_fraction(n, n, p.dx, p.dy,
                           lambda X, Y: (X - 0.5) ** 2 + (Y - 0.75) ** 2 <= 0.125 ** 2, nsub)
    dt = {64: 0.005, 128: 0.0025, 256: 0.00125, 512: 0.0005}.get(n, 0.32 / n)
    return p, C, dt, 6.0


def vortex_velocity(p: Params, t: float, dt: float, T: float):
    """Analytic faces velocity at t + dt/2 (src/module_simulation.f90:2254-2288)."""
    nx, ny = p.nx, p.ny
    cf = math.cos(math.pi * (t + 0.5 * dt) / T)
    u = field(p)
    v = field(p)
    xf = (np.arange(1, nx + 2) - 1) * p.dx            # faces i = 1..nx+1
    yc = ((np.arange(1, ny + 1) - 1) + 0.5) * p.dy     # centres j = 1..ny
    sx = np.sin(math.pi * xf)
    sy = np.sin(2.0 * math.pi * yc)
    u[1:ny + 1, 1:nx + 2] = -(sx[None, :] * sx[None, :]) * sy[:, None] * cf
    xc = ((np.arange(1, nx + 1) - 1) + 0.5) * p.dx
    yf = (np.arange(1, ny + 2) - 1) * p.dy
    sx2 = np.sin(2.0 * math.pi * xc)
    sy2 = np.sin(math.pi * yf)
    v[1:ny + 2, 1:nx + 1] = sx2[None, :] * (sy2[:, None] * sy2[:, None]) * cf
    return u, v


def random_velocity(p: Params, scale: float, seed: int):
    """Seeded random MAC velocity with zero normal velocity on the walls."""
    rng = np.random.default_rng(seed)
    u = field(p)
    v = field(p)
    u[1:p.ny + 1, 1:p.nx + 2] = scale * rng.standard_normal((p.ny, p.nx + 1))
    v[1:p.ny + 2, 1:p.nx + 1] = scale * rng.standard_normal((p.ny + 1, p.nx))
    u[1:p.ny + 1, 1] = 0.0
    u[1:p.ny + 1, p.nx + 1] = 0.0
    v[1, 1:p.nx + 1] = 0.0
    v[p.ny + 1, 1:p.nx + 1] = 0.0
    return u, v


def droplet_array(n: int = 4096, k: int = 64, r_cells: float = 20.0, seed: int = SEED + 6):
    """A k x k array of gas droplets in liquid on the unit square at n x n
    cells, one per (n/k)^2 block with a seeded centre jitter, radius r_cells
    cells: about 2 pi r_cells k^2 interface cells (650k at the defaults), the
    regime where the reconstruction's throughput, not one cell's latency,
    sets its time.  C (liquid fraction) is the signed distance to the
    block's droplet across one cell, clipped to [0, 1] (values strictly
    between 0 and 1 only in the interface band).  Returns (params, C)."""
    p = make_params(n, n, 1.0, 1.0)
    rng = np.random.default_rng(seed)
    b = n // k
    jit = rng.uniform(-0.15, 0.15, size=(k, k, 2)) * b
    C = np.ones((n + 2, n + 2), dtype=np.float64)
    ci = np.arange(n) + 0.5
    blk = np.minimum(np.arange(n) // b, k - 1)
    cx = (blk[None, :] + 0.5) * b + jit[blk[:, None], blk[None, :], 0]
    cy = (blk[:, None] + 0.5) * b + jit[blk[:, None], blk[None, :], 1]
    d = np.hypot(ci[None, :] - cx, ci[:, None] - cy)
    C[1:-1, 1:-1] = np.clip(d - r_cells + 0.5, 0.0, 1.0)
    p.enable_two_phase = 1
    p.recon = capi.RECON_ELVIRA
    return p, C


def droplet_batch(n_cases: int = 256, seed: int = SEED + 4, sizes=(64, 128, 256, 512), nsub: int = 4,
                  mixed: bool = True, shapes=None):
    """Independent droplet / bubble cases: nx, ny drawn from sizes, square
    cells, short side of the domain 1 (dx = dy = 1/min(nx, ny)); 1-3 circles
    with radii 0.1-0.3 of the short side (fluid 1 inside for a droplet,
    outside for a bubble);
    density ratio log-uniform in [10, 1000] (rho1 = 1000), viscosity ratio
    log-uniform in [1, 100] (mu1 = 1e-2), sigma uniform in [0.01, 25],
    g = (0, -0.98); ELVIRA + Weymouth-Yue, BiCGSTAB + Jacobi predictor and the
    Poisson to 1e-10.  dt = min(1e-4, half the capillary limit
    sqrt((rho1 + rho2) h^3 / (4 pi sigma))).  shapes: a list of (nx, ny) in
    place of the drawn sizes (one case each; the rest is drawn as usual).
    Returns [(params, C, dt)]."""
    rng = np.random.default_rng(seed)
    out = []
    for c in range(n_cases if shapes is None else len(shapes)):
        if shapes is None:
            nx, ny = (int(v) for v in rng.choice(sizes, 2))
        else:
            nx, ny = (int(v) for v in shapes[c])
        m = min(nx, ny)
        lx, ly = nx / m, ny / m
        p = make_params(nx, ny, lx, ly)
        short = min(lx, ly)
        k = int(rng.integers(1, 4))
        circles = []
        for _ in range(k):
            r = rng.uniform(0.1, 0.3) * short
            cx = rng.uniform(r, lx - r)
            cy = rng.uniform(r, ly - r)
            circles.append((cx, cy, r))
        droplet = bool(rng.integers(0, 2))

        def inside(X, Y, circles=circles, droplet=droplet):
            m = np.zeros(np.broadcast(X, Y).shape, dtype=bool)
            for cx, cy, r in circles:
                m |= np.hypot(X - cx, Y - cy) < r
            return m if droplet else ~m

        Cf = subsample_fraction(nx, ny, p.dx, p.dy, inside, nsub)
        ratio = math.exp(rng.uniform(math.log(10.0), math.log(1000.0)))
        vratio = math.exp(rng.uniform(0.0, math.log(100.0)))
        p.enable_two_phase = 1
        p.enable_surface_tension = 1
        p.rho1, p.rho2 = 1000.0, 1000.0 / ratio
        p.mu1, p.mu2 = 1.0e-2, 1.0e-2 / vratio
        p.sigma = rng.uniform(0.01, 25.0)
        p.gx, p.gy = 0.0, -0.98
        p.linear_solver = capi.LINEAR_BICGSTAB
        p.tol = 1.0e-10
        p.p_tol = 1.0e-10
        p.p_max_iter = 200000
        p.recon = capi.RECON_ELVIRA
        p.p_precision = capi.PREC_MIXED if mixed else capi.PREC_FP64
        h = min(p.dx, p.dy)
        dt_sigma = math.sqrt((p.rho1 + p.rho2) * h ** 3 / (4.0 * math.pi * p.sigma))
        out.append((p, Cf, min(1.0e-4, 0.5 * dt_sigma)))
    return out


def adjoint_case(n: int = 512, seed: int = SEED + 3, nd: int = 8, ratio: float = 100.0):
    """Projection-adjoint workload: [0,1]^2 with n x n cells, a seeded
    two-phase density (nd random droplets, radii 0.05-0.15, ratio 100),
    Gaussian MAC predictor velocity u* (std 1e-2) and target (std 1e-4),
    dt = 1e-3.  Returns (params, rho_u, rho_v, u*, v*, u_target, v_target, dt)."""
    p = make_params(n, n, 1.0, 1.0)
    rng = np.random.default_rng(seed)
    cx, cy, rr = rng.uniform(0.2, 0.8, nd), rng.uniform(0.2, 0.8, nd), rng.uniform(0.05, 0.15, nd)

    def inside(X, Y):
        m = np.zeros_like(X, dtype=bool)
        for a, b, r in zip(cx, cy, rr):
            m |= (X - a) ** 2 + (Y - b) ** 2 <= r * r
        return m

    C = subsample_fraction(n, n, p.dx, p.dy, inside, 4)
    rho = ratio * C + (1.0 - C)
    rho_u = np.ones_like(rho)
    rho_v = np.ones_like(rho)
    rho_u[1:-1, 1:] = 0.5 * (rho[1:-1, :-1] + rho[1:-1, 1:])
    rho_v[1:, 1:-1] = 0.5 * (rho[:-1, 1:-1] + rho[1:, 1:-1])
    us, vs = random_velocity(p, 1e-2, seed + 1)
    ut, vt = random_velocity(p, 1e-4, seed + 2)
    p.p_tol = 1e-10
    p.p_max_iter = 200000
    return p, rho_u, rho_v, us, vs, ut, vt, 1e-3


def rt_case(nx: int = 4096, ny: int = 4096, seed: int = SEED + 5, nsub: int = 4, mixed: bool = True):
    """Rayleigh-Taylor: [0,1] x [0,4], heavy fluid (rho 3, fluid 1, C = 1)
    above y = 2 + 0.05 cos(2 pi x) + sum_{k=3..32} 1e-3 cos(2 pi k x + phi_k),
    light fluid (rho 1) below, mu = 1e-3 in both, no surface tension,
    g = (0, -9.81), no-slip walls, dt = 2e-5; ELVIRA + Weymouth-Yue,
    BiCGSTAB + Jacobi predictor and the Poisson to 1e-10.  C is the exact
    fraction of each cell above the interface, averaged over nsub x-samples
    (the interface is a graph over x), with cells within 1e-6 of pure made
    pure.  Returns (params, C, dt)."""
    lx, ly = 1.0, 4.0
    p = make_params(nx, ny, lx, ly)
    rng = np.random.default_rng(seed)
    ks = np.arange(3, 33)
    phases = rng.uniform(0.0, 2.0 * math.pi, size=ks.size)
    i = np.arange(0, nx + 2)
    xs = ((i[:, None] - 1) + (np.arange(nsub) + 0.5)[None, :] / nsub) * p.dx       # (nx+2, nsub)
    eta = 2.0 + 0.05 * np.cos(2.0 * math.pi * xs)
    for k, ph in zip(ks, phases):
        eta += 1.0e-3 * np.cos(2.0 * math.pi * k * xs + ph)
    C = np.empty((ny + 2, nx + 2), dtype=np.float64)
    for j0 in range(0, ny + 2, 256):
        j = np.arange(j0, min(j0 + 256, ny + 2))
        ylo = ((j - 1) * p.dy)[:, None, None]
        frac = np.clip((ylo + p.dy - eta[None, :, :]) / p.dy, 0.0, 1.0)        # part above eta
        C[j0:j0 + j.size] = frac.mean(axis=2)
    # cells within 1e-6 of pure are pure for the reconstruction
    # (src/module_interface_reconstruction.f90:368-379), so their sliver of
    # volume would not be fluxed consistently: make them pure
    C[C <= 1.0e-6] = 0.0
    C[C >= 1.0 - 1.0e-6] = 1.0
    p.enable_two_phase = 1
    p.enable_surface_tension = 0
    p.rho1, p.rho2 = 3.0, 1.0
    p.mu1, p.mu2 = 1.0e-3, 1.0e-3
    p.sigma, p.gx, p.gy = 0.0, 0.0, -9.81
    p.linear_solver = capi.LINEAR_BICGSTAB
    p.tol = 1.0e-10
    p.p_tol = 1.0e-10
    p.p_max_iter = 2000000
    p.recon = capi.RECON_ELVIRA
    p.p_precision = capi.PREC_MIXED if mixed else capi.PREC_FP64
    return p, C, 2.0e-5

