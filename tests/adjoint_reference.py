"""TEST INFRASTRUCTURE: explicit-matrix reference for the projection and its
gradient, built from the oracle's Poisson assembly (scipy sparse, direct
solves; the adjoint uses the transposed matrix explicitly)."""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def faces(p):
    """Interior (non-wall) face masks for u (i=2..nx) and v (j=2..ny), walls assumed."""
    mu = np.zeros((p.ny + 2, p.nx + 2), bool)
    mv = np.zeros((p.ny + 2, p.nx + 2), bool)
    mu[1:p.ny + 1, 2:p.nx + 1] = True
    mv[2:p.ny + 1, 1:p.nx + 1] = True
    return mu, mv


def operators(orc, p, dt, rho_u, rho_v):
    """A (cells x cells, pinned or shifted as the gauge says) from the oracle's
    coefficients; D (cells x all DOF faces); G (interior faces x cells); beta."""
    nx, ny = p.nx, p.ny
    z = np.zeros((ny + 2, nx + 2))
    aW, aE, aS, aN, aP, _ = orc.poisson_assemble(p, dt, z, z, rho_u, rho_v)
    n = nx * ny
    idx = lambda i, j: (j - 1) * nx + (i - 1)  # noqa: E731
    rows, cols, vals = [], [], []
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            c = idx(i, j)
            rows.append(c); cols.append(c); vals.append(aP[j - 1, i - 1])
            if i > 1: rows.append(c); cols.append(idx(i - 1, j)); vals.append(-aW[j - 1, i - 1])
            if i < nx: rows.append(c); cols.append(idx(i + 1, j)); vals.append(-aE[j - 1, i - 1])
            if j > 1: rows.append(c); cols.append(idx(i, j - 1)); vals.append(-aS[j - 1, i - 1])
            if j < ny: rows.append(c); cols.append(idx(i, j + 1)); vals.append(-aN[j - 1, i - 1])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    # DOF faces: u (i=1..nx+1, j=1..ny) then v (i=1..nx, j=1..ny+1), flat in field layout
    P = nx + 2
    ufaces = [(i, j) for j in range(1, ny + 1) for i in range(1, nx + 2)]
    vfaces = [(i, j) for j in range(1, ny + 2) for i in range(1, nx + 1)]
    nf = len(ufaces) + len(vfaces)
    Dr, Dc, Dv = [], [], []
    Gr, Gc, Gv = [], [], []
    beta = np.zeros(nf)
    for f, (i, j) in enumerate(ufaces):
        beta[f] = 1.0 / rho_u[j, i]
        if i > 1: Dr.append(idx(i - 1, j)); Dc.append(f); Dv.append(p.dy)     # east face of i-1
        if i <= nx: Dr.append(idx(i, j)); Dc.append(f); Dv.append(-p.dy)      # west face of i
        if 1 < i <= nx:
            Gr += [f, f]; Gc += [idx(i, j), idx(i - 1, j)]; Gv += [1 / p.dx, -1 / p.dx]
    off = len(ufaces)
    for q, (i, j) in enumerate(vfaces):
        f = off + q
        beta[f] = 1.0 / rho_v[j, i]
        if j > 1: Dr.append(idx(i, j - 1)); Dc.append(f); Dv.append(p.dx)
        if j <= ny: Dr.append(idx(i, j)); Dc.append(f); Dv.append(-p.dx)
        if 1 < j <= ny:
            Gr += [f, f]; Gc += [idx(i, j), idx(i, j - 1)]; Gv += [1 / p.dy, -1 / p.dy]
    D = sp.csr_matrix((Dv, (Dr, Dc)), shape=(n, nf))
    G = sp.csr_matrix((Gv, (Gr, Gc)), shape=(nf, n))
    return A, D, G, beta, ufaces, vfaces


def pin(A, pinned):
    """Pinned gauge: row/column of cell (1,1) replaced by identity."""
    if not pinned:
        return A.tocsc()
    A = A.tolil()
    A[0, :] = 0
    A[:, 0] = 0
    A[0, 0] = 1.0
    return A.tocsc()


def to_faces(u, v, ufaces, vfaces):
    return np.array([u[j, i] for i, j in ufaces] + [v[j, i] for i, j in vfaces])


def from_faces(x, p, ufaces, vfaces):
    u = np.zeros((p.ny + 2, p.nx + 2))
    v = np.zeros((p.ny + 2, p.nx + 2))
    for f, (i, j) in enumerate(ufaces):
        u[j, i] = x[f]
    off = len(ufaces)
    for q, (i, j) in enumerate(vfaces):
        v[j, i] = x[off + q]
    return u, v


def vjp(orc, p, dt, rho_u, rho_v, us, vs, gu, gv, pinned):
    """Reference gradient: returns (grad_u*, grad_v*, grad_beta_u, grad_beta_v) as fields."""
    A, D, G, beta, uf, vf = operators(orc, p, dt, rho_u, rho_v)
    Ap = pin(A, pinned)
    xs = to_faces(us, vs, uf, vf)
    b = -D @ xs
    if pinned:
        b[0] = 0.0
    pres = spla.spsolve(Ap, b)
    if not pinned:
        pres -= pres.mean()
    g = to_faces(gu, gv, uf, vf)
    Bg = beta * g
    rhs = -dt * (G.T @ Bg)
    if pinned:
        rhs[0] = 0.0
    psi = spla.spsolve(Ap.T.tocsc(), rhs)
    if not pinned:
        psi -= psi.mean()
    gx = g - D.T @ psi
    Gp = G @ pres
    Gpsi = G @ psi
    dvol = p.dx * p.dy
    gb = -dt * Gp * (g + dvol * Gpsi)
    gxu, gxv = from_faces(gx, p, uf, vf)
    gbu, gbv = from_faces(gb, p, uf, vf)
    return gxu, gxv, gbu, gbv
