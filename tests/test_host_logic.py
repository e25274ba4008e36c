"""Host-side logic on CPU: synthetic workloads, layout conventions, oracle
golden fixtures."""
from __future__ import annotations

import numpy as np


def test_bubble_case_shapes_and_volume(pkg):
    p, C, dt = pkg.cases.bubble_case(nx=32, ny=64, nsub=8)
    assert C.shape == (66, 34) and C.flags.c_contiguous
    assert 0.0 <= C.min() and C.max() <= 1.0
    gas = ((1.0 - C[1:-1, 1:-1]) * p.dx * p.dy).sum()
    assert abs(gas - np.pi * 0.25 ** 2) < 0.01
    assert p.rho1 == 1000.0 and p.rho2 == 1.0 and p.sigma == 24.5 and dt == 1e-4


def test_poisson_inclusions_is_compatible_and_seeded(pkg):
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=64, n_incl=10)
    assert abs(b[1:-1, 1:-1].sum()) < 1e-9
    assert ru.min() >= 1.0 and ru.max() <= 1000.0
    p2, b2, ru2, rv2, _ = pkg.cases.poisson_inclusions(n=64, n_incl=10)
    assert np.array_equal(b, b2) and np.array_equal(ru, ru2)
    assert p.p_gauge == pkg.capi.GAUGE_PINNED and dt == 1.0


def test_vortex_velocity_is_discretely_solenoidal(pkg):
    p, C, dt, T = pkg.cases.vortex_case(32)
    u, v = pkg.cases.vortex_velocity(p, 0.3, dt, T)
    div = (u[1:-1, 2:] - u[1:-1, 1:-1]) / p.dx + (v[2:, 1:-1] - v[1:-1, 1:-1]) / p.dy
    assert np.abs(div).max() < 1e-12


def test_droplet_array_interface_band(pkg):
    """The reconstruction benchmark's droplet array: fractions in [0, 1],
    seeded, and about 2 pi r k^2 x (band factor) interface cells (every
    droplet's boundary crosses about 2 pi r cells, each crossing cell mixed)."""
    import math
    p, C = pkg.cases.droplet_array(512, 8, 20.0)
    p2, C2 = pkg.cases.droplet_array(512, 8, 20.0)
    assert np.array_equal(C, C2)
    assert C.shape == (514, 514) and C.min() >= 0.0 and C.max() <= 1.0
    inner = C[1:-1, 1:-1]
    mixed = int(((inner > 0.0) & (inner < 1.0)).sum())
    ring = 2.0 * math.pi * 20.0 * 8 * 8
    assert 0.8 * ring < mixed < 1.6 * ring, (mixed, ring)
    # gas inside the droplets: about k^2 pi r^2 cells of C = 0
    gas = float((1.0 - inner).sum())
    assert abs(gas - 64 * math.pi * 400.0) < 0.02 * 64 * math.pi * 400.0
