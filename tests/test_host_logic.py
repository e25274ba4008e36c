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
