"""The self-measured FP64 rate (covof_fp64_peak), the denominator of the
interface reconstruction's FP64 figure: positive and within the GB300's
nominal FP64 rate (1.25 TFLOP/s dense) with room for clock variation."""
from __future__ import annotations

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_peak_is_plausible(gpu_pkg):
    pkg = gpu_pkg
    p, C0, dt = pkg.cases.bubble_case(nx=32, ny=64, nsub=4)
    with pkg.Solver(p) as s:
        g = s.fp64_peak()
    assert 100.0 < g < 2500.0, g
