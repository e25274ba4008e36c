"""The allocation-free Poisson entry point (covof_poisson_solve_rhs_static_dev).

Callers that cannot allocate device memory at the call -- a host code whose
pool allocator owns the whole GPU, or a time loop that must not trigger
cudaMalloc's device-wide synchronisation -- use this entry point: it needs no
handle and keeps its scratch in a fixed static device array.  This test calls
it through the C ABI twice in a row (the second call on a smaller mesh, so the
array still holds the first call's larger layout) and compares each result
with the handle-based covof_poisson_solve_rhs_dev.  It sits in a file that
pytest collects last, and needs nothing from earlier tests.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solve_static(pkg, p, dt, b, ru, rv):
    import torch
    dev = torch.device("cuda")
    tb, tru, trv = (torch.from_numpy(a).to(dev) for a in (b, ru, rv))
    tp = torch.zeros_like(tb)
    torch.cuda.synchronize()
    it, rr = C.c_int(), C.c_double()
    st = pkg.capi.load_library().covof_poisson_solve_rhs_static_dev(
        C.byref(p), dt, tb.data_ptr(), tru.data_ptr(), trv.data_ptr(), tp.data_ptr(), C.byref(it), C.byref(rr))
    return tp.cpu().numpy(), it.value, rr.value, st


def _solve_handle(pkg, p, dt, b, ru, rv):
    import torch
    dev = torch.device("cuda")
    tb, tru, trv = (torch.from_numpy(a).to(dev) for a in (b, ru, rv))
    tp = torch.zeros_like(tb)
    with pkg.Solver(p) as s:
        it, rr, st = s.poisson_solve_rhs_dev(dt, tb, tru, trv, tp)
    return tp.cpu().numpy(), it, rr, st


def test_static_entry_matches_handle_entry_twice(pkg):
    import __graft_entry__ as ge
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    ge._load_build_module().build()
    for n, k in ((128, 12), (96, 7)):
        p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=n, n_incl=k)
        p.p_tol = 1e-12
        p.p_precision = pkg.capi.PREC_FP64
        xs, its, rrs, sts = _solve_static(pkg, p, dt, b, ru, rv)
        xh, ith, rrh, sth = _solve_handle(pkg, p, dt, b, ru, rv)
        assert sts == sth == pkg.capi.OK, (n, sts, sth)
        assert rrs <= 1e-12 and its == ith
        assert np.linalg.norm(xs - xh) <= 1e-10 * np.linalg.norm(xh), n


def test_static_entry_rejects_oversize_mesh(pkg):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    p = pkg.cases.make_params(300, 300, 1.0, 1.0)
    z = np.zeros((302, 302))
    _, _, _, st = _solve_static(pkg, p, 1.0, z, z + 1, z + 1)
    assert st == pkg.capi.TOO_LARGE
