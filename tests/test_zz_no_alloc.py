"""The allocation-free Poisson entry point (covof_poisson_solve_rhs_static_dev).

Callers that cannot allocate device memory at the call -- a host code whose
pool allocator owns the whole GPU, or a time loop that must not trigger
cudaMalloc's device-wide synchronisation -- use this entry point: it needs no
handle and keeps its scratch in a fixed static device array.  The tests call
it through the C ABI several times in a row (a smaller mesh after a larger
one, so the array still holds the larger layout) and compare each result
with the handle-based covof_poisson_solve_rhs_dev, in both gauges, and the
reference gauge's result (mean removal included) with the oracle.  They sit
in a file that pytest collects last, and need nothing from earlier tests.
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


def _need_gpu():
    import __graft_entry__ as ge
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    ge._load_build_module().build()


@pytest.mark.parametrize("gauge", ["pinned", "reference"])
def test_static_entry_matches_handle_entry_twice(pkg, gauge):
    _need_gpu()
    for n, k in ((128, 12), (96, 7)):
        p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=n, n_incl=k)
        p.p_tol = 1e-12
        p.p_precision = pkg.capi.PREC_FP64
        p.p_gauge = pkg.capi.GAUGE_PINNED if gauge == "pinned" else pkg.capi.GAUGE_REFERENCE
        xs, its, rrs, sts = _solve_static(pkg, p, dt, b, ru, rv)
        xh, ith, rrh, sth = _solve_handle(pkg, p, dt, b, ru, rv)
        assert sts == sth == pkg.capi.OK, (n, sts, sth)
        # the two launches may cut the mesh into tiles of different sizes, so
        # their reductions associate differently: one iteration apart at most
        assert rrs <= 1e-12 and abs(its - ith) <= 1, (its, ith)
        assert np.linalg.norm(xs - xh) <= 1e-10 * np.linalg.norm(xh), n


def test_static_entry_reference_gauge_matches_oracle(pkg):
    """Reference gauge (diagonal shift, mean removed after the solve), two
    calls in a row against the oracle's solution."""
    import oracle.oracle as orc
    _need_gpu()
    for n, k in ((96, 7), (128, 12)):
        p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=n, n_incl=k)
        p.p_tol = 1e-12
        p.p_precision = pkg.capi.PREC_FP64
        p.p_gauge = pkg.capi.GAUGE_REFERENCE
        ref = np.zeros_like(b)
        _, _, st_o = orc.poisson_solve_rhs(p, dt, b, ru, rv, ref)
        assert st_o == 0
        xs, its, rrs, sts = _solve_static(pkg, p, dt, b, ru, rv)
        assert sts == pkg.capi.OK and rrs <= 1e-12
        assert abs(xs[1:-1, 1:-1].mean()) <= 1e-12 * np.abs(xs).max()
        err = np.linalg.norm(xs[1:-1, 1:-1] - ref[1:-1, 1:-1]) / np.linalg.norm(ref[1:-1, 1:-1])
        assert err < 1e-10, (n, err)


def test_static_entry_refuses_other_solvers(pkg):
    """The entry runs the plain FP64 Jacobi-PCG only: the mixed arithmetic and
    the Gauss-Seidel preconditioner are refused, not silently replaced."""
    _need_gpu()
    p, b, ru, rv, dt = pkg.cases.poisson_inclusions(n=32, n_incl=2)
    for field, value in (("p_precision", pkg.capi.PREC_MIXED), ("p_precision", pkg.capi.PREC_FP64_MG),
                         ("p_precond", pkg.capi.PRECOND_SSOR)):
        q = p.copy()
        setattr(q, field, value)
        _, _, _, st = _solve_static(pkg, q, dt, b, ru, rv)
        assert st == pkg.capi.UNSUPPORTED, (field, value, st)


def test_static_entry_rejects_oversize_mesh(pkg):
    _need_gpu()
    p = pkg.cases.make_params(300, 300, 1.0, 1.0)
    z = np.zeros((302, 302))
    _, _, _, st = _solve_static(pkg, p, 1.0, z, z + 1, z + 1)
    assert st == pkg.capi.TOO_LARGE
