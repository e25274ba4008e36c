"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def pytest_sessionfinish(session, exitstatus):
    """A run under the bounds-check build (COVOF_GPU_CHECKED=1) writes the
    library's out-of-range record to COVOF_CHECKED_REPORT at the end."""
    import os
    out = os.environ.get("COVOF_CHECKED_REPORT")
    if not out:
        return
    import ctypes
    import json
    import __graft_entry__ as ge
    lib = ge.load_package().capi.load_library()
    bad, first = ctypes.c_longlong(), ctypes.c_longlong()
    st = lib.covof_bounds_check(ctypes.byref(bad), ctypes.byref(first))
    Path(out).write_text(json.dumps({"status": st, "bad": bad.value, "first": first.value,
                                     "exitstatus": int(exitstatus)}))


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as ge
    return ge.load_package()


@pytest.fixture(scope="session")
def orc():
    import oracle.oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def gpu_pkg(pkg):
    """Package with the GPU library built and loaded; fails loudly otherwise."""
    import torch
    import __graft_entry__ as ge
    if not torch.cuda.is_available():
        pytest.fail("gpu test selected but no CUDA device is visible")
    ge._load_build_module().build()
    pkg.capi.load_library()
    return pkg
