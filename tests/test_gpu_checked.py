"""The parity suite's small cases under the bounds-check build.

The library is rebuilt with -DCOVOF_CHECKED (every device-side cell index
and every stencil centre checked against the (nx+2) x (ny+2) ghosted
extents, a bad index counted and redirected inside the array instead of
faulting) and the small-mesh GPU parity tests run against it in a child
process; they must pass, and the library's record must show no out-of-range
index.  This stands in for a memory checker on ragged and tiny meshes."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

SUITE = ["tests/test_gpu_poisson.py", "tests/test_gpu_vof.py", "tests/test_gpu_momentum.py",
         "tests/test_gpu_stepping.py", "tests/test_gpu_batch.py", "tests/test_gpu_schemes.py",
         "tests/test_gpu_transport.py", "tests/test_gpu_al.py", "tests/test_gpu_mono.py",
         "tests/test_gpu_sweeps.py", "tests/test_gpu_adjoint.py"]


def test_small_parity_cases_under_bounds_checks(gpu_pkg, tmp_path):
    import importlib.util
    spec = importlib.util.spec_from_file_location("covof_build_checked", ROOT / "covof_2d-fortran_gb300" / "build.py")
    bmod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bmod)
    lib = bmod.build(checked=True)
    assert lib.exists()
    report = tmp_path / "bounds.json"
    env = dict(os.environ, COVOF_GPU_CHECKED="1", COVOF_CHECKED_REPORT=str(report))
    # the small meshes: the full-size and timing-heavy cases stay out
    sel = "not 1024 and not full_size and not 4096 and not 512 and not gradients_match"
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider",
                        "-k", sel] + SUITE, cwd=str(ROOT), env=env, capture_output=True, text=True,
                       timeout=1800)
    tail = (r.stdout + r.stderr)[-3000:]
    assert r.returncode == 0, tail
    rec = json.loads(report.read_text())
    print(f"bounds-check build: {rec}")
    assert rec["status"] == 0, rec        # the checked library was the one loaded
    assert rec["bad"] == 0, rec
