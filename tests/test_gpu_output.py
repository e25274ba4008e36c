"""Asynchronous VTK snapshots (covof_vtk_write_async) against a restatement
of the reference's vtk_write_step (oracle/vtk_writer.py): byte-identical
files; the snapshot holds the state at the call even while later steps run."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_vtk_snapshot_bytes_and_timing(gpu_pkg, orc, tmp_path):
    from oracle import vtk_writer as vw
    pkg = gpu_pkg
    p, C0, dt = pkg.cases.bubble_case(nx=24, ny=40, nsub=4)
    p.enable_svof_smoothing = 1
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.prepare_interface(p, f)
    with pkg.Solver(p) as s:
        s.state_set(f)
        s.run_steps(dt, 3, graph=True)
        snap = f.copy()
        s.state_get(snap)
        assert s.vtk_write_async(tmp_path, "bubble", 3) == 0
        s.run_steps(dt, 4, graph=True)      # runs while the file is written
        assert s.vtk_wait() == 0
        later = f.copy()
        s.state_get(later)
    assert not np.array_equal(later.u, snap.u)
    vtr = (tmp_path / "bubble_p0_000003.vtr").read_text()
    want = vw.vtr_text(p, snap.C, snap.C_s, snap.p, snap.rho, snap.mu, snap.u, snap.v, snap.curvature)
    assert vtr == want
    assert (tmp_path / "bubble_000003.pvtr").read_text() == vw.pvtr_text(p, "bubble", 3)


def test_vtk_creates_directory(gpu_pkg, tmp_path):
    pkg = gpu_pkg
    p = pkg.cases.make_params(8, 8, 1.0, 1.0)
    with pkg.Solver(p) as s:
        s.state_set(pkg.Fields.allocate(p))
        s.vtk_write_async(tmp_path / "a" / "b", "c", 0)
        assert s.vtk_wait() == 0
    assert (tmp_path / "a" / "b" / "c_p0_000000.vtr").exists()


def test_history_records(gpu_pkg, orc, tmp_path):
    from oracle import vtk_writer as vw
    pkg = gpu_pkg
    p, C0, dt = pkg.cases.bubble_case(nx=24, ny=40, nsub=4)
    f = pkg.Fields.allocate(p)
    f.C[...] = C0
    orc.apply_vof_bc(p, f.C)
    orc.prepare_interface(p, f)
    want = vw.HISTORY_HEADER
    with pkg.Solver(p) as s:
        s.state_set(f)
        s.history_open(tmp_path, "bubble")
        for k in range(1, 4):
            s.run_steps(dt, 2, graph=True)
            g = f.copy()
            s.state_get(g)
            s.history_write_async(tmp_path, "bubble", 2 * k, 2 * k * dt, dt)
            want += vw.history_line(p, 2 * k, 2 * k * dt, dt, g.C, g.p, g.rho, g.u, g.v)
        assert s.vtk_wait() == 0
    assert (tmp_path / "bubble_history.csv").read_text() == want
