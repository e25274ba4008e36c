"""TEST INFRASTRUCTURE ONLY: restatement of the reference's VTK step writer
(src/module_vtk_writer.f90:90-386, vtk_write_step) for one rank, used to check
the library's asynchronous writer byte for byte.  Fortran's ES16.8 edit
descriptor is Python's "%16.8E" for exponents of two digits; a record ended by
an empty list-directed write is a newline.  Arrays in the reference layout
(ny+2, nx+2)."""
from __future__ import annotations

import numpy as np


def _es(x) -> str:
    return "%16.8E " % x


def vtr_text(p, C, C_s, pres, rho, mu, u, v, curvature, temperature=300.0) -> str:
    nx, ny, dx, dy = p.nx, p.ny, p.dx, p.dy
    out = ['<?xml version="1.0"?>\n',
           '<VTKFile type="RectilinearGrid" version="0.1" byte_order="LittleEndian">\n',
           '  <RectilinearGrid WholeExtent="%d %d %d %d 0 0">\n' % (0, nx, 0, ny),
           '    <Piece Extent="%d %d %d %d 0 0">\n' % (0, nx, 0, ny),
           '      <CellData Scalars="PhaseIndicator,Pressure,Density,Viscosity,Divergence" Vectors="Velocity">\n']

    def scalar(name, f):
        out.append('        <DataArray type="Float64" Name="%s" format="ascii">\n' % name)
        for j in range(1, ny + 1):
            out.append("".join(_es(f(i, j)) for i in range(1, nx + 1)) + "\n")
        out.append('        </DataArray>\n')

    scalar("PhaseIndicator", lambda i, j: C[j, i])
    scalar("PhaseIndicator_Smoothed", lambda i, j: C_s[j, i])
    scalar("Pressure", lambda i, j: pres[j, i])
    scalar("Density", lambda i, j: rho[j, i])
    scalar("Viscosity", lambda i, j: mu[j, i])
    scalar("Divergence", lambda i, j: (u[j, i + 1] - u[j, i]) / dx + (v[j + 1, i] - v[j, i]) / dy)
    scalar("Temperature", lambda i, j: temperature)
    scalar("Curvature", lambda i, j: curvature[j, i])
    out.append('        <DataArray type="Float64" Name="Velocity" NumberOfComponents="3" format="ascii">\n')
    for j in range(1, ny + 1):
        out.append("".join(_es(0.5 * (u[j, i] + u[j, i + 1])) + _es(0.5 * (v[j, i] + v[j + 1, i])) + "0.0 "
                           for i in range(1, nx + 1)) + "\n")
    out.append('        </DataArray>\n')
    out.append('      </CellData>\n')
    out.append('      <Coordinates>\n')
    out.append('        <DataArray type="Float64" Name="XCoordinates" format="ascii">\n')
    out.append("".join(_es(float(i) * dx) for i in range(nx + 1)) + "\n")
    out.append('        </DataArray>\n')
    out.append('        <DataArray type="Float64" Name="YCoordinates" format="ascii">\n')
    out.append("".join(_es(float(j) * dy) for j in range(ny + 1)) + "\n")
    out.append('        </DataArray>\n')
    out.append('        <DataArray type="Float64" Name="ZCoordinates" format="ascii">\n')
    out.append('          0.0\n')
    out.append('        </DataArray>\n')
    out += ['      </Coordinates>\n', '    </Piece>\n', '  </RectilinearGrid>\n', '</VTKFile>\n']
    return "".join(out)


def pvtr_text(p, case_name: str, step: int) -> str:
    names = ["PhaseIndicator", "PhaseIndicator_Smoothed", "Pressure", "Density", "Viscosity", "Divergence",
             "Temperature", "Curvature"]
    out = ['<?xml version="1.0"?>\n',
           '<VTKFile type="PRectilinearGrid" version="0.1" byte_order="LittleEndian">\n',
           '  <PRectilinearGrid WholeExtent="0 %d 0 %d 0 0" GhostLevel="0">\n' % (p.nx, p.ny),
           '    <PCellData Scalars="PhaseIndicator,Pressure,Density,Viscosity,Divergence" Vectors="Velocity">\n']
    out += ['      <PDataArray type="Float64" Name="%s"/>\n' % n for n in names]
    out += ['      <PDataArray type="Float64" Name="Velocity" NumberOfComponents="3"/>\n',
            '    </PCellData>\n', '    <PCoordinates>\n',
            '      <PDataArray type="Float64" Name="XCoordinates"/>\n',
            '      <PDataArray type="Float64" Name="YCoordinates"/>\n',
            '      <PDataArray type="Float64" Name="ZCoordinates"/>\n',
            '    </PCoordinates>\n',
            '    <Piece Extent="%d %d %d %d 0 0" Source="%s_p0_%06d.vtr"/>\n' % (0, p.nx, 0, p.ny, case_name, step),
            '  </PRectilinearGrid>\n', '</VTKFile>\n']
    return "".join(out)


HISTORY_HEADER = ("step,time,dt,center_of_mass_y,rise_velocity,bubble_volume,kinetic_energy,max_u,max_div,"
                  "avg_rho_gas,avg_p_gas\n")


def history_line(p, step, time, dt, C, pres, rho, u, v, temperature=300.0) -> str:
    """vtk_write_diagnostics (src/module_vtk_writer.f90:392-470), one rank:
    the serial sums in the reference's order, then the I0 / ES14.6 record."""
    import math
    nx, ny, dx, dy = p.nx, p.ny, p.dx, p.dy
    dvol = dx * dy
    vol = gvol = yint = vint = mgas = pgas = ke = 0.0
    umax = dmax = 0.0
    for j in range(1, ny + 1):
        y_pos = (float(j - 1) + 0.5) * dy
        for i in range(1, nx + 1):
            c = float(C[j, i]); pr = float(pres[j, i])
            ib = 1.0 - c
            vol = vol + ib * dvol
            yint = yint + y_pos * ib * dvol
            ig = 1.0 - c
            rg = pr / (287.05 * max(1.0, temperature))
            mgas = mgas + ig * rg * dvol
            pgas = pgas + ig * pr * dvol
            gvol = gvol + ig * dvol
            uw, ue = float(u[j, i]), float(u[j, i + 1])
            vs, vn = float(v[j, i]), float(v[j + 1, i])
            uc = 0.5 * (uw + ue); vc = 0.5 * (vs + vn)
            vint = vint + vc * ib * dvol
            sp2 = uc * uc + vc * vc
            u2p = 0.5 * (uw * uw + ue * ue); v2p = 0.5 * (vs * vs + vn * vn)
            ke = ke + 0.5 * float(rho[j, i]) * (u2p + v2p) * dvol
            sp = math.sqrt(sp2)
            if sp > umax:
                umax = sp
            dv = abs((ue - uw) / dx + (vn - vs) / dy)
            if dv > dmax:
                dmax = dv
    yc = yint / vol if vol > 1e-12 else 0.0
    vcm = vint / vol if vol > 1e-12 else 0.0
    rho_g = mgas / gvol if gvol > 1e-12 else 0.0
    p_g = pgas / gvol if gvol > 1e-12 else 0.0
    vals = (time, dt, yc, vcm, vol, ke, umax, dmax, rho_g, p_g)
    return "%d," % step + ",".join("%14.6E" % x for x in vals) + "\n"
