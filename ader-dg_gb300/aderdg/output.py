"""Output in the reference's formats: the legacy ASCII VTK files of
write_data (cell-average primitive variables on the cell centres,
Euler/write_data.f90:8-95, Baer-Nunziato/write_data.f90, Advection-Diffusion/
write_data.f90) and of plot_troubled_cells (Euler/write_data.f90:101-192).
The cell averages come from the device (Solver.cell_averages /
Batch.cell_averages); this module only formats them.
"""
import math

import numpy as np

from .core import SYS_ADVDIFF, SYS_BN, SYS_EULER


def fortran_e(x, w, d):
    """Fortran `Ew.d` edit descriptor (0.ddd...E+xx, right-aligned in w columns)."""
    x = float(x)
    if not math.isfinite(x):
        return ("NaN" if x != x else ("Infinity" if x > 0 else "-Infinity")).rjust(w)
    if x == 0.0:
        return ("0." + "0" * d + "E+00").rjust(w)
    m, e = ("%.*E" % (d - 1, abs(x))).split("E")  # correctly rounded d significant digits
    digits = m.replace(".", "")
    e = int(e) + 1
    s = "%s0.%sE%s%02d" % ("-" if x < 0 else "", digits, "-" if e < 0 else "+", abs(e))
    return s.rjust(w)


_FIELDS = {
    SYS_EULER: [("SCALARS", "Density", (0,)), ("VECTORS", "Velocity", (1, 2)), ("SCALARS", "Pressure", (3,))],
    SYS_BN: [("SCALARS", "RHO_S", (0,)), ("VECTORS", "V_S", (1, 2)), ("SCALARS", "P_S", (3,)),
             ("SCALARS", "RHO_G", (4,)), ("VECTORS", "V_G", (5, 6)), ("SCALARS", "P_G", (7,)),
             ("SCALARS", "PHI_S", (8,))],
    SYS_ADVDIFF: [("SCALARS", "U", (0,))],
}


def write_vtk(path, cfg, wh, time):
    """write_data: wh = cell-average primitive variables [cell][nVar] (cell = i + IMAX j)."""
    wh = np.asarray(wh, dtype=np.float64).reshape(cfg.cells, cfg.nvar)
    I, J = cfg.imax, cfg.jmax
    dx, dy = (cfg.xr[0] - cfg.xl[0]) / I, (cfg.xr[1] - cfg.xl[1]) / J
    out = ["# vtk DataFile Version 2.0", "2D Euler", "ASCII", "DATASET STRUCTURED_GRID", "FIELD FieldData 1",
           "TIME 1 1 double", fortran_e(time, 15, 9), "DIMENSIONS %5d%5d%5d" % (I, J, 1),
           "POINTS %10d double" % (I * J)]
    for j in range(J):
        for i in range(I):
            xc = cfg.xl[0] + (i + 1 - 0.5) * dx
            yc = cfg.xl[1] + (j + 1 - 0.5) * dy
            out.append(fortran_e(xc, 15, 7) + fortran_e(yc, 15, 7) + fortran_e(0.0, 15, 7))
    out.append("POINT_DATA%10d" % (I * J))
    for kind, name, cols in _FIELDS[cfg.system]:
        if kind == "SCALARS":
            out += ["SCALARS %s double 1" % name, "LOOKUP_TABLE default"]
            out += [fortran_e(v, 15, 7) for v in wh[:, cols[0]]]
        else:
            out.append("VECTORS %s double" % name)
            out += [fortran_e(a, 15, 7) + fortran_e(b, 15, 7) + fortran_e(0.0, 15, 7)
                    for a, b in zip(wh[:, cols[0]], wh[:, cols[1]])]
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")


def write_troubled_cells_vtk(path, cfg, recompute, time):
    """plot_troubled_cells: the recompute map (2 troubled, 1 neighbour, 0 other) on the mesh."""
    rec = np.asarray(recompute).reshape(cfg.cells)
    I, J = cfg.imax, cfg.jmax
    dx, dy = (cfg.xr[0] - cfg.xl[0]) / I, (cfg.xr[1] - cfg.xl[1]) / J
    nn, ne = (I + 1) * (J + 1), I * J
    out = ["# vtk DataFile Version 2.0", "2D Euler", "ASCII", "DATASET UNSTRUCTURED_GRID", "FIELD FieldData 1",
           "TIME 1 1 double", fortran_e(time, 15, 9), "POINTS %10d double" % nn]
    for j in range(J + 1):
        for i in range(I + 1):
            out.append(fortran_e(cfg.xl[0] + i * dx, 15, 7) + fortran_e(cfg.xl[1] + j * dy, 15, 7) +
                       fortran_e(0.0, 15, 7))
    out.append("CELLS %10d%10d" % (ne, ne * 5))
    idxn = lambda i, j: i + (I + 1) * j  # noqa: E731  (0-based node number)
    for j in range(J):
        for i in range(I):
            out.append("%10d%10d%10d%10d%10d" % (4, idxn(i, j), idxn(i + 1, j), idxn(i + 1, j + 1), idxn(i, j + 1)))
    out.append("CELL_TYPES %10d" % ne)
    out += ["%5d" % 9] * ne
    out += ["CELL_DATA%10d" % ne, "SCALARS TCells double 1", "LOOKUP_TABLE default"]
    out += [fortran_e(2.0 if r == 1 else 1.0 if r == 2 else 0.0, 15, 7) for r in rec]
    with open(path, "w") as fh:
        fh.write("\n".join(out) + "\n")
