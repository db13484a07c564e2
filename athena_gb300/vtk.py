"""Legacy VTK output in the reference's format (VTKOutput::WriteOutputFile,
outputs/vtk.cpp:51-223): one file per MeshBlock, ``<basename>.block<gid>.<file_id>.<number
%05d>.vtk``, a RECTILINEAR_GRID of the interior with big-endian FP32 face coordinates and
cell data.  Variables as the reference's output sets them (OutputType::LoadOutputData,
outputs/outputs.cpp:495-660 for MHD): ``prim`` = rho, press, vel, Bcc; ``cons`` = dens,
Etot, mom, Bcc.
"""
import os

import numpy as np

from .restart import reference_order


def _vars(variable, u, w, bcc, b):
    if variable == "prim":
        return [("SCALARS", "rho", w[b, 0:1]), ("SCALARS", "press", w[b, 4:5]),
                ("VECTORS", "vel", w[b, 1:4]), ("VECTORS", "Bcc", bcc[b])]
    if variable == "cons":
        return [("SCALARS", "dens", u[b, 0:1]), ("SCALARS", "Etot", u[b, 4:5]),
                ("VECTORS", "mom", u[b, 1:4]), ("VECTORS", "Bcc", bcc[b])]
    raise ValueError("variable must be prim or cons")


def write(dirpath, mesh, u, w, bcc, time, ncycle, variable="prim", basename="Ref",
          file_id="out1", file_number=0):
    """Write one output of every block of ``mesh`` (arrays in this package's block
    order, ghosts included); returns the file names."""
    ng = mesh.ng
    n1, n2, n3 = mesh.bx
    coords = mesh.coordinate_arrays()   # x1f, dx1f, x2f, dx2f, x3f, dx3f
    names = []
    for gid, (b, _) in enumerate(reference_order(mesh)):
        fname = os.path.join(dirpath, "%s.block%d.%s.%05d.vtk" % (basename, gid, file_id,
                                                                 file_number))
        parts = [("# vtk DataFile Version 2.0\n"
                  "# Athena++ data at time=%e  cycle=%d  variables=%s \n"
                  "BINARY\nDATASET RECTILINEAR_GRID\nDIMENSIONS %d %d %d\n"
                  % (time, ncycle, variable, n1 + 1, n2 + 1, n3 + 1)).encode()]
        for d, (lab, n) in enumerate((("X", n1), ("Y", n2), ("Z", n3))):
            if d:
                parts.append(b"\n")
            parts.append(("%s_COORDINATES %d float\n" % (lab, n + 1)).encode())
            xf = coords[2 * d][b][ng:ng + n + 1]
            parts.append(np.asarray(xf, dtype=">f4").tobytes())
        parts.append(("\nCELL_DATA %d" % (n1 * n2 * n3)).encode())
        for typ, name, arr in _vars(variable, u, w, bcc, b):
            nvar = arr.shape[0]
            parts.append(("\n%s %s float\n" % (typ, name)).encode())
            if nvar == 1:
                parts.append(b"LOOKUP_TABLE default\n")
            inner = arr[:, ng:ng + n3, ng:ng + n2, ng:ng + n1]     # [nvar][k][j][i]
            parts.append(np.ascontiguousarray(np.moveaxis(inner, 0, -1), dtype=">f4")
                         .tobytes())
        with open(fname, "wb") as f:
            f.write(b"".join(parts))
        names.append(fname)
    return names
