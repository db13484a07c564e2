"""The relativistic MHD shock tubes of the reference's regression suite
(tst/regression/scripts/tests/sr/mhd_shocks_hlld.py, inputs/mhd_sr/athinput.mub_{1,2,4}:
Mignone, Ugliano & Bodo 2009 problems 1, 2, 4; VL2 + PLM + HLLD, CFL 0.4, outflow x1)
run as quasi-one-dimensional 3-D meshes (2 x 2 cells across, periodic), and the suite's
comparison: the L1 difference of each conserved variable against the reference's
10000-zone HLLD solution on the union of the two grids, relative to that solution's L1
norm (scripts/utils/comparison.py), with the suite's tolerances (ZERO_TOL below for its zeros)."""
import math
import os

import numpy as np

from athena_gb300 import pgen
from athena_gb300.mesh import MeshSpec

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# problem -> (gamma, nx1, tlim, left, right); states (rho, p, vx, vy, vz, Bx, By, Bz)
PROBLEMS = {
    1: (2.0, 400, 0.4, (1.0, 1.0, 0.0, 0.0, 0.0, 0.5, 1.0, 0.0),
        (0.125, 0.1, 0.0, 0.0, 0.0, 0.5, -1.0, 0.0)),
    2: (1.6666666666666667, 800, 0.55, (1.08, 0.95, 0.4, 0.3, 0.2, 2.0, 0.3, 0.3),
        (1.0, 1.0, -0.45, -0.2, 0.2, 2.0, -0.7, 0.5)),
    4: (1.6666666666666667, 800, 0.5, (1.0, 5.0, 0.0, 0.3, 0.4, 1.0, 6.0, 2.0),
        (0.9, 5.3, 0.0, 0.0, 0.0, 1.0, 5.0, 2.0)),
}
# mhd_shocks_hlld.py tol_sets: dens, Etot, mom x/y/z, B x/y/z
TOLERANCES = {1: (0.02, 0.01, 0.02, 0.04, 0.0, 0.0, 0.01, 0.0),
              2: (0.003, 0.002, 0.007, 0.01, 0.005, 0.0, 0.004, 0.007),
              4: (0.002, 0.001, 0.02, 0.03, 0.004, 0.0, 0.001, 0.003)}
CFL = 0.4
BC = (1, 1, 0, 0, 0, 0)   # outflow x1, periodic x2 and x3


def setup(problem):
    """(mesh, gamma, tlim, (u, b1, b2, b3) per block, w per block)."""
    gamma, nx1, tlim, left, right = PROBLEMS[problem]
    mesh = MeshSpec((nx1, 2, 2), (1, 1, 1), 2, (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5))
    w, f1, f2, f3 = pgen.sr_shock_tube(mesh.nx, mesh.xmin, mesh.xmax, left, right)
    u = pgen.sr_prim_to_cons(w, pgen.cell_centered(f1, f2, f3), gamma)
    ic = (mesh.scatter_cells(u),) + mesh.scatter_faces(f1, f2, f3)
    return mesh, gamma, tlim, ic, mesh.scatter_cells(w)


def l1_norm(faces, vals):
    return math.fsum(abs(vals) * np.ediff1d(faces))


def l1_diff(faces_1, vals_1, faces_2, vals_2):
    faces = np.union1d(faces_1, faces_2)

    def fill(fc, vals):
        out = np.empty(len(faces) - 1)
        idx = np.searchsorted(fc, faces[:-1], side="right") - 1
        out[:] = np.asarray(vals)[np.clip(idx, 0, len(vals) - 1)]
        return out
    return math.fsum(abs(fill(faces_1, vals_1) - fill(faces_2, vals_2)) * np.ediff1d(faces))


def errors(problem, mesh, u, bcc):
    """Relative L1 differences (dens, Etot, mom x/y/z, B x/y/z) of a run's conserved
    state and cell-centred field (one x1 row of the interior) against the reference's
    solution, both in float32 as the suite's VTK files hold them."""
    z = np.load(os.path.join(GOLDEN, "sr_mhd_shocks_ref.npz"))
    xr = z["x1f_%d" % problem].astype(np.float64)
    ref = [z["dens_%d" % problem], z["Etot_%d" % problem]] + \
          [z["mom_%d" % problem][:, a] for a in range(3)] + \
          [z["ccB_%d" % problem][:, a] for a in range(3)]
    ng = mesh.ng
    ui = np.asarray(u)[0][:, ng, ng, ng:-ng]      # block 0: [5][nc3][nc2][nc1]
    bi = np.asarray(bcc)[0][:, ng, ng, ng:-ng]
    # conserved slots: D, M1, M2, M3, E (the VTK's Etot is the total energy E)
    new = [ui[0], ui[4], ui[1], ui[2], ui[3], bi[0], bi[1], bi[2]]
    xn = np.asarray(mesh.coordinate_arrays()[0][0][ng:ng + mesh.bx[0] + 1],
                    dtype=np.float32).astype(np.float64)
    out = []
    for r, v in zip(ref, new):
        e = l1_diff(xr, r.astype(np.float64), xn, v.astype(np.float32).astype(np.float64))
        n = l1_norm(xr, r.astype(np.float64))
        out.append(e if n == 0.0 else e / n)
    return out


# The suite's zero tolerances mark components that stay exactly constant in the
# reference's 1-D build (B_x, and the components with no source in the problem).  The
# quasi-1-D 3-D mesh also runs the x2 and x3 sweeps and their corner EMFs on states that
# are uniform across; the relativistic HLLD returns the flux of two equal states only to
# its secant iteration's roundoff, so those components pick up roundoff (1e-12 of the
# L1 after 400-1100 cycles).  They are held to 1e-9 here.
ZERO_TOL = 1e-9


def within(problem, errs, zero_tol=ZERO_TOL):
    return all((e <= zero_tol) if t == 0.0 else (e <= t) for e, t in
               zip(errs, TOLERANCES[problem]))
