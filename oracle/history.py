"""CPU oracle of the history output (test infrastructure only): the volume-weighted sums
of HistoryOutput::WriteOutputFile (outputs/history.cpp:77-140) over interior cells, in
FP64 with numpy (summation order differs from the reference's sequential loop, so it
agrees with the reference's Ref.hst to rounding)."""
import numpy as np

NAMES = ("mass", "1-mom", "2-mom", "3-mom", "1-KE", "2-KE", "3-KE", "tot-E", "1-ME", "2-ME",
         "3-ME")


def history_sums(mesh, u, b1, b2, b3):
    """u: per-block interior conserved [nb][5][nx3][nx2][nx1]; b1/b2/b3: per-block interior
    face fields [nb][nx3][nx2][nx1+1] etc.; uniform spacings from the mesh."""
    dx = [(mesh.xmax[d] - mesh.xmin[d]) / mesh.nx[d] for d in range(3)]
    vol = dx[0] * dx[1] * dx[2]
    d, m1, m2, m3, e = (u[:, n] for n in range(5))
    bc1 = 0.5 * b1[..., :-1] + 0.5 * b1[..., 1:]
    bc2 = 0.5 * b2[:, :, :-1, :] + 0.5 * b2[:, :, 1:, :]
    bc3 = 0.5 * b3[:, :-1] + 0.5 * b3[:, 1:]
    vals = (vol * d, vol * m1, vol * m2, vol * m3, vol * 0.5 * (m1 * m1) / d,
            vol * 0.5 * (m2 * m2) / d, vol * 0.5 * (m3 * m3) / d, vol * e,
            vol * 0.5 * bc1 * bc1, vol * 0.5 * bc2 * bc2, vol * 0.5 * bc3 * bc3)
    return {k: float(np.sum(v)) for k, v in zip(NAMES, vals)}
