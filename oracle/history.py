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


def wabs_divergence_b(mesh, b1, b2, b3):
    """The reference's |div B| history diagnostic WAbsDivergenceB
    (pgen/field_loop_poles.cpp:634-672), restated per cell with numpy in its operand
    order: |(A1 b1(i+1) - A1 b1(i) + A2 b2(j+1) - A2 b2(j) + A3 b3(k+1) - A3 b3(k)) / V|
    / (|B| / dl) over the interior cells of every block (Cartesian areas and volume from
    the blocks' own spacings, dl the smallest edge, |B| from the cell-centred field of the
    faces, cells with |B| = 0 skipped).  b1/b2/b3: per-block face arrays with ghosts.
    Returns (per-cell values [nb][nx3][nx2][nx1] with NaN where skipped, sum, max,
    count)."""
    ng = mesh.ng
    n1, n2, n3 = mesh.bx
    _, dx1f, _, dx2f, _, dx3f = mesh.coordinate_arrays()
    dx1 = dx1f[:, None, None, ng:ng + n1]
    dx2 = dx2f[:, None, ng:ng + n2, None]
    dx3 = dx3f[:, ng:ng + n3, None, None]
    f1m = b1[:, ng:ng + n3, ng:ng + n2, ng:ng + n1]
    f1p = b1[:, ng:ng + n3, ng:ng + n2, ng + 1:ng + n1 + 1]
    f2m = b2[:, ng:ng + n3, ng:ng + n2, ng:ng + n1]
    f2p = b2[:, ng:ng + n3, ng + 1:ng + n2 + 1, ng:ng + n1]
    f3m = b3[:, ng:ng + n3, ng:ng + n2, ng:ng + n1]
    f3p = b3[:, ng + 1:ng + n3 + 1, ng:ng + n2, ng:ng + n1]
    bc1 = 0.5 * f1m + 0.5 * f1p
    bc2 = 0.5 * f2m + 0.5 * f2p
    bc3 = 0.5 * f3m + 0.5 * f3p
    bmag = np.sqrt(bc1 * bc1 + bc2 * bc2 + bc3 * bc3)
    a1, a2, a3 = dx2 * dx3, dx1 * dx3, dx1 * dx2
    dl = np.minimum(np.minimum(dx1, dx2), dx3)
    vol = dx1 * dx2 * dx3
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.abs(((((a1 * f1p - a1 * f1m) + a2 * f2p) - a2 * f2m) + a3 * f3p - a3 * f3m)
                   / vol) / (bmag / dl)
    v = np.where(bmag != 0.0, v, np.nan)
    ok = ~np.isnan(v)
    return v, float(np.sum(v[ok])), float(np.max(v[ok])) if ok.any() else 0.0, int(ok.sum())
