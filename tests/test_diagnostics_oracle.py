"""The oracle's restatement of the reference's |div B| diagnostic (WAbsDivergenceB,
pgen/field_loop_poles.cpp:634-672) on known fields (CPU)."""
import numpy as np

import history
from athena_gb300 import pgen
from athena_gb300.mesh import MeshSpec


def _faces(mesh, seed=3):
    gu, f1, f2, f3 = pgen.turbulence(mesh.nx, seed=seed, mach=1.0)
    return list(mesh.scatter_faces(f1, f2, f3))


def test_uniform_field_is_divergence_free():
    mesh = MeshSpec((16, 16, 16), (2, 2, 2), 2)
    v, s, m, c = history.wabs_divergence_b(mesh, *_faces(mesh))
    assert s == 0.0 and m == 0.0 and c == 16 ** 3


def test_planted_face_gives_the_analytic_value():
    """Raising one x1 face by delta changes the divergence of its two cells by
    +-delta * A1 / V = +-delta / dx1; the diagnostic divides by |B| / dl."""
    mesh = MeshSpec((16, 8, 8), (1, 1, 1), 2, (0., 0., 0.), (2.0, 1.0, 1.0))
    b1, b2, b3 = _faces(mesh)
    ng, delta = mesh.ng, 1.0e-3
    k, j, i = ng + 3, ng + 4, ng + 5
    b1[0, k, j, i] += delta
    v, s, m, c = history.wabs_divergence_b(mesh, b1, b2, b3)
    dx = 2.0 / 16
    for cell, ii in ((i - 1, i), (i, i)):  # the cells left and right of face i
        bc = np.array([0.5 * b1[0, k, j, cell] + 0.5 * b1[0, k, j, cell + 1],
                       0.5 * b2[0, k, j, cell] + 0.5 * b2[0, k, j + 1, cell],
                       0.5 * b3[0, k, j, cell] + 0.5 * b3[0, k + 1, j, cell]])
        want = (delta / dx) / (np.sqrt((bc ** 2).sum()) / dx)
        got = v[0, k - ng, j - ng, cell - ng]
        assert abs(got - want) < 1e-9 * want
    others = np.ones(v.shape, bool)
    others[0, k - ng, j - ng, i - 1 - ng:i + 1 - ng] = False
    assert np.nanmax(v[others]) < 1e-13
