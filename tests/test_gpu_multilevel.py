"""Multi-level meshes (static mesh refinement) on the GPU.

The CUDA FP64 path must reproduce the reference bit for bit on the multi-level golden
cases (every cycle's dt, per-cell conserved and primitive state, face fields) and the
oracle bit for bit with the ghost zones included; the FP32 path tracks FP64 and keeps
div B at roundoff across refinement boundaries.
"""
import numpy as np
import pytest

import oracle as O
from athena_gb300 import build, pgen
from athena_gb300.meshtree import MultiLevelMesh
from athena_gb300.runtime import StageUpdate
from golden_cases import load_ml_case, ml_case_names

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _run(mesh, c, ic, ncycle, precision="fp64"):
    g = StageUpdate(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"],
                    precision=precision, cfl=c["cfl"], tlim=c["tlim"],
                    integrator=c.get("integrator", "vl2"))
    g.set_state(*ic)
    g.initialize()
    dts = []
    for _ in range(ncycle):
        dts.append(g.dt)
        g.cycle(1)
    out = g.state()
    w, bcc = g.prim()
    g.close()
    return out, np.array(dts), w, bcc


@pytest.mark.parametrize("name", ml_case_names())
def test_multilevel_fp64_matches_reference_bitwise(name):
    c, mesh, ic, ref = load_ml_case(name)
    (u, b1, b2, b3), dts, w, _ = _run(mesh, c, ic, c["ncycle"])
    assert np.array_equal(dts, ref["dt"])
    assert np.array_equal(mesh.interior(u), ref["u"])
    assert np.array_equal(mesh.interior(w), ref["w"])
    for got, want in zip((b1, b2, b3), (ref["b1"], ref["b2"], ref["b3"])):
        assert np.array_equal(mesh.interior_faces(got), want)


def _smooth_case(ng=2, xorder=2, rsolver="hlle", bcs=(0, 0, 0, 0, 0, 0)):
    mesh = MultiLevelMesh((32, 32, 32), (4, 4, 4), ng, (-.5, -.5, -.5), (.5, .5, .5),
                          bcs=bcs, regions=[((0.3, 0.3, 0.3), (0.35, 0.35, 0.35), 2)])
    c = {"gamma": 5.0 / 3.0, "xorder": xorder, "rsolver": rsolver, "cfl": 0.3, "tlim": 1e3}
    return mesh, pgen.smooth_blocks(mesh, seed=5), c


@pytest.mark.parametrize("ng,xorder,rsolver,bcs,integ", [
    (2, 2, "hlle", (0, 0, 0, 0, 0, 0), "vl2"), (4, 3, "hlld", (1, 1, 2, 2, 1, 2), "vl2"),
    (2, 2, "roe", (2, 1, 0, 0, 1, 1), "vl2"), (2, 2, "llf", (0, 0, 1, 2, 0, 0), "vl2"),
    (4, "3f", "hlle", (1, 2, 0, 0, 2, 1), "vl2"), (4, 3, "hlld", (2, 1, 0, 0, 1, 2), "rk2")])
def test_multilevel_fp64_matches_oracle_with_ghosts(ng, xorder, rsolver, bcs, integ):
    """Three levels, 127+ blocks: the state after three cycles equals the oracle's bit for
    bit, ghost zones of W and B included."""
    mesh, ic, c = _smooth_case(ng, xorder, rsolver, bcs)
    c["integrator"] = integ
    (u, b1, b2, b3), dts, w, bcc = _run(mesh, c, ic, 3)
    om = O.OracleMesh(mesh, c["gamma"], xorder=xorder, rsolver=rsolver, tlim=c["tlim"],
                      integrator=integ)
    om.set_state(*ic)
    om.initialize()
    odts = []
    for _ in range(3):
        odts.append(om.dt)
        om.cycle()
    uo, o1, o2, o3 = om.state()
    wo, bcco = om.prim()
    assert np.array_equal(dts, np.array(odts))
    assert np.array_equal(mesh.interior(u), mesh.interior(uo))
    assert np.array_equal(w, wo)
    assert np.array_equal(bcc, bcco)
    for a, b in zip((b1, b2, b3), (o1, o2, o3)):
        assert np.array_equal(a, b)


def _div_b(mesh, b1, b2, b3):
    ng, (n1, n2, n3) = mesh.ng, mesh.bx
    d1 = b1[:, ng:ng + n3, ng:ng + n2, ng + 1:ng + n1 + 1] - b1[:, ng:ng + n3, ng:ng + n2, ng:ng + n1]
    d2 = b2[:, ng:ng + n3, ng + 1:ng + n2 + 1, ng:ng + n1] - b2[:, ng:ng + n3, ng:ng + n2, ng:ng + n1]
    d3 = b3[:, ng + 1:ng + n3 + 1, ng:ng + n2, ng:ng + n1] - b3[:, ng:ng + n3, ng:ng + n2, ng:ng + n1]
    return d1 + d2 + d3


def test_multilevel_fp32_tracks_fp64_and_keeps_div_b():
    mesh, _, c = _smooth_case()
    # a divergence-free initial field: uniform faces, smooth hydro state
    u, b1, b2, b3 = pgen.blast_blocks(mesh, c["gamma"], radius=0.2, pamb=0.1, prat=10.0,
                                      b0=1.0, angle_deg=30.0, center=(0.3, 0.3, 0.3))
    ic = (u, b1, b2, b3)
    (u64, f1, f2, f3), dt64, _, _ = _run(mesh, c, ic, 4, "fp64")
    (u32, g1, g2, g3), dt32, _, _ = _run(mesh, c, ic, 4, "fp32")
    a, b = mesh.interior(u64), mesh.interior(u32)
    for n in (0, 4):
        rel = np.abs(a[:, n] - b[:, n]).mean() / np.abs(a[:, n]).mean()
        assert rel < 1e-5, (n, rel)
    assert np.allclose(dt32, dt64, rtol=1e-5)
    for f in ((f1, f2, f3), (g1, g2, g3)):
        assert np.abs(_div_b(mesh, *f)).max() < 1e-12
