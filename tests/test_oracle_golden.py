"""The oracle against the reference's own outputs (golden fixtures): bit-exact."""
import hashlib
import math

import numpy as np
import pytest

import oracle as O
from athena_gb300.mesh import MeshSpec
from athena_gb300 import pgen
from golden_cases import case_names, load_case, interior_faces, meta


@pytest.mark.parametrize("name", case_names())
def test_oracle_matches_reference_bitwise(name):
    c, mesh, ic, ref = load_case(name)
    om = O.OracleMesh(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"],
                      cfl=c["cfl"], tlim=c["tlim"], relativistic=c.get("relativistic", False),
                      bc=tuple(c.get("bc", (0,) * 6)),
                      integrator=c.get("integrator", "vl2"))
    om.set_state(*ic)
    if "ic_w" in c:
        om.set_prim(c["ic_w"])
    om.initialize()
    dts = []
    for _ in range(c["ncycle"]):
        dts.append(om.dt)
        om.cycle()
    assert np.array_equal(np.array(dts), ref["dt"])
    u, b1, b2, b3 = om.state()
    assert np.array_equal(mesh.interior(u), ref["u"])
    for got, want in ((b1, ref["b1"]), (b2, ref["b2"]), (b3, ref["b3"])):
        assert np.array_equal(interior_faces(mesh, got), want)
    if "w" in ref:
        w, _ = om.prim()
        assert np.array_equal(mesh.interior(w), ref["w"])


def test_linear_wave_ic_matches_reference():
    """Our restatement of linear_wave.cpp gives the reference's initial state bit for bit
    (the golden IC is the state the reference's own problem generator produced)."""
    c, mesh, ic, _ = load_case("lw_hlld_plm_8blk")
    u, b1, b2, b3 = pgen.LinearWave(mesh, gamma=c["gamma"]).generate()
    assert np.array_equal(mesh.interior(u), mesh.interior(ic[0]))
    for got, want in ((b1, ic[1]), (b2, ic[2]), (b3, ic[3])):
        assert np.array_equal(interior_faces(mesh, got), interior_faces(mesh, want))


def test_config1_linear_wave_l1_error():
    """Config 1 (64x32x32, VL2 + PLM + HLLD, one wave period): the oracle reproduces the
    reference's final state bit for bit and its linearwave-errors.dat line."""
    g = meta()["config1_linear_wave"]
    mesh = MeshSpec((64, 32, 32), (1, 1, 1), 2, (0., 0., 0.), (3.0, 1.5, 1.5))
    lw = pgen.LinearWave(mesh, gamma=1.666666666666667)
    om = O.OracleMesh(mesh, 1.666666666666667, xorder=2, rsolver="hlld", cfl=0.3,
                      tlim=lw.period())
    om.set_state(*lw.generate())
    om.initialize()
    n = 0
    while om.time < lw.period():
        om.cycle()
        n += 1
    assert n == g["ncycle"] == 72
    u, b1, b2, b3 = om.state()
    ng = mesh.ng
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(mesh.interior(u)).tobytes())
    for b in (b1, b2, b3):
        h.update(np.ascontiguousarray(b[:, ng:-ng, ng:-ng, ng:-ng]).tobytes())
    assert h.hexdigest() == g["sha256_final"]
    w, bcc = om.prim()
    rms, l1, mx = lw.l1_errors(u, bcc)
    fields = g["errors"].split()
    assert "%e" % rms == fields[4]
    assert ["%e" % v for v in l1] == fields[5:13]
