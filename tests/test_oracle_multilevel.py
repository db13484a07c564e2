"""The oracle's multi-level path (static mesh refinement) against the reference.

The fixtures come from the reference itself (tests/golden/make_golden.py): its own blast
problem generator or per-block loaded states on meshes with two and three refinement
levels, with periodic, outflow and reflecting faces, PLM+HLLE (NGHOST 2) and PPM+HLLD
(NGHOST 4).  The oracle must reproduce every cycle's dt and the final per-cell state bit
for bit; the block tree (gid order, neighbour lists) must be the reference's.
"""
import numpy as np
import pytest

import oracle as O
from athena_gb300 import pgen
from athena_gb300.meshtree import MultiLevelMesh
from golden_cases import load_ml_case, ml_case_names


@pytest.mark.parametrize("name", ml_case_names())
def test_oracle_multilevel_matches_reference_bitwise(name):
    c, mesh, ic, ref = load_ml_case(name)
    om = O.OracleMesh(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"],
                      cfl=c["cfl"], tlim=c["tlim"], integrator=c.get("integrator", "vl2"))
    om.set_state(*ic)
    om.initialize()
    dts = []
    for _ in range(c["ncycle"]):
        dts.append(om.dt)
        om.cycle()
    u, b1, b2, b3 = om.state()
    w, _ = om.prim()
    assert np.array_equal(np.array(dts), ref["dt"])
    assert np.array_equal(mesh.interior(u), ref["u"])
    assert np.array_equal(mesh.interior(w), ref["w"])
    for got, want in zip((b1, b2, b3), (ref["b1"], ref["b2"], ref["b3"])):
        assert np.array_equal(mesh.interior_faces(got), want)


def test_blast_blocks_restates_the_reference_generator():
    """pgen.blast_blocks gives the reference's blast.cpp initial state (the fixture's
    stored state is what the reference evolved: the oracle run above starts from it)."""
    c, mesh, ic, _ = load_ml_case("mlblast_hlle_plm")
    p = {"radius": 0.15, "pamb": 0.1, "prat": 100.0, "b0": 1.0, "angle_deg": 45.0,
         "center": (0.25, 0.25, 0.25)}
    u, b1, b2, b3 = pgen.blast_blocks(mesh, c["gamma"], **p)
    assert np.array_equal(u, ic[0])
    for a, b in zip((b1, b2, b3), ic[1:]):
        assert np.array_equal(a, b)


def test_tree_balance_and_neighbour_lists():
    """2:1 balance across faces, edges and corners, symmetric neighbour relations."""
    m = MultiLevelMesh((16, 16, 16), (4, 4, 4), 2, (-.5, -.5, -.5), (.5, .5, .5),
                       bcs=(0, 0, 0, 0, 0, 0),
                       regions=[((0.3, 0.3, 0.3), (0.35, 0.35, 0.35), 2)])
    assert sorted(set(m.levels.tolist())) == [2, 3, 4]
    for b, nbs in enumerate(m.nbrs):
        for q in nbs:
            assert abs(q.level - m.levels[b]) <= 1
            back = [e for e in m.nbrs[q.gid] if e.gid == b and
                    (e.ox1, e.ox2, e.ox3) == (-q.ox1, -q.ox2, -q.ox3)]
            assert len(back) == 1, (b, q)


def test_gpu_plan_builds_and_stays_in_bounds_on_the_host():
    """The library's multi-level planner (no device needed) accepts the golden meshes and a
    three-level periodic mesh, every operation's indices within the array bounds."""
    from athena_gb300.runtime import ml_plan_check
    for name in ml_case_names():
        _, mesh, _, _ = load_ml_case(name)
        counts = ml_plan_check(mesh)
        assert counts[1] > 0 and counts[2] > 0 and counts[3] > 0
    m = MultiLevelMesh((32, 32, 32), (4, 4, 4), 2, (-.5, -.5, -.5), (.5, .5, .5),
                       bcs=(0, 0, 0, 0, 0, 0),
                       regions=[((0.3, 0.3, 0.3), (0.35, 0.35, 0.35), 2)])
    assert ml_plan_check(m)[3] > 0
