"""The oracle's adaptive mesh refinement against the reference.

The fixtures come from the reference's own blast problem (pgen/blast.cpp) run with
refinement = adaptive (tests/golden/make_golden.py): every cycle's block list and dt and
the last cycle's state.  The oracle, driven by the host refinement logic of
athena_gb300.amr (refinement flags, tree update, regrid maps), must produce the same
block list and dt on every cycle and the same final state bit for bit — through the
initial refinement loop, refinement, derefinement, the face-field corrections of new
children and the re-initialisation after each regrid.
"""
import hashlib

import numpy as np
import pytest

import amr_run
from athena_gb300.amr import (C2F, F2C, SAME, AdaptiveMesh, blast_condition)
from athena_gb300.meshtree import Loc, MultiLevelMesh
from golden_cases import amr_case_names, load_amr_case


def _digest(mesh, u, b1, b2, b3):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(mesh.interior(u)).tobytes())
    for b in (b1, b2, b3):
        h.update(np.ascontiguousarray(mesh.interior_faces(b)).tobytes())
    return h.hexdigest()


def _locs(mesh):
    return [(l.level, l.lx1, l.lx2, l.lx3) for l in mesh.locs]


@pytest.mark.parametrize("name", amr_case_names())
def test_oracle_amr_matches_reference_bitwise(name):
    c, mesh0, ic, ref = load_amr_case(name)
    kw = dict(gamma=c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"], cfl=c["cfl"],
              tlim=c["tlim"], dfloor=c["floor"], pfloor=c["floor"])
    thr = c["problem"]["thr"]
    amr, om = amr_run.initialize(mesh0, ic, c["numlevel"], thr, c["derefine_count"], **kw)
    dts = []
    for _ in range(c["ncycle"]):
        dts.append(om.dt)
        last = {}

        def after(o):
            last["state"] = o.state()
            last["mesh"] = amr.mesh
            last["time"] = o.time
            n = len(dts) - 1
            assert _locs(amr.mesh) == ref["locs"][n], "block list differs at cycle %d" % (n + 1)
        om = amr_run.cycle(amr, om, thr, after_stages=after)
    np.testing.assert_array_equal(np.array(dts), ref["dt"])
    u, b1, b2, b3 = last["state"]
    m = last["mesh"]
    assert last["time"] == ref["time"]
    np.testing.assert_array_equal(m.interior(u).sum(axis=(2, 3, 4)), ref["usum"])
    assert _digest(m, u, b1, b2, b3) == ref["digest"]


def _mesh(nrbx=(2, 2, 2), bcs=(0, 0, 0, 0, 0, 0)):
    return MultiLevelMesh(tuple(8 * n for n in nrbx), nrbx, 2, (-.5, -.5, -.5),
                          (.5, .5, .5), bcs=bcs)


def test_refinement_flags_follow_check_refinement_condition():
    mesh = _mesh()
    mesh.tree.add_block(Loc(2, 0, 0, 0))
    mesh.rebuild()
    amr = AdaptiveMesh(mesh, numlevel=2, derefine_count=3)
    lev = np.array([l.level for l in mesh.locs])
    ret = np.where(lev == 2, -1, 1)
    # level-2 blocks: derefine only after three consecutive -1 results
    for it in range(3):
        flags = amr.check_refinement(ret)
        want = -1 if it == 2 else 0
        assert (flags[lev == 2] == want).all()
        assert (flags[lev == 1] == 1).all()          # root level, below the maximum
    # at the maximum level (root + numlevel - 1 = 2) a refine result gives no flag
    assert (amr.check_refinement(np.ones(mesh.nblocks))[lev == 2] == 0).all()
    # a 0 result resets the counter
    ret0 = ret.copy()
    ret0[lev == 2] = 0
    amr.check_refinement(ret0)
    assert (amr.deref_count[lev == 2] == 0).all()
    assert (blast_condition(np.array([2.0, 0.5, 0.1]), 1.0) == [1, 0, -1]).all()


def test_regrid_plan_maps_kept_restricted_and_prolongated_blocks():
    mesh = _mesh()
    mesh.tree.add_block(Loc(2, 0, 0, 0))
    mesh.rebuild()
    nb0 = mesh.nblocks
    amr = AdaptiveMesh(mesh, numlevel=3, derefine_count=1)
    flags = np.zeros(nb0, dtype=np.int32)
    # refine the root-level block at (1, 0, 0), derefine the eight level-2 siblings
    r = mesh.locs.index(Loc(1, 1, 0, 0))
    flags[r] = 1
    lv2 = [b for b in range(nb0) if mesh.locs[b].level == 2]
    flags[lv2] = -1
    plan = amr.update(flags)
    assert plan is not None
    kinds = list(plan.kind)
    assert kinds.count(F2C) == 1 and kinds.count(C2F) == 8
    n = kinds.index(F2C)
    assert plan.newtoold[n] == lv2[0]
    assert plan.mesh.locs[n] == Loc(1, 0, 0, 0)
    for b in np.nonzero(plan.kind == C2F)[0]:
        assert plan.newtoold[b] == r
    for b in np.nonzero(plan.kind == SAME)[0]:
        assert mesh.locs[plan.newtoold[b]] == plan.mesh.locs[b]
    # the new children take their x1 faces from the old level-2 blocks: the four on the
    # low-x1 side the inner face from lx1 = 1, the four on the high side the outer face
    # from lx1 = 0 across the periodic boundary
    assert len(plan.ffc) == 8
    for nb, face, old in plan.ffc:
        nl, ol = plan.mesh.locs[nb], mesh.locs[old]
        assert plan.kind[nb] == C2F and face == nl.lx1 - 2
        assert (ol.level, ol.lx1, ol.lx2, ol.lx3) == (2, 1 - face, nl.lx2, nl.lx3)


def test_no_regrid_without_flags():
    mesh = _mesh()
    amr = AdaptiveMesh(mesh, numlevel=2)
    assert amr.update(np.zeros(mesh.nblocks, dtype=np.int32)) is None
