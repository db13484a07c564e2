"""The library's native adaptive-mesh host code (athgpu_amr_*) against the Python
restatement (athena_gb300.meshtree, athena_gb300.amr), which the oracle tests pin to the
reference: the same block lists, neighbour tables, neighbour levels, coordinates,
refinement flags, derefinement counters and regrid maps, through random sequences of
refinement and derefinement.  Host code only: no GPU needed.
"""
import numpy as np
import pytest

from athena_gb300.adaptive import NativeAmr, NativeMesh
from athena_gb300.amr import AdaptiveMesh
from athena_gb300.meshtree import MultiLevelMesh


def _compare_meshes(py, nat):
    assert [tuple(l.__dict__.values()) if hasattr(l, "__dict__") else l for l in py.locs] == \
        [tuple(l.__dict__.values()) if hasattr(l, "__dict__") else l for l in nat.locs]
    t0, c0, l0, loc0 = py.neighbor_table()
    t1, c1, l1, loc1 = nat.neighbor_table()
    np.testing.assert_array_equal(c0, c1)
    np.testing.assert_array_equal(l0, l1)
    np.testing.assert_array_equal(loc0, loc1)
    for b in range(py.nblocks):   # entries beyond the count are unused
        np.testing.assert_array_equal(t0[b, :c0[b]], t1[b, :c1[b]])
    for a, b in zip(py.coordinate_arrays(), nat.coordinate_arrays()):
        np.testing.assert_array_equal(a, b)
    for a, b in zip(py.coarse_coordinate_arrays(), nat.coarse_coordinate_arrays()):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("bcs,nrbx,seed", [((0,) * 6, (2, 2, 2), 1),
                                           ((0,) * 6, (4, 2, 3), 2),
                                           ((1, 1, 2, 2, 0, 0), (2, 3, 2), 3)])
def test_native_amr_host_matches_python(bcs, nrbx, seed):
    rng = np.random.default_rng(seed)
    nx = tuple(8 * n for n in nrbx)
    kwm = dict(xmin=(-.5, -.3, -.7), xmax=(.5, .6, .2), bcs=bcs)
    py = AdaptiveMesh(MultiLevelMesh(nx, nrbx, 2, **kwm), numlevel=4, derefine_count=2)
    nat = NativeAmr(nx, nrbx, 2, kwm["xmin"], kwm["xmax"], bcs, 4, 2)
    _compare_meshes(py.mesh, NativeMesh(nat))
    changes = 0
    for it in range(14):
        nb = py.mesh.nblocks
        # refine a few blocks, ask most others to derefine
        ret = np.where(rng.random(nb) < 0.12, 1, np.where(rng.random(nb) < 0.7, -1, 0))
        f0 = py.check_refinement(ret)
        f1 = nat.flags(ret)
        np.testing.assert_array_equal(f0, f1)
        np.testing.assert_array_equal(py.deref_count, nat.deref_counts())
        plan = py.update(f0)
        changed = nat.update(f1)
        assert changed == (plan is not None)
        if plan is None:
            continue
        changes += 1
        newtoold, kind, ffc, dc = nat.pending_maps()
        np.testing.assert_array_equal(plan.newtoold, newtoold)
        np.testing.assert_array_equal(plan.kind, kind)
        np.testing.assert_array_equal(plan.ffc, ffc)
        np.testing.assert_array_equal(plan.deref_count, dc)
        py.accept(plan)
        nat.accept()
        _compare_meshes(py.mesh, NativeMesh(nat))
    assert changes >= 3
    nat.close()


def test_native_static_blocks_match_python_regions():
    from athena_gb300.meshtree import Loc
    mesh = MultiLevelMesh((32, 32, 32), (4, 4, 4), 2, (-.5,) * 3, (.5,) * 3,
                          regions=[((0.1, 0.1, 0.1), (0.2, 0.2, 0.2), 2)])
    nat = NativeAmr(mesh.nx, mesh.nrbx, 2, mesh.xmin, mesh.xmax, mesh.bcs, 3)
    for loc in mesh.locs:
        if loc.level > mesh.tree.root_level:
            nat.add_block(loc)
    _compare_meshes(mesh, NativeMesh(nat))
    with pytest.raises(Exception):
        nat.add_block(Loc(9, 0, 0, 0))       # beyond numlevel
    nat.close()


def test_native_mesh_tables_are_fetched_lazily_and_guarded():
    """A NativeMesh fetches only the block list when made; its neighbour tables and
    coordinates, fetched on first use, equal an eager fetch, and a block list made before
    the tree changed refuses to fetch them afterwards."""
    from athena_gb300.meshtree import Loc
    nat = NativeAmr((16, 16, 16), (2, 2, 2), 2, (-.5,) * 3, (.5,) * 3, (0,) * 6, 3, 2)
    m = NativeMesh(nat)
    assert m.nblocks == 8 and m._tables is None
    loc, t, cnt, lv, fine, coarse = nat.tables()
    t1, c1, l1, loc1 = m.neighbor_table()
    np.testing.assert_array_equal(t1, t)
    np.testing.assert_array_equal(c1, cnt)
    np.testing.assert_array_equal(l1, lv)
    np.testing.assert_array_equal(loc1, loc)
    for a, b in zip(m.coordinate_arrays(), fine):
        np.testing.assert_array_equal(a, b)
    stale = NativeMesh(nat)
    nat.add_block(Loc(2, 0, 0, 0))   # refine the first root block: the tree changes
    assert NativeMesh(nat).nblocks == 15
    with pytest.raises(RuntimeError):
        stale.neighbor_table()
    # the block list itself stays the one it was made with
    assert stale.nblocks == 8 and len(stale.locs) == 8
