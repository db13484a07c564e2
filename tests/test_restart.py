"""Restart files in the reference's format (athena_gb300/restart.py).

* The reference's own restart file (tests/golden/restart_lw.rst: the linear wave on one
  MeshBlock after 3 cycles) is read, written back byte for byte (padding aside), and the
  oracle restarted from it reproduces the reference's restarted run (3 more cycles) bit
  for bit; the CUDA path does the same on the GPU.
* A restart file written by this package from the oracle's state is accepted by the
  reference (`athena -r`, where the reference binary is built) and continues exactly as
  the oracle does.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from athena_gb300 import restart
from athena_gb300.mesh import MeshSpec

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RST = os.path.join(GOLDEN, "restart_lw.rst")


def _case():
    meta = json.load(open(os.path.join(GOLDEN, "golden.json")))["restart"]
    mesh = MeshSpec(tuple(meta["nx"]), tuple(meta["nb"]), meta["ng"], tuple(meta["xmin"]),
                    tuple(meta["xmax"]))
    after = np.load(os.path.join(GOLDEN, "restart_lw_after.npz"))
    return meta, mesh, after


def test_read_reference_restart_and_write_it_back(tmp_path):
    meta, mesh, _ = _case()
    r = restart.read(RST, mesh.bx, mesh.ng)
    assert r.nbtotal == 1 and r.ncycle == 3 and r.locs == [(0, 0, 0, 0)]
    assert r.mesh_size[-3:] == (8, 4, 4)
    assert r.param("time", "nlim") == "3"
    assert r.u.shape == (1, 5, 8, 8, 12)
    out = tmp_path / "back.rst"
    restart.write(out, r)
    a, b = open(RST, "rb").read(), open(out, "rb").read()
    assert len(a) == len(b)
    diff = [i for i in range(len(a)) if a[i] != b[i]]
    # only padding bytes may differ: the 4 after RegionSize and after each
    # LogicalLocation's level
    hdr = a.index(b"<par_end>\n") + len(b"<par_end>\n")
    pads = set(range(hdr + 8 + 84, hdr + 8 + 88))
    loc0 = hdr + 8 + 88 + 28
    for n in range(r.nbtotal):
        pads |= set(range(loc0 + 40 * n + 28, loc0 + 40 * n + 32))
    assert set(diff) <= pads


def test_oracle_restarted_from_reference_file_matches_reference():
    import oracle as O
    meta, mesh, after = _case()
    r = restart.read(RST, mesh.bx, mesh.ng)
    om = O.OracleMesh(mesh, meta["gamma"], xorder=meta["xorder"], rsolver=meta["rsolver"],
                      cfl=meta["cfl"], tlim=1.0e3)
    om.set_state(*restart.state(r, mesh))
    om.set_clock(r.time, r.dt)
    om.initialize()          # Mesh::Initialize(1): first dt from the stored one
    dts = []
    for _ in range(meta["cycles_after"]):
        dts.append(om.dt)
        om.cycle()
    np.testing.assert_array_equal(np.array(dts), after["dt"])
    np.testing.assert_array_equal(mesh.interior(om.state()[0]), after["u"])
    assert om.time == float(after["time"])


def _ref_exe():
    p = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle", "_ref",
                     "mhd_hlld_g2", "athena_lw")
    return p if os.path.exists(p) else None


@pytest.mark.skipif(_ref_exe() is None, reason="the reference binary is built here only")
def test_reference_restarts_from_our_file(tmp_path):
    """Our writer's file, made from the oracle after 2 cycles of a 2-block linear wave,
    restarts the reference, which then matches the oracle's own continuation."""
    import oracle as O
    import ref_run
    from athena_gb300.pgen import LinearWave
    mesh = MeshSpec((16, 8, 8), (2, 1, 1), 2, (0., 0., 0.), (3.0, 1.5, 1.5))
    lw = LinearWave(mesh)
    om = O.OracleMesh(mesh, lw.gam, xorder=2, rsolver="hlld", cfl=0.3, tlim=1.0e3)
    om.set_state(*lw.generate())
    om.initialize()
    om.cycle(2)
    text = ref_run.athinput(mesh, lw.gam, 2, 0.3, 5, 1.0e3, {
        "compute_error": "false", "wave_flag": 0, "amp": 1.0e-6, "vflow": 0.0})
    params = "#------------------------- PAR_DUMP -------------------------\n" + text + \
        "#------------------------- PAR_DUMP -------------------------\n<par_end>\n"
    r = restart.make(mesh, om.state(), om.time, om.dt, 2, params)
    restart.write(tmp_path / "ours.rst", r)
    p = subprocess.run([_ref_exe(), "-r", "ours.rst", "time/nlim=5"], cwd=tmp_path,
                       capture_output=True, text=True)
    assert p.returncode == 0, p.stdout[-2000:] + p.stderr[-2000:]
    om2 = O.OracleMesh(mesh, lw.gam, xorder=2, rsolver="hlld", cfl=0.3, tlim=1.0e3)
    om2.set_state(*restart.state(restart.read(tmp_path / "ours.rst", mesh.bx, mesh.ng), mesh))
    om2.set_clock(om.time, om.dt)
    om2.initialize()
    for c in range(3, 6):
        dump = ref_run.read_dump(os.path.join(tmp_path, "dump.%05d.bin" % c), mesh)
        assert dump["dt"] == om2.dt
        om2.cycle()
    np.testing.assert_array_equal(mesh.interior(om2.state()[0]), mesh.interior(dump["u"]))


@pytest.mark.gpu
def test_gpu_restarted_from_reference_file_matches_reference():
    from athena_gb300.runtime import StageUpdate
    meta, mesh, after = _case()
    g = StageUpdate(mesh, meta["gamma"], xorder=meta["xorder"], rsolver=meta["rsolver"],
                    precision="fp64", cfl=meta["cfl"], tlim=1.0e3)
    r = restart.load(RST, g)
    assert r.ncycle == 3
    dts = []
    for _ in range(meta["cycles_after"]):
        dts.append(g.dt)
        g.cycle(1)
    np.testing.assert_array_equal(np.array(dts), after["dt"])
    np.testing.assert_array_equal(mesh.interior(g.state()[0]), after["u"])
    g.close()


@pytest.mark.gpu
def test_gpu_restart_is_transparent_on_a_multilevel_mesh(tmp_path):
    """A static multi-level run saved and restored (into a fresh context, as a restarted
    run starts) continues bit for bit like the uninterrupted run."""
    from athena_gb300 import pgen
    from athena_gb300.meshtree import MultiLevelMesh
    from athena_gb300.runtime import StageUpdate

    def mesh():
        return MultiLevelMesh((16, 16, 16), (2, 2, 2), 2, (-.5,) * 3, (.5,) * 3,
                              regions=[((0.1, 0.1, 0.1), (0.2, 0.2, 0.2), 1)])
    m = mesh()
    kw = dict(xorder=2, rsolver="hlle", precision="fp64", cfl=0.3, tlim=1.0e3)
    a = StageUpdate(m, 5.0 / 3.0, **kw)
    a.set_state(*pgen.smooth_blocks(m, seed=3))
    a.initialize()
    a.cycle(3)
    params = restart.parameter_dump([("time", [("nlim", 3)])])
    restart.save(tmp_path / "ml.rst", a, 3, params)
    b = StageUpdate(mesh(), 5.0 / 3.0, **kw)
    t_a, dt_a = a.clock()
    a.cycle(3)
    r = restart.load(tmp_path / "ml.rst", b)
    assert (r.time, r.dt) == (t_a, dt_a)
    b.cycle(3)
    assert a.clock() == b.clock()
    np.testing.assert_array_equal(m.interior(a.state()[0]), m.interior(b.state()[0]))
    a.close()
    b.close()
