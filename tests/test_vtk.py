"""VTK output in the reference's format (athena_gb300/vtk.py): the files written from the
oracle's (CPU) or the CUDA path's (GPU) initial state of the linear wave on two MeshBlocks
equal the reference's own VTK outputs of that state byte for byte (tests/golden/vtk)."""
import json
import os

import pytest

from athena_gb300 import vtk
from athena_gb300.mesh import MeshSpec
from athena_gb300.pgen import LinearWave

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _case():
    c = json.load(open(os.path.join(GOLDEN, "golden.json")))["vtk"]
    mesh = MeshSpec(tuple(c["nx"]), tuple(c["nb"]), c["ng"], tuple(c["xmin"]),
                    tuple(c["xmax"]))
    return c, mesh


def _compare(tmp_path, mesh, u, w, bcc, files):
    made = vtk.write(tmp_path, mesh, u, w, bcc, 0.0, 0, "prim", file_id="out8")
    made += vtk.write(tmp_path, mesh, u, w, bcc, 0.0, 0, "cons", file_id="out7")
    assert sorted(os.path.basename(f) for f in made) == sorted(files)
    for f in made:
        want = open(os.path.join(GOLDEN, "vtk", os.path.basename(f)), "rb").read()
        assert open(f, "rb").read() == want, os.path.basename(f)


def test_vtk_of_the_oracle_state_equals_the_reference_files(tmp_path):
    import oracle as O
    c, mesh = _case()
    lw = LinearWave(mesh)
    om = O.OracleMesh(mesh, lw.gam, xorder=2, rsolver="hlld", cfl=0.3, tlim=1.0e3)
    om.set_state(*lw.generate())
    om.initialize()
    w, bcc = om.prim()
    _compare(tmp_path, mesh, om.state()[0], w, bcc, c["files"])


@pytest.mark.gpu
def test_vtk_of_the_gpu_state_equals_the_reference_files(tmp_path):
    from athena_gb300.runtime import StageUpdate
    c, mesh = _case()
    lw = LinearWave(mesh)
    g = StageUpdate(mesh, lw.gam, xorder=2, rsolver="hlld", precision="fp64", tlim=1.0e3)
    g.set_state(*lw.generate())
    g.initialize()
    w, bcc = g.prim()
    _compare(tmp_path, mesh, g.state()[0], w, bcc, c["files"])
    g.close()
