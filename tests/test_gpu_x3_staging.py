"""The x3 sweep's two shared-memory stagings (per-thread cp.async; TMA bulk copies with an
mbarrier) give the same bits: states after several cycles, FP64 and FP32 (with the
compensated update), VL2 and RK2, PLM and PPM, whole columns and segments; and the bulk
staging keeps the FP64 path bit-exact with the reference's golden runs."""
import numpy as np
import pytest

from athena_gb300 import build, pgen
from athena_gb300.mesh import MeshSpec
from athena_gb300.runtime import StageUpdate
from golden_cases import interior_faces, load_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _run(mesh, ic, bulk, precision, xorder, rsolver, integrator, seg=0, ncycle=3):
    g = StageUpdate(mesh, 5.0 / 3.0, xorder=xorder, rsolver=rsolver, precision=precision,
                    cfl=0.6 if integrator == "rk2" else 0.3, integrator=integrator)
    g.set_x3_staging(bulk)
    if seg:
        g.set_sweep_segment(0, seg)
    g.set_state(*ic)
    g.initialize()
    g.cycle(ncycle)
    out = g.state()
    w, bcc = g.prim()
    assert g.x3_staging() == bulk
    st = g.stats()
    assert st["sweep_timeout"] == 0
    g.close()
    return list(out) + [w, bcc]


@pytest.mark.parametrize("precision,xorder,rsolver,integrator,seg", [
    ("fp64", 3, "hlld", "vl2", 0), ("fp32", 3, "hlld", "vl2", 0),
    ("fp32", 2, "hlle", "rk2", 8), ("fp64", 2, "roe", "rk2", 5),
    ("fp32", "3f", "llf", "vl2", 16)])
def test_bulk_staging_matches_cp_async(precision, xorder, rsolver, integrator, seg):
    ng = 3 if xorder in (3, "3f") else 2
    nx = (32, 32, 32)
    mesh = MeshSpec(nx, (2, 2, 2), ng)
    gu, f1, f2, f3 = pgen.turbulence(nx, seed=8, mach=1.5)
    ic = (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3)
    a = _run(mesh, ic, 0, precision, xorder, rsolver, integrator, seg)
    b = _run(mesh, ic, 1, precision, xorder, rsolver, integrator, seg)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("name", ["turb_hlld_ppm_8blk", "blast_hlld_plm_8blk",
                                  "turbrk2_hlld_plm_8blk"])
def test_bulk_staging_reproduces_reference(name):
    c, mesh, ic, ref = load_case(name)
    g = StageUpdate(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"], cfl=c["cfl"],
                    tlim=c["tlim"], bc=c.get("bc"), integrator=c.get("integrator", "vl2"))
    g.set_x3_staging(1)
    g.set_state(*ic)
    g.initialize()
    dts = []
    for _ in range(c["ncycle"]):
        dts.append(g.dt)
        g.cycle(1)
    u, b1, b2, b3 = g.state()
    assert g.x3_staging() == 1
    g.close()
    assert np.array_equal(np.array(dts), ref["dt"])
    assert np.array_equal(mesh.interior(u), ref["u"])
    for got, want in zip((b1, b2, b3), (ref["b1"], ref["b2"], ref["b3"])):
        assert np.array_equal(interior_faces(mesh, got), want)
