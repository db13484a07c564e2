"""Device diagnostics through the C ABI: the |div B| diagnostic (athgpu_divb, the
reference's WAbsDivergenceB) against the oracle's restatement, and the run statistics
(athgpu_stats) of the relativistic con2prim."""
import numpy as np
import pytest

import history
from athena_gb300 import build, pgen
from athena_gb300.mesh import MeshSpec
from athena_gb300.runtime import StageUpdate
from golden_cases import load_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _check_divb(g, mesh):
    s, m, c = g.divb()
    _, b1, b2, b3 = g.state()
    _, rs, rm, rc = history.wabs_divergence_b(mesh, b1, b2, b3)
    assert c == rc
    assert m == rm                      # every cell's value is the same bits
    assert abs(s - rs) <= 1e-12 * abs(rs) + 1e-300
    return s, m, c


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_divb_matches_oracle_on_a_perturbed_field(precision):
    """A face field with random perturbations (div B of order 1e-3 / dx): the device
    diagnostic equals the restatement, cell values bit for bit."""
    nx, nb = (32, 32, 32), (2, 2, 2)
    mesh = MeshSpec(nx, nb, 3)
    gu, f1, f2, f3 = pgen.turbulence(nx, seed=21, mach=1.0)
    rng = np.random.default_rng(4)
    f1 = f1 + 1e-3 * rng.standard_normal(f1.shape)
    f2 = f2 + 1e-3 * rng.standard_normal(f2.shape)
    f3 = f3 + 1e-3 * rng.standard_normal(f3.shape)
    ic = (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3)
    g = StageUpdate(mesh, 5.0 / 3.0, xorder=3, rsolver="hlld", precision=precision, cfl=0.3)
    g.set_state(*ic)
    g.initialize()
    s, m, c = _check_divb(g, mesh)
    assert m > 1e-3 and c == 32 ** 3
    g.cycle(2)  # CT keeps the cell divergences: the diagnostic still matches
    _check_divb(g, mesh)
    g.close()


@pytest.mark.parametrize("name", ["turb_hlld_ppm_8blk", "blast_hlld_plm_8blk",
                                  "turbrk2_hlld_plm_8blk", "blastbc_hlle_ppm_1blk"])
def test_divb_on_reference_final_states(name):
    """The reference's own final states of golden cases: solenoidal to roundoff, and the
    device diagnostic equals the restatement on them."""
    c, mesh, ic, ref = load_case(name)
    ng = mesh.ng
    state = [np.array(a) for a in ic]
    state[0][:, :, ng:-ng, ng:-ng, ng:-ng] = ref["u"]
    for d, key in enumerate(("b1", "b2", "b3")):
        state[1 + d][:, ng:-ng, ng:-ng, ng:-ng] = ref[key]
    g = StageUpdate(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"], cfl=c["cfl"],
                    bc=c.get("bc"), integrator=c.get("integrator", "vl2"))
    g.set_state(*state)
    g.initialize()
    s, m, cnt = _check_divb(g, mesh)
    assert m < 1e-11
    g.close()


def test_stats_count_the_relativistic_con2prim():
    """Every interior cell is solved once per stage; passes per cell within the
    reference's budget; none unconverged on a smooth shear layer; reset zeroes."""
    nx, nb = (32, 32, 32), (2, 2, 2)
    mesh = MeshSpec(nx, nb, 2)
    gw, f1, f2, f3 = pgen.sr_kelvin_helmholtz(nx, seed=4, noise=0.02)
    gu = pgen.sr_prim_to_cons(gw, pgen.cell_centered(f1, f2, f3), 4.0 / 3.0)
    ic = (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3)
    for precision in ("fp64", "fp32"):
        g = StageUpdate(mesh, 4.0 / 3.0, xorder=2, rsolver="hlle", precision=precision,
                        cfl=0.3, relativistic=True)
        g.set_state(*ic)
        g.set_prim(mesh.scatter_cells(gw))
        g.initialize()
        g.stats(reset=True)
        g.cycle(3)
        st = g.stats(reset=True)
        assert st["sr_cells"] == 3 * 2 * 32 ** 3, st
        assert 1.0 <= st["sr_passes"] / st["sr_cells"] <= 15.0, st
        assert st["sr_unconverged"] == 0 and st["net_error"] == 0, st
        assert st["divb_max"] < 1e-11, st
        st2 = g.stats()
        assert st2["sr_cells"] == 0 and st2["sr_passes"] == 0
        g.close()
