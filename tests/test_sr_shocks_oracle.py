"""The oracle's relativistic HLLD on the reference regression suite's SR MHD shock tubes
(sr/mhd_shocks_hlld.py): every conserved variable within the suite's L1 tolerances of the
reference's 10000-zone solutions (tests/golden/sr_mhd_shocks_ref.npz).  Problem 1 here
(400 zones, 16 s on one core); problems 2 and 4 (800 zones, about a minute each on the
oracle) run on the GPU path in test_gpu_sr_shocks.py."""
import pytest

import oracle as O
from sr_shocks import BC, CFL, errors, setup, within


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


@pytest.mark.parametrize("problem", [1])
def test_oracle_sr_hlld_shock_tube(problem):
    mesh, gamma, tlim, ic, w0 = setup(problem)
    om = O.OracleMesh(mesh, gamma, xorder=2, rsolver="hlld", cfl=CFL, tlim=tlim,
                      relativistic=True, bc=BC)
    om.set_state(*ic)
    om.set_prim(w0)
    om.initialize()
    n = 0
    while om.time < tlim and n < 10000:
        om.cycle(1)
        n += 1
    assert abs(om.time - tlim) < 1e-12 * tlim
    u = om.state()[0]
    _, bcc = om.prim()
    errs = errors(problem, mesh, u, bcc)
    assert within(problem, errs), errs
