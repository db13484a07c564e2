"""The CUDA path's relativistic HLLD (FP64 and FP32) on the reference regression suite's
SR MHD shock tubes (sr/mhd_shocks_hlld.py, Mignone, Ugliano & Bodo 2009 problems 1, 2,
4): every conserved variable within the suite's L1 tolerances of the reference's
10000-zone HLLD solutions (tests/golden/sr_mhd_shocks_ref.npz)."""
import pytest

from athena_gb300 import build
from athena_gb300.runtime import StageUpdate
from sr_shocks import BC, CFL, ZERO_TOL, errors, setup, within

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("problem", [1, 2, 4])
def test_gpu_sr_hlld_shock_tube(problem, precision):
    mesh, gamma, tlim, ic, w0 = setup(problem)
    g = StageUpdate(mesh, gamma, xorder=2, rsolver="hlld", precision=precision, cfl=CFL,
                    tlim=tlim, relativistic=True, bc=BC)
    g.set_state(*ic)
    g.set_prim(w0)
    g.initialize()
    g.run_until(tlim, 10000)
    assert abs(g.time - tlim) < 1e-12 * tlim
    u = g.state()[0]
    _, bcc = g.prim()
    st = g.stats()
    g.close()
    errs = errors(problem, mesh, u, bcc)
    print(problem, precision, errs)
    # FP32: the zero-tolerance components carry FP32 roundoff of the transverse sweeps
    assert within(problem, errs, ZERO_TOL if precision == "fp64" else 1e-5), errs
    assert st["sr_unconverged"] == 0, st
