"""The oracle's Riemann solvers face by face: consistency F(U, U) = F(U) for every solver
and finite fluxes over every face family (the relativistic HLLD restatement in particular,
whose secant iteration and HLL fallbacks the end-to-end runs reach only in part)."""
import numpy as np
import pytest

import oracle as O
from riemann_faces import FAMILIES, faces

SOLVERS = [("hlld", False), ("hlle", False), ("llf", False), ("roe", False),
           ("lhlld", False), ("hlld", True), ("hlle", True), ("llf", True)]


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


@pytest.mark.parametrize("rsolver,sr", SOLVERS)
def test_equal_states_give_the_physical_flux(rsolver, sr):
    """With equal L and R states every solver returns the physical flux, which LLF gives
    exactly; the relativistic HLLD reaches it through its secant iteration (1e-9)."""
    wl, _, bx = faces("equal", 1500, seed=1)
    gamma = 4.0 / 3.0 if sr else 5.0 / 3.0
    got = O.riemann_faces(rsolver, wl, wl, bx, gamma, sr)
    exact = O.riemann_faces("llf", wl, wl, bx, gamma, sr)
    tol = 1e-9 if (sr and rsolver == "hlld") else 1e-14
    scale = np.abs(exact).max(axis=0)
    assert np.all(np.abs(got - exact) <= tol * scale), np.abs(got - exact).max(axis=0)


@pytest.mark.parametrize("family", FAMILIES)
def test_sr_hlld_fluxes_are_finite(family):
    wl, wr, bx = faces(family, 800, seed=2)
    f = O.riemann_faces("hlld", wl, wr, bx, 4.0 / 3.0, True)
    assert np.all(np.isfinite(f))
