"""The per-operator entry points (athgpu_op_*, one MeshBlock per call) against the
oracle's restatements of the same member functions (Hydro::CalculateFluxes,
Field::ComputeCornerE, Hydro::AddFluxDivergence, Field::CT,
EquationOfState::ConservedToPrimitive, Hydro::NewBlockTimeStep) on the same arrays: every
output array equal bit for bit (relativistic con2prim: within 1e-12)."""
import numpy as np
import pytest

import oracle as O
from athena_gb300 import build, pgen
from athena_gb300.mesh import MeshSpec
from athena_gb300.runtime import BlockOperators

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _state(mesh, kind, gamma):
    if kind == "sr":
        gw, f1, f2, f3 = pgen.sr_kelvin_helmholtz(mesh.nx, seed=3, noise=0.05)
        gu = pgen.sr_prim_to_cons(gw, pgen.cell_centered(f1, f2, f3), gamma)
        ic = (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3)
        return ic, mesh.scatter_cells(gw)
    gu, f1, f2, f3 = pgen.turbulence(mesh.nx, seed=13, mach=2.0)
    return (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3), None


def _zeros_like_faces(mesh, nvar=None):
    shp = [(mesh.nblocks,) + s for s in mesh.face_shapes]
    if nvar:
        return [np.zeros((nvar,) + s[1:]) for s in shp]
    return [np.zeros(s[1:]) for s in shp]


def _edges(mesh):
    nc1, nc2, nc3 = mesh.nc
    return [np.zeros((nc3 + 1, nc2 + 1, nc1)), np.zeros((nc3 + 1, nc2, nc1 + 1)),
            np.zeros((nc3, nc2 + 1, nc1 + 1))]


CASES = [("hlld", 2, False, 2), ("hlld", 3, False, 3), ("hlle", 1, False, 2),
         ("roe", 2, False, 2), ("llf", 3, False, 3), ("hlld", "3f", False, 3),
         ("hlle", 2, True, 2), ("llf", 3, True, 3), ("hlld", 2, True, 2),
         ("hlld", 3, True, 3), ("lhlld", 2, False, 2), ("lhlld", 3, False, 3)]


@pytest.mark.parametrize("rsolver,order,sr,ng", CASES)
def test_operators_match_oracle(rsolver, order, sr, ng):
    gamma = 4.0 / 3.0 if sr else 5.0 / 3.0
    mesh = MeshSpec((16, 12, 8), (1, 1, 1), ng, (0., 0., 0.), (1.0, 0.75, 0.5))
    ic, w0 = _state(mesh, "sr" if sr else "mhd", gamma)
    om = O.OracleMesh(mesh, gamma, xorder=order, rsolver=rsolver, relativistic=sr, cfl=0.3)
    om.set_state(*ic)
    if sr:
        om.set_prim(w0)
    om.initialize()
    u, b1, b2, b3 = om.state()
    w, bcc = om.prim()
    u, w, bcc = u[0].copy(), w[0].copy(), bcc[0].copy()
    bf = [b1[0].copy(), b2[0].copy(), b3[0].copy()]
    dt = om.dt
    ops = BlockOperators(mesh, gamma, rsolver=rsolver, xorder=order, relativistic=sr, cfl=0.3)
    iorder = 3 if order == "3f" else order

    # Hydro::CalculateFluxes
    fo = _zeros_like_faces(mesh, 5)
    eo = [np.zeros(mesh.face_shapes[d]) for d in (0, 0, 0, 1, 1, 1, 2, 2, 2)]
    om.op_fluxes(0, iorder, dt, fo, eo)
    fg = _zeros_like_faces(mesh, 5)
    eg = [np.zeros(mesh.face_shapes[d]) for d in (0, 0, 0, 1, 1, 1, 2, 2, 2)]
    ops.calculate_fluxes(iorder, dt, w, bcc, bf, fg, eg)
    for a, b in zip(fg + eg, fo + eo):
        assert np.array_equal(a, b)
    assert np.abs(fg[0]).max() > 0

    # Field::ComputeCornerE from those face EMFs
    eco, ecg = _edges(mesh), _edges(mesh)
    om.op_corner_e(0, eo, eco)
    ops.corner_e(w, bcc, eg, ecg)
    for a, b in zip(ecg, eco):
        assert np.array_equal(a, b)

    # Hydro::AddFluxDivergence
    uo, ug = u.copy(), u.copy()
    om.op_add_flux_divergence(0, 0.5 * dt, fo, uo)
    ops.add_flux_divergence(0.5 * dt, fg, ug)
    assert np.array_equal(ug, uo) and not np.array_equal(ug, u)

    # Field::CT
    bo, bg = [a.copy() for a in bf], [a.copy() for a in bf]
    om.op_ct(0, dt, eco, bo)
    ops.ct(dt, ecg, bg)
    for a, b, c in zip(bg, bo, bf):
        assert np.array_equal(a, b)
    assert any(not np.array_equal(a, c) for a, c in zip(bg, bf))

    # Hydro::NewBlockTimeStep on the initial primitives
    assert ops.new_block_dt(w, bcc, bf) == om.op_new_block_dt(0)

    # EquationOfState::ConservedToPrimitive over the interior plus one ghost layer, on the
    # updated state (the oracle runs on its own arrays: load the updated ones first)
    ng_ = mesh.ng
    rng = (ng_ - 1, ng_ + mesh.bx[0], ng_ - 1, ng_ + mesh.bx[1], ng_ - 1, ng_ + mesh.bx[2])
    om.set_state(ug[None], bg[0][None], bg[1][None], bg[2][None])
    cg, pg, bccg = ug.copy(), w.copy(), np.zeros_like(bcc)
    ops.con2prim(cg, bg, pg, bccg, rng)
    om.op_con2prim(0, rng)
    co, _, _, _ = om.state()
    po, bcco = om.prim()
    sl = (slice(None), slice(rng[4], rng[5] + 1), slice(rng[2], rng[3] + 1),
          slice(rng[0], rng[1] + 1))
    if sr:
        scale = np.abs(po[0][sl]).max(axis=(1, 2, 3), keepdims=True)
        assert np.all(np.abs(pg[sl] - po[0][sl]) <= 1e-12 * np.abs(po[0][sl]) + 1e-12 * scale)
    else:
        assert np.array_equal(pg[sl], po[0][sl])
        assert np.array_equal(cg[sl], co[0][sl])
    assert np.array_equal(bccg[sl], bcco[0][sl])
    ops.close()
