"""Adaptive mesh refinement on the GPU (athgpu_refinement_eps, athgpu_regrid,
athgpu_new_time_step, athgpu_amr_step driven by athena_gb300.adaptive).

* FP64 against the reference's own adaptive blast runs (tests/golden): every cycle's
  block list and dt, the final state digest — bit for bit, through the initial refinement
  loop, refinements, derefinements and face-field corrections;
* FP64 against the oracle on the same run, every array including the ghost zones of the
  primitives;
* conservation and div B across regrids in FP64 and FP32.
"""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _adaptive(c, mesh0, ic, precision="fp64", native=True):
    from athena_gb300.adaptive import AdaptiveStageUpdate
    return AdaptiveStageUpdate(mesh0, ic, c["numlevel"], c["problem"]["thr"],
                               c["derefine_count"], native=native, gamma=c["gamma"],
                               xorder=c["xorder"],
                               rsolver=c["rsolver"], precision=precision, cfl=c["cfl"],
                               tlim=c["tlim"], dfloor=c["floor"], pfloor=c["floor"])


def _locs(mesh):
    return [(l.level, l.lx1, l.lx2, l.lx3) for l in mesh.locs]


def _digest(mesh, u, b1, b2, b3):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(mesh.interior(u)).tobytes())
    for b in (b1, b2, b3):
        h.update(np.ascontiguousarray(mesh.interior_faces(b)).tobytes())
    return h.hexdigest()


def _names():
    from golden_cases import amr_case_names
    return amr_case_names()


@pytest.mark.parametrize("native", [True, False])
@pytest.mark.parametrize("name", _names())
def test_gpu_amr_fp64_matches_reference_bitwise(name, native):
    """native: the host side in the library (athgpu_amr_step); else in Python."""
    from golden_cases import load_amr_case
    c, mesh0, ic, ref = load_amr_case(name)
    run = _adaptive(c, mesh0, ic, native=native)
    run.initialize()
    dts, last = [], {}

    def after(r):
        n = len(dts) - 1
        assert _locs(r.mesh) == ref["locs"][n], "block list differs at cycle %d" % (n + 1)
        last["state"], last["mesh"], last["time"] = r.state(), r.mesh, r.time

    for _ in range(c["ncycle"]):
        dts.append(run.dt)
        run.cycle(1, after_stages=after)
    np.testing.assert_array_equal(np.array(dts), ref["dt"])
    u, b1, b2, b3 = last["state"]
    m = last["mesh"]
    assert last["time"] == ref["time"]
    np.testing.assert_array_equal(m.interior(u).sum(axis=(2, 3, 4)), ref["usum"])
    assert _digest(m, u, b1, b2, b3) == ref["digest"]
    assert run.regrids > 0
    run.close()


def test_gpu_amr_fp64_matches_oracle_with_ghosts():
    import amr_run
    from golden_cases import load_amr_case
    c, mesh0, ic, ref = load_amr_case("amrblast_hlle_plm")
    run = _adaptive(c, mesh0, ic)
    run.initialize()
    kw = dict(gamma=c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"], cfl=c["cfl"],
              tlim=c["tlim"], dfloor=c["floor"], pfloor=c["floor"])
    _, mesh0, _, _ = load_amr_case("amrblast_hlle_plm")   # a fresh tree for the oracle
    amr, om = amr_run.initialize(mesh0, ic, c["numlevel"], c["problem"]["thr"],
                                 c["derefine_count"], **kw)
    assert _locs(amr.mesh) == _locs(run.mesh)
    for cyc in range(4):
        run.cycle(1)
        om = amr_run.cycle(amr, om, c["problem"]["thr"])
        assert _locs(amr.mesh) == _locs(run.mesh)
        assert run.dt == om.dt and run.time == om.time
        wg, bg = run.prim()
        wo, bo = om.prim()
        np.testing.assert_array_equal(wg, wo)
        np.testing.assert_array_equal(bg, bo)
        sg, so = run.state(), om.state()
        m = run.mesh
        np.testing.assert_array_equal(m.interior(sg[0]), m.interior(so[0]))
        for a, b in zip(sg[1:], so[1:]):
            np.testing.assert_array_equal(a, b)
    run.close()


def _mass_and_divb(mesh, u, b1, b2, b3):
    """Volume-weighted total mass over the leaf blocks and max |div B| dx / |B|."""
    ng, (n1, n2, n3) = mesh.ng, mesh.bx
    total, divb = 0.0, 0.0
    coords = mesh.coordinate_arrays()
    for b in range(mesh.nblocks):
        dx = [coords[2 * d + 1][b][ng] for d in range(3)]
        vol = dx[0] * dx[1] * dx[2]
        total += mesh.interior(u[b:b + 1])[0, 0].sum() * vol
        f1 = b1[b][ng:ng + n3, ng:ng + n2, ng:ng + n1 + 1]
        f2 = b2[b][ng:ng + n3, ng:ng + n2 + 1, ng:ng + n1]
        f3 = b3[b][ng:ng + n3 + 1, ng:ng + n2, ng:ng + n1]
        d = ((f1[:, :, 1:] - f1[:, :, :-1]) / dx[0] + (f2[:, 1:] - f2[:, :-1]) / dx[1] +
             (f3[1:] - f3[:-1]) / dx[2]) * dx[0]
        divb = max(divb, float(np.abs(d).max()))
    return total, divb


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("fp32", 2e-6)])
def test_gpu_amr_conserves_mass_and_div_b(precision, tol):
    from golden_cases import load_amr_case
    c, mesh0, ic, ref = load_amr_case("amrblast_hlld_ppm")
    run = _adaptive(c, mesh0, ic, precision)
    run.initialize()
    m0, d0 = _mass_and_divb(run.mesh, *run.state())
    nb = [run.mesh.nblocks]
    for _ in range(12):
        run.cycle(1)
        nb.append(run.mesh.nblocks)
    m1, d1 = _mass_and_divb(run.mesh, *run.state())
    assert run.regrids > 1
    assert abs(m1 - m0) <= tol * abs(m0)
    assert d1 < 1e-10
    run.close()
