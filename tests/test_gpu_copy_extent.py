"""ATHGPU_COPY_INTERIOR state copies: only each MeshBlock's x2/x3 range of own cells and
faces moves (with whole x1 rows).  A run whose host arrays carry garbage in their x2/x3
ghost zones gives, bit for bit, the copied elements of a whole-array run, and the
download leaves the host's x2/x3 ghost zones untouched."""
import numpy as np
import pytest

from athena_gb300 import build
from athena_gb300.runtime import COPY_INTERIOR, COPY_WHOLE, StageUpdate
from golden_cases import load_case

pytestmark = pytest.mark.gpu

SENTINEL = 7.25


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _copied(mesh, what):
    """Index of the copied part of U (what 0) or face array b1..b3 (what 1..3): the own
    x3 and x2 ranges (both bounding faces of a face array's own direction), all x1."""
    ng, (n1, n2, n3) = mesh.ng, mesh.bx
    k = slice(ng, ng + n3 + (1 if what == 3 else 0))
    j = slice(ng, ng + n2 + (1 if what == 2 else 0))
    return (slice(None), slice(None), k, j) if what == 0 else (slice(None), k, j)


def _run(c, mesh, ic, precision, extent, ncycle=3, relativistic=False):
    g = StageUpdate(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"],
                    precision=precision, cfl=c["cfl"], tlim=c["tlim"], bc=c.get("bc"),
                    relativistic=relativistic)
    g.set_copy_extent(extent)
    host = [a.copy() for a in ic]
    if extent == COPY_INTERIOR:  # what the copies must not read
        for w, a in enumerate(host):
            keep = a[_copied(mesh, w)].copy()
            a[...] = np.nan
            a[_copied(mesh, w)] = keep
    g.set_state(*host)
    if relativistic:  # the initial primitives, also the con2prim seed
        g.set_prim(c["ic_w"])
    g.initialize()
    g.cycle(ncycle)
    out = [np.full(a.shape, SENTINEL) for a in ic]
    g.state(out=out)
    g.close()
    return out


@pytest.mark.parametrize("name,relativistic", [("turb_hlld_ppm_8blk", False),
                                               ("blastbc_hlld_plm_8blk", False),
                                               ("blastbc_hlle_ppm_1blk", False),
                                               ("srkh_hlle_plm_8blk", True)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_interior_copies_match_whole_copies(name, relativistic, precision):
    c, mesh, ic, _ = load_case(name)
    whole = _run(c, mesh, ic, precision, COPY_WHOLE, relativistic=relativistic)
    part = _run(c, mesh, ic, precision, COPY_INTERIOR, relativistic=relativistic)
    for w, (a, b) in enumerate(zip(whole, part)):
        sel = _copied(mesh, w)
        assert np.array_equal(a[sel], b[sel]), (name, precision, w)
        rest = np.ones(b.shape, bool)
        rest[sel] = False
        assert (b[rest] == SENTINEL).all(), (name, precision, w)


def test_copy_extent_rejects_unknown_values():
    c, mesh, ic, _ = load_case("turb_hlld_ppm_8blk")
    g = StageUpdate(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"],
                    precision="fp64", cfl=c["cfl"], tlim=c["tlim"])
    with pytest.raises(Exception):
        g.set_copy_extent(2)
    g.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_interior_copies_on_a_multilevel_mesh(precision):
    """The same on a statically refined mesh, whose initialize rebuilds the ghost zones
    through the multi-level exchange and prolongation."""
    from golden_cases import load_ml_case, ml_case_names
    c, mesh, ic, _ = load_ml_case(ml_case_names()[0])

    def run(extent):
        g = StageUpdate(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"],
                        precision=precision, cfl=c["cfl"], tlim=c["tlim"],
                        integrator=c.get("integrator", "vl2"))
        g.set_copy_extent(extent)
        host = [a.copy() for a in ic]
        if extent == COPY_INTERIOR:
            for w, a in enumerate(host):
                keep = a[_copied(mesh, w)].copy()
                a[...] = np.nan
                a[_copied(mesh, w)] = keep
        g.set_state(*host)
        g.initialize()
        g.cycle(3)
        out = [np.full(a.shape, SENTINEL) for a in ic]
        g.state(out=out)
        g.close()
        return out

    whole, part = run(COPY_WHOLE), run(COPY_INTERIOR)
    for w, (a, b) in enumerate(zip(whole, part)):
        sel = _copied(mesh, w)
        assert np.array_equal(a[sel], b[sel]), (precision, w)
        rest = np.ones(b.shape, bool)
        rest[sel] = False
        assert (b[rest] == SENTINEL).all(), (precision, w)
