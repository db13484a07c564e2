"""C-ABI library checks that need no GPU: it loads, exports every function the header
declares, and rejects invalid meshes with an error instead of computing anything."""
import ctypes

import numpy as np
import pytest

from athena_gb300 import build
from athena_gb300 import runtime as rt
from athena_gb300.mesh import MeshSpec


@pytest.fixture(scope="module")
def lib():
    build.build()
    return rt.load_library()


def test_exports_every_declared_function(lib):
    names = rt.header_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n


def test_version(lib):
    assert b"sm_103a" in lib.athgpu_version()


def _desc(mesh, **kw):
    coords = [np.ascontiguousarray(c) for c in mesh.coordinate_arrays()]
    d = rt.MeshDesc()
    d.nbx1, d.nbx2, d.nbx3 = mesh.nb
    d.nx1, d.nx2, d.nx3 = mesh.bx
    d.nghost, d.xorder, d.rsolver, d.precision = mesh.ng, 2, 0, 0
    d.gamma, d.dfloor, d.pfloor, d.cfl_number, d.tlim = 5 / 3, 1e-10, 1e-10, 0.3, 1.0
    d.sigma_max, d.beta_min, d.gamma_max = 0.0, 0.0, 1000.0
    d.x1f, d.dx1f, d.x2f, d.dx2f, d.x3f, d.dx3f = [rt._dp(c) for c in coords]
    for k, v in kw.items():
        setattr(d, k, v)
    return d, coords


@pytest.mark.parametrize("field,value,code", [
    ("xorder", 4, -3), ("xorder", 0, -3), ("nghost", 1, -1), ("rsolver", 7, -1),
    ("precision", 9, -1), ("gamma", 1.0, -1),
    ("cfl_number", 0.0, -1), ("nx1", 0, -1), ("ppm_fast", 1, -1), ("integrator", 2, -1),
    ("cfl_number", 0.6, -1)])
def test_invalid_meshes_are_rejected(lib, field, value, code):
    mesh = MeshSpec((16, 8, 8), (1, 1, 1), 2)
    d, keep = _desc(mesh, **{field: value})
    h = ctypes.c_void_p()
    assert lib.athgpu_create(ctypes.byref(h), ctypes.byref(d)) == code
    assert h.value is None
    assert lib.athgpu_last_error()


def test_ppm_needs_three_ghosts(lib):
    mesh = MeshSpec((16, 8, 8), (1, 1, 1), 2)
    d, keep = _desc(mesh, xorder=3)
    h = ctypes.c_void_p()
    assert lib.athgpu_create(ctypes.byref(h), ctypes.byref(d)) == -1
    assert b"nghost" in lib.athgpu_last_error()


def test_integrator_cfl_limits(lib):
    """The integrators' CFL limits in 3-D (time_integrator.cpp:219-222, 445): 0.5 for
    vl2, 1.0 for rk2."""
    mesh = MeshSpec((16, 8, 8), (1, 1, 1), 2)
    for integ, cfl in ((rt.VL2, 0.51), (rt.RK2, 1.01)):
        d, keep = _desc(mesh, integrator=integ, cfl_number=cfl)
        h = ctypes.c_void_p()
        assert lib.athgpu_create(ctypes.byref(h), ctypes.byref(d)) == -1
        assert b"limit" in lib.athgpu_last_error()


def test_null_context_calls_fail(lib):
    assert lib.athgpu_stage(None, 1) == -1
    assert lib.athgpu_cycle(None, 1) == -1
    assert lib.athgpu_initialize(None) == -1
    assert lib.athgpu_destroy(None) == 0


def test_non_uniform_spacing_is_rejected(lib):
    """The kernels implement the reference's uniform-Cartesian branches only."""
    mesh = MeshSpec((16, 8, 8), (2, 1, 1), 2)
    coords = [np.ascontiguousarray(c) for c in mesh.coordinate_arrays()]
    coords[1][1, 5] *= 1.01   # one x1 spacing of block 1
    d, _ = _desc(mesh)
    d.x1f, d.dx1f, d.x2f, d.dx2f, d.x3f, d.dx3f = [rt._dp(c) for c in coords]
    h = ctypes.c_void_p()
    assert lib.athgpu_create(ctypes.byref(h), ctypes.byref(d)) == -3
    assert b"uniform" in lib.athgpu_last_error()


def test_relativistic_options_are_checked(lib):
    mesh = MeshSpec((16, 8, 8), (1, 1, 1), 2)
    h = ctypes.c_void_p()
    d, keep = _desc(mesh, relativistic=1, rsolver=3)      # SR + Roe: no such solver
    assert lib.athgpu_create(ctypes.byref(h), ctypes.byref(d)) == -3
    d, keep = _desc(mesh, relativistic=1, rsolver=1, gamma_max=0.5)
    assert lib.athgpu_create(ctypes.byref(h), ctypes.byref(d)) == -1
    assert b"gamma_max" in lib.athgpu_last_error()
