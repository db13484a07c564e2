"""athgpu_con2prim_timestep_noalloc, the entry point for callers that cannot let the
library allocate device memory (pool-owning hosts, real-time loops, plugins that leave
the device heap alone), against the library's own context path.

athgpu_initialize computes the same primitives, cell-centred field and first time step
on the context's arrays; the no-allocation call, given the context's device arrays and
caller-owned outputs, must reproduce them bit for bit, on two calls in a row (the second
call reuses the library's fixed scratch array as the first left it).  The file is named
to be collected last.
"""
import ctypes

import numpy as np
import pytest

from athena_gb300 import build, pgen
from athena_gb300 import runtime as rt
from athena_gb300.mesh import MeshSpec

pytestmark = pytest.mark.gpu


def _bind(L):
    f = L.athgpu_con2prim_timestep_noalloc
    f.argtypes = [ctypes.c_int] * 5 + [ctypes.c_double] * 4 + [ctypes.c_void_p] * 11
    f.restype = ctypes.c_int
    return f


def test_noalloc_matches_initialize_on_two_calls():
    import torch
    build.build()
    L = rt.load_library()
    noalloc = _bind(L)
    nx, nb, ng = (32, 32, 32), (2, 2, 2), 3
    mesh = MeshSpec(nx, nb, ng)
    gu, f1, f2, f3 = pgen.turbulence(nx, seed=5, mach=1.5)
    ic = (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3)
    gamma, cfl = 5.0 / 3.0, 0.3
    ctx = rt.StageUpdate(mesh, gamma, xorder=3, rsolver="hlld", precision="fp64", cfl=cfl)
    ctx.set_state(*ic)
    ctx.initialize()
    w_ref, bcc_ref = ctx.prim()
    dt_ref = ctx.dt
    ds = ctx.device_state()

    dev = torch.device("cuda", 0)
    coords = mesh.coordinate_arrays()
    dx = [torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in coords[1::2]]
    ncell = mesh.nblocks * mesh.nc[0] * mesh.nc[1] * mesh.nc[2]
    w = torch.empty(5 * ncell, dtype=torch.float64, device=dev)
    bcc = torch.empty(3 * ncell, dtype=torch.float64, device=dev)
    dt = torch.empty(1, dtype=torch.float64, device=dev)
    fl = rt.default_floor()
    for call in range(2):
        w.fill_(float("nan"))
        bcc.fill_(float("nan"))
        dt.fill_(-1.0)
        torch.cuda.synchronize()
        st = noalloc(mesh.nblocks, mesh.bx[0], mesh.bx[1], mesh.bx[2], ng, gamma, fl, fl,
                     cfl, dx[0].data_ptr(), dx[1].data_ptr(), dx[2].data_ptr(), ds.b1,
                     ds.b2, ds.b3, ds.u, w.data_ptr(), bcc.data_ptr(), dt.data_ptr(), None)
        assert st == 0, L.athgpu_last_error()
        torch.cuda.synchronize()
        got_w = w.cpu().numpy().reshape(w_ref.shape)
        got_bcc = bcc.cpu().numpy().reshape(bcc_ref.shape)
        assert np.array_equal(got_w, w_ref), call
        assert np.array_equal(got_bcc, bcc_ref), call
        assert float(dt.item()) == dt_ref, call
    ctx.close()


def test_noalloc_floors_match_initialize():
    """Cells below the density and pressure floors: the call rewrites u there exactly as
    the context path's W(U) does (adiabatic_mhd.cpp:65-84)."""
    import torch
    build.build()
    L = rt.load_library()
    noalloc = _bind(L)
    nx, nb, ng = (32, 32, 32), (2, 2, 2), 2
    mesh = MeshSpec(nx, nb, ng)
    gu, f1, f2, f3 = pgen.turbulence(nx, seed=9, mach=1.0)
    gamma, cfl, floor = 5.0 / 3.0, 0.3, 1.0e-4
    # planted near-vacuum cells at block centres (inside no neighbour's ghost zone):
    # density and pressure 1e-6, below the floors of 1e-4
    rng = np.random.default_rng(3)
    cells = [(int(rng.integers(0, 2)) * 16 + 8 + int(rng.integers(-3, 4)),
              int(rng.integers(0, 2)) * 16 + 8 + int(rng.integers(-3, 4)),
              int(rng.integers(0, 2)) * 16 + 8 + int(rng.integers(-3, 4))) for _ in range(40)]
    bc = pgen.cell_centered(f1, f2, f3)
    for (k, j, i) in cells:
        gu[0, k, j, i] = 1.0e-6
        gu[1:4, k, j, i] = 1.0e-9
        ke = 0.5 * float((gu[1:4, k, j, i] ** 2).sum()) / gu[0, k, j, i]
        me = 0.5 * float((bc[:, k, j, i] ** 2).sum())
        gu[4, k, j, i] = 1.0e-6 / (gamma - 1.0) + ke + me
    ic = (mesh.scatter_cells(gu),) + mesh.scatter_faces(f1, f2, f3)
    # the context path with the floors: the expected u, w, bcc and dt
    ctx = rt.StageUpdate(mesh, gamma, xorder=2, rsolver="hlld", precision="fp64", cfl=cfl,
                         dfloor=floor, pfloor=floor)
    ctx.set_state(*ic)
    ctx.initialize()
    w_ref, bcc_ref = ctx.prim()
    u_ref = ctx.state()[0]
    dt_ref = ctx.dt
    ncount = ctx.floor_count()
    assert ncount >= len(set(cells)), ncount
    # the input of the no-allocation call: the same state with its ghost cells filled and
    # nothing floored (a context whose floors lie below the planted values)
    pre = rt.StageUpdate(mesh, gamma, xorder=2, rsolver="hlld", precision="fp64", cfl=cfl)
    pre.set_state(*ic)
    pre.initialize()
    u_in, b1, b2, b3 = pre.state()
    pre.close()
    dev = torch.device("cuda", 0)
    coords = mesh.coordinate_arrays()
    dx = [torch.from_numpy(np.ascontiguousarray(c)).to(dev) for c in coords[1::2]]
    fb = [torch.from_numpy(a).to(dev) for a in (b1, b2, b3)]
    ncell = mesh.nblocks * mesh.nc[0] * mesh.nc[1] * mesh.nc[2]
    w = torch.empty(5 * ncell, dtype=torch.float64, device=dev)
    bcc = torch.empty(3 * ncell, dtype=torch.float64, device=dev)
    dt = torch.empty(1, dtype=torch.float64, device=dev)
    for call in range(2):
        u = torch.from_numpy(u_in).to(dev)
        w.fill_(float("nan"))
        bcc.fill_(float("nan"))
        dt.fill_(-1.0)
        torch.cuda.synchronize()
        st = noalloc(mesh.nblocks, mesh.bx[0], mesh.bx[1], mesh.bx[2], ng, gamma, floor,
                     floor, cfl, dx[0].data_ptr(), dx[1].data_ptr(), dx[2].data_ptr(),
                     fb[0].data_ptr(), fb[1].data_ptr(), fb[2].data_ptr(), u.data_ptr(),
                     w.data_ptr(), bcc.data_ptr(), dt.data_ptr(), None)
        assert st == 0, L.athgpu_last_error()
        torch.cuda.synchronize()
        got_u = u.cpu().numpy().reshape(u_ref.shape)
        assert np.array_equal(mesh.interior(got_u), mesh.interior(u_ref)), call
        assert not np.array_equal(mesh.interior(got_u), mesh.interior(u_in)), call
        assert np.array_equal(w.cpu().numpy().reshape(w_ref.shape), w_ref), call
        assert np.array_equal(bcc.cpu().numpy().reshape(bcc_ref.shape), bcc_ref), call
        assert float(dt.item()) == dt_ref, call
    ctx.close()


def test_noalloc_rejects_2d_meshes():
    build.build()
    L = rt.load_library()
    noalloc = _bind(L)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the shape check comes first
    for nx2, nx3 in ((1, 32), (32, 1), (1, 1)):
        st = noalloc(4, 32, nx2, nx3, 2, 5.0 / 3.0, 1e-10, 1e-10, 0.3, *([dummy] * 10), None)
        assert st == -3, (nx2, nx3)
        assert b"3-D" in L.athgpu_last_error()


def test_noalloc_rejects_meshes_beyond_its_scratch():
    build.build()
    L = rt.load_library()
    noalloc = _bind(L)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    # 8192 blocks of 32^3 (+ ghosts) exceed the 16,777,216-cell limit
    st = noalloc(8192, 32, 32, 32, 3, 5.0 / 3.0, 1e-10, 1e-10, 0.3, *([dummy] * 10), None)
    assert st == -1
    assert b"no-allocation limit" in L.athgpu_last_error()
    # block sizes whose cell count overflows 32-bit arithmetic are rejected, not wrapped
    st = noalloc(1, 2 ** 30, 2 ** 20, 2 ** 20, 3, 5.0 / 3.0, 1e-10, 1e-10, 0.3,
                 *([dummy] * 10), None)
    assert st == -1
    st = noalloc(2 ** 30, 64, 64, 64, 3, 5.0 / 3.0, 1e-10, 1e-10, 0.3, *([dummy] * 10), None)
    assert st == -1
