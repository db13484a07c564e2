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


def test_noalloc_rejects_meshes_beyond_its_scratch():
    build.build()
    L = rt.load_library()
    noalloc = _bind(L)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    # 8192 blocks of 32^3 (+ ghosts) exceed the 16,777,216-cell limit
    st = noalloc(8192, 32, 32, 32, 3, 5.0 / 3.0, 1e-10, 1e-10, 0.3, *([dummy] * 10), None)
    assert st == -1
    assert b"no-allocation limit" in L.athgpu_last_error()
