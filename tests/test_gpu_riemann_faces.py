"""Every Riemann solver of the CUDA path, face by face, against the oracle's restatement:
bit for bit in FP64 (the solvers use only IEEE-exact operations: +, -, *, /, sqrt), over
face families that reach every region of the relativistic HLLD fan and the degenerate
cases (equal states, zero normal field, no field, near-vacuum, static field-only)."""
import ctypes

import numpy as np
import pytest

import oracle as O
from athena_gb300 import build
from athena_gb300.runtime import _RSOLVERS, _check, load_library
from riemann_faces import FAMILIES, face_velocity_differences, faces

pytestmark = pytest.mark.gpu

SOLVERS = [("hlld", False), ("hlle", False), ("llf", False), ("roe", False),
           ("lhlld", False), ("hlld", True), ("hlle", True), ("llf", True)]


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    O.build()


def _gpu_faces(rsolver, sr, gamma, wl, wr, bx, dv):
    import torch
    L = load_library()
    f = L.athgpu_selftest_riemann
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_longlong] + \
        [ctypes.c_void_p] * 6
    f.restype = ctypes.c_int
    dev = torch.device("cuda", 0)
    tl = torch.from_numpy(np.ascontiguousarray(wl)).to(dev)
    tr = torch.from_numpy(np.ascontiguousarray(wr)).to(dev)
    tb = torch.from_numpy(np.ascontiguousarray(bx)).to(dev)
    td = torch.from_numpy(np.ascontiguousarray(dv)).to(dev)
    out = torch.full((wl.shape[0], 7), float("nan"), dtype=torch.float64, device=dev)
    _check(f(_RSOLVERS[rsolver], 1 if sr else 0, gamma, wl.shape[0], tl.data_ptr(),
             tr.data_ptr(), tb.data_ptr(), td.data_ptr(), out.data_ptr(),
             torch.cuda.current_stream().cuda_stream), "athgpu_selftest_riemann")
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("rsolver,sr", SOLVERS)
def test_riemann_faces_match_oracle_bitwise(rsolver, sr):
    gamma = 4.0 / 3.0 if sr else 5.0 / 3.0
    for fam in FAMILIES:
        wl, wr, bx = faces(fam, 1500, seed=11)
        dv = face_velocity_differences(wl, wr, seed=11)
        got = _gpu_faces(rsolver, sr, gamma, wl, wr, bx, dv)
        want = O.riemann_faces(rsolver, wl, wr, bx, gamma, sr, dv)
        same = (got == want) | (np.isnan(got) & np.isnan(want))
        assert same.all(), (fam, int((~same).sum()), np.argwhere(~same)[:3].tolist())
