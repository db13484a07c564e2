"""Every Riemann solver of the CUDA path, face by face, against the oracle's restatement:
bit for bit in FP64 (the solvers use only IEEE-exact operations: +, -, *, /, sqrt), over
face families that reach every region of the relativistic HLLD fan and the degenerate
cases (equal states, zero normal field, no field, near-vacuum, static field-only); and the
FP32 solvers of the FP32 sweeps within per-family bounds of the same FP64 fluxes."""
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


def _gpu_faces_fp32(rsolver, sr, gamma, wl, wr, bx, dv):
    import torch
    L = load_library()
    f = L.athgpu_selftest_riemann_fp32
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_longlong] + \
        [ctypes.c_void_p] * 6
    f.restype = ctypes.c_int
    dev = torch.device("cuda", 0)
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (wl, wr, bx, dv)]
    out = torch.full((wl.shape[0], 7), float("nan"), dtype=torch.float32, device=dev)
    _check(f(_RSOLVERS[rsolver], 1 if sr else 0, gamma, wl.shape[0],
             *[x.data_ptr() for x in t], out.data_ptr(),
             torch.cuda.current_stream().cuda_stream), "athgpu_selftest_riemann_fp32")
    torch.cuda.synchronize()
    return out.cpu().numpy().astype(np.float64)


# FP32 solvers (HLLD: the packed left/right form the FP32 sweeps run) against the oracle's
# FP64 fluxes of the same FP32-rounded states.  Error of a face: the largest component
# difference over the face's largest flux component.  Bounds (99th percentile, maximum)
# per family; "ultra" (extreme ratios) is less well conditioned.  Left out: the
# near-vacuum family for the HLLD, LHLLD and Roe fluxes, whose components cancel to below
# FP32 resolution (the scalar FP32 HLLD is off by O(1) there as well), and for SR HLLD the
# strongly magnetised, shocked and extreme families, where the FP32 contact iteration and
# its HLLE fallback decide differently from FP64.
FP32_BOUNDS = {"ultra": (1e-2, 5e-2)}
FP32_SKIP = {("hlld", False): {"near_vacuum"}, ("lhlld", False): {"near_vacuum"},
             ("roe", False): {"near_vacuum"},
             ("hlld", True): {"near_vacuum", "shock", "magnetised", "ultra"}}


@pytest.mark.parametrize("rsolver,sr", SOLVERS)
def test_fp32_riemann_faces_track_oracle(rsolver, sr):
    gamma = 4.0 / 3.0 if sr else 5.0 / 3.0
    for fam in FAMILIES:
        if fam in FP32_SKIP.get((rsolver, sr), ()):
            continue
        wl, wr, bx = faces(fam, 1500, seed=11)
        dv = face_velocity_differences(wl, wr, seed=11)
        wl, wr, bx, dv = (a.astype(np.float32) for a in (wl, wr, bx, dv))
        got = _gpu_faces_fp32(rsolver, sr, gamma, wl, wr, bx, dv)
        want = O.riemann_faces(rsolver, wl.astype(np.float64), wr.astype(np.float64),
                               bx.astype(np.float64), gamma, sr, dv.astype(np.float64))
        assert np.isfinite(got).all(), fam
        err = np.abs(got - want).max(axis=1) / (np.abs(want).max(axis=1) + 1e-300)
        p99, mx = FP32_BOUNDS.get(fam, (1e-4, 1e-3))
        assert np.percentile(err, 99) <= p99 and err.max() <= mx, \
            (fam, float(np.percentile(err, 99)), float(err.max()))
