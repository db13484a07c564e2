"""The integer-pipe FP64 <-> FP32 conversions and the FP64 difference of two floats that
the FP32 kernels form against the hardware's, bit for bit, on random values and the
rounding edge cases."""
import ctypes

import numpy as np
import pytest

from athena_gb300 import build
from athena_gb300.runtime import _check, load_library

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def _doubles(rng, n):
    # random bits over the exponents that round to normal floats and beyond
    e = rng.integers(1023 - 160, 1023 + 160, n, dtype=np.uint64)
    frac = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    sign = rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    r = (sign | (e << np.uint64(52)) | frac).view(np.float64)
    # exact ties between two floats (odd and even lower neighbours), and the values just
    # below / above a tie
    f = rng.standard_normal(4096).astype(np.float32)
    lo = f.astype(np.float64)
    hi = np.nextafter(f, np.float32(np.inf)).astype(np.float64)
    tie = 0.5 * (lo + hi)
    ties = np.concatenate([tie, np.nextafter(tie, -np.inf), np.nextafter(tie, np.inf)])
    fmax = float(np.finfo(np.float32).max)
    tiny = float(np.finfo(np.float32).tiny)
    special = np.array([0.0, -0.0, 1.0, -1.0, fmax, -fmax, np.nextafter(fmax, np.inf),
                        fmax * (1 + 2.0 ** -25), fmax * (1 + 2.0 ** -24), 3.5e38, 1e300,
                        tiny, -tiny, np.nextafter(tiny, 0.0), tiny * 0.5, 1e-40, 1e-45,
                        1e-300, 5e-324, np.inf, -np.inf, np.nan,
                        1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, 2.0 - 2.0 ** -25])
    return np.concatenate([r, ties, special])


def _floats(rng, n):
    bits = rng.integers(0, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    special = np.array([0.0, -0.0, 1.0, np.inf, -np.inf, np.nan, 1e-40, -1e-45,
                        np.finfo(np.float32).max, np.finfo(np.float32).tiny],
                       dtype=np.float32)
    return np.concatenate([bits.view(np.float32), special])


def _float_pairs(rng, n):
    """Consecutive pairs (f[2q], f[2q+1]) for the FP64 difference: random bits, close
    values, every exponent gap up to beyond the integer path's 28, equal and opposite
    values, zeros, subnormals, infinities and NaNs."""
    n -= n % 2
    a = rng.standard_normal(n // 2).astype(np.float32) * np.float32(2.0) ** rng.integers(
        -100, 100, n // 2).astype(np.float32)
    kind = np.arange(n // 2) % 6
    gap = rng.integers(0, 36, n // 2)
    b = np.where(kind == 0, rng.integers(0, 1 << 32, n // 2, dtype=np.uint64)
                 .astype(np.uint32).view(np.float32),
                 np.where(kind == 1, a * (1 + rng.standard_normal(n // 2).astype(np.float32)
                                          * np.float32(1e-3)),
                 np.where(kind == 2, rng.standard_normal(n // 2).astype(np.float32) * a
                          * np.float32(2.0) ** -gap.astype(np.float32),
                 np.where(kind == 3, a, np.where(kind == 4, -a,
                          rng.standard_normal(n // 2).astype(np.float32) * a
                          * np.float32(2.0) ** gap.astype(np.float32))))))
    out = np.empty(n, np.float32)
    out[0::2] = a
    out[1::2] = b.astype(np.float32)
    special = np.array([0.0, 1.0, -0.0, 1.0, 1.0, 0.0, 1e-40, 1.0, 1.0, -1e-45, np.inf, 1.0,
                        1.0, np.nan, np.finfo(np.float32).max, -np.finfo(np.float32).max,
                        np.finfo(np.float32).tiny, np.finfo(np.float32).tiny * 2,
                        1.0, 1.0 + 2.0 ** -23, 2.0 ** 28, 1.0, 2.0 ** 29, 1.0,
                        0.0, -0.0, -0.0, 0.0, -0.0, -0.0, 0.0, 0.0, -0.0, 2.5, 3.0, -0.0,
                        0.0, 1e-40, -1e-45, 0.0, 0.0, np.inf, -np.inf, -0.0, np.nan, 0.0],
                       dtype=np.float32)
    return np.concatenate([special, out])


def test_integer_pipe_conversions_match_hardware():
    import torch
    L = load_library()
    f = L.athgpu_selftest_conversions
    f.argtypes = [ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    rng = np.random.default_rng(12)
    d = _doubles(rng, 1 << 20)
    head = _floats(rng, d.size // 2)
    fl = np.concatenate([head[:head.size - head.size % 2], _float_pairs(rng, d.size)])
    fl = np.resize(fl, d.size)
    dev = torch.device("cuda", 0)
    td = torch.from_numpy(d).to(dev)
    tf = torch.from_numpy(fl).to(dev)
    mm = torch.zeros(3, dtype=torch.int64, device=dev)
    _check(f(d.size, td.data_ptr(), tf.data_ptr(), mm.data_ptr(),
             torch.cuda.current_stream().cuda_stream), "athgpu_selftest_conversions")
    torch.cuda.synchronize()
    assert mm.cpu().tolist() == [0, 0, 0]
