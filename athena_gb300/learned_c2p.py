"""Learned initial guess for the special-relativistic con2prim, on the GPU.

``LearnedC2P`` owns the 5 -> 64 -> 64 -> 2 SiLU network of ``csrc/sr_learned.cu``: it
builds training pairs with the library's own FP64 Newman-Hamlin solver (the root of
ConservedToPrimitiveNormal, adiabatic_mhd_sr.cpp:404-522, for each sampled conserved
state), trains the network with the library's FP32 forward/backward/Adam kernels, and
solves cells with the fused BF16 tensor-core guess plus FP64 polish, falling back per
cell to the plain solve.  Device memory is held in torch tensors (plumbing only); every
computation is a call through the C ABI.
"""
import ctypes

import numpy as np

from . import pgen
from .runtime import AthGPUError, _check, load_library

NIN, NH, NOUT = 5, 64, 2
OFF_W1 = 0
OFF_B1 = OFF_W1 + NH * NIN
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NOUT * NH
OFF_XM = OFF_B3 + NOUT
OFF_XS = OFF_XM + NIN
OFF_YM = OFF_XS + NIN
OFF_YS = OFF_YM + NOUT
NPARAM = OFF_YS + NOUT
NTRAIN = OFF_XM

MODE_PLAIN, MODE_LEARNED, MODE_LEARNED_FP32, MODE_REFINED = 0, 1, 2, 3
WARP_MMA = 0x100   # or into a mode: the network on warp-level mma.sync instead of tcgen05

_vp, _ll, _ip = ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int
_SIG = {
    "athgpu_sr_features": ([_ll, _vp, _vp, _vp, _vp], _ip),
    "athgpu_mlp_infer": ([_ll, _vp, _vp, _vp, _vp], _ip),
    "athgpu_mlp_infer_tc": ([_ll, _vp, _vp, _vp, _vp], _ip),
    "athgpu_sr_c2p_cells": ([_ll, ctypes.c_double, ctypes.c_double, _vp, _vp, _vp, _vp, _ip,
                             _ip, _vp, _vp, _vp, _vp, _vp], _ip),
    "athgpu_mlp_loss_grad": ([_vp, _vp, _vp, _ip, _vp, _vp, _vp], _ip),
    "athgpu_mlp_train": ([_vp, _vp, _ll, _vp, _ip, _ip, ctypes.c_float, ctypes.c_ulonglong,
                          _vp, _vp], _ip),
}


def lib():
    L = load_library()
    for name, (args, res) in _SIG.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    return L


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise AthGPUError("the learned con2prim needs a CUDA device")
    return torch


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def init_params(seed=0):
    """Initial parameters (numpy float32 [NPARAM]): uniform +-sqrt(6/(fan_in+fan_out))
    weights, zero biases, identity standardization."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)

    def glorot(n_out, n_in):
        a = np.sqrt(6.0 / (n_in + n_out))
        return rng.uniform(-a, a, (n_out, n_in)).astype(np.float32).ravel()

    p[OFF_W1:OFF_B1] = glorot(NH, NIN)
    p[OFF_W2:OFF_B2] = glorot(NH, NH)
    p[OFF_W3:OFF_B3] = glorot(NOUT, NH)
    p[OFF_XS:OFF_YM] = 1.0
    p[OFF_YS:] = 1.0
    return p


def targets_from_prim(prim, cons):
    """Training targets (log(p_gas/E), log(Lorentz factor)) from solver primitives
    prim[n, 5] (rho, u1, u2, u3, p) and conserved cons[n, 5]."""
    xp = np if isinstance(prim, np.ndarray) else _torch()
    lor = xp.sqrt(1.0 + prim[:, 1] ** 2 + prim[:, 2] ** 2 + prim[:, 3] ** 2)
    return xp.stack([xp.log(prim[:, 4] / cons[:, 4]), xp.log(lor)], 1)


class LearnedC2P:
    """The network's parameters on the device plus the calls that train and use it."""

    def __init__(self, gamma=4.0 / 3.0, pfloor=None, seed=0, device=0):
        torch = _torch()
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.gamma = float(gamma)
        self.pfloor = float(pfloor) if pfloor is not None else 1.0e-12
        self.params = torch.from_numpy(init_params(seed)).to(self.dev)
        self.lib = lib()

    # ---- data -----------------------------------------------------------------------
    def to_dev(self, a, dtype=None):
        t = self.torch.as_tensor(np.ascontiguousarray(a), device=self.dev)
        return t if dtype is None else t.to(dtype)

    def features(self, cons, bcc):
        n = cons.shape[0]
        f = self.torch.empty((n, NIN), dtype=self.torch.float32, device=self.dev)
        _check(self.lib.athgpu_sr_features(n, _ptr(cons), _ptr(bcc), _ptr(f), _stream()),
               "athgpu_sr_features")
        return f

    def solve(self, cons, bcc, mode=MODE_PLAIN, pgas_guess=None, want_iters32=False,
              phase1_iterations=0):
        """Per-cell con2prim of device arrays cons[n,5], bcc[n,3] (float64).  Returns
        (prim[n,5], FP64 passes[n] (-1: not converged), FP32 passes[n] or None,
        fallbacks)."""
        torch = self.torch
        n = cons.shape[0]
        prim = torch.empty((n, 5), dtype=torch.float64, device=self.dev)
        it64 = torch.empty(n, dtype=torch.int32, device=self.dev)
        it32 = torch.zeros(n, dtype=torch.int32, device=self.dev) if want_iters32 else None
        fb = torch.zeros(1, dtype=torch.int32, device=self.dev)
        _check(self.lib.athgpu_sr_c2p_cells(
            n, self.gamma, self.pfloor, _ptr(cons), _ptr(bcc), _ptr(pgas_guess),
            _ptr(self.params), int(mode), int(phase1_iterations), _ptr(prim), _ptr(it64),
            _ptr(it32), _ptr(fb),
            _stream()), "athgpu_sr_c2p_cells")
        return prim, it64, it32, int(fb.item())

    def infer(self, feats):
        out = self.torch.empty((feats.shape[0], NOUT), dtype=self.torch.float32,
                               device=self.dev)
        _check(self.lib.athgpu_mlp_infer(feats.shape[0], _ptr(self.params), _ptr(feats),
                                         _ptr(out), _stream()), "athgpu_mlp_infer")
        return out

    def infer_tc(self, feats):
        """infer() on the tcgen05 tensor-core path (tensor memory accumulators)."""
        out = self.torch.empty((feats.shape[0], NOUT), dtype=self.torch.float32,
                               device=self.dev)
        _check(self.lib.athgpu_mlp_infer_tc(feats.shape[0], _ptr(self.params), _ptr(feats),
                                            _ptr(out), _stream()), "athgpu_mlp_infer_tc")
        return out

    def solver_pairs(self, n, seed):
        """Training pairs generated by the solver: sample isolated SR cells, and solve each
        sampled conserved state with the FP64 solver started from its sampled pressure;
        keep converged cells.  Returns (features, raw targets) on the device."""
        w, bcc, u = pgen.sr_isolated_cells(n, seed=seed, gamma=self.gamma)
        cons = self.to_dev(u)
        b = self.to_dev(bcc)
        prim, it, _, _ = self.solve(cons, b, MODE_PLAIN, pgas_guess=self.to_dev(w[:, 4]))
        ok = it >= 0
        cons, b, prim = cons[ok], b[ok], prim[ok]
        return self.features(cons, b), targets_from_prim(prim, cons).float()

    # ---- training -------------------------------------------------------------------
    def set_standardization(self, feats, targets):
        p = self.params
        p[OFF_XM:OFF_XS] = feats.mean(0)
        p[OFF_XS:OFF_YM] = feats.std(0).clamp_min(1e-6)
        p[OFF_YM:OFF_YS] = targets.mean(0)
        p[OFF_YS:] = targets.std(0).clamp_min(1e-6)

    def train(self, feats, targets, steps=3000, batch=4096, lr=2.0e-3, seed=1):
        """Adam on the device; returns the per-step loss history (numpy)."""
        hist = np.zeros(steps, dtype=np.float32)
        _check(self.lib.athgpu_mlp_train(
            _ptr(feats), _ptr(targets), feats.shape[0], _ptr(self.params), int(steps),
            int(batch), float(lr), int(seed),
            hist.ctypes.data_as(ctypes.c_void_p), _stream()), "athgpu_mlp_train")
        return hist

    def loss_grad(self, x, t):
        """Loss and gradient of standardized batch (x[B,5], t[B,2]) on the device."""
        torch = self.torch
        g = torch.empty(NTRAIN, dtype=torch.float32, device=self.dev)
        loss = torch.empty(1, dtype=torch.float32, device=self.dev)
        _check(self.lib.athgpu_mlp_loss_grad(_ptr(self.params), _ptr(x), _ptr(t), x.shape[0],
                                             _ptr(g), _ptr(loss), _stream()),
               "athgpu_mlp_loss_grad")
        return float(loss.item()), g

    def fit(self, n=1 << 20, steps=3000, batch=4096, lr=2.0e-3, seed=101):
        feats, targets = self.solver_pairs(n, seed)
        self.set_standardization(feats, targets)
        return self.train(feats, targets, steps, batch, lr, seed)

    def save(self, path):
        np.save(path, self.params.cpu().numpy())

    def load(self, path):
        self.params = self.to_dev(np.load(path).astype(np.float32))


def _time_inference(log2n=22, seed=9):
    """Train a small network and time its inference on 2^log2n cells on both tensor-core
    paths (CUDA events, median of 4).  `python -m athena_gb300.learned_c2p [log2n]`."""
    torch = _torch()
    net = LearnedC2P(4.0 / 3.0, seed=3)
    feats, targ = net.solver_pairs(1 << 16, 5)
    net.set_standardization(feats, targ)
    net.train(feats, targ, steps=200, batch=2048, lr=2.0e-3, seed=5)
    w, bcc, u = pgen.sr_isolated_cells(1 << log2n, seed=seed)
    f = net.features(net.to_dev(u), net.to_dev(bcc))
    for name, fn in (("tcgen05", net.infer_tc), ("mma.sync", net.infer)):
        ts = []
        for _ in range(4):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn(f)
            b.record()
            b.synchronize()
            ts.append(a.elapsed_time(b))
        print("%-9s %.3f ms for 2^%d cells" % (name, float(np.median(ts)), log2n))


if __name__ == "__main__":
    import sys
    from . import build
    build.build()
    _time_inference(int(sys.argv[1]) if len(sys.argv) > 1 else 22)
