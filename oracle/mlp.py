"""CPU oracle of the learned con2prim network (test infrastructure only).

FP64 numpy restatement of the network in athena_gb300/csrc/sr_learned.cu: the
5 -> 64 -> 64 -> 2 SiLU multilayer perceptron, its mean-squared-error loss and the
back-propagated gradient, used by the tests to check the GPU forward/backward kernels, and
a BF16-operand forward that rounds the same tensors to bfloat16 as the tensor-core
inference does, to check that path.  The network has no counterpart in the reference (it
replaces the start value of ConservedToPrimitiveNormal, adiabatic_mhd_sr.cpp:404-522), so
this oracle is pinned by finite differences of its own loss (tests/test_mlp_oracle.py),
not by reference vectors.
"""
import numpy as np

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


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[OFF_W1:OFF_B1].reshape(NH, NIN), p[OFF_B1:OFF_W2],
            p[OFF_W2:OFF_B2].reshape(NH, NH), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3].reshape(NOUT, NH), p[OFF_B3:OFF_XM])


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s + z * s * (1.0 - s)


def forward(p, x):
    """Standardized inputs x[B,5] -> (z1, z2, y) in FP64."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    z1 = x @ w1.T + b1
    z2 = silu(z1) @ w2.T + b2
    y = silu(z2) @ w3.T + b3
    return z1, z2, y


def loss_grad(p, x, t):
    """Loss = mean over rows and outputs of (y - t)^2 and its gradient with respect to
    the NTRAIN trainable parameters (same layout as the parameter vector)."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    z1, z2, y = forward(p, x)
    n = y.size
    loss = np.sum((y - t) ** 2) / n
    dy = 2.0 * (y - t) / n
    h2 = silu(z2)
    h1 = silu(z1)
    dz2 = (dy @ w3) * dsilu(z2)
    dz1 = (dz2 @ w2) * dsilu(z1)
    g = np.zeros(NTRAIN)
    g[OFF_W1:OFF_B1] = (dz1.T @ x).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W3:OFF_B3] = (dy.T @ h2).ravel()
    g[OFF_B3:OFF_XM] = dy.sum(0)
    return loss, g


def to_bf16(a):
    """Round float values to bfloat16 (round to nearest, ties to even), returned as
    float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def infer_bf16(p, feats):
    """Raw features[n,5] -> de-standardized outputs[n,2], with the weights and each
    layer's input activations rounded to bfloat16 and everything else in FP64, the
    rounding points of the tensor-core inference."""
    p = np.asarray(p, dtype=np.float32)
    w1, b1, w2, b2, w3, b3 = unpack(p)
    xm, xs = p[OFF_XM:OFF_XS].astype(np.float64), p[OFF_XS:OFF_YM].astype(np.float64)
    ym, ys = p[OFF_YM:OFF_YS].astype(np.float64), p[OFF_YS:].astype(np.float64)
    x = (np.asarray(feats, dtype=np.float64) - xm) / xs
    h1 = silu(to_bf16(x) @ to_bf16(w1).T + b1)
    h2 = silu(to_bf16(h1) @ to_bf16(w2).T + b2)
    y = to_bf16(h2) @ to_bf16(w3).T + b3
    return y * ys + ym


def features(cons, bcc):
    """Oracle of athgpu_sr_features: (log(D/E), log(M^2/E^2), log(B^2/E),
    (M.B)^2/(M^2 B^2), log((E - sqrt(M^2 + D^2))/E)) per cell, in FP64."""
    D, E = cons[:, 0], cons[:, 4]
    M = cons[:, 1:4]
    msq = cons[:, 1] * cons[:, 1] + cons[:, 2] * cons[:, 2] + cons[:, 3] * cons[:, 3]
    bsq = (bcc * bcc).sum(1)
    tt = (M * bcc).sum(1)
    rh = E - np.sqrt(msq + D * D)
    return np.stack([np.log(D / E), np.log(msq / (E * E) + 1e-30), np.log(bsq / E + 1e-30),
                     tt * tt / (msq * bsq + 1e-30),
                     np.log(np.maximum(rh / E, 1e-30))], 1)
