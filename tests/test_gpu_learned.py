"""Learned con2prim guess on the GPU: features, BF16 tensor-core inference, FP32 training
gradients against the CPU oracle, the plain per-cell solve against the oracle's
Newman-Hamlin solve, and what the trained network gains over the plain start."""
import os
import sys

import numpy as np
import pytest

import oracle as O
from athena_gb300 import build, pgen
from athena_gb300.learned_c2p import (MODE_LEARNED, MODE_LEARNED_FP32, MODE_PLAIN,
                                      LearnedC2P)

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))
import mlp  # noqa: E402

pytestmark = pytest.mark.gpu
GAMMA = 4.0 / 3.0


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


@pytest.fixture(scope="module")
def trained():
    """One network trained on solver-generated pairs (2^20 cells, 8000 Adam steps)."""
    net = LearnedC2P(GAMMA, seed=0)
    hist = net.fit(n=1 << 20, steps=8000, batch=4096, lr=2.0e-3, seed=101)
    return net, hist


def _cells(net, n, seed):
    w, bcc, u = pgen.sr_isolated_cells(n, seed=seed, gamma=GAMMA)
    return w, bcc, u, net.to_dev(u), net.to_dev(bcc)


def test_features_match_oracle():
    net = LearnedC2P(GAMMA)
    w, bcc, u, cons, b = _cells(net, 4099, 21)
    f = net.features(cons, b).cpu().numpy()
    want = mlp.features(u, bcc)
    # FP32 with fast logarithms against FP64
    assert np.allclose(f, want, rtol=2e-5, atol=2e-6)


def test_loss_grad_matches_oracle():
    net = LearnedC2P(GAMMA, seed=4)
    rng = np.random.default_rng(8)
    p = net.params.cpu().numpy()
    p[:mlp.NTRAIN] += (0.05 * rng.standard_normal(mlp.NTRAIN)).astype(np.float32)
    net.params = net.to_dev(p)
    x = rng.standard_normal((1000, 5)).astype(np.float32)
    t = rng.standard_normal((1000, 2)).astype(np.float32)
    loss, g = net.loss_grad(net.to_dev(x), net.to_dev(t))
    loss_o, g_o = mlp.loss_grad(p, x, t)
    assert abs(loss - loss_o) <= 1e-5 * loss_o
    g = g.cpu().numpy()
    # FP32 accumulation over 1000 rows: per-entry error against the FP64 oracle
    assert np.all(np.abs(g - g_o) <= 1e-4 * np.abs(g_o).max() + 1e-4 * np.abs(g_o))


def test_bf16_inference_matches_oracle(trained):
    net, _ = trained
    w, bcc, u, cons, b = _cells(net, 5003, 33)   # not a multiple of 32: ragged last warp
    f = net.features(cons, b)
    y = net.infer(f).cpu().numpy()
    want = mlp.infer_bf16(net.params.cpu().numpy(), f.cpu().numpy())
    d = np.abs(y - want)
    # same bf16 rounding points; FP32 accumulation order and SiLU exponent differ
    assert d.mean() < 2e-3 and d.max() < 5e-2, (d.mean(), d.max())


def test_plain_solve_matches_oracle():
    """Mode 0 from the same starts as the oracle: the FP64 solve of
    ConservedToPrimitiveNormal per cell (CUDA acos/cos/cbrt may differ in the last bit
    from the host's, so 1e-12 relative, and iteration counts equal in nearly all cells)."""
    net = LearnedC2P(GAMMA)
    n = 1 << 16
    w, bcc, u, cons, b = _cells(net, n, 44)
    for guess, n1 in ((np.full(n, 1e-12), 0), (w[:, 4] * 1.01, 0), (w[:, 4] * 1.01, 2),
                      (np.full(n, 1e-12), 15)):
        prim, it, _, fb = net.solve(cons, b, MODE_PLAIN, pgas_guess=net.to_dev(guess),
                                    phase1_iterations=n1)
        prim, it = prim.cpu().numpy(), it.cpu().numpy()
        po, ito = O.sr_c2p_cells(u, bcc, guess, GAMMA)
        ito = np.where(ito >= 0, ito + 1, -1)    # loop index at exit -> passes
        assert fb == 0
        assert np.mean(it == ito) > 0.999
        ok = (it >= 0) & (ito >= 0)
        for q in range(5):
            scale = np.abs(po[ok, q]).max()
            assert np.all(np.abs(prim[ok, q] - po[ok, q]) <= 1e-10 * np.abs(po[ok, q])
                          + 1e-12 * scale), q


def test_training_reduces_loss(trained):
    _, hist = trained
    assert np.all(np.isfinite(hist))
    assert hist[-100:].mean() < 0.1 * hist[:10].mean()


def test_learned_start_halves_iterations_with_no_unconverged_cells(trained):
    """On fresh cells: FP64 passes of the learned (+FP32 refined) start against the plain
    start from the pressure floor (an isolated cell has no previous pressure); every cell
    converges (fallback included) and the solution is the plain solve's root."""
    net, _ = trained
    n = 1 << 20
    w, bcc, u, cons, b = _cells(net, n, 777)
    prim0, it0, _, _ = net.solve(cons, b, MODE_PLAIN)
    prim2, it2, it32, fb2 = net.solve(cons, b, MODE_LEARNED_FP32, want_iters32=True)
    prim1, it1, _, fb1 = net.solve(cons, b, MODE_LEARNED)
    it0, it1, it2 = (t.cpu().numpy() for t in (it0, it1, it2))
    passes0 = it0[it0 >= 0].mean()
    passes2 = it2.mean()
    assert np.all(it2 >= 0) and np.all(it1 >= 0)
    assert passes2 <= 0.5 * passes0, (passes0, passes2)
    assert it1.mean() < passes0
    ok = it0 >= 0
    p0, p2 = prim0.cpu().numpy()[ok], prim2.cpu().numpy()[ok]
    # both stop within the solver's 1e-12 absolute pressure tolerance of the root
    rel = np.abs(p2 - p0) / (np.abs(p0) + 1e-300)
    assert np.median(rel[:, 4]) < 1e-12
    assert np.all(np.abs(p2[:, 4] - p0[:, 4]) <= 1e-9 * np.maximum(1.0, np.abs(p0[:, 4])))
    assert fb2 < 1e-4 * n
