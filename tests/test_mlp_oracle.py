"""The CPU oracle of the learned con2prim network, pinned by finite differences of its
own loss (the network has no reference counterpart), and its bfloat16 rounding."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))
import mlp  # noqa: E402

from athena_gb300 import learned_c2p, pgen  # noqa: E402


def test_layout_matches_library_constants():
    assert mlp.NPARAM == learned_c2p.NPARAM == 4688
    assert mlp.NTRAIN == learned_c2p.NTRAIN
    text = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                             "include", "athena_gb300.h")).read()
    assert "#define ATHGPU_MLP_NPARAM 4688" in text


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = learned_c2p.init_params(seed=5).astype(np.float64)
    p[:mlp.NTRAIN] += 0.05 * rng.standard_normal(mlp.NTRAIN)
    x = rng.standard_normal((17, mlp.NIN))
    t = rng.standard_normal((17, mlp.NOUT))
    loss, g = mlp.loss_grad(p, x, t)
    idx = np.concatenate([rng.choice(mlp.NTRAIN, 60, replace=False),
                          [mlp.OFF_B1, mlp.OFF_B2, mlp.OFF_B3, mlp.OFF_B3 + 1,
                           mlp.OFF_W3, mlp.OFF_W1]])
    h = 1e-6
    for q in idx:
        pp, pm = p.copy(), p.copy()
        pp[q] += h
        pm[q] -= h
        fd = (mlp.loss_grad(pp, x, t)[0] - mlp.loss_grad(pm, x, t)[0]) / (2 * h)
        assert abs(fd - g[q]) <= 1e-7 + 1e-5 * abs(g[q]), (q, fd, g[q])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, 1.0 + 2.0 ** -9, -2.5,
                  1.0 + 2.0 ** -7 + 2.0 ** -9, 3.0e38], dtype=np.float32)
    r = mlp.to_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0          # tie rounds to even (down)
    assert r[2] == 1.0 + 2.0 ** -6              # tie rounds to even (up)
    assert r[3] == 1.0 and r[4] == -2.5
    assert r[5] == 1.0 + 2.0 ** -7              # below the half-way point: down
    assert np.isfinite(r[6])


def test_features_are_scale_free_in_the_right_slots():
    w, bcc, u = pgen.sr_isolated_cells(64, seed=2)
    f = mlp.features(u, bcc)
    # scaling rho, p and B^2 by s scales D, M, E by s and B by sqrt(s): no feature moves
    s = 7.0
    f2 = mlp.features(u * s, bcc * np.sqrt(s))
    assert np.allclose(f, f2, rtol=1e-10, atol=1e-10)
    assert np.all((f[:, 3] >= 0) & (f[:, 3] <= 1 + 1e-12))
    # the residual energy feature: 3 p for a cold, slow, unmagnetized cell at gamma 4/3
    w0 = np.array([[1.0, 1e-4, 0.0, 0.0, 1e-6]])
    u0 = pgen.sr_prim_to_cons(w0.T, np.zeros((3, 1)), 4.0 / 3.0).T
    f0 = mlp.features(u0, np.zeros((1, 3)))
    assert abs(np.exp(f0[0, 4]) * u0[0, 4] / (3e-6) - 1.0) < 1e-3
