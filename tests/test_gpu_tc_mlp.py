"""The con2prim network on the tcgen05 tensor cores (tensor-memory accumulators) against
the CPU oracle's bfloat16-rounded forward pass and the mma.sync path."""
import os
import sys

import numpy as np
import pytest

from athena_gb300 import build, pgen
from athena_gb300.learned_c2p import LearnedC2P

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))
import mlp  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def test_tcgen05_inference_matches_oracle():
    net = LearnedC2P(4.0 / 3.0, seed=3)
    feats, targ = net.solver_pairs(1 << 16, 5)
    net.set_standardization(feats, targ)
    net.train(feats, targ, steps=500, batch=2048, lr=2.0e-3, seed=5)
    for n in (1, 127, 128, 5003, 1 << 18):   # ragged last tile, many tiles per CTA
        w, bcc, u = pgen.sr_isolated_cells(n, seed=40 + n)
        f = net.features(net.to_dev(u), net.to_dev(bcc))
        y_tc = net.infer_tc(f).cpu().numpy()
        y_mma = net.infer(f).cpu().numpy()
        want = mlp.infer_bf16(net.params.cpu().numpy(), f.cpu().numpy())
        assert np.all(np.isfinite(y_tc))
        d = np.abs(y_tc - want)
        # same bf16 rounding points; FP32 accumulation order and SiLU exponent differ
        assert d.mean() < 2e-3 and d.max() < 5e-2, (n, d.mean(), d.max())
        assert np.abs(y_tc - y_mma).mean() < 2e-3, n
