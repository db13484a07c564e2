"""History output: the oracle's sums on the reference's final golden state against the
reference's own Ref.hst (CPU), and athgpu_history after every cycle on the GPU."""
import os
import sys

import numpy as np
import pytest

from golden_cases import load_case, meta

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                "oracle"))
import history  # noqa: E402


def _close(got, want, scale):
    return abs(got - want) <= 1e-13 * max(abs(want), scale)


def test_oracle_history_matches_reference_hst():
    h = meta()["history"]
    c, mesh, ic, ref = load_case(h["case"])
    sums = history.history_sums(mesh, ref["u"], ref["b1"], ref["b2"], ref["b3"])
    last = h["rows"][-1]
    for k in history.NAMES:
        assert _close(sums[k], last[k], 1.0), (k, sums[k], last[k])


@pytest.mark.gpu
def test_gpu_history_matches_reference_every_cycle():
    from athena_gb300 import build
    from athena_gb300.runtime import StageUpdate
    build.build()
    h = meta()["history"]
    c, mesh, ic, ref = load_case(h["case"])
    rows = h["rows"]
    for prec, tol in (("fp64", 1e-13), ("fp32", 2e-6)):
        g = StageUpdate(mesh, c["gamma"], xorder=c["xorder"], rsolver=c["rsolver"],
                        precision=prec, cfl=c["cfl"], tlim=c["tlim"], bc=c.get("bc"))
        g.set_state(*ic)
        g.initialize()
        for cyc in range(c["ncycle"] + 1):
            if cyc:
                g.cycle(1)
            got = g.history()
            again = g.history()
            assert got == again   # deterministic reduction
            for k in history.NAMES:
                want = rows[cyc][k]
                assert abs(got[k] - want) <= tol * max(abs(want), 1.0), (prec, cyc, k)
        g.close()
