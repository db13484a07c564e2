"""The reference-side shim (athena_gb300/shim/athgpu_operator_shim.cpp) compiled against
the reference's own headers and linked into the reference with libathgpu.so: the six
stage-update member functions the shim defines take the place of the reference's (CPU
check; the reference tree is needed, so the test is skipped where it is absent)."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_ref  # noqa: E402


def _sizes(path):
    """defined function symbols -> size (nm -S of objects and executables built here)."""
    out = subprocess.run(["nm", "-S", "--defined-only", path], capture_output=True,
                         text=True, check=True).stdout.splitlines()
    sizes = {}
    for line in out:
        p = line.split()
        if len(p) == 4 and p[2] in "TtWw":
            sizes[p[3]] = int(p[1], 16)
    return sizes


@pytest.mark.skipif(not build_ref.reference_present(),
                    reason="the reference source tree is not present")
def test_shim_replaces_the_stage_operators():
    from athena_gb300 import build
    build.build()
    exe = build_ref.build_gpu_variant("mhd_hlld_g2")
    # the executable runs (dynamic libraries resolved) and is the reference's own
    r = subprocess.run([exe, "-c"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert "Riemann solver:             hlld" in r.stdout
    shim = _sizes(os.path.join(os.path.dirname(exe), "obj", "athgpu_operator_shim.o"))
    final = _sizes(exe)
    base_dir = os.path.join(build_ref.OUT, "mhd_hlld_g2", "obj")
    for obj, want in build_ref.SHIM_REPLACES.items():
        mangled = [m for m, d in build_ref.defined_symbols(os.path.join(base_dir, obj))
                   if d.startswith(want)]
        assert len(mangled) == 1, want
        sym = mangled[0]
        ref_size = _sizes(os.path.join(base_dir, obj))[sym]
        # the linked definition is the shim's (its size), not the reference's
        assert sym in shim and final[sym] == shim[sym], want
        assert shim[sym] != ref_size, want
