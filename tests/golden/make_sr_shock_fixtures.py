"""Fixtures for the relativistic MHD shock tubes of the reference's regression suite
(tst/regression/scripts/tests/sr/mhd_shocks_hlld.py, problems 1, 2 and 4 of Mignone,
Ugliano & Bodo 2009, inputs/mhd_sr/athinput.mub_{1,2,4}): the reference's 10000-zone HLLD
solutions tst/regression/data/sr_mhd_shock{1,2,4}_hlld.vtk, read as data (legacy VTK,
rectilinear grid, big-endian float32) and stored as tests/golden/sr_mhd_shocks_ref.npz:
per problem the x1 face coordinates and the conserved density, total energy, the three
momenta and the three cell-centred field components.

Run where the reference's source tree is present:  python tests/golden/make_sr_shock_fixtures.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import build_ref  # noqa: E402  (the reference's location)


def read_vtk(path):
    """Arrays of an Athena++ legacy-VTK dump of a 1-D rectilinear grid."""
    raw = open(path, "rb").read()
    pos = 0
    out = {}

    def line():
        nonlocal pos
        end = raw.index(b"\n", pos)
        s = raw[pos:end].decode("ascii").strip()
        pos = end + 1
        return s

    def floats(n):
        nonlocal pos
        a = np.frombuffer(raw, dtype=">f4", count=n, offset=pos).astype(np.float32)
        pos += 4 * n
        return a

    ncell = None
    while pos < len(raw):
        s = line()
        if not s:
            continue
        w = s.split()
        if w[0] == "X_COORDINATES":
            out["x1f"] = floats(int(w[1]))
        elif w[0] in ("Y_COORDINATES", "Z_COORDINATES"):
            floats(int(w[1]))
        elif w[0] == "CELL_DATA":
            ncell = int(w[1])
        elif w[0] == "SCALARS":
            line()  # LOOKUP_TABLE default
            out[w[1]] = floats(ncell)
        elif w[0] == "VECTORS":
            out[w[1]] = floats(3 * ncell).reshape(ncell, 3)
    return out


def main():
    data = {}
    for p in (1, 2, 4):
        v = read_vtk(os.path.join(build_ref.REF, "tst", "regression", "data",
                                  "sr_mhd_shock%d_hlld.vtk" % p))
        data["x1f_%d" % p] = v["x1f"]
        data["dens_%d" % p] = v["dens"]
        data["Etot_%d" % p] = v["Etot"]
        data["mom_%d" % p] = v["mom"]
        data["ccB_%d" % p] = v["cc-B"]
    np.savez_compressed(os.path.join(HERE, "sr_mhd_shocks_ref.npz"), **data)


if __name__ == "__main__":
    main()
