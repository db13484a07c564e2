"""Shared loaders for the golden fixtures made by tests/golden/make_golden.py."""
import json
import os

import numpy as np

from athena_gb300.mesh import MeshSpec

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def meta():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


def case_names(relativistic=None):
    """Case names; ``relativistic`` True/False selects SR or Newtonian cases only."""
    cases = meta()["cases"]
    return sorted(n for n, c in cases.items()
                  if relativistic is None or bool(c.get("relativistic")) == relativistic)


def load_case(name):
    c = meta()["cases"][name]
    mesh = MeshSpec(tuple(c["nx"]), tuple(c["nb"]), c["ng"], tuple(c["xmin"]),
                    tuple(c["xmax"]))
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    ng = mesh.ng

    def pad_cells(a):
        out = np.zeros((mesh.nblocks, a.shape[1]) + mesh.cell_shape)
        out[:, :, ng:-ng, ng:-ng, ng:-ng] = a
        return out

    def pad_faces(a, d):
        out = np.zeros((mesh.nblocks,) + mesh.face_shapes[d])
        out[:, ng:-ng, ng:-ng, ng:-ng] = a
        return out

    ic = (pad_cells(z["ic_u"]), pad_faces(z["ic_b1"], 0), pad_faces(z["ic_b2"], 1),
          pad_faces(z["ic_b3"], 2))
    if "ic_w" in z.files:   # relativistic: initial primitives (also the first guess)
        c["ic_w"] = pad_cells(z["ic_w"])
    ref = {k: z[k] for k in ("u", "b1", "b2", "b3", "dt")}
    if "w" in z.files:
        ref["w"] = z["w"]
    ref["time"] = float(z["time"])
    return c, mesh, ic, ref


def interior_faces(mesh, b):
    ng = mesh.ng
    return b[:, ng:-ng, ng:-ng, ng:-ng]


def ml_case_names():
    """Names of the multi-level (static refinement) golden cases."""
    return sorted(meta().get("ml_cases", {}))


def load_ml_case(name):
    """(params, MultiLevelMesh, initial state (u, b1, b2, b3) with ghosts zero,
    reference outputs)."""
    from athena_gb300.meshtree import MultiLevelMesh
    c = meta()["ml_cases"][name]
    mesh = MultiLevelMesh(tuple(c["nx"]), tuple(c["nrbx"]), c["ng"], tuple(c["xmin"]),
                          tuple(c["xmax"]), bcs=tuple(c["bc"]),
                          regions=[(tuple(a), tuple(b), lv) for a, b, lv in c["regions"]])
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    ng = mesh.ng

    def pad_cells(a):
        out = np.zeros((mesh.nblocks, a.shape[1]) + mesh.cell_shape)
        out[:, :, ng:-ng, ng:-ng, ng:-ng] = a
        return out

    def pad_faces(a, d):
        out = np.zeros((mesh.nblocks,) + mesh.face_shapes[d])
        out[:, ng:-ng, ng:-ng, ng:-ng] = a
        return out

    ic = (pad_cells(z["ic_u"]), pad_faces(z["ic_b1"], 0), pad_faces(z["ic_b2"], 1),
          pad_faces(z["ic_b3"], 2))
    ref = {k: z[k] for k in ("u", "b1", "b2", "b3", "w", "dt")}
    ref["time"] = float(z["time"])
    return c, mesh, ic, ref


def amr_case_names():
    """Names of the adaptive-refinement golden cases."""
    return sorted(meta().get("amr_cases", {}))


def load_amr_case(name):
    """(params, root MultiLevelMesh, problem generator ic(mesh), reference outputs: per
    cycle block lists and dt, the last cycle's state digest and per-block sums of U)."""
    from athena_gb300 import pgen
    from athena_gb300.meshtree import MultiLevelMesh
    c = meta()["amr_cases"][name]
    mesh0 = MultiLevelMesh(tuple(c["nx"]), tuple(c["nrbx"]), c["ng"], tuple(c["xmin"]),
                           tuple(c["xmax"]), bcs=tuple(c["bc"]))
    p = c["problem"]

    def ic(mesh):
        return pgen.blast_blocks(mesh, c["gamma"], radius=p["radius"], pamb=p["pamb"],
                                 prat=p["prat"], b0=p["b0"], angle_deg=p["angle"],
                                 center=(p["x1_0"], p["x2_0"], p["x3_0"]))
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    offs = z["offsets"]
    locs = [[tuple(int(v) for v in r) for r in z["locs"][offs[i]:offs[i + 1]]]
            for i in range(len(offs) - 1)]
    ref = {"locs": locs, "dt": z["dt"], "usum": z["usum"], "digest": c["digest"],
           "time": c["time"]}
    return c, mesh0, ic, ref
