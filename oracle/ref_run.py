"""Run the reference binaries built by oracle/build_ref.py and read their state dumps.

TEST INFRASTRUCTURE ONLY (used to make and check golden fixtures in this container;
the reference source tree is not present where the GPU tests run).
"""
import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")


BC_NAMES = {0: "periodic", 1: "outflow", 2: "reflecting"}


def athinput(mesh, gamma, xorder, cfl, nlim, tlim, problem, extra_problem=None,
             integrator="vl2", num_threads=1, history_every_cycle=False,
             bc=(0, 0, 0, 0, 0, 0)):
    """Text of an athinput file for a uniform mesh described by MeshSpec (mesh-face
    boundary flags bc: 0 periodic, 1 outflow, 2 reflecting);
    history_every_cycle adds a history output (Ref.hst) written after every cycle at full
    double precision."""
    lines = ["<job>", "problem_id = Ref"]
    if history_every_cycle:
        lines += ["<output1>", "file_type = hst", "dt = 1.0e-12",
                  "data_format = %24.16e"]
    lines += ["<time>", "cfl_number = %r" % cfl,
             "nlim = %d" % nlim, "tlim = %r" % tlim, "integrator = %s" % integrator,
             "xorder = %s" % xorder, "ncycle_out = 100000", "<mesh>"]
    for d, n in enumerate(("1", "2", "3")):
        lines += ["nx%s = %d" % (n, mesh.nx[d]), "x%smin = %r" % (n, mesh.xmin[d]),
                  "x%smax = %r" % (n, mesh.xmax[d]), "ix%s_bc = %s" % (n, BC_NAMES[bc[2 * d]]),
                  "ox%s_bc = %s" % (n, BC_NAMES[bc[2 * d + 1]])]
    lines += ["num_threads = %d" % num_threads, "refinement = none", "<meshblock>"]
    for d, n in enumerate(("1", "2", "3")):
        lines.append("nx%s = %d" % (n, mesh.bx[d]))
    lines += ["<hydro>", "gamma = %r" % gamma, "iso_sound_speed = 1.0", "<problem>"]
    for k, v in (problem or {}).items():
        lines.append("%s = %s" % (k, v))
    for k, v in (extra_problem or {}).items():
        lines.append("%s = %s" % (k, v))
    return "\n".join(lines) + "\n"


def athinput_multilevel(mesh, gamma, xorder, cfl, nlim, tlim, problem,
                        refinement="static", regions=(), numlevel=None, amr=None,
                        integrator="vl2", hydro=None):
    """Text of an athinput file for a multi-level mesh (meshtree.MultiLevelMesh):
    static refinement regions [(xmin3, xmax3, level)] and/or adaptive refinement
    (numlevel, and the <mesh> AMR keys in amr, e.g. derefine_count); extra <hydro> keys
    in hydro (e.g. dfloor, pfloor)."""
    lines = ["<job>", "problem_id = Ref", "<time>", "cfl_number = %r" % cfl,
             "nlim = %d" % nlim, "tlim = %r" % tlim, "integrator = %s" % integrator,
             "xorder = %s" % xorder, "ncycle_out = 100000", "<mesh>"]
    for d, n in enumerate(("1", "2", "3")):
        lines += ["nx%s = %d" % (n, mesh.nx[d]), "x%smin = %r" % (n, mesh.xmin[d]),
                  "x%smax = %r" % (n, mesh.xmax[d]),
                  "ix%s_bc = %s" % (n, BC_NAMES[mesh.bcs[2 * d]]),
                  "ox%s_bc = %s" % (n, BC_NAMES[mesh.bcs[2 * d + 1]])]
    lines += ["num_threads = 1", "refinement = %s" % refinement]
    if numlevel is not None:
        lines.append("numlevel = %d" % numlevel)
    for k, v in (amr or {}).items():
        lines.append("%s = %s" % (k, v))
    lines.append("<meshblock>")
    for d, n in enumerate(("1", "2", "3")):
        lines.append("nx%s = %d" % (n, mesh.bx[d]))
    for r, (lo, hi, lev) in enumerate(regions):
        lines.append("<refinement%d>" % (r + 1))
        for d, n in enumerate(("1", "2", "3")):
            lines += ["x%smin = %r" % (n, lo[d]), "x%smax = %r" % (n, hi[d])]
        lines.append("level = %d" % lev)
    lines += ["<hydro>", "gamma = %r" % gamma, "iso_sound_speed = 1.0"]
    for k, v in (hydro or {}).items():
        lines.append("%s = %s" % (k, v))
    lines.append("<problem>")
    for k, v in (problem or {}).items():
        lines.append("%s = %s" % (k, v))
    return "\n".join(lines) + "\n"


def read_dump_blocks(path):
    """Parse one dump of ref_pgen/dump_hook.cpp in the reference's own block order:
    dict with locs [(level, lx1, lx2, lx3)], arrays u, w, b1, b2, b3, bcc stacked over
    blocks, and ncycle, time, dt."""
    with open(path, "rb") as f:
        data = f.read()
    magic, ver, nbl, ncyc = struct.unpack_from("<4i", data, 0)
    assert magic == 0x41544844 and ver == 1
    t_after, dt_used = struct.unpack_from("<2d", data, 16)
    nc1, nc2, nc3, ng, nh = struct.unpack_from("<5i", data, 32)
    off = 52
    shapes = {"u": (nh, nc3, nc2, nc1), "w": (nh, nc3, nc2, nc1),
              "b1": (nc3, nc2, nc1 + 1), "b2": (nc3, nc2 + 1, nc1),
              "b3": (nc3 + 1, nc2, nc1), "bcc": (3, nc3, nc2, nc1)}
    out = {k: np.zeros((nbl,) + s) for k, s in shapes.items()}
    locs = []
    for b in range(nbl):
        lx1, lx2, lx3 = struct.unpack_from("<3q", data, off)
        (lev,) = struct.unpack_from("<i", data, off + 24)
        locs.append((lev, lx1, lx2, lx3))
        off += 28
        for key in ("u", "w", "b1", "b2", "b3", "bcc"):
            sz = int(np.prod(shapes[key]))
            out[key][b] = np.frombuffer(data, dtype="<f8", count=sz,
                                        offset=off).reshape(shapes[key])
            off += 8 * sz
    out.update(locs=locs, ncycle=ncyc, time=t_after, dt=dt_used)
    return out


def read_history(path):
    """Rows of a reference history file: list of dicts column name -> value."""
    names, rows = None, []
    for line in open(path):
        if line.startswith("#") and "[1]=" in line:
            names = [tok.split("=")[1] for tok in line[1:].split()]
        elif line.strip() and not line.startswith("#"):
            rows.append(dict(zip(names, (float(v) for v in line.split()))))
    return rows


def read_dump(path, mesh):
    """Parse one dump written by ref_pgen/dump_hook.cpp into per-block arrays in the
    lexicographic block order of MeshSpec."""
    with open(path, "rb") as f:
        data = f.read()
    magic, ver, nbl, ncyc = struct.unpack_from("<4i", data, 0)
    assert magic == 0x41544844 and ver == 1
    t_after, dt_used = struct.unpack_from("<2d", data, 16)
    nc1, nc2, nc3, ng, nh = struct.unpack_from("<5i", data, 32)
    off = 52
    ncell = nc1 * nc2 * nc3
    sizes = [nh * ncell, nh * ncell, nc3 * nc2 * (nc1 + 1), nc3 * (nc2 + 1) * nc1,
             (nc3 + 1) * nc2 * nc1, 3 * ncell]
    out = {k: np.zeros((mesh.nblocks,) + s) for k, s in (
        ("u", (5,) + mesh.cell_shape), ("w", (5,) + mesh.cell_shape),
        ("b1", mesh.face_shapes[0]), ("b2", mesh.face_shapes[1]),
        ("b3", mesh.face_shapes[2]), ("bcc", (3,) + mesh.cell_shape))}
    for _ in range(nbl):
        lx1, lx2, lx3 = struct.unpack_from("<3q", data, off)
        off += 28
        b = (lx3 * mesh.nb[1] + lx2) * mesh.nb[0] + lx1
        for key, sz in zip(("u", "w", "b1", "b2", "b3", "bcc"), sizes):
            arr = np.frombuffer(data, dtype="<f8", count=sz, offset=off)
            out[key][b] = arr.reshape(out[key].shape[1:])
            off += 8 * sz
    out.update(ncycle=ncyc, time=t_after, dt=dt_used)
    return out


def write_ic(path, kind, q, f1, f2, f3):
    """Binary initial state read by ref_pgen/load_ic.cpp (global interior arrays)."""
    nx3, nx2, nx1 = q.shape[1:]
    with open(path, "wb") as f:
        f.write(struct.pack("<4i", kind, nx1, nx2, nx3))
        for a in (q, f1, f2, f3):
            f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def write_blocks_ic(path, mesh, u, b1, b2, b3):
    """Per-block initial state read by ref_pgen/load_blocks.cpp (interior cells and
    faces of every block, in gid order)."""
    ng, (n1, n2, n3) = mesh.ng, mesh.bx
    with open(path, "wb") as f:
        f.write(struct.pack("<4i", mesh.nblocks, n1, n2, n3))
        for b, loc in enumerate(mesh.locs):
            f.write(struct.pack("<i3q", loc.level, loc.lx1, loc.lx2, loc.lx3))
            for a in (u[b][:, ng:ng + n3, ng:ng + n2, ng:ng + n1],
                      b1[b][ng:ng + n3, ng:ng + n2, ng:ng + n1 + 1],
                      b2[b][ng:ng + n3, ng:ng + n2 + 1, ng:ng + n1],
                      b3[b][ng:ng + n3 + 1, ng:ng + n2, ng:ng + n1]):
                f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def run_reference(variant, exe, text, workdir=None, ic=None, blocks_ic=None):
    """Run oracle/_ref/<variant>/<exe> on an athinput text; returns (dir, stdout)."""
    binpath = os.path.join(REF_OUT, variant, exe)
    if not os.path.exists(binpath):
        from build_ref import build_variant
        build_variant(variant)
    d = workdir or tempfile.mkdtemp(prefix="athref_")
    if ic is not None:
        write_ic(os.path.join(d, "ic.bin"), *ic)
    if blocks_ic is not None:
        write_blocks_ic(os.path.join(d, "ic.bin"), *blocks_ic)
    with open(os.path.join(d, "athinput"), "w") as f:
        f.write(text)
    r = subprocess.run([binpath, "-i", "athinput"], cwd=d, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    return d, r.stdout
