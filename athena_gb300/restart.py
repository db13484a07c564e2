"""Restart files in the reference's format (RestartOutput::WriteOutputFile,
outputs/restart.cpp:40-246, and the restart branch of the Mesh and MeshBlock
constructors, mesh/mesh.cpp:628-1000), for Newtonian MHD without passive scalars or user
data:

* the parameter dump (ParameterInput::ParameterDump, parameter_input.cpp:835-860), ending
  with ``<par_end>``;
* int nbtotal, int root_level, RegionSize mesh_size (9 doubles, 3 ints, padded to 88
  bytes), double time, double dt, int ncycle, uint64 datasize;
* the ID list: per block LogicalLocation (int64 lx1, lx2, lx3, int level, padded to 32
  bytes) and the double cost;
* per block, in gid order, ``datasize`` bytes: U (5 x nc3 x nc2 x nc1 doubles, ghosts
  included), then the face fields b.x1f, b.x2f, b.x3f (ghosts included).

A run restarted from such a file (``athena -r``, or ``load`` here followed by
initialization) continues exactly as the reference does: Mesh::Initialize(1) makes the
first time step from the stored dt.
"""
import re
import struct
from dataclasses import dataclass, field

import numpy as np

_REGION = struct.Struct("<9d3i4x")       # RegionSize, 88 bytes
_LOC = struct.Struct("<3qi4x")           # LogicalLocation, 32 bytes
_HDR = struct.Struct("<ii")              # nbtotal, root_level
_TAIL = struct.Struct("<ddiQ")           # time, dt, ncycle, datasize (packed, 28 bytes)


@dataclass
class Restart:
    params: str                  # the parameter dump, through "<par_end>\n"
    nbtotal: int
    root_level: int
    mesh_size: tuple             # x1min, x2min, x3min, x1max, x2max, x3max, x1rat,
                                 # x2rat, x3rat, nx1, nx2, nx3
    time: float
    dt: float
    ncycle: int
    locs: list                   # (level, lx1, lx2, lx3) per block in gid order
    costs: np.ndarray
    u: np.ndarray = field(repr=False, default=None)    # [nb][5][nc3][nc2][nc1]
    b1: np.ndarray = field(repr=False, default=None)
    b2: np.ndarray = field(repr=False, default=None)
    b3: np.ndarray = field(repr=False, default=None)

    def param(self, block, name, default=None):
        """The value of <block>/name in the parameter dump (a string), or default."""
        cur = None
        for line in self.params.splitlines():
            line = line.split("#", 1)[0].strip()
            m = re.match(r"<(.+)>", line)
            if m:
                cur = m.group(1).strip()
                continue
            if cur == block and "=" in line:
                k, v = line.split("=", 1)
                if k.strip() == name:
                    return v.strip()
        return default


def block_shapes(nx, ng):
    """Array shapes of one block: U, x1f, x2f, x3f for interior sizes nx (nx1, nx2, nx3)."""
    c1, c2, c3 = (n + 2 * ng for n in nx)
    return (5, c3, c2, c1), (c3, c2, c1 + 1), (c3, c2 + 1, c1), (c3 + 1, c2, c1)


def read(path, nx_block, ng):
    """Read a restart file written by the reference (or by ``write``); nx_block: the
    MeshBlock size (meshblock/nx1..3), ng: NGHOST."""
    data = open(path, "rb").read()
    end = data.index(b"<par_end>")
    end = data.index(b"\n", end) + 1
    params = data[:end].decode()
    off = end
    nbtotal, root_level = _HDR.unpack_from(data, off)
    off += _HDR.size
    mesh_size = _REGION.unpack_from(data, off)
    off += _REGION.size
    time, dt, ncycle, datasize = _TAIL.unpack_from(data, off)
    off += _TAIL.size
    locs, costs = [], []
    for _ in range(nbtotal):
        lx1, lx2, lx3, level = _LOC.unpack_from(data, off)
        off += _LOC.size
        (cost,) = struct.unpack_from("<d", data, off)
        off += 8
        locs.append((level, lx1, lx2, lx3))
        costs.append(cost)
    shapes = block_shapes(nx_block, ng)
    need = sum(int(np.prod(s)) for s in shapes) * 8
    if need != datasize:
        raise ValueError("restart block size %d differs from U + B of this mesh (%d): "
                         "passive scalars or user data are not supported" % (datasize, need))
    arrs = [np.zeros((nbtotal,) + s) for s in shapes]
    for b in range(nbtotal):
        p = off + b * datasize
        for a, s in zip(arrs, shapes):
            n = int(np.prod(s))
            a[b] = np.frombuffer(data, dtype="<f8", count=n, offset=p).reshape(s)
            p += 8 * n
    return Restart(params, nbtotal, root_level, tuple(mesh_size), time, dt, ncycle, locs,
                   np.array(costs), *arrs)


def write(path, r: Restart):
    """Write a Restart in the reference's format (the padding bytes are zero)."""
    shapes = [a.shape[1:] for a in (r.u, r.b1, r.b2, r.b3)]
    datasize = sum(int(np.prod(s)) for s in shapes) * 8
    params = r.params if r.params.endswith("\n") else r.params + "\n"
    if "<par_end>" not in params:
        raise ValueError("the parameter dump must end with <par_end>")
    with open(path, "wb") as f:
        f.write(params.encode())
        f.write(_HDR.pack(r.nbtotal, r.root_level))
        f.write(_REGION.pack(*r.mesh_size))
        f.write(_TAIL.pack(r.time, r.dt, r.ncycle, datasize))
        costs = r.costs if r.costs is not None else np.zeros(r.nbtotal)
        for (level, lx1, lx2, lx3), c in zip(r.locs, costs):
            f.write(_LOC.pack(lx1, lx2, lx3, level))
            f.write(struct.pack("<d", float(c)))
        for b in range(r.nbtotal):
            for a in (r.u, r.b1, r.b2, r.b3):
                f.write(np.ascontiguousarray(a[b], dtype="<f8").tobytes())


def parameter_dump(blocks):
    """A parameter dump (ParameterDump's layout) from [(block, [(name, value), ...])]."""
    out = ["#------------------------- PAR_DUMP -------------------------"]
    for blk, items in blocks:
        out.append("<%s>" % blk)
        if not items:
            continue
        wn = max(len(k) for k, _ in items)
        wv = max(len(str(v)) for _, v in items)
        for k, v in items:
            out.append("%s= %s" % (k.ljust(wn + 1), str(v).ljust(wv + 1)))
    out.append("#------------------------- PAR_DUMP -------------------------")
    out.append("<par_end>")
    return "\n".join(out) + "\n"


# ---- meshes of this package <-> the reference's block order ------------------------------
def _is_multilevel(mesh):
    return hasattr(mesh, "neighbor_table")


def reference_order(mesh):
    """[(our block index, (level, lx1, lx2, lx3))] in the reference's gid order: a
    MultiLevelMesh already lists its blocks so; a uniform MeshSpec (lexicographic order)
    is reordered by the block tree of its root grid (MeshBlockTree::GetMeshBlockList)."""
    if _is_multilevel(mesh):
        return [(b, (l.level, l.lx1, l.lx2, l.lx3)) for b, l in enumerate(mesh.locs)]
    from .meshtree import MeshTree
    t = MeshTree(mesh.nb)
    nb1, nb2 = mesh.nb[0], mesh.nb[1]
    return [((l.lx3 * nb2 + l.lx2) * nb1 + l.lx1, (l.level, l.lx1, l.lx2, l.lx3))
            for l in t.block_list()]


def make(mesh, state, time, dt, ncycle, params, costs=None):
    """A Restart of ``mesh`` from state = (u, b1, b2, b3) in this package's block order."""
    order = reference_order(mesh)
    idx = [b for b, _ in order]
    u, b1, b2, b3 = (np.asarray(a)[idx] for a in state)
    if _is_multilevel(mesh):
        root_level = mesh.tree.root_level
        nx = mesh.nx
    else:
        from .meshtree import MeshTree
        root_level = MeshTree(mesh.nb).root_level
        nx = mesh.nx
    size = tuple(mesh.xmin) + tuple(mesh.xmax) + (1.0, 1.0, 1.0) + tuple(int(v) for v in nx)
    return Restart(params, len(order), root_level, size, float(time), float(dt), int(ncycle),
                   [loc for _, loc in order],
                   np.ones(len(order)) if costs is None else np.asarray(costs), u, b1, b2, b3)


def state(r, mesh):
    """(u, b1, b2, b3) of a Restart in ``mesh``'s block order (the mesh must hold the same
    blocks)."""
    order = reference_order(mesh)
    if sorted(loc for _, loc in order) != sorted(r.locs):
        raise ValueError("the restart file's blocks differ from the mesh's")
    pos = {loc: n for n, loc in enumerate(r.locs)}
    out = [np.zeros_like(a) for a in (r.u, r.b1, r.b2, r.b3)]
    for b, loc in order:
        for o, a in zip(out, (r.u, r.b1, r.b2, r.b3)):
            o[b] = a[pos[loc]]
    return tuple(out)


def save(path, stage_update, ncycle, params, costs=None):
    """Write a restart file of a StageUpdate (or AdaptiveStageUpdate): the state with
    ghost zones, the clock and the block list."""
    from .runtime import COPY_WHOLE
    su = getattr(stage_update, "su", stage_update)   # AdaptiveStageUpdate wraps one
    extent = getattr(su, "copy_extent", COPY_WHOLE)
    if extent != COPY_WHOLE:   # the file holds whole arrays
        su.set_copy_extent(COPY_WHOLE)
    try:
        st = stage_update.state()
    finally:
        if extent != COPY_WHOLE:
            su.set_copy_extent(extent)
    time, dt = stage_update.clock()
    write(path, make(stage_update.mesh, st, time, dt, ncycle, params, costs))


def load(path, stage_update):
    """Restore a StageUpdate from a restart file and make Mesh::Initialize(1)'s first
    time step from the stored dt; returns the Restart (ncycle, params, ...)."""
    m = stage_update.mesh
    r = read(path, m.bx, m.ng)
    stage_update.set_state(*state(r, m))
    stage_update.set_clock(r.time, r.dt)
    stage_update.initialize()
    return r
