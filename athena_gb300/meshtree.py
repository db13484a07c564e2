"""Multi-level MeshBlock tree, block list and neighbour lists (host side).

The stage update advances every MeshBlock of a mesh with refinement levels in one launch
per kernel; this module builds what those launches need, with the reference's semantics:

* the octree of logical locations (MeshBlockTree, mesh/meshblock_tree.cpp): the root
  grid of ``nrbx1 x nrbx2 x nrbx3`` blocks sits at logical level ``root_level`` (the
  smallest L with 2^L >= max nrbx, mesh.cpp:306); refining a leaf also refines every
  coarser neighbour so that adjacent blocks differ by at most one level
  (MeshBlockTree::Refine, meshblock_tree.cpp:166-258);
* the block order (the global id, gid): leaves in depth-first child order
  n = i + 2j + 4k (MeshBlockTree::GetMeshBlockList, meshblock_tree.cpp:336-355);
* static refinement regions (``<refinementN>`` blocks, mesh.cpp:340-484);
* per block the neighbour list in the reference's order, with buffer ids, finer-block
  offsets and the 3x3x3 neighbour-level table (BoundaryBase::SearchAndSetNeighbors,
  bvals/bvals_base.cpp:300-720; NeighborBlock::SetNeighbor, :43-68);
* per block the fine and coarse Cartesian coordinates (Mesh::SetBlockSizeAndBoundaries,
  mesh.cpp:1984-2060; Coordinates constructor, coordinates/coordinates.cpp:28-300 with
  the coarse_flag branch used for prolongation).

Only 3-D meshes are handled (nx2, nx3 > 1), as in the rest of the package.
"""
from dataclasses import dataclass, field

import numpy as np

from .mesh import _gen_x, _uniform_gen

FACE, EDGE, CORNER = 0, 1, 2


@dataclass(frozen=True)
class Loc:
    level: int
    lx1: int
    lx2: int
    lx3: int


class _Node:
    __slots__ = ("loc", "leaf", "gid")

    def __init__(self, loc, gid=-1):
        self.loc = loc
        self.leaf = None      # list of 8 children (None entries outside the root grid)
        self.gid = gid

    def child(self, ox, oy, oz):
        return self.leaf[ox + (oy << 1) + (oz << 2)]


@dataclass
class Neighbor:
    """One entry of a block's neighbour list (NeighborBlock)."""
    gid: int
    level: int
    ox1: int
    ox2: int
    ox3: int
    type: int
    bufid: int
    fi1: int = 0
    fi2: int = 0
    fid: int = -1   # BoundaryFace index of a face neighbour
    eid: int = -1   # edge index of an edge neighbour (0-3 x1x2, 4-7 x1x3, 8-11 x2x3)


class MeshTree:
    """The block octree of one mesh.

    ``nrbx``: root-grid blocks per direction; ``bcs``: six mesh-face flags (0 periodic,
    1 outflow, 2 reflecting)."""

    def __init__(self, nrbx, bcs=(0, 0, 0, 0, 0, 0)):
        self.nrbx = tuple(int(v) for v in nrbx)
        self.bcs = tuple(int(v) for v in bcs)
        nbmax = max(self.nrbx)
        self.root_level = 0
        while (1 << self.root_level) < nbmax:
            self.root_level += 1
        self.root = _Node(Loc(0, 0, 0, 0))
        self._create_root(self.root)
        self.nnew = self.ndel = 0   # blocks made and removed (Refine's nnew, Derefine's ndel)

    # --- construction (meshblock_tree.cpp:87-258) ----------------------------------
    def _create_root(self, node):
        if node.loc.level == self.root_level:
            return
        node.leaf = [None] * 8
        levfac = 1 << (self.root_level - node.loc.level - 1)
        for n in range(8):
            i, j, k = n & 1, (n >> 1) & 1, (n >> 2) & 1
            if ((node.loc.lx3 * 2 + k) * levfac < self.nrbx[2]
                    and (node.loc.lx2 * 2 + j) * levfac < self.nrbx[1]
                    and (node.loc.lx1 * 2 + i) * levfac < self.nrbx[0]):
                c = _Node(self._child_loc(node.loc, i, j, k))
                node.leaf[n] = c
                self._create_root(c)

    @staticmethod
    def _child_loc(loc, i, j, k):
        return Loc(loc.level + 1, (loc.lx1 << 1) + i, (loc.lx2 << 1) + j, (loc.lx3 << 1) + k)

    def nblocks_at(self, d, level):
        return self.nrbx[d] << (level - self.root_level)

    def add_block(self, rloc):
        """AddMeshBlock: make rloc a leaf, refining (and balancing) on the way."""
        self._add(self.root, rloc)

    def _add(self, node, rloc):
        if node.loc.level == rloc.level:
            return
        if node.leaf is None:
            self._refine(node)
        sh = rloc.level - node.loc.level - 1
        n = ((rloc.lx1 >> sh) & 1) + (((rloc.lx2 >> sh) & 1) << 1) + \
            (((rloc.lx3 >> sh) & 1) << 2)
        self._add(node.leaf[n], rloc)

    def refine(self, node):
        """MeshBlockTree::Refine (meshblock_tree.cpp:166-258): split a leaf and refine every
        coarser neighbour so that adjacent blocks differ by at most one level."""
        self._refine(node)

    def _refine(self, node):
        if node.leaf is not None:
            return
        self.nnew += 7
        # the children inherit the parent's gid (meshblock_tree.cpp:62), which maps the new
        # blocks back to the old block they were refined from
        node.leaf = [_Node(self._child_loc(node.loc, n & 1, (n >> 1) & 1, (n >> 2) & 1),
                           node.gid) for n in range(8)]
        lev = node.loc.level
        nmax = [self.nrbx[d] << (lev - self.root_level) for d in range(3)]
        for oz in (-1, 0, 1):
            lz = node.loc.lx3 + oz
            if lz < 0:
                if self.bcs[4] != 0:
                    continue
                lz = nmax[2] - 1
            if lz >= nmax[2]:
                if self.bcs[5] != 0:
                    continue
                lz = 0
            for oy in (-1, 0, 1):
                ly = node.loc.lx2 + oy
                if ly < 0:
                    if self.bcs[2] != 0:
                        continue
                    ly = nmax[1] - 1
                if ly >= nmax[1]:
                    if self.bcs[3] != 0:
                        continue
                    ly = 0
                for ox in (-1, 0, 1):
                    if ox == 0 and oy == 0 and oz == 0:
                        continue
                    lx = node.loc.lx1 + ox
                    if lx < 0:
                        if self.bcs[0] != 0:
                            continue
                        lx = nmax[0] - 1
                    if lx >= nmax[0]:
                        if self.bcs[1] != 0:
                            continue
                        lx = 0
                    self._add(self.root, Loc(lev, lx, ly, lz))
        node.gid = -1

    def derefine_ok(self, node):
        """MeshBlockTree::Derefine's test (meshblock_tree.cpp:261-305): no neighbour of
        the node (at its level) has children that are themselves refined on the side
        facing it."""
        for ox3 in (-1, 0, 1):
            for ox2 in (-1, 0, 1):
                for ox1 in (-1, 0, 1):
                    bt = self.find_neighbor(node.loc, ox1, ox2, ox3, amrflag=True)
                    if bt is None or bt.leaf is None:
                        continue
                    rng = [(1, 1) if o == -1 else (0, 0) if o == 1 else (0, 1)
                           for o in (ox1, ox2, ox3)]
                    for lk in range(rng[2][0], rng[2][1] + 1):
                        for lj in range(rng[1][0], rng[1][1] + 1):
                            for li in range(rng[0][0], rng[0][1] + 1):
                                if bt.leaf[li + (lj << 1) + (lk << 2)].leaf is not None:
                                    return False
        return True

    def derefine(self, node):
        """Make a refined node a leaf again (it inherits its first child's gid)."""
        node.gid = node.leaf[0].gid
        node.leaf = None
        self.ndel += 7

    # --- queries (meshblock_tree.cpp:317-487) --------------------------------------
    def block_list(self, old_gids=None):
        """Leaves in gid order; also stores each leaf's gid.  ``old_gids`` (a list) receives
        each leaf's previous gid: the block it was refined from, the first child it was
        derefined from, or itself (GetMeshBlockList's pglist, meshblock_tree.cpp:336-352)."""
        out = []

        def walk(node):
            if node.leaf is None:
                if old_gids is not None:
                    old_gids.append(node.gid)
                node.gid = len(out)
                out.append(node.loc)
            else:
                for c in node.leaf:
                    if c is not None:
                        walk(c)
        walk(self.root)
        return out

    def find(self, loc):
        node = self.root
        while node.loc.level != loc.level:
            if node.leaf is None:
                return None
            sh = loc.level - node.loc.level - 1
            n = ((loc.lx1 >> sh) & 1) + (((loc.lx2 >> sh) & 1) << 1) + \
                (((loc.lx3 >> sh) & 1) << 2)
            node = node.leaf[n]
            if node is None:
                return None
        return node

    def find_neighbor(self, loc, ox1, ox2, ox3, amrflag=False):
        """The neighbouring tree node in direction (ox1, ox2, ox3): the leaf at the same
        or a coarser level, or, when the neighbour is finer, its parent (which has
        children).  None across a physical mesh face."""
        ll = loc.level
        l = [loc.lx1 + ox1, loc.lx2 + ox2, loc.lx3 + ox3]
        for d in range(3):
            n = self.nblocks_at(d, ll)
            if l[d] < 0:
                if self.bcs[2 * d] != 0:
                    return None
                l[d] = n - 1
            if l[d] >= n:
                if self.bcs[2 * d + 1] != 0:
                    return None
                l[d] = 0
        if ll < 1:
            return self.root
        bt = self.root
        for level in range(ll):
            if bt.leaf is None:
                if level == ll - 1:
                    return bt
                raise RuntimeError("neighbour search failed: the block tree is broken")
            sh = ll - level - 1
            bt = bt.child((l[0] >> sh) & 1, (l[1] >> sh) & 1, (l[2] >> sh) & 1)
            if bt is None:
                raise RuntimeError("neighbour search failed: the block tree is broken")
        if bt.leaf is None:
            return bt
        fl = bt.child(1 if ox1 < 0 else 0, 1 if ox2 < 0 else 0, 1 if ox3 < 0 else 0)
        if fl.leaf is None or amrflag:
            return bt
        raise RuntimeError("neighbour search failed: the block tree is broken")

    # --- neighbour lists (bvals_base.cpp:300-720, 3-D) -----------------------------
    def neighbors(self, loc):
        """(list of Neighbor in the reference's order, nblevel[3][3][3])."""
        nb = []
        nblevel = np.full((3, 3, 3), -1, dtype=np.int64)
        nblevel[1, 1, 1] = loc.level
        myfx = [loc.lx1 & 1, loc.lx2 & 1, loc.lx3 & 1]
        myox = [2 * f - 1 for f in myfx]
        bufid = 0
        # faces: x1, x2, x3; n = -1, +1
        for d in range(3):
            for n in (-1, 1):
                o = [0, 0, 0]
                o[d] = n
                bt = self.find_neighbor(loc, *o)
                if bt is None:
                    bufid += 4
                    continue
                idx = (o[2] + 1, o[1] + 1, o[0] + 1)
                fid = 2 * d + (1 if n > 0 else 0)
                if bt.leaf is not None:   # finer
                    nblevel[idx] = bt.loc.level + 1
                    fface = 1 - (n + 1) // 2
                    for f2 in (0, 1):
                        for f1 in (0, 1):
                            c = [f1, f2]
                            c.insert(d, fface)
                            leaf = bt.child(*c)
                            nb.append(Neighbor(leaf.gid, leaf.loc.level, *o, FACE, bufid,
                                               f1, f2, fid=fid))
                            bufid += 1
                else:
                    nblevel[idx] = bt.loc.level
                    nb.append(Neighbor(bt.gid, bt.loc.level, *o, FACE, bufid, fid=fid))
                    bufid += 4
        # edges: x1x2 (o3 = 0), x1x3 (o2 = 0), x2x3 (o1 = 0); outer loop m over the
        # second axis, inner n over the first
        for (a, b) in ((0, 1), (0, 2), (1, 2)):
            for m in (-1, 1):
                for n in (-1, 1):
                    o = [0, 0, 0]
                    o[a], o[b] = n, m
                    bt = self.find_neighbor(loc, *o)
                    if bt is None:
                        bufid += 2
                        continue
                    idx = (o[2] + 1, o[1] + 1, o[0] + 1)
                    eid = {(0, 1): 0, (0, 2): 4, (1, 2): 8}[(a, b)] + \
                        (((n + 1) >> 1) | ((m + 1) & 2))
                    if bt.leaf is not None:
                        nblevel[idx] = bt.loc.level + 1
                        ff1, ff2 = 1 - (n + 1) // 2, 1 - (m + 1) // 2
                        for f1 in (0, 1):
                            c = [0, 0, 0]
                            c[a], c[b] = ff1, ff2
                            c[3 - a - b] = f1
                            leaf = bt.child(*c)
                            nb.append(Neighbor(leaf.gid, leaf.loc.level, *o, EDGE, bufid,
                                               f1, 0, eid=eid))
                            bufid += 1
                    else:
                        nblevel[idx] = bt.loc.level
                        if bt.loc.level >= loc.level or (myox[a] == n and myox[b] == m):
                            nb.append(Neighbor(bt.gid, bt.loc.level, *o, EDGE, bufid,
                                               eid=eid))
                        bufid += 2
        # corners
        for l in (-1, 1):
            for m in (-1, 1):
                for n in (-1, 1):
                    bt = self.find_neighbor(loc, n, m, l)
                    if bt is None:
                        bufid += 1
                        continue
                    if bt.leaf is not None:
                        bt = bt.child(1 - (n + 1) // 2, 1 - (m + 1) // 2, 1 - (l + 1) // 2)
                    nblevel[l + 1, m + 1, n + 1] = bt.loc.level
                    if bt.loc.level >= loc.level or \
                            (myox[0] == n and myox[1] == m and myox[2] == l):
                        nb.append(Neighbor(bt.gid, bt.loc.level, n, m, l, CORNER, bufid))
                    bufid += 1
        return nb, nblevel


def refinement_region_locs(tree, mesh_min, mesh_max, nx_mesh, reg_min, reg_max, ref_lev):
    """Logical locations that a <refinementN> region adds at level ref_lev above the root
    (mesh.cpp:340-484, uniform generator): pairs of blocks covering [reg_min, reg_max]."""
    lrlev = ref_lev + tree.root_level
    rng = []
    for d in range(3):
        lxmax = tree.nrbx[d] * (1 << ref_lev)
        lo = 0
        while lo < lxmax:
            if _uniform_gen(_gen_x(lo + 1, lxmax), mesh_min[d], mesh_max[d]) > reg_min[d]:
                break
            lo += 1
        hi = lo
        while hi < lxmax:
            if _uniform_gen(_gen_x(hi + 1, lxmax), mesh_min[d], mesh_max[d]) >= reg_max[d]:
                break
            hi += 1
        if lo % 2 == 1:
            lo -= 1
        if hi % 2 == 0:
            hi += 1
        rng.append((lo, hi))
    out = []
    for k in range(rng[2][0], rng[2][1], 2):
        for j in range(rng[1][0], rng[1][1], 2):
            for i in range(rng[0][0], rng[0][1], 2):
                out.append(Loc(lrlev, i, j, k))
    return out


class MultiLevelMesh:
    """A mesh of equal-size MeshBlocks on several refinement levels.

    The interface follows ``mesh.MeshSpec`` (per-block array shapes, coordinate arrays,
    ``interior``) and adds the levels, the neighbour lists and the coarse-buffer
    coordinates that prolongation and restriction use."""

    def __init__(self, nx, nrbx, ng, xmin=(0.0, 0.0, 0.0), xmax=(1.0, 1.0, 1.0),
                 bcs=(0, 0, 0, 0, 0, 0), regions=(), tree=None):
        self.nx = tuple(int(v) for v in nx)          # root-level cells of the mesh
        self.nrbx = tuple(int(v) for v in nrbx)
        self.ng = int(ng)
        self.xmin, self.xmax = tuple(xmin), tuple(xmax)
        self.bcs = tuple(int(v) for v in bcs)
        for d in range(3):
            if self.nx[d] % self.nrbx[d]:
                raise ValueError("mesh size not divisible by the root grid")
        self.bx = tuple(self.nx[d] // self.nrbx[d] for d in range(3))
        if any(b % 2 for b in self.bx):
            raise ValueError("MeshBlock sizes must be even for mesh refinement")
        if self.ng % 2:
            raise ValueError("mesh refinement needs an even number of ghost cells")
        self.nc = tuple(self.bx[d] + 2 * self.ng for d in range(3))
        self.cng = (self.ng + 1) // 2 + 1            # meshblock.cpp:93
        self.ncc = tuple(self.bx[d] // 2 + 2 * self.ng for d in range(3))
        self.tree = tree if tree is not None else MeshTree(self.nrbx, self.bcs)
        for (rmin, rmax, lev) in regions:
            for loc in refinement_region_locs(self.tree, self.xmin, self.xmax, self.nx,
                                              rmin, rmax, lev):
                self.tree.add_block(loc)
        self.rebuild()

    def rebuild(self):
        """Recompute the block list, neighbour lists and coordinates from the tree."""
        old = []
        self.locs = self.tree.block_list(old)
        self.old_gids = np.array(old, dtype=np.int32)
        self.nblocks = len(self.locs)
        self.levels = np.array([l.level for l in self.locs], dtype=np.int32)
        self._nblev = None
        self.nbrs, self.nblevels = [], []
        for loc in self.locs:
            nb, lv = self.tree.neighbors(loc)
            self.nbrs.append(nb)
            self.nblevels.append(lv)

    def nblevel_array(self):
        """The neighbour levels as an int32 array [nblocks][27]."""
        if getattr(self, "_nblev", None) is None or len(self._nblev) != self.nblocks:
            self._nblev = np.array([np.asarray(v).ravel() for v in self.nblevels],
                                   dtype=np.int32).reshape(self.nblocks, 27)
        return self._nblev

    # --- array shapes ----------------------------------------------------------------
    @property
    def cell_shape(self):
        return (self.nc[2], self.nc[1], self.nc[0])

    @property
    def face_shapes(self):
        c1, c2, c3 = self.nc
        return ((c3, c2, c1 + 1), (c3, c2 + 1, c1), (c3 + 1, c2, c1))

    def interior(self, blocks):
        ng, (b1, b2, b3) = self.ng, self.bx
        return blocks[:, :, ng:ng + b3, ng:ng + b2, ng:ng + b1]

    def interior_faces(self, b):
        ng = self.ng
        return b[:, ng:-ng, ng:-ng, ng:-ng]

    # --- coordinates -----------------------------------------------------------------
    def _lx(self, b, d):
        loc = self.locs[b]
        return (loc.lx1, loc.lx2, loc.lx3)[d]

    def block_bounds(self, b, d):
        """block_size.x?min/x?max (Mesh::SetBlockSizeAndBoundaries, mesh.cpp:1984-2060)."""
        lev, lx = self.locs[b].level, self._lx(b, d)
        n = self.nrbx[d] << (lev - self.tree.root_level)
        lo = self.xmin[d] if lx == 0 else _uniform_gen(_gen_x(lx, n), self.xmin[d],
                                                       self.xmax[d])
        hi = self.xmax[d] if lx == n - 1 else _uniform_gen(_gen_x(lx + 1, n), self.xmin[d],
                                                           self.xmax[d])
        return lo, hi

    def _faces(self, b, d, coarse):
        """x?f, dx?f of block b (coarse=True: the coarse buffer's, coordinates.cpp
        coarse_flag branch), with the reflecting-boundary ghost correction
        (coordinates.cpp:148-161)."""
        lev, lx = self.locs[b].level, self._lx(b, d)
        n, ng = self.bx[d], self.ng
        nint = n // 2 if coarse else n
        nc = nint + 2 * ng
        il, iu = ng, ng + nint - 1
        lo, hi = self.block_bounds(b, d)
        nroot = self.nx[d] << (lev - self.tree.root_level)
        xf = np.empty(nc + 1)
        for i in range(nc + 1):
            off = (i - il) * 2 + lx * n if coarse else i - il + lx * n
            xf[i] = _uniform_gen(_gen_x(off, nroot), self.xmin[d], self.xmax[d])
        xf[il] = lo
        xf[iu + 1] = hi
        dx = (hi - lo) / (iu - il + 1)
        dxf = np.full(nc, dx)
        nlev = self.nrbx[d] << (lev - self.tree.root_level)
        if lx == 0 and self.bcs[2 * d] == 2:
            for g in range(1, ng + 1):
                dxf[il - g] = dxf[il + g - 1]
                xf[il - g] = xf[il - g + 1] - dxf[il - g]
        if lx == nlev - 1 and self.bcs[2 * d + 1] == 2:
            for g in range(1, ng + 1):
                dxf[iu + g] = dxf[iu - g + 1]
                xf[iu + g + 1] = xf[iu + g] + dxf[iu + g]
        return xf, dxf

    def coordinate_arrays(self):
        """Per-block (x1f, dx1f, x2f, dx2f, x3f, dx3f) stacked over blocks."""
        out = []
        for d in range(3):
            xf = np.empty((self.nblocks, self.nc[d] + 1))
            dxf = np.empty((self.nblocks, self.nc[d]))
            for b in range(self.nblocks):
                xf[b], dxf[b] = self._faces(b, d, False)
            out += [xf, dxf]
        return out

    def coarse_coordinate_arrays(self):
        """Per-block coarse-buffer (x1f, dx1f, x2f, dx2f, x3f, dx3f)."""
        out = []
        for d in range(3):
            xf = np.empty((self.nblocks, self.ncc[d] + 1))
            dxf = np.empty((self.nblocks, self.ncc[d]))
            for b in range(self.nblocks):
                xf[b], dxf[b] = self._faces(b, d, True)
            out += [xf, dxf]
        return out

    def cell_centers(self, b, d, coarse=False):
        xf, _ = self._faces(b, d, coarse)
        return 0.5 * (xf[1:] + xf[:-1])   # cartesian.cpp:26-28

    # --- neighbour table for the C code ---------------------------------------------
    NBR_FIELDS = 10   # gid, level, ox1, ox2, ox3, type, fi1, fi2, fid, eid
    MAX_NBR = 56

    def neighbor_table(self):
        """(table[nb][MAX_NBR][NBR_FIELDS] int32, counts[nb] int32,
        nblevel[nb][27] int32, loc[nb][4] int64 (level, lx1, lx2, lx3))."""
        t = np.full((self.nblocks, self.MAX_NBR, self.NBR_FIELDS), -1, dtype=np.int32)
        cnt = np.zeros(self.nblocks, dtype=np.int32)
        lv = np.zeros((self.nblocks, 27), dtype=np.int32)
        loc = np.zeros((self.nblocks, 4), dtype=np.int64)
        for b, (nbs, nbl) in enumerate(zip(self.nbrs, self.nblevels)):
            cnt[b] = len(nbs)
            for n, e in enumerate(nbs):
                t[b, n] = (e.gid, e.level, e.ox1, e.ox2, e.ox3, e.type, e.fi1, e.fi2,
                           e.fid, e.eid)
            lv[b] = nbl.ravel()
            l = self.locs[b]
            loc[b] = (l.level, l.lx1, l.lx2, l.lx3)
        return t, cnt, lv, loc
