"""Adaptive mesh refinement, host side (Mesh::LoadBalancingAndAdaptiveMeshRefinement on
one rank, mesh/amr_loadbalance.cpp:40-60).

After the last stage of a cycle every MeshBlock evaluates the refinement condition on its
primitives (on the device: ``athgpu_refinement_eps``); this module turns the per-block
results into refinement flags (MeshRefinement::CheckRefinementCondition,
mesh/mesh_refinement.cpp:1393-1455), updates the block tree
(Mesh::UpdateMeshBlockTree, amr_loadbalance.cpp:178-317) and describes the
redistribution the device carries out (Mesh::RedistributeAndRefineMeshBlocks,
amr_loadbalance.cpp:351-660): for each new block the old block it comes from and how
(kept, restricted from eight children, prolongated from its parent), and the face-field
corrections a new child takes from old same-level neighbours
(PrepareAndSendFaceFieldCorrection, amr_loadbalance.cpp:1225-1340).
"""
from dataclasses import dataclass

import numpy as np

from .meshtree import Loc, MultiLevelMesh

SAME, F2C, C2F = 0, 1, 2   # how a new block is formed from the old mesh
NLEAF = 8                  # children of a refined block (3-D)


def blast_condition(maxeps, thr):
    """RefinementCondition of the blast problem (pgen/blast.cpp:413-443) from each block's
    maximum of |grad p|/p (centred differences over the interior and one ghost layer):
    1 (refine) above thr, -1 (derefine) below thr/4, else 0."""
    maxeps = np.asarray(maxeps, dtype=np.float64)
    ret = np.zeros(maxeps.shape[0], dtype=np.int32)
    ret[maxeps < 0.25 * thr] = -1
    ret[maxeps > thr] = 1
    return ret


@dataclass
class RegridPlan:
    """The redistribution of one tree update."""
    mesh: MultiLevelMesh       # the new mesh (block list, neighbours, coordinates)
    newtoold: np.ndarray       # int32[nnew]: old block of each new block
    kind: np.ndarray           # int32[nnew]: SAME, F2C (from newtoold..+7) or C2F
    ffc: np.ndarray            # int32[nffc, 3]: (new block, receiving face, old block)
    deref_count: np.ndarray    # int32[nnew]: the derefinement counters carried over


class AdaptiveMesh:
    """Refinement state of an adaptive mesh: the mesh, its maximum level and each block's
    derefinement counter (MeshRefinement::deref_count_)."""

    def __init__(self, mesh: MultiLevelMesh, numlevel, derefine_count=10):
        self.mesh = mesh
        self.max_level = mesh.tree.root_level + int(numlevel) - 1   # mesh.cpp:323
        self.derefine_count = int(derefine_count)                   # mesh_refinement.cpp:37
        self.deref_count = np.zeros(mesh.nblocks, dtype=np.int32)

    def check_refinement(self, ret):
        """MeshRefinement::CheckRefinementCondition for every block, from the condition's
        results ret[b] in {1, 0, -1}; updates the derefinement counters and returns the
        refine flags (1 refine, -1 derefine, 0 keep)."""
        m = self.mesh
        root = m.tree.root_level
        aret = np.maximum(np.asarray(ret, dtype=np.int32), -1)
        level = m.levels
        dc = self.deref_count
        dc[aret >= 0] = 0
        flags = np.zeros(m.nblocks, dtype=np.int32)
        flags[(aret > 0) & (level != self.max_level)] = 1
        neg = aret < 0
        dc[neg & (level == root)] = 0
        der = neg & (level != root)
        dc[der] += 1
        # no derefinement next to a finer block
        finer = (m.nblevel_array() > level[:, None]).any(axis=1)
        flags[der & ~finer & (dc >= self.derefine_count)] = -1
        return flags

    def update(self, flags):
        """Mesh::UpdateMeshBlockTree and the maps of RedistributeAndRefineMeshBlocks.
        Returns None when the tree did not change, else a RegridPlan (the tree is
        modified in place; call accept() once the data has been moved)."""
        m = self.mesh
        tree = m.tree
        lref = [m.locs[b] for b in range(m.nblocks) if flags[b] == 1]
        lderef = [m.locs[b] for b in range(m.nblocks) if flags[b] == -1]
        if not lref and len(lderef) < NLEAF:
            return None
        # groups of eight flagged siblings, in gid order (amr_loadbalance.cpp:255-283)
        clderef = []
        if len(lderef) >= NLEAF:
            t = len(lderef)
            for n, L in enumerate(lderef):
                if (L.lx1 & 1) or (L.lx2 & 1) or (L.lx3 & 1):
                    continue
                r, rr = n, 0
                for k in range(2):
                    for j in range(2):
                        for i in range(2):
                            if r < t:
                                R = lderef[r]
                                if (L.lx1 + i == R.lx1 and L.lx2 + j == R.lx2
                                        and L.lx3 + k == R.lx3 and L.level == R.level):
                                    rr += 1
                                r += 1
                if rr == NLEAF:
                    clderef.append(Loc(L.level - 1, L.lx1 >> 1, L.lx2 >> 1, L.lx3 >> 1))
        # sorted by decreasing level; the reference's sort range stops one short of the
        # end, so the last group keeps its place (amr_loadbalance.cpp:286-287)
        if len(clderef) > 1:
            clderef = sorted(clderef[:-1], key=lambda l: -l.level) + clderef[-1:]
        tree.nnew = tree.ndel = 0
        for L in lref:                    # Step 1: refinement
            tree.refine(tree.find(L))
        for L in clderef:                 # Step 2: derefinement
            node = tree.find(L)
            if node.leaf is not None and tree.derefine_ok(node):
                tree.derefine(node)
        if tree.nnew == 0 and tree.ndel == 0:
            return None
        new = MultiLevelMesh(m.nx, m.nrbx, m.ng, m.xmin, m.xmax, m.bcs, tree=tree)
        newtoold = new.old_gids.astype(np.int32)
        kind = np.zeros(new.nblocks, dtype=np.int32)
        dcount = np.zeros(new.nblocks, dtype=np.int32)
        for n in range(new.nblocks):
            on = int(newtoold[n])
            ol, nl = m.locs[on].level, new.locs[n].level
            if nl == ol:
                kind[n] = SAME
                dcount[n] = self.deref_count[on]
            else:
                kind[n] = F2C if nl < ol else C2F
        ffc = self._face_field_corrections(new, newtoold, kind)
        return RegridPlan(new, newtoold, kind, ffc, dcount)

    def _face_field_corrections(self, new, newtoold, kind):
        """PrepareAndSendFaceFieldCorrection (amr_loadbalance.cpp:1225-1340): a child made
        by refinement takes its face field on each face it shares with its parent's
        boundary from an old block of the child's level across that face."""
        m = self.mesh
        root = m.tree.root_level
        old = {loc: i for i, loc in enumerate(m.locs) if loc.level > root}
        out = []
        for n in range(new.nblocks):
            if kind[n] != C2F:
                continue
            nl = new.locs[n]
            lx = [nl.lx1, nl.lx2, nl.lx3]
            for d in range(3):
                xf = lx[d] & 1
                f = list(lx)
                f[d] += 2 * xf - 1
                nmax = m.nrbx[d] << (nl.level - root)
                if f[d] < 0:
                    if m.bcs[2 * d] != 0:
                        continue
                    f[d] = nmax - 1
                elif f[d] >= nmax:
                    if m.bcs[2 * d + 1] != 0:
                        continue
                    f[d] = 0
                i = old.get(Loc(nl.level, f[0], f[1], f[2]))
                if i is not None:
                    out.append((n, 2 * d + xf, i))
        return np.array(out, dtype=np.int32).reshape(-1, 3)

    def accept(self, plan):
        self.mesh = plan.mesh
        self.deref_count = plan.deref_count.copy()
