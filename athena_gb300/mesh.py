"""Uniform MeshBlock decomposition and Cartesian coordinates.

Host-side geometry for the stage update.  A mesh of ``NX1 x NX2 x NX3`` cells is cut
into ``nbx1 x nbx2 x nbx3`` MeshBlocks of ``nx1 x nx2 x nx3`` interior cells with ``ng``
ghost layers, exactly as the reference lays out a single-level mesh:

* every block holds AthenaArray-layout arrays (last index fastest,
  athena_arrays.hpp:140-143), cells ``[nvar][nc3][nc2][nc1]`` with ``ncN = nxN + 2 ng``,
  face fields ``x1f [nc3][nc2][nc1+1]``, ``x2f [nc3][nc2+1][nc1]``,
  ``x3f [nc3+1][nc2][nc1]`` (athena.hpp:128-135);
* blocks are numbered lexicographically, ``b = (lx3*nbx2 + lx2)*nbx1 + lx1``;
* face coordinates follow the reference's uniform mesh generator
  (Mesh::SetBlockSizeAndBoundaries mesh.cpp:1984-2060, ComputeMeshGeneratorX
  mesh.hpp:457-472, UniformMeshGeneratorX1 mesh.hpp:535-538, Coordinates constructor
  coordinates.cpp:92-146), so that the coordinate arrays are bit-identical to the
  reference's.
"""
from dataclasses import dataclass

import numpy as np


def _gen_x(index, nrange):
    """ComputeMeshGeneratorX with sym_interval=true (mesh.hpp:457-472)."""
    noffset = index - nrange // 2
    noffset_ceil = index - (nrange + 1) // 2
    return float(noffset + noffset_ceil) / (2.0 * nrange)


def _uniform_gen(x, xmin, xmax):
    """UniformMeshGeneratorX1/2/3 (mesh.hpp:535-553)."""
    return 0.5 * (xmin + xmax) + (x * xmax - x * xmin)


@dataclass
class MeshSpec:
    nx: tuple            # cells of the whole mesh (NX1, NX2, NX3)
    nb: tuple            # MeshBlocks per direction (nbx1, nbx2, nbx3)
    ng: int              # ghost layers
    xmin: tuple = (0.0, 0.0, 0.0)
    xmax: tuple = (1.0, 1.0, 1.0)

    def __post_init__(self):
        self.nx = tuple(int(v) for v in self.nx)
        self.nb = tuple(int(v) for v in self.nb)
        for d in range(3):
            if self.nx[d] % self.nb[d]:
                raise ValueError("mesh size %d not divisible by %d blocks" %
                                 (self.nx[d], self.nb[d]))
        self.bx = tuple(self.nx[d] // self.nb[d] for d in range(3))  # cells per block
        self.nc = tuple(self.bx[d] + 2 * self.ng for d in range(3))
        self.nblocks = self.nb[0] * self.nb[1] * self.nb[2]

    # --- array shapes (per block, AthenaArray order: slowest first) -------------------
    @property
    def cell_shape(self):
        return (self.nc[2], self.nc[1], self.nc[0])

    @property
    def face_shapes(self):
        c1, c2, c3 = self.nc
        return ((c3, c2, c1 + 1), (c3, c2 + 1, c1), (c3 + 1, c2, c1))

    def block_loc(self, b):
        n1, n2, _ = self.nb
        return b % n1, (b // n1) % n2, b // (n1 * n2)

    # --- coordinates ----------------------------------------------------------------
    def block_bounds(self, d, l):
        """block_size.x?min/x?max of block l along direction d (mesh.cpp:1991-2006)."""
        nr = self.nb[d]
        lo = self.xmin[d] if l == 0 else _uniform_gen(_gen_x(l, nr), self.xmin[d],
                                                        self.xmax[d])
        hi = self.xmax[d] if l == nr - 1 else _uniform_gen(_gen_x(l + 1, nr), self.xmin[d],
                                                             self.xmax[d])
        return lo, hi

    def face_coords(self, d, l):
        """x?f (nc+1) and dx?f (nc) of block l along d (coordinates.cpp:126-146)."""
        n, ng, nc = self.bx[d], self.ng, self.nc[d]
        lo, hi = self.block_bounds(d, l)
        dx = (hi - lo) / n
        nroot = self.nx[d]
        xf = np.empty(nc + 1)
        for i in range(nc + 1):
            noffset = i - ng + l * n
            xf[i] = _uniform_gen(_gen_x(noffset, nroot), self.xmin[d], self.xmax[d])
        xf[ng] = lo
        xf[ng + n] = hi
        return xf, np.full(nc, dx)

    def coordinate_arrays(self):
        """Per-block (x1f, dx1f, x2f, dx2f, x3f, dx3f) stacked over blocks."""
        out = []
        for d in range(3):
            xf = np.empty((self.nblocks, self.nc[d] + 1))
            dxf = np.empty((self.nblocks, self.nc[d]))
            for b in range(self.nblocks):
                xf[b], dxf[b] = self.face_coords(d, self.block_loc(b)[d])
            out += [xf, dxf]
        return out

    def cell_centers(self, d, l):
        xf, _ = self.face_coords(d, l)
        return 0.5 * (xf[1:] + xf[:-1])   # x?v, cartesian.cpp:28-32

    # --- global <-> per-block arrays ---------------------------------------------------
    def scatter_cells(self, g):
        """g[nvar, NX3, NX2, NX1] -> blocks[nb, nvar, nc3, nc2, nc1] (interior only)."""
        nvar = g.shape[0]
        out = np.zeros((self.nblocks, nvar) + self.cell_shape, dtype=g.dtype)
        ng, (b1, b2, b3) = self.ng, self.bx
        for b in range(self.nblocks):
            l1, l2, l3 = self.block_loc(b)
            out[b, :, ng:ng + b3, ng:ng + b2, ng:ng + b1] = \
                g[:, l3 * b3:(l3 + 1) * b3, l2 * b2:(l2 + 1) * b2, l1 * b1:(l1 + 1) * b1]
        return out

    def gather_cells(self, blocks):
        nvar = blocks.shape[1]
        g = np.zeros((nvar, self.nx[2], self.nx[1], self.nx[0]), dtype=blocks.dtype)
        ng, (b1, b2, b3) = self.ng, self.bx
        for b in range(self.nblocks):
            l1, l2, l3 = self.block_loc(b)
            g[:, l3 * b3:(l3 + 1) * b3, l2 * b2:(l2 + 1) * b2, l1 * b1:(l1 + 1) * b1] = \
                blocks[b, :, ng:ng + b3, ng:ng + b2, ng:ng + b1]
        return g

    def scatter_faces(self, f1, f2, f3):
        """Global face arrays f1[NX3,NX2,NX1+1], f2[NX3,NX2+1,NX1], f3[NX3+1,NX2,NX1] ->
        per-block face arrays (each block's own faces, both bounding faces included)."""
        ng, (b1, b2, b3) = self.ng, self.bx
        o1 = np.zeros((self.nblocks,) + self.face_shapes[0])
        o2 = np.zeros((self.nblocks,) + self.face_shapes[1])
        o3 = np.zeros((self.nblocks,) + self.face_shapes[2])
        for b in range(self.nblocks):
            l1, l2, l3 = self.block_loc(b)
            k0, j0, i0 = l3 * b3, l2 * b2, l1 * b1
            o1[b, ng:ng + b3, ng:ng + b2, ng:ng + b1 + 1] = \
                f1[k0:k0 + b3, j0:j0 + b2, i0:i0 + b1 + 1]
            o2[b, ng:ng + b3, ng:ng + b2 + 1, ng:ng + b1] = \
                f2[k0:k0 + b3, j0:j0 + b2 + 1, i0:i0 + b1]
            o3[b, ng:ng + b3 + 1, ng:ng + b2, ng:ng + b1] = \
                f3[k0:k0 + b3 + 1, j0:j0 + b2, i0:i0 + b1]
        return o1, o2, o3

    def interior(self, blocks):
        """View of the interior cells of a [nb, nvar, nc3, nc2, nc1] array."""
        ng, (b1, b2, b3) = self.ng, self.bx
        return blocks[:, :, ng:ng + b3, ng:ng + b2, ng:ng + b1]
