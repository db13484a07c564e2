"""The adaptive main loop on the GPU: StageUpdate on a multi-level mesh whose block list
follows a refinement condition.

* ``AdaptiveStageUpdate.initialize`` is Mesh::Initialize with adaptive refinement
  (mesh.cpp:1622-1964): the problem generator on every block, the boundaries, the
  refinement flags and a regrid, repeated until the block count stops changing, then the
  first time step;
* ``cycle`` is one pass of the main loop (main.cpp:457-541): both stages, time += dt,
  the refinement measure of the last stage's primitives (time_integrator.cpp:2321-2326),
  LoadBalancingAndAdaptiveMeshRefinement (amr_loadbalance.cpp:40-60) and NewTimeStep.

The refinement measure is computed on the device (athgpu_refinement_eps), the flags and
the tree update on the host (athena_gb300.amr), the data movement on the device
(athgpu_regrid).
"""
import ctypes
import time
from types import SimpleNamespace

import numpy as np

from .amr import AdaptiveMesh, blast_condition
from .meshtree import Loc, MultiLevelMesh
from .runtime import StageUpdate, _check, _dp, load_library


class AdaptiveStageUpdate:
    """``ic(mesh) -> (u, b1, b2, b3)``: the problem generator; ``thr``: the threshold of the
    blast problem's refinement condition (or of ``condition(maxeps, thr)``, a refinement
    condition on the per-block measure, which runs the host side in Python); further
    keyword arguments go to StageUpdate.  ``native`` (default): the tree, the flags and the
    tree update run in the library (athgpu_amr_step), otherwise in athena_gb300.amr."""

    def __init__(self, mesh0, ic, numlevel, thr, derefine_count=10, condition=None,
                 native=True, **kw):
        self.ic, self.thr = ic, thr
        self.native = native and condition is None
        self.condition = condition or blast_condition
        self.regrids = 0
        self.t_refine = 0.0   # host seconds in the refinement steps (regrids included)
        self.regrid_ms = []   # milliseconds of each main-loop refinement step that regridded
        if self.native:
            self.namr = NativeAmr(mesh0.nx, mesh0.nrbx, mesh0.ng, mesh0.xmin, mesh0.xmax,
                                  mesh0.bcs, numlevel, derefine_count)
            root = mesh0.tree.root_level
            for loc in mesh0.locs:      # static refinement of the starting mesh
                if loc.level > root:
                    self.namr.add_block(loc)
            self._mesh = NativeMesh(self.namr)
            self.su = StageUpdate(self._mesh, **kw)
        else:
            self.amr = AdaptiveMesh(mesh0, numlevel, derefine_count)
            self.su = StageUpdate(mesh0, **kw)

    @property
    def mesh(self):
        return self._mesh if self.native else self.amr.mesh

    def _set_mesh(self, mesh):
        self._mesh = mesh
        self.su.mesh = mesh

    def _plan(self):
        """Flags and tree update from the current primitives: a regrid plan or None."""
        ret = self.condition(self.su.refinement_eps(), self.thr)
        if not self.native:
            return self.amr.update(self.amr.check_refinement(ret))
        if not self.namr.update(self.namr.flags(ret)):
            return None
        newtoold, kind, ffc, _ = self.namr.pending_maps()
        self.namr.accept()
        return SimpleNamespace(mesh=NativeMesh(self.namr), newtoold=newtoold, kind=kind,
                               ffc=ffc)

    def initialize(self):
        """Mesh::Initialize with adaptive refinement."""
        su = self.su
        while True:
            time0, dt0 = su.clock()
            su.set_state(*self.ic(self.mesh))
            su.initialize()
            plan = self._plan()
            if plan is None:
                # no change: this pass's time step is the one after the loop
                return
            # the loop itself makes no time step: that of initialize() is taken back
            su.set_clock(time0, dt0)
            onb = self.mesh.nblocks
            su.regrid(plan, after_cycle=False)
            if self.native:
                self._set_mesh(plan.mesh)
            else:
                self.amr.accept(plan)
            self.regrids += 1
            if self.mesh.nblocks == onb:
                su.new_time_step()
                return

    def cycle(self, n=1, after_stages=None):
        """n main-loop cycles; after_stages(self) is called after the stages and
        time += dt, before the regrid."""
        su = self.su
        for _ in range(n):
            su.cycle(1)
            if after_stages is not None:
                after_stages(self)
            su.synchronize()   # the step below synchronizes anyway: time only the step
            t0 = time.perf_counter()
            changed = False
            if self.native:
                if self.namr.step(su, self.thr, after_cycle=True):
                    self._set_mesh(NativeMesh(self.namr))
                    changed = True
            else:
                plan = self.amr.update(self.amr.check_refinement(
                    self.condition(su.refinement_eps(), self.thr)))
                if plan is not None:
                    su.regrid(plan, after_cycle=True)
                    self.amr.accept(plan)
                    su.new_time_step()
                    changed = True
            dt = time.perf_counter() - t0
            self.t_refine += dt
            if changed:
                self.regrids += 1
                self.regrid_ms.append(dt * 1e3)

    # the state accessors of StageUpdate
    def state(self):
        return self.su.state()

    def prim(self):
        return self.su.prim()

    def clock(self):
        return self.su.clock()

    @property
    def dt(self):
        return self.su.dt

    @property
    def time(self):
        return self.su.time

    def close(self):
        self.su.close()
        if self.native:
            self.namr.close()


# ---- the native host side (athgpu_amr_*) -------------------------------------------------
def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class NativeAmr:
    """An adaptive mesh whose tree, neighbour lists, coordinates, refinement flags and
    tree update live in the library (athgpu_amr_*)."""

    def __init__(self, nx, nrbx, ng, xmin, xmax, bcs, numlevel, derefine_count=10):
        L = load_library()
        self.nx, self.nrbx, self.ng = tuple(nx), tuple(nrbx), int(ng)
        self.xmin, self.xmax, self.bcs = tuple(xmin), tuple(xmax), tuple(bcs)
        h = ctypes.c_void_p()
        a3 = (ctypes.c_int * 3)
        d3 = (ctypes.c_double * 3)
        _check(L.athgpu_amr_create(ctypes.byref(h), a3(*self.nx), a3(*self.nrbx), self.ng,
                                   d3(*self.xmin), d3(*self.xmax),
                                   (ctypes.c_int * 6)(*self.bcs), int(numlevel),
                                   int(derefine_count)), "athgpu_amr_create")
        self.h = h
        self.generation = 0   # counts the mesh changes (NativeMesh's lazy tables check it)

    def close(self):
        if getattr(self, "h", None):
            load_library().athgpu_amr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def nblocks(self):
        n = ctypes.c_int()
        _check(load_library().athgpu_amr_nblocks(self.h, ctypes.byref(n)), "athgpu_amr_nblocks")
        return n.value

    def add_block(self, loc):
        _check(load_library().athgpu_amr_add_block(self.h, loc.level, loc.lx1, loc.lx2,
                                                   loc.lx3), "athgpu_amr_add_block")
        self.generation += 1

    def tables(self, coords=True, nbrs=True):
        """(loc[nb][4], nbr_table[nb][56][10], nbr_count[nb], nblevel[nb][27], fine
        coordinates (x1f, dx1f, ...), coarse coordinates) of the current mesh; without
        nbrs the three neighbour tables are None, without coords the coordinate lists
        are empty."""
        nb = self.nblocks
        bx = [self.nx[d] // self.nrbx[d] for d in range(3)]
        loc = np.zeros((nb, 4), dtype=np.int64)
        t = cnt = lv = None
        if nbrs:
            t = np.zeros((nb, 56, 10), dtype=np.int32)
            cnt = np.zeros(nb, dtype=np.int32)
            lv = np.zeros((nb, 27), dtype=np.int32)
        inull = ctypes.POINTER(ctypes.c_int)()
        fine, coarse = [], []
        if coords:
            for d in range(3):
                nc, ncc = bx[d] + 2 * self.ng, bx[d] // 2 + 2 * self.ng
                fine += [np.zeros((nb, nc + 1)), np.zeros((nb, nc))]
                coarse += [np.zeros((nb, ncc + 1)), np.zeros((nb, ncc))]
        null = ctypes.POINTER(ctypes.c_double)()
        ptrs = [_dp(a) for a in fine + coarse] if coords else [null] * 12
        _check(load_library().athgpu_amr_tables(
            self.h, loc.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
            *[(_ip(a) if a is not None else inull) for a in (t, cnt, lv)], *ptrs),
            "athgpu_amr_tables")
        return loc, t, cnt, lv, fine, coarse

    def flags(self, ret):
        ret = np.ascontiguousarray(ret, dtype=np.int32)
        out = np.zeros(ret.shape[0], dtype=np.int32)
        _check(load_library().athgpu_amr_flags(self.h, _ip(ret), _ip(out)), "athgpu_amr_flags")
        return out

    def update(self, flags):
        flags = np.ascontiguousarray(flags, dtype=np.int32)
        ch = ctypes.c_int()
        _check(load_library().athgpu_amr_update(self.h, _ip(flags), ctypes.byref(ch)),
               "athgpu_amr_update")
        return bool(ch.value)

    def pending_maps(self):
        """(newtoold, kind, ffc[nffc][3], derefinement counters) of the pending regrid."""
        L = load_library()
        nn, nf = ctypes.c_int(), ctypes.c_int()
        _check(L.athgpu_amr_pending(self.h, ctypes.byref(nn), ctypes.byref(nf)),
               "athgpu_amr_pending")
        newtoold = np.zeros(nn.value, dtype=np.int32)
        kind = np.zeros(nn.value, dtype=np.int32)
        ffc = np.zeros((nf.value, 3), dtype=np.int32)
        dc = np.zeros(nn.value, dtype=np.int32)
        _check(L.athgpu_amr_pending_maps(self.h, _ip(newtoold), _ip(kind), _ip(ffc), _ip(dc)),
               "athgpu_amr_pending_maps")
        return newtoold, kind, ffc, dc

    def accept(self):
        _check(load_library().athgpu_amr_accept(self.h), "athgpu_amr_accept")
        self.generation += 1

    def deref_counts(self):
        out = np.zeros(self.nblocks, dtype=np.int32)
        _check(load_library().athgpu_amr_deref_counts(self.h, _ip(out)),
               "athgpu_amr_deref_counts")
        return out

    def step(self, su, thr, after_cycle=True):
        """athgpu_amr_step on StageUpdate su: True when the mesh changed."""
        r = ctypes.c_int()
        _check(load_library().athgpu_amr_step(su.h, self.h, float(thr), int(after_cycle),
                                              ctypes.byref(r)), "athgpu_amr_step")
        if r.value:
            self.generation += 1
        return bool(r.value)


class _RootInfo:
    def __init__(self, nrbx):
        self.nrbx = tuple(nrbx)
        self.root_level = 0
        while (1 << self.root_level) < max(nrbx):
            self.root_level += 1


class NativeMesh(MultiLevelMesh):
    """The current mesh of a NativeAmr with the interface of MultiLevelMesh (block list,
    shapes, coordinates, neighbour tables); the tables come from the library.  Only the
    block locations are fetched when the object is made (a regrid makes one); the
    neighbour tables, coordinates and Loc list on first use, which must come before the
    tree changes again."""

    def __init__(self, amr: NativeAmr):
        self.nx, self.nrbx, self.ng = amr.nx, amr.nrbx, amr.ng
        self.xmin, self.xmax, self.bcs = amr.xmin, amr.xmax, amr.bcs
        self.bx = tuple(self.nx[d] // self.nrbx[d] for d in range(3))
        self.nc = tuple(self.bx[d] + 2 * self.ng for d in range(3))
        self.cng = (self.ng + 1) // 2 + 1
        self.ncc = tuple(self.bx[d] // 2 + 2 * self.ng for d in range(3))
        self.tree = _RootInfo(self.nrbx)
        self._amr, self._gen = amr, amr.generation
        loc = amr.tables(coords=False, nbrs=False)[0]
        self._loc = loc
        self.nblocks = loc.shape[0]
        self.levels = loc[:, 0].astype(np.int32)
        self._tables = None
        self._locs = None

    def _fetch(self):
        if self._tables is None:
            if self._amr.generation != self._gen:
                raise RuntimeError("the adaptive mesh changed since this block list was made")
            _, t, cnt, lv, fine, coarse = self._amr.tables()
            self._tables = ((t, cnt, lv, self._loc), lv, fine, coarse)
        return self._tables

    @property
    def locs(self):
        if self._locs is None:
            self._locs = [Loc(int(r[0]), int(r[1]), int(r[2]), int(r[3])) for r in self._loc]
        return self._locs

    def neighbor_table(self):
        return self._fetch()[0]

    def nblevel_array(self):
        return self._fetch()[1]

    def coordinate_arrays(self):
        return list(self._fetch()[2])

    def coarse_coordinate_arrays(self):
        return list(self._fetch()[3])
