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
import time

from .amr import AdaptiveMesh, blast_condition
from .runtime import StageUpdate


class AdaptiveStageUpdate:
    """``ic(mesh) -> (u, b1, b2, b3)``: the problem generator; ``condition(maxeps, thr)``:
    the refinement condition on the per-block measure (the blast problem's by default);
    further keyword arguments go to StageUpdate."""

    def __init__(self, mesh0, ic, numlevel, thr, derefine_count=10,
                 condition=blast_condition, **kw):
        self.ic, self.thr, self.condition = ic, thr, condition
        self.amr = AdaptiveMesh(mesh0, numlevel, derefine_count)
        self.su = StageUpdate(mesh0, **kw)
        self.regrids = 0
        self.t_refine = 0.0   # host seconds in the refinement measure, flags, tree update
        self.t_regrid = 0.0   # host seconds in the regrids

    @property
    def mesh(self):
        return self.amr.mesh

    def _flags(self):
        return self.amr.check_refinement(self.condition(self.su.refinement_eps(), self.thr))

    def initialize(self):
        su = self.su
        while True:
            time, dt = su.clock()
            su.set_state(*self.ic(self.amr.mesh))
            su.initialize()
            plan = self.amr.update(self._flags())
            if plan is None:
                # no change: this pass's time step is the one after the loop
                return
            # the loop itself makes no time step: that of initialize() is taken back
            su.set_clock(time, dt)
            onb = self.amr.mesh.nblocks
            su.regrid(plan, after_cycle=False)
            self.amr.accept(plan)
            self.regrids += 1
            if self.amr.mesh.nblocks == onb:
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
            t0 = time.perf_counter()
            plan = self.amr.update(self._flags())
            t1 = time.perf_counter()
            if plan is not None:
                su.regrid(plan, after_cycle=True)
                self.amr.accept(plan)
                su.new_time_step()
                self.regrids += 1
            self.t_refine += t1 - t0
            self.t_regrid += time.perf_counter() - t1

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
