"""Adaptive-refinement runs of the oracle — TEST INFRASTRUCTURE ONLY.

Drives OracleMesh through the reference's adaptive main loop with the host refinement
logic of athena_gb300.amr:

* Mesh::Initialize with adaptive refinement (mesh.cpp:1622-1964): problem generator on
  every block, boundaries, refinement flags, regrid (whose Initialize(2) computes a time
  step), repeated until the block count stops changing; then the first time step;
* the main loop (main.cpp:457-541): the stages, time += dt, the refinement flags of the
  last stage (time_integrator.cpp:2321-2326), LoadBalancingAndAdaptiveMeshRefinement
  (regrid + Initialize(2)) and Mesh::NewTimeStep.
"""
import numpy as np

from athena_gb300.amr import AdaptiveMesh, blast_condition

from oracle import OracleMesh

DBL_MAX = float(np.finfo(np.float64).max)


def initialize(mesh0, ic, numlevel, thr, derefine_count=10, condition=blast_condition,
               **kw):
    """(AdaptiveMesh, OracleMesh) after Mesh::Initialize(0); ic(mesh) -> (u, b1, b2, b3)
    is the problem generator, condition(maxeps, thr) the refinement condition."""
    amr = AdaptiveMesh(mesh0, numlevel, derefine_count)
    om = OracleMesh(amr.mesh, **kw)
    om.set_clock(0.0, DBL_MAX)
    while True:
        # the blocks persist between passes (with their coarse buffers); the problem
        # generator rewrites their state
        om.set_state(*ic(amr.mesh))
        om.boundaries()
        flags = amr.check_refinement(condition(om.refine_eps(), thr))
        onb = amr.mesh.nblocks
        plan = amr.update(flags)
        if plan is None:
            break
        om = om.regrid(plan)
        amr.accept(plan)
        if amr.mesh.nblocks == onb:
            break
    om.new_dt()
    return amr, om


def cycle(amr, om, thr, condition=blast_condition, after_stages=None):
    """One cycle of the adaptive main loop; returns the (possibly new) OracleMesh.
    after_stages(om) is called after the stages and time += dt, before the regrid (where
    the reference's UserWorkInLoop dump is written)."""
    om.advance()
    if after_stages is not None:
        after_stages(om)
    flags = amr.check_refinement(condition(om.refine_eps(), thr))
    plan = amr.update(flags)
    if plan is not None:
        om = om.regrid(plan)
        amr.accept(plan)
    om.new_dt()
    return om
