"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run where the reference source tree is present (oracle/build_ref.py says where):

    python tests/golden/make_golden.py

It builds the reference (oracle/build_ref.py), runs each case below through the
unmodified reference code path (the reference's own linear_wave problem generator, or
the IC-loading generator oracle/ref_pgen/load_ic.cpp for seeded states), and stores the
inputs and the reference's per-cell outputs:

* ``<case>.npz``: ``ic_*`` (initial state as loaded), ``u``, ``b1``, ``b2``, ``b3``
  (per-block interiors after ``ncycle`` cycles), ``dt`` (the dt of every cycle), ``time``;
  the multi-level cases (``ml_cases``: static refinement regions, blocks in the
  reference's gid order) the same;
* ``golden.json``: case parameters, for the full config-1 linear wave the reference's
  linearwave-errors.dat line plus a SHA-256 of its final state, and the reference's
  history output after every cycle of one case (``history``).
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from athena_gb300.mesh import MeshSpec  # noqa: E402
from athena_gb300 import pgen  # noqa: E402
import build_ref  # noqa: E402
import ref_run  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
GAMMA_LW = 1.666666666666667

CASES = {
    # name: (variant, mesh args, problem, xorder, cfl, ncycle)
    "lw_hlld_plm_1blk": ("mhd_hlld_g2", ((16, 8, 8), (1, 1, 1), 2, (0., 0., 0.),
                                         (3.0, 1.5, 1.5)), "linear_wave", 2, 0.3, 3),
    "lw_hlld_plm_8blk": ("mhd_hlld_g2", ((32, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                         (3.0, 1.5, 1.5)), "linear_wave", 2, 0.3, 2),
    "turb_hlld_ppm_8blk": ("mhd_hlld_g3", ((16, 16, 16), (2, 2, 2), 3, (0., 0., 0.),
                                           (1., 1., 1.)), "turbulence", 3, 0.3, 3),
    "turb_hlle_plm_8blk": ("mhd_hlle_g2", ((16, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                           (1., 1., 1.)), "turbulence", 2, 0.3, 3),
    "turb_hlle_ppm_1blk": ("mhd_hlle_g3", ((16, 16, 16), (1, 1, 1), 3, (0., 0., 0.),
                                           (1., 1., 1.)), "turbulence", 3, 0.3, 2),
    "blast_hlld_plm_8blk": ("mhd_hlld_g2", ((16, 16, 16), (2, 2, 2), 2, (-.5, -.5, -.5),
                                            (.5, .5, .5)), "blast", 2, 0.3, 3),
    "blast_hlle_ppm_8blk": ("mhd_hlle_g3", ((16, 16, 16), (2, 2, 2), 3, (-.5, -.5, -.5),
                                            (.5, .5, .5)), "blast", 3, 0.3, 3),
    # local Lax-Friedrichs (--flux=llf)
    "blast_llf_plm_8blk": ("mhd_llf_g2", ((16, 16, 16), (2, 2, 2), 2, (-.5, -.5, -.5),
                                          (.5, .5, .5)), "blast", 2, 0.3, 3),
    "turb_llf_plm_8blk": ("mhd_llf_g2", ((16, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                         (1., 1., 1.)), "turbulence", 2, 0.3, 3),
    # PPM with the fast limiter (time/xorder = 3f, ppm_fast.cpp)
    "turb_hlld_ppmf_8blk": ("mhd_hlld_g3", ((16, 16, 16), (2, 2, 2), 3, (0., 0., 0.),
                                            (1., 1., 1.)), "turbulence", "3f", 0.3, 3),
    "blast_hlle_ppmf_8blk": ("mhd_hlle_g3", ((16, 16, 16), (2, 2, 2), 3, (-.5, -.5, -.5),
                                             (.5, .5, .5)), "blast", "3f", 0.3, 4),
    # Roe's linearisation (--flux=roe)
    "blast_roe_plm_8blk": ("mhd_roe_g2", ((16, 16, 16), (2, 2, 2), 2, (-.5, -.5, -.5),
                                          (.5, .5, .5)), "blast", 2, 0.3, 4),
    "turb_roe_plm_8blk": ("mhd_roe_g2", ((16, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                         (1., 1., 1.)), "turbulence", 2, 0.3, 3),
    # low-dissipation HLLD (--flux=lhlld, lhlld.cpp, with calculate_velocity_differences.cpp)
    "blast_lhlld_plm_8blk": ("mhd_lhlld_g2", ((16, 16, 16), (2, 2, 2), 2, (-.5, -.5, -.5),
                                              (.5, .5, .5)), "blast", 2, 0.3, 4),
    "turb_lhlld_ppm_8blk": ("mhd_lhlld_g3", ((16, 16, 16), (2, 2, 2), 3, (0., 0., 0.),
                                             (1., 1., 1.)), "turbulence", 3, 0.3, 3),
    # special-relativistic MHD (-s -b --flux=hlle): relativistic Kelvin-Helmholtz layer
    "srkh_hlle_plm_8blk": ("srmhd_hlle_g2", ((16, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                            (1., 1., 1.)), "sr_kh", 2, 0.3, 3),
    "srkh_hlle_plm_1blk": ("srmhd_hlle_g2", ((16, 8, 8), (1, 1, 1), 2, (0., 0., 0.),
                                            (1., 1., 1.)), "sr_kh", 2, 0.4, 4),
    # relativistic LLF (-s -b --flux=llf, llf_mhd_rel.cpp)
    "srkh_llf_plm_8blk": ("srmhd_llf_g2", ((16, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                          (1., 1., 1.)), "sr_kh", 2, 0.3, 3),
    "srkh_llf_plm_1blk": ("srmhd_llf_g2", ((16, 8, 8), (1, 1, 1), 2, (0., 0., 0.),
                                          (1., 1., 1.)), "sr_kh", 2, 0.4, 4),
    # relativistic HLLD (-s -b --flux=hlld, hlld_rel.cpp)
    "srkh_hlld_plm_8blk": ("srmhd_hlld_g2", ((16, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                            (1., 1., 1.)), "sr_kh", 2, 0.3, 3),
    "srkh_hlld_plm_1blk": ("srmhd_hlld_g2", ((16, 8, 8), (1, 1, 1), 2, (0., 0., 0.),
                                            (1., 1., 1.)), "sr_kh", 2, 0.4, 4),
    # physical boundaries (flags inner/outer x1, x2, x3: 1 outflow, 2 reflecting)
    "blastbc_hlld_plm_8blk": ("mhd_hlld_g2", ((16, 16, 16), (2, 2, 2), 2, (-.5, -.5, -.5),
                                              (.5, .5, .5)), "blast", 2, 0.3, 4),
    "blastbc_hlle_ppm_1blk": ("mhd_hlle_g3", ((16, 16, 16), (1, 1, 1), 3, (-.5, -.5, -.5),
                                              (.5, .5, .5)), "blast", 3, 0.3, 4),
    # time/integrator = rk2 (Heun / SSPRK(2,2), time_integrator.cpp:338-465)
    "turbrk2_hlld_plm_8blk": ("mhd_hlld_g2", ((16, 16, 16), (2, 2, 2), 2, (0., 0., 0.),
                                              (1., 1., 1.)), "turbulence", 2, 0.6, 3),
    "blastrk2_hlle_ppm_8blk": ("mhd_hlle_g3", ((16, 16, 16), (2, 2, 2), 3, (-.5, -.5, -.5),
                                               (.5, .5, .5)), "blast", 3, 0.4, 3),
}
# time/integrator of the cases that do not use vl2
INTEGRATOR = {"turbrk2_hlld_plm_8blk": "rk2", "blastrk2_hlle_ppm_8blk": "rk2",
              "mlblastrk2_hlle_plm": "rk2"}
# mesh-face boundary flags of the cases that are not periodic
BCS = {"blastbc_hlld_plm_8blk": (1, 1, 2, 2, 0, 0),
       "blastbc_hlle_ppm_1blk": (2, 1, 1, 2, 2, 1)}


# multi-level (static refinement) cases: variant, MultiLevelMesh args (nx, nrbx, ng,
# xmin, xmax, bcs, regions), problem, problem parameters, xorder, cfl, ncycle
ML_CASES = {
    "mlblast_hlle_plm": ("mhd_hlle_g2", ((16, 16, 16), (2, 2, 2), 2, (-.5, -.5, -.5),
                                         (.5, .5, .5), (1, 1, 2, 2, 0, 0),
                                         [((0.1, 0.1, 0.1), (0.2, 0.2, 0.2), 1)]),
                         "blast", {"radius": 0.15, "pamb": 0.1, "prat": 100.0, "b0": 1.0,
                                   "angle": 45.0, "x1_0": 0.25, "x2_0": 0.25,
                                   "x3_0": 0.25}, 2, 0.3, 6),
    "mlsmooth_hlld_ppm": ("mhd_hlld_g4", ((16, 16, 16), (2, 2, 2), 4, (-.5, -.5, -.5),
                                          (.5, .5, .5), (0, 0, 0, 0, 0, 0),
                                          [((-0.4, -0.4, -0.4), (-0.3, -0.3, -0.3), 1)]),
                          "smooth", {"seed": 7}, 3, 0.3, 4),
    "mlsmooth3_hlle_plm": ("mhd_hlle_g2", ((8, 8, 8), (2, 2, 2), 2, (-.5, -.5, -.5),
                                           (.5, .5, .5), (1, 1, 2, 2, 1, 1),
                                           [((0.3, 0.3, 0.3), (0.35, 0.35, 0.35), 2)]),
                           "smooth", {"seed": 11}, 2, 0.3, 4),
    "mlblastrk2_hlle_plm": ("mhd_hlle_g2", ((16, 16, 16), (2, 2, 2), 2, (-.5, -.5, -.5),
                                            (.5, .5, .5), (1, 1, 0, 0, 2, 2),
                                            [((-0.2, 0.1, -0.2), (-0.1, 0.2, -0.1), 1)]),
                            "blast", {"radius": 0.15, "pamb": 0.1, "prat": 100.0,
                                      "b0": 1.0, "angle": 30.0, "x1_0": -0.2,
                                      "x2_0": 0.2, "x3_0": -0.1}, 2, 0.5, 5),
}


# adaptive (blast pressure-gradient) cases: variant, MultiLevelMesh args (nx, nrbx, ng,
# xmin, xmax, bcs), blast parameters (with thr), numlevel, derefine_count, xorder, cfl,
# ncycle.  The floors are given explicitly: with the defaults, the reference's first
# MeshBlock uses sqrt(1024 FLT_MIN) while every later one reads back the 6-digit string
# that GetOrAddReal stored (parameter_input.cpp:603-623), and the blast reaches the
# pressure floor.
AMR_FLOOR = "3.46945e-18"
AMR_CASES = {
    "amrblast_hlle_plm": ("mhd_hlle_g2", ((32, 32, 32), (4, 4, 4), 2, (-.5, -.5, -.5),
                                          (.5, .5, .5), (0, 0, 0, 0, 0, 0)),
                          {"radius": 0.1, "pamb": 0.1, "prat": 100.0, "b0": 1.0,
                           "angle": 45.0, "x1_0": 0.0, "x2_0": 0.0, "x3_0": 0.0,
                           "thr": 0.5}, 3, 2, 2, 0.3, 10),
    "amrblast_hlld_ppm": ("mhd_hlld_g4", ((32, 32, 32), (4, 4, 4), 4, (-.5, -.5, -.5),
                                          (.5, .5, .5), (0, 0, 0, 0, 0, 0)),
                          {"radius": 0.12, "pamb": 0.1, "prat": 100.0, "b0": 1.0,
                           "angle": 30.0, "x1_0": 0.3, "x2_0": 0.0, "x3_0": 0.0,
                           "thr": 1.0}, 3, 1, 3, 0.3, 12),
    # outflow x1 faces, reflecting x2 faces, periodic x3; the blast near a corner
    "amrblastbc_hlle_plm": ("mhd_hlle_g2", ((32, 32, 32), (4, 4, 4), 2, (-.5, -.5, -.5),
                                            (.5, .5, .5), (1, 1, 2, 2, 0, 0)),
                            {"radius": 0.1, "pamb": 0.1, "prat": 100.0, "b0": 1.0,
                             "angle": 60.0, "x1_0": 0.38, "x2_0": -0.4, "x3_0": 0.45,
                             "thr": 0.5}, 3, 2, 2, 0.3, 10),
}


def state_digest(mesh, u, b1, b2, b3):
    """sha256 of the interior conserved state and face field in block order."""
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(mesh.interior(u)).tobytes())
    for b in (b1, b2, b3):
        h.update(np.ascontiguousarray(mesh.interior_faces(b)).tobytes())
    return h.hexdigest()


def run_amr_case(name, spec):
    """An adaptive blast through the reference's own pgen/blast.cpp with
    refinement = adaptive.  Stores every cycle's block list (after the stages, before the
    regrid) and dt, and the last cycle's state as a digest and per-block sums."""
    from athena_gb300.meshtree import MultiLevelMesh
    variant, margs, prob, numlevel, dcount, xorder, cfl, ncycle = spec
    nx, nrbx, ng, xmin, xmax, bcs = margs
    mesh0 = MultiLevelMesh(nx, nrbx, ng, xmin, xmax, bcs=bcs)
    gamma = 5.0 / 3.0
    text = ref_run.athinput_multilevel(mesh0, gamma, xorder, cfl, ncycle, 1.0e3, prob,
                                       refinement="adaptive", numlevel=numlevel,
                                       amr={"derefine_count": dcount},
                                       hydro={"dfloor": AMR_FLOOR, "pfloor": AMR_FLOOR})
    d, _ = ref_run.run_reference(variant, "athena_blast", text)
    locs, offs, dts, nregrid, prev = [], [0], [], 0, None
    for c in range(1, ncycle + 1):
        dump = ref_run.read_dump_blocks(os.path.join(d, "dump.%05d.bin" % c))
        locs += dump["locs"]
        offs.append(len(locs))
        dts.append(dump["dt"])
        nregrid += int(prev is not None and prev != dump["locs"])
        prev = dump["locs"]
    mesh = MultiLevelMesh(nx, nrbx, ng, xmin, xmax, bcs=bcs)
    from athena_gb300.meshtree import Loc
    for lv, a, b, c3 in dump["locs"]:
        mesh.tree.add_block(Loc(lv, a, b, c3))
    mesh.rebuild()
    assert [(l.level, l.lx1, l.lx2, l.lx3) for l in mesh.locs] == dump["locs"]
    sums = mesh.interior(dump["u"]).sum(axis=(2, 3, 4))
    np.savez_compressed(os.path.join(OUT, name + ".npz"),
                        locs=np.array(locs, dtype=np.int32), offsets=np.array(offs),
                        dt=np.array(dts), usum=sums)
    return {"variant": variant, "nx": nx, "nrbx": nrbx, "ng": ng, "xmin": xmin,
            "xmax": xmax, "bc": list(bcs), "problem": prob, "numlevel": numlevel,
            "derefine_count": dcount, "floor": float(AMR_FLOOR), "xorder": xorder,
            "rsolver": variant.split("_")[1], "cfl": cfl,
            "ncycle": ncycle, "gamma": gamma, "tlim": 1.0e3, "time": dump["time"],
            "digest": state_digest(mesh, dump["u"], dump["b1"], dump["b2"], dump["b3"]),
            "nblocks_last": len(dump["locs"]), "regrids": nregrid}


def run_restart_case():
    """A restart through the reference: the linear wave on one 8x4x4 MeshBlock runs 3
    cycles and writes its final restart file (outputs/restart.cpp); a second run restarts
    from that file (``-r``) to cycle 6.  Stores the restart file itself and the restarted
    run's dts and final interior state."""
    import shutil
    import subprocess
    mesh = MeshSpec((8, 4, 4), (1, 1, 1), 2, (0., 0., 0.), (3.0, 1.5, 1.5))
    text = ref_run.athinput(mesh, GAMMA_LW, 2, 0.3, 3, 1.0e3, {
        "compute_error": "false", "wave_flag": 0, "amp": 1.0e-6, "vflow": 0.0})
    text += "<output9>\nfile_type = rst\ndt = 1.0e9\n"
    d, _ = ref_run.run_reference("mhd_hlld_g2", "athena_lw", text)
    exe = os.path.join(ref_run.REF_OUT, "mhd_hlld_g2", "athena_lw")
    # the restarted run writes its own final restart file: keep the first one apart
    shutil.copyfile(os.path.join(d, "Ref.final.rst"), os.path.join(d, "cycle3.rst"))
    shutil.copyfile(os.path.join(d, "Ref.final.rst"), os.path.join(OUT, "restart_lw.rst"))
    r = subprocess.run([exe, "-r", "cycle3.rst", "time/nlim=6"], cwd=d,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    dts = []
    for c in range(4, 7):
        dump = ref_run.read_dump(os.path.join(d, "dump.%05d.bin" % c), mesh)
        dts.append(dump["dt"])
    np.savez_compressed(os.path.join(OUT, "restart_lw_after.npz"),
                        u=mesh.interior(dump["u"]), dt=np.array(dts), time=dump["time"])
    return {"variant": "mhd_hlld_g2", "nx": [8, 4, 4], "nb": [1, 1, 1], "ng": 2,
            "xmin": [0., 0., 0.], "xmax": [3.0, 1.5, 1.5], "gamma": GAMMA_LW, "xorder": 2,
            "rsolver": "hlld", "cfl": 0.3, "cycles_before": 3, "cycles_after": 3}


def run_vtk_case():
    """The reference's VTK outputs (prim as out8, cons as out7) of the initial state of the
    linear wave on two MeshBlocks of 4^3 (the outputs written at t = 0, after
    Mesh::Initialize)."""
    import shutil
    mesh = MeshSpec((8, 4, 4), (2, 1, 1), 2, (0., 0., 0.), (3.0, 1.5, 1.5))
    text = ref_run.athinput(mesh, GAMMA_LW, 2, 0.3, 1, 1.0e3, {
        "compute_error": "false", "wave_flag": 0, "amp": 1.0e-6, "vflow": 0.0})
    text += ("<output8>\nfile_type = vtk\nvariable = prim\ndt = 1.0e9\n"
             "<output7>\nfile_type = vtk\nvariable = cons\ndt = 1.0e9\n")
    d, _ = ref_run.run_reference("mhd_hlld_g2", "athena_lw", text)
    os.makedirs(os.path.join(OUT, "vtk"), exist_ok=True)
    files = sorted(f for f in os.listdir(d) if f.endswith(".vtk"))
    for f in files:
        shutil.copyfile(os.path.join(d, f), os.path.join(OUT, "vtk", f))
    return {"nx": [8, 4, 4], "nb": [2, 1, 1], "ng": 2, "xmin": [0., 0., 0.],
            "xmax": [3.0, 1.5, 1.5], "gamma": GAMMA_LW, "files": files}


def ml_mesh(margs):
    from athena_gb300.meshtree import MultiLevelMesh
    nx, nrbx, ng, xmin, xmax, bcs, regions = margs
    return MultiLevelMesh(nx, nrbx, ng, xmin, xmax, bcs=bcs, regions=regions)


def run_ml_case(name, spec):
    """A multi-level case through the reference (static refinement regions): the blast
    problem through the reference's own pgen/blast.cpp, smooth states through
    oracle/ref_pgen/load_blocks.cpp.  Stores the initial state as this package generates
    it (pgen.blast_blocks restates blast.cpp), the reference's interiors after ncycle
    cycles and every cycle's dt."""
    variant, margs, problem, prob, xorder, cfl, ncycle = spec
    mesh = ml_mesh(margs)
    gamma = 5.0 / 3.0
    regions = margs[6]
    if problem == "blast":
        ic = pgen.blast_blocks(mesh, gamma, radius=prob["radius"], pamb=prob["pamb"],
                               prat=prob["prat"], b0=prob["b0"], angle_deg=prob["angle"],
                               center=(prob["x1_0"], prob["x2_0"], prob["x3_0"]))
        text = ref_run.athinput_multilevel(mesh, gamma, xorder, cfl, ncycle, 1.0e3, prob,
                                           regions=regions,
                                           integrator=INTEGRATOR.get(name, "vl2"))
        d, _ = ref_run.run_reference(variant, "athena_blast", text)
    else:
        ic = pgen.smooth_blocks(mesh, gamma, seed=prob["seed"])
        text = ref_run.athinput_multilevel(mesh, gamma, xorder, cfl, ncycle, 1.0e3,
                                           {"ic_file": "ic.bin"}, regions=regions,
                                           integrator=INTEGRATOR.get(name, "vl2"))
        d, _ = ref_run.run_reference(variant, "athena_blocks", text, blocks_ic=(mesh,) + ic)
    dts = []
    for c in range(1, ncycle + 1):
        dump = ref_run.read_dump_blocks(os.path.join(d, "dump.%05d.bin" % c))
        assert dump["locs"] == [(l.level, l.lx1, l.lx2, l.lx3) for l in mesh.locs]
        dts.append(dump["dt"])
    fi = mesh.interior_faces
    u0, b10, b20, b30 = ic
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        ic_u=mesh.interior(u0), ic_b1=fi(b10), ic_b2=fi(b20), ic_b3=fi(b30),
        u=mesh.interior(dump["u"]), b1=fi(dump["b1"]), b2=fi(dump["b2"]), b3=fi(dump["b3"]),
        w=mesh.interior(dump["w"]), dt=np.array(dts), time=dump["time"])
    nx, nrbx, ng, xmin, xmax, bcs, regs = margs
    return {"variant": variant, "nx": nx, "nrbx": nrbx, "ng": ng, "xmin": xmin,
            "xmax": xmax, "bc": list(bcs), "regions": regs, "nblocks": mesh.nblocks,
            "levels": sorted(set(int(v) for v in mesh.levels)), "problem": problem,
            "xorder": xorder, "rsolver": variant.split("_")[1],
            "cfl": cfl, "ncycle": ncycle, "gamma": gamma, "tlim": 1.0e3,
            "integrator": INTEGRATOR.get(name, "vl2")}


def global_ic(problem, mesh):
    if problem == "turbulence":
        return pgen.turbulence(mesh.nx, seed=7, mach=1.0)
    if problem == "blast":
        return pgen.blast(mesh.nx, xmin=mesh.xmin, xmax=mesh.xmax, radius=0.25)
    raise ValueError(problem)


def gamma_of(problem):
    if problem == "sr_kh":
        return 4.0 / 3.0
    return GAMMA_LW if problem == "linear_wave" else 5.0 / 3.0


def state_hash(u, b1, b2, b3, mesh):
    ng = mesh.ng
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(mesh.interior(u)).tobytes())
    for b in (b1, b2, b3):
        h.update(np.ascontiguousarray(b[:, ng:-ng, ng:-ng, ng:-ng]).tobytes())
    return h.hexdigest()


def run_case(name, spec):
    variant, margs, problem, xorder, cfl, ncycle = spec
    mesh = MeshSpec(*margs)
    gamma = gamma_of(problem)
    if problem == "linear_wave":
        lw = pgen.LinearWave(mesh, gamma=GAMMA_LW)
        u0, b10, b20, b30 = lw.generate()
        text = ref_run.athinput(mesh, gamma, xorder, cfl, ncycle, 1.0e3, {
            "compute_error": "false", "wave_flag": 0, "amp": 1.0e-6, "vflow": 0.0})
        d, _ = ref_run.run_reference(variant, "athena_lw", text)
        tlim = 1.0e3
    elif problem == "sr_kh":
        gw, g1, g2, g3 = pgen.sr_kelvin_helmholtz(mesh.nx, seed=9, noise=0.05)
        gu = pgen.sr_prim_to_cons(gw, pgen.cell_centered(g1, g2, g3), gamma)
        u0 = mesh.scatter_cells(gu)
        w0 = mesh.scatter_cells(gw)
        b10, b20, b30 = mesh.scatter_faces(g1, g2, g3)
        text = ref_run.athinput(mesh, gamma, xorder, cfl, ncycle, 1.0e3,
                                {"ic_file": "ic.bin"})
        d, _ = ref_run.run_reference(variant, "athena_ic", text, ic=(1, gw, g1, g2, g3))
        tlim = 1.0e3
    else:
        gu, g1, g2, g3 = global_ic(problem, mesh)
        u0 = mesh.scatter_cells(gu)
        b10, b20, b30 = mesh.scatter_faces(g1, g2, g3)
        text = ref_run.athinput(mesh, gamma, xorder, cfl, ncycle, 1.0e3,
                                {"ic_file": "ic.bin"}, bc=BCS.get(name, (0,) * 6),
                                integrator=INTEGRATOR.get(name, "vl2"))
        d, _ = ref_run.run_reference(variant, "athena_ic", text, ic=(0, gu, g1, g2, g3))
        tlim = 1.0e3
    dts = []
    for c in range(1, ncycle + 1):
        dump = ref_run.read_dump(os.path.join(d, "dump.%05d.bin" % c), mesh)
        dts.append(dump["dt"])
    ng = mesh.ng
    fi = lambda b: b[:, ng:-ng, ng:-ng, ng:-ng]  # noqa: E731
    extra = {"ic_w": mesh.interior(w0)} if problem == "sr_kh" else {}
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        ic_u=mesh.interior(u0), ic_b1=fi(b10), ic_b2=fi(b20), ic_b3=fi(b30),
        u=mesh.interior(dump["u"]), b1=fi(dump["b1"]), b2=fi(dump["b2"]), b3=fi(dump["b3"]),
        w=mesh.interior(dump["w"]), dt=np.array(dts), time=dump["time"], **extra)
    return {"variant": variant, "nx": mesh.nx, "nb": mesh.nb, "ng": mesh.ng,
            "relativistic": problem == "sr_kh",
            "xmin": mesh.xmin, "xmax": mesh.xmax, "problem": problem, "xorder": xorder,
            "rsolver": variant.split("_")[1], "cfl": cfl,
            "ncycle": ncycle, "gamma": gamma, "tlim": tlim, "bc": list(BCS.get(name, (0,) * 6)),
            "integrator": INTEGRATOR.get(name, "vl2")}


def run_config1():
    """Config 1: 64x32x32 fast wave, one period, compute_error (the reference's own
    problem generator and error routine)."""
    mesh = MeshSpec((64, 32, 32), (1, 1, 1), 2, (0., 0., 0.), (3.0, 1.5, 1.5))
    text = ref_run.athinput(mesh, GAMMA_LW, 2, 0.3, -1, 1.0, {
        "compute_error": "true", "wave_flag": 0, "amp": 1.0e-6, "vflow": 0.0,
        "test": "true"})
    d, out = ref_run.run_reference("mhd_hlld_g2", "athena_lw", text)
    lines = open(os.path.join(d, "linearwave-errors.dat")).read().strip().splitlines()
    files = sorted(f for f in os.listdir(d) if f.startswith("dump."))
    last = ref_run.read_dump(os.path.join(d, files[-1]), mesh)
    zc = [ln for ln in out.splitlines() if "zone-cycles/cpu_second" in ln]
    return {"errors_header": lines[0], "errors": lines[-1],
            "ncycle": last["ncycle"], "time": last["time"],
            "sha256_final": state_hash(last["u"], last["b1"], last["b2"], last["b3"], mesh),
            "reference_zone_cycles_per_cpu_second_here": zc[-1] if zc else None}


def run_history(name="turb_hlld_ppm_8blk"):
    """The reference's history output (outputs/history.cpp) after every cycle of one golden
    case, written at full double precision: pins athgpu_history."""
    variant, margs, problem, xorder, cfl, ncycle = CASES[name]
    mesh = MeshSpec(*margs)
    gu, g1, g2, g3 = global_ic(problem, mesh)
    text = ref_run.athinput(mesh, gamma_of(problem), xorder, cfl, ncycle, 1.0e3,
                            {"ic_file": "ic.bin"}, history_every_cycle=True)
    d, _ = ref_run.run_reference(variant, "athena_ic", text, ic=(0, gu, g1, g2, g3))
    return {"case": name, "rows": ref_run.read_history(os.path.join(d, "Ref.hst"))}


def main(only=None):
    for v in sorted({c[0] for c in CASES.values()} | {c[0] for c in ML_CASES.values()}
                    | {c[0] for c in AMR_CASES.values()}):
        build_ref.build_variant(v)
    meta = {"cases": {}}
    path = os.path.join(OUT, "golden.json")
    if only and os.path.exists(path):
        with open(path) as f:
            meta = json.load(f)
    for name, spec in CASES.items():
        if only and name not in only:
            continue
        print("case", name, flush=True)
        meta["cases"][name] = run_case(name, spec)
    meta.setdefault("ml_cases", {})
    for name, spec in ML_CASES.items():
        if only and name not in only:
            continue
        print("case", name, flush=True)
        meta["ml_cases"][name] = run_ml_case(name, spec)
    meta.setdefault("amr_cases", {})
    for name, spec in AMR_CASES.items():
        if only and name not in only:
            continue
        print("case", name, flush=True)
        meta["amr_cases"][name] = run_amr_case(name, spec)
    if not only or "vtk" in only:
        print("vtk", flush=True)
        meta["vtk"] = run_vtk_case()
    if not only or "restart" in only:
        print("restart", flush=True)
        meta["restart"] = run_restart_case()
    if not only or "history" in only:
        print("history", flush=True)
        meta["history"] = run_history()
    if not only:
        print("config1", flush=True)
        meta["config1_linear_wave"] = run_config1()
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
