"""Python binding of the C ABI (include/athena_gb300.h) over ctypes.

``StageUpdate`` mirrors how the reference drives the hot path: construct it for a
uniform mesh (the MeshBlock/Coordinates set-up), load the conserved state and face field
(what MeshBlock::ProblemGenerator produces), ``initialize()`` (the tail of
Mesh::Initialize), then ``cycle()`` / ``run_until()`` (the main loop over
TimeIntegratorTaskList stages).  There is no CPU fallback: if the CUDA library is
missing or no GPU is present, construction raises.
"""
import ctypes
import math
import os

import numpy as np

from .mesh import MeshSpec

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libathgpu.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "athena_gb300.h")
DIAG_HEADER = os.path.join(os.path.dirname(HERE), "include", "athena_gb300_diag.h")

HLLD, HLLE, LLF, ROE, LHLLD = 0, 1, 2, 3, 4
_RSOLVERS = {"hlld": HLLD, "hlle": HLLE, "llf": LLF, "roe": ROE, "lhlld": LHLLD}
FP64, FP32 = 0, 1
VL2, RK2 = 0, 1
_INTEGRATORS = {"vl2": VL2, "rk2": RK2}
COPY_WHOLE, COPY_INTERIOR = 0, 1


class AthGPUError(RuntimeError):
    pass


class FaceEmfs(ctypes.Structure):
    """athgpu_face_emfs: e3_x1f, e2_x1f, wght_x1f, e1_x2f, e3_x2f, wght_x2f, e1_x3f,
    e2_x3f, wght_x3f"""
    _fields_ = [(n, ctypes.POINTER(ctypes.c_double)) for n in (
        "e3_x1f", "e2_x1f", "wght_x1f", "e1_x2f", "e3_x2f", "wght_x2f", "e1_x3f", "e2_x3f",
        "wght_x3f")]


class RunStats(ctypes.Structure):
    """athgpu_run_stats"""
    _fields_ = [("divb_sum", ctypes.c_double), ("divb_max", ctypes.c_double),
                ("divb_cells", ctypes.c_longlong), ("floor_cells", ctypes.c_longlong),
                ("sr_cells", ctypes.c_longlong), ("sr_passes", ctypes.c_longlong),
                ("sr_fallbacks", ctypes.c_longlong), ("sr_unconverged", ctypes.c_longlong),
                ("net_error", ctypes.c_int), ("sweep_timeout", ctypes.c_int)]


class MeshDesc(ctypes.Structure):
    _fields_ = [("nbx1", ctypes.c_int), ("nbx2", ctypes.c_int), ("nbx3", ctypes.c_int),
                ("nx1", ctypes.c_int), ("nx2", ctypes.c_int), ("nx3", ctypes.c_int),
                ("nghost", ctypes.c_int), ("xorder", ctypes.c_int),
                ("rsolver", ctypes.c_int), ("precision", ctypes.c_int),
                ("relativistic", ctypes.c_int), ("gamma", ctypes.c_double),
                ("dfloor", ctypes.c_double), ("pfloor", ctypes.c_double),
                ("cfl_number", ctypes.c_double), ("tlim", ctypes.c_double),
                ("x1f", ctypes.POINTER(ctypes.c_double)),
                ("dx1f", ctypes.POINTER(ctypes.c_double)),
                ("x2f", ctypes.POINTER(ctypes.c_double)),
                ("dx2f", ctypes.POINTER(ctypes.c_double)),
                ("x3f", ctypes.POINTER(ctypes.c_double)),
                ("dx3f", ctypes.POINTER(ctypes.c_double)),
                ("sigma_max", ctypes.c_double), ("beta_min", ctypes.c_double),
                ("gamma_max", ctypes.c_double), ("bc", ctypes.c_int * 6),
                ("ppm_fast", ctypes.c_int), ("integrator", ctypes.c_int)]


BC_PERIODIC, BC_OUTFLOW, BC_REFLECT = 0, 1, 2
_BC_CODES = {"periodic": BC_PERIODIC, "outflow": BC_OUTFLOW, "reflecting": BC_REFLECT}


def bc_codes(bc):
    """Six mesh-face boundary flags (inner x1, outer x1, ..., outer x3) as integer codes;
    entries may be codes or the reference's names ("periodic", "outflow", "reflecting")."""
    if bc is None:
        return (BC_PERIODIC,) * 6
    out = tuple(_BC_CODES[b] if isinstance(b, str) else int(b) for b in bc)
    if len(out) != 6:
        raise ValueError("bc needs six entries (ix1, ox1, ix2, ox2, ix3, ox3)")
    return out


class DeviceState(ctypes.Structure):
    _fields_ = [("u", ctypes.c_void_p), ("ulo", ctypes.c_void_p), ("w", ctypes.c_void_p),
                ("bcc", ctypes.c_void_p), ("b1", ctypes.c_void_p), ("b2", ctypes.c_void_p),
                ("b3", ctypes.c_void_p), ("real_bytes", ctypes.c_int)]


_lib = None


def load_library(path=LIB_PATH):
    """Load libathgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise AthGPUError("libathgpu.so is missing: run athena_gb300.build.build() first")
    L = ctypes.CDLL(path)
    vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_int
    sig = {
        "athgpu_create": ([ctypes.POINTER(vp), ctypes.POINTER(MeshDesc)], ip),
        "athgpu_destroy": ([vp], ip),
        "athgpu_set_stream": ([vp, vp], ip),
        "athgpu_upload_state": ([vp, dp, dp, dp, dp], ip),
        "athgpu_upload_prim": ([vp, dp], ip),
        "athgpu_download_state": ([vp, dp, dp, dp, dp], ip),
        "athgpu_download_prim": ([vp, dp, dp], ip),
        "athgpu_initialize": ([vp], ip),
        "athgpu_stage": ([vp, ip], ip),
        "athgpu_cycle": ([vp, ip], ip),
        "athgpu_run_until": ([vp, ctypes.c_double, ip, ctypes.POINTER(ip)], ip),
        "athgpu_get_clock": ([vp, dp, dp], ip),
        "athgpu_set_clock": ([vp, ctypes.c_double, ctypes.c_double], ip),
        "athgpu_synchronize": ([vp], ip),
        "athgpu_floor_count": ([vp, ctypes.POINTER(ctypes.c_longlong), ip], ip),
        "athgpu_device_state_ptrs": ([vp, ctypes.POINTER(DeviceState)], ip),
        "athgpu_set_sweep_segment": ([vp, ip, ip], ip),
        "athgpu_autotune": ([vp, ip, ctypes.POINTER(ip), ctypes.POINTER(ip)], ip),
        "athgpu_history": ([vp, dp], ip),
        "athgpu_ml_plan_check": ([ctypes.POINTER(ip), ip, ctypes.POINTER(ip), ip,
                                  ctypes.POINTER(ip), ctypes.POINTER(ip), ctypes.POINTER(ip),
                                  ctypes.POINTER(ctypes.c_longlong),
                                  ctypes.POINTER(ctypes.c_longlong)], ip),
        "athgpu_set_multilevel": ([vp, ctypes.POINTER(ip), ctypes.POINTER(ip),
                                   ctypes.POINTER(ip), ctypes.POINTER(ctypes.c_longlong)] +
                                  [dp] * 6, ip),
        "athgpu_refinement_eps": ([vp, dp], ip),
        "athgpu_regrid": ([vp, ctypes.POINTER(MeshDesc), ctypes.POINTER(ip),
                           ctypes.POINTER(ip), ctypes.POINTER(ip),
                           ctypes.POINTER(ctypes.c_longlong)] + [dp] * 6 +
                          [ctypes.POINTER(ip), ctypes.POINTER(ip), ip, ctypes.POINTER(ip),
                           ip], ip),
        "athgpu_new_time_step": ([vp], ip),
        "athgpu_regrid_profile": ([dp], ip),
        "athgpu_amr_create": ([ctypes.POINTER(vp), ctypes.POINTER(ip), ctypes.POINTER(ip), ip,
                               dp, dp, ctypes.POINTER(ip), ip, ip], ip),
        "athgpu_amr_destroy": ([vp], ip),
        "athgpu_amr_add_block": ([vp, ip, ctypes.c_longlong, ctypes.c_longlong,
                                  ctypes.c_longlong], ip),
        "athgpu_amr_nblocks": ([vp, ctypes.POINTER(ip)], ip),
        "athgpu_amr_tables": ([vp, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ip),
                               ctypes.POINTER(ip), ctypes.POINTER(ip)] + [dp] * 12, ip),
        "athgpu_amr_flags": ([vp, ctypes.POINTER(ip), ctypes.POINTER(ip)], ip),
        "athgpu_amr_update": ([vp, ctypes.POINTER(ip), ctypes.POINTER(ip)], ip),
        "athgpu_amr_pending": ([vp, ctypes.POINTER(ip), ctypes.POINTER(ip)], ip),
        "athgpu_amr_pending_maps": ([vp] + [ctypes.POINTER(ip)] * 4, ip),
        "athgpu_amr_accept": ([vp], ip),
        "athgpu_amr_deref_counts": ([vp, ctypes.POINTER(ip)], ip),
        "athgpu_amr_step": ([vp, vp, ctypes.c_double, ip, ctypes.POINTER(ip)], ip),
        "athgpu_launch_count": ([vp, ctypes.POINTER(ctypes.c_longlong), ip], ip),
        "athgpu_profile_cycle": ([vp, ip, ctypes.POINTER(ctypes.c_float),
                                  ctypes.POINTER(ip)], ip),
        "athgpu_profile_label": ([vp, ip], ctypes.c_char_p),
        "athgpu_last_error": ([], ctypes.c_char_p),
        "athgpu_version": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes, f.restype = args, res
    _lib = L
    return L


def header_functions(paths=(HEADER, DIAG_HEADER)):
    """Names of the functions declared in include/athena_gb300.h and the diagnostics
    header include/athena_gb300_diag.h."""
    import re
    text = "".join(open(p).read() for p in paths)
    return sorted(set(re.findall(r"\b(athgpu_[a-z_0-9]+)\s*\(", text)))


def _check(status, what):
    if status != 0:
        msg = load_library().athgpu_last_error().decode()
        raise AthGPUError("%s failed (%d): %s" % (what, status, msg))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_floor():
    """sqrt(1024 * FLT_MIN), the reference's dfloor/pfloor default
    (adiabatic_mhd.cpp:29-30)."""
    return math.sqrt(1024 * float(np.finfo(np.float32).tiny))


class StageUpdate:
    """All MeshBlocks of one uniform mesh advanced by the GPU stage update."""

    def __init__(self, mesh: MeshSpec, gamma, xorder=2, rsolver="hlld", precision="fp64",
                 cfl=0.3, tlim=1.0e30, dfloor=None, pfloor=None, relativistic=False,
                 sigma_max=0.0, beta_min=0.0, gamma_max=1000.0, bc=None, integrator="vl2"):
        L = load_library()
        self.kw = dict(gamma=gamma, xorder=xorder, rsolver=rsolver, precision=precision,
                       cfl=cfl, tlim=tlim, dfloor=dfloor, pfloor=pfloor,
                       relativistic=relativistic, sigma_max=sigma_max, beta_min=beta_min,
                       gamma_max=gamma_max, bc=bc, integrator=integrator)
        multilevel = hasattr(mesh, "neighbor_table")
        self._describe(mesh)
        h = ctypes.c_void_p()
        _check(L.athgpu_create(ctypes.byref(h), ctypes.byref(self.desc)), "athgpu_create")
        self.h = h
        if multilevel:
            ml, cc = self._ml_tables(mesh)
            _check(L.athgpu_set_multilevel(h, *ml, *cc), "athgpu_set_multilevel")

    def _describe(self, mesh):
        """The athgpu_mesh_desc of a mesh (keeps the coordinate arrays alive)."""
        k = self.kw
        fl = default_floor()
        multilevel = hasattr(mesh, "neighbor_table")
        bc = mesh.bcs if multilevel else k["bc"]
        self.mesh = mesh
        self.coords = [np.ascontiguousarray(c) for c in mesh.coordinate_arrays()]
        d = MeshDesc()
        d.nbx1, d.nbx2, d.nbx3 = (mesh.nblocks, 1, 1) if multilevel else mesh.nb
        d.nx1, d.nx2, d.nx3 = mesh.bx
        # time/xorder: 1, 2, 3 or "3f" (PPM with the fast limiter, ppm_fast.cpp)
        d.nghost = mesh.ng
        d.xorder, d.ppm_fast = (3, 1) if str(k["xorder"]) == "3f" else (int(k["xorder"]), 0)
        d.rsolver = _RSOLVERS[k["rsolver"]]
        d.precision = FP64 if k["precision"] == "fp64" else FP32
        d.relativistic = 1 if k["relativistic"] else 0
        d.sigma_max, d.beta_min, d.gamma_max = k["sigma_max"], k["beta_min"], k["gamma_max"]
        d.gamma = k["gamma"]
        d.dfloor = fl if k["dfloor"] is None else k["dfloor"]
        d.pfloor = fl if k["pfloor"] is None else k["pfloor"]
        d.cfl_number, d.tlim = k["cfl"], k["tlim"]
        d.bc = (ctypes.c_int * 6)(*bc_codes(bc))
        d.integrator = _INTEGRATORS[k["integrator"]]
        d.x1f, d.dx1f, d.x2f, d.dx2f, d.x3f, d.dx3f = [_dp(c) for c in self.coords]
        self.desc = d
        return d

    def _ml_tables(self, mesh):
        """ctypes arguments of the multi-level tables and coarse coordinates of a mesh."""
        t, cnt, lv, loc = mesh.neighbor_table()
        self._ml = [np.ascontiguousarray(a) for a in (t, cnt, lv, loc)]
        self._cc = [np.ascontiguousarray(c) for c in mesh.coarse_coordinate_arrays()]
        ipp = ctypes.POINTER(ctypes.c_int)
        ml = [self._ml[0].ctypes.data_as(ipp), self._ml[1].ctypes.data_as(ipp),
              self._ml[2].ctypes.data_as(ipp),
              self._ml[3].ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))]
        return ml, [_dp(c) for c in self._cc]

    # --- adaptive mesh refinement -----------------------------------------------------
    def refinement_eps(self):
        """Per-block maximum of |grad p|/p (the blast problem's refinement measure)."""
        out = np.zeros(self.mesh.nblocks)
        _check(load_library().athgpu_refinement_eps(self.h, _dp(out)),
               "athgpu_refinement_eps")
        return out

    def regrid(self, plan, after_cycle=True):
        """Move onto plan.mesh (an athena_gb300.amr.RegridPlan): redistribution and
        Initialize(2); after_cycle takes back the last cycle's NewTimeStep first."""
        L = load_library()
        d = self._describe(plan.mesh)
        ml, cc = self._ml_tables(plan.mesh)
        ipp = ctypes.POINTER(ctypes.c_int)
        maps = [np.ascontiguousarray(a, dtype=np.int32) for a in
                (plan.newtoold, plan.kind, plan.ffc.reshape(-1))]
        _check(L.athgpu_regrid(self.h, ctypes.byref(d), *ml, *cc,
                               maps[0].ctypes.data_as(ipp), maps[1].ctypes.data_as(ipp),
                               int(plan.ffc.shape[0]), maps[2].ctypes.data_as(ipp),
                               1 if after_cycle else 0), "athgpu_regrid")

    def new_time_step(self):
        """Mesh::NewTimeStep again from the last W(U)'s block time steps."""
        _check(load_library().athgpu_new_time_step(self.h), "athgpu_new_time_step")

    def close(self):
        if getattr(self, "h", None):
            load_library().athgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- state ------------------------------------------------------------------------
    def set_state(self, u, b1, b2, b3):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, b1, b2, b3)]
        _check(load_library().athgpu_upload_state(self.h, *[_dp(a) for a in arrs]),
               "athgpu_upload_state")

    def set_prim(self, w):
        """Initial primitives (relativistic runs: also the con2prim seed)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        _check(load_library().athgpu_upload_prim(self.h, _dp(w)), "athgpu_upload_prim")

    def state(self, out=None):
        """Download (u, b1, b2, b3); `out` = four C-contiguous float64 arrays of those
        shapes to fill (pinned host memory makes the copy a direct DMA)."""
        m = self.mesh
        shapes = [(m.nblocks, 5) + m.cell_shape] + [(m.nblocks,) + s for s in m.face_shapes]
        if out is None:
            out = [np.zeros(sh) for sh in shapes]
        else:
            for a, sh in zip(out, shapes):
                if a.shape != sh or a.dtype != np.float64 or not a.flags.c_contiguous:
                    raise ValueError("state(out=...) needs C-contiguous float64 %s" % (sh,))
        u, b1, b2, b3 = out
        _check(load_library().athgpu_download_state(self.h, _dp(u), _dp(b1), _dp(b2),
                                                    _dp(b3)), "athgpu_download_state")
        return u, b1, b2, b3

    def prim(self):
        m = self.mesh
        w = np.zeros((m.nblocks, 5) + m.cell_shape)
        bcc = np.zeros((m.nblocks, 3) + m.cell_shape)
        _check(load_library().athgpu_download_prim(self.h, _dp(w), _dp(bcc)),
               "athgpu_download_prim")
        return w, bcc

    # --- time integration -------------------------------------------------------------
    def initialize(self):
        _check(load_library().athgpu_initialize(self.h), "athgpu_initialize")

    def stage(self, s):
        _check(load_library().athgpu_stage(self.h, s), "athgpu_stage")

    def cycle(self, n=1):
        _check(load_library().athgpu_cycle(self.h, n), "athgpu_cycle")

    def run_until(self, tlim, max_cycles=1 << 30):
        n = ctypes.c_int(0)
        _check(load_library().athgpu_run_until(self.h, tlim, max_cycles, ctypes.byref(n)),
               "athgpu_run_until")
        return n.value

    def synchronize(self):
        _check(load_library().athgpu_synchronize(self.h), "athgpu_synchronize")

    def clock(self):
        t, dt = ctypes.c_double(), ctypes.c_double()
        _check(load_library().athgpu_get_clock(self.h, ctypes.byref(t), ctypes.byref(dt)),
               "athgpu_get_clock")
        return t.value, dt.value

    @property
    def time(self):
        return self.clock()[0]

    @property
    def dt(self):
        return self.clock()[1]

    def set_clock(self, time, dt):
        _check(load_library().athgpu_set_clock(self.h, time, dt), "athgpu_set_clock")

    def floor_count(self, reset=False):
        n = ctypes.c_longlong()
        _check(load_library().athgpu_floor_count(self.h, ctypes.byref(n), int(reset)),
               "athgpu_floor_count")
        return n.value

    def launch_count(self, reset=False):
        n = ctypes.c_longlong()
        _check(load_library().athgpu_launch_count(self.h, ctypes.byref(n), int(reset)),
               "athgpu_launch_count")
        return n.value

    def profile_cycle(self):
        """One non-graph cycle with per-kernel CUDA-event timings: [(name, ms), ...]."""
        L = load_library()
        buf = (ctypes.c_float * 256)()
        n = ctypes.c_int()
        _check(L.athgpu_profile_cycle(self.h, 256, buf, ctypes.byref(n)),
               "athgpu_profile_cycle")
        return [(L.athgpu_profile_label(self.h, i).decode(), buf[i])
                for i in range(min(n.value, 256))]

    HISTORY_NAMES = ("mass", "1-mom", "2-mom", "3-mom", "1-KE", "2-KE", "3-KE", "tot-E",
                     "1-ME", "2-ME", "3-ME")

    def history(self):
        """The reference's history-output sums (dict name -> value)."""
        out = np.zeros(len(self.HISTORY_NAMES))
        _check(load_library().athgpu_history(self.h, _dp(out)), "athgpu_history")
        return dict(zip(self.HISTORY_NAMES, out.tolist()))

    def divb(self):
        """The reference's |div B| diagnostic (WAbsDivergenceB): (sum over interior cells,
        maximum, cells counted)."""
        out = np.zeros(3)
        _check(load_library().athgpu_divb(self.h, _dp(out)), "athgpu_divb")
        return float(out[0]), float(out[1]), int(out[2])

    def stats(self, reset=False):
        """Run statistics (athgpu_stats) as a dict."""
        st = RunStats()
        _check(load_library().athgpu_stats(self.h, ctypes.byref(st), int(reset)),
               "athgpu_stats")
        return {name: getattr(st, name) for name, _ in RunStats._fields_}

    C2P_STARTS = {"stale": 0, "refined": 1, "network": 2}

    def set_c2p_start(self, start, params=None):
        """Start of the relativistic con2prim solve: "stale" (the reference's), "refined"
        (that pressure refined in FP32) or "network" (params: the network's
        ATHGPU_MLP_NPARAM floats, a device tensor or a numpy array)."""
        ptr = None
        if params is not None:
            if hasattr(params, "data_ptr"):
                ptr = ctypes.c_void_p(params.data_ptr())
            else:
                self._net_host = np.ascontiguousarray(params, dtype=np.float32)
                ptr = self._net_host.ctypes.data_as(ctypes.c_void_p)
        L = load_library()
        L.athgpu_set_c2p_start.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        _check(L.athgpu_set_c2p_start(self.h, self.C2P_STARTS[start], ptr),
               "athgpu_set_c2p_start")

    def autotune(self, cycles=2):
        """Pick the x2/x3 sweep segment lengths by timing (state left unchanged);
        returns (seg_x2, seg_x3)."""
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        _check(load_library().athgpu_autotune(self.h, int(cycles), ctypes.byref(a),
                                              ctypes.byref(b)), "athgpu_autotune")
        return a.value, b.value

    def set_sweep_segment(self, seg_x2, seg_x3):
        _check(load_library().athgpu_set_sweep_segment(self.h, seg_x2, seg_x3),
               "athgpu_set_sweep_segment")

    def set_host_copy(self, mode):
        """0: chunked DMA over several copy streams (default); 1: conversion kernels on
        page-locked host memory."""
        _check(load_library().athgpu_set_host_copy(self.h, int(mode)), "athgpu_set_host_copy")

    def set_copy_extent(self, extent):
        """COPY_WHOLE (default): set_state/state move whole arrays; COPY_INTERIOR: only
        each MeshBlock's x2/x3 range of own cells and faces, with whole x1 rows (the
        host's x2/x3 ghost zones neither read nor written; initialize() recomputes every
        ghost zone after an upload)."""
        _check(load_library().athgpu_set_copy_extent(self.h, int(extent)),
               "athgpu_set_copy_extent")
        self.copy_extent = int(extent)

    def set_x3_staging(self, bulk):
        """x3 sweep staging: 0 per-thread cp.async, 1 TMA bulk copies."""
        _check(load_library().athgpu_set_x3_staging(self.h, int(bulk)),
               "athgpu_set_x3_staging")

    def x3_staging(self):
        v = ctypes.c_int()
        _check(load_library().athgpu_get_x3_staging(self.h, ctypes.byref(v)),
               "athgpu_get_x3_staging")
        return v.value

    def set_stream(self, stream_ptr):
        _check(load_library().athgpu_set_stream(self.h, ctypes.c_void_p(stream_ptr)),
               "athgpu_set_stream")

    def device_state(self):
        s = DeviceState()
        _check(load_library().athgpu_device_state_ptrs(self.h, ctypes.byref(s)),
               "athgpu_device_state_ptrs")
        return s


def ml_plan_check(mesh):
    """Build and bounds-check the multi-level operation lists of a MultiLevelMesh on the
    host (no device needed).  Returns (restriction ops, exchange ops, prolongation ops,
    flux-correction tasks); raises AthGPUError on an inconsistent mesh."""
    L = load_library()
    t, cnt, lv, loc = [np.ascontiguousarray(a) for a in mesh.neighbor_table()]
    ip = ctypes.POINTER(ctypes.c_int)
    nx = (ctypes.c_int * 3)(*mesh.bx)
    bc = (ctypes.c_int * 6)(*mesh.bcs)
    out = (ctypes.c_longlong * 4)()
    _check(L.athgpu_ml_plan_check(nx, mesh.ng, bc, mesh.nblocks, t.ctypes.data_as(ip),
                                  cnt.ctypes.data_as(ip), lv.ctypes.data_as(ip),
                                  loc.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                  out), "athgpu_ml_plan_check")
    return tuple(out)


class BlockOperators:
    """The per-operator entry points (athgpu_op_*) on ONE MeshBlock: the reference's
    member functions of the stage update, one call each, on numpy arrays in the block's
    AthenaArray layout (ghosts included).  mesh: a MeshSpec of one block."""

    def __init__(self, mesh, gamma, rsolver="hlld", xorder=2, relativistic=False, **kw):
        if mesh.nblocks != 1:
            raise ValueError("BlockOperators takes a mesh of one MeshBlock")
        self.mesh = mesh
        self.su = StageUpdate(mesh, gamma, xorder=xorder, rsolver=rsolver, precision="fp64",
                              relativistic=relativistic, **kw)
        L = load_library()
        dp, vp = ctypes.POINTER(ctypes.c_double), ctypes.c_void_p
        L.athgpu_op_calculate_fluxes.argtypes = [vp, ctypes.c_int, ctypes.c_double] + \
            [dp] * 8 + [ctypes.POINTER(FaceEmfs)]
        L.athgpu_op_corner_e.argtypes = [vp, dp, dp, ctypes.POINTER(FaceEmfs), dp, dp, dp]
        L.athgpu_op_add_flux_divergence.argtypes = [vp, ctypes.c_double, dp, dp, dp, dp]
        L.athgpu_op_ct.argtypes = [vp, ctypes.c_double] + [dp] * 6
        L.athgpu_op_con2prim.argtypes = [vp] + [dp] * 6 + [ctypes.c_int] * 6 + \
            [ctypes.POINTER(ctypes.c_longlong)]
        L.athgpu_op_new_block_dt.argtypes = [vp] + [dp] * 5 + [dp]
        self.L = L

    @staticmethod
    def _emfs(emf):
        e = FaceEmfs()
        for (name, _), a in zip(FaceEmfs._fields_, emf):
            setattr(e, name, _dp(a))
        return e

    def calculate_fluxes(self, order, dt, w, bcc, b, flx, emf):
        e = self._emfs(emf)
        _check(self.L.athgpu_op_calculate_fluxes(
            self.su.h, order, dt, _dp(w), _dp(bcc), _dp(b[0]), _dp(b[1]), _dp(b[2]),
            _dp(flx[0]), _dp(flx[1]), _dp(flx[2]), ctypes.byref(e)),
            "athgpu_op_calculate_fluxes")

    def corner_e(self, w, bcc, emf, e):
        fe = self._emfs(emf)
        _check(self.L.athgpu_op_corner_e(self.su.h, _dp(w), _dp(bcc), ctypes.byref(fe),
                                         _dp(e[0]), _dp(e[1]), _dp(e[2])),
               "athgpu_op_corner_e")

    def add_flux_divergence(self, wght, flx, u):
        _check(self.L.athgpu_op_add_flux_divergence(self.su.h, wght, _dp(flx[0]),
                                                    _dp(flx[1]), _dp(flx[2]), _dp(u)),
               "athgpu_op_add_flux_divergence")

    def ct(self, wght, e, b):
        _check(self.L.athgpu_op_ct(self.su.h, wght, _dp(e[0]), _dp(e[1]), _dp(e[2]),
                                   _dp(b[0]), _dp(b[1]), _dp(b[2])), "athgpu_op_ct")

    def con2prim(self, cons, b, prim, bcc, rng):
        n = ctypes.c_longlong()
        _check(self.L.athgpu_op_con2prim(self.su.h, _dp(cons), _dp(b[0]), _dp(b[1]),
                                         _dp(b[2]), _dp(prim), _dp(bcc), *rng,
                                         ctypes.byref(n)), "athgpu_op_con2prim")
        return n.value

    def new_block_dt(self, w, bcc, b):
        out = ctypes.c_double()
        _check(self.L.athgpu_op_new_block_dt(self.su.h, _dp(w), _dp(bcc), _dp(b[0]),
                                             _dp(b[1]), _dp(b[2]), ctypes.byref(out)),
               "athgpu_op_new_block_dt")
        return out.value

    def close(self):
        self.su.close()
