"""ctypes wrapper of the C oracle (athena_oracle.c) — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "athena_oracle.c")


def build(force=False):
    """Compile liboracle.so (plain C, no FMA contraction, OpenMP over MeshBlocks)."""
    deps = [SRC, os.path.join(HERE, "athena_oracle.h"), os.path.join(HERE, "athena_oracle_ml.c")]
    if not force and os.path.exists(LIB) and \
            os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-o", LIB + ".tmp", SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


# time/integrator values (athena_oracle.h ORC_VL2, ORC_RK2, ORC_RK1)
INTEGRATORS = {"vl2": 0, "rk2": 1, "rk1": 2}


class Params(ctypes.Structure):
    _fields_ = [("nbx1", ctypes.c_int), ("nbx2", ctypes.c_int), ("nbx3", ctypes.c_int),
                ("nx1", ctypes.c_int), ("nx2", ctypes.c_int), ("nx3", ctypes.c_int),
                ("ng", ctypes.c_int), ("xorder", ctypes.c_int), ("rsolver", ctypes.c_int),
                ("relativistic", ctypes.c_int), ("gamma", ctypes.c_double),
                ("dfloor", ctypes.c_double), ("pfloor", ctypes.c_double),
                ("cfl_number", ctypes.c_double), ("tlim", ctypes.c_double),
                ("sigma_max", ctypes.c_double), ("beta_min", ctypes.c_double),
                ("gamma_max", ctypes.c_double), ("bc", ctypes.c_int * 6),
                ("ppm_fast", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(Params)] + [dp] * 6
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_set_state.argtypes = [ctypes.c_void_p, dp, dp, dp, dp]
        L.orc_set_prim.argtypes = [ctypes.c_void_p, dp]
        L.orc_get_state.argtypes = [ctypes.c_void_p, dp, dp, dp, dp]
        L.orc_get_prim.argtypes = [ctypes.c_void_p, dp, dp]
        L.orc_get_dt.argtypes = [ctypes.c_void_p]
        L.orc_get_dt.restype = ctypes.c_double
        L.orc_get_time.argtypes = [ctypes.c_void_p]
        L.orc_get_time.restype = ctypes.c_double
        L.orc_set_dt.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_initialize.argtypes = [ctypes.c_void_p]
        L.orc_cycle.argtypes = [ctypes.c_void_p]
        L.orc_stage.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_num_threads.argtypes = [ctypes.c_int]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_c2p_failures.argtypes = [ctypes.c_void_p]
        L.orc_c2p_failures.restype = ctypes.c_long
        L.orc_sr_c2p_cells.argtypes = [ctypes.c_long, ctypes.c_double, ctypes.c_double,
                                       dp, dp, dp, dp, ctypes.POINTER(ctypes.c_int)]
        L.orc_sr_prim_to_cons.argtypes = [ctypes.c_long, ctypes.c_double, dp, dp, dp]
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_set_multilevel.argtypes = [ctypes.c_void_p, ip, ip, ip,
                                         ctypes.POINTER(ctypes.c_longlong)] + [dp] * 6
        L.orc_set_multilevel.restype = ctypes.c_int
        L.orc_set_integrator.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_advance.argtypes = [ctypes.c_void_p]
        L.orc_new_dt.argtypes = [ctypes.c_void_p]
        L.orc_set_time.argtypes = [ctypes.c_void_p, ctypes.c_double]
        L.orc_ml_boundaries.argtypes = [ctypes.c_void_p]
        L.orc_refine_eps.argtypes = [ctypes.c_void_p, dp]
        L.orc_regrid.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ip, ip, ctypes.c_int, ip]
        L.orc_regrid.restype = ctypes.c_int
        vp = ctypes.c_void_p
        L.orc_op_fluxes.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, dp,
                                    dp, ctypes.POINTER(dp)]
        L.orc_op_corner_e.argtypes = [vp, ctypes.c_int, ctypes.POINTER(dp), dp, dp, dp]
        L.orc_op_add_flux_divergence.argtypes = [vp, ctypes.c_int, ctypes.c_double, dp, dp,
                                                 dp, dp]
        L.orc_op_ct.argtypes = [vp, ctypes.c_int, ctypes.c_double, dp, dp, dp, dp, dp, dp]
        L.orc_op_con2prim.argtypes = [vp, ctypes.c_int] + [ctypes.c_int] * 6
        L.orc_op_con2prim.restype = ctypes.c_long
        L.orc_op_new_block_dt.argtypes = [vp, ctypes.c_int]
        L.orc_op_new_block_dt.restype = ctypes.c_double
        L.orc_riemann_face.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, dp,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class OracleMesh:
    """The oracle's mesh: the same MeshSpec, parameters and arrays as the CUDA path."""

    def __init__(self, mesh, gamma, xorder=2, rsolver="hlld", cfl=0.3, tlim=1e30,
                 dfloor=None, pfloor=None, relativistic=False, threads=0, sigma_max=0.0,
                 beta_min=0.0, gamma_max=1000.0, bc=(0, 0, 0, 0, 0, 0), integrator="vl2"):
        L = lib()
        self.kw = dict(gamma=gamma, xorder=xorder, rsolver=rsolver, cfl=cfl, tlim=tlim,
                       dfloor=dfloor, pfloor=pfloor, relativistic=relativistic,
                       threads=threads, sigma_max=sigma_max, beta_min=beta_min,
                       gamma_max=gamma_max, bc=bc, integrator=integrator)
        import math
        fmin = float(np.finfo(np.float32).tiny)
        floor = math.sqrt(1024 * fmin)   # adiabatic_mhd.cpp:29-30
        self.mesh = mesh
        multilevel = hasattr(mesh, "neighbor_table")
        if multilevel:
            bc = mesh.bcs
        nbl = (mesh.nblocks, 1, 1) if multilevel else mesh.nb
        # time/xorder: 1, 2, 3 or "3f" (PPM with the fast limiter, ppm_fast.cpp)
        xo, ppmf = (3, 1) if str(xorder) == "3f" else (int(xorder), 0)
        rs = {"hlld": 0, "hlle": 1, "llf": 2, "roe": 3, "lhlld": 4}[rsolver]
        self.p = Params(nbl[0], nbl[1], nbl[2], mesh.bx[0], mesh.bx[1],
                        mesh.bx[2], mesh.ng, xo, rs,
                        1 if relativistic else 0, gamma,
                        floor if dfloor is None else dfloor,
                        floor if pfloor is None else pfloor, cfl, tlim, sigma_max,
                        beta_min, gamma_max, (ctypes.c_int * 6)(*bc), ppmf)
        self.coords = [np.ascontiguousarray(c) for c in mesh.coordinate_arrays()]
        self.h = L.orc_create(ctypes.byref(self.p), *[_p(c) for c in self.coords])
        L.orc_set_integrator(self.h, INTEGRATORS[integrator])
        if multilevel:
            t, cnt, lv, loc = mesh.neighbor_table()
            self._ml = [np.ascontiguousarray(a) for a in (t, cnt, lv, loc)]
            self._cc = [np.ascontiguousarray(c) for c in mesh.coarse_coordinate_arrays()]
            ip = ctypes.POINTER(ctypes.c_int)
            rc = L.orc_set_multilevel(
                self.h, self._ml[0].ctypes.data_as(ip), self._ml[1].ctypes.data_as(ip),
                self._ml[2].ctypes.data_as(ip),
                self._ml[3].ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                *[_p(c) for c in self._cc])
            if rc != 0:
                raise ValueError("unsupported multi-level configuration (%d)" % rc)
        if threads:
            L.orc_num_threads(threads)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_state(self, u, b1, b2, b3):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (u, b1, b2, b3)]
        lib().orc_set_state(self.h, *[_p(a) for a in arrs])

    def set_prim(self, w):
        """Initial primitives (SR: also the first con2prim guess)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        lib().orc_set_prim(self.h, _p(w))

    def state(self):
        m = self.mesh
        u = np.zeros((m.nblocks, 5) + m.cell_shape)
        b = [np.zeros((m.nblocks,) + s) for s in m.face_shapes]
        lib().orc_get_state(self.h, _p(u), *[_p(x) for x in b])
        return u, b[0], b[1], b[2]

    def prim(self):
        m = self.mesh
        w = np.zeros((m.nblocks, 5) + m.cell_shape)
        bcc = np.zeros((m.nblocks, 3) + m.cell_shape)
        lib().orc_get_prim(self.h, _p(w), _p(bcc))
        return w, bcc

    @property
    def dt(self):
        return lib().orc_get_dt(self.h)

    @property
    def time(self):
        return lib().orc_get_time(self.h)

    def initialize(self):
        lib().orc_initialize(self.h)

    def cycle(self, n=1):
        for _ in range(n):
            lib().orc_cycle(self.h)

    def stage(self, s):
        lib().orc_stage(self.h, s)

    # --- per-operator restatements (block b; the checkers of the operator calls) ----
    def _emf_ptrs(self, emf):
        return (ctypes.POINTER(ctypes.c_double) * 9)(*[_p(a) for a in emf])

    def op_fluxes(self, b, order, dt, flx, emf):
        """Hydro::CalculateFluxes of block b into flx (3 arrays) and emf (9 arrays)."""
        lib().orc_op_fluxes(self.h, b, order, dt, _p(flx[0]), _p(flx[1]), _p(flx[2]),
                            self._emf_ptrs(emf))

    def op_corner_e(self, b, emf, e):
        lib().orc_op_corner_e(self.h, b, self._emf_ptrs(emf), _p(e[0]), _p(e[1]), _p(e[2]))

    def op_add_flux_divergence(self, b, wght, flx, u):
        lib().orc_op_add_flux_divergence(self.h, b, wght, _p(flx[0]), _p(flx[1]), _p(flx[2]),
                                         _p(u))

    def op_ct(self, b, wght, e, bf):
        lib().orc_op_ct(self.h, b, wght, _p(e[0]), _p(e[1]), _p(e[2]), _p(bf[0]), _p(bf[1]),
                        _p(bf[2]))

    def op_con2prim(self, b, rng):
        return lib().orc_op_con2prim(self.h, b, *rng)

    def op_new_block_dt(self, b):
        return lib().orc_op_new_block_dt(self.h, b)

    # --- adaptive refinement ---------------------------------------------------------
    def advance(self):
        """The stages of one cycle and time += dt, without the new time step."""
        lib().orc_advance(self.h)

    def new_dt(self):
        lib().orc_new_dt(self.h)

    def boundaries(self):
        """Multi-level mesh: initialize() without the time step."""
        lib().orc_ml_boundaries(self.h)

    def set_clock(self, time, dt):
        lib().orc_set_time(self.h, time)
        lib().orc_set_dt(self.h, dt)

    def refine_eps(self):
        out = np.zeros(self.mesh.nblocks)
        lib().orc_refine_eps(self.h, _p(out))
        return out

    def regrid(self, plan):
        """A new OracleMesh for plan.mesh filled from this one
        (RedistributeAndRefineMeshBlocks), then Mesh::Initialize(2): ghost exchange,
        ProlongateBoundaries, W(U), physical boundaries, NewBlockTimeStep +
        NewTimeStep."""
        new = OracleMesh(plan.mesh, **self.kw)
        ip = ctypes.POINTER(ctypes.c_int)
        arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in
                (plan.newtoold, plan.kind, plan.ffc.reshape(-1))]
        rc = lib().orc_regrid(new.h, self.h, *[a.ctypes.data_as(ip) for a in arrs[:2]],
                              int(plan.ffc.shape[0]), arrs[2].ctypes.data_as(ip))
        if rc != 0:
            raise ValueError("regrid failed (%d)" % rc)
        new.initialize()
        return new


def sr_c2p_cells(cons, bcc, guess, gamma):
    """Per-cell SR con2prim (Newman-Hamlin) on independent cells: cons[n,5] (D, M1..M3,
    E), bcc[n,3], pgas guesses[n] -> prim[n,5], iterations[n] (-1: not converged)."""
    n = cons.shape[0]
    cons = np.ascontiguousarray(cons, dtype=np.float64)
    bcc = np.ascontiguousarray(bcc, dtype=np.float64)
    guess = np.ascontiguousarray(guess, dtype=np.float64)
    prim = np.zeros((n, 5))
    it = np.zeros(n, dtype=np.int32)
    lib().orc_sr_c2p_cells(n, gamma, 0.0, _p(cons), _p(bcc), _p(guess), _p(prim),
                           it.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return prim, it


def sr_prim_to_cons(w, bcc, gamma):
    n = w.shape[0]
    w = np.ascontiguousarray(w, dtype=np.float64)
    bcc = np.ascontiguousarray(bcc, dtype=np.float64)
    u = np.zeros((n, 5))
    lib().orc_sr_prim_to_cons(n, gamma, _p(w), _p(bcc), _p(u))
    return u


def riemann_faces(rsolver, wl, wr, bx, gamma, relativistic=False, dv=None):
    """One Riemann solve per face: wl, wr [n, 7] primitive states in the solvers' local
    order (d, v_n, v_t1, v_t2, p, B_t1, B_t2), bx [n], dv [n, 2] the faces' velocity
    differences (dvn, dvt; LHLLD only) -> flux [n, 7] in the same order."""
    rs = {"hlld": 0, "hlle": 1, "llf": 2, "roe": 3, "lhlld": 4}[rsolver]
    wl = np.ascontiguousarray(wl, dtype=np.float64)
    wr = np.ascontiguousarray(wr, dtype=np.float64)
    out = np.zeros((wl.shape[0], 7))
    L = lib()
    dv = np.zeros((wl.shape[0], 2)) if dv is None else np.asarray(dv, dtype=np.float64)
    for q in range(wl.shape[0]):
        L.orc_riemann_face(rs, 1 if relativistic else 0, gamma, _p(wl[q]), _p(wr[q]),
                           float(bx[q]), float(dv[q, 0]), float(dv[q, 1]), _p(out[q]))
    return out
