"""Problem generators (initial conditions) for the stage-update workloads.

Each generator returns per-block arrays in the layout of :mod:`athena_gb300.mesh`:
``u[nb, 5, nc3, nc2, nc1]`` (conserved: density, momenta, total energy) and face fields
``b1, b2, b3`` (``w`` primitive instead of ``u`` for the relativistic problems).
Ghost zones are left at zero; the stage update fills them by the ghost exchange.

The linear wave restates the reference's ``pgen/linear_wave.cpp`` (InitUserMeshData
:78-188, Eigensystem :626-855, ProblemGenerator :436-585, vector potential A1-A3
:588-624) with the same libm calls, so its arrays are bit-identical to the reference's
when ``exact=True``.  The other generators are seeded synthetic inputs with the shapes,
sizes and value distributions of the benchmark configurations.
"""
import math

import numpy as np

from .mesh import MeshSpec

IDN, IM1, IM2, IM3, IEN = 0, 1, 2, 3, 4
TINY_NUMBER = 1.0e-20


def _sign(x):
    return -1.0 if x < 0.0 else 1.0


def mhd_right_eigenvectors(gm1, d, v1, v2, v3, h, b1, b2, b3, x, y):
    """Adiabatic-MHD eigenvalues and right eigenvectors (columns), the branch of
    Eigensystem in linear_wave.cpp:633-763 used for the MHD linear wave."""
    vsq = v1 * v1 + v2 * v2 + v3 * v3
    btsq = b2 * b2 + b3 * b3
    bt_starsq = (gm1 - (gm1 - 1.0) * y) * btsq
    vaxsq = b1 * b1 / d
    hp = h - (vaxsq + btsq / d)
    twid_asq = max((gm1 * (hp - 0.5 * vsq) - (gm1 - 1.0) * x), TINY_NUMBER)
    ct2 = bt_starsq / d
    tsum = vaxsq + ct2 + twid_asq
    tdif = vaxsq + ct2 - twid_asq
    cf2_cs2 = math.sqrt(tdif * tdif + 4.0 * twid_asq * ct2)
    cfsq = 0.5 * (tsum + cf2_cs2)
    cf = math.sqrt(cfsq)
    cssq = twid_asq * vaxsq / cfsq
    cs = math.sqrt(cssq)
    bt = math.sqrt(btsq)
    bt_star = math.sqrt(bt_starsq)
    if bt == 0.0:
        bet2, bet3 = 1.0, 0.0
    else:
        bet2, bet3 = b2 / bt, b3 / bt
    bet2_star = bet2 / math.sqrt(gm1 - (gm1 - 1.0) * y)
    bet3_star = bet3 / math.sqrt(gm1 - (gm1 - 1.0) * y)
    bet_starsq = bet2_star * bet2_star + bet3_star * bet3_star
    vbet = v2 * bet2_star + v3 * bet3_star
    if (cfsq - cssq) == 0.0:
        alpha_f, alpha_s = 1.0, 0.0
    elif (twid_asq - cssq) <= 0.0:
        alpha_f, alpha_s = 0.0, 1.0
    elif (cfsq - twid_asq) <= 0.0:
        alpha_f, alpha_s = 1.0, 0.0
    else:
        alpha_f = math.sqrt((twid_asq - cssq) / (cfsq - cssq))
        alpha_s = math.sqrt((cfsq - twid_asq) / (cfsq - cssq))
    sqrtd = math.sqrt(d)
    isqrtd = 1.0 / sqrtd
    s = _sign(b1)
    twid_a = math.sqrt(twid_asq)
    qf = cf * alpha_f * s
    qs = cs * alpha_s * s
    af_prime = twid_a * alpha_f * isqrtd
    as_prime = twid_a * alpha_s * isqrtd
    afpbb = af_prime * bt_star * bet_starsq
    aspbb = as_prime * bt_star * bet_starsq
    vax = math.sqrt(vaxsq)
    ev = [v1 - cf, v1 - vax, v1 - cs, v1, v1 + cs, v1 + vax, v1 + cf]
    r = [[0.0] * 7 for _ in range(7)]
    r[0] = [alpha_f, 0.0, alpha_s, 1.0, alpha_s, 0.0, alpha_f]
    r[1] = [alpha_f * ev[0], 0.0, alpha_s * ev[2], v1, alpha_s * ev[4], 0.0,
            alpha_f * ev[6]]
    qa, qb, qc, qd = alpha_f * v2, alpha_s * v2, qs * bet2_star, qf * bet2_star
    r[2] = [qa + qc, -bet3, qb - qd, v2, qb + qd, bet3, qa - qc]
    qa, qb, qc, qd = alpha_f * v3, alpha_s * v3, qs * bet3_star, qf * bet3_star
    r[3] = [qa + qc, bet2, qb - qd, v3, qb + qd, -bet2, qa - qc]
    r41 = -(v2 * bet3 - v3 * bet2)
    r[4] = [alpha_f * (hp - v1 * cf) + qs * vbet + aspbb, r41,
            alpha_s * (hp - v1 * cs) - qf * vbet - afpbb, 0.5 * vsq + (gm1 - 1.0) * x / gm1,
            alpha_s * (hp + v1 * cs) + qf * vbet - afpbb, -r41,
            alpha_f * (hp + v1 * cf) - qs * vbet + aspbb]
    r50, r51, r52 = as_prime * bet2_star, -bet3 * s * isqrtd, -af_prime * bet2_star
    r[5] = [r50, r51, r52, 0.0, r52, r51, r50]
    r60, r61, r62 = as_prime * bet3_star, bet2 * s * isqrtd, -af_prime * bet3_star
    r[6] = [r60, r61, r62, 0.0, r62, r61, r60]
    return ev, r


class LinearWave:
    """Adiabatic-MHD linear wave on a periodic box, wavevector along the grid diagonal
    (linear_wave.cpp:78-188)."""

    def __init__(self, mesh: MeshSpec, gamma=1.666666666666667, wave_flag=0, amp=1.0e-6,
                 vflow=0.0):
        self.mesh, self.gam, self.wave_flag, self.amp = mesh, gamma, wave_flag, amp
        self.gm1 = gamma - 1.0
        x1size = mesh.xmax[0] - mesh.xmin[0]
        x2size = mesh.xmax[1] - mesh.xmin[1]
        x3size = mesh.xmax[2] - mesh.xmin[2]
        ang_3 = math.atan(x1size / x2size)
        self.sin_a3, self.cos_a3 = math.sin(ang_3), math.cos(ang_3)
        ang_2 = math.atan(0.5 * (x1size * self.cos_a3 + x2size * self.sin_a3) / x3size)
        self.sin_a2, self.cos_a2 = math.sin(ang_2), math.cos(ang_2)
        x1 = x1size * self.cos_a2 * self.cos_a3
        x2 = x2size * self.cos_a2 * self.sin_a3
        x3 = x3size * self.sin_a2
        lam = x1
        if ang_3 != 0.0:
            lam = min(lam, x2)
        if ang_2 != 0.0:
            lam = min(lam, x3)
        self.lam = lam
        self.k_par = 2.0 * 3.1415926535897932 / lam
        self.d0, self.u0 = 1.0, vflow
        self.bx0, self.by0, self.bz0 = 1.0, math.sqrt(2.0), 0.5
        self.p0 = 1.0 / gamma
        h0 = ((self.p0 / self.gm1 + 0.5 * self.d0 * (self.u0 * self.u0)) + self.p0) / self.d0
        h0 += (self.bx0 * self.bx0 + self.by0 * self.by0 + self.bz0 * self.bz0) / self.d0
        self.ev, self.rem = mhd_right_eigenvectors(self.gm1, self.d0, self.u0, 0.0, 0.0, h0,
                                                   self.bx0, self.by0, self.bz0, 0.0, 1.0)
        self.dby = amp * self.rem[5][wave_flag]
        self.dbz = amp * self.rem[6][wave_flag]

    def period(self):
        """tlim for problem/test = true with tlim = 1 (linear_wave.cpp:174-179)."""
        return self.lam / abs(self.ev[self.wave_flag]) * 1.0

    def _xy(self, x1, x2, x3):
        x = x1 * self.cos_a2 * self.cos_a3 + x2 * self.cos_a2 * self.sin_a3 + x3 * self.sin_a2
        y = -x1 * self.sin_a3 + x2 * self.cos_a3
        return x, y

    def A1(self, x1, x2, x3):
        x, y = self._xy(x1, x2, x3)
        Ay = self.bz0 * x - (self.dbz / self.k_par) * math.cos(self.k_par * (x))
        Az = -self.by0 * x + (self.dby / self.k_par) * math.cos(self.k_par * (x)) + \
            self.bx0 * y
        return -Ay * self.sin_a3 - Az * self.sin_a2 * self.cos_a3

    def A2(self, x1, x2, x3):
        x, y = self._xy(x1, x2, x3)
        Ay = self.bz0 * x - (self.dbz / self.k_par) * math.cos(self.k_par * (x))
        Az = -self.by0 * x + (self.dby / self.k_par) * math.cos(self.k_par * (x)) + \
            self.bx0 * y
        return Ay * self.cos_a3 - Az * self.sin_a2 * self.sin_a3

    def A3(self, x1, x2, x3):
        x, y = self._xy(x1, x2, x3)
        Az = -self.by0 * x + (self.dby / self.k_par) * math.cos(self.k_par * (x)) + \
            self.bx0 * y
        return Az * self.cos_a2

    def generate(self):
        """Per-block u, b1, b2, b3 (ProblemGenerator, linear_wave.cpp:436-585)."""
        m = self.mesh
        ng = m.ng
        n1, n2, n3 = m.bx
        u = np.zeros((m.nblocks, 5) + m.cell_shape)
        b1 = np.zeros((m.nblocks,) + m.face_shapes[0])
        b2 = np.zeros((m.nblocks,) + m.face_shapes[1])
        b3 = np.zeros((m.nblocks,) + m.face_shapes[2])
        wf, amp, rem = self.wave_flag, self.amp, self.rem
        for b in range(m.nblocks):
            l1, l2, l3 = m.block_loc(b)
            x1f, dx1f = m.face_coords(0, l1)
            x2f, dx2f = m.face_coords(1, l2)
            x3f, dx3f = m.face_coords(2, l3)
            x1v, x2v, x3v = m.cell_centers(0, l1), m.cell_centers(1, l2), m.cell_centers(2, l3)
            sh = (n3 + 1, n2 + 1, n1 + 1)
            a1, a2, a3 = np.zeros(sh), np.zeros(sh), np.zeros(sh)
            for kk in range(n3 + 1):
                k = ng + kk
                for jj in range(n2 + 1):
                    j = ng + jj
                    for ii in range(n1 + 1):
                        i = ng + ii
                        a1[kk, jj, ii] = self.A1(x1v[i], x2f[j], x3f[k])
                        a2[kk, jj, ii] = self.A2(x1f[i], x2v[j], x3f[k])
                        a3[kk, jj, ii] = self.A3(x1f[i], x2f[j], x3v[k])
            for kk in range(n3):
                for jj in range(n2):
                    for ii in range(n1 + 1):
                        b1[b, ng + kk, ng + jj, ng + ii] = \
                            (a3[kk, jj + 1, ii] - a3[kk, jj, ii]) / dx2f[ng + jj] - \
                            (a2[kk + 1, jj, ii] - a2[kk, jj, ii]) / dx3f[ng + kk]
            for kk in range(n3):
                for jj in range(n2 + 1):
                    for ii in range(n1):
                        b2[b, ng + kk, ng + jj, ng + ii] = \
                            (a1[kk + 1, jj, ii] - a1[kk, jj, ii]) / dx3f[ng + kk] - \
                            (a3[kk, jj, ii + 1] - a3[kk, jj, ii]) / dx1f[ng + ii]
            for kk in range(n3 + 1):
                for jj in range(n2):
                    for ii in range(n1):
                        b3[b, ng + kk, ng + jj, ng + ii] = \
                            (a2[kk, jj, ii + 1] - a2[kk, jj, ii]) / dx1f[ng + ii] - \
                            (a1[kk, jj + 1, ii] - a1[kk, jj, ii]) / dx2f[ng + jj]
            ca2, sa2, ca3, sa3 = self.cos_a2, self.sin_a2, self.cos_a3, self.sin_a3
            for kk in range(n3):
                k = ng + kk
                for jj in range(n2):
                    j = ng + jj
                    for ii in range(n1):
                        i = ng + ii
                        x = ca2 * (x1v[i] * ca3 + x2v[j] * sa3) + x3v[k] * sa2
                        sn = math.sin(self.k_par * x)
                        u[b, IDN, k, j, i] = self.d0 + amp * sn * rem[0][wf]
                        mx = self.d0 * self.u0 + amp * sn * rem[1][wf]
                        my = amp * sn * rem[2][wf]
                        mz = amp * sn * rem[3][wf]
                        u[b, IM1, k, j, i] = mx * ca2 * ca3 - my * sa3 - mz * sa2 * ca3
                        u[b, IM2, k, j, i] = mx * ca2 * sa3 + my * ca3 - mz * sa2 * sa3
                        u[b, IM3, k, j, i] = mx * sa2 + mz * ca2
                        e = self.p0 / self.gm1 + 0.5 * self.d0 * self.u0 * self.u0 + \
                            amp * sn * rem[4][wf]
                        e += 0.5 * (self.bx0 * self.bx0 + self.by0 * self.by0 +
                                    self.bz0 * self.bz0)
                        u[b, IEN, k, j, i] = e
        return u, b1, b2, b3

    def l1_errors(self, u, bcc):
        """L1 errors of cell-centred conserved variables and fields against the initial
        wave (Mesh::UserWorkAfterLoop, linear_wave.cpp:190-424).  Returns
        (rms_l1, l1[8], max[8])."""
        m = self.mesh
        ng = m.ng
        n1, n2, n3 = m.bx
        l1 = np.zeros(8)
        mx_err = np.zeros(8)
        wf, amp, rem = self.wave_flag, self.amp, self.rem
        ca2, sa2, ca3, sa3 = self.cos_a2, self.sin_a2, self.cos_a3, self.sin_a3
        for b in range(m.nblocks):
            l1b, l2b, l3b = m.block_loc(b)
            x1v, x2v, x3v = m.cell_centers(0, l1b), m.cell_centers(1, l2b), \
                m.cell_centers(2, l3b)
            _, dx1f = m.face_coords(0, l1b)
            _, dx2f = m.face_coords(1, l2b)
            _, dx3f = m.face_coords(2, l3b)
            for k in range(ng, ng + n3):
                for j in range(ng, ng + n2):
                    for i in range(ng, ng + n1):
                        x = ca2 * (x1v[i] * ca3 + x2v[j] * sa3) + x3v[k] * sa2
                        sn = math.sin(self.k_par * x)
                        d1 = self.d0 + amp * sn * rem[0][wf]
                        mx = self.d0 * self.u0 + amp * sn * rem[1][wf]
                        my = amp * sn * rem[2][wf]
                        mz = amp * sn * rem[3][wf]
                        m1 = mx * ca2 * ca3 - my * sa3 - mz * sa2 * ca3
                        m2 = mx * ca2 * sa3 + my * ca3 - mz * sa2 * sa3
                        m3 = mx * sa2 + mz * ca2
                        e0 = self.p0 / self.gm1 + 0.5 * self.d0 * self.u0 * self.u0 + \
                            amp * sn * rem[4][wf]
                        e0 += 0.5 * (self.bx0 * self.bx0 + self.by0 * self.by0 +
                                     self.bz0 * self.bz0)
                        bx = self.bx0
                        by = self.by0 + amp * sn * rem[5][wf]
                        bz = self.bz0 + amp * sn * rem[6][wf]
                        bb1 = bx * ca2 * ca3 - by * sa3 - bz * sa2 * ca3
                        bb2 = bx * ca2 * sa3 + by * ca3 - bz * sa2 * sa3
                        bb3 = bx * sa2 + bz * ca2
                        vol = dx1f[i] * dx2f[j] * dx3f[k]
                        ref = (d1, m1, m2, m3, e0)
                        for n in range(5):
                            err = abs(ref[n] - u[b, n, k, j, i])
                            l1[n] += err * vol
                            mx_err[n] = max(err, mx_err[n])
                        for n, bref in enumerate((bb1, bb2, bb3)):
                            err = abs(bref - bcc[b, n, k, j, i])
                            l1[5 + n] += err * vol
                            mx_err[5 + n] = max(err, mx_err[5 + n])
        vol = (m.xmax[0] - m.xmin[0]) * (m.xmax[1] - m.xmin[1]) * (m.xmax[2] - m.xmin[2])
        l1 = l1 / vol
        rms = math.sqrt(sum(v * v for v in l1))
        return rms, l1, mx_err


def prim_to_cons(w, bcc, gamma):
    """Newtonian adiabatic MHD W -> U (EquationOfState::PrimitiveToConserved,
    adiabatic_mhd.cpp:99-136)."""
    igm1 = 1.0 / (gamma - 1.0)
    u = np.empty_like(w)
    d, vx, vy, vz, p = w
    u[0] = d
    u[1] = vx * d
    u[2] = vy * d
    u[3] = vz * d
    u[4] = p * igm1 + 0.5 * (d * (vx * vx + vy * vy + vz * vz) +
                             (bcc[0] * bcc[0] + bcc[1] * bcc[1] + bcc[2] * bcc[2]))
    return u


def faces_from_uniform(nx, b):
    """Global face arrays of a uniform field b = (b1, b2, b3)."""
    n1, n2, n3 = nx
    return (np.full((n3, n2, n1 + 1), b[0]), np.full((n3, n2 + 1, n1), b[1]),
            np.full((n3 + 1, n2, n1), b[2]))


def cell_centered(f1, f2, f3):
    """Uniform-mesh cell-centred field from global face arrays (field.cpp:112-180)."""
    return np.stack([0.5 * f1[:, :, :-1] + 0.5 * f1[:, :, 1:],
                     0.5 * f2[:, :-1, :] + 0.5 * f2[:, 1:, :],
                     0.5 * f3[:-1, :, :] + 0.5 * f3[1:, :, :]])


def solenoidal_velocity(nx, kmin, kmax, seed):
    """Seeded random-phase solenoidal field with power in kmin <= |k| <= kmax (integer
    wavenumbers of the periodic box), unit rms.  Returns v[3, NX3, NX2, NX1]."""
    n1, n2, n3 = nx
    rng = np.random.default_rng(seed)
    k3 = np.fft.fftfreq(n3, 1.0 / n3)[:, None, None]
    k2 = np.fft.fftfreq(n2, 1.0 / n2)[None, :, None]
    k1 = np.fft.rfftfreq(n1, 1.0 / n1)[None, None, :]
    kk = np.sqrt(k1 * k1 + k2 * k2 + k3 * k3)
    shell = (kk >= kmin) & (kk <= kmax)
    shape = kk.shape
    vk = []
    for _ in range(3):
        amp = rng.standard_normal(shape)
        ph = rng.uniform(0.0, 2.0 * np.pi, shape)
        vk.append(np.where(shell, amp * np.exp(1j * ph), 0.0))
    kvec = (k1 + 0 * k2 + 0 * k3, k2 + 0 * k1 + 0 * k3, k3 + 0 * k1 + 0 * k2)
    ksq = np.where(kk > 0, kk * kk, 1.0)
    div = (kvec[0] * vk[0] + kvec[1] * vk[1] + kvec[2] * vk[2]) / ksq
    vk = [vk[d] - kvec[d] * div for d in range(3)]
    v = np.stack([np.fft.irfftn(vk[d], s=(n3, n2, n1), axes=(0, 1, 2)) for d in range(3)])
    rms = np.sqrt(np.mean(np.sum(v * v, axis=0)))
    return v / rms


def turbulence(nx, seed=20261204, gamma=5.0 / 3.0, mach=1.0, beta=1.0, p0=1.0,
               kmin=1.0, kmax=4.0):
    """Decaying-MHD-turbulence initial state on a periodic unit box: rho = 1, uniform
    B along x with plasma beta = 2 p / B^2, seeded solenoidal velocity with power in
    kmin <= |k| <= kmax scaled to rms Mach `mach`.  Global arrays (u, f1, f2, f3)."""
    bx = np.sqrt(2.0 * p0 / beta)
    cs = np.sqrt(gamma * p0 / 1.0)
    v = solenoidal_velocity(nx, kmin, kmax, seed) * (mach * cs)
    n1, n2, n3 = nx
    w = np.empty((5, n3, n2, n1))
    w[0] = 1.0
    w[1:4] = v
    w[4] = p0
    f1, f2, f3 = faces_from_uniform(nx, (bx, 0.0, 0.0))
    u = prim_to_cons(w, cell_centered(f1, f2, f3), gamma)
    return u, f1, f2, f3


def blast(nx, xmin=(-0.5, -0.5, -0.5), xmax=(0.5, 0.5, 0.5), gamma=5.0 / 3.0, p_in=10.0,
          p_out=0.1, radius=0.1, b=(1.0 / np.sqrt(2.0),) * 3):
    """MHD blast wave: rho = 1, p = p_in inside r < radius, p_out outside, uniform B
    (components b).  Global arrays (u, f1, f2, f3)."""
    n1, n2, n3 = nx
    xs = [xmin[d] + (np.arange(nx[d]) + 0.5) * (xmax[d] - xmin[d]) / nx[d] for d in range(3)]
    r = np.sqrt(xs[0][None, None, :] ** 2 + xs[1][None, :, None] ** 2 +
                xs[2][:, None, None] ** 2)
    w = np.zeros((5, n3, n2, n1))
    w[0] = 1.0
    w[4] = np.where(r < radius, p_in, p_out)
    f1, f2, f3 = faces_from_uniform(nx, b)
    return prim_to_cons(w, cell_centered(f1, f2, f3), gamma), f1, f2, f3


# ---------------------------------------------------------------------------------------
# Special-relativistic MHD states.  Primitives are (rho, u1, u2, u3, p) with u^i = gamma
# v^i, the reference's SR convention (adiabatic_mhd_sr.cpp:489-520).

def sr_prim_to_cons(w, bcc, gamma):
    """SR-MHD W -> U (EquationOfState::PrimitiveToConserved, adiabatic_mhd_sr.cpp:284-332),
    elementwise in the reference's operand order.  w[5, ...], bcc[3, ...]."""
    gamma_adi_red = gamma / (gamma - 1.0)
    rho, u1, u2, u3, pgas = w[0], w[1], w[2], w[3], w[4]
    bb1, bb2, bb3 = bcc[0], bcc[1], bcc[2]
    u0 = np.sqrt(1.0 + u1 * u1 + u2 * u2 + u3 * u3)
    b0 = bb1 * u1 + bb2 * u2 + bb3 * u3
    b1 = (bb1 + b0 * u1) / u0
    b2 = (bb2 + b0 * u2) / u0
    b3 = (bb3 + b0 * u3) / u0
    b_sq = -(b0 * b0) + b1 * b1 + b2 * b2 + b3 * b3
    wtot_u02 = (rho + gamma_adi_red * pgas + b_sq) * u0 * u0
    u = np.empty_like(w)
    u[0] = rho * u0
    u[4] = wtot_u02 - b0 * b0 - (pgas + 0.5 * b_sq)
    u[1] = wtot_u02 * u1 / u0 - b0 * b1
    u[2] = wtot_u02 * u2 / u0 - b0 * b2
    u[3] = wtot_u02 * u3 / u0 - b0 * b3
    return u


def sr_shock_tube(nx, xmin, xmax, left, right, shock_pos=0.0):
    """Relativistic MHD shock tube along x1 (pgen/gr_shock_tube.cpp:44-330, SR branch):
    left/right = (rho, p, v^x, v^y, v^z, B^x, B^y, B^z) with 3-velocities, cell (k,j,i) on
    the left where x1v(i) < shock_pos.  The face fields take the state of the cell of the
    same index (x1v(i) decides face i too, :248-262, the last face that of the next ghost
    cell).  Returns global primitives w[5, NX3, NX2, NX1] (4-velocity u^i = u^0 v^i) and
    the face fields (f1, f2, f3)."""
    n1, n2, n3 = nx
    dx = (xmax[0] - xmin[0]) / n1
    xf = xmin[0] + dx * np.arange(n1 + 2)
    x1v = 0.5 * (xf[:-1] + xf[1:])            # cell centres of cells 0..n1 (n1: ghost)
    side = x1v < shock_pos                    # True: left state

    def state(q):
        rho, p, vx, vy, vz, bx, by, bz = q
        ut = np.sqrt(1.0 / (1.0 - (vx * vx + vy * vy + vz * vz)))
        return rho, p, ut * vx, ut * vy, ut * vz, bx, by, bz

    L, R = state(left), state(right)
    cols = np.array([L if s else R for s in side])   # [n1+1, 8]
    w = np.empty((5, n3, n2, n1))
    for n in range(5):
        src = {0: 0, 1: 2, 2: 3, 3: 4, 4: 1}[n]      # rho, u1, u2, u3, p
        w[n] = cols[:n1, src][None, None, :]
    f1 = np.broadcast_to(cols[:, 5][None, None, :], (n3, n2, n1 + 1)).copy()
    f2 = np.broadcast_to(cols[:n1, 6][None, None, :], (n3, n2 + 1, n1)).copy()
    f3 = np.broadcast_to(cols[:n1, 7][None, None, :], (n3 + 1, n2, n1)).copy()
    return w, f1, f2, f3


def sr_kelvin_helmholtz(nx, seed=20261204, gamma=4.0 / 3.0, vshear=0.5, width=0.01,
                        rho_in=1.0, rho_out=0.1, p0=1.0, sigma=0.1, noise=1.0e-3):
    """Relativistic Kelvin-Helmholtz shear layer on a periodic unit box: v_x = +vshear
    for |y - 1/2| < 1/4 and -vshear outside, with tanh transitions of the given width,
    density rho_in inside / rho_out outside, uniform pressure p0, uniform B_x with
    magnetization sigma = B^2 / (rho_in h) of the inner layer, and seeded velocity noise.
    Returns global primitives w[5, NX3, NX2, NX1] and face fields (f1, f2, f3)."""
    n1, n2, n3 = nx
    rng = np.random.default_rng(seed)
    y = (np.arange(n2) + 0.5) / n2
    prof = 0.5 * (np.tanh((y - 0.25) / width) - np.tanh((y - 0.75) / width))  # 1 inside
    vx = (-vshear + 2.0 * vshear * prof)[None, :, None] * np.ones((n3, n2, n1))
    rho = (rho_out + (rho_in - rho_out) * prof)[None, :, None] * np.ones((n3, n2, n1))
    vx = vx + noise * rng.uniform(-1.0, 1.0, (n3, n2, n1))
    vy = noise * rng.uniform(-1.0, 1.0, (n3, n2, n1))
    vz = noise * rng.uniform(-1.0, 1.0, (n3, n2, n1))
    lor = 1.0 / np.sqrt(1.0 - (vx * vx + vy * vy + vz * vz))
    h = 1.0 + gamma / (gamma - 1.0) * p0 / rho_in
    bx = np.sqrt(sigma * rho_in * h)
    w = np.empty((5, n3, n2, n1))
    w[0] = rho
    w[1], w[2], w[3] = lor * vx, lor * vy, lor * vz
    w[4] = p0
    f1, f2, f3 = faces_from_uniform(nx, (bx, 0.0, 0.0))
    return w, f1, f2, f3


def sr_isolated_cells(n, seed=20261204, gamma=4.0 / 3.0, lorentz=(1.0, 10.0),
                      sigma=(1.0e-2, 1.0e2), rho=(1.0e-4, 1.0), p_over_rho=(1.0e-3, 10.0)):
    """Independent SR-MHD cells for the con2prim benchmark: Lorentz factor, magnetization
    sigma = b^2/(rho h), rho and p/rho log-uniform in the given ranges, isotropic
    directions of v and B.  Returns primitives w[n, 5] (rho, u1, u2, u3, p), lab-frame
    field bcc[n, 3] and conserved u[n, 5] (D, M1, M2, M3, E)."""
    rng = np.random.default_rng(seed)

    def logu(lo_hi):
        lo, hi = lo_hi
        return np.exp(rng.uniform(np.log(lo), np.log(hi), n))

    def unit():
        v = rng.standard_normal((n, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    lor = logu(lorentz)
    sig = logu(sigma)
    d = logu(rho)
    p = d * logu(p_over_rho)
    uvec = np.sqrt(lor * lor - 1.0)[:, None] * unit()
    bdir = unit()
    h = 1.0 + gamma / (gamma - 1.0) * p / d
    # comoving b^2 = sigma rho h; for lab field B along bdir with b^2 = (B^2 + (B.u)^2)/lor^2
    bu = np.einsum("ij,ij->i", bdir, uvec)
    bmag = np.sqrt(sig * d * h * lor * lor / (1.0 + bu * bu))
    bcc = bmag[:, None] * bdir
    w = np.stack([d, uvec[:, 0], uvec[:, 1], uvec[:, 2], p], axis=1)
    u = sr_prim_to_cons(w.T, bcc.T, gamma).T
    return w, bcc, u


def blast_blocks(mesh, gamma=5.0 / 3.0, radius=0.1, pamb=1.0, damb=1.0, prat=100.0,
                 drat=1.0, b0=1.0, angle_deg=45.0, center=(0.0, 0.0, 0.0), bfield=None):
    """The reference's blast problem generator (pgen/blast.cpp:53-213, Cartesian, no
    ramp) evaluated on every block of a mesh with per-block coordinates (a
    MultiLevelMesh): rho = drat*damb and p = prat*pamb inside r < radius, damb and pamb
    outside, zero velocity, face field (b0 cos a, b0 sin a, 0), E = p/(gamma-1) + b0^2/2.
    bfield = (bx, by, bz) replaces the planar field by that uniform field (E then adds
    |B|^2/2).  Returns per-block (u, b1, b2, b3), interior cells and faces set, ghosts
    zero."""
    ng, (n1, n2, n3) = mesh.ng, mesh.bx
    gm1 = gamma - 1.0
    angle = (3.14159265358979323846 / 180.0) * angle_deg   # PI, defs.hpp.in
    u = np.zeros((mesh.nblocks, 5) + mesh.cell_shape)
    f = [np.zeros((mesh.nblocks,) + s) for s in mesh.face_shapes]
    bx, by, bz = b0 * math.cos(angle), b0 * math.sin(angle), 0.0
    emag = 0.5 * b0 * b0
    if bfield is not None:
        bx, by, bz = (float(v) for v in bfield)
        emag = 0.5 * (bx * bx + by * by + bz * bz)
    for b in range(mesh.nblocks):
        xv = [mesh.cell_centers(b, d) for d in range(3)]
        x = xv[0][ng:ng + n1][None, None, :] - center[0]
        y = xv[1][ng:ng + n2][None, :, None] - center[1]
        z = xv[2][ng:ng + n3][:, None, None] - center[2]
        rad = np.sqrt(x * x + y * y + z * z)
        inside = rad < radius
        u[b, 0, ng:ng + n3, ng:ng + n2, ng:ng + n1] = np.where(inside, drat * damb, damb)
        pres = np.where(inside, prat * pamb, pamb)
        u[b, 4, ng:ng + n3, ng:ng + n2, ng:ng + n1] = pres / gm1 + emag
        f[0][b, ng:ng + n3, ng:ng + n2, ng:ng + n1 + 1] = bx
        f[1][b, ng:ng + n3, ng:ng + n2 + 1, ng:ng + n1] = by
        f[2][b, ng:ng + n3 + 1, ng:ng + n2, ng:ng + n1] = bz
    return u, f[0], f[1], f[2]


def smooth_blocks(mesh, gamma=5.0 / 3.0, seed=7, amp=0.2):
    """A smooth non-uniform MHD state on every block of a mesh with per-block
    coordinates: density, pressure and velocity with a few random-phase Fourier modes of
    the cell-centre position, and a face field sampled from a smooth analytic field at
    the face centres.  Per-block (u, b1, b2, b3), interior cells and faces set."""
    rng = np.random.default_rng(seed)
    ng, (n1, n2, n3) = mesh.ng, mesh.bx
    L = [mesh.xmax[d] - mesh.xmin[d] for d in range(3)]
    modes = []
    for _ in range(4):
        k = rng.integers(1, 3, size=3) * 2.0 * np.pi / np.array(L)
        modes.append((k, rng.uniform(0, 2 * np.pi), rng.normal(size=8)))

    def field(x, y, z, c):
        out = 0.0
        for k, ph, a in modes:
            out = out + a[c] * np.sin(k[0] * x + k[1] * y + k[2] * z + ph)
        return out

    u = np.zeros((mesh.nblocks, 5) + mesh.cell_shape)
    f = [np.zeros((mesh.nblocks,) + s) for s in mesh.face_shapes]
    for b in range(mesh.nblocks):
        xf = [mesh._faces(b, d, False)[0] for d in range(3)]
        xv = [0.5 * (xf[d][1:] + xf[d][:-1]) for d in range(3)]
        x = xv[0][ng:ng + n1][None, None, :]
        y = xv[1][ng:ng + n2][:, None][None]
        z = xv[2][ng:ng + n3][:, None, None]
        rho = 1.0 + amp * field(x, y, z, 0) * 0.3
        p = 1.0 + amp * field(x, y, z, 1) * 0.3
        v = [amp * field(x, y, z, 2 + c) for c in range(3)]
        # face fields at face centres: x1 faces at (x1f, x2v, x3v), ...
        fx = [xf[0][ng:ng + n1 + 1][None, None, :], y, z]
        b1 = 1.0 + amp * field(fx[0], fx[1], fx[2], 5)
        fy = [x, xf[1][ng:ng + n2 + 1][None, :, None], z]
        b2 = 0.5 + amp * field(fy[0], fy[1], fy[2], 6)
        fz = [x, y, xf[2][ng:ng + n3 + 1][:, None, None]]
        b3 = 0.25 + amp * field(fz[0], fz[1], fz[2], 7)
        f[0][b, ng:ng + n3, ng:ng + n2, ng:ng + n1 + 1] = b1
        f[1][b, ng:ng + n3, ng:ng + n2 + 1, ng:ng + n1] = b2
        f[2][b, ng:ng + n3 + 1, ng:ng + n2, ng:ng + n1] = b3
        bc1 = 0.5 * (b1[:, :, 1:] + b1[:, :, :-1])
        bc2 = 0.5 * (b2[:, 1:, :] + b2[:, :-1, :])
        bc3 = 0.5 * (b3[1:] + b3[:-1])
        sl = (b, slice(None), slice(ng, ng + n3), slice(ng, ng + n2), slice(ng, ng + n1))
        u[sl][0] = rho
        for c in range(3):
            u[sl][1 + c] = rho * v[c]
        u[sl][4] = p / (gamma - 1.0) + 0.5 * rho * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2) + \
            0.5 * (bc1 ** 2 + bc2 ** 2 + bc3 ** 2)
    return u, f[0], f[1], f[2]
