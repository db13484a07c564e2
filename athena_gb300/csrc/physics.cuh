// Device physics of the MHD stage update: equation of state, reconstruction, Riemann
// solvers.  Templated on the bulk arithmetic type Real (double for the FP64 path, float
// for the FP32 path).  Every function keeps the operand order and grouping of the
// reference routine it cites, so that the FP64 instantiation compiled without FMA
// contraction (-fmad=false) reproduces the reference's results bit for bit.
#pragma once
#include <cuda_runtime.h>

namespace athgpu {

enum { IDN = 0, IVX = 1, IVY = 2, IVZ = 3, IPR = 4, IBY = 5, IBZ = 6, NWAVE = 7 };
enum { NHYDRO = 5 };

#define RC(x) static_cast<Real>(x)

// std::min / std::max semantics: first argument unless the second is strictly
// smaller / larger
template <typename Real>
__device__ __forceinline__ Real smin(Real a, Real b) { return (b < a) ? b : a; }
template <typename Real>
__device__ __forceinline__ Real smax(Real a, Real b) { return (a < b) ? b : a; }
template <typename Real>
__device__ __forceinline__ Real sgn(Real x) { return (x < RC(0.0)) ? RC(-1.0) : RC(1.0); }

__device__ __forceinline__ double dsqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float dsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double dabs(double x) { return fabs(x); }
__device__ __forceinline__ float dabs(float x) { return fabsf(x); }

// EquationOfState::FastMagnetosonicSpeed, eos/adiabatic_mhd.cpp:149-156
template <typename Real>
__device__ __forceinline__ Real fast_ms(Real gamma, Real d, Real p, Real by, Real bz,
                                        Real bx) {
  Real asq = gamma * p;
  Real vaxsq = bx * bx;
  Real ct2 = (by * by + bz * bz);
  Real qsq = vaxsq + ct2 + asq;
  Real tmp = vaxsq + ct2 - asq;
  return dsqrt(RC(0.5) * (qsq + dsqrt(tmp * tmp + RC(4.0) * asq * ct2)) / d);
}

// Hydro::GetWeightForCT, hydro/hydro.cpp:154-158
template <typename Real>
__device__ __forceinline__ Real weight_for_ct(Real dflx, Real rhol, Real rhor, Real dx,
                                              Real dt) {
  Real v_over_c = (RC(1024.0)) * dt * dflx / (dx * (rhol + rhor));
  Real tmp_min = smin(RC(0.5), v_over_c);
  return RC(0.5) + smax(RC(-0.5), tmp_min);
}

// Riemann solvers.  wl/wr: local order (d, v_normal, v_t1, v_t2, p, By, Bz)
// (hlld.cpp:59-75).  f[0..4]: mass, normal, two transverse momentum and energy fluxes;
// f[5] = F(By), f[6] = F(Bz).
template <typename Real>
struct Cons1D { Real d, mx, my, mz, e, by, bz; };

// HLLD (Miyoshi & Kusano 2005), hydro/rsolvers/mhd/hlld.cpp:36-376
template <typename Real>
__device__ __forceinline__ void hlld(Real gamma, const Real* wli, const Real* wri, Real bxi,
                                     Real* f) {
  const Real SMALL_NUMBER = RC(1.0e-4);
  Real igm1 = RC(1.0) / (gamma - RC(1.0));
  Cons1D<Real> ul, ur, ulst, uldst, urdst, urst, fl, fr;
  Real spd[5];
  Real bxsq = bxi * bxi;
  Real pbl = RC(0.5) * (bxsq + (wli[IBY] * wli[IBY] + wli[IBZ] * wli[IBZ]));
  Real pbr = RC(0.5) * (bxsq + (wri[IBY] * wri[IBY] + wri[IBZ] * wri[IBZ]));
  Real kel = RC(0.5) * wli[IDN] *
             (wli[IVX] * wli[IVX] + (wli[IVY] * wli[IVY] + wli[IVZ] * wli[IVZ]));
  Real ker = RC(0.5) * wri[IDN] *
             (wri[IVX] * wri[IVX] + (wri[IVY] * wri[IVY] + wri[IVZ] * wri[IVZ]));
  ul.d = wli[IDN];
  ul.mx = wli[IVX] * ul.d;
  ul.my = wli[IVY] * ul.d;
  ul.mz = wli[IVZ] * ul.d;
  ul.e = wli[IPR] * igm1 + kel + pbl;
  ul.by = wli[IBY];
  ul.bz = wli[IBZ];
  ur.d = wri[IDN];
  ur.mx = wri[IVX] * ur.d;
  ur.my = wri[IVY] * ur.d;
  ur.mz = wri[IVZ] * ur.d;
  ur.e = wri[IPR] * igm1 + ker + pbr;
  ur.by = wri[IBY];
  ur.bz = wri[IBZ];

  Real cfl = fast_ms(gamma, wli[IDN], wli[IPR], wli[IBY], wli[IBZ], bxi);
  Real cfr = fast_ms(gamma, wri[IDN], wri[IPR], wri[IBY], wri[IBZ], bxi);
  spd[0] = smin(wli[IVX] - cfl, wri[IVX] - cfr);
  spd[4] = smax(wli[IVX] + cfl, wri[IVX] + cfr);

  Real ptl = wli[IPR] + pbl;
  Real ptr = wri[IPR] + pbr;
  fl.d = ul.mx;
  fl.mx = ul.mx * wli[IVX] + ptl - bxsq;
  fl.my = ul.my * wli[IVX] - bxi * ul.by;
  fl.mz = ul.mz * wli[IVX] - bxi * ul.bz;
  fl.e = wli[IVX] * (ul.e + ptl - bxsq) - bxi * (wli[IVY] * ul.by + wli[IVZ] * ul.bz);
  fl.by = ul.by * wli[IVX] - bxi * wli[IVY];
  fl.bz = ul.bz * wli[IVX] - bxi * wli[IVZ];
  fr.d = ur.mx;
  fr.mx = ur.mx * wri[IVX] + ptr - bxsq;
  fr.my = ur.my * wri[IVX] - bxi * ur.by;
  fr.mz = ur.mz * wri[IVX] - bxi * ur.bz;
  fr.e = wri[IVX] * (ur.e + ptr - bxsq) - bxi * (wri[IVY] * ur.by + wri[IVZ] * ur.bz);
  fr.by = ur.by * wri[IVX] - bxi * wri[IVY];
  fr.bz = ur.bz * wri[IVX] - bxi * wri[IVZ];

  Real sdl = spd[0] - wli[IVX];
  Real sdr = spd[4] - wri[IVX];
  spd[2] = (sdr * ur.mx - sdl * ul.mx + (ptl - ptr)) / (sdr * ur.d - sdl * ul.d);
  Real sdml = spd[0] - spd[2];
  Real sdmr = spd[4] - spd[2];
  Real sdml_inv = RC(1.0) / sdml;
  Real sdmr_inv = RC(1.0) / sdmr;
  ulst.d = ul.d * sdl * sdml_inv;
  urst.d = ur.d * sdr * sdmr_inv;
  Real ulst_d_inv = RC(1.0) / ulst.d;
  Real urst_d_inv = RC(1.0) / urst.d;
  Real sqrtdl = dsqrt(ulst.d);
  Real sqrtdr = dsqrt(urst.d);
  spd[1] = spd[2] - dabs(bxi) / sqrtdl;
  spd[3] = spd[2] + dabs(bxi) / sqrtdr;

  Real ptstl = ptl + ul.d * sdl * (spd[2] - wli[IVX]);
  Real ptstr = ptr + ur.d * sdr * (spd[2] - wri[IVX]);
  Real ptst = RC(0.5) * (ptstr + ptstl);

  ulst.mx = ulst.d * spd[2];
  if (dabs(ul.d * sdl * sdml - bxsq) < (SMALL_NUMBER)*ptst) {
    ulst.my = ulst.d * wli[IVY];
    ulst.mz = ulst.d * wli[IVZ];
    ulst.by = ul.by;
    ulst.bz = ul.bz;
  } else {
    Real tmp = bxi * (sdl - sdml) / (ul.d * sdl * sdml - bxsq);
    ulst.my = ulst.d * (wli[IVY] - ul.by * tmp);
    ulst.mz = ulst.d * (wli[IVZ] - ul.bz * tmp);
    tmp = (ul.d * (sdl * sdl) - bxsq) / (ul.d * sdl * sdml - bxsq);
    ulst.by = ul.by * tmp;
    ulst.bz = ul.bz * tmp;
  }
  Real vbstl = (ulst.mx * bxi + (ulst.my * ulst.by + ulst.mz * ulst.bz)) * ulst_d_inv;
  ulst.e = (sdl * ul.e - ptl * wli[IVX] + ptst * spd[2] +
            bxi * (wli[IVX] * bxi + (wli[IVY] * ul.by + wli[IVZ] * ul.bz) - vbstl)) *
           sdml_inv;

  urst.mx = urst.d * spd[2];
  if (dabs(ur.d * sdr * sdmr - bxsq) < (SMALL_NUMBER)*ptst) {
    urst.my = urst.d * wri[IVY];
    urst.mz = urst.d * wri[IVZ];
    urst.by = ur.by;
    urst.bz = ur.bz;
  } else {
    Real tmp = bxi * (sdr - sdmr) / (ur.d * sdr * sdmr - bxsq);
    urst.my = urst.d * (wri[IVY] - ur.by * tmp);
    urst.mz = urst.d * (wri[IVZ] - ur.bz * tmp);
    tmp = (ur.d * (sdr * sdr) - bxsq) / (ur.d * sdr * sdmr - bxsq);
    urst.by = ur.by * tmp;
    urst.bz = ur.bz * tmp;
  }
  Real vbstr = (urst.mx * bxi + (urst.my * urst.by + urst.mz * urst.bz)) * urst_d_inv;
  urst.e = (sdr * ur.e - ptr * wri[IVX] + ptst * spd[2] +
            bxi * (wri[IVX] * bxi + (wri[IVY] * ur.by + wri[IVZ] * ur.bz) - vbstr)) *
           sdmr_inv;

  Real invsumd = RC(1.0) / (sqrtdl + sqrtdr);
  Real bxsig = (bxi > RC(0.0) ? RC(1.0) : RC(-1.0));
  uldst.d = ulst.d;
  urdst.d = urst.d;
  uldst.mx = ulst.mx;
  urdst.mx = urst.mx;
  Real tmp = invsumd * (sqrtdl * (ulst.my * ulst_d_inv) + sqrtdr * (urst.my * urst_d_inv) +
                        bxsig * (urst.by - ulst.by));
  uldst.my = uldst.d * tmp;
  urdst.my = urdst.d * tmp;
  tmp = invsumd * (sqrtdl * (ulst.mz * ulst_d_inv) + sqrtdr * (urst.mz * urst_d_inv) +
                   bxsig * (urst.bz - ulst.bz));
  uldst.mz = uldst.d * tmp;
  urdst.mz = urdst.d * tmp;
  tmp = invsumd * (sqrtdl * urst.by + sqrtdr * ulst.by +
                   bxsig * sqrtdl * sqrtdr * ((urst.my * urst_d_inv) - (ulst.my * ulst_d_inv)));
  uldst.by = urdst.by = tmp;
  tmp = invsumd * (sqrtdl * urst.bz + sqrtdr * ulst.bz +
                   bxsig * sqrtdl * sqrtdr * ((urst.mz * urst_d_inv) - (ulst.mz * ulst_d_inv)));
  uldst.bz = urdst.bz = tmp;
  tmp = spd[2] * bxi + (uldst.my * uldst.by + uldst.mz * uldst.bz) / uldst.d;
  uldst.e = ulst.e - sqrtdl * bxsig * (vbstl - tmp);
  urdst.e = urst.e + sqrtdr * bxsig * (vbstr - tmp);

  // select the upwind state first, then form the jumps it needs (hlld.cpp:302-370);
  // the arithmetic of every selected flux is the reference's
  if (spd[0] >= RC(0.0)) {
    f[0] = fl.d; f[1] = fl.mx; f[2] = fl.my; f[3] = fl.mz; f[4] = fl.e;
    f[5] = fl.by; f[6] = fl.bz;
  } else if (spd[4] <= RC(0.0)) {
    f[0] = fr.d; f[1] = fr.mx; f[2] = fr.my; f[3] = fr.mz; f[4] = fr.e;
    f[5] = fr.by; f[6] = fr.bz;
  } else if (spd[1] >= RC(0.0)) {
    f[0] = fl.d + spd[0] * (ulst.d - ul.d);
    f[1] = fl.mx + spd[0] * (ulst.mx - ul.mx);
    f[2] = fl.my + spd[0] * (ulst.my - ul.my);
    f[3] = fl.mz + spd[0] * (ulst.mz - ul.mz);
    f[4] = fl.e + spd[0] * (ulst.e - ul.e);
    f[5] = fl.by + spd[0] * (ulst.by - ul.by);
    f[6] = fl.bz + spd[0] * (ulst.bz - ul.bz);
  } else if (spd[3] <= RC(0.0)) {
    f[0] = fr.d + spd[4] * (urst.d - ur.d);
    f[1] = fr.mx + spd[4] * (urst.mx - ur.mx);
    f[2] = fr.my + spd[4] * (urst.my - ur.my);
    f[3] = fr.mz + spd[4] * (urst.mz - ur.mz);
    f[4] = fr.e + spd[4] * (urst.e - ur.e);
    f[5] = fr.by + spd[4] * (urst.by - ur.by);
    f[6] = fr.bz + spd[4] * (urst.bz - ur.bz);
  } else if (spd[2] >= RC(0.0)) {
    f[0] = fl.d + spd[0] * (ulst.d - ul.d) + spd[1] * (uldst.d - ulst.d);
    f[1] = fl.mx + spd[0] * (ulst.mx - ul.mx) + spd[1] * (uldst.mx - ulst.mx);
    f[2] = fl.my + spd[0] * (ulst.my - ul.my) + spd[1] * (uldst.my - ulst.my);
    f[3] = fl.mz + spd[0] * (ulst.mz - ul.mz) + spd[1] * (uldst.mz - ulst.mz);
    f[4] = fl.e + spd[0] * (ulst.e - ul.e) + spd[1] * (uldst.e - ulst.e);
    f[5] = fl.by + spd[0] * (ulst.by - ul.by) + spd[1] * (uldst.by - ulst.by);
    f[6] = fl.bz + spd[0] * (ulst.bz - ul.bz) + spd[1] * (uldst.bz - ulst.bz);
  } else {
    f[0] = fr.d + spd[4] * (urst.d - ur.d) + spd[3] * (urdst.d - urst.d);
    f[1] = fr.mx + spd[4] * (urst.mx - ur.mx) + spd[3] * (urdst.mx - urst.mx);
    f[2] = fr.my + spd[4] * (urst.my - ur.my) + spd[3] * (urdst.my - urst.my);
    f[3] = fr.mz + spd[4] * (urst.mz - ur.mz) + spd[3] * (urdst.mz - urst.mz);
    f[4] = fr.e + spd[4] * (urst.e - ur.e) + spd[3] * (urdst.e - urst.e);
    f[5] = fr.by + spd[4] * (urst.by - ur.by) + spd[3] * (urdst.by - urst.by);
    f[6] = fr.bz + spd[4] * (urst.bz - ur.bz) + spd[3] * (urdst.bz - urst.bz);
  }
}

// HLLE, hydro/rsolvers/mhd/hlle_mhd.cpp:25-182
template <typename Real>
__device__ __forceinline__ void hlle(Real gamma, const Real* wli, const Real* wri, Real bxi,
                                     Real* flxi) {
  Real gm1 = gamma - RC(1.0);
  Real fl[NWAVE], fr[NWAVE];
  Real sqrtdl = dsqrt(wli[IDN]);
  Real sqrtdr = dsqrt(wri[IDN]);
  Real isdlpdr = RC(1.0) / (sqrtdl + sqrtdr);
  Real wroe_d = sqrtdl * sqrtdr;
  Real wroe_vx = (sqrtdl * wli[IVX] + sqrtdr * wri[IVX]) * isdlpdr;
  Real wroe_vy = (sqrtdl * wli[IVY] + sqrtdr * wri[IVY]) * isdlpdr;
  Real wroe_vz = (sqrtdl * wli[IVZ] + sqrtdr * wri[IVZ]) * isdlpdr;
  Real wroe_by = (sqrtdr * wli[IBY] + sqrtdl * wri[IBY]) * isdlpdr;
  Real wroe_bz = (sqrtdr * wli[IBZ] + sqrtdl * wri[IBZ]) * isdlpdr;
  Real dby = wli[IBY] - wri[IBY], dbz = wli[IBZ] - wri[IBZ], sdd = sqrtdl + sqrtdr;
  Real x = RC(0.5) * (dby * dby + dbz * dbz) / (sdd * sdd);
  Real y = RC(0.5) * (wli[IDN] + wri[IDN]) / wroe_d;
  Real pbl = RC(0.5) * (bxi * bxi + wli[IBY] * wli[IBY] + wli[IBZ] * wli[IBZ]);
  Real pbr = RC(0.5) * (bxi * bxi + wri[IBY] * wri[IBY] + wri[IBZ] * wri[IBZ]);
  Real el = wli[IPR] / gm1 +
            RC(0.5) * wli[IDN] *
                (wli[IVX] * wli[IVX] + wli[IVY] * wli[IVY] + wli[IVZ] * wli[IVZ]) + pbl;
  Real er = wri[IPR] / gm1 +
            RC(0.5) * wri[IDN] *
                (wri[IVX] * wri[IVX] + wri[IVY] * wri[IVY] + wri[IVZ] * wri[IVZ]) + pbr;
  Real hroe = ((el + wli[IPR] + pbl) / sqrtdl + (er + wri[IPR] + pbr) / sqrtdr) * isdlpdr;
  Real cl = fast_ms(gamma, wli[IDN], wli[IPR], wli[IBY], wli[IBZ], bxi);
  Real cr = fast_ms(gamma, wri[IDN], wri[IPR], wri[IBY], wri[IBZ], bxi);
  Real btsq = wroe_by * wroe_by + wroe_bz * wroe_bz;
  Real vaxsq = bxi * bxi / wroe_d;
  Real bt_starsq = (gm1 - (gm1 - RC(1.0)) * y) * btsq;
  Real hp = hroe - (vaxsq + btsq / wroe_d);
  Real vsq = wroe_vx * wroe_vx + wroe_vy * wroe_vy + wroe_vz * wroe_vz;
  Real twid_asq = smax((gm1 * (hp - RC(0.5) * vsq) - (gm1 - RC(1.0)) * x), RC(0.0));
  Real ct2 = bt_starsq / wroe_d;
  Real tsum = vaxsq + ct2 + twid_asq;
  Real tdif = vaxsq + ct2 - twid_asq;
  Real cf2_cs2 = dsqrt(tdif * tdif + RC(4.0) * twid_asq * ct2);
  Real cfsq = RC(0.5) * (tsum + cf2_cs2);
  Real a = dsqrt(cfsq);
  Real al = smin((wroe_vx - a), (wli[IVX] - cl));
  Real ar = smax((wroe_vx + a), (wri[IVX] + cr));
  Real bp = ar > RC(0.0) ? ar : RC(0.0);
  Real bm = al < RC(0.0) ? al : RC(0.0);
  Real vxl = wli[IVX] - bm;
  Real vxr = wri[IVX] - bp;
  fl[IDN] = wli[IDN] * vxl;
  fr[IDN] = wri[IDN] * vxr;
  fl[IVX] = wli[IDN] * wli[IVX] * vxl + pbl - bxi * bxi;
  fr[IVX] = wri[IDN] * wri[IVX] * vxr + pbr - bxi * bxi;
  fl[IVY] = wli[IDN] * wli[IVY] * vxl - bxi * wli[IBY];
  fr[IVY] = wri[IDN] * wri[IVY] * vxr - bxi * wri[IBY];
  fl[IVZ] = wli[IDN] * wli[IVZ] * vxl - bxi * wli[IBZ];
  fr[IVZ] = wri[IDN] * wri[IVZ] * vxr - bxi * wri[IBZ];
  fl[IVX] += wli[IPR];
  fr[IVX] += wri[IPR];
  fl[IPR] = el * vxl + wli[IVX] * (wli[IPR] + pbl - bxi * bxi);
  fr[IPR] = er * vxr + wri[IVX] * (wri[IPR] + pbr - bxi * bxi);
  fl[IPR] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IPR] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * vxl - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * vxr - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * vxl - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * vxr - bxi * wri[IVZ];
  Real tmp = RC(0.0);
  if (bp != bm) tmp = RC(0.5) * (bp + bm) / (bp - bm);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n)
    flxi[n] = RC(0.5) * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

// PiecewiseLinearX1/2/3, uniform van Leer branch (reconstruct/plm.cpp:103-112) and the
// interface values (:148-152).  One wave component.
template <typename Real>
__device__ __forceinline__ void plm_one(Real qm, Real q0, Real qp, Real cp, Real cm,
                                        Real& qlp, Real& qrm) {
  Real dwl = (q0 - qm);
  Real dwr = (qp - q0);
  Real dw2 = dwl * dwr;
  Real dwm = RC(2.0) * dw2 / (dwl + dwr);
  if (dw2 <= RC(0.0)) dwm = RC(0.0);
  qlp = q0 + cp * dwm;
  qrm = q0 - cm * dwm;
}

// PiecewiseParabolicX1/2/3, uniform-Cartesian Colella-Sekora branch
// (reconstruct/ppm.cpp:113-315), coefficients c1..c6 = 1/2,1/2,1/2,1/2,1/6,-1/6
// (reconstruct/reconstruction.cpp:499-504).  One wave component; q_im2..q_ip2 stencil.
template <typename Real>
__device__ __forceinline__ void ppm_one(Real q_im2, Real q_im1, Real qc, Real q_ip1,
                                        Real q_ip2, Real& qlp, Real& qrm) {
  const Real C2 = RC(1.25);
  const Real c1 = RC(0.5), c2 = RC(0.5), c3 = RC(0.5), c4 = RC(0.5);
  const Real c5 = RC(1.0 / 6.0), c6 = RC(-1.0 / 6.0);
  Real qa = (qc - q_im1);
  Real qb = (q_ip1 - qc);
  Real dd_im1 = c1 * qa + c2 * (q_im1 - q_im2);
  Real dd = c1 * qb + c2 * qa;
  Real dd_ip1 = c1 * (q_ip2 - q_ip1) + c2 * qb;
  Real dph = (c3 * q_im1 + c4 * qc) + (c5 * dd_im1 + c6 * dd);
  Real dph_ip1 = (c3 * qc + c4 * q_ip1) + (c5 * dd + c6 * dd_ip1);
  Real d2qc_im1 = q_im2 + qc - RC(2.0) * q_im1;
  Real d2qc = q_im1 + q_ip1 - RC(2.0) * qc;
  Real d2qc_ip1 = qc + q_ip2 - RC(2.0) * q_ip1;
  {
    Real qa_tmp = dph - q_im1;
    Real qb_tmp = qc - dph;
    Real a = RC(3.0) * (q_im1 + qc - RC(2.0) * dph);
    Real b = d2qc_im1, c = d2qc, d = RC(0.0);
    if (sgn(a) == sgn(b) && sgn(a) == sgn(c))
      d = sgn(a) * smin(C2 * dabs(b), smin(C2 * dabs(c), dabs(a)));
    Real dph_tmp = RC(0.5) * (q_im1 + qc) - d / RC(6.0);
    if (qa_tmp * qb_tmp < RC(0.0)) dph = dph_tmp;
  }
  {
    Real qa_tmp = dph_ip1 - qc;
    Real qb_tmp = q_ip1 - dph_ip1;
    Real a = RC(3.0) * (qc + q_ip1 - RC(2.0) * dph_ip1);
    Real b = d2qc, c = d2qc_ip1, d = RC(0.0);
    if (sgn(a) == sgn(b) && sgn(a) == sgn(c))
      d = sgn(a) * smin(C2 * dabs(b), smin(C2 * dabs(c), dabs(a)));
    Real dphip1_tmp = RC(0.5) * (qc + q_ip1) - d / RC(6.0);
    if (qa_tmp * qb_tmp < RC(0.0)) dph_ip1 = dphip1_tmp;
  }
  Real d2qf = RC(6.0) * (dph + dph_ip1 - RC(2.0) * qc);
  Real qminus = dph, qplus = dph_ip1;
  Real dqf_minus = qc - qminus;
  Real dqf_plus = qplus - qc;
  {
    Real qa_tmp = dqf_minus * dqf_plus;
    Real qb_tmp = (q_ip1 - qc) * (qc - q_im1);
    Real a = d2qc_im1, b = d2qc, c = d2qc_ip1, d = d2qf, e = RC(0.0);
    if (sgn(a) == sgn(b) && sgn(a) == sgn(c) && sgn(a) == sgn(d))
      e = sgn(d) * smin(smin(C2 * dabs(a), C2 * dabs(b)), smin(C2 * dabs(c), dabs(d)));
    a = smax(dabs(q_im1), dabs(q_im2));
    b = smax(smax(dabs(qc), dabs(q_ip1)), dabs(q_ip2));
    Real rho = RC(0.0);
    if (dabs(d) > (RC(1.0e-12)) * smax(a, b)) rho = e / d;
    Real tmp_m = qc - rho * dqf_minus;
    Real tmp_p = qc + rho * dqf_plus;
    Real tmp2_m = qc - RC(2.0) * dqf_plus;
    Real tmp2_p = qc + RC(2.0) * dqf_minus;
    if ((qa_tmp <= RC(0.0) || qb_tmp <= RC(0.0))) {
      if (rho <= (RC(1.0) - (RC(1.0e-12)))) {
        qminus = tmp_m;
        qplus = tmp_p;
      }
    } else {
      if (dabs(dqf_minus) >= RC(2.0) * dabs(dqf_plus)) qminus = tmp2_m;
      if (dabs(dqf_plus) >= RC(2.0) * dabs(dqf_minus)) qplus = tmp2_p;
    }
  }
  qlp = qplus;
  qrm = qminus;
}

#undef RC
}  // namespace athgpu
