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

// FP64 <-> FP32 conversions on the integer pipe.  GB300's FP64 pipe also executes the
// F2F conversion instructions, at about two lane-operations per clock per SM; a kernel
// already bound by that pipe (the CT update) converts with integer bit arithmetic
// instead: IEEE-754 round to nearest, ties to even, for every value whose result is a
// normal float (or zero); denormal results, infinities and NaNs take the hardware
// conversion.  Both give the same bits as the hardware conversion.
__device__ __forceinline__ float d2f_rn(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(u >> 32), lo = (unsigned)u;
  const unsigned sign = hi & 0x80000000u;
  const int fe = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;  // biased FP32 exponent
  if (fe >= 1 && fe <= 254) {
    // keep the top 23 of the 52 fraction bits, round on the 29 dropped bits
    unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu, half = 0x10000000u;
    m += (rem > half) | ((rem == half) & (m & 1u));
    // a carry out of the fraction increments the exponent (to infinity from 254)
    return __uint_as_float(sign | (((unsigned)fe << 23) + m));
  }
  if ((u << 1) == 0ull) return __uint_as_float(sign);  // +-0
  return (float)x;
}
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  if (e - 1u < 254u) {  // normal
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
  }
  if ((b << 1) == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);  // +-0
  return (double)f;
}
// The FP64 difference of two floats, (double)a - (double)b, on the integer pipe: when both
// are normal and their exponents differ by at most 28, the exact difference has at most 53
// significant bits (2^52 + 2^24 < 2^53), so it is an FP64 number; it is formed from the
// two significands aligned in one 64-bit integer, normalised with a leading-zero count.
// Other operands take a function of its own (a real branch, so that nothing of it is
// issued predicated-off on the common path): a zero operand gives the other one widened
// on the integer pipe (f2d_exact; two zeros: -0 only for (-0) - (+0), as IEEE addition of
// a + (-b)), anything else the FP64 subtraction.  Same bits as the hardware in every case.
static __device__ __noinline__ double fsub_f64_slow(float a, float b) {
  const unsigned ua = __float_as_uint(a), ub = __float_as_uint(b) ^ 0x80000000u;
  if ((ub << 1) == 0u) {
    if ((ua << 1) != 0u) return f2d_exact(a);
    return __longlong_as_double((long long)(ua & ub & 0x80000000u) << 32);
  }
  if ((ua << 1) == 0u) return f2d_exact(__uint_as_float(ub));
  return (double)a - (double)b;
}
__device__ __forceinline__ double fsub_f64(float a, float b) {
  unsigned ua = __float_as_uint(a), ub = __float_as_uint(b) ^ 0x80000000u;  // a + (-b)
  unsigned ea = (ua >> 23) & 0xffu, eb = (ub >> 23) & 0xffu;
  if (ea < eb) {  // (ua, ea): the operand of the larger exponent
    const unsigned tu = ua, te = ea;
    ua = ub; ea = eb; ub = tu; eb = te;
  }
  const unsigned d = ea - eb;
  if (eb - 1u < 254u && ea < 255u && d <= 28u) {
    long long x = (long long)((ua & 0x7fffffu) | 0x800000u) << d;
    const long long y = (long long)((ub & 0x7fffffu) | 0x800000u);
    x = ((ua ^ ub) >> 31) ? x - y : x + y;
    unsigned long long sign = ua >> 31;
    if (x < 0) {
      x = -x;
      sign ^= 1ull;
    }
    if (x == 0) return 0.0;  // exact cancellation: +0 under round to nearest
    const int nb = 64 - __clzll(x);  // significant bits, 1..53
    // value = x * 2^(eb - 150): the aligned significand's leading bit lands in the exponent
    // field as +1, hence nb + eb + 872 - 1
    const unsigned long long bits = ((unsigned long long)x << (53 - nb)) +
                                    ((unsigned long long)(nb + (int)eb + 871) << 52) +
                                    (sign << 63);
    return __longlong_as_double((long long)bits);
  }
  return fsub_f64_slow(a, b);
}
__device__ __forceinline__ double fsub_f64(double a, double b) { return a - b; }
// a face-field (always FP64) value in the bulk precision (hardware conversion: where the
// kernel is not bound by the FP64 pipe, F2F costs fewer issue slots than d2f_rn)
__device__ __forceinline__ double to_real(double x, double) { return x; }
__device__ __forceinline__ float to_real(double x, float) { return (float)x; }

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

// Packed FP32x2 arithmetic (Blackwell FADD2 / FMUL2 / FFMA2): one instruction for two
// independent float operations, each rounded to nearest as the scalar one.
__device__ __forceinline__ float2 pk(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {  // a + (-1)*b: one rounding
  return __ffma2_rn(pk(-1.0f), b, a);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  return __ffma2_rn(a, b, c);
}

// Riemann solvers.  wl/wr: local order (d, v_normal, v_t1, v_t2, p, By, Bz)
// (hlld.cpp:59-75).  f[0..4]: mass, normal, two transverse momentum and energy fluxes;
// f[5] = F(By), f[6] = F(Bz).
template <typename Real>
struct Cons1D { Real d, mx, my, mz, e, by, bz; };

// HLLD in FP32 with the left and right states as the two halves of packed FP32x2
// operands (x = left, y = right): the conserved states, fast speeds, fluxes and
// single-star states of both sides are formed by one instruction each; what mixes the
// sides (wave speeds, the double-star state, the flux selection), the divisions and the
// square roots run per side.  Same operations as hlld<float> below (hlld.cpp:36-376),
// with the FMA contractions written out.
__device__ __forceinline__ float2 lr(const float* wli, const float* wri, int n) {
  return make_float2(wli[n], wri[n]);
}
__device__ __forceinline__ void hlld_pk(float gamma, const float* wli, const float* wri,
                                        float bxi, float* f) {
  const float SMALL_NUMBER = 1.0e-4f;
  const float igm1 = 1.0f / (gamma - 1.0f);
  const float2 d = lr(wli, wri, IDN), vx = lr(wli, wri, IVX), vy = lr(wli, wri, IVY),
               vz = lr(wli, wri, IVZ), p = lr(wli, wri, IPR), by = lr(wli, wri, IBY),
               bz = lr(wli, wri, IBZ);
  const float bxsq = bxi * bxi;
  const float2 ct2 = fma2(by, by, mul2(bz, bz));  // by^2 + bz^2
  const float2 pb = mul2(pk(0.5f), add2(pk(bxsq), ct2));
  const float2 ke = mul2(mul2(pk(0.5f), d), fma2(vx, vx, fma2(vy, vy, mul2(vz, vz))));
  const float2 mx = mul2(vx, d), my = mul2(vy, d), mz = mul2(vz, d);
  const float2 e = add2(fma2(p, pk(igm1), ke), pb);

  // FastMagnetosonicSpeed of both sides (eos/adiabatic_mhd.cpp:149-156)
  const float2 asq = mul2(pk(gamma), p);
  const float2 vc = add2(pk(bxsq), ct2);
  const float2 qsq = add2(vc, asq), tq = sub2(vc, asq);
  const float2 rad = fma2(tq, tq, mul2(mul2(pk(4.0f), asq), ct2));
  const float2 hq = mul2(pk(0.5f), add2(qsq, make_float2(sqrtf(rad.x), sqrtf(rad.y))));
  const float2 cf = make_float2(sqrtf(hq.x / d.x), sqrtf(hq.y / d.y));
  const float2 vm = sub2(vx, cf), vp = add2(vx, cf);
  const float spd0 = smin(vm.x, vm.y), spd4 = smax(vp.x, vp.y);

  const float2 pt = add2(p, pb);
  const float2 nbx = pk(-bxi);
  const float2 vb = fma2(vy, by, mul2(vz, bz));
  const float2 fmx = sub2(fma2(mx, vx, pt), pk(bxsq));
  const float2 fmy = fma2(nbx, by, mul2(my, vx));
  const float2 fmz = fma2(nbx, bz, mul2(mz, vx));
  const float2 fe = fma2(nbx, vb, mul2(vx, sub2(add2(e, pt), pk(bxsq))));
  const float2 fby = fma2(nbx, vy, mul2(by, vx));
  const float2 fbz = fma2(nbx, vz, mul2(bz, vx));

  const float2 sd = sub2(make_float2(spd0, spd4), vx);  // sdl, sdr
  const float2 sdd = mul2(sd, d);                        // ul.d*sdl, ur.d*sdr
  const float2 sm = mul2(sd, mx);
  const float spd2 = ((sm.y - sm.x) + (pt.x - pt.y)) / (sdd.y - sdd.x);
  const float2 sdm = sub2(make_float2(spd0, spd4), pk(spd2));  // sdml, sdmr
  const float2 sdm_inv = make_float2(1.0f / sdm.x, 1.0f / sdm.y);
  const float2 sd_ = mul2(sdd, sdm_inv);  // ulst.d, urst.d
  const float2 sd_inv = make_float2(1.0f / sd_.x, 1.0f / sd_.y);
  const float sqrtdl = sqrtf(sd_.x), sqrtdr = sqrtf(sd_.y);
  const float spd1 = spd2 - dabs(bxi) / sqrtdl;
  const float spd3 = spd2 + dabs(bxi) / sqrtdr;
  const float2 ptsts = fma2(sdd, sub2(pk(spd2), vx), pt);  // ptstl, ptstr
  const float ptst = 0.5f * (ptsts.y + ptsts.x);

  // single-star states of both sides (hlld.cpp:196-250)
  const float2 smx = mul2(sd_, pk(spd2));
  const float2 den = fma2(sdd, sdm, pk(-bxsq));  // ul.d*sdl*sdml - bxsq
  const float2 xa = mul2(pk(bxi), sub2(sd, sdm));
  const float2 xb = fma2(d, mul2(sd, sd), pk(-bxsq));
  const float2 nta = make_float2(-(xa.x / den.x), -(xa.y / den.y));
  const float2 tb = make_float2(xb.x / den.x, xb.y / den.y);
  float2 smy = mul2(sd_, fma2(by, nta, vy));
  float2 smz = mul2(sd_, fma2(bz, nta, vz));
  float2 sby = mul2(by, tb), sbz = mul2(bz, tb);
  const float2 smy0 = mul2(sd_, vy), smz0 = mul2(sd_, vz);
  if (dabs(den.x) < SMALL_NUMBER * ptst) {
    smy.x = smy0.x;
    smz.x = smz0.x;
    sby.x = by.x;
    sbz.x = bz.x;
  }
  if (dabs(den.y) < SMALL_NUMBER * ptst) {
    smy.y = smy0.y;
    smz.y = smz0.y;
    sby.y = by.y;
    sbz.y = bz.y;
  }
  const float2 vbst =
      mul2(fma2(smx, pk(bxi), fma2(smy, sby, mul2(smz, sbz))), sd_inv);
  const float2 t1 = add2(sub2(mul2(sd, e), mul2(pt, vx)), pk(ptst * spd2));
  const float2 t2 = sub2(fma2(vx, pk(bxi), vb), vbst);
  const float2 se = mul2(fma2(pk(bxi), t2, t1), sdm_inv);

  // double-star states (hlld.cpp:254-300)
  const float invsumd = 1.0f / (sqrtdl + sqrtdr);
  const float bxsig = (bxi > 0.0f ? 1.0f : -1.0f);
  const float2 vyst = mul2(smy, sd_inv), vzst = mul2(smz, sd_inv);
  float tmp = invsumd * (sqrtdl * vyst.x + sqrtdr * vyst.y + bxsig * (sby.y - sby.x));
  const float2 ddmy = mul2(sd_, pk(tmp));
  tmp = invsumd * (sqrtdl * vzst.x + sqrtdr * vzst.y + bxsig * (sbz.y - sbz.x));
  const float2 ddmz = mul2(sd_, pk(tmp));
  const float ddby = invsumd * (sqrtdl * sby.y + sqrtdr * sby.x +
                                bxsig * sqrtdl * sqrtdr * (vyst.y - vyst.x));
  const float ddbz = invsumd * (sqrtdl * sbz.y + sqrtdr * sbz.x +
                                bxsig * sqrtdl * sqrtdr * (vzst.y - vzst.x));
  tmp = spd2 * bxi + (ddmy.x * ddby + ddmz.x * ddbz) / sd_.x;
  const float ddel = se.x - sqrtdl * bxsig * (vbst.x - tmp);
  const float dder = se.y + sqrtdr * bxsig * (vbst.y - tmp);

  // the upwind flux (hlld.cpp:302-370), components paired as (d, mx), (my, mz), (e, by), bz
  const bool left = spd2 >= 0.0f;  // the side of the contact (used past the outer waves)
  auto pick = [&](float2 v) { return left ? v.x : v.y; };
  float u[7] = {pick(d), pick(mx), pick(my), pick(mz), pick(e), pick(by), pick(bz)};
  float fs[7] = {pick(mx), pick(fmx), pick(fmy), pick(fmz), pick(fe), pick(fby), pick(fbz)};
  if (spd0 >= 0.0f || spd4 <= 0.0f) {
    const bool l = spd0 >= 0.0f;
    f[0] = l ? mx.x : mx.y;
    f[1] = l ? fmx.x : fmx.y;
    f[2] = l ? fmy.x : fmy.y;
    f[3] = l ? fmz.x : fmz.y;
    f[4] = l ? fe.x : fe.y;
    f[5] = l ? fby.x : fby.y;
    f[6] = l ? fbz.x : fbz.y;
    return;
  }
  const float so = left ? spd0 : spd4;  // the outer wave
  const float st[7] = {pick(sd_), pick(smx), pick(smy), pick(smz), pick(se), pick(sby),
                       pick(sbz)};
  const float2 s2 = pk(so);
  float2 a = fma2(s2, sub2(make_float2(st[0], st[1]), make_float2(u[0], u[1])),
                  make_float2(fs[0], fs[1]));
  float2 b = fma2(s2, sub2(make_float2(st[2], st[3]), make_float2(u[2], u[3])),
                  make_float2(fs[2], fs[3]));
  float2 c = fma2(s2, sub2(make_float2(st[4], st[5]), make_float2(u[4], u[5])),
                  make_float2(fs[4], fs[5]));
  float g = fs[6] + so * (st[6] - u[6]);
  const bool inner = left ? !(spd1 >= 0.0f) : !(spd3 <= 0.0f);  // past the Alfven wave
  if (inner) {
    const float si = left ? spd1 : spd3;
    const float dd[7] = {st[0], st[1], left ? ddmy.x : ddmy.y, left ? ddmz.x : ddmz.y,
                         left ? ddel : dder, ddby, ddbz};
    const float2 s1 = pk(si);
    a = fma2(s1, sub2(make_float2(dd[0], dd[1]), make_float2(st[0], st[1])), a);
    b = fma2(s1, sub2(make_float2(dd[2], dd[3]), make_float2(st[2], st[3])), b);
    c = fma2(s1, sub2(make_float2(dd[4], dd[5]), make_float2(st[4], st[5])), c);
    g = g + si * (dd[6] - st[6]);
  }
  f[0] = a.x;
  f[1] = a.y;
  f[2] = b.x;
  f[3] = b.y;
  f[4] = c.x;
  f[5] = c.y;
  f[6] = g;
}

// HLLD (Miyoshi & Kusano 2005), hydro/rsolvers/mhd/hlld.cpp:36-376.  LD: the
// low-dissipation HLLD of Minoshima et al. 2021, hydro/rsolvers/mhd/lhlld.cpp:33-380,
// which scales the pressure jump in the middle speed by the shock detector th of the
// face's velocity differences dvn, dvt (:157-163), takes the star total pressure with the
// low-Mach factor phi (:184-188) and groups a few products as sdld = sdl*ul.d (:153-234).
template <typename Real, bool LD = false>
__device__ __forceinline__ void hlld(Real gamma, const Real* wli, const Real* wri, Real bxi,
                                     Real* f, Real dvn = RC(0.0), Real dvt = RC(0.0)) {
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
  const Real sdld = sdl * ul.d, sdrd = sdr * ur.d;
  const Real cfmax = smax(cfl, cfr);
  if (LD) {
    const Real th1 = smin(RC(1.0), (cfmax - smin(dvn, RC(0.0))) / (cfmax - smin(dvt, RC(0.0))));
    const Real th = th1 * th1 * th1 * th1;
    spd[2] = (sdr * ur.mx - sdl * ul.mx + th * (ptl - ptr)) / (sdrd - sdld);
  } else {
    spd[2] = (sdr * ur.mx - sdl * ul.mx + (ptl - ptr)) / (sdr * ur.d - sdl * ul.d);
  }
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

  Real ptst;
  if (LD) {
    const Real clsq =
        ((pbl + kel) + dsqrt((pbl + kel) * (pbl + kel) - RC(2.0) * kel * bxsq)) / ul.d;
    const Real crsq =
        ((pbr + ker) + dsqrt((pbr + ker) * (pbr + ker) - RC(2.0) * ker * bxsq)) / ur.d;
    const Real chi = smin(RC(1.0), dsqrt(smax(clsq, crsq)) / cfmax);
    const Real phi = chi * (RC(2.0) - chi);
    ptst = (sdrd * ptl - sdld * ptr + phi * sdrd * sdld * (wri[IVX] - wli[IVX])) /
           (sdrd - sdld);
  } else {
    Real ptstl = ptl + ul.d * sdl * (spd[2] - wli[IVX]);
    Real ptstr = ptr + ur.d * sdr * (spd[2] - wri[IVX]);
    ptst = RC(0.5) * (ptstr + ptstl);
  }

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
    tmp = (LD ? sdld * sdl - bxsq : ul.d * (sdl * sdl) - bxsq) / (ul.d * sdl * sdml - bxsq);
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
    tmp = (LD ? sdrd * sdr - bxsq : ur.d * (sdr * sdr) - bxsq) / (ur.d * sdr * sdmr - bxsq);
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

// local Lax-Friedrichs, hydro/rsolvers/mhd/llf_mhd.cpp:29-153 (adiabatic branch)
template <typename Real>
__device__ __forceinline__ void llf(Real gamma, const Real* wli, const Real* wri, Real bxi,
                                    Real* flxi) {
  const Real gm1 = gamma - RC(1.0);
  Real fl[NWAVE], fr[NWAVE], du[NWAVE];
  const Real cfl = fast_ms(gamma, wli[IDN], wli[IPR], wli[IBY], wli[IBZ], bxi);
  const Real cfr = fast_ms(gamma, wri[IDN], wri[IPR], wri[IBY], wri[IBZ], bxi);
  const Real a = RC(0.5) * smax(fabs(wli[IVX]) + cfl, fabs(wri[IVX]) + cfr);
  const Real mxl = wli[IDN] * wli[IVX];
  const Real mxr = wri[IDN] * wri[IVX];
  const Real pbl = RC(0.5) * (bxi * bxi + wli[IBY] * wli[IBY] + wli[IBZ] * wli[IBZ]);
  const Real pbr = RC(0.5) * (bxi * bxi + wri[IBY] * wri[IBY] + wri[IBZ] * wri[IBZ]);
  fl[IDN] = mxl;
  fr[IDN] = mxr;
  fl[IVX] = mxl * wli[IVX] + pbl - bxi * bxi;
  fr[IVX] = mxr * wri[IVX] + pbr - bxi * bxi;
  fl[IVY] = mxl * wli[IVY] - bxi * wli[IBY];
  fr[IVY] = mxr * wri[IVY] - bxi * wri[IBY];
  fl[IVZ] = mxl * wli[IVZ] - bxi * wli[IBZ];
  fr[IVZ] = mxr * wri[IVZ] - bxi * wri[IBZ];
  const Real el = wli[IPR] / gm1 +
                  RC(0.5) * wli[IDN] *
                      (wli[IVX] * wli[IVX] + wli[IVY] * wli[IVY] + wli[IVZ] * wli[IVZ]) + pbl;
  const Real er = wri[IPR] / gm1 +
                  RC(0.5) * wri[IDN] *
                      (wri[IVX] * wri[IVX] + wri[IVY] * wri[IVY] + wri[IVZ] * wri[IVZ]) + pbr;
  fl[IVX] += wli[IPR];
  fr[IVX] += wri[IPR];
  fl[IPR] = (el + wli[IPR] + pbl - bxi * bxi) * wli[IVX];
  fr[IPR] = (er + wri[IPR] + pbr - bxi * bxi) * wri[IVX];
  fl[IPR] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IPR] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * wli[IVX] - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * wri[IVX] - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * wli[IVX] - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * wri[IVX] - bxi * wri[IVZ];
  du[IDN] = wri[IDN] - wli[IDN];
  du[IVX] = wri[IDN] * wri[IVX] - wli[IDN] * wli[IVX];
  du[IVY] = wri[IDN] * wri[IVY] - wli[IDN] * wli[IVY];
  du[IVZ] = wri[IDN] * wri[IVZ] - wli[IDN] * wli[IVZ];
  du[IPR] = er - el;
  du[IBY] = wri[IBY] - wli[IBY];
  du[IBZ] = wri[IBZ] - wli[IBZ];
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) flxi[n] = RC(0.5) * (fl[n] + fr[n]) - a * du[n];
}

// Roe's linearised solver, adiabatic branch of hydro/rsolvers/mhd/roe_mhd.cpp:45-221 and
// its RoeFlux eigensystem (:223-460; Stone et al. 2008, ApJS 178, 137, eqs. B17-B29).  The
// sums over waves keep the reference's order, which fixes the rounding.  Upwind fluxes
// outside the fan; the LLF flux replaces the hydro components (not the field ones) when an
// intermediate density of the fan is negative.
template <typename Real>
__device__ __forceinline__ void roe(Real gamma, const Real* wli, const Real* wri, Real bxi,
                                    Real* flxi) {
  const Real gm1 = gamma - RC(1.0);
  Real fl[NWAVE], fr[NWAVE], du[NWAVE], ev[NWAVE], a[NWAVE], cf_[NWAVE];
  // Roe averages: density-weighted velocity, inverse-weighted transverse field, enthalpy
  Real sl = sqrt(wli[IDN]), sr = sqrt(wri[IDN]);
  Real isum = RC(1.0) / (sl + sr);
  Real d = sl * sr;
  Real v1 = (sl * wli[IVX] + sr * wri[IVX]) * isum;
  Real v2 = (sl * wli[IVY] + sr * wri[IVY]) * isum;
  Real v3 = (sl * wli[IVZ] + sr * wri[IVZ]) * isum;
  Real b2 = (sr * wli[IBY] + sl * wri[IBY]) * isum;
  Real b3 = (sr * wli[IBZ] + sl * wri[IBZ]) * isum;
  const Real dby = wli[IBY] - wri[IBY], dbz = wli[IBZ] - wri[IBZ];
  Real x = RC(0.5) * (dby * dby + dbz * dbz) / ((sl + sr) * (sl + sr));
  Real y = RC(0.5) * (wli[IDN] + wri[IDN]) / d;
  Real pbl = RC(0.5) * (bxi * bxi + wli[IBY] * wli[IBY] + wli[IBZ] * wli[IBZ]);
  Real pbr = RC(0.5) * (bxi * bxi + wri[IBY] * wri[IBY] + wri[IBZ] * wri[IBZ]);
  Real el = wli[IPR] / gm1 +
           RC(0.5) * wli[IDN] *
               (wli[IVX] * wli[IVX] + wli[IVY] * wli[IVY] + wli[IVZ] * wli[IVZ]) + pbl;
  Real er = wri[IPR] / gm1 +
           RC(0.5) * wri[IDN] *
               (wri[IVX] * wri[IVX] + wri[IVY] * wri[IVY] + wri[IVZ] * wri[IVZ]) + pbr;
  Real h = ((el + wli[IPR] + pbl) / sl + (er + wri[IPR] + pbr) / sr) * isum;
  // left and right physical fluxes
  Real mxl = wli[IDN] * wli[IVX], mxr = wri[IDN] * wri[IVX];
  fl[IDN] = mxl;
  fr[IDN] = mxr;
  fl[IVX] = mxl * wli[IVX] + pbl - bxi * bxi;
  fr[IVX] = mxr * wri[IVX] + pbr - bxi * bxi;
  fl[IVY] = mxl * wli[IVY] - bxi * wli[IBY];
  fr[IVY] = mxr * wri[IVY] - bxi * wri[IBY];
  fl[IVZ] = mxl * wli[IVZ] - bxi * wli[IBZ];
  fr[IVZ] = mxr * wri[IVZ] - bxi * wri[IBZ];
  fl[IVX] += wli[IPR];
  fr[IVX] += wri[IPR];
  fl[IPR] = (el + wli[IPR] + pbl - bxi * bxi) * wli[IVX];
  fr[IPR] = (er + wri[IPR] + pbr - bxi * bxi) * wri[IVX];
  fl[IPR] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IPR] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * wli[IVX] - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * wri[IVX] - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * wli[IVX] - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * wri[IVX] - bxi * wri[IVZ];
  // jump in the conserved variables
  du[IDN] = wri[IDN] - wli[IDN];
  du[IVX] = wri[IDN] * wri[IVX] - wli[IDN] * wli[IVX];
  du[IVY] = wri[IDN] * wri[IVY] - wli[IDN] * wli[IVY];
  du[IVZ] = wri[IDN] * wri[IVZ] - wli[IDN] * wli[IVZ];
  du[IPR] = er - el;
  du[IBY] = wri[IBY] - wli[IBY];
  du[IBZ] = wri[IBZ] - wli[IBZ];
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) flxi[n] = RC(0.5) * (fl[n] + fr[n]);

  // wave speeds of the Roe matrix (eq. B17-B18)
  Real di = RC(1.0) / d;
  Real btsq = b2 * b2 + b3 * b3;
  Real vaxsq = bxi * bxi * di;
  Real vsq = v1 * v1 + v2 * v2 + v3 * v3;
  Real hp = h - (vaxsq + btsq * di);
  Real ystar = gm1 - (gm1 - RC(1.0)) * y;
  Real bt_starsq = ystar * btsq;
  Real csq = smax((gm1 * (hp - RC(0.5) * vsq) - (gm1 - RC(1.0)) * x), RC(1.0e-20));
  Real ct2 = bt_starsq * di;
  Real tsum = vaxsq + ct2 + csq;
  Real tdif = vaxsq + ct2 - csq;
  Real root = sqrt(tdif * tdif + RC(4.0) * csq * ct2);
  Real cfsq = RC(0.5) * (tsum + root);
  Real cf = sqrt(cfsq);
  Real cssq = csq * vaxsq / cfsq;
  Real cs = sqrt(cssq);
  // transverse-field directions (eq. A17, B20, B28)
  Real bt = sqrt(btsq), bt_star = sqrt(bt_starsq);
  Real be2 = RC(0.0), be3 = RC(0.0);
  if (bt != RC(0.0)) {
    be2 = b2 / bt;
    be3 = b3 / bt;
  }
  Real be2s = be2 / sqrt(ystar);
  Real be3s = be3 / sqrt(ystar);
  Real bes_sq = be2s * be2s + be3s * be3s;
  Real vbet = v2 * be2s + v3 * be3s;
  Real q2s = RC(0.0), q3s = RC(0.0);
  if (bes_sq != RC(0.0)) {
    q2s = be2s / bes_sq;
    q3s = be3s / bes_sq;
  }
  // fast/slow normalisations (eq. A16), with their degenerate limits
  Real af_, as_;
  if ((cfsq - cssq) <= RC(0.0)) { af_ = RC(1.0); as_ = RC(0.0); }
  else if ((csq - cssq) <= RC(0.0)) { af_ = RC(0.0); as_ = RC(1.0); }
  else if ((cfsq - csq) <= RC(0.0)) { af_ = RC(1.0); as_ = RC(0.0); }
  else {
    af_ = sqrt((csq - cssq) / (cfsq - cssq));
    as_ = sqrt((cfsq - csq) / (cfsq - cssq));
  }
  Real sqd = sqrt(d), isqd = RC(1.0) / sqd;
  Real sgn = (bxi < RC(0.0)) ? -RC(1.0) : RC(1.0);
  Real c = sqrt(csq);
  Real qf = cf * af_ * sgn, qs = cs * as_ * sgn;
  Real afp = c * af_ * isqd, asp = c * as_ * isqd;
  Real afpbb = afp * bt_star * bes_sq, aspbb = asp * bt_star * bes_sq;
  Real vq = (v2 * q2s + v3 * q3s);
  Real vax = sqrt(vaxsq);
  Real nrm = RC(0.5) / csq;
  Real cff = nrm * af_ * cf, css = nrm * as_ * cs;
  Real qfh = qf * nrm, qsh = qs * nrm;
  Real afd = nrm * afp * d, asd = nrm * asp * d;
  Real afpb = nrm * afp * bt_star, aspb = nrm * asp * bt_star;
  ev[0] = v1 - cf;
  ev[1] = v1 - vax;
  ev[2] = v1 - cs;
  ev[3] = v1;
  ev[4] = v1 + cs;
  ev[5] = v1 + vax;
  ev[6] = v1 + cf;
  // projection of du on the left eigenvectors (eq. B29), term by term
  Real afb = af_ * gm1 * nrm, asb = as_ * gm1 * nrm;
  Real gm1a = gm1 / csq;
  a[0] = du[0] * (afb * (vsq - hp) + cff * (cf + v1) - qsh * vq - aspb);
  a[0] -= du[1] * (afb * v1 + cff);
  a[0] -= du[2] * (afb * v2 - qsh * q2s);
  a[0] -= du[3] * (afb * v3 - qsh * q3s);
  a[0] += du[4] * afb;
  a[0] += du[5] * (asd * q2s - afb * b2);
  a[0] += du[6] * (asd * q3s - afb * b3);
  a[1] = du[0] * (v2 * be3 - v3 * be2);
  a[1] -= du[2] * be3;
  a[1] += du[3] * be2;
  a[1] -= du[5] * sqd * be3 * sgn;
  a[1] += du[6] * sqd * be2 * sgn;
  a[1] *= RC(0.5);
  a[2] = du[0] * (asb * (vsq - hp) + css * (cs + v1) + qfh * vq + afpb);
  a[2] -= du[1] * (asb * v1 + css);
  a[2] -= du[2] * (asb * v2 + qfh * q2s);
  a[2] -= du[3] * (asb * v3 + qfh * q3s);
  a[2] += du[4] * asb;
  a[2] -= du[5] * (afd * q2s + asb * b2);
  a[2] -= du[6] * (afd * q3s + asb * b3);
  a[3] = du[0] * (RC(1.0) - gm1a * (RC(0.5) * vsq - (gm1 - RC(1.0)) * x / gm1));
  a[3] += du[1] * gm1a * v1;
  a[3] += du[2] * gm1a * v2;
  a[3] += du[3] * gm1a * v3;
  a[3] -= du[4] * gm1a;
  a[3] += du[5] * gm1a * b2;
  a[3] += du[6] * gm1a * b3;
  a[4] = du[0] * (asb * (vsq - hp) + css * (cs - v1) - qfh * vq + afpb);
  a[4] -= du[1] * (asb * v1 - css);
  a[4] -= du[2] * (asb * v2 - qfh * q2s);
  a[4] -= du[3] * (asb * v3 - qfh * q3s);
  a[4] += du[4] * asb;
  a[4] -= du[5] * (afd * q2s + asb * b2);
  a[4] -= du[6] * (afd * q3s + asb * b3);
  a[5] = du[0] * (v3 * be2 - v2 * be3);
  a[5] += du[2] * be3;
  a[5] -= du[3] * be2;
  a[5] -= du[5] * sqd * be3 * sgn;
  a[5] += du[6] * sqd * be2 * sgn;
  a[5] *= RC(0.5);
  a[6] = du[0] * (afb * (vsq - hp) + cff * (cf - v1) + qsh * vq - aspb);
  a[6] -= du[1] * (afb * v1 - cff);
  a[6] -= du[2] * (afb * v2 + qsh * q2s);
  a[6] -= du[3] * (afb * v3 + qsh * q3s);
  a[6] += du[4] * afb;
  a[6] += du[5] * (asd * q2s - afb * b2);
  a[6] += du[6] * (asd * q3s - afb * b3);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) cf_[n] = -RC(0.5) * fabs(ev[n]) * a[n];
  // density of the intermediate states left to right (first row of the right
  // eigenvectors): a negative one selects the LLF flux below
  int neg = 0;
  Real dens = wli[IDN] + a[0] * af_;
  neg |= dens < RC(0.0);
  dens += a[2] * as_;
  neg |= dens < RC(0.0);
  dens += a[3];
  neg |= dens < RC(0.0);
  dens += a[4] * as_;
  neg |= dens < RC(0.0);
  // dissipation: sum of the waves times the right eigenvectors (eq. B21)
  flxi[0] += cf_[0] * af_;
  flxi[0] += cf_[2] * as_;
  flxi[0] += cf_[3];
  flxi[0] += cf_[4] * as_;
  flxi[0] += cf_[6] * af_;
  flxi[1] += cf_[0] * (af_ * (v1 - cf));
  flxi[1] += cf_[2] * (as_ * (v1 - cs));
  flxi[1] += cf_[3] * v1;
  flxi[1] += cf_[4] * (as_ * (v1 + cs));
  flxi[1] += cf_[6] * (af_ * (v1 + cf));
  flxi[2] += cf_[0] * (af_ * v2 + qs * be2s);
  flxi[2] -= cf_[1] * be3;
  flxi[2] += cf_[2] * (as_ * v2 - qf * be2s);
  flxi[2] += cf_[3] * v2;
  flxi[2] += cf_[4] * (as_ * v2 + qf * be2s);
  flxi[2] += cf_[5] * be3;
  flxi[2] += cf_[6] * (af_ * v2 - qs * be2s);
  flxi[3] += cf_[0] * (af_ * v3 + qs * be3s);
  flxi[3] += cf_[1] * be2;
  flxi[3] += cf_[2] * (as_ * v3 - qf * be3s);
  flxi[3] += cf_[3] * v3;
  flxi[3] += cf_[4] * (as_ * v3 + qf * be3s);
  flxi[3] -= cf_[5] * be2;
  flxi[3] += cf_[6] * (af_ * v3 - qs * be3s);
  flxi[4] += cf_[0] * (af_ * (hp - v1 * cf) + qs * vbet + aspbb);
  flxi[4] -= cf_[1] * (v2 * be3 - v3 * be2);
  flxi[4] += cf_[2] * (as_ * (hp - v1 * cs) - qf * vbet - afpbb);
  flxi[4] += cf_[3] * (RC(0.5) * vsq + (gm1 - RC(1.0)) * x / gm1);
  flxi[4] += cf_[4] * (as_ * (hp + v1 * cs) + qf * vbet - afpbb);
  flxi[4] += cf_[5] * (v1 * be3 - v3 * be2);
  flxi[4] += cf_[6] * (af_ * (hp + v1 * cf) - qs * vbet + aspbb);
  flxi[5] += cf_[0] * asp * be2s;
  flxi[5] -= cf_[1] * be3 * sgn * isqd;
  flxi[5] -= cf_[2] * afp * be2s;
  flxi[5] -= cf_[4] * afp * be2s;
  flxi[5] -= cf_[5] * be3 * sgn * isqd;
  flxi[5] += cf_[6] * asp * be2s;
  flxi[6] += cf_[0] * asp * be3s;
  flxi[6] += cf_[1] * be2 * sgn * isqd;
  flxi[6] -= cf_[2] * afp * be3s;
  flxi[6] -= cf_[4] * afp * be3s;
  flxi[6] += cf_[5] * be2 * sgn * isqd;
  flxi[6] += cf_[6] * asp * be3s;
  // supersonic: the upwind flux
  if (ev[0] >= RC(0.0)) {
#pragma unroll
    for (int n = 0; n < NWAVE; ++n) flxi[n] = fl[n];
  }
  if (ev[NWAVE - 1] <= RC(0.0)) {
#pragma unroll
    for (int n = 0; n < NWAVE; ++n) flxi[n] = fr[n];
  }
  if (neg) {
    const Real cl = fast_ms(gamma, wli[IDN], wli[IPR], wli[IBY], wli[IBZ], bxi);
    const Real cr = fast_ms(gamma, wri[IDN], wri[IPR], wri[IBY], wri[IBZ], bxi);
    Real s = RC(0.5) * smax((fabs(wli[IVX]) + cl), (fabs(wri[IVX]) + cr));
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) flxi[n] = RC(0.5) * (fl[n] + fr[n]) - s * du[n];
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

// HLLE in FP32 with the left and right states as the halves of packed FP32x2 operands
// (x = left, y = right): the magnetic pressures, energies, fast speeds and the seven
// fluxes of both sides by one instruction each; the Roe averages and the wave speeds,
// which mix the sides, and the divisions and roots per side.  Same operations as
// hlle<float> above (hlle_mhd.cpp:33-175), with the FMA contractions written out.
__device__ __forceinline__ void hlle_pk(float gamma, const float* wli, const float* wri,
                                        float bxi, float* flxi) {
  const float gm1 = gamma - 1.0f;
  const float2 d = lr(wli, wri, IDN), vx = lr(wli, wri, IVX), vy = lr(wli, wri, IVY),
               vz = lr(wli, wri, IVZ), p = lr(wli, wri, IPR), by = lr(wli, wri, IBY),
               bz = lr(wli, wri, IBZ);
  const float sqrtdl = sqrtf(d.x), sqrtdr = sqrtf(d.y);
  const float isdlpdr = 1.0f / (sqrtdl + sqrtdr);
  const float wroe_d = sqrtdl * sqrtdr;
  const float wroe_vx = (sqrtdl * vx.x + sqrtdr * vx.y) * isdlpdr;
  const float wroe_vy = (sqrtdl * vy.x + sqrtdr * vy.y) * isdlpdr;
  const float wroe_vz = (sqrtdl * vz.x + sqrtdr * vz.y) * isdlpdr;
  const float wroe_by = (sqrtdr * by.x + sqrtdl * by.y) * isdlpdr;
  const float wroe_bz = (sqrtdr * bz.x + sqrtdl * bz.y) * isdlpdr;
  const float dby = by.x - by.y, dbz = bz.x - bz.y, sdd = sqrtdl + sqrtdr;
  const float x = 0.5f * (dby * dby + dbz * dbz) / (sdd * sdd);
  const float y = 0.5f * (d.x + d.y) / wroe_d;
  const float bxsq = bxi * bxi;
  const float2 ct2s = fma2(by, by, mul2(bz, bz));  // by^2 + bz^2 of each side
  const float2 pb = mul2(pk(0.5f), add2(pk(bxsq), ct2s));
  const float2 e = add2(fma2(p, pk(1.0f / gm1),
                             mul2(mul2(pk(0.5f), d), fma2(vx, vx, fma2(vy, vy, mul2(vz, vz))))),
                        pb);
  const float2 h = add2(add2(e, p), pb);
  const float hroe = (h.x / sqrtdl + h.y / sqrtdr) * isdlpdr;
  // FastMagnetosonicSpeed of both sides (eos/adiabatic_mhd.cpp:149-156)
  const float2 asq = mul2(pk(gamma), p);
  const float2 vc = add2(pk(bxsq), ct2s);
  const float2 qsq = add2(vc, asq), tq = sub2(vc, asq);
  const float2 rad = fma2(tq, tq, mul2(mul2(pk(4.0f), asq), ct2s));
  const float2 hq = mul2(pk(0.5f), add2(qsq, make_float2(sqrtf(rad.x), sqrtf(rad.y))));
  const float cl = sqrtf(hq.x / d.x), cr = sqrtf(hq.y / d.y);
  const float btsq = wroe_by * wroe_by + wroe_bz * wroe_bz;
  const float vaxsq = bxsq / wroe_d;
  const float bt_starsq = (gm1 - (gm1 - 1.0f) * y) * btsq;
  const float hp = hroe - (vaxsq + btsq / wroe_d);
  const float vsq = wroe_vx * wroe_vx + wroe_vy * wroe_vy + wroe_vz * wroe_vz;
  const float twid_asq = smax((gm1 * (hp - 0.5f * vsq) - (gm1 - 1.0f) * x), 0.0f);
  const float ct2 = bt_starsq / wroe_d;
  const float tsum = vaxsq + ct2 + twid_asq;
  const float tdif = vaxsq + ct2 - twid_asq;
  const float cf2_cs2 = sqrtf(tdif * tdif + 4.0f * twid_asq * ct2);
  const float cfsq = 0.5f * (tsum + cf2_cs2);
  const float a = sqrtf(cfsq);
  const float al = smin((wroe_vx - a), (vx.x - cl));
  const float ar = smax((wroe_vx + a), (vx.y + cr));
  const float bp = ar > 0.0f ? ar : 0.0f;
  const float bm = al < 0.0f ? al : 0.0f;
  const float2 vxs = sub2(vx, make_float2(bm, bp));  // vxl, vxr
  const float2 nbx = pk(-bxi);
  const float2 dvx = mul2(d, vxs);
  const float2 f0 = dvx;
  const float2 f1 = add2(sub2(fma2(mul2(d, vx), vxs, pb), pk(bxsq)), p);
  const float2 f2 = fma2(mul2(d, vy), vxs, mul2(nbx, by));
  const float2 f3 = fma2(mul2(d, vz), vxs, mul2(nbx, bz));
  const float2 f4 = fma2(nbx, fma2(by, vy, mul2(bz, vz)),
                         fma2(e, vxs, mul2(vx, sub2(add2(p, pb), pk(bxsq)))));
  const float2 f5 = fma2(by, vxs, mul2(nbx, vy));
  const float2 f6 = fma2(bz, vxs, mul2(nbx, vz));
  float tmp = 0.0f;
  if (bp != bm) tmp = 0.5f * (bp + bm) / (bp - bm);
  // 0.5*(fl + fr) + (fl - fr)*tmp, components paired
  const float2 fs[7] = {f0, f1, f2, f3, f4, f5, f6};
#pragma unroll
  for (int n = 0; n + 1 < NWAVE; n += 2) {
    const float2 sm = make_float2(fs[n].x + fs[n].y, fs[n + 1].x + fs[n + 1].y);
    const float2 df = make_float2(fs[n].x - fs[n].y, fs[n + 1].x - fs[n + 1].y);
    const float2 o = fma2(df, pk(tmp), mul2(pk(0.5f), sm));
    flxi[n] = o.x;
    flxi[n + 1] = o.y;
  }
  flxi[NWAVE - 1] = 0.5f * (fs[NWAVE - 1].x + fs[NWAVE - 1].y) +
                    (fs[NWAVE - 1].x - fs[NWAVE - 1].y) * tmp;
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

// plm_one on two wave components at once (FP32): the differences, products and face
// values as packed pairs, the van Leer quotient and the sign test per component
__device__ __forceinline__ void plm_two(float2 qm, float2 q0, float2 qp, float cp, float cm,
                                        float2& qlp, float2& qrm) {
  const float2 dwl = sub2(q0, qm);
  const float2 dwr = sub2(qp, q0);
  const float2 dw2 = mul2(dwl, dwr);
  const float2 num = mul2(pk(2.0f), dw2), den = add2(dwl, dwr);
  float2 dwm = make_float2(num.x / den.x, num.y / den.y);
  if (dw2.x <= 0.0f) dwm.x = 0.0f;
  if (dw2.y <= 0.0f) dwm.y = 0.0f;
  qlp = fma2(pk(cp), dwm, q0);
  qrm = fma2(pk(-cm), dwm, q0);
}

// PiecewiseParabolicX1/2/3, uniform-Cartesian Colella-Sekora branch
// (reconstruct/ppm.cpp:113-315), coefficients c1..c6 = 1/2,1/2,1/2,1/2,1/6,-1/6
// (reconstruct/reconstruction.cpp:499-504).  One wave component; q_im2..q_ip2 stencil.
// Limited PPM interface value between cells i-1 and i from cells i-2..i+1: the
// interface estimate of Step 1 (ppm.cpp:115-127) and the Step 2a limiter of that
// interface (ppm.cpp:139-166).  The upper interface of cell i is ppm_face(q_im1, qc, q_ip1, q_ip2),
// the same operations as the lower interface of cell i+1, so a sweep computes each
// interface once and carries it to the next cell.
template <typename Real>
__device__ __forceinline__ Real ppm_face(Real q_im2, Real q_im1, Real qc, Real q_ip1) {
  const Real C2 = RC(1.25);
  const Real c1 = RC(0.5), c2 = RC(0.5), c3 = RC(0.5), c4 = RC(0.5);
  const Real c5 = RC(1.0 / 6.0), c6 = RC(-1.0 / 6.0);
  Real qa = (qc - q_im1);
  Real qb = (q_ip1 - qc);
  Real dd_im1 = c1 * qa + c2 * (q_im1 - q_im2);
  Real dd = c1 * qb + c2 * qa;
  Real dph = (c3 * q_im1 + c4 * qc) + (c5 * dd_im1 + c6 * dd);
  Real d2qc_im1 = q_im2 + qc - RC(2.0) * q_im1;
  Real d2qc = q_im1 + q_ip1 - RC(2.0) * qc;
  Real qa_tmp = dph - q_im1;
  Real qb_tmp = qc - dph;
  Real a = RC(3.0) * (q_im1 + qc - RC(2.0) * dph);
  Real b = d2qc_im1, c = d2qc, d = RC(0.0);
  if (sgn(a) == sgn(b) && sgn(a) == sgn(c))
    d = sgn(a) * smin(C2 * dabs(b), smin(C2 * dabs(c), dabs(a)));
  Real dph_tmp = RC(0.5) * (q_im1 + qc) - d / RC(6.0);
  if (qa_tmp * qb_tmp < RC(0.0)) dph = dph_tmp;
  return dph;
}

// PPM cell values from the limited interfaces dph (i-1/2) and dph_ip1 (i+1/2): d2qf of
// Step 2a (ppm.cpp:192) and the Step 3 limiter of the parabola (ppm.cpp:216-315, uniform
// branch).
template <typename Real>
__device__ __forceinline__ void ppm_finish(Real q_im2, Real q_im1, Real qc, Real q_ip1,
                                           Real q_ip2, Real dph, Real dph_ip1, Real& qlp,
                                           Real& qrm, bool fast) {
  if (fast) {  // time/xorder = 3f: Mignone's limiter (ppm_fast.cpp:142-165), ratios 2 on a
               // uniform Cartesian mesh (reconstruction.cpp:490-491)
    const Real dqm = qc - dph, dqp = dph_ip1 - qc;
    Real qm = dph, qp = dph_ip1;
    if (dqm * dqp <= RC(0.0)) {
      qm = qc;
      qp = qc;
    } else {
      if (dabs(dqm) >= RC(2.0) * dabs(dqp)) qm = qc - RC(2.0) * dqp;
      if (dabs(dqp) >= RC(2.0) * dabs(dqm)) qp = qc + RC(2.0) * dqm;
    }
    qlp = qp;
    qrm = qm;
    return;
  }
  const Real C2 = RC(1.25);
  Real d2qc_im1 = q_im2 + qc - RC(2.0) * q_im1;
  Real d2qc = q_im1 + q_ip1 - RC(2.0) * qc;
  Real d2qc_ip1 = qc + q_ip2 - RC(2.0) * q_ip1;
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

template <typename Real>
__device__ __forceinline__ void ppm_one(Real q_im2, Real q_im1, Real qc, Real q_ip1,
                                        Real q_ip2, Real& qlp, Real& qrm, bool fast) {
  ppm_finish<Real>(q_im2, q_im1, qc, q_ip1, q_ip2, ppm_face<Real>(q_im2, q_im1, qc, q_ip1),
                   ppm_face<Real>(q_im1, qc, q_ip1, q_ip2), qlp, qrm, fast);
}

// FP32 PPM on two wave components at once.  The additions, multiplications and FMAs of
// ppm_face / ppm_finish run as packed FP32x2 instructions (one instruction, two
// independent IEEE operations rounded to nearest); the limiters' comparisons and
// selections run per component.  The operations are those of the scalar functions with
// the FMA contractions written out, so each component matches the scalar FP32 result up
// to where the compiler's own contraction of the scalar code differs.
// the Step 2a curvature limiter of one interface (ppm.cpp:150-158)
__device__ __forceinline__ float ppm_face_d(float a, float b, float c) {
  float d = 0.0f;
  if (sgn(a) == sgn(b) && sgn(a) == sgn(c))
    d = sgn(a) * smin(1.25f * dabs(b), smin(1.25f * dabs(c), dabs(a)));
  return d;
}

__device__ __forceinline__ float2 ppm_face2(float2 q_im2, float2 q_im1, float2 qc,
                                            float2 q_ip1) {
  const float2 half = pk(0.5f), m2 = pk(-2.0f);
  const float2 qa = sub2(qc, q_im1);
  const float2 qb = sub2(q_ip1, qc);
  const float2 dd_im1 = fma2(half, qa, mul2(half, sub2(q_im1, q_im2)));
  const float2 dd = fma2(half, qb, mul2(half, qa));
  const float2 s = add2(q_im1, qc);
  float2 dph = add2(fma2(half, q_im1, mul2(half, qc)),
                    fma2(pk(1.0f / 6.0f), dd_im1, mul2(pk(-1.0f / 6.0f), dd)));
  const float2 d2qc_im1 = fma2(m2, q_im1, add2(q_im2, qc));
  const float2 d2qc = fma2(m2, qc, add2(q_im1, q_ip1));
  const float2 qq = mul2(sub2(dph, q_im1), sub2(qc, dph));
  const float2 a = mul2(pk(3.0f), fma2(m2, dph, s));
  const float2 d = make_float2(ppm_face_d(a.x, d2qc_im1.x, d2qc.x),
                               ppm_face_d(a.y, d2qc_im1.y, d2qc.y));
  const float2 dph_tmp = fma2(pk(-1.0f / 6.0f), d, mul2(half, s));
  if (qq.x < 0.0f) dph.x = dph_tmp.x;
  if (qq.y < 0.0f) dph.y = dph_tmp.y;
  return dph;
}

// the Step 3 limiter of one component (ppm.cpp:236-315) from the packed parts below
__device__ __forceinline__ float ppm_rho(float q_im2, float q_im1, float qc, float q_ip1,
                                         float q_ip2, float d2qc_im1, float d2qc,
                                         float d2qc_ip1, float d2qf) {
  float e = 0.0f;
  if (sgn(d2qc_im1) == sgn(d2qc) && sgn(d2qc_im1) == sgn(d2qc_ip1) &&
      sgn(d2qc_im1) == sgn(d2qf))
    e = sgn(d2qf) * smin(smin(1.25f * dabs(d2qc_im1), 1.25f * dabs(d2qc)),
                         smin(1.25f * dabs(d2qc_ip1), dabs(d2qf)));
  const float a = smax(dabs(q_im1), dabs(q_im2));
  const float b = smax(smax(dabs(qc), dabs(q_ip1)), dabs(q_ip2));
  float rho = 0.0f;
  if (dabs(d2qf) > 1.0e-12f * smax(a, b)) rho = e / d2qf;
  return rho;
}
__device__ __forceinline__ void ppm_pick(float qa_tmp, float qb_tmp, float rho,
                                         float dqf_minus, float dqf_plus, float tmp_m,
                                         float tmp_p, float tmp2_m, float tmp2_p,
                                         float& qminus, float& qplus) {
  if (qa_tmp <= 0.0f || qb_tmp <= 0.0f) {
    if (rho <= (1.0f - 1.0e-12f)) {
      qminus = tmp_m;
      qplus = tmp_p;
    }
  } else {
    if (dabs(dqf_minus) >= 2.0f * dabs(dqf_plus)) qminus = tmp2_m;
    if (dabs(dqf_plus) >= 2.0f * dabs(dqf_minus)) qplus = tmp2_p;
  }
}

__device__ __forceinline__ void ppm_finish2(float2 q_im2, float2 q_im1, float2 qc,
                                            float2 q_ip1, float2 q_ip2, float2 dph,
                                            float2 dph_ip1, float2& qlp, float2& qrm) {
  const float2 m2 = pk(-2.0f), two = pk(2.0f);
  const float2 d2qc_im1 = fma2(m2, q_im1, add2(q_im2, qc));
  const float2 d2qc = fma2(m2, qc, add2(q_im1, q_ip1));
  const float2 d2qc_ip1 = fma2(m2, q_ip1, add2(qc, q_ip2));
  const float2 d2qf = mul2(pk(6.0f), fma2(m2, qc, add2(dph, dph_ip1)));
  const float2 dqf_minus = sub2(qc, dph);
  const float2 dqf_plus = sub2(dph_ip1, qc);
  const float2 qa_tmp = mul2(dqf_minus, dqf_plus);
  const float2 qb_tmp = mul2(sub2(q_ip1, qc), sub2(qc, q_im1));
  const float2 rho =
      make_float2(ppm_rho(q_im2.x, q_im1.x, qc.x, q_ip1.x, q_ip2.x, d2qc_im1.x, d2qc.x,
                          d2qc_ip1.x, d2qf.x),
                  ppm_rho(q_im2.y, q_im1.y, qc.y, q_ip1.y, q_ip2.y, d2qc_im1.y, d2qc.y,
                          d2qc_ip1.y, d2qf.y));
  const float2 tmp_m = fma2(make_float2(-rho.x, -rho.y), dqf_minus, qc);
  const float2 tmp_p = fma2(rho, dqf_plus, qc);
  const float2 tmp2_m = fma2(m2, dqf_plus, qc);
  const float2 tmp2_p = fma2(two, dqf_minus, qc);
  float2 qminus = dph, qplus = dph_ip1;
  ppm_pick(qa_tmp.x, qb_tmp.x, rho.x, dqf_minus.x, dqf_plus.x, tmp_m.x, tmp_p.x, tmp2_m.x,
           tmp2_p.x, qminus.x, qplus.x);
  ppm_pick(qa_tmp.y, qb_tmp.y, rho.y, dqf_minus.y, dqf_plus.y, tmp_m.y, tmp_p.y, tmp2_m.y,
           tmp2_p.y, qminus.y, qplus.y);
  qlp = qplus;
  qrm = qminus;
}


// ---------------------------------------------------------------------------------------
// Special-relativistic MHD.  Primitive velocities are the spatial 4-velocity u^i.

// FastMagnetosonicSpeedsGR with the SR metric (g00, g01, g11) = (-1, 0, 1),
// eos/adiabatic_mhd_sr.cpp:350-370
template <typename Real>
__device__ __forceinline__ void sr_fast_speeds(Real gamma_adi, Real wgas, Real pgas, Real u0,
                                               Real u1, Real b_sq, Real* lp, Real* lm) {
  const Real g00 = RC(-1.0), g01 = RC(0.0), g11 = RC(1.0);
  Real cs_sq = gamma_adi * pgas / wgas;
  Real va_sq = b_sq / (b_sq + wgas);
  Real cms_sq = cs_sq + va_sq - cs_sq * va_sq;
  Real a = u0 * u0 - (g00 + u0 * u0) * cms_sq;
  Real b = RC(-2.0) * (u0 * u1 - (g01 + u0 * u1) * cms_sq);
  Real c = u1 * u1 - (g11 + u1 * u1) * cms_sq;
  Real a1 = b / a;
  Real a0 = c / a;
  Real s = dsqrt(smax(a1 * a1 - RC(4.0) * a0, RC(0.0)));
  *lp = (a1 >= RC(0.0)) ? RC(-2.0) * a0 / (a1 + s) : (-a1 + s) / RC(2.0);
  *lm = (a1 >= RC(0.0)) ? (-a1 - s) / RC(2.0) : RC(-2.0) * a0 / (a1 - s);
}

// The L and R states of the SR frame-transforming solvers (Mignone & Bodo 2005; the same
// operations in hlle_mhd_rel.cpp:160-260 and llf_mhd_rel.cpp:136-220): conserved state and
// flux of each side (MUB 8, 15) and its fast speeds.  Local order as for hlld().
template <typename Real>
__device__ __forceinline__ void sr_states(Real gamma_adi, const Real* wli, const Real* wri,
                                          Real bb1, Real* cl, Real* cr, Real* fl, Real* fr,
                                          Real& lml, Real& lpl, Real& lmr, Real& lpr) {
#pragma unroll
  for (int sd = 0; sd < 2; ++sd) {
    const Real* w = sd == 0 ? wli : wri;
    Real* c = sd == 0 ? cl : cr;
    Real* ff = sd == 0 ? fl : fr;
    Real rho = w[IDN], pgas = w[IPR];
    Real u0 = dsqrt(RC(1.0) + w[IVX] * w[IVX] + w[IVY] * w[IVY] + w[IVZ] * w[IVZ]);
    Real u1 = w[IVX], u2 = w[IVY], u3 = w[IVZ];
    Real bb2 = w[IBY], bb3 = w[IBZ];
    Real b0 = bb1 * u1 + bb2 * u2 + bb3 * u3;
    Real b1 = (bb1 + b0 * u1) / u0;
    Real b2 = (bb2 + b0 * u2) / u0;
    Real b3 = (bb3 + b0 * u3) / u0;
    Real b_sq = -(b0 * b0) + b1 * b1 + b2 * b2 + b3 * b3;
    Real wgas = rho + gamma_adi / (gamma_adi - RC(1.0)) * pgas;
    if (sd == 0) sr_fast_speeds(gamma_adi, wgas, pgas, u0, u1, b_sq, &lpl, &lml);
    else sr_fast_speeds(gamma_adi, wgas, pgas, u0, u1, b_sq, &lpr, &lmr);
    Real wtot = wgas + b_sq, ptot = pgas + RC(0.5) * b_sq;
    c[0] = rho * u0;
    c[4] = wtot * u0 * u0 - b0 * b0 - ptot;
    c[1] = wtot * u1 * u0 - b1 * b0;
    c[2] = wtot * u2 * u0 - b2 * b0;
    c[3] = wtot * u3 * u0 - b3 * b0;
    c[5] = b2 * u0 - b0 * u2;
    c[6] = b3 * u0 - b0 * u3;
    ff[0] = rho * u1;
    ff[4] = wtot * u0 * u1 - b0 * b1;
    ff[1] = wtot * u1 * u1 - b1 * b1 + ptot;
    ff[2] = wtot * u2 * u1 - b2 * b1;
    ff[3] = wtot * u3 * u1 - b3 * b1;
    ff[5] = b2 * u1 - b1 * u2;
    ff[6] = b3 * u1 - b1 * u3;
  }
}

// SR frame-transforming HLLE, hydro/rsolvers/mhd/hlle_mhd_rel.cpp:103-330 (SR branch)
template <typename Real>
__device__ __forceinline__ void hlle_sr(Real gamma_adi, const Real* wli, const Real* wri,
                                        Real bb1, Real* f) {
  Real cl[NWAVE], cr[NWAVE], fl[NWAVE], fr[NWAVE];
  Real lml, lpl, lmr, lpr;
  sr_states<Real>(gamma_adi, wli, wri, bb1, cl, cr, fl, fr, lml, lpl, lmr, lpr);
  Real lambda_l = smin(lml, lmr);
  Real lambda_r = smax(lpl, lpr);
  Real lambda_diff_inv = RC(1.0) / (lambda_r - lambda_l);
  const Real v_interface = RC(0.0);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) {
    if (lambda_l >= v_interface) f[n] = fl[n];
    else if (lambda_r <= v_interface) f[n] = fr[n];
    else f[n] = (lambda_r * fl[n] - lambda_l * fr[n] + lambda_l * lambda_r * (cr[n] - cl[n])) *
                lambda_diff_inv;
  }
}

// SR frame-transforming LLF, hydro/rsolvers/mhd/llf_mhd_rel.cpp:101-280 (SR branch):
// lambda = max(lambda_r, -lambda_l) (MB 55), F = (F_l + F_r - lambda (U_r - U_l)) / 2
template <typename Real>
__device__ __forceinline__ void llf_sr(Real gamma_adi, const Real* wli, const Real* wri,
                                       Real bb1, Real* f) {
  Real cl[NWAVE], cr[NWAVE], fl[NWAVE], fr[NWAVE];
  Real lml, lpl, lmr, lpr;
  sr_states<Real>(gamma_adi, wli, wri, bb1, cl, cr, fl, fr, lml, lpl, lmr, lpr);
  Real lambda_l = smin(lml, lmr);
  Real lambda_r = smax(lpl, lpr);
  Real lambda = smax(lambda_r, -lambda_l);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) f[n] = RC(0.5) * (fl[n] + fr[n] - lambda * (cr[n] - cl[n]));
}

// Relativistic HLLD (Mignone, Ugliano & Bodo 2009, "MUB"), hydro/rsolvers/mhd/
// hlld_rel.cpp:116-890 (SR branch), with the enthalpy residual of Mignone & McKinney 2007
// ("MM") at hlld_rel.cpp:928-975.  Same steps, constants and operand order as the
// reference: HLL state (MB 29, 31); its total pressure from two Newton steps on W
// (MM A26-A27 start); the initial total pressure (MUB 53-55); four secant steps on the
// contact condition (MUB 48); the aL, aR (MUB 21-35, 43) and contact (MUB 45-52) states;
// the fan region at the interface; HLL wherever the HLLD states are not finite.
template <typename Real>
__device__ __forceinline__ Real hlldsr_eres(Real w_guess, Real dd, Real ee, Real m_sq,
                                            Real bb_sq, Real ss_sq, Real gamma_prime) {
  Real v_sq = (m_sq + ss_sq / (w_guess * w_guess) * (RC(2.0) * w_guess + bb_sq)) /
              ((w_guess + bb_sq) * (w_guess + bb_sq));
  Real gamma_sq = RC(1.0) / (RC(1.0) - v_sq);
  Real gamma_lorentz = dsqrt(gamma_sq);
  Real chi = (RC(1.0) - v_sq) * (w_guess - gamma_lorentz * dd);
  Real pgas = chi / gamma_prime;
  Real ee_calc = w_guess - pgas + RC(0.5) * bb_sq * (RC(1.0) + v_sq) -
                 ss_sq / (RC(2.0) * (w_guess * w_guess));
  return ee_calc - ee;
}

template <typename Real>
__device__ __forceinline__ Real hlldsr_eres_prime(Real w_guess, Real dd, Real m_sq,
                                                  Real bb_sq, Real ss_sq, Real gamma_prime) {
  Real v_sq = (m_sq + ss_sq / (w_guess * w_guess) * (RC(2.0) * w_guess + bb_sq)) /
              ((w_guess + bb_sq) * (w_guess + bb_sq));
  Real gamma_sq = RC(1.0) / (RC(1.0) - v_sq);
  Real gamma_lorentz = dsqrt(gamma_sq);
  Real chi = (RC(1.0) - v_sq) * (w_guess - gamma_lorentz * dd);
  Real w_cu = (w_guess * w_guess) * w_guess;
  Real w_b_cu = ((w_guess + bb_sq) * (w_guess + bb_sq)) * (w_guess + bb_sq);
  Real dv_sq_dw = RC(-2.0) / (w_cu * w_b_cu) *
                  (ss_sq * (RC(3.0) * w_guess * (w_guess + bb_sq) + bb_sq * bb_sq) +
                   m_sq * w_cu);
  Real dchi_dw = RC(1.0) - v_sq -
                 gamma_lorentz / RC(2.0) * (dd + RC(2.0) * gamma_lorentz * chi) * dv_sq_dw;
  Real drho_dw = -gamma_lorentz * dd / RC(2.0) * dv_sq_dw;
  Real dpgas_dchi = RC(1.0) / gamma_prime;
  Real dpgas_drho = RC(0.0);
  // the zero term stays: it makes a non-finite drho_dw reach the result as it does there
  Real dpgas_dw = dpgas_dchi * dchi_dw + dpgas_drho * drho_dw;
  return RC(1.0) - dpgas_dw + RC(0.5) * bb_sq * dv_sq_dw + ss_sq / w_cu;
}

// The Alfven-region quantities at one total pressure and the contact-condition residual
// (MUB 21-49; hlld_rel.cpp:437-517, the same steps at :521-598 and :618-697)
template <typename Real>
struct HlldSrAlfven {
  Real vx_al, vy_al, vz_al, vx_ar, vy_ar, vz_ar;
  Real by_al, bz_al, by_ar, bz_ar;
  Real kx_l, ky_l, kz_l, kx_r, ky_r, kz_r, eta_l, eta_r;
};

template <typename Real>
__device__ __forceinline__ Real hlldsr_residual(Real ptot, Real bbx, Real lambda_l,
                                                Real lambda_r, const Real* r_l,
                                                const Real* r_r, HlldSrAlfven<Real>& a) {
  const Real delta_kx_aug = RC(1.0e-12);
  const Real bbx_sq = bbx * bbx;
  {
    Real al = r_l[1] - lambda_l * r_l[4] + ptot * (RC(1.0) - lambda_l * lambda_l);
    Real gl = r_l[5] * r_l[5] + r_l[6] * r_l[6];
    Real cl = r_l[2] * r_l[5] + r_l[3] * r_l[6];
    Real ql = -al - gl + bbx_sq * (RC(1.0) - lambda_l * lambda_l);
    Real xl_inv = RC(1.0) / (bbx * (al * lambda_l * bbx + cl) -
                             (al + gl) * (lambda_l * ptot + r_l[4]));
    a.vx_al = (bbx * (al * bbx + lambda_l * cl) - (al + gl) * (ptot + r_l[1])) * xl_inv;
    Real tl = cl + bbx * (lambda_l * r_l[1] - r_l[4]);
    a.vy_al = (ql * r_l[2] + r_l[5] * tl) * xl_inv;
    a.vz_al = (ql * r_l[3] + r_l[6] * tl) * xl_inv;
  }
  {
    Real ar = r_r[1] - lambda_r * r_r[4] + ptot * (RC(1.0) - lambda_r * lambda_r);
    Real gr = r_r[5] * r_r[5] + r_r[6] * r_r[6];
    Real cr = r_r[2] * r_r[5] + r_r[3] * r_r[6];
    Real qr = -ar - gr + bbx_sq * (RC(1.0) - lambda_r * lambda_r);
    Real xr_inv = RC(1.0) / (bbx * (ar * lambda_r * bbx + cr) -
                             (ar + gr) * (lambda_r * ptot + r_r[4]));
    a.vx_ar = (bbx * (ar * bbx + lambda_r * cr) - (ar + gr) * (ptot + r_r[1])) * xr_inv;
    Real tr = cr + bbx * (lambda_r * r_r[1] - r_r[4]);
    a.vy_ar = (qr * r_r[2] + r_r[5] * tr) * xr_inv;
    a.vz_ar = (qr * r_r[3] + r_r[6] * tr) * xr_inv;
  }
  a.by_al = (r_l[5] - bbx * a.vy_al) / (lambda_l - a.vx_al);
  a.bz_al = (r_l[6] - bbx * a.vz_al) / (lambda_l - a.vx_al);
  a.by_ar = (r_r[5] - bbx * a.vy_ar) / (lambda_r - a.vx_ar);
  a.bz_ar = (r_r[6] - bbx * a.vz_ar) / (lambda_r - a.vx_ar);
  Real v_rm_l = a.vx_al * r_l[1] + a.vy_al * r_l[2] + a.vz_al * r_l[3];
  Real wtot_al = ptot + (r_l[4] - v_rm_l) / (lambda_l - a.vx_al);
  Real v_rm_r = a.vx_ar * r_r[1] + a.vy_ar * r_r[2] + a.vz_ar * r_r[3];
  Real wtot_ar = ptot + (r_r[4] - v_rm_r) / (lambda_r - a.vx_ar);
  a.eta_l = -copysign(dsqrt(wtot_al), bbx);
  a.eta_r = copysign(dsqrt(wtot_ar), bbx);
  Real dl_inv = RC(1.0) / (lambda_l * ptot + r_l[4] + bbx * a.eta_l);
  a.kx_l = (r_l[1] + ptot + lambda_l * bbx * a.eta_l) * dl_inv;
  a.ky_l = (r_l[2] + r_l[5] * a.eta_l) * dl_inv;
  a.kz_l = (r_l[3] + r_l[6] * a.eta_l) * dl_inv;
  Real dr_inv = RC(1.0) / (lambda_r * ptot + r_r[4] + bbx * a.eta_r);
  a.kx_r = (r_r[1] + ptot + lambda_r * bbx * a.eta_r) * dr_inv;
  a.ky_r = (r_r[2] + r_r[5] * a.eta_r) * dr_inv;
  a.kz_r = (r_r[3] + r_r[6] * a.eta_r) * dr_inv;
  // the Alfven speeds are kx_l and kx_r
  Real delta_kx = a.kx_r - a.kx_l + delta_kx_aug;
  Real bbx_c = bbx * delta_kx;
  Real by_c = a.by_ar * (a.kx_r - a.vx_ar) - a.by_al * (a.kx_l - a.vx_al) +
              bbx * (a.vy_ar - a.vy_al);
  Real bz_c = a.bz_ar * (a.kx_r - a.vx_ar) - a.bz_al * (a.kx_l - a.vx_al) +
              bbx * (a.vz_ar - a.vz_al);
  Real k_sq_l = a.kx_l * a.kx_l + a.ky_l * a.ky_l + a.kz_l * a.kz_l;
  Real y_l = (RC(1.0) - k_sq_l) /
             (a.eta_l * delta_kx - (a.kx_l * bbx_c + a.ky_l * by_c + a.kz_l * bz_c));
  Real k_sq_r = a.kx_r * a.kx_r + a.ky_r * a.ky_r + a.kz_r * a.kz_r;
  Real y_r = (RC(1.0) - k_sq_r) /
             (a.eta_r * delta_kx - (a.kx_r * bbx_c + a.ky_r * by_c + a.kz_r * bz_c));
  return delta_kx * (RC(1.0) - bbx * (y_r - y_l));
}

template <typename Real>
__device__ __forceinline__ bool all_finite7(const Real* c, const Real* f) {
  bool ok = true;
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) ok = ok && isfinite(c[n]) && isfinite(f[n]);
  return ok;
}

template <typename Real>
__device__ __forceinline__ void hlld_sr(Real gamma_adi, const Real* wli, const Real* wri,
                                        Real bbx, Real* f) {
  const Real p_transition = RC(0.01), vc_extension = RC(1.0e-6);
  const Real delta_kx_aug = RC(1.0e-12), initial_offset = RC(1.0e-5), tol_res = RC(1.0e-12);
  const Real gamma_prime = gamma_adi / (gamma_adi - RC(1.0));
  Real cl[NWAVE], cr[NWAVE], fl[NWAVE], fr[NWAVE];
  Real lml, lpl, lmr, lpr;
  sr_states<Real>(gamma_adi, wli, wri, bbx, cl, cr, fl, fr, lml, lpl, lmr, lpr);
  const Real lambda_l = smin(lml, lmr);
  const Real lambda_r = smax(lpl, lpr);
  // A face outside the fan takes the L or R flux whatever the fan holds, unless that state
  // is not finite (then the reference's choice depends on the fan: the full path below).
  if (lambda_l >= RC(0.0) && all_finite7(cl, fl)) {
#pragma unroll
    for (int n = 0; n < NWAVE; ++n) f[n] = fl[n];
    return;
  }
  if (lambda_r <= RC(0.0) && lambda_l < RC(0.0) && all_finite7(cr, fr)) {
#pragma unroll
    for (int n = 0; n < NWAVE; ++n) f[n] = fr[n];
    return;
  }
  Real r_l[NWAVE], r_r[NWAVE], u_hll[NWAVE], f_hll[NWAVE];
  const Real lambda_diff_inv = RC(1.0) / (lambda_r - lambda_l);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) {
    r_l[n] = lambda_l * cl[n] - fl[n];
    r_r[n] = lambda_r * cr[n] - fr[n];
    u_hll[n] = (r_r[n] - r_l[n]) * lambda_diff_inv;
    f_hll[n] = (lambda_l * r_r[n] - lambda_r * r_l[n]) * lambda_diff_inv;
  }
  // total pressure of the HLL state (MM A26-A27 start, two Newton steps, MM A3-A17, MM 2)
  Real ptot_hll;
  {
    Real m_sq = u_hll[1] * u_hll[1] + u_hll[2] * u_hll[2] + u_hll[3] * u_hll[3];
    Real bb_sq = bbx * bbx + u_hll[5] * u_hll[5] + u_hll[6] * u_hll[6];
    Real m_dot_bb = u_hll[1] * bbx + u_hll[2] * u_hll[5] + u_hll[3] * u_hll[6];
    Real ss_sq = m_dot_bb * m_dot_bb;
    Real a1 = RC(4.0) / RC(3.0) * (bb_sq - u_hll[4]);
    Real a0 = RC(0.33333333333333333) * (m_sq + bb_sq * (bb_sq - RC(2.0) * u_hll[4]));
    Real s2 = a1 * a1 - RC(4.0) * a0;
    Real s = (s2 < RC(0.0)) ? RC(0.0) : dsqrt(s2);
    Real w = (s2 >= RC(0.0) && a1 >= RC(0.0)) ? RC(-2.0) * a0 / (a1 + s)
                                              : RC(0.5) * (-a1 + s);
    Real res = hlldsr_eres(w, u_hll[0], u_hll[4], m_sq, bb_sq, ss_sq, gamma_prime);
#pragma unroll
    for (int n = 0; n < 2; ++n) {
      Real derivative = hlldsr_eres_prime(w, u_hll[0], m_sq, bb_sq, ss_sq, gamma_prime);
      w = w + -res / derivative;
      res = hlldsr_eres(w, u_hll[0], u_hll[4], m_sq, bb_sq, ss_sq, gamma_prime);
    }
    Real v_sq = (m_sq + ss_sq / (w * w) * (RC(2.0) * w + bb_sq)) / ((w + bb_sq) * (w + bb_sq));
    Real gamma_lor_sq = RC(1.0) / (RC(1.0) - v_sq);
    Real gamma_lor = dsqrt(gamma_lor_sq);
    Real chi = (RC(1.0) - v_sq) * (w - gamma_lor * u_hll[0]);
    Real pgas = RC(1.0) / gamma_prime * chi;
    Real vx = (u_hll[1] + m_dot_bb / w * bbx) / (w + bb_sq);
    Real vy = (u_hll[2] + m_dot_bb / w * u_hll[5]) / (w + bb_sq);
    Real vz = (u_hll[3] + m_dot_bb / w * u_hll[6]) / (w + bb_sq);
    Real v_bb = vx * bbx + vy * u_hll[5] + vz * u_hll[6];
    Real b_sq = bb_sq / gamma_lor_sq + v_bb * v_bb;
    ptot_hll = pgas + RC(0.5) * b_sq;
  }
  Real ptot_init;
  if (bbx * bbx / ptot_hll < p_transition) {  // weak field (MUB 55)
    Real a1 = u_hll[4] - f_hll[1];
    Real a0 = u_hll[1] * f_hll[4] - f_hll[1] * u_hll[4];
    Real s2 = a1 * a1 - RC(4.0) * a0;
    Real s = (s2 < RC(0.0)) ? RC(0.0) : dsqrt(s2);
    ptot_init = (s2 >= RC(0.0) && a1 >= RC(0.0)) ? RC(-2.0) * a0 / (a1 + s)
                                                 : (-a1 + s) / RC(2.0);
  } else {
    ptot_init = ptot_hll;
  }
  bool to_hll = !isfinite(ptot_init) || ptot_init <= RC(0.0);
  // secant iteration on the contact condition
  HlldSrAlfven<Real> a;
  Real ptot_last = ptot_init;
  Real res_last = hlldsr_residual(ptot_last, bbx, lambda_l, lambda_r, r_l, r_r, a);
  Real ptot_n = ptot_init * (RC(1.0) + initial_offset);
  Real res_n = hlldsr_residual(ptot_n, bbx, lambda_l, lambda_r, r_l, r_r, a);
  // FP64: the reference's stopping tests.  FP32: the pressure test at 1e-6 (eight ulps;
  // 1e-8 is below one) and no step when the two residuals are equal, so that a secant
  // that has reached the rounding noise of FP32 stops instead of dividing by zero and
  // sending the face to the HLL fallback that FP64 does not take.
  constexpr bool kFp64 = sizeof(Real) == 8;
  const Real tol_ptot = (kFp64 ? RC(1.0e-8) : RC(1.0e-6)) * ptot_init;
#pragma unroll 1
  for (int n = 0; n < 4; ++n) {
    const Real ptot_old = ptot_last, res_old = res_last;
    ptot_last = ptot_n;
    res_last = res_n;
    if (dabs(res_last) > tol_res && dabs(ptot_last - ptot_old) > tol_ptot &&
        (kFp64 || res_last != res_old))
      ptot_n = (res_last * ptot_old - res_old * ptot_last) / (res_last - res_old);
    else
      ptot_n = ptot_last;
    res_n = hlldsr_residual(ptot_n, bbx, lambda_l, lambda_r, r_l, r_r, a);
  }
  const Real ptot_c = ptot_n;
  const Real lambda_al = a.kx_l, lambda_ar = a.kx_r;
  if (!isfinite(lambda_al) || !isfinite(lambda_ar) || !isfinite(ptot_c) || ptot_c <= RC(0.0))
    to_hll = true;
  // aL and aR states (MUB 32-34) and fluxes (MUB 11-12)
  Real u_al[NWAVE], u_ar[NWAVE];
  u_al[5] = a.by_al;
  u_al[6] = a.bz_al;
  u_ar[5] = a.by_ar;
  u_ar[6] = a.bz_ar;
  {
    Real v_bb = a.vx_al * bbx + a.vy_al * u_al[5] + a.vz_al * u_al[6];
    u_al[0] = r_l[0] / (lambda_l - a.vx_al);
    u_al[4] = (r_l[4] + ptot_c * a.vx_al - v_bb * bbx) / (lambda_l - a.vx_al);
    u_al[1] = (u_al[4] + ptot_c) * a.vx_al - v_bb * bbx;
    u_al[2] = (u_al[4] + ptot_c) * a.vy_al - v_bb * u_al[5];
    u_al[3] = (u_al[4] + ptot_c) * a.vz_al - v_bb * u_al[6];
  }
  {
    Real v_bb = a.vx_ar * bbx + a.vy_ar * u_ar[5] + a.vz_ar * u_ar[6];
    u_ar[0] = r_r[0] / (lambda_r - a.vx_ar);
    u_ar[4] = (r_r[4] + ptot_c * a.vx_ar - v_bb * bbx) / (lambda_r - a.vx_ar);
    u_ar[1] = (u_ar[4] + ptot_c) * a.vx_ar - v_bb * bbx;
    u_ar[2] = (u_ar[4] + ptot_c) * a.vy_ar - v_bb * u_ar[5];
    u_ar[3] = (u_ar[4] + ptot_c) * a.vz_ar - v_bb * u_ar[6];
  }
  // contact field (MUB 45) and velocity (MUB 47, the mean of the L and R estimates)
  Real u_c[NWAVE];
  {
    Real denom_c_inv = RC(1.0) / (lambda_ar - lambda_al + delta_kx_aug);
    Real nl = u_al[5] * (lambda_al - a.vx_al) + bbx * a.vy_al;
    Real nr = u_ar[5] * (lambda_ar - a.vx_ar) + bbx * a.vy_ar;
    u_c[5] = (nr - nl) * denom_c_inv;
    nl = u_al[6] * (lambda_al - a.vx_al) + bbx * a.vz_al;
    nr = u_ar[6] * (lambda_ar - a.vx_ar) + bbx * a.vz_ar;
    u_c[6] = (nr - nl) * denom_c_inv;
  }
  Real vx_c, vy_c, vz_c;
  {
    Real k_sq_l = a.kx_l * a.kx_l + a.ky_l * a.ky_l + a.kz_l * a.kz_l;
    Real k_bc_l = a.kx_l * bbx + a.ky_l * u_c[5] + a.kz_l * u_c[6];
    Real vx_cl = a.kx_l - bbx * (RC(1.0) - k_sq_l) / (a.eta_l - k_bc_l);
    Real vy_cl = a.ky_l - u_c[5] * (RC(1.0) - k_sq_l) / (a.eta_l - k_bc_l);
    Real vz_cl = a.kz_l - u_c[6] * (RC(1.0) - k_sq_l) / (a.eta_l - k_bc_l);
    Real k_sq_r = a.kx_r * a.kx_r + a.ky_r * a.ky_r + a.kz_r * a.kz_r;
    Real k_bc_r = a.kx_r * bbx + a.ky_r * u_c[5] + a.kz_r * u_c[6];
    Real vx_cr = a.kx_r - bbx * (RC(1.0) - k_sq_r) / (a.eta_r - k_bc_r);
    Real vy_cr = a.ky_r - u_c[5] * (RC(1.0) - k_sq_r) / (a.eta_r - k_bc_r);
    Real vz_cr = a.kz_r - u_c[6] * (RC(1.0) - k_sq_r) / (a.eta_r - k_bc_r);
    vx_c = RC(0.5) * (vx_cl + vx_cr);
    vy_c = RC(0.5) * (vy_cl + vy_cr);
    vz_c = RC(0.5) * (vz_cl + vz_cr);
  }
  // the contact state on the side of the contact that vx_c names (MUB 50-52)
  const bool c_left = vx_c >= RC(0.0);
  const Real lam_s = c_left ? lambda_al : lambda_ar;
  const Real vx_s = c_left ? a.vx_al : a.vx_ar;
  Real u_s[NWAVE], f_s[NWAVE];
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) {
    u_s[n] = c_left ? u_al[n] : u_ar[n];
    // flux of the aL / aR state (MUB 11-12)
    f_s[n] = c_left ? lambda_l * u_al[n] - r_l[n] : lambda_r * u_ar[n] - r_r[n];
  }
  {
    Real v_bb = vx_c * bbx + vy_c * u_c[5] + vz_c * u_c[6];
    u_c[0] = u_s[0] * (lam_s - vx_s) / (lam_s - vx_c);
    u_c[4] = (lam_s * u_s[4] - u_s[1] + ptot_c * vx_c - v_bb * bbx) / (lam_s - vx_c);
    u_c[1] = (u_c[4] + ptot_c) * vx_c - v_bb * bbx;
    u_c[2] = (u_c[4] + ptot_c) * vy_c - v_bb * u_c[5];
    u_c[3] = (u_c[4] + ptot_c) * vz_c - v_bb * u_c[6];
  }
  // region of the fan at the interface (v_interface = 0 in SR): 0 L, 1 R, 2 HLL, 3 aL,
  // 4 aR, 5 contact
  const int region = lambda_l >= RC(0.0) ? 0
                     : lambda_r <= RC(0.0) ? 1
                     : to_hll ? 2
                     : lambda_al >= RC(0.0) - vc_extension ? 3
                     : lambda_ar <= RC(0.0) + vc_extension ? 4 : 5;
  Real ui[NWAVE], fi[NWAVE];
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) {
    Real f_al = lambda_l * u_al[n] - r_l[n];
    Real f_ar = lambda_r * u_ar[n] - r_r[n];
    Real f_c = f_s[n] + lam_s * (u_c[n] - u_s[n]);
    ui[n] = region == 0 ? cl[n] : region == 1 ? cr[n] : region == 2 ? u_hll[n]
            : region == 3 ? u_al[n] : region == 4 ? u_ar[n] : u_c[n];
    fi[n] = region == 0 ? fl[n] : region == 1 ? fr[n] : region == 2 ? f_hll[n]
            : region == 3 ? f_al : region == 4 ? f_ar : f_c;
  }
  // HLL where the chosen state is not finite (an HLL, L or R choice under to_hll stands)
  const bool hll = !to_hll && !all_finite7(ui, fi);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) f[n] = hll ? f_hll[n] : fi[n];
}

// Newman & Hamlin (2014) fixed-point con2prim with Aitken acceleration,
// ConservedToPrimitiveNormal, eos/adiabatic_mhd_sr.cpp:404-522.  prim[5] in natural
// slots (rho, u1, u2, u3, p).  *iters = loop index at exit.  The FP64 instantiation is the
// reference's solve; the FP32 one (tolerance relative to p) only refines a starting guess.
__device__ __forceinline__ double m_acos(double x) { return acos(x); }
__device__ __forceinline__ float m_acos(float x) { return acosf(x); }
__device__ __forceinline__ double m_cos(double x) { return cos(x); }
__device__ __forceinline__ float m_cos(float x) { return __cosf(x); }
__device__ __forceinline__ double m_cbrt(double x) { return cbrt(x); }
__device__ __forceinline__ float m_cbrt(float x) { return cbrtf(x); }

// Loop indices [n0, n1) of the iteration on pgas[3] (the whole solver state at a loop
// index: a solve stopped at any index resumes exactly).  Returns the index at which the
// convergence test passed, or n1.  *last receives the most recently written pressure.
template <typename Real>
__device__ __forceinline__ int sr_nh_loop(Real gamma_adi, Real dd, Real ee, Real mm_sq,
                                          Real bb_sq, Real tt, Real d, Real pgas_min,
                                          Real* pgas, int n0, int n1, Real tol, bool rel_tol,
                                          Real* last) {
  const Real a_min = RC(1.0e-12);
  const Real v_sq_max = RC(1.0) - RC(1.0e-12);
  const Real rr_max = RC(1.0) - RC(1.0e-12);
  const Real PI_ = RC(3.1415926535897932);
  int n;
  for (n = n0; n < n1; ++n) {
    if (n % 3 != 2) {
      Real a = ee + pgas[n % 3] + RC(0.5) * bb_sq;
      a = smax(a, a_min);
      Real phi = m_acos(RC(1.0) / a * dsqrt(RC(27.0) * d / (RC(4.0) * a)));
      Real eee = a / RC(3.0) - RC(2.0) / RC(3.0) * a * m_cos(RC(2.0) / RC(3.0) * (phi + PI_));
      Real ll = eee - bb_sq;
      Real v_sq = (mm_sq * (ll * ll) + (tt * tt) * (bb_sq + RC(2.0) * ll)) /
                  ((ll * (bb_sq + ll)) * (ll * (bb_sq + ll)));
      v_sq = smin(smax(v_sq, RC(0.0)), v_sq_max);
      Real gamma_sq = RC(1.0) / (RC(1.0) - v_sq);
      Real gamma = dsqrt(gamma_sq);
      Real wgas = ll / gamma_sq;
      Real rho = dd / gamma;
      Real pn = (gamma_adi - RC(1.0)) / gamma_adi * (wgas - rho);
      pn = smax(pn, pgas_min);
      pgas[(n + 1) % 3] = pn;
      *last = pn;
      const Real lim = rel_tol ? tol * pn : tol;
      if (pn > pgas_min && dabs(pn - pgas[n % 3]) < lim) break;
    } else {
      Real rr = (pgas[2] - pgas[1]) / (pgas[1] - pgas[0]);
      if (!isfinite(rr) || dabs(rr) > rr_max) continue;
      pgas[0] = pgas[1] + (pgas[2] - pgas[1]) / (RC(1.0) - rr);
      pgas[0] = smax(pgas[0], pgas_min);
      *last = pgas[0];
      const Real lim = rel_tol ? tol * pgas[0] : tol;
      if (pgas[0] > pgas_min && dabs(pgas[0] - pgas[2]) < lim) break;
    }
  }
  return n;
}

// the quantities of the solve that do not change between iterations (NH 5.7-5.9)
template <typename Real>
__device__ __forceinline__ void sr_nh_setup(Real ee, Real mm_sq, Real bb_sq, Real tt,
                                            Real* d_out, Real* pgas_min_out) {
  const Real pgas_uniform_min = RC(1.0e-12);
  Real d = RC(0.5) * (mm_sq * bb_sq - tt * tt);
  d = smax(d, RC(0.0));
  Real pgas_min = m_cbrt(RC(27.0) / RC(4.0) * d) - ee - RC(0.5) * bb_sq;
  *d_out = d;
  *pgas_min_out = smax(pgas_min, pgas_uniform_min);
}

// primitives from the converged pressure (adiabatic_mhd_sr.cpp:486-521)
template <typename Real>
__device__ __forceinline__ bool sr_nh_finish(Real dd, Real ee, Real mm_sq, Real mm1,
                                             Real mm2, Real mm3, Real bb_sq, Real bb1,
                                             Real bb2, Real bb3, Real tt, Real d, Real pgas,
                                             Real* prim, Real* p_gamma_lor, Real* p_pmag) {
  const Real a_min = RC(1.0e-12);
  const Real v_sq_max = RC(1.0) - RC(1.0e-12);
  const Real PI_ = RC(3.1415926535897932);
  prim[IPR] = pgas;
  if (!isfinite(prim[IPR])) return false;
  Real a = ee + prim[IPR] + RC(0.5) * bb_sq;
  a = smax(a, a_min);
  Real phi = m_acos(RC(1.0) / a * dsqrt(RC(27.0) * d / (RC(4.0) * a)));
  Real eee = a / RC(3.0) - RC(2.0) / RC(3.0) * a * m_cos(RC(2.0) / RC(3.0) * (phi + PI_));
  Real ll = eee - bb_sq;
  Real v_sq = (mm_sq * (ll * ll) + (tt * tt) * (bb_sq + RC(2.0) * ll)) /
              ((ll * (bb_sq + ll)) * (ll * (bb_sq + ll)));
  v_sq = smin(smax(v_sq, RC(0.0)), v_sq_max);
  Real gamma_sq = RC(1.0) / (RC(1.0) - v_sq);
  Real gamma = dsqrt(gamma_sq);
  prim[IDN] = dd / gamma;
  if (!isfinite(prim[IDN])) return false;
  Real ss = tt / ll;
  Real v1 = (mm1 + ss * bb1) / (ll + bb_sq);
  Real v2 = (mm2 + ss * bb2) / (ll + bb_sq);
  Real v3 = (mm3 + ss * bb3) / (ll + bb_sq);
  prim[IVX] = gamma * v1;
  prim[IVY] = gamma * v2;
  prim[IVZ] = gamma * v3;
  if (!isfinite(prim[IVX]) || !isfinite(prim[IVY]) || !isfinite(prim[IVZ])) return false;
  *p_gamma_lor = gamma;
  *p_pmag = RC(0.5) * (bb_sq / gamma_sq + ss * ss);
  return true;
}

template <typename Real>
__device__ __forceinline__ bool sr_normal_t(Real gamma_adi, Real dd, Real ee, Real mm_sq,
                                            Real mm1, Real mm2, Real mm3, Real bb_sq,
                                            Real bb1, Real bb2, Real bb3, Real tt,
                                            Real pgas_old, Real* prim, Real* p_gamma_lor,
                                            Real* p_pmag, int* iters, int max_iterations,
                                            Real tol, bool rel_tol) {
  Real d, pgas_min, last;
  sr_nh_setup<Real>(ee, mm_sq, bb_sq, tt, &d, &pgas_min);
  Real pgas[3];
  pgas[0] = smax(pgas_old, pgas_min);
  const int n = sr_nh_loop<Real>(gamma_adi, dd, ee, mm_sq, bb_sq, tt, d, pgas_min, pgas, 0,
                                 max_iterations, tol, rel_tol, &last);
  *iters = n;
  if (n == max_iterations) return false;
  return sr_nh_finish<Real>(dd, ee, mm_sq, mm1, mm2, mm3, bb_sq, bb1, bb2, bb3, tt, d,
                            pgas[(n + 1) % 3], prim, p_gamma_lor, p_pmag);
}

// the reference's solve: at most 15 iterations, absolute tolerance 1e-12 on p
// (adiabatic_mhd_sr.cpp:409-411)
__device__ __forceinline__ bool sr_normal(double gamma_adi, double dd, double ee,
                                          double mm_sq, double mm1, double mm2, double mm3,
                                          double bb_sq, double bb1, double bb2, double bb3,
                                          double tt, double pgas_old, double* prim,
                                          double* p_gamma_lor, double* p_pmag, int* iters) {
  return sr_normal_t<double>(gamma_adi, dd, ee, mm_sq, mm1, mm2, mm3, bb_sq, bb1, bb2, bb3,
                             tt, pgas_old, prim, p_gamma_lor, p_pmag, iters, 15, 1.0e-12,
                             false);
}

// A start for the FP64 solve: up to max_it FP32 iterations of the same fixed-point scheme
// from p0 (test relative to p, tol), returning the converged or the last FP32 iterate (p0
// itself if the FP32 iteration produced nothing usable).  *iters = FP32 passes.
__device__ __forceinline__ double sr_refine_f32(double gamma_adi, double dd, double ee,
                                                double mm_sq, double bb_sq, double tt,
                                                double p0, int max_it, float tol,
                                                int* iters) {
  float d, pmin, last = (float)p0, pg[3];
  sr_nh_setup<float>((float)ee, (float)mm_sq, (float)bb_sq, (float)tt, &d, &pmin);
  pg[0] = fmaxf((float)p0, pmin);
  const int k = sr_nh_loop<float>((float)gamma_adi, (float)dd, (float)ee, (float)mm_sq,
                                  (float)bb_sq, (float)tt, d, pmin, pg, 0, max_it, tol, true,
                                  &last);
  *iters = k < max_it ? k + 1 : max_it;
  const float p = k < max_it ? pg[(k + 1) % 3] : last;
  return (isfinite(p) && p > 0.0f) ? (double)p : p0;
}

struct SRFloors { double gamma_adi, dfloor, pfloor, sigma_max, beta_min, gamma_max; };

// One cell of EquationOfState::ConservedToPrimitive (SR), adiabatic_mhd_sr.cpp:87-268:
// conserved floors, solve from the guess in prim (the output array's stale value,
// :143-154), fallback, floors, gamma ceiling, conserved re-sync.  cons[5] (natural slots)
// may be rewritten (*fixed set).  Returns false if the solve failed.
//
// pstart > 0 replaces the first solve's start (the FP32 path passes the stale pressure
// refined in FP32; the fallback state is still the stale primitives), and max_first < 15
// caps the first solve: a cell that has not converged by then returns with *deferred set
// and prim, cons untouched, to be solved again in full by a later pass (the solve is
// deterministic, so the result is the same as one uncapped call).
//
// When the first solve starts from pstart and fails within the reference's 15 passes, the
// cell is solved again from the reference's own start, the stale pressure (*fallback_out
// set): the reference's solve is the per-cell fallback of any other start.  *passes_out
// (may be NULL) receives the FP64 loop passes of every solve the cell ran.
__device__ __forceinline__ bool sr_c2p_cell(const SRFloors& fp, double* cons, double bc1,
                                            double bc2, double bc3, double* prim,
                                            bool* fixed_out, int* iters, double pstart = 0.0,
                                            int max_first = 15, bool* deferred = nullptr,
                                            int* passes_out = nullptr,
                                            bool* fallback_out = nullptr) {
  const double gamma_adi = fp.gamma_adi;
  const double mm_sq_ee_sq_max = 1.0 - 1.0e-12;
  double dd = cons[IDN], ee = cons[IPR];
  double mm_sq = cons[IVX] * cons[IVX] + cons[IVY] * cons[IVY] + cons[IVZ] * cons[IVZ];
  double mm1 = cons[IVX], mm2 = cons[IVY], mm3 = cons[IVZ];
  double bb_sq = bc1 * bc1 + bc2 * bc2 + bc3 * bc3;
  double tt = cons[IVX] * bc1 + cons[IVY] * bc2 + cons[IVZ] * bc3;
  bool fixed = false;
  double density_floor_local = fp.dfloor, pressure_floor_local = fp.pfloor;
  if (dd < density_floor_local) { dd = density_floor_local; fixed = true; }
  double ee_min = density_floor_local + pressure_floor_local / (gamma_adi - 1.0) + 0.5 * bb_sq;
  if (ee < ee_min) { ee = ee_min; fixed = true; }
  double mm_sq_max = mm_sq_ee_sq_max * (ee * ee);
  if (mm_sq > mm_sq_max) {
    double factor = sqrt(mm_sq_max / mm_sq);
    mm_sq = mm_sq_max;
    mm1 *= factor; mm2 *= factor; mm3 *= factor;
    tt *= factor;
    fixed = true;
  }
  double rho_old = smax(prim[IDN], density_floor_local);
  double pgas_old = smax(prim[IPR], pressure_floor_local);
  double u1_old = prim[IVX], u2_old = prim[IVY], u3_old = prim[IVZ];
  double gamma = 0.0, pmag = 0.0;
  bool success = sr_normal_t<double>(gamma_adi, dd, ee, mm_sq, mm1, mm2, mm3, bb_sq, bc1, bc2,
                                     bc3, tt, pstart > 0.0 ? pstart : pgas_old, prim, &gamma,
                                     &pmag, iters, max_first, 1.0e-12, false);
  if (!success && max_first < 15 && *iters == max_first) {  // capped: finish later
    if (deferred) *deferred = true;
    *fixed_out = false;
    return false;
  }
  int passes = *iters < 15 ? *iters + 1 : 15;
  if (!success && pstart > 0.0) {  // the reference's start, the stale pressure
    int it_ref;
    success = sr_normal_t<double>(gamma_adi, dd, ee, mm_sq, mm1, mm2, mm3, bb_sq, bc1, bc2,
                                  bc3, tt, pgas_old, prim, &gamma, &pmag, &it_ref, 15,
                                  1.0e-12, false);
    passes += it_ref < 15 ? it_ref + 1 : 15;
    if (fallback_out) *fallback_out = true;
  }
  if (!success) {
    prim[IDN] = rho_old; prim[IPR] = pgas_old;
    prim[IVX] = u1_old; prim[IVY] = u2_old; prim[IVZ] = u3_old;
    fixed = true;
  }
  if (fp.sigma_max > 0.0)
    density_floor_local = smax(density_floor_local, 2.0 * pmag / fp.sigma_max);
  if (fp.beta_min > 0.0)
    pressure_floor_local = smax(pressure_floor_local, fp.beta_min * pmag);
  double rho_add = smax(density_floor_local - prim[IDN], 0.0);
  double pgas_add = smax(pressure_floor_local - prim[IPR], 0.0);
  if (success && (rho_add > 0.0 || pgas_add > 0.0)) {
    double wgas_add = rho_add + gamma_adi / (gamma_adi - 1.0) * pgas_add;
    dd += rho_add * gamma;
    ee += wgas_add * (gamma * gamma) + pgas_add;
    int it2;
    success = sr_normal(gamma_adi, dd, ee, mm_sq, mm1, mm2, mm3, bb_sq, bc1, bc2, bc3, tt,
                        pgas_old, prim, &gamma, &pmag, &it2);
    passes += it2 < 15 ? it2 + 1 : 15;
    if (!success) {
      prim[IDN] = rho_old; prim[IPR] = pgas_old;
      prim[IVX] = u1_old; prim[IVY] = u2_old; prim[IVZ] = u3_old;
    }
    fixed = true;
  }
  if (!success)
    gamma = sqrt(1.0 + prim[IVX] * prim[IVX] + prim[IVY] * prim[IVY] + prim[IVZ] * prim[IVZ]);
  bool velocity_ceiling = false;
  if (gamma > fp.gamma_max) {
    double factor = sqrt((fp.gamma_max * fp.gamma_max - 1.0) / (gamma * gamma - 1.0));
    prim[IVX] *= factor; prim[IVY] *= factor; prim[IVZ] *= factor;
    fixed = true;
    velocity_ceiling = true;
  }
  if (velocity_ceiling) {
    double b0 = prim[IVX] * bc1 + prim[IVY] * bc2 + prim[IVZ] * bc3;
    pmag = 0.5 * (bb_sq / (gamma * gamma) + (b0 / gamma) * (b0 / gamma));
  }
  density_floor_local = fp.dfloor;
  if (fp.sigma_max > 0.0)
    density_floor_local = smax(density_floor_local, 2.0 * pmag / fp.sigma_max);
  pressure_floor_local = fp.pfloor;
  if (fp.beta_min > 0.0)
    pressure_floor_local = smax(pressure_floor_local, fp.beta_min * pmag);
  if (prim[IDN] < density_floor_local) { prim[IDN] = density_floor_local; fixed = true; }
  if (prim[IPR] < pressure_floor_local) { prim[IPR] = pressure_floor_local; fixed = true; }
  if (!success) {
    prim[IDN] = density_floor_local;
    prim[IPR] = pressure_floor_local;
    prim[IVX] = prim[IVY] = prim[IVZ] = 0.0;
  }
  if (fixed) {
    double u1 = prim[IVX], u2 = prim[IVY], u3 = prim[IVZ], rho = prim[IDN], pg = prim[IPR];
    gamma = sqrt(1.0 + u1 * u1 + u2 * u2 + u3 * u3);
    double b0 = bc1 * u1 + bc2 * u2 + bc3 * u3;
    double b1 = (bc1 + b0 * u1) / gamma;
    double b2 = (bc2 + b0 * u2) / gamma;
    double b3 = (bc3 + b0 * u3) / gamma;
    double b_sq = -(b0 * b0) + b1 * b1 + b2 * b2 + b3 * b3;
    double wgas = rho + gamma_adi / (gamma_adi - 1.0) * pg;
    double wtot = wgas + b_sq;
    pmag = 0.5 * b_sq;
    cons[IDN] = rho * gamma;
    cons[IPR] = wtot * (gamma * gamma) - (b0 * b0) - (pg + pmag);
    cons[IVX] = wtot * gamma * u1 - b0 * b1;
    cons[IVY] = wtot * gamma * u2 - b0 * b2;
    cons[IVZ] = wtot * gamma * u3 - b0 * b3;
  }
  *fixed_out = fixed;
  if (passes_out) *passes_out = passes;
  return success;
}

#undef RC
}  // namespace athgpu
