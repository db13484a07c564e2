// Stage-update kernels over all MeshBlocks of a uniform single-level mesh.
//
// Device layout: every field is one allocation holding all MeshBlocks back to back, each
// block in the reference's AthenaArray layout (athena_arrays.hpp:140-143, ghosts
// included): cells [nb][nvar][nc3][nc2][nc1], x1 faces [nb][nc3][nc2][nc1+1], x2 faces
// [nb][nc3][nc2+1][nc1], x3 faces [nb][nc3+1][nc2][nc1], edges x1e [nb][nc3+1][nc2+1][nc1],
// x2e [nb][nc3+1][nc2][nc1+1], x3e [nb][nc3][nc2+1][nc1+1] (athena.hpp:128-148).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "physics.cuh"
#include "c2p_net.cuh"

namespace athgpu {

typedef long long i64;

// Multi-level mesh data (mesh refinement; all zero/null on a uniform mesh).  Coarse
// buffers hold, per block, the half-resolution arrays that restriction and prolongation
// use (the reference's coarse_cons_, coarse_prim_, coarse_b_, coarse_bcc_): cells
// [ncc3][ncc2][ncc1] with ncc = nx/2 + 2 NGHOST, coarse interior cis..cie etc.
struct DevML {
  int on;
  const int* nblev;     // [nb][27] neighbour levels, (ox3+1)*9+(ox2+1)*3+(ox1+1); -1 none
  const int* nbrt;      // [nb][56][10] neighbour lists (gid, level, ox1..3, type, fi1, fi2, fid, eid)
  const int* nnbr;      // [nb]
  const int* eflag;     // [nb][12] block edge touches no finer block
  const int* nfine;     // [nb][12] blocks of the finest level around the edge
  const int* fmask;     // [nb] bit f: face f has finer neighbours (flux correction)
  const int* level;     // [nb]
  int ncc1, ncc2, ncc3, cis, cie, cjs, cje, cks, cke, cng;
  i64 nccell, ncf1, ncf2, ncf3;
  void* ccons;          // coarse U   [nb][5][ncc]   (bulk precision)
  void* cprim;          // coarse W   [nb][5][ncc]
  void* cbcc;           // coarse bcc [nb][3][ncc]
  double *cb1, *cb2, *cb3;   // coarse face field
  void* scons;          // restricted U as sent to coarser blocks
  double *sb1, *sb2, *sb3;   // restricted face field as sent
  const double *cx1v, *cx2v, *cx3v;   // coarse cell centres [nb][ncc?]
  const double *fx1v, *fx2v, *fx3v;   // fine cell centres [nb][nc?]
  void* fcorr;          // restricted fine fluxes [nb][6][nfmax][5]
  int nfmax;            // max over faces of nx_a * nx_b
  void *ecorr1, *ecorr2, *ecorr3;     // corrected block-boundary edges (edge layout)
};

// Division of an int in [0, 2^31) by a divisor d >= 2 fixed when the mesh is set up, in
// two instructions instead of the ~20 of a division by a run-time value: with
// l = ceil(log2 d), mul = ceil(2^(31+l) / d) < 2^32 and x < 2^31, floor(x * mul / 2^(31+l))
// = floor(x / d) (the round-up multiplier's error x (mul - 2^(31+l)/d) / 2^(31+l) stays
// below 2^-l <= 1/d, so it never reaches the next multiple of d).
struct FastDiv {
  unsigned mul;
  int shift;  // l - 1
};
inline FastDiv make_fastdiv(int d) {
  int l = 0;
  while ((1LL << l) < d) ++l;
  FastDiv f;
  f.mul = (unsigned)(((1ULL << (31 + l)) + (unsigned long long)d - 1) / (unsigned long long)d);
  f.shift = l - 1;
  return f;
}
__device__ __forceinline__ int fdiv(int x, FastDiv f) {
  return (int)(__umulhi((unsigned)x, f.mul) >> f.shift);
}

struct DevMesh {
  int nb, nbx1, nbx2, nbx3;
  int nx1, nx2, nx3, ng;
  int nc1, nc2, nc3;
  int is, ie, js, je, ks, ke;
  i64 ncell, nf1, nf2, nf3, ne1, ne2, ne3;  // per-block element counts
  FastDiv fd_nc1, fd_nc2, fd_n1, fd_n2;     // divisors nc1, nc2, nx1 + 1, nx2 + 1
  FastDiv fd_r1, fd_r2;                     // divisors nx1 + 2, nx2 + 2
  double gamma, dfloor, pfloor, cfl, tlim;
  const double* dx1f;  // [nb][nc1]
  const double* dx2f;  // [nb][nc2]
  const double* dx3f;  // [nb][nc3]
  const double* plm;   // [nb][3][2][ncmax]: (x?f(c+1)-x?v(c))/dx?f(c), (x?v(c)-x?f(c))/dx?f(c)
  int ncmax;
  const int* nbr;      // [nb][27] neighbour block for offset ((o3+1)*3+(o2+1))*3+(o1+1)
  // FP32 copies of the scalars and coordinate arrays above (rounded once on the host,
  // the values the FP32 kernels would otherwise convert per use)
  float gammaf, dfloorf, pfloorf;
  const float* dx1f32;
  const float* dx2f32;
  const float* dx3f32;
  const float* plm32;
  // mesh-face boundary flags (inner x1, outer x1, ..., outer x3: 0 periodic, 1 outflow,
  // 2 reflecting); any_bc is set when one of them is not periodic
  int bc[6];
  int any_bc;
  DevML ml;
};

// device-resident scalars of the time integrator
struct DevClock {
  double dt, time;
  unsigned long long dtmin_bits;  // min over cells of dx/speed, as ordered bits
  int c2p_floor_count;
  float dtf;                      // dt rounded to FP32 (written with dt)
  double dt_prev;                 // the dt of the last completed cycle
  unsigned long long dtmin_prev_bits;  // the minimum the last NewTimeStep used
  // relativistic con2prim statistics since the last reset (athgpu_stats): cells solved,
  // FP64 Newman-Hamlin passes over all attempts, cells re-solved from the reference's
  // start after their own start failed, cells left unconverged
  unsigned long long sr_cells, sr_passes, sr_fallbacks, sr_unconverged;
  int sweep_timeout;  // a bulk-copy wait of a sweep timed out (athgpu_stats)
};

// The mesh scalars, coordinates and dt in the kernel's arithmetic type: the FP64 kernels
// read the FP64 values, the FP32 kernels their FP32 roundings (the same values a
// conversion at each use would give, without the FP64-pipe conversion).
__device__ __forceinline__ double rgamma(const DevMesh& m, double) { return m.gamma; }
__device__ __forceinline__ float rgamma(const DevMesh& m, float) { return m.gammaf; }
__device__ __forceinline__ double rdfloor(const DevMesh& m, double) { return m.dfloor; }
__device__ __forceinline__ float rdfloor(const DevMesh& m, float) { return m.dfloorf; }
__device__ __forceinline__ double rpfloor(const DevMesh& m, double) { return m.pfloor; }
__device__ __forceinline__ float rpfloor(const DevMesh& m, float) { return m.pfloorf; }
__device__ __forceinline__ const double* rdx(const DevMesh& m, int d, double) {
  return d == 0 ? m.dx1f : d == 1 ? m.dx2f : m.dx3f;
}
__device__ __forceinline__ const float* rdx(const DevMesh& m, int d, float) {
  return d == 0 ? m.dx1f32 : d == 1 ? m.dx2f32 : m.dx3f32;
}
__device__ __forceinline__ const double* rplm(const DevMesh& m, double) { return m.plm; }
__device__ __forceinline__ const float* rplm(const DevMesh& m, float) { return m.plm32; }
__device__ __forceinline__ double rdt(const DevClock* c, double) { return c->dt; }
__device__ __forceinline__ float rdt(const DevClock* c, float) { return c->dtf; }

__device__ __forceinline__ i64 cidx(const DevMesh& m, int b, int n, int nvar, int k, int j,
                                    int i) {
  return (((i64)b * nvar + n) * m.nc3 + k) * m.nc2 * m.nc1 + (i64)j * m.nc1 + i;
}
__device__ __forceinline__ i64 f1idx(const DevMesh& m, int b, int k, int j, int i) {
  return (i64)b * m.nf1 + ((i64)k * m.nc2 + j) * (m.nc1 + 1) + i;
}
__device__ __forceinline__ i64 f2idx(const DevMesh& m, int b, int k, int j, int i) {
  return (i64)b * m.nf2 + ((i64)k * (m.nc2 + 1) + j) * m.nc1 + i;
}
__device__ __forceinline__ i64 f3idx(const DevMesh& m, int b, int k, int j, int i) {
  return (i64)b * m.nf3 + ((i64)k * m.nc2 + j) * m.nc1 + i;
}
__device__ __forceinline__ i64 e1idx(const DevMesh& m, int b, int k, int j, int i) {
  return (i64)b * m.ne1 + ((i64)k * (m.nc2 + 1) + j) * m.nc1 + i;
}
__device__ __forceinline__ i64 e2idx(const DevMesh& m, int b, int k, int j, int i) {
  return (i64)b * m.ne2 + ((i64)k * m.nc2 + j) * (m.nc1 + 1) + i;
}
__device__ __forceinline__ i64 e3idx(const DevMesh& m, int b, int k, int j, int i) {
  return (i64)b * m.ne3 + ((i64)k * (m.nc2 + 1) + j) * (m.nc1 + 1) + i;
}
// per-block face-array offset of (k,j,i) for the face arrays of direction DIR
template <int DIR>
__device__ __forceinline__ i64 fidx(const DevMesh& m, int b, int k, int j, int i) {
  return DIR == 0 ? f1idx(m, b, k, j, i) : DIR == 1 ? f2idx(m, b, k, j, i)
                                                    : f3idx(m, b, k, j, i);
}
// flux scratch arrays are variable-major over the whole mesh, [5][nb][face]: stride of
// one variable
template <int DIR>
__device__ __forceinline__ i64 fsize(const DevMesh& m) {
  return (i64)m.nb * (DIR == 0 ? m.nf1 : DIR == 1 ? m.nf2 : m.nf3);
}

// Asynchronous global -> shared copies of single elements (cp.async, completion tracked
// per thread with commit/wait groups).
template <typename Real>
__device__ __forceinline__ void cp_async_elem(Real* smem_dst, const Real* gsrc) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  if (sizeof(Real) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(gsrc) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Bulk copies of the tensor-memory-access (TMA) unit: one thread moves a contiguous row
// global -> shared (16-byte aligned addresses, size a multiple of 16), completion counted
// in bytes on an mbarrier.  A CTA's consumers wait on the mbarrier's phase with a bounded
// spin (about 0.1 s of SM clock) that records a timeout in *err instead of hanging.
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gsrc, unsigned bytes,
                                         unsigned long long* mbar) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
  const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar);
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
      "[%3];\n" ::"r"(d),
      "l"(gsrc), "r"(bytes), "r"(mb)
      : "memory");
}
__device__ __forceinline__ void mbar_init_1(unsigned long long* mbar) {
  const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar);
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mb) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// the single producer arrival of a phase, announcing `bytes` of copies to come
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long* mbar, unsigned bytes) {
  const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar);
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mb),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_parity(unsigned long long* mbar, unsigned parity) {
  const unsigned mb = (unsigned)__cvta_generic_to_shared(mbar);
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(mb), "r"(parity)
      : "memory");
  return done != 0;
}
__device__ __forceinline__ void mbar_wait_bounded(unsigned long long* mbar, unsigned parity,
                                                  int* err) {
  if (mbar_try_parity(mbar, parity)) return;
  const long long t0 = clock64();
  while (!mbar_try_parity(mbar, parity)) {
    if (clock64() - t0 > 200000000LL) {  // about 0.1 s: record and stop waiting
      if (err) atomicExch(err, 1);
      return;
    }
  }
}

// PLM of the seven wave components of one cell from its stencil window q[0..2][n] (cells
// c-1 .. c+1) and the cell's PLM coefficients cp, cm; FP32: components (0,1), (2,3), (4,5)
// as packed pairs (plm_two)
template <typename Real>
__device__ __forceinline__ void plm_waves(const Real (*q)[NWAVE], Real cp, Real cm, Real* qlp,
                                          Real* qrm) {
  int n = 0;
  if constexpr (sizeof(Real) == 4) {
#pragma unroll
    for (; n + 1 < NWAVE; n += 2) {
      float2 a, c;
      plm_two(make_float2(q[0][n], q[0][n + 1]), make_float2(q[1][n], q[1][n + 1]),
              make_float2(q[2][n], q[2][n + 1]), cp, cm, a, c);
      qlp[n] = a.x;
      qlp[n + 1] = a.y;
      qrm[n] = c.x;
      qrm[n + 1] = c.y;
    }
  }
#pragma unroll
  for (; n < NWAVE; ++n) plm_one<Real>(q[0][n], q[1][n], q[2][n], cp, cm, qlp[n], qrm[n]);
}

// PPM of the seven wave components of one cell from its stencil window q[0..4][n] (cells
// c-2 .. c+2 along the sweep).  lo[n]: the cell's limited lower interface, formed here
// unless CARRY (then the caller's: the previous cell's upper one); up[n] receives the
// limited upper interface (lo and up may alias).  FP32: the components (0,1), (2,3), (4,5)
// as packed pairs (ppm_face2, ppm_finish2).
template <typename Real, bool CARRY>
__device__ __forceinline__ void ppm_waves(const Real (*q)[NWAVE], Real* lo, Real* up,
                                          Real* qlp, Real* qrm, bool fast) {
  if constexpr (sizeof(Real) == 4) {
    if (!fast) {
#pragma unroll
      for (int n = 0; n + 1 < NWAVE; n += 2) {
        float2 v[5];
#pragma unroll
        for (int t = 0; t < 5; ++t) v[t] = make_float2(q[t][n], q[t][n + 1]);
        const float2 l = CARRY ? make_float2(lo[n], lo[n + 1])
                               : ppm_face2(v[0], v[1], v[2], v[3]);
        const float2 u = ppm_face2(v[1], v[2], v[3], v[4]);
        float2 a, c;
        ppm_finish2(v[0], v[1], v[2], v[3], v[4], l, u, a, c);
        qlp[n] = a.x;
        qlp[n + 1] = a.y;
        qrm[n] = c.x;
        qrm[n + 1] = c.y;
        up[n] = u.x;
        up[n + 1] = u.y;
      }
      if constexpr (NWAVE % 2 == 1) {
        constexpr int n = NWAVE - 1;
        const Real l = CARRY ? lo[n] : ppm_face<Real>(q[0][n], q[1][n], q[2][n], q[3][n]);
        up[n] = ppm_face<Real>(q[1][n], q[2][n], q[3][n], q[4][n]);
        ppm_finish<Real>(q[0][n], q[1][n], q[2][n], q[3][n], q[4][n], l, up[n], qlp[n],
                         qrm[n], false);
      }
      return;
    }
  }
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) {
    const Real l = CARRY ? lo[n] : ppm_face<Real>(q[0][n], q[1][n], q[2][n], q[3][n]);
    up[n] = ppm_face<Real>(q[1][n], q[2][n], q[3][n], q[4][n]);
    ppm_finish<Real>(q[0][n], q[1][n], q[2][n], q[3][n], q[4][n], l, up[n], qlp[n], qrm[n],
                     fast);
  }
}

// ---------------------------------------------------------------------------------------
// Reconstruction of one cell along DIR: wave vector (natural order d, v1, v2, v3, p, then
// the two transverse cell-centred field components, plm.cpp:45-57 / :196-208) of the
// cell and its neighbours; returns the upper-face value qlp and lower-face value qrm.
template <typename Real, int DIR, int ORDER>
__device__ __forceinline__ void recon_cell(const DevMesh& m, const Real* __restrict__ w,
                                           const Real* __restrict__ bcc, int b, int k,
                                           int j, int i, Real* qlp, Real* qrm) {
  const i64 sw = DIR == 0 ? 1 : DIR == 1 ? (i64)m.nc1 : (i64)m.nc1 * m.nc2;
  const i64 base_w = cidx(m, b, 0, NHYDRO, k, j, i);
  const i64 base_b = cidx(m, b, 0, 3, k, j, i);
  const i64 vs = m.ncell;  // variable stride within a block
  Real q5[ORDER >= 3 ? 5 : ORDER == 2 ? 3 : 1][NWAVE];  // PLM / PPM: every component's stencil
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) {
    const Real* src;
    i64 o;
    if (n < NHYDRO) {
      src = w;
      o = base_w + n * vs;
    } else {
      src = bcc;
      o = base_b + (i64)((DIR + n - NHYDRO + 1) % 3) * vs;
    }
    if (ORDER == 1) {  // DonorCellX1/2/3, reconstruct/dc.cpp:24-104
      Real q = __ldg(src + o);
      qlp[n] = q;
      qrm[n] = q;
    } else if (ORDER == 2) {
#pragma unroll
      for (int t = 0; t < 3; ++t) q5[t][n] = __ldg(src + o + (t - 1) * sw);
    } else {
#pragma unroll
      for (int t = 0; t < 5; ++t) q5[t][n] = __ldg(src + o + (t - 2) * sw);
    }
  }
  if (ORDER == 2) {
    const int c = DIR == 0 ? i : DIR == 1 ? j : k;
    const Real* pc = rplm(m, Real()) + ((i64)b * 3 + DIR) * 2 * m.ncmax;
    plm_waves<Real>(q5, __ldg(pc + c), __ldg(pc + m.ncmax + c), qlp, qrm);
  }
  if (ORDER >= 3) {
    Real up[NWAVE];
    ppm_waves<Real, false>(q5, nullptr, up, qlp, qrm, ORDER == 4);
  }
  if (ORDER == 3) {  // ApplyPrimitiveFloors, adiabatic_mhd.cpp:162-172 (ppm.cpp:326-331)
    const Real dfl = rdfloor(m, Real()), pfl = rpfloor(m, Real());
    qlp[IDN] = (qlp[IDN] > dfl) ? qlp[IDN] : dfl;
    qlp[IPR] = (qlp[IPR] > pfl) ? qlp[IPR] : pfl;
    qrm[IDN] = (qrm[IDN] > dfl) ? qrm[IDN] : dfl;
    qrm[IPR] = (qrm[IPR] > pfl) ? qrm[IPR] : pfl;
  }
}

// The seven wave variables of one cell for a sweep along DIR: w[0..4] at wp + n*vs, the
// two transverse cell-centred field components (DIR+1)%3, (DIR+2)%3 at bp.
template <typename Real, int DIR>
__device__ __forceinline__ void load_wave(const Real* __restrict__ wp,
                                          const Real* __restrict__ bp, i64 vs, Real* v) {
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) v[n] = __ldg(wp + n * vs);
  v[IBY] = __ldg(bp + ((DIR + 1) % 3) * vs);
  v[IBZ] = __ldg(bp + ((DIR + 2) % 3) * vs);
}

// ApplyPrimitiveFloors on the PPM face states (adiabatic_mhd.cpp:162-172, ppm.cpp:326-331)
template <typename Real>
__device__ __forceinline__ void ppm_floors(const DevMesh& m, Real* qlp, Real* qrm) {
  const Real dfl = rdfloor(m, Real()), pfl = rpfloor(m, Real());
  qlp[IDN] = (qlp[IDN] > dfl) ? qlp[IDN] : dfl;
  qlp[IPR] = (qlp[IPR] > pfl) ? qlp[IPR] : pfl;
  qrm[IDN] = (qrm[IDN] > dfl) ? qrm[IDN] : dfl;
  qrm[IPR] = (qrm[IPR] > pfl) ? qrm[IPR] : pfl;
}

// recon_cell on a stencil window: win[q] is cell c - R + q along the
// sweep (R = 0, 1, 2 for DC, PLM, PPM); cp/cm are the PLM coefficients of cell c.  Same
// arithmetic as recon_cell.
template <typename Real, int ORDER>
__device__ __forceinline__ void recon_window(const DevMesh& m, const Real (*win)[NWAVE],
                                             Real cp, Real cm, Real* qlp, Real* qrm) {
  if constexpr (ORDER >= 3) {
    Real up[NWAVE];
    ppm_waves<Real, false>(win, nullptr, up, qlp, qrm, ORDER == 4);
  } else {
    if (ORDER == 2) {
      plm_waves<Real>(win, cp, cm, qlp, qrm);
    } else {
#pragma unroll
      for (int n = 0; n < NWAVE; ++n) {
        qlp[n] = win[0][n];
        qrm[n] = win[0][n];
      }
    }
  }
  if (ORDER == 3) ppm_floors(m, qlp, qrm);
}

// The per-cell parts of Hydro::CalculateVelocityDifferences
// (hydro/calculate_velocity_differences.cpp:23-64, 3-D) for faces normal to DIR: the
// normal velocity vn and, for the transverse axes a1 = (DIR+1)%3 and a2 = (DIR+2)%3, the
// smaller one-sided difference of that axis's velocity along that axis (t1, t2).  The face
// between cells c-1 and c then has dvn = vn(c) - vn(c-1) and
// dvt = min(min(t1(c-1), t1(c)), min(t2(c-1), t2(c))), the reference's dvl, dvr, dwl, dwr.
template <typename Real, int DIR>
__device__ __forceinline__ void vel_cell(const DevMesh& m, const Real* __restrict__ w, int b,
                                         int k, int j, int i, Real& vn, Real& t1, Real& t2) {
  const Real* p = w + cidx(m, b, 0, NHYDRO, k, j, i);
  const i64 vs = m.ncell;
  constexpr int a1 = (DIR + 1) % 3, a2 = (DIR + 2) % 3;
  const i64 s1 = a1 == 0 ? 1 : a1 == 1 ? (i64)m.nc1 : (i64)m.nc1 * m.nc2;
  const i64 s2 = a2 == 0 ? 1 : a2 == 1 ? (i64)m.nc1 : (i64)m.nc1 * m.nc2;
  vn = __ldg(p + (IVX + DIR) * vs);
  const Real* q1 = p + (IVX + a1) * vs;
  const Real c1 = __ldg(q1);
  t1 = smin(__ldg(q1 + s1) - c1, c1 - __ldg(q1 - s1));
  const Real* q2 = p + (IVX + a2) * vs;
  const Real c2 = __ldg(q2);
  t2 = smin(__ldg(q2 + s2) - c2, c2 - __ldg(q2 - s2));
}

// Riemann solve on one face of direction DIR: stores the two face EMFs and the CT weight
// (calculate_fluxes.cpp:102/:221/:340; hlld.cpp:372-376) and returns the five hydro
// fluxes in natural slots (IDN, IM1, IM2, IM3, IEN).
// RS 7 (LHLLD) also takes the face's velocity differences dvn, dvt (vel_cell below).
// PK: FP32 HLLD / HLLE on packed left/right pairs (hlld_pk, hlle_pk); off where the
// caller's register budget would spill with it (the donor-cell x3 sweep).
template <typename Real, int DIR, int RS, bool PK = true>
__device__ __forceinline__ void solve_face(const DevMesh& m, const Real* wl, const Real* wr,
                                           Real bx, Real dx, Real dt, i64 fo, Real* fn,
                                           Real* __restrict__ ey, Real* __restrict__ ez,
                                           Real* __restrict__ wct, Real dvn = Real(0),
                                           Real dvt = Real(0)) {
  // local order: d, v_normal, v_t1, v_t2, p, By, Bz (hlld.cpp:42-43)
  const int ivx = IVX + DIR, ivy = IVX + (DIR + 1) % 3, ivz = IVX + (DIR + 2) % 3;
  Real wli[NWAVE] = {wl[IDN], wl[ivx], wl[ivy], wl[ivz], wl[IPR], wl[IBY], wl[IBZ]};
  Real wri[NWAVE] = {wr[IDN], wr[ivx], wr[ivy], wr[ivz], wr[IPR], wr[IBY], wr[IBZ]};
  Real f[NWAVE];
  const Real gam = rgamma(m, Real());
  if constexpr (RS == 0 && PK && sizeof(Real) == 4) hlld_pk(gam, wli, wri, bx, f);
  else if constexpr (RS == 1 && PK && sizeof(Real) == 4) hlle_pk(gam, wli, wri, bx, f);
  else if (RS == 0) hlld<Real>(gam, wli, wri, bx, f);
  else if (RS == 1) hlle<Real>(gam, wli, wri, bx, f);
  else if (RS == 3) llf<Real>(gam, wli, wri, bx, f);
  else if (RS == 4) roe<Real>(gam, wli, wri, bx, f);
  else if (RS == 7) hlld<Real, true>(gam, wli, wri, bx, f, dvn, dvt);  // low-dissipation
  else if (RS == 5) llf_sr<Real>(gam, wli, wri, bx, f);  // special relativity, LLF
  else if (RS == 6) hlld_sr<Real>(gam, wli, wri, bx, f);  // special relativity, HLLD
  else hlle_sr<Real>(gam, wli, wri, bx, f);  // RS 2: special relativity, HLLE
  fn[IDN] = f[0];
  fn[ivx] = f[1];
  fn[ivy] = f[2];
  fn[ivz] = f[3];
  fn[IPR] = f[4];
  ey[fo] = -f[5];
  ez[fo] = f[6];
  wct[fo] = weight_for_ct<Real>(f[0], wl[IDN], wr[IDN], dx, dt);
}

// Multi-level meshes: the flux of block b through its face fid (0..5) at transverse
// position (pa, pb) (pa along the first transverse axis, of extent nta), replaced by the
// finer blocks' restricted fluxes when that face is shared with finer blocks
// (flux_correction_cc.cpp:237-286; written by ml_fine_flux_kernel)
template <typename Real>
__device__ __forceinline__ bool ml_face_override(const DevMesh& m, int b, int fid, int pa,
                                                 int pb, int nta, Real* fn) {
  if (!m.ml.on || !((__ldg(m.ml.fmask + b) >> fid) & 1)) return false;
  const Real* p = (const Real*)m.ml.fcorr +
                  (((i64)b * 6 + fid) * m.ml.nfmax + (i64)pb * nta + pa) * NHYDRO;
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) fn[n] = p[n];
  return true;
}

// The flux divergence of Hydro::AddFluxDivergence (add_flux_divergence.cpp:50-94) is
// accumulated by the three sweeps in the reference's order: the x1 sweep stores
// dflx = A1*F1(i+1) - A1*F1(i), the x2 sweep adds (A2*F2(j+1) - A2*F2(j)), the x3 sweep
// adds (A3*F3(k+1) - A3*F3(k)) and applies u_out = u_in - wght*dflx/vol.  So no flux
// array is stored.  Cartesian areas and volumes, coordinates.cpp:448-548.
struct UpdateArgs {
  double beta;            // stage weight (time_integrator.cpp:216-217 vl2, :441-444 rk2)
  int stage;
  const void* uin;        // U^n
  void* uout;             // U* (stage 1) or U^n+1 (stage 2; may alias uin)
  void* ulo;              // compensation of U (FP32 path)
  // rk2 stage 2: the register average u = g1*U* + g2*U^n (WeightedAve with gamma =
  // (1/2, 1/2, 0), weighted_ave.cpp:161-230) before the flux divergence; NULL otherwise
  // (vl2's gamma = (0, 1, 0) is a register swap)
  const void* uavg;
  double g1, g2;
  int* err;               // set when a bulk-copy wait of a sweep timed out
};

// x1 sweep: rows (k in [ks-1,ke+1], j in [js-1,je+1]) of cells i in [is-1, ie+1] of block
// blockIdx.y, flattened over rows.  A warp reconstructs 32 consecutive cells: lane L > 0
// solves the left face of its cell with the upper-face state of lane L-1 (shuffle up), and
// lanes 1..30 form their cell's x1 flux difference with the face flux of lane L+1 (shuffle
// down).  Warps advance by 30 cells, so every cell is reconstructed at most twice, every
// face solved at most twice (identical duplicate stores) and every difference formed once.
// (FP32: eight CTAs per SM for donor cell, measured faster despite a few spilled
// registers; seven, i.e. at most 73 registers, otherwise)
template <typename Real, int ORDER, int RS>
__global__ void __launch_bounds__(128, sizeof(Real) == 4 ? (ORDER == 1 ? 8 : 7) : 1)
flux_x1_kernel(DevMesh m, const Real* __restrict__ w, const Real* __restrict__ bcc,
               const double* __restrict__ b1, const DevClock* __restrict__ clk,
               Real* __restrict__ dflx, Real* __restrict__ e3, Real* __restrict__ e2,
               Real* __restrict__ wct) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int ncr = m.nx1 + 2, nrj = m.nx2 + 2, nrk = m.nx3 + 2;
  const int per = nrk * nrj * ncr;
  const int g = warp * 30 + lane - 1;
  const bool valid = (g >= 0) && (g < per);
  Real qlp[NWAVE], qrm[NWAVE];
  const int b = blockIdx.y;
  int k = 0, j = 0, c = 0;
  if (valid) {
    const int row = fdiv(g, m.fd_r1);
    c = g - row * ncr;
    const int kq = fdiv(row, m.fd_r2);
    j = row - kq * nrj + m.js - 1;
    k = kq + m.ks - 1;
    recon_cell<Real, 0, ORDER>(m, w, bcc, b, k, j, m.is - 1 + c, qlp, qrm);
  } else {
#pragma unroll
    for (int n = 0; n < NWAVE; ++n) qlp[n] = qrm[n] = Real(0);
  }
  Real wl[NWAVE];
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) wl[n] = __shfl_up_sync(0xffffffffu, qlp[n], 1);
  // LHLLD: the face's velocity differences from this cell and the one of lane L-1
  Real dvn = Real(0), dvt = Real(0);
  if (RS == 7) {
    Real vn = Real(0), t1 = Real(0), t2 = Real(0);
    if (valid) vel_cell<Real, 0>(m, w, b, k, j, m.is - 1 + c, vn, t1, t2);
    const Real vnl = __shfl_up_sync(0xffffffffu, vn, 1);
    const Real t1l = __shfl_up_sync(0xffffffffu, t1, 1);
    const Real t2l = __shfl_up_sync(0xffffffffu, t2, 1);
    dvn = vn - vnl;
    dvt = smin(smin(t1l, t1), smin(t2l, t2));
  }
  const int i = m.is - 1 + c;
  Real fn[NHYDRO] = {Real(0), Real(0), Real(0), Real(0), Real(0)};
  const bool has_face = valid && lane > 0 && c > 0;
  if (has_face) {
    const i64 fo = f1idx(m, b, k, j, i);
    solve_face<Real, 0, RS>(m, wl, qrm, to_real(__ldg(b1 + fo), Real()),
                            __ldg(rdx(m, 0, Real()) + (i64)b * m.nc1 + i), rdt(clk, Real()),
                            fo, fn, e3, e2, wct, dvn, dvt);
    if (m.ml.on && (i == m.is || i == m.ie + 1) && j >= m.js && j <= m.je && k >= m.ks &&
        k <= m.ke)
      ml_face_override<Real>(m, b, i == m.is ? 0 : 1, j - m.js, k - m.ks, m.nx2, fn);
  }
  Real fp[NHYDRO];
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) fp[n] = __shfl_down_sync(0xffffffffu, fn[n], 1);
  if (has_face && lane <= 30 && i <= m.ie && j >= m.js && j <= m.je && k >= m.ks &&
      k <= m.ke) {
    const Real x1area = rdx(m, 1, Real())[(i64)b * m.nc2 + j] * rdx(m, 2, Real())[(i64)b * m.nc3 + k];
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n)
      dflx[cidx(m, b, n, NHYDRO, k, j, i)] = (x1area * fp[n] - x1area * fn[n]);
  }
}

// x2 / x3 sweeps: a thread owns one column (b, transverse index, i) and walks a segment
// of cells along the sweep, carrying the previous cell's upper-face state and the
// previous face's flux in registers (the reference's wl/wlb swap,
// calculate_fluxes.cpp:184-237 and :304-356).  Columns: x2: k in [ks-1,ke+1],
// i in [is-1,ie+1]; x3: j in [js-1,je+1], i in [is-1,ie+1].  A segment of cells
// [c0,c1] solves faces c0..c1+1, so neighbouring segments share one face.
//
// BULK (x3 only, uniform meshes): the stencil cells, the face field and the update
// operands are staged by the TMA unit instead of per-thread cp.async.  The CTA's threads
// then own consecutive positions of a k-plane (rows js-1..je+1 at full width nc1, columns
// outside [is-1,ie+1] idle), so every staged row is one contiguous 16-byte-aligned range
// that one thread copies with cp.async.bulk, completion counted on an mbarrier; a CTA
// barrier per step frees the ring slot the next copy overwrites.  Same arithmetic and
// results as the cp.async staging.
template <typename Real, int DIR, int ORDER, int RS, int KAHAN, int BULK = 0>
__global__ void __launch_bounds__(128, sizeof(Real) == 4 ? 4 : 1)
flux_sweep_kernel(DevMesh m, int seg, const Real* __restrict__ w,
                  const Real* __restrict__ bcc, const double* __restrict__ bn,
                  const DevClock* __restrict__ clk, Real* __restrict__ dflx,
                  Real* __restrict__ ey, Real* __restrict__ ez, Real* __restrict__ wct,
                  UpdateArgs ua) {
  static_assert(!BULK || DIR == 2, "bulk staging is the x3 sweep's");
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  const int ni = m.nx1 + 2;
  const int nt = (DIR == 1) ? m.nx3 + 2 : m.nx2 + 2;
  const int ncellsw = (DIR == 1) ? m.nx2 : m.nx3;
  const int nseg = (ncellsw + seg - 1) / seg;
  int ii, tt, b, sg;
  bool active = true;
  int bq = 0;  // BULK: this CTA's first plane position
  if (BULK) {
    const int np = nt * m.nc1;                   // plane positions of rows js-1..je+1
    const int nq = (np + blockDim.x - 1) / blockDim.x;
    if ((i64)blockIdx.x >= (i64)nq * m.nb * nseg) return;  // whole CTA
    const int q = (int)(blockIdx.x % nq);
    const int r2 = (int)(blockIdx.x / nq);
    b = r2 % m.nb;
    sg = r2 / m.nb;
    bq = q * blockDim.x;
    const int p = bq + threadIdx.x;
    tt = p / m.nc1;
    ii = p % m.nc1 - (m.is - 1);
    active = p < np && ii >= 0 && ii < ni;
    if (!active) {  // idle column: keep every index in range (nothing is stored)
      tt = 0;
      ii = 0;
    }
  } else {
    const i64 total = (i64)nseg * m.nb * nt * ni;
    if (t >= total) return;
    ii = (int)(t % ni);
    i64 r = t / ni;
    tt = (int)(r % nt);
    r /= nt;
    b = (int)(r % m.nb);
    sg = (int)(r / m.nb);
  }
  const int i = m.is - 1 + ii;
  const int lo = (DIR == 1) ? m.js : m.ks;
  const int c0 = lo + sg * seg;
  const int c1 = min(c0 + seg - 1, lo + ncellsw - 1);
  const int trans = (DIR == 1 ? m.ks : m.js) - 1 + tt;  // k for x2, j for x3
  const bool interior = active && ii >= 1 && ii <= m.nx1 &&
                        trans >= (DIR == 1 ? m.ks : m.js) && trans <= (DIR == 1 ? m.ke : m.je);
  const Real dt = rdt(clk, Real());
  const Real* dxs = rdx(m, DIR, Real()) + (i64)b * (DIR == 1 ? m.nc2 : m.nc3);
  // area of this direction's faces (the same for every face of a uniform block)
  const Real dx1 = rdx(m, 0, Real())[(i64)b * m.nc1 + i];
  const Real dxt = (DIR == 1) ? rdx(m, 2, Real())[(i64)b * m.nc3 + trans]
                              : rdx(m, 1, Real())[(i64)b * m.nc2 + trans];
  const Real area = dx1 * dxt;
  const int k0 = (DIR == 1) ? trans : 0, j0 = (DIR == 2) ? trans : 0;
  // Shared-memory staging, per thread (layout [slot][variable][thread]: conflict-free; no
  // thread reads another thread's column, so no barrier is needed):
  //  * ring: WN+1 cell slots x 7 wave variables.  The cell s+R+1 needed by the next step
  //    is copied in with cp.async while this step's face is solved, so each cell's seven
  //    values are read from memory once and the load latency hides behind a Riemann solve;
  //  * fbuf: the normal face field of faces s and s+1 (FP64, double-buffered);
  //  * aux: the divergence register (x2) or divergence, U^n and compensation (x3) of the
  //    cell updated in this step, copied in before the face solve.
  constexpr int R = ORDER >= 3 ? 2 : ORDER == 2 ? 1 : 0;
  constexpr int WN = 2 * R + 1;
  constexpr int NS = WN + 1;
  constexpr int NAUX = DIR == 1 ? NHYDRO : 3 * NHYDRO;
  extern __shared__ __align__(16) unsigned char sweep_smem[];
  const int bd = blockDim.x;
  double* fbuf = reinterpret_cast<double*>(sweep_smem) + threadIdx.x;          // [2][bd]
  Real* ring = reinterpret_cast<Real*>(sweep_smem + 2 * sizeof(double) * bd) + threadIdx.x;
  Real* aux = ring + NS * NWAVE * bd;                                            // [NAUX][bd]
  const i64 sw = (DIR == 1) ? (i64)m.nc1 : (i64)m.nc1 * m.nc2;
  const i64 vs = m.ncell;
  const int cfirst = c0 - 1 - R;
  const Real* wp = w + ((DIR == 1) ? cidx(m, b, 0, NHYDRO, k0, cfirst, i)
                                   : cidx(m, b, 0, NHYDRO, cfirst, j0, i));
  const Real* bp = bcc + ((DIR == 1) ? cidx(m, b, 0, 3, k0, cfirst, i)
                                     : cidx(m, b, 0, 3, cfirst, j0, i));
  // BULK: the CTA's rows start at plane position bq of row js-1 (column 0); thread 0 issues
  // every copy of a step, counted on the CTA's mbarrier
  __shared__ unsigned long long sweep_mbar;
  unsigned mbar_phase = 0;
  const i64 prow = BULK ? (i64)(m.js - 1) * m.nc1 + bq : 0;
  Real* ring0 = ring - threadIdx.x;  // the CTA's row starts (BULK)
  double* fbuf0 = fbuf - threadIdx.x;
  Real* aux0 = aux - threadIdx.x;
  const unsigned rowb = (unsigned)(bd * sizeof(Real));
  auto issue = [&](int rel) {  // cell cfirst + rel -> slot rel % NS
    const int slot = rel % NS;
    if (BULK) {
      if (threadIdx.x != 0) return;
      const int c = cfirst + rel;
#pragma unroll
      for (int n = 0; n < NWAVE; ++n) {
        const Real* src = n < NHYDRO ? w + cidx(m, b, n, NHYDRO, c, 0, 0) + prow
                                     : bcc + cidx(m, b, (DIR + 1 + (n - NHYDRO)) % 3, 3, c,
                                                  0, 0) + prow;
        bulk_g2s(ring0 + (slot * NWAVE + n) * bd, src, rowb, &sweep_mbar);
      }
      return;
    }
    const Real* wc = wp + rel * sw;
    const Real* bc = bp + rel * sw;
#pragma unroll
    for (int n = 0; n < NWAVE; ++n) {
      const Real* src = n < NHYDRO ? wc + n * vs
                                   : bc + ((DIR + 1 + (n - NHYDRO)) % 3) * vs;
      cp_async_elem<Real>(ring + (slot * NWAVE + n) * bd, src);
    }
  };
  auto issue_face = [&](int f) {  // normal field of face f
    if (BULK) {
      if (threadIdx.x != 0) return;
      bulk_g2s(fbuf0 + (f & 1) * bd, bn + f3idx(m, b, f, 0, 0) + prow,
               (unsigned)(bd * sizeof(double)), &sweep_mbar);
      return;
    }
    const i64 fo = (DIR == 1) ? f2idx(m, b, k0, f, i) : f3idx(m, b, f, j0, i);
    cp_async_elem<double>(fbuf + (f & 1) * bd, bn + fo);
  };
  // BULK: the producer's arrival of a step, announcing its bytes, comes before its copies
  const unsigned cell_bytes = NWAVE * rowb, face_bytes = (unsigned)(bd * sizeof(double));
  const unsigned aux_bytes = (KAHAN ? 3 : 2) * NHYDRO * rowb;
  auto bulk_expect = [&](unsigned bytes) {
    if (threadIdx.x == 0) mbar_arrive_tx(&sweep_mbar, bytes);
  };
  auto bulk_wait = [&]() {
    mbar_wait_bounded(&sweep_mbar, mbar_phase, ua.err);
    mbar_phase ^= 1u;
  };
  auto window = [&](int rel0, Real (*win)[NWAVE]) {  // cells cfirst+rel0 .. +WN-1
#pragma unroll
    for (int q = 0; q < WN; ++q) {
      const int slot = (rel0 + q) % NS;
#pragma unroll
      for (int n = 0; n < NWAVE; ++n) win[q][n] = ring[(slot * NWAVE + n) * bd];
    }
  };
  if (BULK) {
    if (threadIdx.x == 0) mbar_init_1(&sweep_mbar);
    __syncthreads();
    bulk_expect((WN + 1) * cell_bytes + face_bytes);
  }
  for (int q = 0; q <= WN; ++q) issue(q);  // cells c0-1-R .. c0+R
  issue_face(c0);
  if (BULK) {
    bulk_wait();
  } else {
    cp_async_commit();
    cp_async_wait_all();
  }
  const Real* pc = rplm(m, Real()) + ((i64)b * 3 + DIR) * 2 * m.ncmax;
  Real wl[NWAVE], qlp[NWAVE], qrm[NWAVE];
  Real fprev[NHYDRO];
  Real dphc[ORDER >= 3 ? NWAVE : 1];  // PPM: limited lower interface of the current cell
  {
    Real win[WN][NWAVE];
    window(0, win);
    if constexpr (ORDER >= 3) {
      ppm_waves<Real, false>(win, nullptr, dphc, wl, qrm, ORDER == 4);
      if (ORDER == 3) ppm_floors(m, wl, qrm);  // time/floor_ppm_fast is false
    } else {
      recon_window<Real, ORDER>(m, win, ORDER == 2 ? __ldg(pc + c0 - 1) : Real(0),
                                ORDER == 2 ? __ldg(pc + m.ncmax + c0 - 1) : Real(0), wl,
                                qrm);
    }
  }
  const Real* uin = (const Real*)ua.uin;
  Real* uout = (Real*)ua.uout;
  Real* ulo = (Real*)ua.ulo;
  const Real* uavg = (const Real*)ua.uavg;
  // LHLLD: the velocity-difference parts of the cell below the next face (vel_cell)
  Real vn_p = Real(0), t1_p = Real(0), t2_p = Real(0);
  if (RS == 7 && active)
    vel_cell<Real, DIR>(m, w, b, DIR == 1 ? k0 : c0 - 1, DIR == 1 ? c0 - 1 : j0, i, vn_p,
                        t1_p, t2_p);
  for (int s = c0; s <= c1 + 1; ++s) {
    const int rel0 = s - R - cfirst;  // window = cells s-R..s+R
    const bool upd = s > c0 && interior;  // this step finishes cell s-1
    const int kc = (DIR == 1) ? k0 : s - 1, jc = (DIR == 1) ? s - 1 : j0;
    const i64 cc0 = cidx(m, b, 0, NHYDRO, kc, jc, i);
    // BULK: every thread is done with the slot, the face buffer and the update operands
    // of the previous step before they are overwritten
    if (BULK) {
      __syncthreads();
      bulk_expect((s <= c1 ? cell_bytes + face_bytes : 0u) + (s > c0 ? aux_bytes : 0u));
    }
    if (s <= c1) {  // prefetch cell s+R+1 into the slot of cell s-R-1, and face s+1
      issue(rel0 + WN);
      issue_face(s + 1);
    }
    if (BULK) {
      if (s > c0 && threadIdx.x == 0) {  // the update operands of cell s-1, whole rows
#pragma unroll
        for (int n = 0; n < NHYDRO; ++n) {
          bulk_g2s(aux0 + n * bd, dflx + cidx(m, b, n, NHYDRO, s - 1, 0, 0) + prow, rowb,
                   &sweep_mbar);
          bulk_g2s(aux0 + (NHYDRO + n) * bd, uin + cidx(m, b, n, NHYDRO, s - 1, 0, 0) + prow,
                   rowb, &sweep_mbar);
          if (KAHAN)
            bulk_g2s(aux0 + (2 * NHYDRO + n) * bd,
                     ulo + cidx(m, b, n, NHYDRO, s - 1, 0, 0) + prow, rowb, &sweep_mbar);
        }
      }
    } else {
      if (upd) {
#pragma unroll
        for (int n = 0; n < NHYDRO; ++n) {
          cp_async_elem<Real>(aux + n * bd, dflx + cc0 + n * vs);
          if (DIR == 2) {
            cp_async_elem<Real>(aux + (NHYDRO + n) * bd, uin + cc0 + n * vs);
            if (KAHAN) cp_async_elem<Real>(aux + (2 * NHYDRO + n) * bd, ulo + cc0 + n * vs);
          }
        }
      }
      cp_async_commit();
    }
    {
      Real win[WN][NWAVE];
      window(rel0, win);
      if constexpr (ORDER >= 3) {  // the lower interface is the previous cell's upper one
        ppm_waves<Real, true>(win, dphc, dphc, qlp, qrm, ORDER == 4);
        if (ORDER == 3) ppm_floors(m, qlp, qrm);
      } else {
        recon_window<Real, ORDER>(m, win, ORDER == 2 ? __ldg(pc + s) : Real(0),
                                  ORDER == 2 ? __ldg(pc + m.ncmax + s) : Real(0), qlp, qrm);
      }
    }
    const i64 fo = (DIR == 1) ? f2idx(m, b, k0, s, i) : f3idx(m, b, s, j0, i);
    Real fn[NHYDRO];
    if (active) {
      Real dvn = Real(0), dvt = Real(0);
      if (RS == 7) {
        Real vn, t1, t2;
        vel_cell<Real, DIR>(m, w, b, DIR == 1 ? k0 : s, DIR == 1 ? s : j0, i, vn, t1, t2);
        dvn = vn - vn_p;
        dvt = smin(smin(t1_p, t1), smin(t2_p, t2));
        vn_p = vn;
        t1_p = t1;
        t2_p = t2;
      }
      solve_face<Real, DIR, RS, !(DIR == 2 && ORDER == 1)>(m, wl, qrm,
                                                         to_real(fbuf[(s & 1) * bd], Real()),
                                __ldg(dxs + s), dt, fo, fn, ey, ez, wct, dvn, dvt);
    } else {
#pragma unroll
      for (int n = 0; n < NHYDRO; ++n) fn[n] = Real(0);
    }
    if (m.ml.on && interior && (s == lo || s == lo + ncellsw))
      ml_face_override<Real>(m, b, 2 * DIR + (s == lo ? 0 : 1), i - m.is,
                             trans - (DIR == 1 ? m.ks : m.js), m.nx1, fn);
    // this step's aux values and the next step's cell and face
    if (BULK) bulk_wait();
    else cp_async_wait_all();
    if (upd) {
      // cell s-1: this direction's flux difference
      if (DIR == 1) {
        int n0 = 0;
        if constexpr (sizeof(Real) == 4) {  // FP32: components (0,1), (2,3) packed
#pragma unroll
          for (; n0 + 1 < NHYDRO; n0 += 2) {
            const float2 d = add2(make_float2(aux[n0 * bd], aux[(n0 + 1) * bd]),
                                  fma2(pk(area), make_float2(fn[n0], fn[n0 + 1]),
                                       mul2(pk(-area), make_float2(fprev[n0], fprev[n0 + 1]))));
            dflx[cc0 + n0 * vs] = d.x;
            dflx[cc0 + (n0 + 1) * vs] = d.y;
          }
        }
#pragma unroll
        for (int n = n0; n < NHYDRO; ++n) {
          Real d = aux[n * bd];
          d += (area * fn[n] - area * fprev[n]);
          dflx[cc0 + n * vs] = d;
        }
      } else {
        const Real dx2 = rdx(m, 1, Real())[(i64)b * m.nc2 + jc];
        const Real dx3 = rdx(m, 2, Real())[(i64)b * m.nc3 + kc];
        const Real vol = dx1 * dx2 * dx3;
        // beta is 1/2 or 1, so beta * (FP32 dt) equals the FP32 rounding of beta * dt
        const Real wght = (sizeof(Real) == 8) ? (Real)(ua.beta * clk->dt)
                                              : (Real)ua.beta * dt;
        int n0 = 0;
        if constexpr (sizeof(Real) == 4 && KAHAN == 1) {
          if (!uavg) {
            // FP32, no register average: components (0,1), (2,3) on packed pairs, the
            // update as du = (-wght/vol)*d, then the compensated sum of the scalar path
            const float sc = -(wght / vol);
            for (; n0 + 1 < NHYDRO; n0 += 2) {
              const i64 cc = cc0 + n0 * vs;
              const float2 d = add2(make_float2(aux[n0 * bd], aux[(n0 + 1) * bd]),
                                    fma2(pk(area), make_float2(fn[n0], fn[n0 + 1]),
                                         mul2(pk(-area),
                                              make_float2(fprev[n0], fprev[n0 + 1]))));
              const float2 du = mul2(pk(sc), d);
              const float2 hi = make_float2(aux[(NHYDRO + n0) * bd],
                                            aux[(NHYDRO + n0 + 1) * bd]);
              const float2 lw = make_float2(aux[(2 * NHYDRO + n0) * bd],
                                            aux[(2 * NHYDRO + n0 + 1) * bd]);
              if (ua.stage == 1) {
                const float2 o = add2(hi, add2(lw, du));
                uout[cc] = o.x;
                uout[cc + vs] = o.y;
              } else {
                const float2 y = add2(du, lw);
                const float2 t2 = add2(hi, y);
                const float2 r = sub2(y, sub2(t2, hi));
                ulo[cc] = r.x;
                ulo[cc + vs] = r.y;
                uout[cc] = t2.x;
                uout[cc + vs] = t2.y;
              }
            }
            {  // the last component, the same operations
              const int n = NHYDRO - 1;
              const i64 cc = cc0 + n * vs;
              const float d = aux[n * bd] + (area * fn[n] - area * fprev[n]);
              const float du = sc * d;
              const float hi = aux[(NHYDRO + n) * bd], lw = aux[(2 * NHYDRO + n) * bd];
              if (ua.stage == 1) {
                uout[cc] = hi + (lw + du);
              } else {
                const float y = du + lw;
                const float t2 = hi + y;
                ulo[cc] = y - (t2 - hi);
                uout[cc] = t2;
              }
            }
            n0 = NHYDRO;
          }
        }
#pragma unroll
        for (int n = n0; n < NHYDRO; ++n) {
          const i64 cc = cc0 + n * vs;
          Real d = aux[n * bd];
          d += (area * fn[n] - area * fprev[n]);
          if (KAHAN == 0) {
            Real base = aux[(NHYDRO + n) * bd];
            if (uavg) base = (Real)ua.g1 * uavg[cc] + (Real)ua.g2 * base;
            uout[cc] = base - wght * d / vol;
          } else {
            const Real du = -(wght * d / vol);
            Real hi = aux[(NHYDRO + n) * bd], lw = aux[(2 * NHYDRO + n) * bd];
            if (uavg) {
              // g1*U* + g2*(hi + lw) as a new (hi, lw) pair: the products are exact
              // (g = 1/2), their sum's rounding error is recovered (two-sum) into lw
              const Real a = (Real)ua.g1 * uavg[cc], c = (Real)ua.g2 * hi;
              const Real sum = a + c, bv = sum - a;
              lw = ((a - (sum - bv)) + (c - bv)) + (Real)ua.g2 * lw;
              hi = sum;
            }
            if (ua.stage == 1) {
              uout[cc] = hi + (lw + du);
            } else {
              const Real y = du + lw;
              const Real tt2 = hi + y;
              ulo[cc] = y - (tt2 - hi);
              uout[cc] = tt2;
            }
          }
        }
      }
    }
#pragma unroll
    for (int n = 0; n < NWAVE; ++n) wl[n] = qlp[n];
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) fprev[n] = fn[n];
  }
}

// shared-memory bytes of the x2/x3 sweep's staging for a CTA of `threads` threads
__host__ __device__ inline int sweep_smem_bytes(int dir, int order, int real_bytes,
                                                int threads) {
  const int r = order >= 3 ? 2 : order == 2 ? 1 : 0;
  const int naux = dir == 1 ? NHYDRO : 3 * NHYDRO;
  return 2 * 8 * threads + ((2 * r + 2) * NWAVE + naux) * threads * real_bytes;
}

// ---------------------------------------------------------------------------------------
// Field::ComputeCornerE, calculate_corner_e.cpp:124-236 (3-D branch).  The cell-centred
// E = -v x B (cc_e_, :174-181; SR: -(u x B)/u0 with u^i the 4-velocity, :161-172) is
// written by W(U) (store_cce below) and read here.  One thread per corner point
// (b, k, j, i) in [ks,ke+1]x[js,je+1]x[is,ie+1].
// Store the cell-centred E = -v x B of one cell (the values cce() forms), from the
// primitives and cell-centred field just written by W(U): the corner-EMF kernel then reads
// three values per cell instead of forming them from six.
template <typename Real, bool SR>
__device__ __forceinline__ void store_cce(Real* __restrict__ cc, i64 cb, i64 vs, Real v1,
                                          Real v2, Real v3, Real b1, Real b2, Real b3) {
  if (SR) {
    const Real u0 = dsqrt(Real(1.0) + v1 * v1 + v2 * v2 + v3 * v3);
    cc[cb] = (v3 * b2 - v2 * b3) / u0;
    cc[cb + vs] = (v1 * b3 - v3 * b1) / u0;
    cc[cb + 2 * vs] = (v2 * b1 - v1 * b2) / u0;
  } else {
    cc[cb] = v3 * b2 - v2 * b3;
    cc[cb + vs] = v1 * b3 - v3 * b1;
    cc[cb + 2 * vs] = v2 * b1 - v1 * b2;
  }
}

template <typename Real, bool SR>
__global__ void __launch_bounds__(128)
corner_e_kernel(DevMesh m, const Real* __restrict__ cc, const Real* __restrict__ e3x1, const Real* __restrict__ e2x1,
                const Real* __restrict__ w1f, const Real* __restrict__ e1x2,
                const Real* __restrict__ e3x2, const Real* __restrict__ w2f,
                const Real* __restrict__ e1x3, const Real* __restrict__ e2x3,
                const Real* __restrict__ w3f, Real* __restrict__ e1, Real* __restrict__ e2,
                Real* __restrict__ e3) {
  // blockIdx.y (strided) is the MeshBlock, blockIdx.x/threadIdx.x the corner point of it;
  // every array is read at a 32-bit offset from the block's base, relative to (k,j,i)
  const int n1 = m.nx1 + 1, n2 = m.nx2 + 1, n3 = m.nx3 + 1;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n1 * n2 * n3) return;
  const int q = fdiv(r, m.fd_n1);
  const int kq = fdiv(q, m.fd_n2);
  const int i = m.is + (r - q * n1), j = m.js + (q - kq * n2), k = m.ks + kq;
  const int c1 = m.nc1, c2 = m.nc2;
  // in-block offsets of (k,j,i) and the (k, j, i) strides of each layout
  const int of1 = (k * c2 + j) * (c1 + 1) + i, s1j = c1 + 1, s1k = c2 * (c1 + 1);
  const int of2 = (k * (c2 + 1) + j) * c1 + i, s2j = c1, s2k = (c2 + 1) * c1;
  const int of3 = (k * c2 + j) * c1 + i, s3j = c1, s3k = c2 * c1;
  const Real one = Real(1.0), quarter = Real(0.25);
  for (int b = blockIdx.y; b < m.nb; b += gridDim.y) {
  const Real* W1 = w1f + (i64)b * m.nf1;
  const Real* W2 = w2f + (i64)b * m.nf2;
  const Real* W3 = w3f + (i64)b * m.nf3;
  const Real* A3X1 = e3x1 + (i64)b * m.nf1;
  const Real* A2X1 = e2x1 + (i64)b * m.nf1;
  const Real* A1X2 = e1x2 + (i64)b * m.nf2;
  const Real* A3X2 = e3x2 + (i64)b * m.nf2;
  const Real* A1X3 = e1x3 + (i64)b * m.nf3;
  const Real* A2X3 = e2x3 + (i64)b * m.nf3;
  const Real* CB = cc + (i64)b * 3 * m.ncell;
#define OF1(kk, jj, ii) (of1 + ((kk) - k) * s1k + ((jj) - j) * s1j + ((ii) - i))
#define OF2(kk, jj, ii) (of2 + ((kk) - k) * s2k + ((jj) - j) * s2j + ((ii) - i))
#define OF3(kk, jj, ii) (of3 + ((kk) - k) * s3k + ((jj) - j) * s3j + ((ii) - i))
#define W1F(kk, jj, ii) __ldg(W1 + OF1(kk, jj, ii))
#define W2F(kk, jj, ii) __ldg(W2 + OF2(kk, jj, ii))
#define W3F(kk, jj, ii) __ldg(W3 + OF3(kk, jj, ii))
#define E3X1(kk, jj, ii) __ldg(A3X1 + OF1(kk, jj, ii))
#define E2X1(kk, jj, ii) __ldg(A2X1 + OF1(kk, jj, ii))
#define E1X2(kk, jj, ii) __ldg(A1X2 + OF2(kk, jj, ii))
#define E3X2(kk, jj, ii) __ldg(A3X2 + OF2(kk, jj, ii))
#define E1X3(kk, jj, ii) __ldg(A1X3 + OF3(kk, jj, ii))
#define E2X3(kk, jj, ii) __ldg(A2X3 + OF3(kk, jj, ii))
#define CC(n, kk, jj, ii) __ldg(CB + (i64)(n) * m.ncell + OF3(kk, jj, ii))
  if (i <= m.ie) {
    Real de1_l3 = (one - W2F(k - 1, j, i)) * (E1X3(k, j, i) - CC(0, k - 1, j, i)) +
                  (W2F(k - 1, j, i)) * (E1X3(k, j - 1, i) - CC(0, k - 1, j - 1, i));
    Real de1_r3 = (one - W2F(k, j, i)) * (E1X3(k, j, i) - CC(0, k, j, i)) +
                  (W2F(k, j, i)) * (E1X3(k, j - 1, i) - CC(0, k, j - 1, i));
    Real de1_l2 = (one - W3F(k, j - 1, i)) * (E1X2(k, j, i) - CC(0, k, j - 1, i)) +
                  (W3F(k, j - 1, i)) * (E1X2(k - 1, j, i) - CC(0, k - 1, j - 1, i));
    Real de1_r2 = (one - W3F(k, j, i)) * (E1X2(k, j, i) - CC(0, k, j, i)) +
                  (W3F(k, j, i)) * (E1X2(k - 1, j, i) - CC(0, k - 1, j, i));
    e1[(i64)b * m.ne1 + (k * (c2 + 1) + j) * c1 + i] =
        quarter * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + E1X2(k - 1, j, i) + E1X2(k, j, i) +
                   E1X3(k, j - 1, i) + E1X3(k, j, i));
  }
  if (j <= m.je) {
    Real de2_l3 = (one - W1F(k - 1, j, i)) * (E2X3(k, j, i) - CC(1, k - 1, j, i)) +
                  (W1F(k - 1, j, i)) * (E2X3(k, j, i - 1) - CC(1, k - 1, j, i - 1));
    Real de2_r3 = (one - W1F(k, j, i)) * (E2X3(k, j, i) - CC(1, k, j, i)) +
                  (W1F(k, j, i)) * (E2X3(k, j, i - 1) - CC(1, k, j, i - 1));
    Real de2_l1 = (one - W3F(k, j, i - 1)) * (E2X1(k, j, i) - CC(1, k, j, i - 1)) +
                  (W3F(k, j, i - 1)) * (E2X1(k - 1, j, i) - CC(1, k - 1, j, i - 1));
    Real de2_r1 = (one - W3F(k, j, i)) * (E2X1(k, j, i) - CC(1, k, j, i)) +
                  (W3F(k, j, i)) * (E2X1(k - 1, j, i) - CC(1, k - 1, j, i));
    e2[(i64)b * m.ne2 + (k * c2 + j) * (c1 + 1) + i] =
        quarter * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + E2X3(k, j, i - 1) + E2X3(k, j, i) +
                   E2X1(k - 1, j, i) + E2X1(k, j, i));
  }
  if (k <= m.ke) {
    Real de3_l2 = (one - W1F(k, j - 1, i)) * (E3X2(k, j, i) - CC(2, k, j - 1, i)) +
                  (W1F(k, j - 1, i)) * (E3X2(k, j, i - 1) - CC(2, k, j - 1, i - 1));
    Real de3_r2 = (one - W1F(k, j, i)) * (E3X2(k, j, i) - CC(2, k, j, i)) +
                  (W1F(k, j, i)) * (E3X2(k, j, i - 1) - CC(2, k, j, i - 1));
    Real de3_l1 = (one - W2F(k, j, i - 1)) * (E3X1(k, j, i) - CC(2, k, j, i - 1)) +
                  (W2F(k, j, i - 1)) * (E3X1(k, j - 1, i) - CC(2, k, j - 1, i - 1));
    Real de3_r1 = (one - W2F(k, j, i)) * (E3X1(k, j, i) - CC(2, k, j, i)) +
                  (W2F(k, j, i)) * (E3X1(k, j - 1, i) - CC(2, k, j - 1, i));
    e3[(i64)b * m.ne3 + (k * (c2 + 1) + j) * (c1 + 1) + i] =
        quarter * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + E3X2(k, j, i - 1) + E3X2(k, j, i) +
                   E3X1(k, j - 1, i) + E3X1(k, j, i));
  }
  }
#undef OF1
#undef OF2
#undef OF3
#undef W1F
#undef W2F
#undef W3F
#undef E3X1
#undef E2X1
#undef E1X2
#undef E3X2
#undef E1X3
#undef E2X3
#undef CC
}

// ---------------------------------------------------------------------------------------
// Same-level EMF correction (flux_correction_fc.cpp:51-260, :689-940, :1355-1530): an
// edge on a block face is the sum of the pre-averaging values of the blocks sharing it,
// own value first and the others in neighbour-list order (faces x1, x2, x3, then the
// edge neighbour; bvals_base.cpp:326-720), times 1/2 (two blocks) or 1/4 (four blocks).
// The neighbour block across offset (o1, o2, o3), or -1 across a physical mesh face.
__device__ __forceinline__ int nbr_of(const DevMesh& m, int b, int o1, int o2, int o3) {
  return __ldg(m.nbr + (i64)b * 27 + ((o3 + 1) * 3 + (o2 + 1)) * 3 + (o1 + 1));
}

// The average of the block-face edges over the blocks sharing them on a same-level mesh,
// done before CT in two launches so that every value averaged is a pre-average one:
// edge_fix_kernel writes the averages of the plan's edges into scratch, edge_put_kernel
// stores them into the edge arrays.  The plan (edge_plan, built when the mesh is set up)
// lists per block its own edges on block faces, x1-directed (n0), then x2- (n1) and
// x3-directed (n2): the in-block offset, then the candidates to add in the order above
// (x1-, x2-, x3-face neighbour, then the edge neighbour for an edge on two faces), each as
// (offset index << 27) | offset in the neighbour, ~0u past the last.
// blockIdx.x covers the plan, blockIdx.y the MeshBlocks: EB per thread, their loads
// issued together.
constexpr int EB = 4;
// MeshBlocks per thread of the face-field ghost exchange (exchange_plan_kernel)
constexpr int EXCHANGE_XB = 8;
template <typename Real>
__global__ void __launch_bounds__(128)
edge_fix_kernel(DevMesh m, const int4* __restrict__ plan, int n0, int n1, int n2,
                const Real* __restrict__ e1, const Real* __restrict__ e2,
                const Real* __restrict__ e3, Real* __restrict__ scratch) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = n0 + n1 + n2;
  if (p >= np) return;
  const int4 q = __ldg(plan + p);
  const Real* e = p < n0 ? e1 : p < n0 + n1 ? e2 : e3;
  const i64 ne = p < n0 ? m.ne1 : p < n0 + n1 ? m.ne2 : m.ne3;
  const unsigned cand[3] = {(unsigned)q.y, (unsigned)q.z, (unsigned)q.w};
  const bool two = cand[1] != ~0u;  // an edge on two block faces: three candidates
  for (int b0 = blockIdx.y; b0 < m.nb; b0 += EB * gridDim.y) {
    Real own[EB], v[EB][3];
    int ok[EB][3];
#pragma unroll
    for (int u = 0; u < EB; ++u) {
      const int b = b0 + u * gridDim.y;
      const bool live = b < m.nb;
      own[u] = live ? __ldg(e + (i64)b * ne + q.x) : Real(0);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const int nb = (live && cand[c] != ~0u)
                           ? __ldg(m.nbr + (i64)b * 27 + (int)(cand[c] >> 27)) : -1;
        ok[u][c] = nb >= 0;
        v[u][c] = nb >= 0 ? __ldg(e + (i64)nb * ne + (int)(cand[c] & 0x7ffffffu)) : Real(0);
      }
    }
#pragma unroll
    for (int u = 0; u < EB; ++u) {
      const int b = b0 + u * gridDim.y;
      if (b >= m.nb) break;
      Real sum = own[u];
      int count = 1;
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (ok[u][c]) { sum += v[u][c]; ++count; }
      Real r;
      if (two) {
        // an edge shared by four blocks is scaled by 1/4; along a physical mesh face by
        // 1/count (flux_correction_fc.cpp:1477-1481)
        r = count == 4 ? sum * Real(0.25) : count == 1 ? own[u]
                                                       : sum * (Real(1.0) / Real(count));
      } else {
        r = count == 2 ? sum * Real(0.5) : own[u];  // (flux_correction_fc.cpp:1362-1380)
      }
      scratch[(i64)b * np + p] = r;
    }
  }
}
template <typename Real>
__global__ void __launch_bounds__(128)
edge_put_kernel(DevMesh m, const int4* __restrict__ plan, int n0, int n1, int n2,
                Real* __restrict__ e1, Real* __restrict__ e2, Real* __restrict__ e3,
                const Real* __restrict__ scratch) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = n0 + n1 + n2;
  if (p >= np) return;
  const int off = __ldg(plan + p).x;
  Real* e = p < n0 ? e1 : p < n0 + n1 ? e2 : e3;
  const i64 ne = p < n0 ? m.ne1 : p < n0 + n1 ? m.ne2 : m.ne3;
  for (int b0 = blockIdx.y; b0 < m.nb; b0 += EB * gridDim.y) {
    Real v[EB];
#pragma unroll
    for (int u = 0; u < EB; ++u) {
      const int b = b0 + u * gridDim.y;
      v[u] = b < m.nb ? scratch[(i64)b * np + p] : Real(0);
    }
#pragma unroll
    for (int u = 0; u < EB; ++u) {
      const int b = b0 + u * gridDim.y;
      if (b < m.nb) e[(i64)b * ne + off] = v[u];
    }
  }
}

// Field::CT, field/ct.cpp:31-116, plus the register average (weighted_ave.cpp), which
// for VL2 and the first RK2 stage reduces to out = in and an in-place update on the
// second VL2 stage; on the second RK2 stage the face starts from g1*B* + g2*B^n (bavg =
// B*, bin = B^n; NULL bavg: no average).  blockIdx.y is the MeshBlock; the CTA computes the block's (wght/area) factors
// once (areas and edge lengths are constant on a uniform block).  A thread owns the cell
// point (k,j,i) of [ks,ke+1]x[js,je+1]x[is,ie+1] and updates the faces whose lower corner
// it is: x1 face (k,j,i) for j<=je, k<=ke; x2 face for i<=ie, k<=ke; x3 face for i<=ie,
// j<=je.  The three faces share the edges e1, e2, e3 at (k,j,i), so a thread reads nine
// edge values for up to three faces.  The block-face edges already hold their corrected
// values: on a same-level mesh the averages (edge_fix_kernel, edge_put_kernel), on a
// multi-level mesh the cross-level corrections (ml_emf_kernel, ml_emf_put_kernel).
// FP64 path (Real = double): (wght/area)*(len*e(+) - len*e(-)) exactly as the reference.
// FP32 path: the corner EMFs are FP32 and the update is ((wght/area)*len)*(e(+) - e(-)) in
// FP64, the difference of the two floats formed on the integer pipe (fsub_f64: the FP64
// subtraction's bits), which leaves two FP64 operations per face on GB300's narrow FP64
// pipe instead of four.  bin/bout may alias.
template <typename Real>
__global__ void __launch_bounds__(256)
ct_kernel(DevMesh m, double beta, const DevClock* __restrict__ clk,
          const Real* __restrict__ e1, const Real* __restrict__ e2,
          const Real* __restrict__ e3, const double* b1in, const double* b2in,
          const double* b3in, double* b1out, double* b2out, double* b3out,
          const double* b1avg, const double* b2avg, const double* b3avg, double g1,
          double g2) {
  const int b = blockIdx.y;
  const double* dx1f = m.dx1f + (i64)b * m.nc1;
  const double* dx2f = m.dx2f + (i64)b * m.nc2;
  const double* dx3f = m.dx3f + (i64)b * m.nc3;
  __shared__ double q[3], ql[6];
  if (threadIdx.x < 3) {
    const double wght = beta * clk->dt;
    const double area = threadIdx.x == 0 ? dx2f[m.js] * dx3f[m.ks]
                      : threadIdx.x == 1 ? dx1f[m.is] * dx3f[m.ks] : dx1f[m.is] * dx2f[m.js];
    q[threadIdx.x] = wght / area;
  }
  __syncthreads();
  if (threadIdx.x < 6) {  // FP32 path: the (wght/area)*len products of the block
    const double lq[6] = {dx3f[m.ks], dx2f[m.js], dx3f[m.ks], dx1f[m.is], dx2f[m.js],
                          dx1f[m.is]};
    ql[threadIdx.x] = q[threadIdx.x / 2] * lq[threadIdx.x];
  }
  __syncthreads();
  const int n1 = m.nx1 + 1, n2 = m.nx2 + 1, n3 = m.nx3 + 1;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n1 * n2 * n3) return;
  const int qr = fdiv(r, m.fd_n1);
  const int kq = fdiv(qr, m.fd_n2);
  const int i = m.is + (r - qr * n1);
  const int j = m.js + (qr - kq * n2);
  const int k = m.ks + kq;
  const bool f1 = j <= m.je && k <= m.ke;
  const bool f2 = i <= m.ie && k <= m.ke;
  const bool f3 = i <= m.ie && j <= m.je;
  const double l1 = dx1f[m.is], l2 = dx2f[m.js], l3 = dx3f[m.ks];
  const bool exact = sizeof(Real) == 8;
  // v -/+ the term of edges ep, em: FP64 path (wght/area)*(len*ep - len*em), then the
  // sum, as the reference; FP32 path one FMA of ((wght/area)*len) and the exact edge
  // difference (written out: the compiler does not contract it through the difference)
  auto upd = [&](double v, bool minus, double qd, double len, double qlen, Real ep,
                 Real em) -> double {
    if (exact) {
      const double t = qd * (len * (double)ep - len * (double)em);
      return minus ? v - t : v + t;
    }
    return __fma_rn(minus ? -qlen : qlen, fsub_f64(ep, em), v);
  };
  // in-block offsets of the edges at (k,j,i) and the block bases of the edge arrays
  const int c1 = m.nc1, c2 = m.nc2;
  const int oe1 = (k * (c2 + 1) + j) * c1 + i;
  const int oe2 = (k * c2 + j) * (c1 + 1) + i;
  const int oe3 = (k * (c2 + 1) + j) * (c1 + 1) + i;
  const Real* E1 = e1 + (i64)b * m.ne1;
  const Real* E2 = e2 + (i64)b * m.ne2;
  const Real* E3 = e3 + (i64)b * m.ne3;
  // the shared edges, each read once (and only where a face of this thread uses it)
  const Real e1c = (f2 || f3) ? __ldg(E1 + oe1) : Real(0);
  const Real e2c = (f1 || f3) ? __ldg(E2 + oe2) : Real(0);
  const Real e3c = (f1 || f2) ? __ldg(E3 + oe3) : Real(0);
  if (f1) {
    const i64 o = (i64)b * m.nf1 + (k * c2 + j) * (c1 + 1) + i;
    double v = b1in[o];
    if (b1avg) v = g1 * b1avg[o] + g2 * v;
    v = upd(v, true, q[0], l3, ql[0],
              __ldg(E3 + oe3 + (c1 + 1)), e3c);
    v = upd(v, false, q[0], l2, ql[1],
              __ldg(E2 + oe2 + c2 * (c1 + 1)), e2c);
    b1out[o] = v;
  }
  if (f2) {
    const i64 o = (i64)b * m.nf2 + (k * (c2 + 1) + j) * c1 + i;
    double v = b2in[o];
    if (b2avg) v = g1 * b2avg[o] + g2 * v;
    v = upd(v, false, q[1], l3, ql[2], __ldg(E3 + oe3 + 1),
              e3c);
    v = upd(v, true, q[1], l1, ql[3],
              __ldg(E1 + oe1 + (c2 + 1) * c1), e1c);
    b2out[o] = v;
  }
  if (f3) {
    const i64 o = (i64)b * m.nf3 + (k * c2 + j) * c1 + i;
    double v = b3in[o];
    if (b3avg) v = g1 * b3avg[o] + g2 * v;
    v = upd(v, true, q[2], l2, ql[4], __ldg(E2 + oe2 + 1),
              e2c);
    v = upd(v, false, q[2], l1, ql[5], __ldg(E1 + oe1 + c1),
              e1c);
    b3out[o] = v;
  }
}

// ---------------------------------------------------------------------------------------
// Same-level periodic ghost exchange: every ghost cell / face receives the value of the
// neighbour block that owns it (bvals_cc.cpp:287-430; face fields bvals_fc.cpp:344-397,
// where a block's own faces along the normal are [is, ie+1]).  In the stage only the face
// fields are exchanged: W(U) reads a ghost cell's conserved state from the owning block
// directly (src_cell below), which is the value the exchange would have copied.  Threads enumerate ghost
// elements only: per block and array, the k slabs, then the j slabs of the interior k
// range, then the i slabs of the interior (k, j) range.
__device__ __forceinline__ int own_map(int idx, int lo, int hi, int n, int* o) {
  if (idx < lo) { *o = -1; return idx + n; }
  if (idx > hi) { *o = 1; return idx - n; }
  *o = 0;
  return idx;
}

// r-th ghost element of an array of extent (N1,N2,N3) whose own part has extent
// (I1,I2,I3) starting at ng in every direction
__device__ __forceinline__ void ghost_coord(int r, int N1, int N2, int N3, int I1, int I2,
                                            int I3, int ng, int& k, int& j, int& i) {
  // per-block ghost counts fit in 32 bits
  const int A = 2 * ng * N2 * N1;
  if (r < A) {
    const int kk = r / (N2 * N1);
    const int rem = r - kk * N2 * N1;
    k = kk < ng ? kk : kk - ng + ng + I3;
    j = rem / N1;
    i = rem % N1;
    return;
  }
  r -= A;
  const int B = 2 * ng * N1 * I3;
  if (r < B) {
    const int kk = r / (2 * ng * N1);
    const int rem = r - kk * 2 * ng * N1;
    k = ng + kk;
    const int jj = rem / N1;
    j = jj < ng ? jj : jj - ng + ng + I2;
    i = rem % N1;
    return;
  }
  r -= B;
  const int kk = r / (2 * ng * I2);
  const int rem = r - kk * 2 * ng * I2;
  k = ng + kk;
  j = ng + rem / (2 * ng);
  const int ii = rem % (2 * ng);
  i = ii < ng ? ii : ii - ng + ng + I1;
}

// I: index type of the element enumeration (32-bit when the whole mesh's ghost count
// fits, which the launch checks).
template <typename T, typename I>
__global__ void __launch_bounds__(256)
exchange_kernel(DevMesh m, int with_u, T* __restrict__ u, double* __restrict__ b1,
                double* __restrict__ b2, double* __restrict__ b3) {
  I t = (I)blockIdx.x * blockDim.x + threadIdx.x;
  const int n1 = m.nx1, n2 = m.nx2, n3 = m.nx3, ng = m.ng;
  // ghost counts per block: cells (none when U's ghosts are not exchanged), x1/x2/x3 faces
  const int gc = with_u ? (int)(m.ncell - (i64)n1 * n2 * n3) : 0;
  const int g1 = (int)(m.nf1 - (i64)(n1 + 1) * n2 * n3);
  const int g2 = (int)(m.nf2 - (i64)n1 * (n2 + 1) * n3);
  const int g3 = (int)(m.nf3 - (i64)n1 * n2 * (n3 + 1));
  int what;
  int per;
  if (t < (I)gc * m.nb) { what = 0; per = gc; }
  else if ((t -= (I)gc * m.nb) < (I)g1 * m.nb) { what = 1; per = g1; }
  else if ((t -= (I)g1 * m.nb) < (I)g2 * m.nb) { what = 2; per = g2; }
  else if ((t -= (I)g2 * m.nb) < (I)g3 * m.nb) { what = 3; per = g3; }
  else return;
  const int b = (int)(t / per);
  const int r = (int)(t - (I)b * per);
  int k, j, i;
  ghost_coord(r, m.nc1 + (what == 1), m.nc2 + (what == 2), m.nc3 + (what == 3),
              n1 + (what == 1), n2 + (what == 2), n3 + (what == 3), ng, k, j, i);
  int o1, o2, o3;
  const int si = own_map(i, m.is, m.ie + (what == 1), n1, &o1);
  const int sj = own_map(j, m.js, m.je + (what == 2), n2, &o2);
  const int sk = own_map(k, m.ks, m.ke + (what == 3), n3, &o3);
  const int sb = nbr_of(m, b, o1, o2, o3);
  if (sb < 0) return;
  if (what == 0) {
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n)
      u[cidx(m, b, n, NHYDRO, k, j, i)] = u[cidx(m, sb, n, NHYDRO, sk, sj, si)];
  } else if (what == 1) {
    b1[f1idx(m, b, k, j, i)] = b1[f1idx(m, sb, sk, sj, si)];
  } else if (what == 2) {
    b2[f2idx(m, b, k, j, i)] = b2[f2idx(m, sb, sk, sj, si)];
  } else {
    b3[f3idx(m, b, k, j, i)] = b3[f3idx(m, sb, sk, sj, si)];
  }
}

// The same exchange from the block's ghost plan (exchange_plan, built when the mesh is set
// up): plan element p is one ghost element of a block, its in-block offset in bits 0-26
// and in bits 27-31 the offset index ((o3+1)*3 + (o2+1))*3 + (o1+1) of the neighbour that
// owns it; the owner's element is at offset dst - delta[what][dir].  The plan holds the
// cell ghosts (n0), then the x1 (n1), x2 (n2) and x3 (n3) face ghosts; blockIdx.x covers
// the plan from p0 (0 with U's ghosts, n0 without), blockIdx.y the MeshBlocks (strided).
// No index division: one plan word and one neighbour-table word per copy.
template <typename T>
__global__ void __launch_bounds__(256)
exchange_plan_kernel(DevMesh m, const unsigned* __restrict__ plan, int p0, int n0, int n1,
                     int n2, int n3, const int* __restrict__ delta, T* u, double* b1,
                     double* b2, double* b3) {
  const int p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n0 + n1 + n2 + n3) return;
  const unsigned wd = __ldg(plan + p);
  const int dst = (int)(wd & 0x7ffffffu), dir = (int)(wd >> 27);
  const int what = p < n0 ? 0 : p < n0 + n1 ? 1 : p < n0 + n1 + n2 ? 2 : 3;
  const int src = dst - __ldg(delta + what * 27 + dir);
  if (what == 0) {
    for (int b = blockIdx.y; b < m.nb; b += gridDim.y) {
      const int sb = __ldg(m.nbr + (i64)b * 27 + dir);
      if (sb < 0) continue;  // a physical mesh face: the boundary functions fill it
#pragma unroll
      for (int n = 0; n < NHYDRO; ++n)
        u[((i64)b * NHYDRO + n) * m.ncell + dst] = u[((i64)sb * NHYDRO + n) * m.ncell + src];
    }
    return;
  }
  // face fields: XB blocks per thread (blockIdx.y + q gridDim.y), their neighbour words
  // and values all loaded before the stores, so the loads overlap (an owner's element is
  // never a ghost, so no store here changes a value loaded here)
  double* f = what == 1 ? b1 : what == 2 ? b2 : b3;
  const i64 nf = what == 1 ? m.nf1 : what == 2 ? m.nf2 : m.nf3;
  constexpr int XB = EXCHANGE_XB;
  for (int b0 = blockIdx.y; b0 < m.nb; b0 += XB * gridDim.y) {
    int sb[XB];
    double v[XB];
#pragma unroll
    for (int q = 0; q < XB; ++q) {
      const int b = b0 + q * gridDim.y;
      sb[q] = b < m.nb ? __ldg(m.nbr + (i64)b * 27 + dir) : -1;
    }
#pragma unroll
    for (int q = 0; q < XB; ++q) v[q] = sb[q] >= 0 ? f[(i64)sb[q] * nf + src] : 0.0;
#pragma unroll
    for (int q = 0; q < XB; ++q)
      if (sb[q] >= 0) f[(i64)(b0 + q * gridDim.y) * nf + dst] = v[q];
  }
}

// ---------------------------------------------------------------------------------------
// Reductions for the CFL time step of W(U) (Hydro::NewBlockTimeStep): warp shuffles, a
// CTA reduction in shared memory and one atomicMin per CTA on the order-preserving bit
// pattern of the positive double.
__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_min(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
// "no time step limit" marker of a cell outside the interior
__device__ __forceinline__ double big_dt(double) { return 1.0e300; }
__device__ __forceinline__ float big_dt(float) { return 3.0e38f; }

// Minimum of v over the CTA, then one atomicMin on the ordered bits of the double (positive
// doubles order like their bit patterns), skipped when it would not lower the stored
// value: most CTAs' minima do not, so the single address sees few atomics.  Every thread
// of the CTA must call it.
template <typename Real>
__device__ __forceinline__ void cta_min_to_clock(Real v, DevClock* clk) {
  __shared__ Real red[32];
  v = warp_min(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    Real x = lane < nw ? red[lane] : big_dt(Real());
    x = warp_min(x);
    if (lane == 0 && x < big_dt(Real())) {
      const unsigned long long bits =
          (unsigned long long)__double_as_longlong((double)x);
      if (bits < *(volatile unsigned long long*)&clk->dtmin_bits)
        atomicMin(&clk->dtmin_bits, bits);
    }
  }
}

// Where W(U) reads the conserved state of cell (b,k,j,i): the cell itself in the
// interior, else the cell of the neighbour block that owns it (same-level mesh); -1 for a
// ghost cell beyond a physical mesh face, which the boundary functions fill instead
// (time_integrator.cpp:2206-2212 leaves those out of W(U)).
__device__ __forceinline__ i64 src_cell(const DevMesh& m, int b, int k, int j, int i,
                                        int nvar, bool* ghost) {
  *ghost = i < m.is || i > m.ie || j < m.js || j > m.je || k < m.ks || k > m.ke;
  if (!*ghost) return cidx(m, b, 0, nvar, k, j, i);
  if (m.ml.on) {
    // multi-level mesh: the ghost cell's own (exchanged or prolongated) U, over the
    // ranges of time_integrator.cpp:2206-2212 (ghosts along an axis only where that face
    // has a neighbour)
    const int* lv = m.ml.nblev + (i64)b * 27;
    if ((i < m.is && lv[12] == -1) || (i > m.ie && lv[14] == -1) ||
        (j < m.js && lv[10] == -1) || (j > m.je && lv[16] == -1) ||
        (k < m.ks && lv[4] == -1) || (k > m.ke && lv[22] == -1))
      return -1;
    return cidx(m, b, 0, nvar, k, j, i);
  }
  int o1, o2, o3;
  const int si = own_map(i, m.is, m.ie, m.nx1, &o1);
  const int sj = own_map(j, m.js, m.je, m.nx2, &o2);
  const int sk = own_map(k, m.ks, m.ke, m.nx3, &o3);
  const int sb = nbr_of(m, b, o1, o2, o3);
  return sb < 0 ? (i64)-1 : cidx(m, sb, 0, nvar, sk, sj, si);
}

// Field::CalculateCellCenteredField (field.cpp:112-180, uniform weights) and the
// Newtonian EquationOfState::ConservedToPrimitive (adiabatic_mhd.cpp:41-90) of one cell,
// from the conserved state at cs (the cell itself, or its owner for a ghost cell) without
// writing anything.
template <typename Real>
struct C2POne {
  Real u_d, u_e, vx, vy, vz, w_p, bcc1, bcc2, bcc3, b1lr, b2lr, b3lr;
  bool dfloored, pfloored;
};
// W(U) of one cell from its six face values and its conserved state at u[cs + n ncell]
template <typename Real>
__device__ __forceinline__ C2POne<Real> c2p_cell(const DevMesh& m, double b1l, double b1r,
                                                 double b2l, double b2r, double b3l,
                                                 double b3r, const Real* u, i64 cs) {
  C2POne<Real> o;
  // the lower faces in the bulk precision (also the dt's |b_face - bcc| term)
  o.b1lr = to_real(b1l, Real());
  o.b2lr = to_real(b2l, Real());
  o.b3lr = to_real(b3l, Real());
  if constexpr (sizeof(Real) == 8) {  // the reference's arithmetic
    const double lw = 0.5, rw = 0.5;
    o.bcc1 = lw * b1l + rw * b1r;
    o.bcc2 = lw * b2l + rw * b2r;
    o.bcc3 = lw * b3l + rw * b3r;
  } else {  // FP32 path: average of the FP32-rounded faces
    o.bcc1 = Real(0.5) * o.b1lr + Real(0.5) * to_real(b1r, Real());
    o.bcc2 = Real(0.5) * o.b2lr + Real(0.5) * to_real(b2r, Real());
    o.bcc3 = Real(0.5) * o.b3lr + Real(0.5) * to_real(b3r, Real());
  }
  const i64 vs = m.ncell;
  const Real gm1 = rgamma(m, Real()) - Real(1.0);
  const Real dfl = rdfloor(m, Real()), pfl = rpfloor(m, Real());
  Real u_d = u[cs], u_m1 = u[cs + vs], u_m2 = u[cs + 2 * vs], u_m3 = u[cs + 3 * vs],
       u_e = u[cs + 4 * vs];
  o.dfloored = !(u_d > dfl);
  u_d = (u_d > dfl) ? u_d : dfl;
  Real di = Real(1.0) / u_d;
  o.vx = u_m1 * di;
  o.vy = u_m2 * di;
  o.vz = u_m3 * di;
  Real pb = Real(0.5) * (o.bcc1 * o.bcc1 + o.bcc2 * o.bcc2 + o.bcc3 * o.bcc3);
  Real e_k = Real(0.5) * di * (u_m1 * u_m1 + u_m2 * u_m2 + u_m3 * u_m3);
  Real w_p = gm1 * (u_e - e_k - pb);
  o.pfloored = !(w_p > pfl);
  o.u_e = (w_p > pfl) ? u_e : ((pfl / gm1) + e_k + pb);
  o.w_p = (w_p > pfl) ? w_p : pfl;
  o.u_d = u_d;
  return o;
}
// the same at cell (b,k,j,i), reading the face fields after the ghost exchange (a ghost
// cell's faces hold its owner's values)
template <typename Real>
__device__ __forceinline__ C2POne<Real> c2p_one(const DevMesh& m, int b, int k, int j, int i,
                                                const double* __restrict__ b1,
                                                const double* __restrict__ b2,
                                                const double* __restrict__ b3,
                                                const Real* u, i64 cs) {
  return c2p_cell<Real>(m, __ldg(b1 + f1idx(m, b, k, j, i)), __ldg(b1 + f1idx(m, b, k, j, i + 1)),
                        __ldg(b2 + f2idx(m, b, k, j, i)), __ldg(b2 + f2idx(m, b, k, j + 1, i)),
                        __ldg(b3 + f3idx(m, b, k, j, i)), __ldg(b3 + f3idx(m, b, k + 1, j, i)),
                        u, cs);
}

// W(U) over whole blocks (ghosts included: a ghost cell reads its conserved state from the
// block that owns it, its faces from the exchanged face fields), fused with
// Hydro::NewBlockTimeStep
// (new_blockdt.cpp:80-103) on the interior when do_dt is set.  The floors' rewrite of U
// (adiabatic_mhd.cpp:83-84) is not done here: an interior cell that needs it is appended
// to flist, and c2p_floor_writeback_kernel rewrites U after every cell (ghost copies
// included) has read the pre-floor state, as with the reference's exchanged ghost copies.
template <typename Real, int KAHAN>
__global__ void __launch_bounds__(128)
c2p_kernel(DevMesh m, int do_dt, const double* __restrict__ b1,
           const double* __restrict__ b2, const double* __restrict__ b3, const Real* u,
           Real* __restrict__ w, Real* __restrict__ bcc, Real* __restrict__ cc,
           DevClock* clk, int* __restrict__ flist, unsigned* __restrict__ fcount) {
  // blockIdx.y (strided) is the MeshBlock, blockIdx.x/threadIdx.x the cell r of it:
  // r = (k nc2 + j) nc1 + i, so q = r / nc1 = k nc2 + j, and the face offsets follow from
  // r, q and k without 64-bit arithmetic
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  Real cell_dt = big_dt(Real());
  if (r < (int)m.ncell) {
    const int q = fdiv(r, m.fd_nc1);
    const int i = r - q * m.nc1;
    const int k = fdiv(q, m.fd_nc2);
    const int j = q - k * m.nc2;
    const bool ghost =
        i < m.is || i > m.ie || j < m.js || j > m.je || k < m.ks || k > m.ke;
    for (int b = blockIdx.y; b < m.nb; b += gridDim.y) {
      bool gh;
      const i64 cs = ghost ? src_cell(m, b, k, j, i, NHYDRO, &gh)
                           : (i64)b * NHYDRO * m.ncell + r;
      if (cs < 0) continue;  // a physical-boundary ghost
      const double* f1 = b1 + (i64)b * m.nf1 + (r + q);
      const double* f2 = b2 + (i64)b * m.nf2 + (r + k * m.nc1);
      const double* f3 = b3 + (i64)b * m.nf3 + r;
      const C2POne<Real> o = c2p_cell<Real>(m, __ldg(f1), __ldg(f1 + 1), __ldg(f2),
                                            __ldg(f2 + m.nc1), __ldg(f3),
                                            __ldg(f3 + (i64)m.nc2 * m.nc1), u, cs);
      const i64 vs = m.ncell;
      const i64 c = (i64)b * NHYDRO * m.ncell + r;
      const i64 cb = (i64)b * 3 * m.ncell + r;
      if ((o.dfloored || o.pfloored) && !ghost) {
        const unsigned slot = atomicAdd(fcount, 1u);
        flist[slot] = (int)(((i64)b * m.nx3 + (k - m.ks)) * m.nx2 * m.nx1 +
                            (i64)(j - m.js) * m.nx1 + (i - m.is));
      }
      if ((o.dfloored || o.pfloored) && do_dt) atomicAdd(&clk->c2p_floor_count, 1);
      w[c] = o.u_d;
      w[c + vs] = o.vx;
      w[c + 2 * vs] = o.vy;
      w[c + 3 * vs] = o.vz;
      w[c + 4 * vs] = o.w_p;
      bcc[cb] = o.bcc1;
      bcc[cb + vs] = o.bcc2;
      bcc[cb + 2 * vs] = o.bcc3;
      store_cce<Real, false>(cc, cb, vs, o.vx, o.vy, o.vz, o.bcc1, o.bcc2, o.bcc3);
      if (do_dt && !ghost) {
        // new_blockdt.cpp:80-103, in the bulk precision on the stored primitives (FP64
        // path: the reference's arithmetic; FP32 path: FP32, reduced in FP64)
        const Real gam = rgamma(m, Real());
        Real dt1 = rdx(m, 0, Real())[(i64)b * m.nc1 + i],
             dt2 = rdx(m, 1, Real())[(i64)b * m.nc2 + j],
             dt3 = rdx(m, 2, Real())[(i64)b * m.nc3 + k];
        Real bx = o.bcc1 + dabs(o.b1lr - o.bcc1);
        Real cf = fast_ms<Real>(gam, o.u_d, o.w_p, o.bcc2, o.bcc3, bx);
        Real speed = smax<Real>(Real(0.0), (dabs(o.vx) + cf));
        dt1 /= (speed);
        bx = o.bcc2 + dabs(o.b2lr - o.bcc2);
        cf = fast_ms<Real>(gam, o.u_d, o.w_p, o.bcc3, o.bcc1, bx);
        speed = smax<Real>(Real(0.0), (dabs(o.vy) + cf));
        dt2 /= (speed);
        bx = o.bcc3 + dabs(o.b3lr - o.bcc3);
        cf = fast_ms<Real>(gam, o.u_d, o.w_p, o.bcc1, o.bcc2, bx);
        speed = smax<Real>(Real(0.0), (dabs(o.vz) + cf));
        dt3 /= (speed);
        cell_dt = smin<Real>(cell_dt, smin<Real>(smin<Real>(dt1, dt2), dt3));
      }
    }
  }
  if (do_dt) cta_min_to_clock<Real>(cell_dt, clk);  // reduced in the bulk precision
}

// The floors' rewrite of U for the interior cells c2p_kernel listed (grid-stride over the
// list; usually empty): density and/or energy replaced by their floored values, the
// compensation of a rewritten component cleared.
template <typename Real, int KAHAN>
__global__ void __launch_bounds__(128)
c2p_floor_writeback_kernel(DevMesh m, const double* __restrict__ b1,
                           const double* __restrict__ b2, const double* __restrict__ b3,
                           Real* u, Real* ulo, const int* __restrict__ flist,
                           const unsigned* __restrict__ fcount) {
  const unsigned n = *fcount;
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int q = flist[e];
    const int nint = m.nx1 * m.nx2 * m.nx3;
    const int b = q / nint;
    int r = q - b * nint;
    const int i = m.is + r % m.nx1;
    r /= m.nx1;
    const int j = m.js + r % m.nx2;
    const int k = m.ks + r / m.nx2;
    const i64 c = cidx(m, b, 0, NHYDRO, k, j, i);
    const C2POne<Real> o = c2p_one<Real>(m, b, k, j, i, b1, b2, b3, u, c);
    const i64 vs = m.ncell;
    if (o.dfloored) {
      u[c] = o.u_d;
      if (KAHAN && ulo) ulo[c] = Real(0);
    }
    if (o.pfloored) {
      u[c + 4 * vs] = o.u_e;
      if (KAHAN && ulo) ulo[c + 4 * vs] = Real(0);
    }
  }
}

// EquationOfState::ConservedToPrimitive for SR MHD (adiabatic_mhd_sr.cpp:72-272) on the
// interior cells, in FP64: the Newman-Hamlin solve of every cell is seeded from the output
// array's previous contents (wout holds the primitives of two con2prim calls ago, the
// reference's w1 register, :143-154 and time_integrator.cpp:2221-2269).  In FP32 mode the
// conserved input is hi + lo and a re-synced conserved state is split back.  When do_dt
// is set the interior cells contribute min(dx1, dx2, dx3) to the CFL reduction (the SR
// branch of new_blockdt.cpp:74 keeps the widths: signal speed 1).
//
// The start of the FP64 solve (START):
//   C2P_START_STALE    the stale pressure, the reference's start (the FP64 path);
//   C2P_START_REFINED  the stale pressure refined by FP32 iterations of the same scheme;
//   C2P_START_NETWORK  the con2prim network's pressure for the cell (BF16 tcgen05
//                      evaluation of the CTA's 128 cells, c2p_net.cuh), refined in FP32.
// A start other than the stale pressure that does not converge within the reference's 15
// passes is followed by the reference's own solve from the stale pressure (sr_c2p_cell).
//
// Warp-coherent two-phase schedule: the iteration count varies from cell to cell and a
// warp runs as long as its slowest lane, so phase 1 caps the first solve at max_first
// passes and appends each cell still iterating to the queue (with its start pressure in
// qstart); phase 2 runs the whole con2prim of the queued cells again from that start
// (grid-stride over the count).  The solve is deterministic, so the result equals one
// uncapped pass.  Ghost cells are not solved: a ghost's primitives equal its owner's (same
// conserved state, same stale guess, both kept equal since initialization), so
// copy_ghost_prims_kernel copies them afterwards.  Every finished cell adds to the
// con2prim statistics of the clock (warp-aggregated).
constexpr int C2P_START_STALE = 0, C2P_START_REFINED = 1, C2P_START_NETWORK = 2;

template <typename Real, int KAHAN, int START>
__global__ void __launch_bounds__(128)
c2p_sr_kernel(DevMesh m, SRFloors fp, int do_dt, const double* __restrict__ b1,
              const double* __restrict__ b2, const double* __restrict__ b3, Real* u,
              Real* ulo, Real* __restrict__ wout, Real* __restrict__ bcc,
              Real* __restrict__ cc, DevClock* clk, int phase, int max_first,
              int* __restrict__ queue, unsigned* __restrict__ qcount,
              double* __restrict__ qstart, const float* __restrict__ net,
              int* __restrict__ net_err) {
  const int n1 = m.nx1, n2 = m.nx2, n3 = m.nx3;
  const long long ninterior = (long long)m.nb * n1 * n2 * n3;
  long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long count = phase == 1 ? ninterior : (long long)*qcount;
  // the network's operands in shared memory (phase 1 of the network start only)
  extern __shared__ __align__(128) unsigned char c2p_smem[];
  c2pnet::TcNet& tnet = *reinterpret_cast<c2pnet::TcNet*>(c2p_smem);
  const bool with_net = START == C2P_START_NETWORK && phase == 1;
  if (with_net) c2pnet::tc_setup(net, tnet);
  // phase 1 runs one pass over the cells (with the CTA-wide dt reduction at the end);
  // phase 2 strides over the queue
  for (; phase == 2 ? e < count : true; e += stride) {
    double cell_dt = 1.0e300;
    bool enqueue = false, finished = false, fell_back = false, failed = false;
    int passes = 0;
    long long t = -1;
    if (e < count) t = phase == 1 ? e : (long long)queue[e];
    int b = 0, i = 0, j = 0, k = 0;
    double bc1 = 0.0, bc2 = 0.0, bc3 = 0.0;
    double cons[NHYDRO] = {1.0, 0.0, 0.0, 0.0, 2.0}, prim[NHYDRO];
    i64 c = 0, cb = 0;
    const i64 vs = m.ncell;
    if (t >= 0) {
      b = (int)(t / ((long long)n1 * n2 * n3));
      int r = (int)(t - (long long)b * n1 * n2 * n3);
      i = m.is + r % n1;
      r /= n1;
      j = m.js + r % n2;
      k = m.ks + r / n2;
      const double lw = 0.5, rw = 0.5;
      bc1 = lw * b1[f1idx(m, b, k, j, i)] + rw * b1[f1idx(m, b, k, j, i + 1)];
      bc2 = lw * b2[f2idx(m, b, k, j, i)] + rw * b2[f2idx(m, b, k, j + 1, i)];
      bc3 = lw * b3[f3idx(m, b, k, j, i)] + rw * b3[f3idx(m, b, k + 1, j, i)];
      c = cidx(m, b, 0, NHYDRO, k, j, i);
      cb = cidx(m, b, 0, 3, k, j, i);
#pragma unroll
      for (int n = 0; n < NHYDRO; ++n) {
        cons[n] = (double)u[c + n * vs] + ((KAHAN && ulo) ? (double)ulo[c + n * vs] : 0.0);
        prim[n] = (double)wout[c + n * vs];
      }
    }
    double pstart = 0.0;
    if (START != C2P_START_STALE) {
      const double mm_sq = cons[IVX] * cons[IVX] + cons[IVY] * cons[IVY] +
                           cons[IVZ] * cons[IVZ];
      const double bb_sq = bc1 * bc1 + bc2 * bc2 + bc3 * bc3;
      const double tt = cons[IVX] * bc1 + cons[IVY] * bc2 + cons[IVZ] * bc3;
      if (phase == 2) {
        pstart = qstart[e];  // the start phase 1 used
      } else if (START == C2P_START_REFINED) {
        if (t >= 0) {
          int it32;
          pstart = sr_refine_f32(fp.gamma_adi, cons[IDN], cons[IPR], mm_sq, bb_sq, tt,
                                 smax(prim[IPR], fp.pfloor), 12, 1.0e-6f, &it32);
        }
      } else {
        // every thread of the CTA takes part in the tensor-core evaluation (a thread
        // without a cell evaluates the network on a dummy state)
        float f[c2pnet::NIN], xin[c2pnet::NIN], y[c2pnet::NOUT];
        const double uu[5] = {cons[IDN], cons[IVX], cons[IVY], cons[IVZ], cons[IPR]};
        const double bb[3] = {bc1, bc2, bc3};
        c2pnet::features(uu, bb, f);
#pragma unroll
        for (int q = 0; q < c2pnet::NIN; ++q) xin[q] = (f[q] - tnet.xm[q]) / tnet.xs[q];
        uint32_t ph = 0;
        c2pnet::tc_infer_tile(tnet, xin, y, ph, net_err);
        c2pnet::tc_teardown(tnet);
        if (t >= 0) {
          int it32;
          double guess = cons[IPR] * (double)__expf(y[0]);
          if (!(guess > fp.pfloor)) guess = smax(prim[IPR], fp.pfloor);  // NaN: no result
          pstart = sr_refine_f32(fp.gamma_adi, cons[IDN], cons[IPR], mm_sq, bb_sq, tt, guess,
                                 12, 1.0e-6f, &it32);
        }
      }
      if (!(pstart > fp.pfloor)) pstart = smax(prim[IPR], fp.pfloor);
    }
    if (t >= 0) {
      bool fixed = false, deferred = false;
      int it = 0;
      const bool ok = sr_c2p_cell(fp, cons, bc1, bc2, bc3, prim, &fixed, &it, pstart,
                                  phase == 1 ? max_first : 15, &deferred, &passes,
                                  &fell_back);
      if (deferred) {
        enqueue = true;
      } else {
        finished = true;
        failed = !ok;
#pragma unroll
        for (int n = 0; n < NHYDRO; ++n) wout[c + n * vs] = (Real)prim[n];
        bcc[cb] = (Real)bc1;
        bcc[cb + vs] = (Real)bc2;
        bcc[cb + 2 * vs] = (Real)bc3;
        store_cce<Real, true>(cc, cb, vs, (Real)prim[IVX], (Real)prim[IVY], (Real)prim[IVZ],
                              (Real)bc1, (Real)bc2, (Real)bc3);
        if (fixed) {
#pragma unroll
          for (int n = 0; n < NHYDRO; ++n) {
            const Real hi = (Real)cons[n];
            u[c + n * vs] = hi;
            if (KAHAN && ulo) ulo[c + n * vs] = (Real)(cons[n] - (double)hi);
          }
        }
        if (do_dt && (fixed || !ok)) atomicAdd(&clk->c2p_floor_count, 1);
      }
      if (phase == 1 && do_dt) {
        const double dt1 = m.dx1f[(i64)b * m.nc1 + i], dt2 = m.dx2f[(i64)b * m.nc2 + j],
                     dt3 = m.dx3f[(i64)b * m.nc3 + k];
        cell_dt = smin<double>(smin<double>(dt1, dt2), dt3);
      }
    }
    if (phase == 2) {  // statistics of the queued cells: per thread (few cells)
      if (finished) {
        atomicAdd(&clk->sr_cells, 1ull);
        atomicAdd(&clk->sr_passes, (unsigned long long)passes);
        if (fell_back) atomicAdd(&clk->sr_fallbacks, 1ull);
        if (failed) atomicAdd(&clk->sr_unconverged, 1ull);
      }
      continue;
    }
    // phase 1 (every lane runs this body once): statistics of the cells finished here,
    // one atomic per counter and warp
    {
      const unsigned nfin = __popc(__ballot_sync(0xffffffffu, finished));
      const unsigned psum = __reduce_add_sync(0xffffffffu, finished ? (unsigned)passes : 0u);
      const unsigned nfb = __popc(__ballot_sync(0xffffffffu, finished && fell_back));
      const unsigned nfail = __popc(__ballot_sync(0xffffffffu, failed));
      if ((threadIdx.x & 31) == 0 && nfin) {
        atomicAdd(&clk->sr_cells, (unsigned long long)nfin);
        atomicAdd(&clk->sr_passes, (unsigned long long)psum);
        if (nfb) atomicAdd(&clk->sr_fallbacks, (unsigned long long)nfb);
        if (nfail) atomicAdd(&clk->sr_unconverged, (unsigned long long)nfail);
      }
    }
    // phase 1: warp-aggregated append of the deferred cells, then the dt reduction
    const unsigned mask = __ballot_sync(0xffffffffu, enqueue);
    if (mask) {
      const int lane = threadIdx.x & 31, leader = __ffs(mask) - 1;
      unsigned base = 0;
      if (lane == leader) base = atomicAdd(qcount, (unsigned)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (enqueue) {
        const unsigned slot = base + __popc(mask & ((1u << lane) - 1u));
        queue[slot] = (int)t;
        if (START != C2P_START_STALE) qstart[slot] = pstart;
      }
    }
    if (do_dt) cta_min_to_clock<double>(cell_dt, clk);
    break;
  }
}

// Ghost cells of the primitives, the cell-centred field and the cell-centred E, copied
// from the blocks that own them (the relativistic W(U) solves interior cells only).
template <typename Real>
__global__ void __launch_bounds__(256)
copy_ghost_prims_kernel(DevMesh m, Real* __restrict__ w, Real* __restrict__ bcc,
                        Real* __restrict__ cc) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int gc = (int)(m.ncell - (i64)m.nx1 * m.nx2 * m.nx3);
  if (t >= (long long)gc * m.nb) return;
  const int b = (int)(t / gc);
  int k, j, i;
  ghost_coord((int)(t - (long long)b * gc), m.nc1, m.nc2, m.nc3, m.nx1, m.nx2, m.nx3, m.ng,
              k, j, i);
  bool ghost;
  const i64 s5 = src_cell(m, b, k, j, i, NHYDRO, &ghost);
  const i64 s3 = src_cell(m, b, k, j, i, 3, &ghost);
  if (s5 < 0) return;  // filled by the boundary functions
  const i64 d5 = cidx(m, b, 0, NHYDRO, k, j, i), d3 = cidx(m, b, 0, 3, k, j, i);
  const i64 vs = m.ncell;
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) w[d5 + n * vs] = w[s5 + n * vs];
#pragma unroll
  for (int n = 0; n < 3; ++n) {
    bcc[d3 + n * vs] = bcc[s3 + n * vs];
    cc[d3 + n * vs] = cc[s3 + n * vs];
  }
}

// Mesh::NewTimeStep (mesh.cpp:1236-1281) after the main loop's time += dt
// (main.cpp:535): dt = min(2 dt_old, cfl * min cell dt), clipped to tlim.
// mode 0: Mesh::NewTimeStep from the blocks' minimum (mesh.cpp:1236-1281); mode 1: time +=
// dt first (the end of a main-loop cycle, main.cpp:535-541); mode 2: NewTimeStep again
// from the minimum the previous call used (the main loop's call after a regrid, whose
// Initialize(2) made the first one)
static __global__ void advance_clock_kernel(DevClock* clk, double cfl, double tlim, int mode) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (mode == 1) {
    clk->dt_prev = clk->dt;
    clk->time = clk->time + clk->dt;
  }
  const unsigned long long bits = mode == 2 ? clk->dtmin_prev_bits : clk->dtmin_bits;
  double block_dt = __longlong_as_double((long long)bits) * cfl;
  double dt = 2.0 * clk->dt;
  dt = smin<double>(dt, block_dt);
  if (clk->time < tlim && (tlim - clk->time) < dt) dt = tlim - clk->time;
  clk->dt = dt;
  clk->dtf = (float)dt;
  if (mode != 2) {
    clk->dtmin_prev_bits = clk->dtmin_bits;
    clk->dtmin_bits = 0x7fefffffffffffffULL;  // DBL_MAX for the next reduction
  }
}

}  // namespace athgpu
