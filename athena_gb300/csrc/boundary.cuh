// Physical mesh boundaries: BoundaryValues::ApplyPhysicalBoundaries (bvals/bvals.cpp:
// 453-680) for outflow and reflecting faces, on the primitives (bvals/cc/outflow_cc.cpp,
// bvals/cc/hydro/reflect_hydro.cpp), the face field (bvals/fc/outflow_fc.cpp,
// bvals/fc/reflect_fc.cpp), then the cell-centred field and (Newtonian) the conserved
// state of the filled ghost cells (bvals.cpp:508-515), axis by axis (x1, x2, x3), after
// W(U).  A refined parent's halo reads that conserved state (a regrid); the relativistic
// path reads no ghost U and does not form it.
//
// Per axis a two launches: bc_fill_kernel (primitives and face field of both sides), then
// bc_cc_kernel (cell-centred field and cell-centred E of the filled ghost cells, from the
// faces just written).  A thread owns one (side, ghost layer g, transverse position) of a
// block on the mesh face; the two sides of an axis write disjoint ghost layers and read
// only the block's own cells along the axis, so one launch holds both.
#pragma once
#include "kernels.cuh"

namespace athgpu {

// does block b have a neighbour (a block or a periodic image) across block face f
// (0 inner x1, 1 outer x1, ..., 5 outer x3)?
__device__ __forceinline__ bool has_nbr(const DevMesh& m, int b, int f) {
  const int a = f >> 1, o = (f & 1) ? 1 : -1;
  return nbr_of(m, b, a == 0 ? o : 0, a == 1 ? o : 0, a == 2 ? o : 0) >= 0;
}

// Transverse index ranges [rl, rh] of the boundary function along axis a
// (bvals.cpp:457-470, 596): x1 extends j and k into the ghosts only where those block
// faces have neighbours, x2 takes the full i range and extends k only where the x3 faces
// have neighbours, x3 takes the full i and j ranges.
__device__ __forceinline__ void bc_ranges(const DevMesh& m, int b, int a, int rl[3],
                                          int rh[3]) {
  rl[0] = m.is; rh[0] = m.ie;
  rl[1] = m.js; rh[1] = m.je;
  rl[2] = m.ks; rh[2] = m.ke;
  const int ng = m.ng;
  if (a == 0) {
    if (has_nbr(m, b, 2)) rl[1] -= ng;
    if (has_nbr(m, b, 3)) rh[1] += ng;
    if (has_nbr(m, b, 4)) rl[2] -= ng;
    if (has_nbr(m, b, 5)) rh[2] += ng;
  } else if (a == 1) {
    rl[0] -= ng; rh[0] += ng;
    if (has_nbr(m, b, 4)) rl[2] -= ng;
    if (has_nbr(m, b, 5)) rh[2] += ng;
  } else {
    rl[0] -= ng; rh[0] += ng;
    rl[1] -= ng; rh[1] += ng;
  }
}

// Thread t of an axis-a launch -> (block, side, ghost layer g in 1..ng, transverse position
// p0 along axis t0, p1 along axis t1), with t0 < t1 the two axes other than a.  Blocks are
// those on the mesh face of the side; positions run over the whole ghost-inclusive extent
// plus one (face components along a transverse axis have one more).  Returns false past
// the end.
struct BcThread {
  int b, side, g, t0, t1, p0, p1;
};
__device__ __forceinline__ int ncells(const DevMesh& m, int a) {
  return a == 0 ? m.nc1 : a == 1 ? m.nc2 : m.nc3;
}
__device__ __forceinline__ bool bc_thread(const DevMesh& m, int a, long long t, BcThread& q) {
  q.t0 = a == 0 ? 1 : 0;
  q.t1 = a == 2 ? 1 : 2;
  const int e0 = ncells(m, q.t0) + 1, e1 = ncells(m, q.t1) + 1;
  const int nbx[3] = {m.nbx1, m.nbx2, m.nbx3};
  // blocks on one mesh face (multi-level mesh: every block; those without a physical face
  // on this side return)
  const int nbt = m.ml.on ? m.nb : nbx[q.t0] * nbx[q.t1];
  const long long per_block = (long long)m.ng * e0 * e1;
  if (t >= 2LL * nbt * per_block) return false;
  long long r = t % per_block;
  const long long bs = t / per_block;  // side * nbt + block on the face
  q.side = (int)(bs / nbt);
  const int bt = (int)(bs % nbt);
  q.p0 = (int)(r % e0);
  r /= e0;
  q.p1 = (int)(r % e1);
  q.g = 1 + (int)(r / e1);
  if (m.ml.on) {
    q.b = bt;
    return true;
  }
  int l[3];
  l[a] = q.side ? nbx[a] - 1 : 0;
  l[q.t0] = bt % nbx[q.t0];
  l[q.t1] = bt / nbx[q.t0];
  q.b = (l[2] * m.nbx2 + l[1]) * m.nbx1 + l[0];
  return true;
}

__device__ __forceinline__ i64 face_index(const DevMesh& m, int d, int b, const int c[3]) {
  return d == 0 ? f1idx(m, b, c[2], c[1], c[0])
       : d == 1 ? f2idx(m, b, c[2], c[1], c[0]) : f3idx(m, b, c[2], c[1], c[0]);
}

// Outflow copies the last own cell (face) into every ghost layer; reflecting mirrors the
// own cells (faces) about the boundary and flips the normal velocity (face field).
template <typename Real>
__global__ void __launch_bounds__(256)
bc_fill_kernel(DevMesh m, int a, Real* __restrict__ w, double* __restrict__ b1,
               double* __restrict__ b2, double* __restrict__ b3) {
  BcThread q;
  if (!bc_thread(m, a, (long long)blockIdx.x * blockDim.x + threadIdx.x, q)) return;
  const int f = 2 * a + q.side;
  if (has_nbr(m, q.b, f)) return;
  const int kind = m.bc[f];  // ATHGPU_BC_OUTFLOW or ATHGPU_BC_REFLECT
  int rl[3], rh[3];
  bc_ranges(m, q.b, a, rl, rh);
  const int lo = a == 0 ? m.is : a == 1 ? m.js : m.ks;
  const int hi = a == 0 ? m.ie : a == 1 ? m.je : m.ke;
  const int g = q.g;
  const bool refl = kind == 2;
  // cells (and face components along a transverse axis) of layer g
  const int cdst = q.side ? hi + g : lo - g;
  const int csrc = !refl ? (q.side ? hi : lo) : (q.side ? hi - g + 1 : lo + g - 1);
  int dc[3], sc[3];
  dc[a] = cdst;
  sc[a] = csrc;
  dc[q.t0] = sc[q.t0] = q.p0;
  dc[q.t1] = sc[q.t1] = q.p1;
  const bool in0 = q.p0 >= rl[q.t0] && q.p0 <= rh[q.t0];
  const bool in1 = q.p1 >= rl[q.t1] && q.p1 <= rh[q.t1];
  const bool in0f = q.p0 >= rl[q.t0] && q.p0 <= rh[q.t0] + 1;  // faces along t0
  const bool in1f = q.p1 >= rl[q.t1] && q.p1 <= rh[q.t1] + 1;  // faces along t1
  if (in0 && in1) {
    const i64 vs = m.ncell;
    const i64 dcell = cidx(m, q.b, 0, NHYDRO, dc[2], dc[1], dc[0]);
    const i64 scell = cidx(m, q.b, 0, NHYDRO, sc[2], sc[1], sc[0]);
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) {
      const Real v = w[scell + n * vs];
      w[dcell + n * vs] = (refl && n == IVX + a) ? -v : v;
    }
    // the normal face component, layer g: faces lo-g (inner) or hi+1+g (outer)
    int df[3] = {dc[0], dc[1], dc[2]}, sf[3] = {sc[0], sc[1], sc[2]};
    df[a] = q.side ? hi + 1 + g : lo - g;
    sf[a] = !refl ? (q.side ? hi + 1 : lo) : (q.side ? hi + 1 - g : lo + g);
    double* F = a == 0 ? b1 : a == 1 ? b2 : b3;
    const double v = F[face_index(m, a, q.b, sf)];
    F[face_index(m, a, q.b, df)] = refl ? -v : v;
  }
  // transverse face components: one more face along their own direction
  if (in0f && in1) {
    double* F = q.t0 == 0 ? b1 : b2;
    F[face_index(m, q.t0, q.b, dc)] = F[face_index(m, q.t0, q.b, sc)];
  }
  if (in0 && in1f) {
    double* F = q.t1 == 1 ? b2 : b3;
    F[face_index(m, q.t1, q.b, dc)] = F[face_index(m, q.t1, q.b, sc)];
  }
}

// Cell-centred field (field.cpp:112-180, the arithmetic of the path's W(U)) and cell-centred
// E of the ghost cells bc_fill_kernel filled along axis a.
template <typename Real, bool SR>
__global__ void __launch_bounds__(256)
bc_cc_kernel(DevMesh m, int a, const Real* __restrict__ w, const double* __restrict__ b1,
             const double* __restrict__ b2, const double* __restrict__ b3,
             Real* __restrict__ bcc, Real* __restrict__ cc, Real* __restrict__ u) {
  BcThread q;
  if (!bc_thread(m, a, (long long)blockIdx.x * blockDim.x + threadIdx.x, q)) return;
  if (has_nbr(m, q.b, 2 * a + q.side)) return;
  int rl[3], rh[3];
  bc_ranges(m, q.b, a, rl, rh);
  if (q.p0 < rl[q.t0] || q.p0 > rh[q.t0] || q.p1 < rl[q.t1] || q.p1 > rh[q.t1]) return;
  const int lo = a == 0 ? m.is : a == 1 ? m.js : m.ks;
  const int hi = a == 0 ? m.ie : a == 1 ? m.je : m.ke;
  int c[3];
  c[a] = q.side ? hi + q.g : lo - q.g;
  c[q.t0] = q.p0;
  c[q.t1] = q.p1;
  const int i = c[0], j = c[1], k = c[2];
  const double b1l = b1[f1idx(m, q.b, k, j, i)], b1r = b1[f1idx(m, q.b, k, j, i + 1)];
  const double b2l = b2[f2idx(m, q.b, k, j, i)], b2r = b2[f2idx(m, q.b, k, j + 1, i)];
  const double b3l = b3[f3idx(m, q.b, k, j, i)], b3r = b3[f3idx(m, q.b, k + 1, j, i)];
  Real c1, c2, c3;
  if (SR || sizeof(Real) == 8) {  // FP64 average (rounded once for the FP32 SR path)
    const double lw = 0.5, rw = 0.5;
    c1 = (Real)(lw * b1l + rw * b1r);
    c2 = (Real)(lw * b2l + rw * b2r);
    c3 = (Real)(lw * b3l + rw * b3r);
  } else {  // FP32 Newtonian path: average of the FP32-rounded faces
    c1 = Real(0.5) * to_real(b1l, Real()) + Real(0.5) * to_real(b1r, Real());
    c2 = Real(0.5) * to_real(b2l, Real()) + Real(0.5) * to_real(b2r, Real());
    c3 = Real(0.5) * to_real(b3l, Real()) + Real(0.5) * to_real(b3r, Real());
  }
  const i64 vs = m.ncell;
  const i64 cw = cidx(m, q.b, 0, NHYDRO, k, j, i);
  const i64 cb = cidx(m, q.b, 0, 3, k, j, i);
  bcc[cb] = c1;
  bcc[cb + vs] = c2;
  bcc[cb + 2 * vs] = c3;
  store_cce<Real, SR>(cc, cb, vs, w[cw + IVX * vs], w[cw + IVY * vs], w[cw + IVZ * vs], c1,
                      c2, c3);
  if (!SR) {  // PrimitiveToConserved (adiabatic_mhd.cpp:99-133), bulk precision
    const Real igm1 = Real(1) / (Real)(m.gamma - 1.0);
    const Real w_d = w[cw], w_vx = w[cw + IVX * vs], w_vy = w[cw + IVY * vs],
               w_vz = w[cw + IVZ * vs], w_p = w[cw + IPR * vs];
    u[cw] = w_d;
    u[cw + vs] = w_vx * w_d;
    u[cw + 2 * vs] = w_vy * w_d;
    u[cw + 3 * vs] = w_vz * w_d;
    u[cw + 4 * vs] = w_p * igm1 + Real(0.5) * (w_d * (w_vx * w_vx + w_vy * w_vy + w_vz * w_vz) +
                                               (c1 * c1 + c2 * c2 + c3 * c3));
  }
}

// threads of one axis-a launch
inline long long bc_threads(const DevMesh& m, int a) {
  const int t0 = a == 0 ? 1 : 0, t1 = a == 2 ? 1 : 2;
  const int nc[3] = {m.nc1, m.nc2, m.nc3};
  const int nbx[3] = {m.nbx1, m.nbx2, m.nbx3};
  const long long nbt = m.ml.on ? (long long)m.nb : (long long)nbx[t0] * nbx[t1];
  return 2LL * nbt * m.ng * (nc[t0] + 1) * (nc[t1] + 1);
}

}  // namespace athgpu
