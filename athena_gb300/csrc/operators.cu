// Per-operator entry points: the reference's per-MeshBlock member functions of the stage
// update, one call each, on one MeshBlock's arrays in the reference's own AthenaArray
// layout.  A caller that keeps the reference's TimeIntegratorTaskList and replaces only the
// bodies of Hydro::CalculateFluxes, Hydro::AddFluxDivergence, Hydro::NewBlockTimeStep,
// Field::ComputeCornerE, Field::CT and EquationOfState::ConservedToPrimitive calls these
// (the shim in athena_gb300/shim/).  The context is an ordinary athgpu context of ONE
// MeshBlock (nbx1 = nbx2 = nbx3 = 1, the block's own coordinates, FP64); its registers
// hold the operands on the device.  Arrays may be host or device memory (they are copied
// with cudaMemcpyDefault); every call is synchronous.  Outputs are written over the
// reference's index ranges only: each output array is copied in before and out after the
// computation, so its other elements come back unchanged.
//
// The kernels are the per-face / per-cell restatements the batched stage fuses: the same
// reconstruction and Riemann solvers (recon_cell, solve_face), the same corner-EMF
// kernel, and the reference's operand order in the flux divergence, CT, W(U) and the time
// step, so every result is the reference's bit for bit (FP64, compiled without FMA
// contraction).
#include <cuda_runtime.h>
#include <float.h>
#include <string.h>

#include <string>

#include "../../include/athena_gb300.h"
#include "ctx.h"

namespace athgpu {
void set_last_error(const std::string& msg);  // api.cu
}

namespace {
using namespace athgpu;

athgpu_status op_fail(athgpu_status s, const std::string& msg) {
  set_last_error(msg);
  return s;
}
#define OCK(call)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return op_fail(ATHGPU_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

inline unsigned grid_of(long long n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

// ---------------------------------------------------------------------------------------
// Hydro::CalculateFluxes (calculate_fluxes.cpp:38-415), 3-D MHD: the faces of direction
// DIR over the reference's ranges (x1: k in [ks-1,ke+1], j in [js-1,je+1], i in
// [is,ie+1]; x2: k in [ks-1,ke+1], j in [js,je+1], i in [is-1,ie+1]; x3: k in [ks,ke+1],
// j in [js-1,je+1], i in [is-1,ie+1]), one thread per face: the left state is the upper
// face value of the cell below, the right state the lower face value of the cell above
// (wl(i+1) and wr(i) of the reconstruction), then the Riemann solver, which writes the
// two face EMFs and the CT weight (dxw = the width of the cell above the face,
// CenterWidth?, cartesian.cpp) and the five fluxes flx[n][face].
template <int DIR, int ORDER, int RS>
__global__ void __launch_bounds__(128)
op_flux_kernel(DevMesh m, double dt, const double* __restrict__ w,
               const double* __restrict__ bcc, const double* __restrict__ bn,
               double* __restrict__ flx, double* __restrict__ ey, double* __restrict__ ez,
               double* __restrict__ wct) {
  const int ni = DIR == 0 ? m.nx1 + 1 : m.nx1 + 2;
  const int nj = DIR == 1 ? m.nx2 + 1 : m.nx2 + 2;
  const int nk = DIR == 2 ? m.nx3 + 1 : m.nx3 + 2;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj * nk) return;
  const int i = (DIR == 0 ? m.is : m.is - 1) + (int)(t % ni);
  const int j = (DIR == 1 ? m.js : m.js - 1) + (int)((t / ni) % nj);
  const int k = (DIR == 2 ? m.ks : m.ks - 1) + (int)(t / ((long long)ni * nj));
  double qlp[NWAVE], qrm[NWAVE], wl[NWAVE], wr[NWAVE];
  // cell below the face along DIR: its upper-face value is the left state
  recon_cell<double, DIR, ORDER>(m, w, bcc, 0, k - (DIR == 2), j - (DIR == 1),
                                 i - (DIR == 0), qlp, qrm);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) wl[n] = qlp[n];
  recon_cell<double, DIR, ORDER>(m, w, bcc, 0, k, j, i, qlp, qrm);
#pragma unroll
  for (int n = 0; n < NWAVE; ++n) wr[n] = qrm[n];
  const i64 fo = fidx<DIR>(m, 0, k, j, i);
  const int c = DIR == 0 ? i : DIR == 1 ? j : k;
  const double dxw = (DIR == 0 ? m.dx1f : DIR == 1 ? m.dx2f : m.dx3f)[c];
  double fn[NHYDRO];
  double dvn = 0.0, dvt = 0.0;
  if (RS == 7) {  // LHLLD: the face's velocity differences (vel_cell)
    double vnl, t1l, t2l, vnr, t1r, t2r;
    vel_cell<double, DIR>(m, w, 0, k - (DIR == 2), j - (DIR == 1), i - (DIR == 0), vnl, t1l,
                          t2l);
    vel_cell<double, DIR>(m, w, 0, k, j, i, vnr, t1r, t2r);
    dvn = vnr - vnl;
    dvt = smin(smin(t1l, t1r), smin(t2l, t2r));
  }
  solve_face<double, DIR, RS>(m, wl, wr, bn[fo], dxw, dt, fo, fn, ey, ez, wct, dvn, dvt);
  const i64 nf = DIR == 0 ? m.nf1 : DIR == 1 ? m.nf2 : m.nf3;
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) flx[n * nf + fo] = fn[n];
}

// cell-centred E over every cell (calculate_corner_e.cpp:131-185; SR: from the
// 4-velocity, :161-172), the corner-EMF kernel's input
template <bool SR>
__global__ void __launch_bounds__(256)
op_cce_kernel(DevMesh m, const double* __restrict__ w, const double* __restrict__ bcc,
              double* __restrict__ cc) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= m.ncell) return;
  const i64 vs = m.ncell;
  store_cce<double, SR>(cc, t, vs, w[t + IVX * vs], w[t + IVY * vs], w[t + IVZ * vs], bcc[t],
                        bcc[t + vs], bcc[t + 2 * vs]);
}

// Hydro::AddFluxDivergence (add_flux_divergence.cpp:39-96): u(n) -= wght * dflx(n) / vol
// over the interior with dflx formed x1, x2, x3 in the reference's order
__global__ void __launch_bounds__(256)
op_divergence_kernel(DevMesh m, double wght, const double* __restrict__ f1,
                     const double* __restrict__ f2, const double* __restrict__ f3,
                     double* __restrict__ u) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)m.nx1 * m.nx2 * m.nx3) return;
  const int i = m.is + (int)(t % m.nx1);
  const int j = m.js + (int)((t / m.nx1) % m.nx2);
  const int k = m.ks + (int)(t / ((long long)m.nx1 * m.nx2));
  const double dx1 = m.dx1f[i], dx2 = m.dx2f[j], dx3 = m.dx3f[k];
  // Face1Area (both faces of the cell), Face2Area at j and j+1, Face3Area at k and k+1,
  // CellVolume (coordinates.cpp:448-548)
  const double a1 = dx2 * dx3, a2 = dx1 * dx3, a2p = dx1 * dx3, a3 = dx1 * dx2,
               a3p = dx1 * dx2;
  const double vol = dx1 * dx2 * dx3;
  for (int n = 0; n < NHYDRO; ++n) {
    double d = (a1 * f1[n * m.nf1 + f1idx(m, 0, k, j, i + 1)] -
                a1 * f1[n * m.nf1 + f1idx(m, 0, k, j, i)]);
    d += (a2p * f2[n * m.nf2 + f2idx(m, 0, k, j + 1, i)] -
          a2 * f2[n * m.nf2 + f2idx(m, 0, k, j, i)]);
    d += (a3p * f3[n * m.nf3 + f3idx(m, 0, k + 1, j, i)] -
          a3 * f3[n * m.nf3 + f3idx(m, 0, k, j, i)]);
    const i64 c = cidx(m, 0, n, NHYDRO, k, j, i);
    u[c] -= wght * d / vol;
  }
}

// Field::CT (ct.cpp:31-116), 3-D: each face of [is,ie+1]x[js,je]x[ks,ke] (x1),
// [is,ie]x[js,je+1]x[ks,ke] (x2), [is,ie]x[js,je]x[ks,ke+1] (x3), the two curl terms in
// the reference's order
template <int DIR>
__global__ void __launch_bounds__(256)
op_ct_kernel(DevMesh m, double wght, const double* __restrict__ e1,
             const double* __restrict__ e2, const double* __restrict__ e3,
             double* __restrict__ bf) {
  const int ni = m.nx1 + (DIR == 0), nj = m.nx2 + (DIR == 1), nk = m.nx3 + (DIR == 2);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj * nk) return;
  const int i = m.is + (int)(t % ni);
  const int j = m.js + (int)((t / ni) % nj);
  const int k = m.ks + (int)(t / ((long long)ni * nj));
  const double dx1 = m.dx1f[i], dx2 = m.dx2f[j], dx3 = m.dx3f[k];
  if (DIR == 0) {
    // Face1Area = dx2 dx3; Edge3Length (k,j) and (k,j+1) = dx3f(k); Edge2Length = dx2f(j)
    const double area = dx2 * dx3, l3 = dx3, l3p = dx3, l2 = dx2, l2p = dx2;
    double& b = bf[f1idx(m, 0, k, j, i)];
    b -= (wght / area) * (l3p * e3[e3idx(m, 0, k, j + 1, i)] - l3 * e3[e3idx(m, 0, k, j, i)]);
    b += (wght / area) * (l2p * e2[e2idx(m, 0, k + 1, j, i)] - l2 * e2[e2idx(m, 0, k, j, i)]);
  } else if (DIR == 1) {
    // Face2Area = dx1 dx3; Edge3Length(i), (i+1) = dx3f(k); Edge1Length = dx1f(i)
    const double area = dx1 * dx3, l3 = dx3, l3p = dx3, l1 = dx1, l1p = dx1;
    double& b = bf[f2idx(m, 0, k, j, i)];
    b += (wght / area) * (l3p * e3[e3idx(m, 0, k, j, i + 1)] - l3 * e3[e3idx(m, 0, k, j, i)]);
    b -= (wght / area) * (l1p * e1[e1idx(m, 0, k + 1, j, i)] - l1 * e1[e1idx(m, 0, k, j, i)]);
  } else {
    // Face3Area = dx1 dx2; Edge2Length(i), (i+1) = dx2f(j); Edge1Length = dx1f(i)
    const double area = dx1 * dx2, l2 = dx2, l2p = dx2, l1 = dx1, l1p = dx1;
    double& b = bf[f3idx(m, 0, k, j, i)];
    b -= (wght / area) * (l2p * e2[e2idx(m, 0, k, j, i + 1)] - l2 * e2[e2idx(m, 0, k, j, i)]);
    b += (wght / area) * (l1p * e1[e1idx(m, 0, k, j + 1, i)] - l1 * e1[e1idx(m, 0, k, j, i)]);
  }
}

// EquationOfState::ConservedToPrimitive over [il,iu]x[jl,ju]x[kl,ku]: first
// Field::CalculateCellCenteredField there (field.cpp:112-180, uniform: 1/2, 1/2), then
// per cell the Newtonian W(U) with floors and the rewrite of cons (adiabatic_mhd.cpp:
// 41-90) or the relativistic solve seeded from prim's previous contents
// (adiabatic_mhd_sr.cpp:72-272)
template <bool SR>
__global__ void __launch_bounds__(128)
op_c2p_kernel(DevMesh m, SRFloors fp, int il, int iu, int jl, int ju, int kl, int ku,
              const double* __restrict__ b1, const double* __restrict__ b2,
              const double* __restrict__ b3, double* __restrict__ cons,
              double* __restrict__ prim, double* __restrict__ bcc,
              unsigned long long* __restrict__ nfloor) {
  const int ni = iu - il + 1, nj = ju - jl + 1, nk = ku - kl + 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ni * nj * nk) return;
  const int i = il + (int)(t % ni);
  const int j = jl + (int)((t / ni) % nj);
  const int k = kl + (int)(t / ((long long)ni * nj));
  const double lw = 0.5, rw = 0.5;
  const double bc1 = lw * b1[f1idx(m, 0, k, j, i)] + rw * b1[f1idx(m, 0, k, j, i + 1)];
  const double bc2 = lw * b2[f2idx(m, 0, k, j, i)] + rw * b2[f2idx(m, 0, k, j + 1, i)];
  const double bc3 = lw * b3[f3idx(m, 0, k, j, i)] + rw * b3[f3idx(m, 0, k + 1, j, i)];
  const i64 vs = m.ncell;
  const i64 c = cidx(m, 0, 0, NHYDRO, k, j, i);
  const i64 cb = cidx(m, 0, 0, 3, k, j, i);
  bcc[cb] = bc1;
  bcc[cb + vs] = bc2;
  bcc[cb + 2 * vs] = bc3;
  if (SR) {
    double cu[NHYDRO], pr[NHYDRO];
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) {
      cu[n] = cons[c + n * vs];
      pr[n] = prim[c + n * vs];
    }
    bool fixed = false;
    int it = 0;
    const bool ok = sr_c2p_cell(fp, cu, bc1, bc2, bc3, pr, &fixed, &it);
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) {
      prim[c + n * vs] = pr[n];
      if (fixed) cons[c + n * vs] = cu[n];
    }
    if (fixed || !ok) atomicAdd(nfloor, 1ull);
    return;
  }
  const double gm1 = m.gamma - 1.0;
  double u_d = cons[c], u_m1 = cons[c + vs], u_m2 = cons[c + 2 * vs],
         u_m3 = cons[c + 3 * vs], u_e = cons[c + 4 * vs];
  const bool dfloored = !(u_d > m.dfloor);
  u_d = (u_d > m.dfloor) ? u_d : m.dfloor;
  const double di = 1.0 / u_d;
  const double pb = 0.5 * (bc1 * bc1 + bc2 * bc2 + bc3 * bc3);
  const double e_k = 0.5 * di * (u_m1 * u_m1 + u_m2 * u_m2 + u_m3 * u_m3);
  double w_p = gm1 * (u_e - e_k - pb);
  const bool pfloored = !(w_p > m.pfloor);
  u_e = (w_p > m.pfloor) ? u_e : ((m.pfloor / gm1) + e_k + pb);
  w_p = (w_p > m.pfloor) ? w_p : m.pfloor;
  if (dfloored) cons[c] = u_d;
  if (pfloored) cons[c + 4 * vs] = u_e;
  prim[c] = u_d;
  prim[c + vs] = u_m1 * di;
  prim[c + 2 * vs] = u_m2 * di;
  prim[c + 3 * vs] = u_m3 * di;
  prim[c + 4 * vs] = w_p;
  if (dfloored || pfloored) atomicAdd(nfloor, 1ull);
}

// Hydro::NewBlockTimeStep (new_blockdt.cpp:45-230), ideal MHD: the minimum over interior
// cells of dx_d / (|v_d| + c_f) with bx = bcc + |b_face - bcc| (:80-103); relativistic:
// the widths (signal speed 1, :74).  The minimum of doubles is exact in any order; one
// atomicMin on the ordered bits of the non-negative double per CTA.
template <bool SR>
__global__ void __launch_bounds__(256)
op_dt_kernel(DevMesh m, const double* __restrict__ w, const double* __restrict__ bcc,
             const double* __restrict__ b1, const double* __restrict__ b2,
             const double* __restrict__ b3, unsigned long long* __restrict__ dtmin_bits) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double cell_dt = DBL_MAX;
  if (t < (long long)m.nx1 * m.nx2 * m.nx3) {
    const int i = m.is + (int)(t % m.nx1);
    const int j = m.js + (int)((t / m.nx1) % m.nx2);
    const int k = m.ks + (int)(t / ((long long)m.nx1 * m.nx2));
    double dt1 = m.dx1f[i], dt2 = m.dx2f[j], dt3 = m.dx3f[k];
    if (!SR) {
      const i64 vs = m.ncell;
      const i64 c = cidx(m, 0, 0, NHYDRO, k, j, i), cb = cidx(m, 0, 0, 3, k, j, i);
      const double d = w[c], vx = w[c + vs], vy = w[c + 2 * vs], vz = w[c + 3 * vs],
                   p = w[c + 4 * vs];
      const double bc1 = bcc[cb], bc2 = bcc[cb + vs], bc3 = bcc[cb + 2 * vs];
      double bx = bc1 + fabs(b1[f1idx(m, 0, k, j, i)] - bc1);
      double cf = fast_ms<double>(m.gamma, d, p, bc2, bc3, bx);
      double speed = smax<double>(0.0, (fabs(vx) + cf));
      dt1 /= (speed);
      bx = bc2 + fabs(b2[f2idx(m, 0, k, j, i)] - bc2);
      cf = fast_ms<double>(m.gamma, d, p, bc3, bc1, bx);
      speed = smax<double>(0.0, (fabs(vy) + cf));
      dt2 /= (speed);
      bx = bc3 + fabs(b3[f3idx(m, 0, k, j, i)] - bc3);
      cf = fast_ms<double>(m.gamma, d, p, bc1, bc2, bx);
      speed = smax<double>(0.0, (fabs(vz) + cf));
      dt3 /= (speed);
    }
    cell_dt = smin<double>(smin<double>(dt1, dt2), dt3);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cell_dt = fmin(cell_dt, __shfl_xor_sync(0xffffffffu, cell_dt, o));
  __shared__ double wm[8];
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = cell_dt;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = wm[0];
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) v = fmin(v, wm[q]);
    atomicMin(dtmin_bits, (unsigned long long)__double_as_longlong(v));
  }
}

athgpu_status check_block(athgpu_ctx* c) {
  if (!c) return op_fail(ATHGPU_ERR_ARG, "operator: null context");
  if (c->m.nb != 1)
    return op_fail(ATHGPU_ERR_ARG, "operator calls need a context of one MeshBlock");
  if (c->desc.precision != ATHGPU_FP64)
    return op_fail(ATHGPU_ERR_UNSUPPORTED, "operator calls are FP64");
  if (c->m.ml.on) return op_fail(ATHGPU_ERR_UNSUPPORTED, "operator calls on a uniform block");
  return ATHGPU_OK;
}

// copy between caller memory (host or device) and a register
athgpu_status put(athgpu_ctx* c, void* dev, const void* src, i64 bytes) {
  if (!src) return op_fail(ATHGPU_ERR_ARG, "operator: null input array");
  OCK(cudaMemcpyAsync(dev, src, bytes, cudaMemcpyDefault, c->stream));
  return ATHGPU_OK;
}
athgpu_status get(athgpu_ctx* c, void* dst, const void* dev, i64 bytes) {
  if (!dst) return op_fail(ATHGPU_ERR_ARG, "operator: null output array");
  OCK(cudaMemcpyAsync(dst, dev, bytes, cudaMemcpyDefault, c->stream));
  return ATHGPU_OK;
}

// two counter words of the operator calls (floored cells, dt minimum)
athgpu_status op_words(athgpu_ctx* c) {
  if (c->op_words) return ATHGPU_OK;
  OCK(pool_alloc((void**)&c->op_words, 2 * sizeof(unsigned long long), c->stream));
  return ATHGPU_OK;
}

// flux scratch of the operator calls: [5][nf1] | [5][nf2] | [5][nf3]
athgpu_status op_flux_scratch(athgpu_ctx* c) {
  if (c->op_flx) return ATHGPU_OK;
  const i64 n = 5 * (c->m.nf1 + c->m.nf2 + c->m.nf3);
  OCK(pool_alloc((void**)&c->op_flx, sizeof(double) * n, c->stream));
  OCK(cudaMemsetAsync(c->op_flx, 0, sizeof(double) * n, c->stream));
  return ATHGPU_OK;
}

int solver_index(const athgpu_ctx* c) {
  return c->desc.relativistic ? (c->desc.rsolver == ATHGPU_LLF    ? 5
                                 : c->desc.rsolver == ATHGPU_HLLD ? 6 : 2)
         : c->desc.rsolver == ATHGPU_LLF   ? 3
         : c->desc.rsolver == ATHGPU_ROE   ? 4
         : c->desc.rsolver == ATHGPU_LHLLD ? 7 : c->desc.rsolver;
}

template <int ORDER, int RS>
void launch_op_fluxes(athgpu_ctx* c, double dt, double* f1, double* f2, double* f3) {
  const DevMesh& m = c->m;
  Registers& r = c->r;
  const double* w = (const double*)r.wbuf[0];
  const double* bcc = (const double*)r.bcc;
  const long long n1 = (long long)(m.nx1 + 1) * (m.nx2 + 2) * (m.nx3 + 2);
  const long long n2 = (long long)(m.nx1 + 2) * (m.nx2 + 1) * (m.nx3 + 2);
  const long long n3 = (long long)(m.nx1 + 2) * (m.nx2 + 2) * (m.nx3 + 1);
  op_flux_kernel<0, ORDER, RS><<<grid_of(n1, 128), 128, 0, c->stream>>>(
      m, dt, w, bcc, r.b1, f1, (double*)r.e3x1, (double*)r.e2x1, (double*)r.w1f);
  op_flux_kernel<1, ORDER, RS><<<grid_of(n2, 128), 128, 0, c->stream>>>(
      m, dt, w, bcc, r.b2, f2, (double*)r.e1x2, (double*)r.e3x2, (double*)r.w2f);
  op_flux_kernel<2, ORDER, RS><<<grid_of(n3, 128), 128, 0, c->stream>>>(
      m, dt, w, bcc, r.b3, f3, (double*)r.e2x3, (double*)r.e1x3, (double*)r.w3f);
  c->launches += 3;
}

template <int ORDER>
void launch_op_fluxes_rs(athgpu_ctx* c, int rs, double dt, double* f1, double* f2,
                         double* f3) {
  if (rs == 0) launch_op_fluxes<ORDER, 0>(c, dt, f1, f2, f3);
  else if (rs == 1) launch_op_fluxes<ORDER, 1>(c, dt, f1, f2, f3);
  else if (rs == 2) launch_op_fluxes<ORDER, 2>(c, dt, f1, f2, f3);
  else if (rs == 3) launch_op_fluxes<ORDER, 3>(c, dt, f1, f2, f3);
  else if (rs == 5) launch_op_fluxes<ORDER, 5>(c, dt, f1, f2, f3);
  else if (rs == 6) launch_op_fluxes<ORDER, 6>(c, dt, f1, f2, f3);
  else if (rs == 7) launch_op_fluxes<ORDER, 7>(c, dt, f1, f2, f3);
  else launch_op_fluxes<ORDER, 4>(c, dt, f1, f2, f3);
}

}  // namespace

extern "C" {

athgpu_status athgpu_op_calculate_fluxes(athgpu_ctx* c, int order, double dt, const double* w,
                                         const double* bcc, const double* b1,
                                         const double* b2, const double* b3, double* flx1,
                                         double* flx2, double* flx3,
                                         athgpu_face_emfs* emfs) {
  athgpu_status st = check_block(c);
  if (st != ATHGPU_OK) return st;
  if (order < 1 || order > 4 || (order >= 3 && c->desc.nghost < 3))
    return op_fail(ATHGPU_ERR_ARG,
                   "operator: order must be 1, 2, 3 or 4 (3 and 4 need nghost 3)");
  if (!emfs) return op_fail(ATHGPU_ERR_ARG, "operator: null face-EMF arrays");
  const DevMesh& m = c->m;
  Registers& r = c->r;
  if ((st = op_flux_scratch(c)) != ATHGPU_OK) return st;
  double* f1 = c->op_flx;
  double* f2 = f1 + 5 * m.nf1;
  double* f3 = f2 + 5 * m.nf2;
  const i64 cb = 8 * m.ncell;
  if ((st = put(c, r.wbuf[0], w, 5 * cb)) || (st = put(c, r.bcc, bcc, 3 * cb)) ||
      (st = put(c, r.b1, b1, 8 * m.nf1)) || (st = put(c, r.b2, b2, 8 * m.nf2)) ||
      (st = put(c, r.b3, b3, 8 * m.nf3)) || (st = put(c, f1, flx1, 40 * m.nf1)) ||
      (st = put(c, f2, flx2, 40 * m.nf2)) || (st = put(c, f3, flx3, 40 * m.nf3)) ||
      (st = put(c, r.e3x1, emfs->e3_x1f, 8 * m.nf1)) ||
      (st = put(c, r.e2x1, emfs->e2_x1f, 8 * m.nf1)) ||
      (st = put(c, r.w1f, emfs->wght_x1f, 8 * m.nf1)) ||
      (st = put(c, r.e1x2, emfs->e1_x2f, 8 * m.nf2)) ||
      (st = put(c, r.e3x2, emfs->e3_x2f, 8 * m.nf2)) ||
      (st = put(c, r.w2f, emfs->wght_x2f, 8 * m.nf2)) ||
      (st = put(c, r.e1x3, emfs->e1_x3f, 8 * m.nf3)) ||
      (st = put(c, r.e2x3, emfs->e2_x3f, 8 * m.nf3)) ||
      (st = put(c, r.w3f, emfs->wght_x3f, 8 * m.nf3)))
    return st;
  const int rs = solver_index(c);
  const int ord = order == 3 && c->desc.ppm_fast ? 4 : order;
  if (ord == 1) launch_op_fluxes_rs<1>(c, rs, dt, f1, f2, f3);
  else if (ord == 2) launch_op_fluxes_rs<2>(c, rs, dt, f1, f2, f3);
  else if (ord == 3) launch_op_fluxes_rs<3>(c, rs, dt, f1, f2, f3);
  else launch_op_fluxes_rs<4>(c, rs, dt, f1, f2, f3);
  OCK(cudaGetLastError());
  if ((st = get(c, flx1, f1, 40 * m.nf1)) || (st = get(c, flx2, f2, 40 * m.nf2)) ||
      (st = get(c, flx3, f3, 40 * m.nf3)) ||
      (st = get(c, emfs->e3_x1f, r.e3x1, 8 * m.nf1)) ||
      (st = get(c, emfs->e2_x1f, r.e2x1, 8 * m.nf1)) ||
      (st = get(c, emfs->wght_x1f, r.w1f, 8 * m.nf1)) ||
      (st = get(c, emfs->e1_x2f, r.e1x2, 8 * m.nf2)) ||
      (st = get(c, emfs->e3_x2f, r.e3x2, 8 * m.nf2)) ||
      (st = get(c, emfs->wght_x2f, r.w2f, 8 * m.nf2)) ||
      (st = get(c, emfs->e1_x3f, r.e1x3, 8 * m.nf3)) ||
      (st = get(c, emfs->e2_x3f, r.e2x3, 8 * m.nf3)) ||
      (st = get(c, emfs->wght_x3f, r.w3f, 8 * m.nf3)))
    return st;
  OCK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_op_corner_e(athgpu_ctx* c, const double* w, const double* bcc,
                                 const athgpu_face_emfs* emfs, double* e1, double* e2,
                                 double* e3) {
  athgpu_status st = check_block(c);
  if (st != ATHGPU_OK) return st;
  if (!emfs) return op_fail(ATHGPU_ERR_ARG, "operator: null face-EMF arrays");
  const DevMesh& m = c->m;
  Registers& r = c->r;
  const i64 cb = 8 * m.ncell;
  if ((st = put(c, r.wbuf[0], w, 5 * cb)) || (st = put(c, r.bcc, bcc, 3 * cb)) ||
      (st = put(c, r.e3x1, emfs->e3_x1f, 8 * m.nf1)) ||
      (st = put(c, r.e2x1, emfs->e2_x1f, 8 * m.nf1)) ||
      (st = put(c, r.w1f, emfs->wght_x1f, 8 * m.nf1)) ||
      (st = put(c, r.e1x2, emfs->e1_x2f, 8 * m.nf2)) ||
      (st = put(c, r.e3x2, emfs->e3_x2f, 8 * m.nf2)) ||
      (st = put(c, r.w2f, emfs->wght_x2f, 8 * m.nf2)) ||
      (st = put(c, r.e1x3, emfs->e1_x3f, 8 * m.nf3)) ||
      (st = put(c, r.e2x3, emfs->e2_x3f, 8 * m.nf3)) ||
      (st = put(c, r.w3f, emfs->wght_x3f, 8 * m.nf3)) ||
      (st = put(c, r.e1, e1, 8 * m.ne1)) || (st = put(c, r.e2, e2, 8 * m.ne2)) ||
      (st = put(c, r.e3, e3, 8 * m.ne3)))
    return st;
  const bool sr = c->desc.relativistic;
  (sr ? op_cce_kernel<true> : op_cce_kernel<false>)<<<grid_of(m.ncell, 256), 256, 0,
                                                      c->stream>>>(
      m, (const double*)r.wbuf[0], (const double*)r.bcc, (double*)r.cce);
  const long long n = (long long)(m.nx3 + 1) * (m.nx2 + 1) * (m.nx1 + 1);
  (sr ? corner_e_kernel<double, true>
      : corner_e_kernel<double, false>)<<<dim3(grid_of(n, 128), m.nb < 65535 ? m.nb : 65535),
                                          128, 0, c->stream>>>(
      m, (const double*)r.cce, (double*)r.e3x1, (double*)r.e2x1, (double*)r.w1f,
      (double*)r.e1x2, (double*)r.e3x2, (double*)r.w2f, (double*)r.e1x3, (double*)r.e2x3,
      (double*)r.w3f, (double*)r.e1, (double*)r.e2, (double*)r.e3);
  c->launches += 2;
  OCK(cudaGetLastError());
  if ((st = get(c, e1, r.e1, 8 * m.ne1)) || (st = get(c, e2, r.e2, 8 * m.ne2)) ||
      (st = get(c, e3, r.e3, 8 * m.ne3)))
    return st;
  OCK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_op_add_flux_divergence(athgpu_ctx* c, double wght, const double* flx1,
                                            const double* flx2, const double* flx3,
                                            double* u) {
  athgpu_status st = check_block(c);
  if (st != ATHGPU_OK) return st;
  const DevMesh& m = c->m;
  if ((st = op_flux_scratch(c)) != ATHGPU_OK) return st;
  double* f1 = c->op_flx;
  double* f2 = f1 + 5 * m.nf1;
  double* f3 = f2 + 5 * m.nf2;
  if ((st = put(c, f1, flx1, 40 * m.nf1)) || (st = put(c, f2, flx2, 40 * m.nf2)) ||
      (st = put(c, f3, flx3, 40 * m.nf3)) || (st = put(c, c->r.u, u, 40 * m.ncell)))
    return st;
  const long long n = (long long)m.nx1 * m.nx2 * m.nx3;
  op_divergence_kernel<<<grid_of(n, 256), 256, 0, c->stream>>>(m, wght, f1, f2, f3,
                                                               (double*)c->r.u);
  c->launches += 1;
  OCK(cudaGetLastError());
  if ((st = get(c, u, c->r.u, 40 * m.ncell))) return st;
  OCK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_op_ct(athgpu_ctx* c, double wght, const double* e1, const double* e2,
                           const double* e3, double* b1, double* b2, double* b3) {
  athgpu_status st = check_block(c);
  if (st != ATHGPU_OK) return st;
  const DevMesh& m = c->m;
  Registers& r = c->r;
  if ((st = put(c, r.e1, e1, 8 * m.ne1)) || (st = put(c, r.e2, e2, 8 * m.ne2)) ||
      (st = put(c, r.e3, e3, 8 * m.ne3)) || (st = put(c, r.b1, b1, 8 * m.nf1)) ||
      (st = put(c, r.b2, b2, 8 * m.nf2)) || (st = put(c, r.b3, b3, 8 * m.nf3)))
    return st;
  const double* ee1 = (const double*)r.e1;
  const double* ee2 = (const double*)r.e2;
  const double* ee3 = (const double*)r.e3;
  const long long n1 = (long long)(m.nx1 + 1) * m.nx2 * m.nx3;
  const long long n2 = (long long)m.nx1 * (m.nx2 + 1) * m.nx3;
  const long long n3 = (long long)m.nx1 * m.nx2 * (m.nx3 + 1);
  op_ct_kernel<0><<<grid_of(n1, 256), 256, 0, c->stream>>>(m, wght, ee1, ee2, ee3, r.b1);
  op_ct_kernel<1><<<grid_of(n2, 256), 256, 0, c->stream>>>(m, wght, ee1, ee2, ee3, r.b2);
  op_ct_kernel<2><<<grid_of(n3, 256), 256, 0, c->stream>>>(m, wght, ee1, ee2, ee3, r.b3);
  c->launches += 3;
  OCK(cudaGetLastError());
  if ((st = get(c, b1, r.b1, 8 * m.nf1)) || (st = get(c, b2, r.b2, 8 * m.nf2)) ||
      (st = get(c, b3, r.b3, 8 * m.nf3)))
    return st;
  OCK(cudaStreamSynchronize(c->stream));
  return ATHGPU_OK;
}

athgpu_status athgpu_op_con2prim(athgpu_ctx* c, double* cons, const double* b1,
                                 const double* b2, const double* b3, double* prim,
                                 double* bcc, int il, int iu, int jl, int ju, int kl, int ku,
                                 long long* nfloored) {
  athgpu_status st = check_block(c);
  if (st != ATHGPU_OK) return st;
  const DevMesh& m = c->m;
  Registers& r = c->r;
  if (il < 0 || jl < 0 || kl < 0 || iu >= m.nc1 || ju >= m.nc2 || ku >= m.nc3 || il > iu ||
      jl > ju || kl > ku)
    return op_fail(ATHGPU_ERR_ARG, "operator: con2prim range outside the block");
  const i64 cb = 8 * m.ncell;
  if ((st = put(c, r.u, cons, 5 * cb)) || (st = put(c, r.wbuf[0], prim, 5 * cb)) ||
      (st = put(c, r.bcc, bcc, 3 * cb)) || (st = put(c, r.b1, b1, 8 * m.nf1)) ||
      (st = put(c, r.b2, b2, 8 * m.nf2)) || (st = put(c, r.b3, b3, 8 * m.nf3)))
    return st;
  if ((st = op_words(c)) != ATHGPU_OK) return st;
  unsigned long long* cnt = c->op_words;
  OCK(cudaMemsetAsync(cnt, 0, sizeof(*cnt), c->stream));
  SRFloors fp{c->desc.gamma, c->desc.dfloor, c->desc.pfloor, c->desc.sigma_max,
              c->desc.beta_min, c->desc.gamma_max};
  const long long n = (long long)(iu - il + 1) * (ju - jl + 1) * (ku - kl + 1);
  (c->desc.relativistic ? op_c2p_kernel<true> : op_c2p_kernel<false>)<<<grid_of(n, 128), 128,
                                                                        0, c->stream>>>(
      m, fp, il, iu, jl, ju, kl, ku, r.b1, r.b2, r.b3, (double*)r.u, (double*)r.wbuf[0],
      (double*)r.bcc, cnt);
  c->launches += 1;
  OCK(cudaGetLastError());
  unsigned long long nf = 0;
  OCK(cudaMemcpyAsync(&nf, cnt, sizeof(nf), cudaMemcpyDeviceToHost, c->stream));
  if ((st = get(c, cons, r.u, 5 * cb)) || (st = get(c, prim, r.wbuf[0], 5 * cb)) ||
      (st = get(c, bcc, r.bcc, 3 * cb)))
    return st;
  OCK(cudaStreamSynchronize(c->stream));
  if (nfloored) *nfloored = (long long)nf;
  return ATHGPU_OK;
}

athgpu_status athgpu_op_new_block_dt(athgpu_ctx* c, const double* w, const double* bcc,
                                     const double* b1, const double* b2, const double* b3,
                                     double* dt_out) {
  athgpu_status st = check_block(c);
  if (st != ATHGPU_OK) return st;
  if (!dt_out) return op_fail(ATHGPU_ERR_ARG, "operator: null dt_out");
  const DevMesh& m = c->m;
  Registers& r = c->r;
  const i64 cb = 8 * m.ncell;
  if ((st = put(c, r.wbuf[0], w, 5 * cb)) || (st = put(c, r.bcc, bcc, 3 * cb)) ||
      (st = put(c, r.b1, b1, 8 * m.nf1)) || (st = put(c, r.b2, b2, 8 * m.nf2)) ||
      (st = put(c, r.b3, b3, 8 * m.nf3)))
    return st;
  if ((st = op_words(c)) != ATHGPU_OK) return st;
  unsigned long long* bits = c->op_words + 1;
  unsigned long long init = 0;
  const double big = DBL_MAX;
  memcpy(&init, &big, 8);
  OCK(cudaMemcpyAsync(bits, &init, 8, cudaMemcpyHostToDevice, c->stream));
  const long long n = (long long)m.nx1 * m.nx2 * m.nx3;
  (c->desc.relativistic ? op_dt_kernel<true> : op_dt_kernel<false>)<<<grid_of(n, 256), 256,
                                                                      0, c->stream>>>(
      m, (const double*)r.wbuf[0], (const double*)r.bcc, r.b1, r.b2, r.b3, bits);
  c->launches += 1;
  OCK(cudaGetLastError());
  unsigned long long got = 0;
  OCK(cudaMemcpyAsync(&got, bits, 8, cudaMemcpyDeviceToHost, c->stream));
  OCK(cudaStreamSynchronize(c->stream));
  double mn;
  memcpy(&mn, &got, 8);
  *dt_out = mn * c->desc.cfl_number;  // new_blockdt.cpp:193
  return ATHGPU_OK;
}

}  // extern "C"
