// Multi-level meshes (static or adaptive mesh refinement): the parts of the stage that
// differ from a uniform mesh.
//
//  * ml_ops_kernel: one CTA per MeshBlock executes that block's list of box operations in
//    order (a barrier between operations).  Three lists per stage, built on the host
//    (ml_plan.cpp): the restriction of a block's cells and faces for its coarser
//    neighbours into its send buffers; the ghost exchange (same-level copies, restricted
//    values from finer neighbours, coarse-buffer filling from coarser neighbours) in the
//    order of the block's neighbour list, which decides the faces that edges and corners
//    overwrite; and ProlongateBoundaries (the same-level ghost-ghost restriction, W(U) and
//    the physical boundaries on the coarse level, prolongation of the primitives and the
//    face field, the cell-centred field and U(W) of the filled ghosts).  Reference:
//    bvals/cc/bvals_cc.cpp, bvals/fc/bvals_fc.cpp, bvals/bvals_refine.cpp,
//    mesh/mesh_refinement.cpp.
//  * ml_fine_flux_kernel: the hydro fluxes of finer blocks on faces they share with a
//    coarser block, area-weighted into the coarse faces (flux_correction_cc.cpp); the
//    sweeps use them in place of the coarse block's own fluxes there.
//  * ml_emf_kernel: every block-boundary edge EMF corrected across levels
//    (flux_correction_fc.cpp): own value plus same-level neighbours' in list order, or
//    (on edges shared with finer blocks) the sum of the finer blocks' restricted values,
//    then the division by the number of contributions.
//
// Restriction, prolongation, W(U) and U(W) on the coarse level and the ghost zones are
// computed in FP64 with the reference's operand order (values are stored in the bulk
// precision), so the FP64 path is bit-identical to the reference.
#pragma once
#include "kernels.cuh"
#include "ml_types.h"

namespace athgpu {

template <typename Real>
struct MlArrays {
  Real* u;        // fine U [nb][5][ncell]
  Real* w;        // fine W written by the prolongation
  Real* bcc;      // fine cell-centred field
  double *b1, *b2, *b3;
};

// ---- indexing --------------------------------------------------------------------------
__device__ __forceinline__ i64 ccidx(const DevMesh& m, int b, int n, int nvar, int k, int j,
                                     int i) {
  return (((i64)b * nvar + n) * m.ml.ncc3 + k) * (i64)m.ml.ncc2 * m.ml.ncc1 +
         (i64)j * m.ml.ncc1 + i;
}
// face index of component d in a fine (coarse = false) or coarse array of block b
__device__ __forceinline__ i64 fcidx(const DevMesh& m, bool coarse, int d, int b, int k,
                                     int j, int i) {
  const int n1 = coarse ? m.ml.ncc1 : m.nc1, n2 = coarse ? m.ml.ncc2 : m.nc2,
            n3 = coarse ? m.ml.ncc3 : m.nc3;
  const i64 per = coarse ? (d == 0 ? m.ml.ncf1 : d == 1 ? m.ml.ncf2 : m.ml.ncf3)
                         : (d == 0 ? m.nf1 : d == 1 ? m.nf2 : m.nf3);
  const int a1 = n1 + (d == 0), a2 = n2 + (d == 1);
  (void)n3;
  return (i64)b * per + ((i64)k * a2 + j) * a1 + i;
}
__device__ __forceinline__ int box_count(const MlOp& op) {
  return (op.e[0] - op.s[0] + 1) * (op.e[1] - op.s[1] + 1) * (op.e[2] - op.s[2] + 1);
}
__device__ __forceinline__ void box_pos(const MlOp& op, int t, int& k, int& j, int& i) {
  const int n0 = op.e[0] - op.s[0] + 1, n1 = op.e[1] - op.s[1] + 1;
  i = op.s[0] + t % n0;
  t /= n0;
  j = op.s[1] + t % n1;
  k = op.s[2] + t / n1;
}
__device__ __forceinline__ double ldr(const double* p) { return *p; }
__device__ __forceinline__ double ldr(const float* p) { return (double)*p; }

template <typename T>
__device__ __forceinline__ T mm_grad(T cm, T c0, T cp, T dxm, T dxp) {
  const T gm = (c0 - cm) / dxm, gp = (cp - c0) / dxp;
  const T sg = ((gm < T(0)) ? T(-1) : T(1)) + ((gp < T(0)) ? T(-1) : T(1));
  const T am = fabs(gm), ap = fabs(gp);
  return T(0.5) * sg * ((ap < am) ? ap : am);
}

// ---- the per-block operation executor ------------------------------------------------
// CODE: the operation code as a template parameter, so that each instance keeps only its
// own branch of the element loop
template <typename Real, int CODE>
__device__ __forceinline__ void ml_op_code(const DevMesh& m, const MlArrays<Real>& A, int b,
                                           const MlOp& op, int t0, int dt) {
  const DevML& L = m.ml;
  const int nel = box_count(op);
  const double* dx[3] = {m.dx1f + (i64)b * m.nc1, m.dx2f + (i64)b * m.nc2,
                         m.dx3f + (i64)b * m.nc3};
  const int clo[3] = {L.cis, L.cjs, L.cks}, flo[3] = {m.is, m.js, m.ks};
  // face arrays by component (selected, not indexed: no local-memory pointer tables)
  auto FB = [&](int d) -> double* { return d == 0 ? A.b1 : d == 1 ? A.b2 : A.b3; };
  auto CBS = [&](int d) -> double* { return d == 0 ? L.cb1 : d == 1 ? L.cb2 : L.cb3; };
  auto SBS = [&](int d) -> double* { return d == 0 ? L.sb1 : d == 1 ? L.sb2 : L.sb3; };
  Real* cu = (Real*)L.ccons;
  Real* su = (Real*)L.scons;
  Real* cw = (Real*)L.cprim;
  Real* cbcc = (Real*)L.cbcc;
  if (CODE == ML_COPY_U || CODE == ML_COPY_B) {
    // copies: four elements per thread per pass, all loads issued before the stores
    // (the copies are latency-bound reads of other blocks' data)
    constexpr int U = 4;
    const bool ssend = op.src_kind == ML_SEND, dcoarse = op.dst_kind == ML_COARSE;
    for (int t = t0; t < nel; t += U * dt) {
      i64 sidx[U], didx[U];
      bool ok[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int tt = t + u * dt;
        ok[u] = tt < nel;
        int k, j, i;
        box_pos(op, ok[u] ? tt : t, k, j, i);
        const int sk = op.o[2] + (k - op.s[2]), sj = op.o[1] + (j - op.s[1]),
                  si = op.o[0] + (i - op.s[0]);
        if (CODE == ML_COPY_U) {
          sidx[u] = ssend ? ccidx(m, op.src, 0, NHYDRO, sk, sj, si)
                          : cidx(m, op.src, 0, NHYDRO, sk, sj, si);
          didx[u] = dcoarse ? ccidx(m, b, 0, NHYDRO, k, j, i) : cidx(m, b, 0, NHYDRO, k, j, i);
        } else {
          sidx[u] = fcidx(m, ssend, op.d, op.src, sk, sj, si);
          didx[u] = fcidx(m, dcoarse, op.d, b, k, j, i);
        }
      }
      if (CODE == ML_COPY_U) {
        const Real* sp = ssend ? su : A.u;
        Real* dp = dcoarse ? cu : A.u;
        const i64 svs = ssend ? L.nccell : m.ncell, dvs = dcoarse ? L.nccell : m.ncell;
        Real v[U][NHYDRO];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int n = 0; n < NHYDRO; ++n)
            if (ok[u]) v[u][n] = sp[sidx[u] + n * svs];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
          for (int n = 0; n < NHYDRO; ++n)
            if (ok[u]) dp[didx[u] + n * dvs] = v[u][n];
      } else {
        const double* sp = ssend ? SBS(op.d) : FB(op.d);
        double* dp = dcoarse ? CBS(op.d) : FB(op.d);
        double v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u]) v[u] = sp[sidx[u]];
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (ok[u]) dp[didx[u]] = v[u];
      }
    }
    return;
  }
  for (int t = t0; t < nel; t += dt) {
    int k, j, i;
    box_pos(op, t, k, j, i);
    switch (CODE) {
      case ML_COPY_U: {
        const int sk = op.o[2] + (k - op.s[2]), sj = op.o[1] + (j - op.s[1]),
                  si = op.o[0] + (i - op.s[0]);
        const bool ssend = op.src_kind == ML_SEND, dcoarse = op.dst_kind == ML_COARSE;
        const Real* sp = ssend ? su + ccidx(m, op.src, 0, NHYDRO, sk, sj, si)
                               : A.u + cidx(m, op.src, 0, NHYDRO, sk, sj, si);
        Real* dp = dcoarse ? cu + ccidx(m, b, 0, NHYDRO, k, j, i)
                           : A.u + cidx(m, b, 0, NHYDRO, k, j, i);
        const i64 svs = ssend ? L.nccell : m.ncell, dvs = dcoarse ? L.nccell : m.ncell;
#pragma unroll
        for (int n = 0; n < NHYDRO; ++n) dp[n * dvs] = sp[n * svs];
        break;
      }
      case ML_COPY_B: {
        const int sk = op.o[2] + (k - op.s[2]), sj = op.o[1] + (j - op.s[1]),
                  si = op.o[0] + (i - op.s[0]);
        const double v = op.src_kind == ML_SEND
                             ? SBS(op.d)[fcidx(m, true, op.d, op.src, sk, sj, si)]
                             : FB(op.d)[fcidx(m, false, op.d, op.src, sk, sj, si)];
        if (op.dst_kind == ML_COARSE) CBS(op.d)[fcidx(m, true, op.d, b, k, j, i)] = v;
        else FB(op.d)[fcidx(m, false, op.d, b, k, j, i)] = v;
        break;
      }
      case ML_RESTRICT_U: {  // mesh_refinement.cpp:116-189, CellVolume = dx1 dx2 dx3
        // cell-centred operations compute in the bulk precision (FP64: the reference's
        // arithmetic; FP32 path: FP32)
        using Acc = Real;
        const int fk = (k - L.cks) * 2 + m.ks, fj = (j - L.cjs) * 2 + m.js,
                  fi = (i - L.cis) * 2 + m.is;
        const Acc d1a = (Acc)dx[0][fi], d1b = (Acc)dx[0][fi + 1], d2a = (Acc)dx[1][fj],
                  d2b = (Acc)dx[1][fj + 1], d3a = (Acc)dx[2][fk], d3b = (Acc)dx[2][fk + 1];
        const Acc v000 = d1a * d2a * d3a, v001 = d1b * d2a * d3a;
        const Acc v010 = d1a * d2b * d3a, v011 = d1b * d2b * d3a;
        const Acc v100 = d1a * d2a * d3b, v101 = d1b * d2a * d3b;
        const Acc v110 = d1a * d2b * d3b, v111 = d1b * d2b * d3b;
        const Acc tvol = ((v000 + v010) + (v001 + v011)) + ((v100 + v110) + (v101 + v111));
        // ML_SEND: the values sent to coarser blocks, also kept in the coarse buffer as the
        // prolongation stencil's inner side (LoadBoundaryBufferToCoarser restricts into it)
        const bool both = op.src_kind == ML_SEND;
        const i64 pj = m.nc1, pk = (i64)m.nc1 * m.nc2;
        const Real* ub = A.u + cidx(m, b, 0, NHYDRO, fk, fj, fi);
        const i64 cb0 = ccidx(m, b, 0, NHYDRO, k, j, i);
        for (int n = 0; n < NHYDRO; ++n) {
          const Real* un = ub + n * m.ncell;
          auto f = [&](int kk, int jj, int ii) { return un[kk * pk + jj * pj + ii]; };
          const Acc v = (((f(0, 0, 0) * v000 + f(0, 1, 0) * v010) +
                          (f(0, 0, 1) * v001 + f(0, 1, 1) * v011)) +
                         ((f(1, 0, 0) * v100 + f(1, 1, 0) * v110) +
                          (f(1, 0, 1) * v101 + f(1, 1, 1) * v111))) / tvol;
          cu[cb0 + n * L.nccell] = (Real)v;
          if (both) su[cb0 + n * L.nccell] = (Real)v;
        }
        break;
      }
      case ML_RESTRICT_B: {  // mesh_refinement.cpp:272-463
        const int fk = (k - L.cks) * 2 + m.ks, fj = (j - L.cjs) * 2 + m.js,
                  fi = (i - L.cis) * 2 + m.is;
        const double* F = FB(op.d);
        auto f = [&](int kk, int jj, int ii) {
          return F[fcidx(m, false, op.d, b, fk + kk, fj + jj, fi + ii)];
        };
        double v;
        if (op.d == 0) {
          const double a00 = dx[1][fj] * dx[2][fk], a01 = dx[1][fj + 1] * dx[2][fk];
          const double a10 = dx[1][fj] * dx[2][fk + 1], a11 = dx[1][fj + 1] * dx[2][fk + 1];
          const double tarea = a00 + a01 + a10 + a11;
          v = (f(0, 0, 0) * a00 + f(0, 1, 0) * a01 + f(1, 0, 0) * a10 + f(1, 1, 0) * a11) / tarea;
        } else if (op.d == 1) {
          const double s0i = dx[0][fi] * dx[2][fk], s0p = dx[0][fi + 1] * dx[2][fk];
          const double s1i = dx[0][fi] * dx[2][fk + 1], s1p = dx[0][fi + 1] * dx[2][fk + 1];
          const double tarea = s0i + s0p + s1i + s1p;
          v = (f(0, 0, 0) * s0i + f(0, 0, 1) * s0p + f(1, 0, 0) * s1i + f(1, 0, 1) * s1p) / tarea;
        } else {
          const double s0i = dx[0][fi] * dx[1][fj], s0p = dx[0][fi + 1] * dx[1][fj];
          const double s1i = dx[0][fi] * dx[1][fj + 1], s1p = dx[0][fi + 1] * dx[1][fj + 1];
          const double tarea = s0i + s0p + s1i + s1p;
          v = (f(0, 0, 0) * s0i + f(0, 0, 1) * s0p + f(0, 1, 0) * s1i + f(0, 1, 1) * s1p) / tarea;
        }
        CBS(op.d)[fcidx(m, true, op.d, b, k, j, i)] = v;
        if (op.src_kind == ML_SEND) SBS(op.d)[fcidx(m, true, op.d, b, k, j, i)] = v;
        break;
      }
      case ML_C2P_COARSE: {  // adiabatic_mhd.cpp:41-90 with field.cpp:112-180
        using Acc = Real;
        const i64 vs = L.nccell;
        const i64 c = ccidx(m, b, 0, NHYDRO, k, j, i);
        const i64 cb = ccidx(m, b, 0, 3, k, j, i);
        const double lw = 0.5, rw = 0.5;
        const Acc bc1 = (Acc)(lw * L.cb1[fcidx(m, true, 0, b, k, j, i)] +
                              rw * L.cb1[fcidx(m, true, 0, b, k, j, i + 1)]);
        const Acc bc2 = (Acc)(lw * L.cb2[fcidx(m, true, 1, b, k, j, i)] +
                              rw * L.cb2[fcidx(m, true, 1, b, k, j + 1, i)]);
        const Acc bc3 = (Acc)(lw * L.cb3[fcidx(m, true, 2, b, k, j, i)] +
                              rw * L.cb3[fcidx(m, true, 2, b, k + 1, j, i)]);
        cbcc[cb] = (Real)bc1;
        cbcc[cb + vs] = (Real)bc2;
        cbcc[cb + 2 * vs] = (Real)bc3;
        const Acc gm1 = (Acc)(m.gamma - 1.0), dfl = (Acc)m.dfloor, pfl = (Acc)m.pfloor;
        Acc u_d = cu[c], u_e = cu[c + 4 * vs];
        const Acc u_m1 = cu[c + vs], u_m2 = cu[c + 2 * vs], u_m3 = cu[c + 3 * vs];
        u_d = (u_d > dfl) ? u_d : dfl;
        cu[c] = (Real)u_d;
        const Acc di = Acc(1) / u_d;
        cw[c] = (Real)u_d;
        cw[c + vs] = (Real)(u_m1 * di);
        cw[c + 2 * vs] = (Real)(u_m2 * di);
        cw[c + 3 * vs] = (Real)(u_m3 * di);
        const Acc pb = Acc(0.5) * (bc1 * bc1 + bc2 * bc2 + bc3 * bc3);
        const Acc e_k = Acc(0.5) * di * (u_m1 * u_m1 + u_m2 * u_m2 + u_m3 * u_m3);
        const Acc w_p = gm1 * (u_e - e_k - pb);
        cu[c + 4 * vs] = (Real)((w_p > pfl) ? u_e : ((pfl / gm1) + e_k + pb));
        cw[c + 4 * vs] = (Real)((w_p > pfl) ? w_p : pfl);
        break;
      }
      case ML_BC_COARSE: {
        // the element enumerates (layer g, transverse position) via the box: the box's
        // normal-axis extent is 1..ng (layers), the others the transverse ranges
        const int f = op.aux & 7, kind = op.aux >> 4;
        const int a = f >> 1, side = f & 1;
        const int chi[3] = {L.cie, L.cje, L.cke};
        int pos[3] = {i, j, k};
        const int g = pos[a];
        const int lo = clo[a], hi = chi[a];
        const int dst = side ? hi + g : lo - g;
        const int srcc = (kind == 1) ? (side ? hi : lo) : (side ? hi - g + 1 : lo + g - 1);
        const bool in_cell = true;
        (void)in_cell;
        // cells: the transverse box is the cell range; the e[] of the face components
        // along a transverse axis extend one further (handled by the box being built one
        // larger and this cell branch skipping the extra entries)
        int tr_ok[3] = {1, 1, 1};
        for (int q = 0; q < 3; ++q)
          if (q != a && pos[q] == op.e[q]) tr_ok[q] = 0;  // the extra face row
        const bool cell_ok = tr_ok[0] && tr_ok[1] && tr_ok[2];
        if (cell_ok) {
          int c3[3] = {pos[0], pos[1], pos[2]}, s3[3] = {pos[0], pos[1], pos[2]};
          c3[a] = dst;
          s3[a] = srcc;
          for (int n = 0; n < NHYDRO; ++n) {
            const Real v = cw[ccidx(m, b, n, NHYDRO, s3[2], s3[1], s3[0])];
            cw[ccidx(m, b, n, NHYDRO, c3[2], c3[1], c3[0])] =
                (kind == 2 && n == IVX + a) ? -v : v;
          }
        }
        for (int d = 0; d < 3; ++d) {
          // component d covers the cell range, plus one along its own direction d != a
          bool ok = true;
          for (int q = 0; q < 3; ++q)
            if (q != a && q != d && !tr_ok[q]) ok = false;
          if (!ok) continue;
          int c3[3] = {pos[0], pos[1], pos[2]}, s3[3] = {pos[0], pos[1], pos[2]};
          double sgn = 1.0;
          if (d == a) {
            c3[a] = side ? hi + 1 + g : lo - g;
            s3[a] = (kind == 1) ? (side ? hi + 1 : lo) : (side ? hi + 1 - g : lo + g);
            if (kind == 2) sgn = -1.0;
          } else {
            c3[a] = dst;
            s3[a] = srcc;
          }
          const double v = CBS(d)[fcidx(m, true, d, b, s3[2], s3[1], s3[0])];
          CBS(d)[fcidx(m, true, d, b, c3[2], c3[1], c3[0])] = sgn < 0.0 ? -v : v;
        }
        break;
      }
      case ML_PROLONG_U: {  // mesh_refinement.cpp:464-540
        // coarse W into W (ProlongateBoundaries), or with src_kind ML_COARSE the coarse
        // U into U (ProlongateMeshBlock after a refinement, amr_loadbalance.cpp:1172-1180)
        using Acc = Real;
        const Real* csrc = op.src_kind == ML_COARSE ? cu : cw;
        Real* fdst = op.src_kind == ML_COARSE ? A.u : A.w;
        const int fk = (k - L.cks) * 2 + m.ks, fj = (j - L.cjs) * 2 + m.js,
                  fi = (i - L.cis) * 2 + m.is;
        const double* cx1 = L.cx1v + (i64)b * L.ncc1;
        const double* cx2 = L.cx2v + (i64)b * L.ncc2;
        const double* cx3 = L.cx3v + (i64)b * L.ncc3;
        const double* fx1 = L.fx1v + (i64)b * m.nc1;
        const double* fx2 = L.fx2v + (i64)b * m.nc2;
        const double* fx3 = L.fx3v + (i64)b * m.nc3;
        // coordinate differences in FP64 (exact in the FP64 path), then the bulk precision
        const Acc dx3m = (Acc)(cx3[k] - cx3[k - 1]), dx3p = (Acc)(cx3[k + 1] - cx3[k]);
        const Acc dx3fm = (Acc)(cx3[k] - fx3[fk]), dx3fp = (Acc)(fx3[fk + 1] - cx3[k]);
        const Acc dx2m = (Acc)(cx2[j] - cx2[j - 1]), dx2p = (Acc)(cx2[j + 1] - cx2[j]);
        const Acc dx2fm = (Acc)(cx2[j] - fx2[fj]), dx2fp = (Acc)(fx2[fj + 1] - cx2[j]);
        const Acc dx1m = (Acc)(cx1[i] - cx1[i - 1]), dx1p = (Acc)(cx1[i + 1] - cx1[i]);
        const Acc dx1fm = (Acc)(cx1[i] - fx1[fi]), dx1fp = (Acc)(fx1[fi + 1] - cx1[i]);
        const i64 cj = L.ncc1, ck = (i64)L.ncc1 * L.ncc2;
        const i64 fj1 = m.nc1, fk1 = (i64)m.nc1 * m.nc2;
        const Real* cbase = csrc + ccidx(m, b, 0, NHYDRO, k, j, i);
        Real* fbase = fdst + cidx(m, b, 0, NHYDRO, fk, fj, fi);
        for (int n = 0; n < NHYDRO; ++n) {
          const Real* cn = cbase + n * L.nccell;
          Real* fn = fbase + n * m.ncell;
          auto cv = [&](int kk, int jj, int ii) -> Acc { return cn[kk * ck + jj * cj + ii]; };
          const Acc cc = cv(0, 0, 0);
          const Acc g1 = mm_grad<Acc>(cv(0, 0, -1), cc, cv(0, 0, 1), dx1m, dx1p);
          const Acc g2 = mm_grad<Acc>(cv(0, -1, 0), cc, cv(0, 1, 0), dx2m, dx2p);
          const Acc g3 = mm_grad<Acc>(cv(-1, 0, 0), cc, cv(1, 0, 0), dx3m, dx3p);
          auto put = [&](int kk, int jj, int ii, Acc v) {
            fn[kk * fk1 + jj * fj1 + ii] = (Real)v;
          };
          put(0, 0, 0, cc - (g1 * dx1fm + g2 * dx2fm + g3 * dx3fm));
          put(0, 0, 1, cc + (g1 * dx1fp - g2 * dx2fm - g3 * dx3fm));
          put(0, 1, 0, cc - (g1 * dx1fm - g2 * dx2fp + g3 * dx3fm));
          put(0, 1, 1, cc + (g1 * dx1fp + g2 * dx2fp - g3 * dx3fm));
          put(1, 0, 0, cc - (g1 * dx1fm + g2 * dx2fm - g3 * dx3fp));
          put(1, 0, 1, cc + (g1 * dx1fp - g2 * dx2fm + g3 * dx3fp));
          put(1, 1, 0, cc - (g1 * dx1fm - g2 * dx2fp - g3 * dx3fp));
          put(1, 1, 1, cc + (g1 * dx1fp + g2 * dx2fp + g3 * dx3fp));
        }
        break;
      }
      case ML_PROLONG_SHARED: {  // mesh_refinement.cpp:829-870, 974-1012, 1118-1156
        const int d = op.d;
        const int ta = (d == 0) ? 1 : 0, tb = (d == 2) ? 1 : 2;
        const double* cxs[3] = {L.cx1v + (i64)b * L.ncc1, L.cx2v + (i64)b * L.ncc2,
                                L.cx3v + (i64)b * L.ncc3};
        const double* fxs[3] = {L.fx1v + (i64)b * m.nc1, L.fx2v + (i64)b * m.nc2,
                                L.fx3v + (i64)b * m.nc3};
        const int cidx3[3] = {i, j, k};
        int f3[3];
        for (int a = 0; a < 3; ++a) f3[a] = (cidx3[a] - clo[a]) * 2 + flo[a];
        const double* C = CBS(d);
        auto cv = [&](int kk, int jj, int ii) { return C[fcidx(m, true, d, b, kk, jj, ii)]; };
        const double cc = cv(k, j, i);
        double g[3] = {0, 0, 0}, am[3] = {0, 0, 0}, ap[3] = {0, 0, 0};
        for (int q = 0; q < 2; ++q) {
          const int a = q ? tb : ta;
          int mi[3] = {i, j, k}, pi[3] = {i, j, k};
          mi[a]--;
          pi[a]++;
          const double xc = cxs[a][cidx3[a]];
          g[a] = mm_grad(cv(mi[2], mi[1], mi[0]), cc, cv(pi[2], pi[1], pi[0]),
                         xc - cxs[a][cidx3[a] - 1], cxs[a][cidx3[a] + 1] - xc);
          am[a] = xc - fxs[a][f3[a]];
          ap[a] = fxs[a][f3[a] + 1] - xc;
        }
        double* F = FB(d);
        for (int ob = 0; ob < 2; ++ob)
          for (int oa = 0; oa < 2; ++oa) {
            int ff[3] = {f3[0], f3[1], f3[2]};
            ff[ta] += oa;
            ff[tb] += ob;
            const double tat = oa ? g[ta] * ap[ta] : g[ta] * am[ta];
            const double tbt = ob ? g[tb] * ap[tb] : g[tb] * am[tb];
            double v = oa ? cc + tat : cc - tat;
            v = ob ? v + tbt : v - tbt;
            F[fcidx(m, false, d, b, ff[2], ff[1], ff[0])] = v;
          }
        break;
      }
      case ML_PROLONG_INTERNAL: {  // mesh_refinement.cpp:1223-1300
        const int fk = (k - L.cks) * 2 + m.ks, fj = (j - L.cjs) * 2 + m.js,
                  fi = (i - L.cis) * 2 + m.is;
        const double *d1 = dx[0], *d2 = dx[1], *d3 = dx[2];
        auto X1 = [&](int kk, int jj, int ii) -> double& {
          return A.b1[fcidx(m, false, 0, b, kk, jj, ii)];
        };
        auto X2 = [&](int kk, int jj, int ii) -> double& {
          return A.b2[fcidx(m, false, 1, b, kk, jj, ii)];
        };
        auto X3 = [&](int kk, int jj, int ii) -> double& {
          return A.b3[fcidx(m, false, 2, b, kk, jj, ii)];
        };
        auto A1 = [&](int kk, int jj) { return d2[fj + jj] * d3[fk + kk]; };
        auto A2 = [&](int kk, int ii) { return d1[ii] * d3[fk + kk]; };
        auto A3 = [&](int jj, int ii) { return d1[ii] * d2[fj + jj]; };
        double Uxx = 0.0, Vyy = 0.0, Wzz = 0.0, Uxyz = 0.0, Vxyz = 0.0, Wxyz = 0.0;
        for (int jj = 0; jj < 2; ++jj) {
          const double sj = (double)(2 * jj - 1);
          const int fjj = fj + jj, fjp = fj + 2 * jj;
          for (int ii = 0; ii < 2; ++ii) {
            const double si = (double)(2 * ii - 1);
            const int fii = fi + ii, fip = fi + 2 * ii;
            const double x2lo = X2(fk, fjp, fii) * A2(0, fii);
            const double x2hi = X2(fk + 1, fjp, fii) * A2(1, fii);
            const double x3lo = X3(fk, fjj, fii) * A3(jj, fii);
            const double x3hi = X3(fk + 2, fjj, fii) * A3(jj, fii);
            const double x1lo = X1(fk, fjj, fip) * A1(0, jj);
            const double x1hi = X1(fk + 1, fjj, fip) * A1(1, jj);
            Uxx += si * (sj * (x2lo + x2hi) + (x3hi - x3lo));
            Vyy += sj * ((x3hi - x3lo) + si * (x1lo + x1hi));
            Wzz += si * (x1hi - x1lo) + sj * (x2hi - x2lo);
            Uxyz += (si * sj) * (x1hi - x1lo);
            Vxyz += (si * sj) * (x2hi - x2lo);
            Wxyz += (si * sj) * (x3hi - x3lo);
          }
        }
        const double Sdx1 = (d1[fi] + d1[fi + 1]) * (d1[fi] + d1[fi + 1]);
        const double Sdx2 = (d2[fj] + d2[fj + 1]) * (d2[fj] + d2[fj + 1]);
        const double Sdx3 = (d3[fk] + d3[fk + 1]) * (d3[fk] + d3[fk + 1]);
        Uxx *= 0.125;
        Vyy *= 0.125;
        Wzz *= 0.125;
        Uxyz *= 0.125 / (Sdx2 + Sdx3);
        Vxyz *= 0.125 / (Sdx1 + Sdx3);
        Wxyz *= 0.125 / (Sdx1 + Sdx2);
        for (int kk = 0; kk < 2; ++kk)
          for (int jj = 0; jj < 2; ++jj) {
            const double a = A1(kk, jj);
            double v = 0.5 * (X1(fk + kk, fj + jj, fi) * a + X1(fk + kk, fj + jj, fi + 2) * a) + Uxx;
            v = kk ? v + Sdx3 * Vxyz : v - Sdx3 * Vxyz;
            v = jj ? v + Sdx2 * Wxyz : v - Sdx2 * Wxyz;
            X1(fk + kk, fj + jj, fi + 1) = v / a;
          }
        for (int kk = 0; kk < 2; ++kk)
          for (int ii = 0; ii < 2; ++ii) {
            const double a = A2(kk, fi + ii);
            double v = 0.5 * (X2(fk + kk, fj, fi + ii) * a + X2(fk + kk, fj + 2, fi + ii) * a) + Vyy;
            v = kk ? v + Sdx3 * Uxyz : v - Sdx3 * Uxyz;
            v = ii ? v + Sdx1 * Wxyz : v - Sdx1 * Wxyz;
            X2(fk + kk, fj + 1, fi + ii) = v / a;
          }
        for (int jj = 0; jj < 2; ++jj)
          for (int ii = 0; ii < 2; ++ii) {
            const double a = A3(jj, fi + ii);
            double v = 0.5 * (X3(fk + 2, fj + jj, fi + ii) * a + X3(fk, fj + jj, fi + ii) * a) + Wzz;
            v = jj ? v + Sdx2 * Uxyz : v - Sdx2 * Uxyz;
            v = ii ? v + Sdx1 * Vxyz : v - Sdx1 * Vxyz;
            X3(fk + 1, fj + jj, fi + ii) = v / a;
          }
        break;
      }
      case ML_FINE_P2C: {  // field.cpp:112-180 then adiabatic_mhd.cpp:99-133
        const i64 vs = m.ncell;
        const i64 c = cidx(m, b, 0, NHYDRO, k, j, i);
        const i64 cb = cidx(m, b, 0, 3, k, j, i);
        const double lw = 0.5, rw = 0.5;
        const double bc1 = lw * A.b1[f1idx(m, b, k, j, i)] + rw * A.b1[f1idx(m, b, k, j, i + 1)];
        const double bc2 = lw * A.b2[f2idx(m, b, k, j, i)] + rw * A.b2[f2idx(m, b, k, j + 1, i)];
        const double bc3 = lw * A.b3[f3idx(m, b, k, j, i)] + rw * A.b3[f3idx(m, b, k + 1, j, i)];
        A.bcc[cb] = (Real)bc1;
        A.bcc[cb + vs] = (Real)bc2;
        A.bcc[cb + 2 * vs] = (Real)bc3;
        using Acc = Real;   // U(W) in the bulk precision
        const Acc igm1 = Acc(1) / (Acc)(m.gamma - 1.0);
        const Acc w_d = A.w[c], w_vx = A.w[c + vs], w_vy = A.w[c + 2 * vs],
                  w_vz = A.w[c + 3 * vs], w_p = A.w[c + 4 * vs];
        // the FP32 path's cell-centred field is the FP32 rounding of the FP64 average
        const Acc b1c = A.bcc[cb], b2c = A.bcc[cb + vs], b3c = A.bcc[cb + 2 * vs];
        A.u[c] = (Real)w_d;
        A.u[c + vs] = (Real)(w_vx * w_d);
        A.u[c + 2 * vs] = (Real)(w_vy * w_d);
        A.u[c + 3 * vs] = (Real)(w_vz * w_d);
        A.u[c + 4 * vs] = (Real)(w_p * igm1 + Acc(0.5) * (w_d * (w_vx * w_vx + w_vy * w_vy +
                                                                 w_vz * w_vz) +
                                                          (b1c * b1c + b2c * b2c + b3c * b3c)));
        break;
      }
      default:
        break;
    }
  }
}

// the operation codes of one list: 0 the restriction list (RESTRICT_U/B), 1 the exchange
// list (COPY_U/B), 2 any code (ProlongateBoundaries, the regrid); the first two compile to
// small kernels (few registers, high occupancy)
template <typename Real, int LIST>
__device__ __forceinline__ void ml_op(const DevMesh& m, const MlArrays<Real>& A, int b,
                                      const MlOp& op, int t0, int dt) {
  if (LIST == 0) {
    if (op.code == ML_RESTRICT_U) ml_op_code<Real, ML_RESTRICT_U>(m, A, b, op, t0, dt);
    else if (op.code == ML_RESTRICT_B) ml_op_code<Real, ML_RESTRICT_B>(m, A, b, op, t0, dt);
    return;
  }
  if (LIST == 1) {
    if (op.code == ML_COPY_U) ml_op_code<Real, ML_COPY_U>(m, A, b, op, t0, dt);
    else if (op.code == ML_COPY_B) ml_op_code<Real, ML_COPY_B>(m, A, b, op, t0, dt);
    return;
  }
  switch (op.code) {
    case ML_COPY_U: ml_op_code<Real, ML_COPY_U>(m, A, b, op, t0, dt); break;
    case ML_COPY_B: ml_op_code<Real, ML_COPY_B>(m, A, b, op, t0, dt); break;
    case ML_RESTRICT_U: ml_op_code<Real, ML_RESTRICT_U>(m, A, b, op, t0, dt); break;
    case ML_RESTRICT_B: ml_op_code<Real, ML_RESTRICT_B>(m, A, b, op, t0, dt); break;
    case ML_C2P_COARSE: ml_op_code<Real, ML_C2P_COARSE>(m, A, b, op, t0, dt); break;
    case ML_BC_COARSE: ml_op_code<Real, ML_BC_COARSE>(m, A, b, op, t0, dt); break;
    case ML_PROLONG_U: ml_op_code<Real, ML_PROLONG_U>(m, A, b, op, t0, dt); break;
    case ML_PROLONG_SHARED: ml_op_code<Real, ML_PROLONG_SHARED>(m, A, b, op, t0, dt); break;
    case ML_PROLONG_INTERNAL: ml_op_code<Real, ML_PROLONG_INTERNAL>(m, A, b, op, t0, dt); break;
    case ML_FINE_P2C: ml_op_code<Real, ML_FINE_P2C>(m, A, b, op, t0, dt); break;
    default: break;
  }
}

// One CTA per block.  The restriction and exchange lists (LIST 0, 1: many small
// operations) give each operation of a barrier-free run to one warp (lanes over its
// elements); ProlongateBoundaries (LIST 2: larger, mostly dependent operations) spreads
// every operation over the whole CTA.  A barrier closes each run.
template <typename Real, int LIST>
__global__ void __launch_bounds__(128, LIST == 2 ? 4 : 1)
ml_ops_kernel(DevMesh m, MlArrays<Real> A, const MlOp* __restrict__ ops,
              const int* __restrict__ off, const int* __restrict__ blk) {
  const int b = blk[blockIdx.x];
  const int qe = off[blockIdx.x + 1];
  if (LIST == 2) {
    for (int q = off[blockIdx.x]; q < qe; ++q) {
      const MlOp op = ops[q];
      ml_op<Real, LIST>(m, A, b, op, threadIdx.x, blockDim.x);
      // the flag is the same for every thread of the CTA
      if (!op.nosync) __syncthreads();
    }
    return;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
  int q = off[blockIdx.x];
  while (q < qe) {
    int r = q;   // the run: q .. r (r the first operation followed by a barrier)
    while (r < qe - 1 && ops[r].nosync) ++r;
    for (int p = q + warp; p <= r; p += nwarps) {
      const MlOp op = ops[p];
      ml_op<Real, LIST>(m, A, b, op, lane, 32);
    }
    __syncthreads();
    q = r + 1;
  }
}

// ---- hydro flux correction ----------------------------------------------------------
// The x-direction hydro flux through face (k, j, i) (face index along DIR) of block b,
// exactly as the sweeps form it: reconstruction of the two adjacent cells and the
// Riemann solver; no EMF or weight is stored.
template <typename Real, int DIR, int ORDER, int RS>
__device__ __forceinline__ void face_flux(const DevMesh& m, const Real* __restrict__ w,
                                          const Real* __restrict__ bcc,
                                          const double* __restrict__ bn, int b, int k,
                                          int j, int i, Real* fn) {
  Real lp[NWAVE], lm[NWAVE], rp[NWAVE], rm[NWAVE];
  recon_cell<Real, DIR, ORDER>(m, w, bcc, b, k - (DIR == 2), j - (DIR == 1), i - (DIR == 0),
                               lp, lm);
  recon_cell<Real, DIR, ORDER>(m, w, bcc, b, k, j, i, rp, rm);
  const i64 fo = DIR == 0 ? f1idx(m, b, k, j, i) : DIR == 1 ? f2idx(m, b, k, j, i)
                                                            : f3idx(m, b, k, j, i);
  const int ivx = IVX + DIR, ivy = IVX + (DIR + 1) % 3, ivz = IVX + (DIR + 2) % 3;
  Real wli[NWAVE] = {lp[IDN], lp[ivx], lp[ivy], lp[ivz], lp[IPR], lp[IBY], lp[IBZ]};
  Real wri[NWAVE] = {rm[IDN], rm[ivx], rm[ivy], rm[ivz], rm[IPR], rm[IBY], rm[IBZ]};
  Real f[NWAVE];
  const Real gam = rgamma(m, Real());
  const Real bx = to_real(__ldg(bn + fo), Real());
  // the solver the sweep of that direction runs (FP32 HLLD / HLLE: packed, but for the
  // donor-cell x3 sweep), so that both sides of a coarse/fine face use the same fluxes bit
  // for bit
  constexpr bool PK = sizeof(Real) == 4 && !(DIR == 2 && ORDER == 1);
  if constexpr (RS == 0 && PK) hlld_pk(gam, wli, wri, bx, f);
  else if constexpr (RS == 1 && PK) hlle_pk(gam, wli, wri, bx, f);
  else if (RS == 0) hlld<Real>(gam, wli, wri, bx, f);
  else if (RS == 3) llf<Real>(gam, wli, wri, bx, f);
  else if (RS == 4) roe<Real>(gam, wli, wri, bx, f);
  else hlle<Real>(gam, wli, wri, bx, f);
  fn[IDN] = f[0];
  fn[ivx] = f[1];
  fn[ivy] = f[2];
  fn[ivz] = f[3];
  fn[IPR] = f[4];
}

// One thread per (correction task, coarse face point): the four finer-block fluxes on the
// fine faces inside the coarse face, area-weighted (LoadFluxBoundaryBufferToCoarser,
// flux_correction_cc.cpp:54-140).  Task t = (coarse block, finer block, face, fi1, fi2).
// Output: fcorr[coarse block][face][transverse index of the coarse face][5].
template <typename Real, int ORDER, int RS>
__global__ void __launch_bounds__(128)
ml_fine_flux_kernel(DevMesh m, const int4* __restrict__ tasks, int ntasks,
                    const Real* __restrict__ w, const Real* __restrict__ bcc,
                    const double* __restrict__ b1, const double* __restrict__ b2,
                    const double* __restrict__ b3) {
  const int per = m.ml.nfmax / 4;  // coarse face points of one quarter face (upper bound)
  const i64 t = (i64)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (i64)ntasks * per) return;
  const int4 tk = tasks[t / per];
  const int q = (int)(t % per);
  const int cb = tk.x, fbk = tk.y, fid = tk.z & 7, fi1 = (tk.z >> 4) & 1, fi2 = (tk.z >> 5) & 1;
  const int ax = fid >> 1;
  const int ta = ax == 0 ? 1 : 0, tb = ax == 2 ? 1 : 2;   // transverse axes
  const int nxs[3] = {m.nx1, m.nx2, m.nx3};
  const int na = nxs[ta] / 2, nbn = nxs[tb] / 2;
  if (q >= na * nbn) return;
  const int pa = q % na, pb = q / na;             // position in the quarter
  const int lo[3] = {m.is, m.js, m.ks};
  // coarse face position (transverse indices) and the fine face plane
  const int ca = lo[ta] + (fi1 ? nxs[ta] / 2 : 0) + pa;
  const int cbq = lo[tb] + (fi2 ? nxs[tb] / 2 : 0) + pb;
  const int hi_ax = (ax == 0 ? m.ie : ax == 1 ? m.je : m.ke);
  const int ffp = (fid & 1) ? lo[ax] : hi_ax + 1;   // the finer block's face facing me
  const int fa = lo[ta] + 2 * pa, fbb = lo[tb] + 2 * pb;
  const double* dxs[3] = {m.dx1f + (i64)fbk * m.nc1, m.dx2f + (i64)fbk * m.nc2,
                          m.dx3f + (i64)fbk * m.nc3};
  Real F[2][2][NHYDRO];
  for (int ob = 0; ob < 2; ++ob)
    for (int oa = 0; oa < 2; ++oa) {
      int p[3];
      p[ax] = ffp;
      p[ta] = fa + oa;
      p[tb] = fbb + ob;
      if (ax == 0) {
        if (ORDER == 1) face_flux<Real, 0, 1, RS>(m, w, bcc, b1, fbk, p[2], p[1], p[0], F[ob][oa]);
        else if (ORDER == 2) face_flux<Real, 0, 2, RS>(m, w, bcc, b1, fbk, p[2], p[1], p[0], F[ob][oa]);
        else face_flux<Real, 0, ORDER, RS>(m, w, bcc, b1, fbk, p[2], p[1], p[0], F[ob][oa]);
      } else if (ax == 1) {
        if (ORDER == 1) face_flux<Real, 1, 1, RS>(m, w, bcc, b2, fbk, p[2], p[1], p[0], F[ob][oa]);
        else if (ORDER == 2) face_flux<Real, 1, 2, RS>(m, w, bcc, b2, fbk, p[2], p[1], p[0], F[ob][oa]);
        else face_flux<Real, 1, ORDER, RS>(m, w, bcc, b2, fbk, p[2], p[1], p[0], F[ob][oa]);
      } else {
        if (ORDER == 1) face_flux<Real, 2, 1, RS>(m, w, bcc, b3, fbk, p[2], p[1], p[0], F[ob][oa]);
        else if (ORDER == 2) face_flux<Real, 2, 2, RS>(m, w, bcc, b3, fbk, p[2], p[1], p[0], F[ob][oa]);
        else face_flux<Real, 2, ORDER, RS>(m, w, bcc, b3, fbk, p[2], p[1], p[0], F[ob][oa]);
      }
    }
  // areas of the four fine faces, in the bulk precision (as the coarse block's own
  // Cartesian areas)
  const Real* rdxs[3] = {rdx(m, 0, Real()) + (i64)fbk * m.nc1, rdx(m, 1, Real()) + (i64)fbk * m.nc2,
                         rdx(m, 2, Real()) + (i64)fbk * m.nc3};
  (void)dxs;
  Real ar[2][2];
  for (int ob = 0; ob < 2; ++ob)
    for (int oa = 0; oa < 2; ++oa) {
      // Face1Area = dx2 dx3 (j, k), Face2Area = dx1 dx3 (i, k), Face3Area = dx1 dx2 (i, j)
      ar[ob][oa] = rdxs[ta][fa + oa] * rdxs[tb][fbb + ob];
    }
  // x1 faces pack (k, j) with area order (k,j),(k,j+1),(k+1,j),(k+1,j+1): oa runs along
  // j (ta = 1), ob along k (tb = 2); x2 faces (k, i): oa along i, ob along k; x3 faces
  // (j, i): oa along i, ob along j -- the reference's term order is (ob, oa) row-major
  const Real tarea = ar[0][0] + ar[0][1] + ar[1][0] + ar[1][1];
  Real* out = (Real*)m.ml.fcorr + (((i64)cb * 6 + fid) * m.ml.nfmax +
                                   (i64)(cbq - lo[tb]) * nxs[ta] + (ca - lo[ta])) * NHYDRO;
  for (int n = 0; n < NHYDRO; ++n)
    out[n] = (F[0][0][n] * ar[0][0] + F[0][1][n] * ar[0][1] + F[1][0][n] * ar[1][0] +
              F[1][1][n] * ar[1][1]) / tarea;
}

// ---- EMF correction across levels ---------------------------------------------------
template <typename Real>
__device__ __forceinline__ void ml_emf_position(const DevMesh& m, const Real* __restrict__ e1,
                                                const Real* __restrict__ e2,
                                                const Real* __restrict__ e3, int b, int c,
                                                int k, int j, int i, const int* nt, int nn,
                                                const int* s_lev, const int* s_ef,
                                                const int* s_nf) {
  const int nx1 = m.nx1, nx2 = m.nx2, nx3 = m.nx3;
  const int p3[3] = {i, j, k};
  const int lo[3] = {m.is, m.js, m.ks}, hi[3] = {m.ie + 1, m.je + 1, m.ke + 1};
  // faces this position lies on: along the two axes other than c
  int onf[3] = {0, 0, 0};  // -1 / +1 / 0 per axis
  for (int a = 0; a < 3; ++a) {
    if (a == c) continue;
    onf[a] = (p3[a] == lo[a]) ? -1 : (p3[a] == hi[a]) ? 1 : 0;
  }
  if (onf[0] == 0 && onf[1] == 0 && onf[2] == 0) return;
  const Real* E = c == 0 ? e1 : c == 1 ? e2 : e3;
  auto eidx = [&](int bb, int kk, int jj, int ii) -> i64 {
    return c == 0 ? e1idx(m, bb, kk, jj, ii) : c == 1 ? e2idx(m, bb, kk, jj, ii)
                                                      : e3idx(m, bb, kk, jj, ii);
  };
  const DevML& L = m.ml;
  const int lev = __ldg(L.level + b);
  // the block edge this position lies on (both transverse offsets nonzero), and its eid
  const int ta = c == 0 ? 1 : 0, tb = c == 2 ? 1 : 2;   // transverse axes, ta < tb
  const bool on_edge = onf[ta] != 0 && onf[tb] != 0;
  int eid = -1;
  if (on_edge) {
    const int base = c == 2 ? 0 : c == 1 ? 4 : 8;
    eid = base + (((onf[ta] + 1) >> 1) | ((onf[tb] + 1) & 2));
  }
  Real val = E[eidx(b, k, j, i)];
  // same level
  for (int q = 0; q < nn; ++q) {
    const int* e = nt + q * 10;
    const int type = e[5];
    if (type != 0 && type != 1) break;
    if (e[1] != lev) continue;
    const int o[3] = {e[2], e[3], e[4]};
    if (type == 0) {
      const int a = e[8] >> 1;
      if (a == c || onf[a] != o[a]) continue;   // not on this face
      int s3[3] = {i, j, k};
      s3[a] = o[a] > 0 ? lo[a] : hi[a];          // the neighbour's face facing me
      val += E[eidx(e[0], s3[2], s3[1], s3[0])];
    } else {
      if (!on_edge || e[9] != eid || !s_ef[eid]) continue;
      int s3[3] = {i, j, k};
      s3[ta] = o[ta] > 0 ? lo[ta] : hi[ta];
      s3[tb] = o[tb] > 0 ? lo[tb] : hi[tb];
      val += E[eidx(e[0], s3[2], s3[1], s3[0])];
    }
  }
  // ClearCoarseFluxBoundary
  bool cleared = false;
  for (int a = 0; a < 3; ++a) {
    if (a == c || onf[a] == 0) continue;
    int o[3] = {0, 0, 0};
    o[a] = onf[a];
    if ((s_lev[(o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1)]) <= lev)
      continue;
    // the face-interior range of component c on face a (block edges excluded)
    bool inside = true;
    for (int q = 0; q < 3; ++q)
      if (q != a && q != c && (p3[q] == lo[q] || p3[q] == hi[q])) inside = false;
    if (inside) cleared = true;
  }
  if (on_edge && !s_ef[eid]) cleared = true;
  if (cleared) val = Real(0);
  // finer blocks
  const double* fdx[3];
  for (int q = 0; q < nn; ++q) {
    const int* e = nt + q * 10;
    const int type = e[5];
    if (type != 0 && type != 1) break;
    if (e[1] != lev + 1) continue;
    const int s = e[0];
    const int o[3] = {e[2], e[3], e[4]};
    const int fi1 = e[6], fi2 = e[7];
    fdx[0] = m.dx1f + (i64)s * m.nc1;
    fdx[1] = m.dx2f + (i64)s * m.nc2;
    fdx[2] = m.dx3f + (i64)s * m.nc3;
    const int nxs[3] = {nx1, nx2, nx3};
    if (type == 0) {
      const int a = e[8] >> 1;
      if (a == c || onf[a] != o[a]) continue;
      // the two in-face axes: first (fi1) and second (fi2) in increasing axis order
      const int f1ax = a == 0 ? 1 : 0, f2ax = a == 2 ? 1 : 2;
      int l3[3], u3[3];   // the quarter of my face (cell ranges along in-face axes)
      l3[f1ax] = lo[f1ax] + (fi1 ? nxs[f1ax] / 2 : 0);
      u3[f1ax] = fi1 ? hi[f1ax] - 1 : lo[f1ax] + nxs[f1ax] / 2 - 1;
      l3[f2ax] = lo[f2ax] + (fi2 ? nxs[f2ax] / 2 : 0);
      u3[f2ax] = fi2 ? hi[f2ax] - 1 : lo[f2ax] + nxs[f2ax] / 2 - 1;
      // component c runs along axis c (a cell range), the other in-face axis is a face
      // range (one more)
      const int other = (f1ax == c) ? f2ax : f1ax;
      if (p3[c] < l3[c] || p3[c] > u3[c]) continue;
      if (p3[other] < l3[other] || p3[other] > u3[other] + 1) continue;
      int s3[3];
      s3[a] = o[a] > 0 ? lo[a] : hi[a];
      s3[c] = lo[c] + 2 * (p3[c] - l3[c]);
      s3[other] = lo[other] + 2 * (p3[other] - l3[other]);
      // restriction along c: (e(x) l(x) + e(x+1) l(x+1)) / (l(x) + l(x+1))
      int s3p[3] = {s3[0], s3[1], s3[2]};
      s3p[c] += 1;
      const double l1 = fdx[c][s3[c]], l2 = fdx[c][s3[c] + 1];
      const Real v = (Real)((ldr(E + eidx(s, s3[2], s3[1], s3[0])) * l1 +
                             ldr(E + eidx(s, s3p[2], s3p[1], s3p[0])) * l2) / (l1 + l2));
      val += v;
    } else {
      if (!on_edge || e[9] != eid) continue;
      int l = lo[c] + (fi1 ? nxs[c] / 2 : 0);
      int u = fi1 ? hi[c] - 1 : lo[c] + nxs[c] / 2 - 1;
      if (p3[c] < l || p3[c] > u) continue;
      int s3[3];
      s3[ta] = o[ta] > 0 ? lo[ta] : hi[ta];
      s3[tb] = o[tb] > 0 ? lo[tb] : hi[tb];
      s3[c] = lo[c] + 2 * (p3[c] - l);
      int s3p[3] = {s3[0], s3[1], s3[2]};
      s3p[c] += 1;
      const double l1 = fdx[c][s3[c]], l2 = fdx[c][s3[c] + 1];
      const Real v = (Real)((ldr(E + eidx(s, s3[2], s3[1], s3[0])) * l1 +
                             ldr(E + eidx(s, s3p[2], s3p[1], s3p[0])) * l2) / (l1 + l2));
      val += v;
    }
  }
  // AverageFluxBoundary
  if (on_edge) {
    const int nf = s_nf[eid];
    if (nf != 1) val *= (Real)(1.0 / (double)nf);
  } else {
    // the one face this position lies on
    int a = -1;
    for (int q = 0; q < 3; ++q)
      if (q != c && onf[q] != 0) a = q;
    int o[3] = {0, 0, 0};
    o[a] = onf[a];
    const int nl = (s_lev[(o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1)]);
    if (nl == lev) {
      val *= Real(0.5);
    } else if (nl > lev) {
      const int other = 3 - a - c;  // the in-face axis that is not c
      const int nxs[3] = {nx1, nx2, nx3};
      if (p3[other] == lo[other] + nxs[other] / 2) val *= Real(0.5);
    }
  }
  Real* out = (Real*)(c == 0 ? L.ecorr1 : c == 1 ? L.ecorr2 : L.ecorr3);
  out[eidx(b, k, j, i)] = val;
}

// Grid (blocks, position chunks): the CTAs of block blockIdx.x stage its neighbour list
// and levels in shared memory; a thread takes edge positions on the block boundary (for
// component c, the positions with a transverse index on the block's first or last face).
// Same-level contributions in neighbour-list order, clearing of the positions shared with
// finer blocks, the finer blocks' restricted values in list order, then the averaging
// (flux_correction_fc.cpp:689-1545).
__host__ __device__ __forceinline__ i64 ml_emf_positions(const DevMesh& m) {
  // per component c: nx_c cells times the perimeter 2 (nx_ta + nx_tb) of the transverse
  // rectangle of (nx_ta + 1) x (nx_tb + 1) positions
  return (i64)m.nx1 * 2 * (m.nx2 + m.nx3) + (i64)m.nx2 * 2 * (m.nx1 + m.nx3) +
         (i64)m.nx3 * 2 * (m.nx1 + m.nx2);
}

// The corrected EMFs into the edge arrays themselves, at the same positions, once every
// correction is formed (ml_emf_kernel reads the neighbours' uncorrected values): CT then
// reads plain edges on a multi-level mesh as on a uniform one.
template <typename Real>
__global__ void __launch_bounds__(128)
ml_emf_put_kernel(DevMesh m, Real* __restrict__ e1, Real* __restrict__ e2,
                  Real* __restrict__ e3) {
  const int nx1 = m.nx1, nx2 = m.nx2, nx3 = m.nx3;
  const int b = blockIdx.x;
  const DevML& L = m.ml;
  const i64 npos = ml_emf_positions(m);
  for (i64 r0 = (i64)blockIdx.y * blockDim.x + threadIdx.x; r0 < npos;
       r0 += (i64)gridDim.y * blockDim.x) {
    // the position's component c and (k, j, i), as in ml_emf_kernel
    const int nxs[3] = {nx1, nx2, nx3};
    int c = 0;
    i64 r = r0;
    for (; c < 2; ++c) {
      const int ta_ = c == 0 ? 1 : 0, tb_ = c == 2 ? 1 : 2;
      const i64 nc = (i64)nxs[c] * 2 * (nxs[ta_] + nxs[tb_]);
      if (r < nc) break;
      r -= nc;
    }
    const int ta0 = c == 0 ? 1 : 0, tb0 = c == 2 ? 1 : 2;
    const int na = nxs[ta0], nbt = nxs[tb0];
    const int per = 2 * (na + nbt);
    const int pc = (int)(r / per);
    int pr = (int)(r % per), pa, pb;
    if (pr < na + 1) { pa = pr; pb = 0; }
    else if ((pr -= na + 1) < na + 1) { pa = pr; pb = nbt; }
    else { pr -= na + 1; pa = (pr & 1) ? na : 0; pb = 1 + (pr >> 1); }
    int q3[3];
    q3[c] = pc;
    q3[ta0] = pa;
    q3[tb0] = pb;
    const int i = m.is + q3[0], j = m.js + q3[1], k = m.ks + q3[2];
    const i64 idx = c == 0 ? e1idx(m, b, k, j, i) : c == 1 ? e2idx(m, b, k, j, i)
                                                           : e3idx(m, b, k, j, i);
    const Real* ec = (const Real*)(c == 0 ? L.ecorr1 : c == 1 ? L.ecorr2 : L.ecorr3);
    Real* e = c == 0 ? e1 : c == 1 ? e2 : e3;
    e[idx] = ec[idx];
  }
}

template <typename Real>
__global__ void __launch_bounds__(128)
ml_emf_kernel(DevMesh m, const Real* __restrict__ e1, const Real* __restrict__ e2,
              const Real* __restrict__ e3) {
  const int nx1 = m.nx1, nx2 = m.nx2, nx3 = m.nx3;
  const int b = blockIdx.x;
  __shared__ int s_nt[56 * 10];
  __shared__ int s_lev[27];
  __shared__ int s_ef[12], s_nf[12];
  const DevML& L = m.ml;
  const int nn = __ldg(L.nnbr + b);
  for (int q = threadIdx.x; q < nn * 10; q += blockDim.x) s_nt[q] = __ldg(L.nbrt + (i64)b * 560 + q);
  if (threadIdx.x < 27) s_lev[threadIdx.x] = __ldg(L.nblev + (i64)b * 27 + threadIdx.x);
  if (threadIdx.x < 12) {
    s_ef[threadIdx.x] = __ldg(L.eflag + b * 12 + threadIdx.x);
    s_nf[threadIdx.x] = __ldg(L.nfine + b * 12 + threadIdx.x);
  }
  __syncthreads();
  const i64 npos = ml_emf_positions(m);
  for (i64 r0 = (i64)blockIdx.y * blockDim.x + threadIdx.x; r0 < npos;
       r0 += (i64)gridDim.y * blockDim.x) {
    // component c, cell index along c, perimeter index of the transverse rectangle
    const int nxs[3] = {nx1, nx2, nx3};
    int c = 0;
    i64 r = r0;
    for (; c < 2; ++c) {
      const int ta_ = c == 0 ? 1 : 0, tb_ = c == 2 ? 1 : 2;
      const i64 nc = (i64)nxs[c] * 2 * (nxs[ta_] + nxs[tb_]);
      if (r < nc) break;
      r -= nc;
    }
    const int ta0 = c == 0 ? 1 : 0, tb0 = c == 2 ? 1 : 2;
    const int na = nxs[ta0], nbt = nxs[tb0];
    const int per = 2 * (na + nbt);
    const int pc = (int)(r / per);
    int pr = (int)(r % per), pa, pb;
    if (pr < na + 1) { pa = pr; pb = 0; }
    else if ((pr -= na + 1) < na + 1) { pa = pr; pb = nbt; }
    else { pr -= na + 1; pa = (pr & 1) ? na : 0; pb = 1 + (pr >> 1); }
    int q3[3];
    q3[c] = pc;
    q3[ta0] = pa;
    q3[tb0] = pb;
    const int i = m.is + q3[0], j = m.js + q3[1], k = m.ks + q3[2];
    ml_emf_position<Real>(m, e1, e2, e3, b, c, k, j, i, s_nt, nn, s_lev, s_ef, s_nf);
  }
}


}  // namespace athgpu
