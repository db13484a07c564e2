// Host planner of the multi-level stage: from the neighbour lists of all MeshBlocks it
// builds the per-block operation lists that ml_ops_kernel executes (restriction for
// coarser neighbours, the ghost exchange, ProlongateBoundaries), the flux-correction
// tasks of ml_fine_flux_kernel and the per-block edge tables of ml_emf_kernel.
//
// The index ranges follow the reference's buffer functions, stated per axis:
// CellCenteredBoundaryVariable (bvals/cc/bvals_cc.cpp:252-540), FaceCenteredBoundary-
// Variable (bvals/fc/bvals_fc.cpp:344-973), BoundaryValues::ProlongateBoundaries and its
// helpers (bvals/bvals_refine.cpp:97-637), FaceCenteredBoundaryVariable::CountFineEdges
// (bvals/fc/bvals_fc.cpp:1129-1196).  A transfer copies a source box to a destination box
// of the same shape element by element in (k, j, i) order, which is the order the
// reference packs and unpacks its buffers.
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ml_plan.h"

namespace athgpu {
namespace {

struct Box {
  int s[3], e[3];
};

struct Ix {
  int lo[3], hi[3];    // fine interior (is..ie, ...)
  int clo[3], chi[3];  // coarse interior
  int n[3];            // nx1, nx2, nx3
  int ng, cng;
};

void off3(const MlNbr& q, int o[3]) { o[0] = q.ox1; o[1] = q.ox2; o[2] = q.ox3; }

// the fine-block offset that selects the half of axis a (a has offset 0)
int half_sel(const MlNbr& q, int a) {
  if (a == 0) return q.fi1;
  if (a == 1) return q.ox1 != 0 ? q.fi1 : q.fi2;
  return (q.ox1 != 0 && q.ox2 != 0) ? q.fi1 : q.fi2;
}

// ---- cell-centred (U) regions ----
Box cc_send_same(const Ix& x, const MlNbr& q) {  // LoadBoundaryBufferSameLevel
  Box r; int o[3]; off3(q, o);
  for (int a = 0; a < 3; ++a) {
    r.s[a] = (o[a] > 0) ? x.hi[a] - x.ng + 1 : x.lo[a];
    r.e[a] = (o[a] < 0) ? x.lo[a] + x.ng - 1 : x.hi[a];
  }
  return r;
}
Box cc_recv_same(const Ix& x, const MlNbr& q) {  // SetBoundarySameLevel
  Box r; int o[3]; off3(q, o);
  for (int a = 0; a < 3; ++a) {
    if (o[a] == 0) { r.s[a] = x.lo[a]; r.e[a] = x.hi[a]; }
    else if (o[a] > 0) { r.s[a] = x.hi[a] + 1; r.e[a] = x.hi[a] + x.ng; }
    else { r.s[a] = x.lo[a] - x.ng; r.e[a] = x.lo[a] - 1; }
  }
  return r;
}
Box cc_send_coarser(const Ix& x, const MlNbr& q) {  // LoadBoundaryBufferToCoarser
  Box r; int o[3]; off3(q, o);
  const int cn = x.ng - 1;
  for (int a = 0; a < 3; ++a) {
    r.s[a] = (o[a] > 0) ? x.chi[a] - cn : x.clo[a];
    r.e[a] = (o[a] < 0) ? x.clo[a] + cn : x.chi[a];
  }
  return r;
}
Box cc_recv_finer(const Ix& x, const MlNbr& q) {  // SetBoundaryFromFiner
  Box r; int o[3]; off3(q, o);
  for (int a = 0; a < 3; ++a) {
    if (o[a] == 0) {
      r.s[a] = x.lo[a]; r.e[a] = x.hi[a];
      if (half_sel(q, a) == 1) r.s[a] += x.n[a] / 2; else r.e[a] -= x.n[a] / 2;
    } else if (o[a] > 0) { r.s[a] = x.hi[a] + 1; r.e[a] = x.hi[a] + x.ng; }
    else { r.s[a] = x.lo[a] - x.ng; r.e[a] = x.lo[a] - 1; }
  }
  return r;
}
Box cc_send_finer(const Ix& x, const MlNbr& q) {  // LoadBoundaryBufferToFiner
  Box r; int o[3]; off3(q, o);
  const int cn = x.cng - 1;
  for (int a = 0; a < 3; ++a) {
    r.s[a] = (o[a] > 0) ? x.hi[a] - cn : x.lo[a];
    r.e[a] = (o[a] < 0) ? x.lo[a] + cn : x.hi[a];
    if (o[a] == 0) {
      if (half_sel(q, a) == 1) r.s[a] += x.n[a] / 2 - x.cng;
      else r.e[a] -= x.n[a] / 2 - x.cng;
    }
  }
  return r;
}
Box cc_recv_coarser(const Ix& x, const MlNbr& q, const int par[3]) {  // SetBoundaryFromCoarser
  Box r; int o[3]; off3(q, o);
  for (int a = 0; a < 3; ++a) {
    if (o[a] == 0) {
      r.s[a] = x.clo[a]; r.e[a] = x.chi[a];
      if (par[a] == 0) r.e[a] += x.cng; else r.s[a] -= x.cng;
    } else if (o[a] > 0) { r.s[a] = x.chi[a] + 1; r.e[a] = x.chi[a] + x.cng; }
    else { r.s[a] = x.clo[a] - x.cng; r.e[a] = x.clo[a] - 1; }
  }
  return r;
}

// ---- face-field regions, component d (axis d runs over faces) ----
Box fc_send_same(const Ix& x, const MlNbr& q, int d) {
  Box r; int o[3]; off3(q, o);
  const int ng = x.ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) { r.s[a] = x.lo[a]; r.e[a] = x.hi[a] + 1; }
      else if (o[a] > 0) { r.s[a] = x.hi[a] - ng + 1; r.e[a] = x.hi[a]; }
      else { r.s[a] = x.lo[a] + 1; r.e[a] = x.lo[a] + ng; }
      if (q.type != ML_FACE) {  // the overlapping face of edges and corners
        if (o[a] > 0) r.e[a]++;
        else if (o[a] < 0) r.s[a]--;
      }
    } else {
      if (o[a] == 0) { r.s[a] = x.lo[a]; r.e[a] = x.hi[a]; }
      else if (o[a] > 0) { r.s[a] = x.hi[a] - ng + 1; r.e[a] = x.hi[a]; }
      else { r.s[a] = x.lo[a]; r.e[a] = x.lo[a] + ng - 1; }
    }
  }
  return r;
}
Box fc_recv_same(const Ix& x, const MlNbr& q, int d) {
  Box r; int o[3]; off3(q, o);
  const int ng = x.ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) { r.s[a] = x.lo[a]; r.e[a] = x.hi[a] + 1; }
      else if (o[a] > 0) { r.s[a] = x.hi[a] + 2; r.e[a] = x.hi[a] + ng + 1; }
      else { r.s[a] = x.lo[a] - ng; r.e[a] = x.lo[a] - 1; }
      if (q.type != ML_FACE) {
        if (o[a] > 0) r.s[a]--;
        else if (o[a] < 0) r.e[a]++;
      }
    } else {
      if (o[a] == 0) { r.s[a] = x.lo[a]; r.e[a] = x.hi[a]; }
      else if (o[a] > 0) { r.s[a] = x.hi[a] + 1; r.e[a] = x.hi[a] + ng; }
      else { r.s[a] = x.lo[a] - ng; r.e[a] = x.lo[a] - 1; }
    }
  }
  return r;
}
Box fc_send_coarser(const Ix& x, const MlNbr& q, int d) {  // ghost width NGHOST
  Box r; int o[3]; off3(q, o);
  const int cg = x.ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) { r.s[a] = x.clo[a]; r.e[a] = x.chi[a] + 1; }
      else if (o[a] > 0) { r.s[a] = x.chi[a] - cg + 1; r.e[a] = x.chi[a]; }
      else { r.s[a] = x.clo[a] + 1; r.e[a] = x.clo[a] + cg; }
      if (q.type != ML_FACE) {
        if (o[a] > 0) r.e[a]++;
        else if (o[a] < 0) r.s[a]--;
      }
    } else {
      if (o[a] == 0) { r.s[a] = x.clo[a]; r.e[a] = x.chi[a]; }
      else if (o[a] > 0) { r.s[a] = x.chi[a] - cg + 1; r.e[a] = x.chi[a]; }
      else { r.s[a] = x.clo[a]; r.e[a] = x.clo[a] + cg - 1; }
    }
  }
  return r;
}
Box fc_recv_finer(const Ix& x, const MlNbr& q, int d) {
  Box r; int o[3]; off3(q, o);
  const int ng = x.ng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) {
        r.s[a] = x.lo[a]; r.e[a] = x.hi[a] + 1;
        if (half_sel(q, a) == 1) r.s[a] += x.n[a] / 2; else r.e[a] -= x.n[a] / 2;
      } else if (o[a] > 0) { r.s[a] = x.hi[a] + 2; r.e[a] = x.hi[a] + ng + 1; }
      else { r.s[a] = x.lo[a] - ng; r.e[a] = x.lo[a] - 1; }
      if (q.type != ML_FACE) {
        if (o[a] > 0) r.s[a]--;
        else if (o[a] < 0) r.e[a]++;
      }
    } else {
      if (o[a] == 0) {
        r.s[a] = x.lo[a]; r.e[a] = x.hi[a];
        if (half_sel(q, a) == 1) r.s[a] += x.n[a] / 2; else r.e[a] -= x.n[a] / 2;
      } else if (o[a] > 0) { r.s[a] = x.hi[a] + 1; r.e[a] = x.hi[a] + ng; }
      else { r.s[a] = x.lo[a] - ng; r.e[a] = x.lo[a] - 1; }
    }
  }
  return r;
}
Box fc_send_finer(const Ix& x, const MlNbr& q, int d) {
  Box r; int o[3]; off3(q, o);
  const int cg = x.cng, cn = x.cng - 1;
  for (int a = 0; a < 3; ++a) {
    const int h = x.n[a] / 2 - cg;
    if (a == d) {
      if (o[a] == 0) {
        r.s[a] = x.lo[a]; r.e[a] = x.hi[a] + 1;
        if (half_sel(q, a) == 1) r.s[a] += h; else r.e[a] -= h;
      } else if (o[a] > 0) { r.s[a] = x.hi[a] + 1 - cg; r.e[a] = x.hi[a] + 1; }
      else { r.s[a] = x.lo[a]; r.e[a] = x.lo[a] + cg; }
    } else {
      if (o[a] == 0) {
        r.s[a] = x.lo[a]; r.e[a] = x.hi[a];
        if (half_sel(q, a) == 1) r.s[a] += h; else r.e[a] -= h;
      } else if (o[a] > 0) { r.s[a] = x.hi[a] - cn; r.e[a] = x.hi[a]; }
      else { r.s[a] = x.lo[a]; r.e[a] = x.lo[a] + cn; }
    }
  }
  return r;
}
Box fc_recv_coarser(const Ix& x, const MlNbr& q, int d, const int par[3]) {
  Box r; int o[3]; off3(q, o);
  const int cg = x.cng;
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      if (o[a] == 0) {
        r.s[a] = x.clo[a]; r.e[a] = x.chi[a] + 1;
        if (par[a] == 0) r.e[a] += cg; else r.s[a] -= cg;
      } else if (o[a] > 0) { r.s[a] = x.chi[a] + 1; r.e[a] = x.chi[a] + 1 + cg; }
      else { r.s[a] = x.clo[a] - cg; r.e[a] = x.clo[a]; }
    } else {
      if (o[a] == 0) {
        r.s[a] = x.clo[a]; r.e[a] = x.chi[a];
        if (par[a] == 0) r.e[a] += cg; else r.s[a] -= cg;
      } else if (o[a] > 0) { r.s[a] = x.chi[a] + 1; r.e[a] = x.chi[a] + cg; }
      else { r.s[a] = x.clo[a] - cg; r.e[a] = x.clo[a] - 1; }
    }
  }
  return r;
}

MlOp make_op(int code, int d, const Box& dst) {
  MlOp op{};
  op.code = code;
  op.d = d;
  for (int a = 0; a < 3; ++a) { op.s[a] = dst.s[a]; op.e[a] = dst.e[a]; }
  return op;
}
bool same_shape(const Box& a, const Box& b) {
  for (int q = 0; q < 3; ++q)
    if (a.e[q] - a.s[q] != b.e[q] - b.s[q]) return false;
  return true;
}
bool empty(const Box& a) {
  for (int q = 0; q < 3; ++q)
    if (a.e[q] < a.s[q]) return true;
  return false;
}

// Every array index an operation will touch, checked on the host before anything runs on
// the device (fine arrays: cells 0..nc-1, faces 0..nc along their own axis; coarse
// buffers: 0..ncc-1, 0..ncc).
struct Bounds {
  int nc[3], ncc[3];
  bool in(int lo, int hi, int n) const { return lo >= 0 && hi <= n - 1 && lo <= hi + 1; }
  bool cells(const int s[3], const int e[3], bool coarse, int pad) const {
    for (int a = 0; a < 3; ++a)
      if (!in(s[a] - pad, e[a] + pad, coarse ? ncc[a] : nc[a])) return false;
    return true;
  }
  bool faces(const int s[3], const int e[3], bool coarse, int d, int pad) const {
    for (int a = 0; a < 3; ++a) {
      const int n = (coarse ? ncc[a] : nc[a]) + (a == d ? 1 : 0);
      if (!in(s[a] - (a == d ? 0 : pad), e[a] + (a == d ? 0 : pad), n)) return false;
    }
    return true;
  }
};

bool check_op(const MlOp& op, const Ix& x, const Bounds& B) {
  int e2[3], s2[3], fe[3];
  for (int a = 0; a < 3; ++a) {
    s2[a] = op.o[a];
    e2[a] = op.o[a] + op.e[a] - op.s[a];
  }
  switch (op.code) {
    case ML_COPY_U:
      return B.cells(op.s, op.e, op.dst_kind == ML_COARSE, 0) &&
             B.cells(s2, e2, op.src_kind == ML_SEND, 0);
    case ML_COPY_B:
      return B.faces(op.s, op.e, op.dst_kind == ML_COARSE, op.d, 0) &&
             B.faces(s2, e2, op.src_kind == ML_SEND, op.d, 0);
    case ML_RESTRICT_U: {
      int fs[3];
      for (int a = 0; a < 3; ++a) {
        fs[a] = (op.s[a] - x.clo[a]) * 2 + x.lo[a];
        fe[a] = (op.e[a] - x.clo[a]) * 2 + x.lo[a] + 1;
      }
      return B.cells(op.s, op.e, true, 0) && B.cells(fs, fe, false, 0);
    }
    case ML_RESTRICT_B: {
      int fs[3];
      for (int a = 0; a < 3; ++a) {
        fs[a] = (op.s[a] - x.clo[a]) * 2 + x.lo[a];
        fe[a] = (op.e[a] - x.clo[a]) * 2 + x.lo[a] + (a == op.d ? 0 : 1);
      }
      return B.faces(op.s, op.e, true, op.d, 0) && B.faces(fs, fe, false, op.d, 0);
    }
    case ML_C2P_COARSE:
      return B.cells(op.s, op.e, true, 0);
    case ML_BC_COARSE: {
      const int f = op.aux & 7, a = f >> 1;
      int cs[3], ce[3];
      for (int q = 0; q < 3; ++q) {
        cs[q] = op.s[q];
        ce[q] = op.e[q] - (q == a ? 0 : 1);
      }
      cs[a] = x.clo[a] - x.ng;
      ce[a] = x.chi[a] + x.ng;
      if (!B.cells(cs, ce, true, 0)) return false;
      for (int d = 0; d < 3; ++d) {
        int fs[3] = {cs[0], cs[1], cs[2]}, fe2[3] = {ce[0], ce[1], ce[2]};
        if (d != a) fe2[d] += 1;
        else fe2[a] += 1;
        if (!B.faces(fs, fe2, true, d, 0)) return false;
      }
      return op.s[a] >= 1 && op.e[a] <= x.ng;
    }
    case ML_PROLONG_U: {
      int fs[3];
      for (int a = 0; a < 3; ++a) {
        fs[a] = (op.s[a] - x.clo[a]) * 2 + x.lo[a];
        fe[a] = (op.e[a] - x.clo[a]) * 2 + x.lo[a] + 1;
      }
      return B.cells(op.s, op.e, true, 1) && B.cells(fs, fe, false, 0);
    }
    case ML_PROLONG_SHARED: {
      int fs[3];
      for (int a = 0; a < 3; ++a) {
        fs[a] = (op.s[a] - x.clo[a]) * 2 + x.lo[a];
        fe[a] = (op.e[a] - x.clo[a]) * 2 + x.lo[a] + (a == op.d ? 0 : 1);
      }
      // the slopes read the transverse neighbours of the coarse face
      return B.faces(op.s, op.e, true, op.d, 1) && B.faces(fs, fe, false, op.d, 0);
    }
    case ML_PROLONG_INTERNAL: {
      int fs[3];
      for (int a = 0; a < 3; ++a) {
        fs[a] = (op.s[a] - x.clo[a]) * 2 + x.lo[a];
        fe[a] = (op.e[a] - x.clo[a]) * 2 + x.lo[a] + 2;   // faces fi .. fi+2
      }
      for (int d = 0; d < 3; ++d) {
        int fe2[3] = {fe[0] - 1, fe[1] - 1, fe[2] - 1};
        fe2[d] += 1;
        if (!B.faces(fs, fe2, false, d, 0)) return false;
      }
      return true;
    }
    case ML_FINE_P2C:
      return B.cells(op.s, op.e, false, 0) && op.e[0] + 1 <= B.nc[0] &&
             op.e[1] + 1 <= B.nc[1] && op.e[2] + 1 <= B.nc[2];
    default:
      return false;
  }
}

// ---- barriers between operations ------------------------------------------------------
// The arrays an operation reads and writes, as boxes of one block's array, so that runs of
// operations on disjoint data execute without a barrier between them.
enum RegArr {
  RA_U, RA_W, RA_BCC, RA_B1, RA_B2, RA_B3, RA_CU, RA_CW, RA_CBCC, RA_CB1, RA_CB2, RA_CB3,
  RA_SU, RA_SB1, RA_SB2, RA_SB3
};
struct Reg {
  int arr, blk, s[3], e[3];
};
bool overlap(const Reg& a, const Reg& b) {
  if (a.arr != b.arr || a.blk != b.blk) return false;
  for (int q = 0; q < 3; ++q)
    if (a.e[q] < b.s[q] || b.e[q] < a.s[q]) return false;
  return true;
}
Reg reg(int arr, int blk, const int s[3], const int e[3], int pad = 0) {
  Reg r;
  r.arr = arr;
  r.blk = blk;
  for (int q = 0; q < 3; ++q) { r.s[q] = s[q] - pad; r.e[q] = e[q] + pad; }
  return r;
}
// the fine box under a coarse box (extra: faces beyond the last cell)
void fine_of(const MlOp& op, const Ix& x, int extra, int fs[3], int fe[3]) {
  for (int a = 0; a < 3; ++a) {
    fs[a] = (op.s[a] - x.clo[a]) * 2 + x.lo[a];
    fe[a] = (op.e[a] - x.clo[a]) * 2 + x.lo[a] + 1 + extra;
  }
}
// conservative read and write sets of one operation of block b
void op_regions(const MlOp& op, int b, const Ix& x, std::vector<Reg>* rd, std::vector<Reg>* wr) {
  rd->clear();
  wr->clear();
  int fs[3], fe[3], os[3], oe[3];
  const int all_s[3] = {-1000, -1000, -1000}, all_e[3] = {1000, 1000, 1000};
  for (int a = 0; a < 3; ++a) {
    os[a] = op.o[a];
    oe[a] = op.o[a] + op.e[a] - op.s[a];
  }
  switch (op.code) {
    case ML_COPY_U:
      wr->push_back(reg(op.dst_kind == ML_COARSE ? RA_CU : RA_U, b, op.s, op.e));
      rd->push_back(reg(op.src_kind == ML_SEND ? RA_SU : RA_U, op.src, os, oe));
      break;
    case ML_COPY_B:
      wr->push_back(reg((op.dst_kind == ML_COARSE ? RA_CB1 : RA_B1) + op.d, b, op.s, op.e));
      rd->push_back(reg((op.src_kind == ML_SEND ? RA_SB1 : RA_B1) + op.d, op.src, os, oe));
      break;
    case ML_RESTRICT_U:
      wr->push_back(reg(RA_CU, b, op.s, op.e));
      if (op.src_kind == ML_SEND) wr->push_back(reg(RA_SU, b, op.s, op.e));
      fine_of(op, x, 0, fs, fe);
      rd->push_back(reg(RA_U, b, fs, fe));
      break;
    case ML_RESTRICT_B:
      wr->push_back(reg(RA_CB1 + op.d, b, op.s, op.e));
      if (op.src_kind == ML_SEND) wr->push_back(reg(RA_SB1 + op.d, b, op.s, op.e));
      fine_of(op, x, 0, fs, fe);
      rd->push_back(reg(RA_B1 + op.d, b, fs, fe));
      break;
    case ML_C2P_COARSE:
      wr->push_back(reg(RA_CU, b, op.s, op.e));
      wr->push_back(reg(RA_CW, b, op.s, op.e));
      wr->push_back(reg(RA_CBCC, b, op.s, op.e));
      rd->push_back(reg(RA_CU, b, op.s, op.e));
      for (int d = 0; d < 3; ++d) rd->push_back(reg(RA_CB1 + d, b, op.s, op.e, 1));
      break;
    case ML_PROLONG_U:
      rd->push_back(reg(op.src_kind == ML_COARSE ? RA_CU : RA_CW, b, op.s, op.e, 1));
      fine_of(op, x, 0, fs, fe);
      wr->push_back(reg(op.src_kind == ML_COARSE ? RA_U : RA_W, b, fs, fe));
      break;
    case ML_PROLONG_SHARED:
      rd->push_back(reg(RA_CB1 + op.d, b, op.s, op.e, 1));
      fine_of(op, x, 0, fs, fe);
      wr->push_back(reg(RA_B1 + op.d, b, fs, fe));
      break;
    case ML_PROLONG_INTERNAL:
      fine_of(op, x, 1, fs, fe);
      for (int d = 0; d < 3; ++d) {
        rd->push_back(reg(RA_B1 + d, b, fs, fe));
        wr->push_back(reg(RA_B1 + d, b, fs, fe));
      }
      break;
    case ML_FINE_P2C:
      for (int d = 0; d < 3; ++d) rd->push_back(reg(RA_B1 + d, b, op.s, op.e, 1));
      rd->push_back(reg(RA_W, b, op.s, op.e));
      rd->push_back(reg(RA_BCC, b, op.s, op.e));
      wr->push_back(reg(RA_BCC, b, op.s, op.e));
      wr->push_back(reg(RA_U, b, op.s, op.e));
      break;
    default:  // ML_BC_COARSE and anything else: the whole coarse level of the block
      for (int arr = RA_CU; arr <= RA_CB3; ++arr) {
        rd->push_back(reg(arr, b, all_s, all_e));
        wr->push_back(reg(arr, b, all_s, all_e));
      }
      break;
  }
}

// mark the operations after which no barrier is needed: an operation joins the current
// run unless it writes a box of its block's arrays that the run writes or reads, or reads
// one that the run writes.  Boxes are compared only within the same array of the block
// (reads of other blocks cannot conflict: a list writes its own block's arrays only).
template <typename F>
bool for_blocks(int nb, F f);

void mark_runs(MlOpList* L, const Ix& x) {
  const int nq = L->off.empty() ? 0 : (int)L->off.size() - 1;
  for_blocks(nq, [&](int q) {
    std::vector<Reg> rd, wr;
    std::vector<Reg> run_w[RA_SB3 + 1], run_r[RA_SB3 + 1];
    unsigned used = 0;
    const int b = L->blk[q];
    auto hits = [](const Reg& a, const std::vector<Reg>& v) {
      for (const Reg& g : v)
        if (overlap(a, g)) return true;
      return false;
    };
    for (int i = L->off[q]; i < L->off[q + 1]; ++i) {
      MlOp& op = L->ops[i];
      op_regions(op, b, x, &rd, &wr);
      bool conflict = false;
      for (const Reg& w : wr)
        if (hits(w, run_w[w.arr]) || hits(w, run_r[w.arr])) { conflict = true; break; }
      if (!conflict)
        for (const Reg& r : rd)
          if (r.blk == b && hits(r, run_w[r.arr])) { conflict = true; break; }
      if (conflict && i > L->off[q]) {
        L->ops[i - 1].nosync = 0;
        for (int a = 0; a <= RA_SB3; ++a)
          if (used & (1u << a)) { run_w[a].clear(); run_r[a].clear(); }
        used = 0;
      }
      for (const Reg& w : wr) { run_w[w.arr].push_back(w); used |= 1u << w.arr; }
      for (const Reg& r : rd)
        if (r.blk == b) { run_r[r.arr].push_back(r); used |= 1u << r.arr; }
      op.nosync = 1;
    }
    return true;
  });
}

// Host threads kept for the planner's parallel loops: creating threads costs tens of
// microseconds each, several times per regrid otherwise.  run(n, f) calls f(i) for
// i in [0, n) in chunks of 32 on the pool's threads and the caller's; one run at a time.
class PlanPool {
 public:
  static PlanPool& get() {
    static PlanPool pool;
    return pool;
  }
  void run(int n, const std::function<void(int)>& f) {
    std::lock_guard<std::mutex> one(run_mu_);
    const int nt = std::min<int>((int)workers_.size() + 1, n / 64 + 1);
    if (nt <= 1) {
      for (int i = 0; i < n; ++i) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &f;
      n_ = n;
      next_.store(0);
      helpers_ = nt - 1;
      busy_ = nt - 1;
      ++gen_;
    }
    cv_.notify_all();
    work(f, n);
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return busy_ == 0; });
    job_ = nullptr;
  }
  ~PlanPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : workers_) t.join();
  }

 private:
  PlanPool() {
    const unsigned hw = std::thread::hardware_concurrency();
    const int nw = std::max(0, std::min(16, hw ? (int)hw : 1) - 1);
    for (int t = 0; t < nw; ++t) workers_.emplace_back([this] { loop(); });
  }
  void work(const std::function<void(int)>& f, int n) {
    for (;;) {
      const int i0 = next_.fetch_add(32);
      if (i0 >= n) return;
      const int i1 = std::min(n, i0 + 32);
      for (int i = i0; i < i1; ++i) f(i);
    }
  }
  void loop() {
    unsigned long long seen = 0;
    for (;;) {
      const std::function<void(int)>* f;
      int n;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || (gen_ != seen && helpers_ > 0); });
        if (stop_) return;
        seen = gen_;
        --helpers_;  // this run takes at most nt - 1 helpers
        f = job_;
        n = n_;
      }
      work(*f, n);
      std::lock_guard<std::mutex> lk(mu_);
      if (--busy_ == 0) done_cv_.notify_one();
    }
  }
  std::vector<std::thread> workers_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int n_ = 0, helpers_ = 0, busy_ = 0;
  unsigned long long gen_ = 0;
  bool stop_ = false;
  std::atomic<int> next_{0};
};

// f(b) for every block on the host's cores; false if any call returned false
template <typename F>
bool for_blocks(int nb, F f) {
  std::atomic<bool> ok{true};
  PlanPool::get().run(nb, [&](int b) {
    if (!f(b)) ok = false;
  });
  return ok;
}

// the per-block lists in block order as one operation list (blocks with no operations
// left out), copied in parallel
void gather(const std::vector<std::vector<MlOp>>& per, MlOpList* L) {
  const int nb = (int)per.size();
  L->clear();
  std::vector<size_t> start(nb + 1, 0);
  for (int b = 0; b < nb; ++b) start[b + 1] = start[b] + per[b].size();
  L->ops.resize(start[nb]);
  L->off.push_back(0);
  for (int b = 0; b < nb; ++b)
    if (!per[b].empty()) {
      L->blk.push_back(b);
      L->off.push_back((int)start[b + 1]);
    }
  for_blocks(nb, [&](int b) {
    if (!per[b].empty())
      memcpy(L->ops.data() + start[b], per[b].data(), per[b].size() * sizeof(MlOp));
    return true;
  });
}

}  // namespace

bool build_ml_plan(const MlDims& dims, int nb, const int* nbr_table, const int* nbr_count,
                   const int* nblevel, const long long* loc, MlPlan* P, std::string* err) {
  Ix x;
  const int ng = dims.ng;
  for (int a = 0; a < 3; ++a) {
    x.n[a] = dims.nx[a];
    x.lo[a] = ng;
    x.hi[a] = ng + dims.nx[a] - 1;
    x.clo[a] = ng;
    x.chi[a] = ng + dims.nx[a] / 2 - 1;
  }
  x.ng = ng;
  x.cng = (ng + 1) / 2 + 1;  // meshblock.cpp:93
  auto nbr = [&](int b, int n) {
    const int* t = nbr_table + ((long long)b * ML_MAXNB + n) * ML_NF;
    MlNbr q;
    q.gid = t[0]; q.level = t[1]; q.ox1 = t[2]; q.ox2 = t[3]; q.ox3 = t[4];
    q.type = t[5]; q.fi1 = t[6]; q.fi2 = t[7]; q.fid = t[8]; q.eid = t[9];
    return q;
  };
  auto nbl = [&](int b, int o1, int o2, int o3) {
    return nblevel[(long long)b * 27 + (o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)];
  };
  auto level = [&](int b) { return (int)loc[(long long)b * 4]; };
  std::mutex err_mu;
  auto fail = [&](const char* what, int b) {
    char buf[160];
    snprintf(buf, sizeof buf, "multi-level plan: %s (block %d)", what, b);
    std::lock_guard<std::mutex> lk(err_mu);
    if (err->empty()) *err = buf;
    return false;
  };
  err->clear();
  P->level.resize(nb);
  for (int b = 0; b < nb; ++b) {
    P->level[b] = level(b);
    if (nbr_count[b] < 0 || nbr_count[b] > ML_MAXNB) return fail("bad neighbour count", b);
    for (int n = 0; n < nbr_count[b]; ++n)
      if (nbr(b, n).gid < 0 || nbr(b, n).gid >= nb)
        return fail("neighbour gid out of range", b);
  }
  // ---- phase R: restriction for coarser neighbours (into the send and coarse buffers) --
  P->r.clear(); P->x.clear(); P->p.clear();
  std::vector<std::vector<MlOp>>& per = P->per;
  per.resize(nb);
  for (auto& v : per) v.clear();
  for_blocks(nb, [&](int s) {
    std::vector<MlOp>& ops = per[s];
    for (int n = 0; n < nbr_count[s]; ++n) {
      MlNbr q = nbr(s, n);
      if (q.level >= level(s)) continue;
      MlOp op = make_op(ML_RESTRICT_U, 0, cc_send_coarser(x, q));
      op.src_kind = ML_SEND;
      ops.push_back(op);
      for (int d = 0; d < 3; ++d) {
        MlOp ob = make_op(ML_RESTRICT_B, d, fc_send_coarser(x, q, d));
        ob.src_kind = ML_SEND;
        ops.push_back(ob);
      }
    }
    return true;
  });
  gather(per, &P->r);
  // ---- phase X: the ghost exchange, per receiver in neighbour-list order; all U copies
  // first (SETB_HYD), then all face-field copies (SETB_FLD)
  // the entry of each block's list by (neighbour gid, offset), sorted, for the lookups of
  // the sender's entry that points back at the receiver
  std::vector<std::vector<std::pair<long long, int>>> keys(nb);
  auto key = [](long long gid, int o1, int o2, int o3) {
    return (gid << 5) | (long long)((o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1));
  };
  for_blocks(nb, [&](int s) {
    auto& k = keys[s];
    k.reserve(nbr_count[s]);
    for (int n = 0; n < nbr_count[s]; ++n) {
      const MlNbr q = nbr(s, n);
      k.push_back({key(q.gid, q.ox1, q.ox2, q.ox3), n});
    }
    std::sort(k.begin(), k.end());
    return true;
  });
  auto back_fast = [&](int s, int r, const MlNbr& f, MlNbr* out) {
    const auto& k = keys[s];
    const long long want = key(r, -f.ox1, -f.ox2, -f.ox3);
    auto it = std::lower_bound(k.begin(), k.end(), std::make_pair(want, -1));
    if (it == k.end() || it->first != want) return false;
    *out = nbr(s, it->second);
    return true;
  };
  for (auto& v : per) v.clear();
  const bool xok = for_blocks(nb, [&](int r) {
    // U copies into the list, face-field copies behind them (at most 3 per neighbour)
    std::vector<MlOp>& all = per[r];
    all.reserve(4 * nbr_count[r]);
    MlOp bcopies[3 * ML_MAXNB];
    int nbc = 0;
    const int par[3] = {(int)(loc[(long long)r * 4 + 1] & 1), (int)(loc[(long long)r * 4 + 2] & 1),
                        (int)(loc[(long long)r * 4 + 3] & 1)};
    for (int n = 0; n < nbr_count[r]; ++n) {
      MlNbr q = nbr(r, n), qs;
      const int s = q.gid;
      if (!back_fast(s, r, q, &qs)) return fail("inconsistent neighbour lists", r);
      Box du, su;
      int ud, us;
      if (q.level == level(r)) {
        du = cc_recv_same(x, q); su = cc_send_same(x, qs); ud = ML_FINE; us = ML_FINE;
      } else if (q.level < level(r)) {
        du = cc_recv_coarser(x, q, par); su = cc_send_finer(x, qs); ud = ML_COARSE;
        us = ML_FINE;
      } else {
        du = cc_recv_finer(x, q); su = cc_send_coarser(x, qs); ud = ML_FINE; us = ML_SEND;
      }
      if (!same_shape(du, su)) return fail("mismatched cell transfer boxes", r);
      MlOp op = make_op(ML_COPY_U, 0, du);
      op.src_kind = us; op.dst_kind = ud; op.src = s;
      for (int a = 0; a < 3; ++a) op.o[a] = su.s[a];
      all.push_back(op);
      for (int d = 0; d < 3; ++d) {
        Box db, sb;
        if (q.level == level(r)) { db = fc_recv_same(x, q, d); sb = fc_send_same(x, qs, d); }
        else if (q.level < level(r)) {
          db = fc_recv_coarser(x, q, d, par); sb = fc_send_finer(x, qs, d);
        } else { db = fc_recv_finer(x, q, d); sb = fc_send_coarser(x, qs, d); }
        if (!same_shape(db, sb)) return fail("mismatched face transfer boxes", r);
        MlOp ob = make_op(ML_COPY_B, d, db);
        ob.src_kind = us; ob.dst_kind = ud; ob.src = s;
        for (int a = 0; a < 3; ++a) ob.o[a] = sb.s[a];
        bcopies[nbc++] = ob;
      }
    }
    all.insert(all.end(), bcopies, bcopies + nbc);
    return true;
  });
  if (!xok) return false;
  gather(per, &P->x);
  // ---- phase P: ProlongateBoundaries per block with coarser neighbours ------------------
  const int cn = x.cng - 1;
  for (auto& v : per) v.clear();
  for_blocks(nb, [&](int b) {
    const int lev = level(b);
    std::vector<MlOp>& ops = per[b];
    for (int n = 0; n < nbr_count[b]; ++n) {
      MlNbr q = nbr(b, n);
      if (q.level >= lev) continue;
      int o[3]; off3(q, o);
      int ns[3], ne[3];
      for (int a = 0; a < 3; ++a) {
        ns[a] = (o[a] - 1 > -1) ? o[a] - 1 : -1;
        ne[a] = (o[a] + 1 < 1) ? o[a] + 1 : 1;
      }
      // RestrictGhostCellsOnSameLevel (bvals_refine.cpp:262-352)
      for (int nk = ns[2]; nk <= ne[2]; ++nk)
        for (int nj = ns[1]; nj <= ne[1]; ++nj)
          for (int ni = ns[0]; ni <= ne[0]; ++ni) {
            const int ntype = (ni != 0) + (nj != 0) + (nk != 0);
            if (ntype == 0 || nbl(b, ni, nj, nk) != lev) continue;
            const int nn[3] = {ni, nj, nk};
            Box r;
            for (int a = 0; a < 3; ++a) {
              if (nn[a] == 0) {
                r.s[a] = x.clo[a]; r.e[a] = x.chi[a];
                if (o[a] == 1) r.s[a] = x.chi[a];
                else if (o[a] == -1) r.e[a] = x.clo[a];
              } else if (nn[a] == 1) {
                r.s[a] = r.e[a] = x.chi[a] + 1;
              } else {
                r.s[a] = r.e[a] = x.clo[a] - 1;
              }
            }
            MlOp ru = make_op(ML_RESTRICT_U, 0, r);
            ru.src_kind = ML_COARSE;
            ops.push_back(ru);
            for (int d = 0; d < 3; ++d) {
              Box rf = r;
              int rs = r.s[d], re = r.e[d] + 1;
              int om[3] = {ni, nj, nk}, op3[3] = {ni, nj, nk};
              om[d] -= 1;
              op3[d] += 1;
              if (rs == x.clo[d] && nbl(b, om[0], om[1], om[2]) < lev) rs++;
              if (re == x.chi[d] + 1 && nbl(b, op3[0], op3[1], op3[2]) < lev) re--;
              rf.s[d] = rs;
              rf.e[d] = re;
              MlOp rb = make_op(ML_RESTRICT_B, d, rf);
              rb.src_kind = ML_COARSE;
              if (!empty(rf)) ops.push_back(rb);
            }
          }
      Box c;
      for (int a = 0; a < 3; ++a) {
        if (o[a] == 0) {
          c.s[a] = x.clo[a]; c.e[a] = x.chi[a];
          if ((loc[(long long)b * 4 + 1 + a] & 1LL) == 0LL) c.e[a] += cn; else c.s[a] -= cn;
        } else if (o[a] > 0) { c.s[a] = x.chi[a] + 1; c.e[a] = x.chi[a] + cn; }
        else { c.s[a] = x.clo[a] - cn; c.e[a] = x.clo[a] - 1; }
      }
      // ApplyPhysicalBoundariesOnCoarseLevel (bvals_refine.cpp:366-505)
      Box cx = c;
      for (int a = 0; a < 3; ++a) {
        int om[3] = {0, 0, 0}, op3[3] = {0, 0, 0};
        om[a] = -1; op3[a] = 1;
        int fm = 1, fp = 1;
        if (o[a] == 0) {
          fm = nbl(b, om[0], om[1], om[2]) != -1;
          fp = nbl(b, op3[0], op3[1], op3[2]) != -1;
        }
        cx.s[a] -= fm;
        cx.e[a] += fp;
      }
      ops.push_back(make_op(ML_C2P_COARSE, 0, cx));
      for (int a = 0; a < 3; ++a) {
        if (o[a] != 0) continue;
        for (int side = 0; side < 2; ++side) {
          int od[3] = {0, 0, 0};
          od[a] = side ? 1 : -1;
          if (nbl(b, od[0], od[1], od[2]) != -1) continue;  // not a physical face
          // box: layers 1..ng along a, transverse ranges of c extended by one (the face
          // components along a transverse axis have one more entry)
          Box bx;
          for (int q3 = 0; q3 < 3; ++q3) {
            if (q3 == a) { bx.s[q3] = 1; bx.e[q3] = ng; }
            else { bx.s[q3] = c.s[q3]; bx.e[q3] = c.e[q3] + 1; }
          }
          MlOp ob = make_op(ML_BC_COARSE, 0, bx);
          ob.aux = (2 * a + side) | (dims.bc[2 * a + side] << 4);
          ops.push_back(ob);
        }
      }
      ops.push_back(make_op(ML_PROLONG_U, 0, c));
      for (int d = 0; d < 3; ++d) {
        Box cf = c;
        int lo = c.s[d], hi = c.e[d] + 1;
        int om[3] = {o[0], o[1], o[2]}, op3[3] = {o[0], o[1], o[2]};
        om[d] -= 1;
        op3[d] += 1;
        if (o[d] >= 0 && nbl(b, om[0], om[1], om[2]) >= lev) lo++;
        if (o[d] <= 0 && nbl(b, op3[0], op3[1], op3[2]) >= lev) hi--;
        cf.s[d] = lo;
        cf.e[d] = hi;
        if (!empty(cf)) ops.push_back(make_op(ML_PROLONG_SHARED, d, cf));
      }
      ops.push_back(make_op(ML_PROLONG_INTERNAL, 0, c));
      Box fb;
      for (int a = 0; a < 3; ++a) {
        fb.s[a] = (c.s[a] - x.clo[a]) * 2 + x.lo[a];
        fb.e[a] = (c.e[a] - x.clo[a]) * 2 + x.lo[a] + 1;
      }
      ops.push_back(make_op(ML_FINE_P2C, 0, fb));
    }
    return true;
  });
  gather(per, &P->p);
  // ---- flux correction tasks: (coarse block, finer block, face | fi1 << 4 | fi2 << 5) --
  P->flux_tasks.clear();
  P->fmask.assign(nb, 0);
  for (int b = 0; b < nb; ++b)
    for (int n = 0; n < nbr_count[b]; ++n) {
      MlNbr q = nbr(b, n);
      if (q.type != ML_FACE || q.level != level(b) + 1) continue;
      P->flux_tasks.push_back(MlFluxTask{b, q.gid, q.fid | (q.fi1 << 4) | (q.fi2 << 5), 0});
      P->fmask[b] |= 1 << q.fid;
    }
  // ---- bounds of every operation ------------------------------------------------------
  {
    Bounds B;
    for (int a = 0; a < 3; ++a) {
      B.nc[a] = dims.nx[a] + 2 * ng;
      B.ncc[a] = dims.nx[a] / 2 + 2 * ng;
    }
    const MlOpList* lists[3] = {&P->r, &P->x, &P->p};
    for (const MlOpList* L : lists) {
      const int nq = L->off.empty() ? 0 : (int)L->off.size() - 1;
      const bool ok = for_blocks(nq, [&](int q) {
        for (int i = L->off[q]; i < L->off[q + 1]; ++i)
          if (!check_op(L->ops[i], x, B)) {
            char buf[200];
            const MlOp& o = L->ops[i];
            snprintf(buf, sizeof buf,
                     "multi-level plan: operation %d (d %d) box [%d..%d, %d..%d, %d..%d] out "
                     "of bounds", o.code, o.d, o.s[0], o.e[0], o.s[1], o.e[1], o.s[2], o.e[2]);
            std::lock_guard<std::mutex> lk(err_mu);
            if (err->empty()) *err = buf;
            return false;
          }
        return true;
      });
      if (!ok) return false;
    }
    mark_runs(&P->r, x);
    mark_runs(&P->x, x);
    mark_runs(&P->p, x);
    for (const MlFluxTask& t : P->flux_tasks)
      if (t.coarse < 0 || t.coarse >= nb || t.fine < 0 || t.fine >= nb) {
        *err = "multi-level plan: flux task block out of range";
        return false;
      }
  }
  // ---- CountFineEdges ---------------------------------------------------------------
  P->eflag.assign((size_t)nb * 12, 0);
  P->nfine.assign((size_t)nb * 12, 0);
  for (int b = 0; b < nb; ++b) {
    const int lev = level(b);
    int eid = 0;
    for (int t = 0; t < 3; ++t) {
      const int a = (t == 2) ? 1 : 0, cax = (t == 0) ? 1 : 2;
      for (int oc = -1; oc <= 1; oc += 2)
        for (int oa = -1; oa <= 1; oa += 2) {
          const int nas = (oa - 1 > -1) ? oa - 1 : -1, nae = (oa + 1 < 1) ? oa + 1 : 1;
          const int ncs = (oc - 1 > -1) ? oc - 1 : -1, nce = (oc + 1 < 1) ? oc + 1 : 1;
          int nf = 0, fl = lev;
          for (int nc = ncs; nc <= nce; ++nc)
            for (int na = nas; na <= nae; ++na) {
              int o[3] = {0, 0, 0};
              o[a] = na;
              o[cax] = nc;
              const int l = nbl(b, o[0], o[1], o[2]);
              if (l > fl) { fl++; nf = 0; }
              if (l == fl) nf++;
            }
          P->eflag[(size_t)b * 12 + eid] = (fl == lev);
          P->nfine[(size_t)b * 12 + eid] = nf;
          eid++;
        }
    }
  }
  return true;
}

void MlOpList::add(int block, const std::vector<MlOp>& ops) {
  if (off.empty()) off.push_back(0);
  blk.push_back(block);
  this->ops.insert(this->ops.end(), ops.begin(), ops.end());
  off.push_back((int)this->ops.size());
}

void MlOpList::clear() {
  ops.clear();
  off.clear();
  blk.clear();
}

}  // namespace athgpu
