// Box operations of the multi-level stage (shared by the host planner, ml_plan.cu, and
// the device executor, multilevel.cuh).
#pragma once

namespace athgpu {

enum MlOpCode : int {
  ML_COPY_U = 0,       // cells, 5 variables: dst box of this block <- src box
  ML_COPY_B = 1,       // face component d
  ML_RESTRICT_U = 2,   // this block's fine U -> coarse-indexed box of ccons or scons
  ML_RESTRICT_B = 3,   // this block's fine face component d -> cb or sb
  ML_C2P_COARSE = 4,   // W(U) and bcc on the coarse buffers over the box
  ML_BC_COARSE = 5,    // physical boundary of face `aux & 7`, kind `aux >> 4`, on coarse W, B
  ML_PROLONG_U = 6,    // coarse W -> fine W (the box is in coarse cells)
  ML_PROLONG_SHARED = 7,   // coarse face component d -> fine faces in it
  ML_PROLONG_INTERNAL = 8, // fine faces inside coarse cells (Toth & Roe)
  ML_FINE_P2C = 9,     // fine bcc and U(W) over the box (fine cells)
};

// array selectors of ML_COPY_*: source and destination kinds
enum MlArr : int { ML_FINE = 0, ML_COARSE = 1, ML_SEND = 2 };

struct MlOp {
  int code;
  int d;          // face component (0..2) of the B operations
  int src_kind;   // MlArr of the source (copies) / destination (restrictions)
  int dst_kind;   // MlArr of the destination (copies)
  int src;        // source block (copies)
  int aux;        // boundary face and kind (ML_BC_COARSE)
  int s[3], e[3]; // destination box (inclusive), index 0 = i
  int o[3];       // source box origin (copies)
  int nosync;     // 1: the next operation touches nothing this one writes or reads
                  // (no barrier between them); 0 (the default): barrier
};

// a neighbour-list entry as the host passes it (BoundaryBase::neighbor, bvals_base.cpp)
struct MlNbr {
  int gid, level, ox1, ox2, ox3, type, fi1, fi2, fid, eid;
};
enum { ML_NF = 10, ML_MAXNB = 56, ML_FACE = 0, ML_EDGE = 1, ML_CORNER = 2 };

}  // namespace athgpu
