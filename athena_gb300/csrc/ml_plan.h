// Host planner of the multi-level stage (ml_plan.cu).
#pragma once
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "ml_types.h"

namespace athgpu {

// An allocator whose value-initialisation leaves trivial elements as they are: the planner
// sizes its flat operation lists first and then writes every element, so zeroing them
// first (tens of MB on large meshes) is wasted.
template <typename T>
struct NoInitAlloc : std::allocator<T> {
  template <typename U>
  struct rebind {
    using other = NoInitAlloc<U>;
  };
  NoInitAlloc() = default;
  template <typename U>
  NoInitAlloc(const NoInitAlloc<U>&) {}
  template <typename U>
  void construct(U* p) {
    ::new ((void*)p) U;
  }
  template <typename U, typename... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};

struct MlDims {
  int nx[3];   // interior cells per MeshBlock
  int ng;      // ghost layers (even)
  int bc[6];   // mesh-face boundary flags (0 periodic, 1 outflow, 2 reflecting)
};

// per-block operation lists, flattened: block blk[q] executes ops[off[q] .. off[q+1])
struct MlOpList {
  std::vector<MlOp, NoInitAlloc<MlOp>> ops;
  std::vector<int> off, blk;
  void add(int block, const std::vector<MlOp>& ops);
  void clear();
};

struct MlFluxTask {
  int coarse, fine, face, pad;  // face | fi1 << 4 | fi2 << 5
};

struct MlPlan {
  MlOpList r, x, p;          // restriction for coarser, exchange, prolongation
  std::vector<MlFluxTask> flux_tasks;
  std::vector<int> fmask;    // per block: faces shared with finer blocks
  std::vector<int> eflag, nfine, level;
  std::vector<std::vector<MlOp>> per;  // the planner's per-block lists (storage kept)
};

bool build_ml_plan(const MlDims& dims, int nb, const int* nbr_table, const int* nbr_count,
                   const int* nblevel, const long long* loc, MlPlan* plan, std::string* err);

}  // namespace athgpu
