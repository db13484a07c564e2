// Test-infrastructure hook linked into the reference (Athena++) build made by
// oracle/build_ref.py.  It is NOT part of the product.
//
// Mesh::UserWorkInLoop() is a weak no-op in the reference
// (src/pgen/default_pgen.cpp:52).  This strong definition replaces it and, after every
// cycle (it is called from src/main.cpp after the stage loop, before ncycle++ and
// NewTimeStep), writes the complete state of every MeshBlock to
//   dump.<ncycle+1, 5 digits>.bin   (in the working directory)
// so that the oracle and the CUDA path can be compared cell by cell against the
// reference itself.
//
// File layout (little-endian, native sizes):
//   int32 magic 0x41544844, int32 version 1
//   int32 nblocks, int32 ncycle_after, double time_after, double dt_used
//   int32 nc1, nc2, nc3, ng, nhydro
//   per block: int64 lx1, lx2, lx3, int32 level,
//              double u[nhydro][nc3][nc2][nc1], w[nhydro][nc3][nc2][nc1],
//              double b1[nc3][nc2][nc1+1], b2[nc3][nc2+1][nc1], b3[nc3+1][nc2][nc1],
//              double bcc[3][nc3][nc2][nc1]
#include <cstdint>
#include <cstdio>
#include <string>

#include "athena.hpp"
#include "athena_arrays.hpp"
#include "field/field.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"

namespace {
void WriteArray(std::FILE *f, const AthenaArray<Real> &a) {
  std::fwrite(a.data(), sizeof(Real), a.GetSize(), f);
}
}  // namespace

void Mesh::UserWorkInLoop() {
  char name[512];
  std::snprintf(name, sizeof(name), "dump.%05d.bin", ncycle + 1);
  std::FILE *f = std::fopen(name, "wb");
  if (f == nullptr) return;
  std::int32_t hdr[4] = {0x41544844, 1, nblocal, ncycle + 1};
  std::fwrite(hdr, sizeof(hdr), 1, f);
  double t_after = time + dt, dt_used = dt;
  std::fwrite(&t_after, sizeof(double), 1, f);
  std::fwrite(&dt_used, sizeof(double), 1, f);
  MeshBlock *pmb0 = my_blocks(0);
  std::int32_t dims[5] = {pmb0->ncells1, pmb0->ncells2, pmb0->ncells3, NGHOST, NHYDRO};
  std::fwrite(dims, sizeof(dims), 1, f);
  for (int b = 0; b < nblocal; ++b) {
    MeshBlock *pmb = my_blocks(b);
    std::int64_t loc[3] = {pmb->loc.lx1, pmb->loc.lx2, pmb->loc.lx3};
    std::int32_t level = pmb->loc.level;
    std::fwrite(loc, sizeof(loc), 1, f);
    std::fwrite(&level, sizeof(level), 1, f);
    WriteArray(f, pmb->phydro->u);
    WriteArray(f, pmb->phydro->w);
    WriteArray(f, pmb->pfield->b.x1f);
    WriteArray(f, pmb->pfield->b.x2f);
    WriteArray(f, pmb->pfield->b.x3f);
    WriteArray(f, pmb->pfield->bcc);
  }
  std::fclose(f);
}
