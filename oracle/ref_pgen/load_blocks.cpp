// Test-infrastructure problem generator linked into the reference (Athena++) build made
// by oracle/build_ref.py.  It is NOT part of the product.
//
// MeshBlock::ProblemGenerator is the reference's user extension point
// (src/pgen/default_pgen.cpp:86, selected at link time).  This one loads the initial state
// of every MeshBlock of a (possibly multi-level) mesh from the binary file named by
// <problem>/ic_file, block by block in the reference's own gid order, so that the
// reference, the oracle and the CUDA path start from bit-identical inputs on meshes
// with refinement levels.
//
// ic_file layout (little-endian):
//   int32 nblocks, int32 nx1, int32 nx2, int32 nx3,
//   per block (gid order): int32 level, int64 lx1, lx2, lx3,
//     double u[5][nx3][nx2][nx1], b1[nx3][nx2][nx1+1], b2[nx3][nx2+1][nx1],
//     double b3[nx3+1][nx2][nx1]
#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "athena.hpp"
#include "athena_arrays.hpp"
#include "field/field.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"
#include "parameter_input.hpp"

void MeshBlock::ProblemGenerator(ParameterInput *pin) {
  std::string fname = pin->GetString("problem", "ic_file");
  std::FILE *f = std::fopen(fname.c_str(), "rb");
  if (f == nullptr) throw std::runtime_error("load_blocks: cannot open " + fname);
  std::int32_t hdr[4];
  if (std::fread(hdr, sizeof(hdr), 1, f) != 1) throw std::runtime_error("load_blocks: hdr");
  const std::int64_t n1 = hdr[1], n2 = hdr[2], n3 = hdr[3];
  if (n1 != block_size.nx1 || n2 != block_size.nx2 || n3 != block_size.nx3 || gid >= hdr[0])
    throw std::runtime_error("load_blocks: block size or count mismatch");
  const std::int64_t nu = 5 * n3 * n2 * n1, nf1 = n3 * n2 * (n1 + 1),
                     nf2 = n3 * (n2 + 1) * n1, nf3 = (n3 + 1) * n2 * n1;
  const std::int64_t rec = 4 + 3 * 8 + 8 * (nu + nf1 + nf2 + nf3);
  std::fseek(f, 16 + rec * static_cast<long>(gid), SEEK_SET);
  std::int32_t lev;
  std::int64_t lx[3];
  bool ok = std::fread(&lev, sizeof(lev), 1, f) == 1;
  ok = ok && std::fread(lx, sizeof(lx), 1, f) == 1;
  std::vector<double> q(nu), b1(nf1), b2(nf2), b3(nf3);
  ok = ok && std::fread(q.data(), sizeof(double), q.size(), f) == q.size();
  ok = ok && std::fread(b1.data(), sizeof(double), b1.size(), f) == b1.size();
  ok = ok && std::fread(b2.data(), sizeof(double), b2.size(), f) == b2.size();
  ok = ok && std::fread(b3.data(), sizeof(double), b3.size(), f) == b3.size();
  std::fclose(f);
  if (!ok) throw std::runtime_error("load_blocks: short file " + fname);
  if (lev != loc.level || lx[0] != loc.lx1 || lx[1] != loc.lx2 || lx[2] != loc.lx3)
    throw std::runtime_error("load_blocks: block order differs from the reference's");
  for (int n = 0; n < 5; ++n)
    for (int k = 0; k < n3; ++k)
      for (int j = 0; j < n2; ++j)
        for (int i = 0; i < n1; ++i)
          phydro->u(n, ks + k, js + j, is + i) = q[((n * n3 + k) * n2 + j) * n1 + i];
  for (int k = 0; k < n3; ++k)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i <= n1; ++i)
        pfield->b.x1f(ks + k, js + j, is + i) = b1[(k * n2 + j) * (n1 + 1) + i];
  for (int k = 0; k < n3; ++k)
    for (int j = 0; j <= n2; ++j)
      for (int i = 0; i < n1; ++i)
        pfield->b.x2f(ks + k, js + j, is + i) = b2[(k * (n2 + 1) + j) * n1 + i];
  for (int k = 0; k <= n3; ++k)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i)
        pfield->b.x3f(ks + k, js + j, is + i) = b3[(k * n2 + j) * n1 + i];
}

// With nlim = 0 the main loop does not run: dump the initialized state (ghost zones after
// Mesh::Initialize) through the dump hook, as dump.00001.bin.
void Mesh::UserWorkAfterLoop(ParameterInput *pin) {
  if (ncycle == 0) UserWorkInLoop();
}
