// Test-infrastructure problem generator linked into the reference (Athena++) build made
// by oracle/build_ref.py.  It is NOT part of the product.
//
// MeshBlock::ProblemGenerator is the reference's user extension point
// (src/pgen/default_pgen.cpp:86, selected at link time, Makefile.in:74).  This one
// loads an initial state for the whole (uniform, single-level) mesh from the binary file
// named by <problem>/ic_file, so that the reference, the oracle and the CUDA path all
// start from bit-identical inputs.
//
// ic_file layout (little-endian):
//   int32 kind (0 = conserved U, 1 = primitive W converted with the EOS), int32 NX1,
//   int32 NX2, int32 NX3,
//   double q[5][NX3][NX2][NX1], b1[NX3][NX2][NX1+1], b2[NX3][NX2+1][NX1],
//   double b3[NX3+1][NX2][NX1]
#include <cstdint>
#include <cstdio>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "athena.hpp"
#include "athena_arrays.hpp"
#include "coordinates/coordinates.hpp"
#include "eos/eos.hpp"
#include "field/field.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"
#include "parameter_input.hpp"

void MeshBlock::ProblemGenerator(ParameterInput *pin) {
  std::string fname = pin->GetString("problem", "ic_file");
  std::FILE *f = std::fopen(fname.c_str(), "rb");
  if (f == nullptr) throw std::runtime_error("load_ic: cannot open " + fname);
  std::int32_t hdr[4];
  if (std::fread(hdr, sizeof(hdr), 1, f) != 1) throw std::runtime_error("load_ic: hdr");
  const int kind = hdr[0];
  const std::int64_t NX1 = hdr[1], NX2 = hdr[2], NX3 = hdr[3];
  std::vector<double> q(5*NX3*NX2*NX1), b1(NX3*NX2*(NX1+1)), b2(NX3*(NX2+1)*NX1),
      b3((NX3+1)*NX2*NX1);
  bool ok = std::fread(q.data(), sizeof(double), q.size(), f) == q.size();
  ok = ok && std::fread(b1.data(), sizeof(double), b1.size(), f) == b1.size();
  ok = ok && std::fread(b2.data(), sizeof(double), b2.size(), f) == b2.size();
  ok = ok && std::fread(b3.data(), sizeof(double), b3.size(), f) == b3.size();
  std::fclose(f);
  if (!ok) throw std::runtime_error("load_ic: short file " + fname);

  const std::int64_t o1 = loc.lx1*block_size.nx1, o2 = loc.lx2*block_size.nx2,
                     o3 = loc.lx3*block_size.nx3;
  AthenaArray<Real> &dst = (kind == 0) ? phydro->u : phydro->w;
  for (int n = 0; n < 5; ++n)
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie; ++i) {
          std::int64_t gk = o3 + k - ks, gj = o2 + j - js, gi = o1 + i - is;
          dst(n, k, j, i) = q[((n*NX3 + gk)*NX2 + gj)*NX1 + gi];
        }
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie+1; ++i) {
        std::int64_t gk = o3 + k - ks, gj = o2 + j - js, gi = o1 + i - is;
        pfield->b.x1f(k, j, i) = b1[(gk*NX2 + gj)*(NX1+1) + gi];
      }
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je+1; ++j)
      for (int i = is; i <= ie; ++i) {
        std::int64_t gk = o3 + k - ks, gj = o2 + j - js, gi = o1 + i - is;
        pfield->b.x2f(k, j, i) = b2[(gk*(NX2+1) + gj)*NX1 + gi];
      }
  for (int k = ks; k <= ke+1; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        std::int64_t gk = o3 + k - ks, gj = o2 + j - js, gi = o1 + i - is;
        pfield->b.x3f(k, j, i) = b3[(gk*NX2 + gj)*NX1 + gi];
      }
  if (kind == 1) {
    // primitive input: cell-centred field then W -> U with the reference's own EOS
    pfield->CalculateCellCenteredField(pfield->b, pfield->bcc, pcoord, is, ie, js, je, ks,
                                       ke);
    peos->PrimitiveToConserved(phydro->w, pfield->bcc, phydro->u, pcoord, is, ie, js, je,
                               ks, ke);
    phydro->w1 = phydro->w;
  }
}
