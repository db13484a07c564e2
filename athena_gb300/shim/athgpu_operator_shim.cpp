//! \file athgpu_operator_shim.cpp
//! \brief The reference's stage-update member functions, forwarded to libathgpu.so.
//!
//! Compiled into Athena++ as one more source file, this file defines
//!   Hydro::CalculateFluxes           (hydro.hpp:72-73)
//!   Hydro::AddFluxDivergence         (hydro.hpp:67)
//!   Hydro::NewBlockTimeStep          (hydro.hpp:66)
//!   Field::ComputeCornerE            (field.hpp:66)
//!   Field::CT                        (field.hpp:63)
//!   EquationOfState::ConservedToPrimitive (eos.hpp:37-40)
//! with the reference's own signatures, so that TimeIntegratorTaskList, the boundary
//! exchange, the EMF averaging, Mesh::Initialize and the main loop drive them unchanged.
//! Each body forwards the MeshBlock's own AthenaArrays to the library's per-operator entry
//! points (include/athena_gb300.h, athgpu_op_*), which run the operator on the GPU and
//! return the reference's results bit for bit.  The reference's definitions of these six
//! functions are made weak in their object files at link time (oracle/build_ref.py,
//! variant "*_gpu") so that these take their place; nothing in the reference's sources
//! changes.
//!
//! One athgpu context of one MeshBlock is kept per MeshBlock (created at its first call,
//! replaced when a MeshBlock at the same address has other coordinates, as after a
//! regrid).  This path moves each operator's arrays to the device and back on every call:
//! it is the drop-in for parity and integration work; the batched whole-mesh calls
//! (athgpu_cycle) are the fast path.

#include <cmath>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>

#include "athena.hpp"
#include "athena_arrays.hpp"
#include "coordinates/coordinates.hpp"
#include "eos/eos.hpp"
#include "field/field.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"
#include "reconstruct/reconstruction.hpp"

#include "athena_gb300.h"

namespace {

//! the physics parameters of a block's context that only some members can read
struct ShimPhysics {
  Real sigma_max, beta_min, gamma_max;
  bool known;
};

struct BlockContext {
  athgpu_ctx *ctx;
  Real x1, x2, x3, dx;  // the block's first interior face and spacing (identity check)
};

std::mutex g_mu;
std::map<const MeshBlock *, BlockContext> g_ctx;

void Check(athgpu_status st, const char *what) {
  if (st != ATHGPU_OK) {
    std::stringstream msg;
    msg << "### FATAL ERROR in " << what << ": " << athgpu_last_error() << std::endl;
    throw std::runtime_error(msg.str());
  }
}

int SolverCode() {
  const std::string rs(RIEMANN_SOLVER);
  if (rs == "hlld") return ATHGPU_HLLD;
  if (rs == "hlle") return ATHGPU_HLLE;
  if (rs == "llf") return ATHGPU_LLF;
  if (rs == "roe") return ATHGPU_ROE;
  if (rs == "lhlld") return ATHGPU_LHLLD;
  throw std::runtime_error("### FATAL ERROR in athgpu shim: unsupported Riemann solver " + rs);
}

//! the context of MeshBlock pmb (created at the first call on it)
athgpu_ctx *ContextOf(MeshBlock *pmb, const ShimPhysics &phys) {
  Coordinates *pco = pmb->pcoord;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_ctx.find(pmb);
  if (it != g_ctx.end()) {
    const BlockContext &bc = it->second;
    if (bc.x1 == pco->x1f(pmb->is) && bc.x2 == pco->x2f(pmb->js) &&
        bc.x3 == pco->x3f(pmb->ks) && bc.dx == pco->dx1f(pmb->is))
      return bc.ctx;
    athgpu_destroy(bc.ctx);  // another MeshBlock at the same address
    g_ctx.erase(it);
  }
  athgpu_mesh_desc d = {};
  d.nbx1 = d.nbx2 = d.nbx3 = 1;
  d.nx1 = pmb->block_size.nx1;
  d.nx2 = pmb->block_size.nx2;
  d.nx3 = pmb->block_size.nx3;
  d.nghost = NGHOST;
  // the reconstruction order comes with each flux call; the largest one the ghost width
  // allows here
  d.xorder = NGHOST >= 3 ? 3 : 2;
  d.rsolver = SolverCode();
  d.precision = ATHGPU_FP64;
  d.relativistic = RELATIVISTIC_DYNAMICS ? 1 : 0;
  d.gamma = pmb->peos->GetGamma();
  d.dfloor = pmb->peos->GetDensityFloor();
  d.pfloor = pmb->peos->GetPressureFloor();
  // the time step's CFL factor is applied here (NewBlockTimeStep below), so the context's
  // is 1, under the limit of the integrator it names (the operators use none)
  d.cfl_number = 1.0;
  d.integrator = ATHGPU_RK2;
  d.tlim = pmb->pmy_mesh->tlim;
  d.sigma_max = phys.known ? phys.sigma_max : 0.0;
  d.beta_min = phys.known ? phys.beta_min : 0.0;
  d.gamma_max = phys.known ? phys.gamma_max : 1000.0;
  d.x1f = pco->x1f.data();
  d.dx1f = pco->dx1f.data();
  d.x2f = pco->x2f.data();
  d.dx2f = pco->dx2f.data();
  d.x3f = pco->x3f.data();
  d.dx3f = pco->dx3f.data();
  // the operator context does no boundary work: its mesh faces are left periodic
  athgpu_ctx *ctx = nullptr;
  Check(athgpu_create(&ctx, &d), "athgpu_create (operator context)");
  g_ctx[pmb] = BlockContext{ctx, pco->x1f(pmb->is), pco->x2f(pmb->js), pco->x3f(pmb->ks),
                            pco->dx1f(pmb->is)};
  return ctx;
}

ShimPhysics Unknown() { return ShimPhysics{0.0, 0.0, 1000.0, false}; }

athgpu_face_emfs FaceEmfs(Field *pf) {
  athgpu_face_emfs e;
  e.e3_x1f = pf->e3_x1f.data();
  e.e2_x1f = pf->e2_x1f.data();
  e.wght_x1f = pf->wght.x1f.data();
  e.e1_x2f = pf->e1_x2f.data();
  e.e3_x2f = pf->e3_x2f.data();
  e.wght_x2f = pf->wght.x2f.data();
  e.e1_x3f = pf->e1_x3f.data();
  e.e2_x3f = pf->e2_x3f.data();
  e.wght_x3f = pf->wght.x3f.data();
  return e;
}

}  // namespace

//----------------------------------------------------------------------------------------
// Hydro::CalculateFluxes: reconstruction + Riemann solver on every face, the face EMFs and
// the CT weights (calculate_fluxes.cpp:38-415)
void Hydro::CalculateFluxes(AthenaArray<Real> &w, FaceField &b, AthenaArray<Real> &bcc,
                            const int order) {
  MeshBlock *pmb = pmy_block;
  ShimPhysics phys{pmb->peos->sigma_max_, pmb->peos->beta_min_, pmb->peos->gamma_max_, true};
  athgpu_ctx *ctx = ContextOf(pmb, phys);
  // xorder = 3f (PiecewiseParabolicFast) is order 4 of the operator call
  const int op_order = (order == 3 && pmb->precon->rec3m_ == REC3METHOD::PPMF) ? 4 : order;
  athgpu_face_emfs e = FaceEmfs(pmb->pfield);
  Check(athgpu_op_calculate_fluxes(ctx, op_order, pmb->pmy_mesh->dt, w.data(), bcc.data(),
                                   b.x1f.data(), b.x2f.data(), b.x3f.data(),
                                   flux[X1DIR].data(), flux[X2DIR].data(),
                                   flux[X3DIR].data(), &e),
        "Hydro::CalculateFluxes");
}

//----------------------------------------------------------------------------------------
// Hydro::AddFluxDivergence: u_out -= wght div(F) / V (add_flux_divergence.cpp:39-96)
void Hydro::AddFluxDivergence(const Real wght, AthenaArray<Real> &u_out) {
  MeshBlock *pmb = pmy_block;
  ShimPhysics phys{pmb->peos->sigma_max_, pmb->peos->beta_min_, pmb->peos->gamma_max_, true};
  Check(athgpu_op_add_flux_divergence(ContextOf(pmb, phys), wght, flux[X1DIR].data(),
                                      flux[X2DIR].data(), flux[X3DIR].data(), u_out.data()),
        "Hydro::AddFluxDivergence");
}

//----------------------------------------------------------------------------------------
// Hydro::NewBlockTimeStep: the block's CFL time step (new_blockdt.cpp:45-230; no
// diffusion, orbital advection or user time step in the paths this library covers)
void Hydro::NewBlockTimeStep() {
  MeshBlock *pmb = pmy_block;
  Field *pf = pmb->pfield;
  ShimPhysics phys{pmb->peos->sigma_max_, pmb->peos->beta_min_, pmb->peos->gamma_max_, true};
  Real min_dt = 0.0;  // the minimum over cells (the context's CFL factor is 1)
  Check(athgpu_op_new_block_dt(ContextOf(pmb, phys), w.data(), pf->bcc.data(),
                               pf->b.x1f.data(), pf->b.x2f.data(), pf->b.x3f.data(),
                               &min_dt),
        "Hydro::NewBlockTimeStep");
  Real dt = min_dt;
  dt *= pmb->pmy_mesh->cfl_number;  // new_blockdt.cpp:193
  const Real big = std::numeric_limits<Real>::max();
  pmb->new_block_dt_ = dt;
  pmb->new_block_dt_hyperbolic_ = dt;
  pmb->new_block_dt_parabolic_ = big;
  pmb->new_block_dt_user_ = big;
}

//----------------------------------------------------------------------------------------
// Field::ComputeCornerE: the edge EMFs from the face EMFs (calculate_corner_e.cpp:28-236)
void Field::ComputeCornerE(AthenaArray<Real> &w, AthenaArray<Real> &bcc) {
  MeshBlock *pmb = pmy_block;
  athgpu_face_emfs fe = FaceEmfs(this);
  Check(athgpu_op_corner_e(ContextOf(pmb, Unknown()), w.data(), bcc.data(), &fe,
                           e.x1e.data(), e.x2e.data(), e.x3e.data()),
        "Field::ComputeCornerE");
}

//----------------------------------------------------------------------------------------
// Field::CT: the face-field update from the (averaged) edge EMFs (ct.cpp:31-116)
void Field::CT(const Real wght, FaceField &b_out) {
  MeshBlock *pmb = pmy_block;
  Check(athgpu_op_ct(ContextOf(pmb, Unknown()), wght, e.x1e.data(), e.x2e.data(),
                     e.x3e.data(), b_out.x1f.data(), b_out.x2f.data(), b_out.x3f.data()),
        "Field::CT");
}

//----------------------------------------------------------------------------------------
// EquationOfState::ConservedToPrimitive over [il,iu]x[jl,ju]x[kl,ku], with the cell-centred
// field of the same range (adiabatic_mhd.cpp:41-90; adiabatic_mhd_sr.cpp:72-272)
void EquationOfState::ConservedToPrimitive(
    AthenaArray<Real> &cons, const AthenaArray<Real> &prim_old, const FaceField &b,
    AthenaArray<Real> &prim, AthenaArray<Real> &bcc, Coordinates *pco, int il, int iu,
    int jl, int ju, int kl, int ku) {
  ShimPhysics phys{sigma_max_, beta_min_, gamma_max_, true};
  Check(athgpu_op_con2prim(ContextOf(pmy_block_, phys), cons.data(), b.x1f.data(),
                           b.x2f.data(), b.x3f.data(), prim.data(), bcc.data(), il, iu, jl,
                           ju, kl, ku, nullptr),
        "EquationOfState::ConservedToPrimitive");
}
