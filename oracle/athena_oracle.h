/* CPU oracle for the Athena++ MHD stage update — TEST INFRASTRUCTURE, not the product.
 *
 * A plain-C, FP64 restatement of the reference's algorithm for the hot path
 * (reconstruction, Riemann solvers, flux divergence, corner EMF + constrained transport,
 * conserved->primitive, CFL time step, same-level ghost exchange, the VL2 stage
 * sequence).  Each routine in athena_oracle.c cites the reference file:line it follows.
 * It keeps the reference's floating-point association term for term so that its
 * results can be compared bit for bit with the reference binary built by
 * oracle/build_ref.py, and it is the checker for the CUDA path in tests/, in
 * __graft_entry__.smoke() and in bench.py's CPU-baseline leg.  Nothing in the
 * athena_gb300 package links or calls it.
 *
 * Data layout: every MeshBlock keeps the reference's AthenaArray layout
 * (athena_arrays.hpp:140-143, last index fastest, ghosts included); blocks are stored
 * in lexicographic order b = (lx3*nbx2 + lx2)*nbx1 + lx1.  A uniform single-level 3-D
 * mesh with periodic, outflow or reflecting mesh faces is supported.
 */
#ifndef ATHENA_ORACLE_H_
#define ATHENA_ORACLE_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nbx1, nbx2, nbx3;   /* MeshBlocks per direction */
  int nx1, nx2, nx3;      /* interior cells per MeshBlock */
  int ng;                 /* ghost layers (NGHOST) */
  int xorder;             /* 2 = PLM, 3 = PPM in the second VL2 stage */
  int rsolver;            /* 0 = HLLD, 1 = HLLE, 2 = LLF, 3 = Roe, 4 = LHLLD */
  int relativistic;       /* 0 = Newtonian adiabatic MHD, 1 = special relativistic */
  double gamma, dfloor, pfloor, cfl_number, tlim;
  double sigma_max, beta_min, gamma_max; /* SR floors (adiabatic_mhd_sr.cpp:46-48) */
  /* boundary flags of the mesh faces inner/outer x1, x2, x3: 0 periodic, 1 outflow,
   * 2 reflecting (bvals/cc/outflow_cc.cpp, bvals/cc/hydro/reflect_hydro.cpp,
   * bvals/fc/outflow_fc.cpp, bvals/fc/reflect_fc.cpp) */
  int bc[6];
  int ppm_fast;           /* time/xorder = 3f: PiecewiseParabolicFast (ppm_fast.cpp) */
} orc_params;

typedef struct orc_mesh orc_mesh;

/* x?f: per block, nc?+1 face coordinates; dx?f: per block, nc? face spacings, exactly
 * as the reference's Coordinates holds them (coordinates.cpp:92-146). */
orc_mesh *orc_create(const orc_params *p, const double *x1f, const double *dx1f,
                     const double *x2f, const double *dx2f, const double *x3f,
                     const double *dx3f);
void orc_destroy(orc_mesh *m);
int orc_num_threads(int n);

/* state I/O, whole-mesh arrays in block order (ghosts included) */
void orc_set_state(orc_mesh *m, const double *u, const double *b1, const double *b2,
                   const double *b3);
void orc_set_prim(orc_mesh *m, const double *w);  /* SR: initial W and NH guess */
void orc_get_state(const orc_mesh *m, double *u, double *b1, double *b2, double *b3);
void orc_get_prim(const orc_mesh *m, double *w, double *bcc);
double orc_get_dt(const orc_mesh *m);
double orc_get_time(const orc_mesh *m);
void orc_set_dt(orc_mesh *m, double dt);

/* Mesh::Initialize tail (mesh.cpp:1698-1833,1962): ghost exchange, W(U) on the whole
 * block, first time step. */
void orc_initialize(orc_mesh *m);
/* one VL2 cycle (main.cpp:512-541): both stages, time += dt, NewTimeStep */
void orc_cycle(orc_mesh *m);
/* one stage only (for intermediate comparisons); stage = 1 or 2 */
void orc_stage(orc_mesh *m, int stage);
/* counts of cells that hit the SR fallback in the last W(U) call */
long orc_c2p_failures(const orc_mesh *m);

/* Turn the mesh into a multi-level one (SMR/AMR; Newtonian MHD, even NGHOST): the
 * blocks (p.nbx1 of them, p.nbx2 = p.nbx3 = 1) in the reference's gid order with, per
 * block, its neighbour list nbr_table[b][56][10] (gid, level, ox1, ox2, ox3, type 0 face /
 * 1 edge / 2 corner, fi1, fi2, fid, eid), nbr_count[b], the 3x3x3 neighbour levels
 * nblevel[b][27] (-1: none), loc[b][4] (level, lx1, lx2, lx3) and the coarse-buffer face
 * coordinates cx?f[b][ncc+1], cdx?f[b][ncc] (ncc = nx/2 + 2 NGHOST).  Returns 0, or <0
 * for an unsupported configuration. */
int orc_set_multilevel(orc_mesh *m, const int *nbr_table, const int *nbr_count,
                       const int *nblevel, const long long *loc, const double *cx1f,
                       const double *cdx1f, const double *cx2f, const double *cdx2f,
                       const double *cx3f, const double *cdx3f);

/* time/integrator (task_list/time_integrator.cpp): ORC_VL2 (the default), ORC_RK2, or
 * ORC_RK1 (one stage; diagnostics) */
#define ORC_VL2 0
#define ORC_RK2 1
#define ORC_RK1 2
void orc_set_integrator(orc_mesh *m, int integrator);

/* per-operator restatements on block b (the member functions of one stage, one at a
 * time; see athena_oracle.c) */
void orc_op_fluxes(orc_mesh *m, int b, int order, double dt, double *flx1, double *flx2,
                   double *flx3, double *const emf[9]);
void orc_op_corner_e(orc_mesh *m, int b, const double *const emf[9], double *e1, double *e2,
                     double *e3);
void orc_op_add_flux_divergence(orc_mesh *m, int b, double wght, const double *flx1,
                                const double *flx2, const double *flx3, double *u);
void orc_op_ct(orc_mesh *m, int b, double wght, const double *e1, const double *e2,
               const double *e3, double *b1, double *b2, double *b3);
long orc_op_con2prim(orc_mesh *m, int b, int il, int iu, int jl, int ju, int kl, int ku);
double orc_op_new_block_dt(orc_mesh *m, int b);

/* One Riemann solve on a face, states in the solvers' local order (d, v_n, v_t1, v_t2, p,
 * B_t1, B_t2); rsolver 0 HLLD, 1 HLLE, 2 LLF, 3 Roe, 4 LHLLD (with the face's velocity
 * differences dvn, dvt); relativistic selects the SR solvers (hlld_rel.cpp,
 * hlle_mhd_rel.cpp, llf_mhd_rel.cpp).  flx7 in the same local order. */
void orc_riemann_face(int rsolver, int relativistic, double gamma, const double *wli,
                      const double *wri, double bx, double dvn, double dvt, double *flx7);
/* the stages of one cycle and time += dt, without the new time step (adaptive runs
 * regrid in between); then orc_new_dt: NewBlockTimeStep + Mesh::NewTimeStep */
void orc_advance(orc_mesh *m);
void orc_new_dt(orc_mesh *m);
void orc_set_time(orc_mesh *m, double t);
/* multi-level mesh: orc_initialize without the time step (one pass of the loop of
 * Mesh::Initialize with adaptive refinement) */
void orc_ml_boundaries(orc_mesh *m);
/* the blast problem's refinement measure per block (max |grad p|/p), maxeps[nb] */
void orc_refine_eps(const orc_mesh *m, double *maxeps);
/* fill the new multi-level mesh d from the old mesh s (one rank's
 * RedistributeAndRefineMeshBlocks): kind[n] 0 kept, 1 restricted from newtoold[n]..+7,
 * 2 prolongated from newtoold[n] with the face-field corrections ffc[nffc][3] =
 * (new block, receiving face, old block); copies time and dt. */
int orc_regrid(orc_mesh *d, orc_mesh *s, const int *newtoold, const int *kind, int nffc,
               const int *ffc);

/* per-cell SR conserved->primitive (adiabatic_mhd_sr.cpp:404-522) on independent
 * cells: cons[n][5] (D, E, M1..M3 in the reference's IDN,IEN,IM1..IM3 slots), bcc[n][3],
 * guess pgas[n]; out prim[n][5] and iterations[n] (-1 = not converged). */
void orc_sr_c2p_cells(long n, double gamma, double pgas_floor, const double *cons,
                      const double *bcc, const double *pgas_guess, double *prim,
                      int *iterations);

/* SR prim -> cons (adiabatic_mhd_sr.cpp:284-332) on independent cells: w[n][5] natural
 * slots (rho, u1, u2, u3, p), bcc[n][3] -> u[n][5] (D, M1..M3, E in IDN, IM1.., IEN). */
void orc_sr_prim_to_cons(long n, double gamma, const double *w, const double *bcc,
                         double *u);

#ifdef __cplusplus
}
#endif
#endif
