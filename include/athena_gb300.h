/* athena_gb300 — GB300-native MHD stage update behind a C ABI.
 *
 * The library advances every MeshBlock of a uniform, single-level, periodic 3-D mesh
 * through the reference's (Athena++) VL2 stage update on one GPU.  Arrays cross the
 * boundary as plain pointers in the reference's AthenaArray layout (last index fastest,
 * ghosts included, athena_arrays.hpp:140-143), with all MeshBlocks back to back in
 * lexicographic block order b = (lx3*nbx2 + lx2)*nbx1 + lx1:
 *   cells  u, w        [nb][5][nc3][nc2][nc1]      (ncN = nxN + 2*nghost)
 *          bcc         [nb][3][nc3][nc2][nc1]
 *   faces  b.x1f       [nb][nc3][nc2][nc1+1]
 *          b.x2f       [nb][nc3][nc2+1][nc1]
 *          b.x3f       [nb][nc3+1][nc2][nc1]
 * Host pointers are FP64 (Real = double, the reference's default build); the FP32
 * precision mode converts on upload/download.
 *
 * Every call returns an athgpu_status: 0 on success, a negative code on failure; the
 * message of the last failure on the calling thread is athgpu_last_error().
 * Calls on one context are not thread-safe (the reference runs one OpenMP thread per
 * MeshBlock at a time, task_list.cpp:71-82).
 */
#ifndef ATHENA_GB300_H_
#define ATHENA_GB300_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef int athgpu_status;
#define ATHGPU_OK 0
#define ATHGPU_ERR_ARG (-1)      /* invalid argument */
#define ATHGPU_ERR_CUDA (-2)     /* CUDA runtime error (message has the CUDA string) */
#define ATHGPU_ERR_UNSUPPORTED (-3)
#define ATHGPU_ERR_STATE (-4)    /* call out of order (e.g. stage before initialize) */

#define ATHGPU_HLLD 0            /* --flux=hlld  (hydro/rsolvers/mhd/hlld.cpp; relativistic:
                                    hlld_rel.cpp) */
#define ATHGPU_HLLE 1            /* --flux=hlle  (hydro/rsolvers/mhd/hlle_mhd.cpp) */
#define ATHGPU_LLF 2             /* --flux=llf   (hydro/rsolvers/mhd/llf_mhd.cpp; relativistic:
                                    llf_mhd_rel.cpp) */
#define ATHGPU_ROE 3             /* --flux=roe   (hydro/rsolvers/mhd/roe_mhd.cpp) */
#define ATHGPU_LHLLD 4           /* --flux=lhlld (hydro/rsolvers/mhd/lhlld.cpp, with
                                    hydro/calculate_velocity_differences.cpp); uniform
                                    meshes, Newtonian MHD */
#define ATHGPU_FP64 0            /* every operation in FP64: bit-identical to the reference */
#define ATHGPU_FP32 1            /* FP32 reconstruction/Riemann/divergence, compensated
                                    (Kahan) conserved update, FP64 CT and time step */

typedef struct athgpu_ctx athgpu_ctx;

/* Mesh and physics description.  Replaces the configuration the reference reads in
 * the Mesh/MeshBlock constructors (mesh.cpp:100-400, <mesh>/<meshblock>/<time>/<hydro>
 * input blocks, parameter_input.cpp) and fixes at create time what configure.py fixes at
 * compile time (NGHOST, the Riemann solver, configure.py:451-531). */
typedef struct {
  int nbx1, nbx2, nbx3;   /* MeshBlocks per direction (mesh/nx / meshblock/nx) */
  int nx1, nx2, nx3;      /* interior cells per MeshBlock (meshblock/nx1..3) */
  int nghost;             /* NGHOST: 2 for PLM, >= 3 for PPM (reconstruction.cpp:117-127) */
  int xorder;             /* time/xorder: 2 = PLM, 3 = PPM (stage 1 is donor cell) */
  int rsolver;            /* ATHGPU_HLLD, ATHGPU_HLLE, ATHGPU_LLF, ATHGPU_ROE or
                             ATHGPU_LHLLD */
  int precision;          /* ATHGPU_FP64 or ATHGPU_FP32 */
  int relativistic;       /* 1: special-relativistic MHD (-s): the HLLD, HLLE or LLF
                             solver (hlld_rel.cpp, hlle_mhd_rel.cpp, llf_mhd_rel.cpp),
                             FP64 Newman-Hamlin con2prim (adiabatic_mhd_sr.cpp) */
  double gamma;           /* hydro/gamma */
  double dfloor, pfloor;  /* hydro/dfloor, hydro/pfloor (adiabatic_mhd.cpp:29-30) */
  double cfl_number;      /* time/cfl_number */
  double tlim;            /* time/tlim: the time step is clipped to it (mesh.cpp:1271) */
  /* per-block coordinate arrays exactly as Coordinates holds them (coordinates.cpp:92-146):
   * x?f [nb][nc?+1] face positions, dx?f [nb][nc?] face spacings (host memory) */
  const double *x1f, *dx1f, *x2f, *dx2f, *x3f, *dx3f;
  /* SR floors and ceiling: hydro/sigma_max, beta_min (0 = off), gamma_max (reference
   * default 1000), adiabatic_mhd_sr.cpp:46-48 */
  double sigma_max, beta_min, gamma_max;
  /* Boundary flags of the mesh faces inner x1, outer x1, inner x2, outer x2, inner x3,
   * outer x3 (mesh/ix1_bc ... ox3_bc): ATHGPU_BC_PERIODIC (0, the zero-initialized
   * default), ATHGPU_BC_OUTFLOW, ATHGPU_BC_REFLECT (bvals/cc/outflow_cc.cpp,
   * bvals/cc/hydro/reflect_hydro.cpp, bvals/fc/outflow_fc.cpp, bvals/fc/reflect_fc.cpp,
   * applied as BoundaryValues::ApplyPhysicalBoundaries does, bvals/bvals.cpp:453-680). */
  int bc[6];
  /* 1: time/xorder = 3f, PiecewiseParabolicFast (reconstruct/ppm_fast.cpp): the PPM
   * interface values with Mignone's limiter and no floors (time/floor_ppm_fast false);
   * needs xorder 3.  0 (the zero-initialized default): the standard PPM. */
  int ppm_fast;
  /* time/integrator (task_list/time_integrator.cpp): ATHGPU_VL2 (0, the zero-initialized
   * default: van Leer predictor-corrector, donor cell on stage 1, :111-236) or ATHGPU_RK2
   * (Heun / SSPRK(2,2): xorder on both stages, stage weights beta = 1, 1/2 and the
   * register average u = (u* + u^n)/2 on stage 2, :338-465).  cfl_number must not
   * exceed the integrator's limit in 3-D (0.5 for vl2, 1.0 for rk2, :219-222, :445). */
  int integrator;
} athgpu_mesh_desc;
#define ATHGPU_VL2 0
#define ATHGPU_RK2 1
#define ATHGPU_BC_PERIODIC 0
#define ATHGPU_BC_OUTFLOW 1
#define ATHGPU_BC_REFLECT 2

/* Host-only check of a multi-level mesh description (no device needed): builds the
 * operation lists athgpu_set_multilevel would upload and checks every index they touch
 * against the array bounds.  nx[3] interior cells per block, bc[6] mesh-face flags, the
 * tables as for athgpu_set_multilevel.  counts (optional, 4 entries): operations of the
 * restriction, exchange and prolongation lists, flux-correction tasks. */
athgpu_status athgpu_ml_plan_check(const int* nx, int nghost, const int* bc, int nblocks,
                                   const int* nbr_table, const int* nbr_count,
                                   const int* nblevel, const long long* loc,
                                   long long* counts);

/* Turn the context into a multi-level mesh (static or adaptive mesh refinement;
 * Newtonian MHD, even nghost, even MeshBlock sizes >= 4).  Call after athgpu_create and
 * before athgpu_initialize.  The descriptor then lists the MeshBlocks as nbx1 = number of
 * blocks, nbx2 = nbx3 = 1, in the reference's gid order (MeshBlockTree::GetMeshBlockList,
 * mesh/meshblock_tree.cpp:336-355) with every block's own coordinates.  Per block:
 *   nbr_table[b][56][10]  its neighbour list (BoundaryBase::neighbor, bvals/bvals_base.cpp:
 *                         300-720): gid, level, ox1, ox2, ox3, type (0 face, 1 edge,
 *                         2 corner), fi1, fi2, fid, eid; nbr_count[b] entries used;
 *   nblevel[b][27]        neighbour levels at (ox3+1)*9+(ox2+1)*3+(ox1+1), -1 for none
 *                         (BoundaryBase::nblevel);
 *   loc[b][4]             level, lx1, lx2, lx3 (LogicalLocation);
 *   cx?f[b][ncc?+1], cdx?f[b][ncc?]  the coarse-buffer face coordinates (the reference's
 *                         MeshRefinement::pcoarsec, ncc = nx/2 + 2 nghost).
 * Replaces: the multilevel branches of TimeIntegratorTaskList (time_integrator.cpp:
 * 926-1162: flux and EMF correction, PROLONG), BoundaryValues::ProlongateBoundaries
 * (bvals/bvals_refine.cpp:97) and the buffer functions of bvals/cc and bvals/fc. */
athgpu_status athgpu_set_multilevel(athgpu_ctx* ctx, const int* nbr_table,
                                    const int* nbr_count, const int* nblevel,
                                    const long long* loc, const double* cx1f,
                                    const double* cdx1f, const double* cx2f,
                                    const double* cdx2f, const double* cx3f,
                                    const double* cdx3f);

/* Adaptive mesh refinement (multi-level contexts).
 * athgpu_refinement_eps: the blast problem's refinement measure (pgen/blast.cpp:413-443)
 * per MeshBlock from the current primitives: maxeps[b] (HOST, nblocks entries) = the
 * maximum over the interior and one ghost layer of |grad p| / p with centred
 * differences, in FP64.  The host turns it into refinement flags
 * (MeshRefinement::CheckRefinementCondition, mesh/mesh_refinement.cpp:1393-1455) and a new
 * block tree (Mesh::UpdateMeshBlockTree, mesh/amr_loadbalance.cpp:178-317).  Synchronous. */
athgpu_status athgpu_refinement_eps(athgpu_ctx* ctx, double* maxeps);
/* Move the mesh onto a new block list: one rank's Mesh::RedistributeAndRefineMeshBlocks
 * (mesh/amr_loadbalance.cpp:351-660) followed by its Initialize(2) (ghost exchange,
 * ProlongateBoundaries, W(U), NewBlockTimeStep + Mesh::NewTimeStep).
 *   desc        the new mesh (nbx1 = new block count, every block's coordinates; block size,
 *               nghost, precision, solver and boundary flags unchanged);
 *   nbr_table .. cdx3f   the new mesh's tables as for athgpu_set_multilevel;
 *   newtoold[n] the old block each new block n comes from (MeshBlockTree::GetMeshBlockList's
 *               previous gids); kind[n] 0: kept; 1: derefined, made from the eight old
 *               children newtoold[n] .. newtoold[n]+7 by restriction; 2: refined, prolongated
 *               from the old parent newtoold[n];
 *   ffc[nffc][3] (new child, receiving face 0..5, old block): the face field a new child
 *               takes from an old block of its own level across a face of its parent's
 *               boundary (PrepareAndSendFaceFieldCorrection, amr_loadbalance.cpp:1225-1340).
 *   after_cycle 1: the call follows athgpu_cycle, whose Mesh::NewTimeStep is taken back
 *               first (the reference makes it after the regrid: LoadBalancingAndAdaptive-
 *               MeshRefinement comes between time += dt and NewTimeStep, main.cpp:535-541;
 *               call athgpu_new_time_step next); 0: the clock is used as it is (the
 *               regrids of the initial refinement loop, mesh.cpp:1627-1958).
 * The maps are checked against the old and new locations.  The context handle stays valid;
 * its CUDA graph is rebuilt on the next athgpu_cycle.  Synchronous. */
athgpu_status athgpu_regrid(athgpu_ctx* ctx, const athgpu_mesh_desc* desc,
                            const int* nbr_table, const int* nbr_count, const int* nblevel,
                            const long long* loc, const double* cx1f, const double* cdx1f,
                            const double* cx2f, const double* cdx2f, const double* cx3f,
                            const double* cdx3f, const int* newtoold, const int* kind,
                            int nffc, const int* ffc, int after_cycle);
/* Mesh::NewTimeStep again from the block time steps of the last W(U) (the main loop's call
 * after a regrid, main.cpp:541, or the one after the initial refinement loop).
 * Synchronous. */
athgpu_status athgpu_new_time_step(athgpu_ctx* ctx);
/* ---- Adaptive mesh, host side (native) ----
 * The block tree of an adaptive mesh (MeshBlockTree, mesh/meshblock_tree.cpp), its block
 * list in gid order, every block's neighbour list, neighbour levels and fine and coarse
 * coordinates (BoundaryBase::SearchAndSetNeighbors, bvals/bvals_base.cpp:300-720;
 * Mesh::SetBlockSizeAndBoundaries, mesh/mesh.cpp:1984-2060; the uniform mesh generator),
 * the derefinement counters, the refinement flags and the tree update. */
typedef struct athgpu_amr athgpu_amr;
/* nx[3]: root-level cells of the mesh (mesh/nx1..3); nrbx[3]: root-grid blocks per
 * direction (MeshBlock size nx/nrbx, even, >= 4); nghost even; xmin/xmax[3] the mesh
 * extent; bc[6] the mesh-face flags; numlevel (mesh/numlevel); derefine_count
 * (mesh/derefine_count, the reference's default 10).  The mesh starts as the root grid. */
athgpu_status athgpu_amr_create(athgpu_amr** amr, const int* nx, const int* nrbx, int nghost,
                                const double* xmin, const double* xmax, const int* bc,
                                int numlevel, int derefine_count);
athgpu_status athgpu_amr_destroy(athgpu_amr* amr);
/* MeshBlockTree::AddMeshBlock: make (level, lx1, lx2, lx3) a block (static refinement). */
athgpu_status athgpu_amr_add_block(athgpu_amr* amr, int level, long long lx1, long long lx2,
                                   long long lx3);
athgpu_status athgpu_amr_nblocks(const athgpu_amr* amr, int* nblocks);
/* The current mesh's tables in the layouts of athgpu_set_multilevel: loc, nbr_table,
 * nbr_count, nblevel, coarse coordinates; the fine coordinates as the mesh description
 * takes them; any
 * pointer may be NULL. */
athgpu_status athgpu_amr_tables(const athgpu_amr* amr, long long* loc, int* nbr_table,
                                int* nbr_count, int* nblevel, double* x1f, double* dx1f,
                                double* x2f, double* dx2f, double* x3f, double* dx3f,
                                double* cx1f, double* cdx1f, double* cx2f, double* cdx2f,
                                double* cx3f, double* cdx3f);
/* MeshRefinement::CheckRefinementCondition for every block from the refinement
 * condition's results ret[b] in {1, 0, -1}: flags[b] (1 refine, -1 derefine, 0 keep);
 * updates the derefinement counters (mesh/mesh_refinement.cpp:1393-1455). */
athgpu_status athgpu_amr_flags(athgpu_amr* amr, const int* ret, int* flags);
/* Mesh::UpdateMeshBlockTree (mesh/amr_loadbalance.cpp:178-317): refinement, then the
 * derefinement of complete groups of flagged siblings.  *changed = 1 when the tree
 * changed; the new block list and its maps are then pending until athgpu_amr_accept. */
athgpu_status athgpu_amr_update(athgpu_amr* amr, const int* flags, int* changed);
/* Sizes and contents of the pending maps: the new block count, the face-field
 * corrections; newtoold[n], kind[n] and ffc[nffc][3] as athgpu_regrid takes them, and the
 * derefinement counters the new blocks carry. */
athgpu_status athgpu_amr_pending(const athgpu_amr* amr, int* nblocks_new, int* nffc);
athgpu_status athgpu_amr_pending_maps(const athgpu_amr* amr, int* newtoold, int* kind,
                                      int* ffc, int* deref_count);
/* Make the pending block list current (its tables are rebuilt). */
athgpu_status athgpu_amr_accept(athgpu_amr* amr);
athgpu_status athgpu_amr_deref_counts(const athgpu_amr* amr, int* deref_count);
/* The whole end-of-cycle refinement step on a multi-level context that holds this mesh:
 * the blast problem's refinement measure (athgpu_refinement_eps) with threshold thr
 * (pgen/blast.cpp:439-441), the flags, the tree update, and on a change the regrid
 * (athgpu_regrid with after_cycle) and, with after_cycle, athgpu_new_time_step.
 * *regridded = 1 when the mesh changed.  Synchronous. */
athgpu_status athgpu_amr_step(athgpu_ctx* ctx, athgpu_amr* amr, double thr, int after_cycle,
                              int* regridded);
/* Allocate all device registers of the stage update for the mesh (replaces the
 * Hydro/Field/EquationOfState/Reconstruction constructors, hydro.cpp:31-148,
 * field.cpp:27-105). */
athgpu_status athgpu_create(athgpu_ctx **ctx, const athgpu_mesh_desc *desc);
athgpu_status athgpu_destroy(athgpu_ctx *ctx);

/* Use a caller-provided CUDA stream (cudaStream_t passed as void*) for all work;
 * NULL restores the context's own stream. */
athgpu_status athgpu_set_stream(athgpu_ctx *ctx, void *stream);

/* Host <-> device copies of the conserved state U = phydro->u and the face field
 * B = pfield->b (the arrays MeshBlock::ProblemGenerator fills and restart.cpp:193-201
 * writes); any pointer may be NULL to skip that array.  Synchronous. */
athgpu_status athgpu_upload_state(athgpu_ctx *ctx, const double *u, const double *b1,
                                  const double *b2, const double *b3);
athgpu_status athgpu_download_state(athgpu_ctx *ctx, double *u, double *b1, double *b2,
                                    double *b3);
/* How the state calls above move data between host and device memory.  mode 0 (the
 * default): DMA copies in 64 MB chunks spread over several streams (copy engines), the
 * FP32 conversions on the device overlapping the remaining copies; mode 1: for FP32
 * contexts and page-locked host arrays, conversion kernels that read or write the host
 * arrays in place over the host link (no device staging).  Results are identical. */
athgpu_status athgpu_set_host_copy(athgpu_ctx *ctx, int mode);
/* Which part of the host arrays the state calls move.  ATHGPU_COPY_WHOLE (the default):
 * the whole arrays, ghost zones included.  ATHGPU_COPY_INTERIOR: per MeshBlock only the
 * x2/x3 range of its own cells (U; face arrays: its own faces, both bounding faces
 * included) with whole x1 rows, as one 3-D copy per chunk: the host's x2/x3 ghost zones
 * are neither read nor written, the x1 ghost cells of those rows are copied (download:
 * the exchanged values).  An upload must be followed by athgpu_initialize, which
 * recomputes every ghost zone on the device.  For the 32^3-cell, 3-ghost blocks of a
 * 256^3 mesh this moves 1.29 GB instead of 1.82 GB each way.  (athgpu_set_host_copy's
 * mode 1 applies to whole arrays only.) */
#define ATHGPU_COPY_WHOLE 0
#define ATHGPU_COPY_INTERIOR 1
athgpu_status athgpu_set_copy_extent(athgpu_ctx *ctx, int extent);

/* Initial primitives W = phydro->w (relativistic runs: also the initial guess of the
 * con2prim solve, which the reference seeds from its w / w1 registers,
 * adiabatic_mhd_sr.cpp:143-154).  Synchronous. */
athgpu_status athgpu_upload_prim(athgpu_ctx *ctx, const double *w);
/* primitives W = phydro->w and bcc = pfield->bcc of the last conserved->primitive call */
athgpu_status athgpu_download_prim(athgpu_ctx *ctx, double *w, double *bcc);

/* Tail of Mesh::Initialize (mesh.cpp:1698-1833 and :1959-1964): ghost exchange of U and
 * B, EquationOfState::ConservedToPrimitive over whole blocks, NewBlockTimeStep and
 * Mesh::NewTimeStep. */
athgpu_status athgpu_initialize(athgpu_ctx *ctx);

/* One VL2 stage for all MeshBlocks, i.e. the MHD task list of
 * TimeIntegratorTaskList::DoTaskListOneStage for stage 1 or 2
 * (time_integrator.cpp:904-1208): CalculateHydroFlux (donor cell on stage 1,
 * :1700-1703) -> Hydro::CalculateFluxes + RiemannSolver; CalculateEMF ->
 * Field::ComputeCornerE; Send/ReceiveFluxCorrection (same-level EMF averaging);
 * IntegrateHydro -> WeightedAve + Hydro::AddFluxDivergence; IntegrateField ->
 * WeightedAve + Field::CT; ghost exchange of U and B; Primitives ->
 * EquationOfState::ConservedToPrimitive; on stage 2 NewBlockTimeStep.  Asynchronous on
 * the context's stream. */
athgpu_status athgpu_stage(athgpu_ctx *ctx, int stage);

/* ncycles full cycles of the main loop (main.cpp:457-541): both stages, time += dt,
 * Mesh::NewTimeStep.  The cycle is captured once into a CUDA graph and replayed; dt and
 * time stay on the device.  Asynchronous on the context's stream. */
athgpu_status athgpu_cycle(athgpu_ctx *ctx, int ncycles);

/* Run whole cycles while time < tlim (main.cpp:457-458), at most max_cycles; returns the
 * number of cycles run in *ncycles_run. Synchronous. */
athgpu_status athgpu_run_until(athgpu_ctx *ctx, double tlim, int max_cycles,
                               int *ncycles_run);

/* Mesh::time and Mesh::dt (synchronous read). */
athgpu_status athgpu_get_clock(athgpu_ctx *ctx, double *time, double *dt);
athgpu_status athgpu_set_clock(athgpu_ctx *ctx, double time, double dt);

/* Wait for the context's stream. */
athgpu_status athgpu_synchronize(athgpu_ctx *ctx);

/* Cells whose density or pressure floor was applied by the conserved->primitive calls
 * that computed a time step since the last reset (adiabatic_mhd.cpp:65-84). */
athgpu_status athgpu_floor_count(athgpu_ctx *ctx, long long *count, int reset);

/* Device pointers of the registers, for callers that keep their data on the GPU
 * (u and ustar: Real = double in FP64 mode, float in FP32 mode).  The stages keep the
 * ghost cells of w, bcc and the face fields current but not those of u (W(U) reads a ghost
 * cell's conserved state from the block that owns it); athgpu_initialize and
 * athgpu_download_state refresh u's ghosts. */
typedef struct {
  void *u, *ulo, *w, *bcc;
  double *b1, *b2, *b3;
  int real_bytes;
} athgpu_device_state;
athgpu_status athgpu_device_state_ptrs(athgpu_ctx *ctx, athgpu_device_state *out);

/* Start of the relativistic con2prim solve in the stage's W(U) (the Newman-Hamlin
 * iteration of adiabatic_mhd_sr.cpp:404-522, seeded by the reference from the stale
 * pressure, :143-154):
 *   ATHGPU_C2P_START_STALE    the stale pressure (the reference's start; FP64 default);
 *   ATHGPU_C2P_START_REFINED  the stale pressure refined by FP32 iterations of the same
 *                             scheme (FP32 default);
 *   ATHGPU_C2P_START_NETWORK  the con2prim network's pressure (see athgpu_mlp_infer_tc;
 *                             BF16 tcgen05 evaluation of each 128-cell tile inside the
 *                             W(U) kernel), refined in FP32; params = ATHGPU_MLP_NPARAM
 *                             floats in host or device memory, copied into the context.
 * Any start other than the stale pressure that does not converge within the reference's 15
 * passes is followed by the reference's solve from the stale pressure, so the per-cell
 * outcome is the reference's whenever its start converges; the results of the starts
 * agree to the solver's tolerance (absolute 1e-12 on the pressure).  Relativistic contexts
 * only.  No counterpart in the reference (the start is a solver detail there).
 * Synchronous; the next athgpu_cycle captures its graph again. */
#define ATHGPU_C2P_START_STALE 0
#define ATHGPU_C2P_START_REFINED 1
#define ATHGPU_C2P_START_NETWORK 2
athgpu_status athgpu_set_c2p_start(athgpu_ctx *ctx, int start, const float *params);

/* Launch tiling of the x2/x3 flux sweeps: faces per thread along the sweep (the
 * autotuner's knob); 0 = heuristic default. */
athgpu_status athgpu_set_sweep_segment(athgpu_ctx *ctx, int seg_x2, int seg_x3);

/* Staging of the x3 sweep's stencil cells, face field and update operands in shared
 * memory: 0 (default) per-thread asynchronous copies (cp.async); 1 the TMA unit's bulk
 * copies (cp.async.bulk, one thread per CTA, completion on an mbarrier), on uniform meshes
 * whose k-planes and rows are 16-byte aligned (otherwise the call is accepted and the
 * sweep keeps per-thread copies).  Results are identical; athgpu_autotune times both. */
athgpu_status athgpu_set_x3_staging(athgpu_ctx *ctx, int bulk);
/* The staging the x3 sweep uses now (1: TMA bulk copies). */
athgpu_status athgpu_get_x3_staging(athgpu_ctx *ctx, int *bulk);

/* History output (HistoryOutput::WriteOutputFile, outputs/history.cpp:77-140): out[11]
 * (HOST) = volume-weighted sums over the interior cells of all MeshBlocks of mass, 1-mom,
 * 2-mom, 3-mom, 1-KE, 2-KE, 3-KE, tot-E, 1-ME, 2-ME, 3-ME, in FP64, reduced
 * deterministically (the same bits on every call; the order differs from the
 * reference's sequential sum).  Synchronous. */
#define ATHGPU_NHISTORY 11
athgpu_status athgpu_history(athgpu_ctx *ctx, double *out);

/* |div B| diagnostic of the face field (the reference's history diagnostic
 * WAbsDivergenceB, pgen/field_loop_poles.cpp:634-672): over the interior cells of all
 * MeshBlocks, |(sum over faces of +-area * B_normal) / volume| / (|B| / dl) with dl the
 * smallest edge length and |B| from the cell-centred field, cells with |B| = 0 skipped.
 * out[3] (HOST): the sum over cells (the reference's "wabsdivB" column summed over
 * blocks), the maximum, and the number of cells counted.  FP64 in both precision modes
 * (the face field is FP64); each cell's value is the reference's bit for bit, the sum is
 * reduced deterministically (the same bits on every call, not the reference's summation
 * order).  Synchronous. */
athgpu_status athgpu_divb(athgpu_ctx *ctx, double *out);

/* Run statistics (athgpu_stats): the div B diagnostic above, the cells floored by the
 * conserved->primitive calls that computed a time step (athgpu_floor_count), and the
 * relativistic con2prim counters of every W(U) call since the last reset: cells solved,
 * FP64 Newman-Hamlin loop passes summed over all attempts, cells re-solved from the
 * reference's start (the previous pressure) because their own start (FP32-refined or
 * learned) did not converge within the reference's 15 passes, and cells left unconverged
 * (the reference's failure branch: old primitives and floors, adiabatic_mhd_sr.cpp:
 * 156-164).  Replaces the diagnostics the reference prints or writes to history files;
 * the reference counts no con2prim iterations.  reset = 1 zeroes the counters after
 * reading them.  Synchronous. */
typedef struct {
  double divb_sum, divb_max;
  long long divb_cells;
  long long floor_cells;
  long long sr_cells, sr_passes, sr_fallbacks, sr_unconverged;
  int net_error;  /* 1: a tensor-core wait of the network start timed out (its cells then
                     started from the stale pressure) */
  int sweep_timeout;  /* 1: a bulk-copy wait of the x3 sweep timed out (results invalid) */
} athgpu_run_stats;
athgpu_status athgpu_stats(athgpu_ctx *ctx, athgpu_run_stats *out, int reset);

/* Autotuner of the sweep tiling: times `cycles` cycles (after one warm-up) for each
 * candidate segment length of the x2 sweep (the whole column, then halves down to 4
 * cells), keeps the fastest, then does the same for the x3 sweep, then times the x3
 * sweep's two stagings (athgpu_set_x3_staging) at those segments, and applies the choice
 * (*seg_x2, *seg_x3 receive the segments; either may be NULL).  The simulation state, the clock and
 * the primitive-buffer rotation are snapshotted on the device before and restored after,
 * so the call does not advance the run.  Allocates the snapshot (one copy of the state)
 * for the duration of the call.  Synchronous. */
athgpu_status athgpu_autotune(athgpu_ctx *ctx, int cycles, int *seg_x2, int *seg_x3);

/* Timing and self-check entry points (per-kernel profile, launch counts, regrid phases,
 * device checks of the integer-pipe arithmetic and of the Riemann solvers) are declared
 * in athena_gb300_diag.h; the library exports them beside these. */
const char *athgpu_last_error(void);
const char *athgpu_version(void);

/* ---- Per-operator entry points (one MeshBlock per call) ----
 * The bodies of the reference's per-MeshBlock member functions of the stage update, for a
 * caller that keeps its own TimeIntegratorTaskList, boundary exchange and EMF averaging
 * and replaces only these operators (the shim in athena_gb300/shim/ does so inside the
 * reference).  ctx: a context of ONE MeshBlock (athgpu_create with nbx1 = nbx2 = nbx3 = 1
 * and that block's coordinates, FP64; athgpu_initialize is not needed).  Arrays are the
 * block's AthenaArrays (ghosts included, layouts at the top of this file; fluxes
 * flx? [5][nc3][nc2][nc1+1] etc., edge EMFs e1 [nc3+1][nc2+1][nc1], e2 [nc3+1][nc2][nc1+1],
 * e3 [nc3][nc2+1][nc1+1]) in host or device memory.  Outputs are written over the
 * reference's index ranges only (their other elements come back unchanged).  Results are
 * the reference's bit for bit.  Synchronous. */
typedef struct {
  /* the face EMFs and CT weights Hydro::CalculateFluxes writes and Field::ComputeCornerE
   * reads (pfield->e3_x1f, e2_x1f, wght.x1f, e1_x2f, e3_x2f, wght.x2f, e1_x3f, e2_x3f,
   * wght.x3f; each shaped like the face field of its direction) */
  double *e3_x1f, *e2_x1f, *wght_x1f;
  double *e1_x2f, *e3_x2f, *wght_x2f;
  double *e1_x3f, *e2_x3f, *wght_x3f;
} athgpu_face_emfs;
/* Hydro::CalculateFluxes(w, b, bcc, order) (hydro.hpp:72-73, calculate_fluxes.cpp:38-415):
 * reconstruction of order 1 (donor cell), 2 (PLM), 3 (PPM, or fast PPM when the context
 * has ppm_fast) or 4 (fast PPM, time/xorder = 3f) and the context's Riemann solver on every
 * face the reference solves;
 * fluxes into flx1..3, face EMFs and CT weights into emfs.  dt = Mesh::dt (the CT weights,
 * hydro.cpp:154-158). */
athgpu_status athgpu_op_calculate_fluxes(athgpu_ctx *ctx, int order, double dt,
                                         const double *w, const double *bcc,
                                         const double *b1, const double *b2,
                                         const double *b3, double *flx1, double *flx2,
                                         double *flx3, athgpu_face_emfs *emfs);
/* Field::ComputeCornerE(w, bcc) (field.hpp:66, calculate_corner_e.cpp:28-236): the edge
 * EMFs e1, e2, e3 (pfield->e.x1e, x2e, x3e) from the face EMFs and weights and the
 * cell-centred E of w and bcc. */
athgpu_status athgpu_op_corner_e(athgpu_ctx *ctx, const double *w, const double *bcc,
                                 const athgpu_face_emfs *emfs, double *e1, double *e2,
                                 double *e3);
/* Hydro::AddFluxDivergence(wght, u_out) (hydro.hpp:67, add_flux_divergence.cpp:39-96):
 * u -= wght * div(flux) / vol over the interior. */
athgpu_status athgpu_op_add_flux_divergence(athgpu_ctx *ctx, double wght, const double *flx1,
                                            const double *flx2, const double *flx3,
                                            double *u);
/* Field::CT(wght, b_out) (field.hpp:63, ct.cpp:31-116): the face fields b1..b3 updated
 * in place from the edge EMFs. */
athgpu_status athgpu_op_ct(athgpu_ctx *ctx, double wght, const double *e1, const double *e2,
                           const double *e3, double *b1, double *b2, double *b3);
/* EquationOfState::ConservedToPrimitive(cons, prim_old, b, prim, bcc, pco, il, iu, jl, ju,
 * kl, ku) (eos.hpp:37-40; adiabatic_mhd.cpp:41-90, relativistic: adiabatic_mhd_sr.cpp:
 * 72-272, seeded from prim's previous contents): bcc from the faces, prim, and cons
 * rewritten where floors apply, over the given cell range.  *nfloored (may be NULL):
 * cells whose floors applied (relativistic: also failed solves). */
athgpu_status athgpu_op_con2prim(athgpu_ctx *ctx, double *cons, const double *b1,
                                 const double *b2, const double *b3, double *prim,
                                 double *bcc, int il, int iu, int jl, int ju, int kl, int ku,
                                 long long *nfloored);
/* Hydro::NewBlockTimeStep() (hydro.hpp:66, new_blockdt.cpp:45-230), ideal MHD or SR:
 * *dt_out = cfl_number times the minimum over interior cells of dx_d / (|v_d| + c_f)
 * (the value the reference stores in MeshBlock::new_block_dt_). */
athgpu_status athgpu_op_new_block_dt(athgpu_ctx *ctx, const double *w, const double *bcc,
                                     const double *b1, const double *b2, const double *b3,
                                     double *dt_out);

/* ---- Learned initial guess for the special-relativistic con2prim ----
 * A 5 -> 64 -> 64 -> 2 SiLU network predicts (log(p_gas/E), log(Lorentz factor)) from the
 * features of athgpu_sr_features; its start replaces the previous-pressure start of the
 * Newman-Hamlin iteration in EquationOfState::ConservedToPrimitive
 * (adiabatic_mhd_sr.cpp:143-154, solve :404-522).  No counterpart in the reference.
 * Parameters are ATHGPU_MLP_NPARAM floats (device): W1[64][5], b1[64], W2[64][64], b2[64],
 * W3[2][64], b3[2], then input means[5], input scales[5], output means[2], output
 * scales[2] (inputs and targets are standardized as (v - mean)/scale).
 * Per-cell arrays are cell-major: cons[n][5] = (D, M1, M2, M3, E) with E the total energy
 * density including rest mass, bcc[n][3], prim[n][5] = (rho, u1, u2, u3, p_gas) (the
 * reference's slots IDN, IVX, IVY, IVZ, IPR; u^i the spatial 4-velocity), features[n][5].
 * All pointers are DEVICE pointers; calls are asynchronous on `stream` unless stated. */
#define ATHGPU_MLP_NPARAM 4688

/* features[n][5] = (log(D/E), log(M^2/E^2), log(B^2/E), (M.B)^2/(M^2 B^2),
 * log((E - sqrt(M^2 + D^2))/E)), the last difference formed in FP64. */
athgpu_status athgpu_sr_features(long long n, const double *cons, const double *bcc,
                                 float *features, void *stream);

/* Network outputs out[n][2] (de-standardized) for raw features[n][5], evaluated by the
 * same BF16 tensor-core code (FP32 accumulation) as the fused con2prim. */
athgpu_status athgpu_mlp_infer(long long n, const float *params, const float *features,
                               float *out, void *stream);

/* The same network on the fifth-generation tensor cores: persistent CTAs of 128 threads
 * evaluate 128-row tiles with tcgen05.mma (BF16 operands in shared memory, FP32
 * accumulators in tensor memory).  Synchronous; ATHGPU_ERR_CUDA if a tensor-core wait
 * timed out (the outputs are then NaN). */
athgpu_status athgpu_mlp_infer_tc(long long n, const float *params, const float *features,
                                  float *out, void *stream);

/* Flag or-ed into athgpu_sr_c2p_cells' mode: evaluate the network with warp-level
 * mma.sync tiles instead of the default tcgen05 path. */
#define ATHGPU_C2P_WARP_MMA 0x100

/* Newman-Hamlin root find per independent cell.  mode 0: start from pgas_guess[c] (the
 * reference's start) or from pfloor when pgas_guess is NULL; mode 1: start from the
 * network; mode 2: network start refined by at most 12 FP32 iterations of the same scheme;
 * mode 3: the mode-0 start refined the same way (no network; params may be NULL).
 * Two launches: loop indices [0, phase1_iterations) for every cell (0 = default: 7 in
 * mode 0, 4 in modes 1-2), then the cells still iterating, resumed exactly.  Mode 0 is the
 * reference's solve.  Modes 1-3 solve a cell again from the mode-0 start when their start
 * does not converge within the reference's 15 FP64 iterations, and then from that
 * attempt's last iterate (*fallbacks, may be NULL, counts cells that needed it).
 * prim[n][5] as ConservedToPrimitiveNormal leaves it (zeros before the solve),
 * iters64[n] = FP64 loop passes over all attempts (-1 = not converged), iters32[n] (may
 * be NULL) = FP32 refinement passes.  Modes 1-2 evaluate the network on the tcgen05
 * tensor cores (one 128-cell tile per CTA) unless ATHGPU_C2P_WARP_MMA is set.  Allocates a
 * queue of 40 bytes per cell with cudaMallocAsync on the stream and synchronizes the
 * stream at the end (ATHGPU_ERR_CUDA if a tensor-core wait timed out). */
athgpu_status athgpu_sr_c2p_cells(long long n, double gamma, double pfloor, const double *cons,
                                  const double *bcc, const double *pgas_guess,
                                  const float *params, int mode, int phase1_iterations,
                                  double *prim, int *iters64, int *iters32, int *fallbacks,
                                  void *stream);

/* Gradient of the mean squared error over batch rows and both outputs of standardized
 * inputs x[batch][5] against standardized targets t[batch][2] with respect to the 4674
 * trainable parameters: grad[4674], loss[1].  FP32 forward/backward kernels (the
 * batch-chunk partial sums of the weight gradient are added atomically, so the last bits
 * may vary between calls); allocates scratch with cudaMallocAsync on the stream. */
athgpu_status athgpu_mlp_loss_grad(const float *params, const float *x, const float *t,
                                   int batch, float *grad, float *loss, void *stream);

/* Adam training (beta 0.9/0.999, eps 1e-8, step size decaying from lr to lr/50 on a
 * cosine) on n (features, raw targets) rows for `steps`
 * mini-batches of `batch` rows drawn with replacement (seeded); params updated in place
 * (standardization entries must be filled in).  loss_history (HOST, may be NULL) receives
 * the per-step loss.  Synchronous. */
athgpu_status athgpu_mlp_train(const float *features, const float *targets, long long n,
                               float *params, int steps, int batch, float lr,
                               unsigned long long seed, float *loss_history, void *stream);

/* Conserved->primitive over whole MeshBlocks plus the first CFL time step, for callers
 * that cannot let a library allocate device memory: hosts whose device memory belongs
 * to their own pool allocator, real-time loops that forbid allocation latency, plugins
 * that must leave the device heap untouched.  No counterpart in the reference: it has no
 * device memory; this computes what EquationOfState::ConservedToPrimitive
 * (adiabatic_mhd.cpp:41-90) followed by Hydro::NewBlockTimeStep (new_blockdt.cpp:45-230)
 * and the block minimum of Mesh::NewTimeStep compute, bit for bit like
 * athgpu_initialize, on arrays the caller owns.
 *
 * All array arguments are DEVICE pointers in the layout at the top of this file: u (may be
 * rewritten where the density/pressure floors apply), face field b1/b2/b3, outputs w and
 * bcc, per-block spacings dx?f [nblocks][nc?], and dt_out (one double: cfl_number times the
 * minimum over interior cells of dx/(|v|+c_f)).  Asynchronous on `stream` (a
 * cudaStream_t, NULL = legacy default stream).
 *
 * Allocates nothing: no cudaMalloc/cudaFree and no allocating library routine.  The
 * reduction's scratch is a fixed array of 65,536 doubles inside the library, held by every
 * GPU that loads it until the process exits, so a call covers at most
 * ATHGPU_NOALLOC_MAX_CELLS cells (ghosts included, all blocks) and larger meshes are
 * rejected with ATHGPU_ERR_ARG; meshes with nx2 or nx3 < 2 are rejected with
 * ATHGPU_ERR_UNSUPPORTED, as by athgpu_create.  The first call in each CUDA context (per
 * device, normally the runtime's primary context) looks up the array's device address
 * (cudaGetSymbolAddress) with that context current; make that first call before any
 * stream capture.  Every call on a device shares the one array, which keeps the last
 * call's contents: calls that overlap on the GPU (different streams, no ordering) race;
 * order them on one stream or with events. */
#define ATHGPU_NOALLOC_MAX_CELLS 16777216LL
athgpu_status athgpu_con2prim_timestep_noalloc(
    int nblocks, int nx1, int nx2, int nx3, int nghost, double gamma, double dfloor,
    double pfloor, double cfl_number, const double *dx1f, const double *dx2f,
    const double *dx3f, const double *b1, const double *b2, const double *b3, double *u,
    double *w, double *bcc, double *dt_out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* ATHENA_GB300_H_ */
