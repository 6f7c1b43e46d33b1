/* aither_gb300 — GB300-native per-iteration structured-grid solver step.
 *
 * C ABI between the host side (the reference's procBlock / linearSolver /
 * gridLevel call surface, input and Plot3D formats) and the sm_103a CUDA
 * kernels.  Plain pointers and sizes only; every function returns an int
 * status (0 = ATH_OK, negative = error) and never exits the process.  The
 * text of the last error of a thread is returned by ath_last_error().
 *
 * Reference interfaces replaced (paths inside the reference project):
 *   ath_setup_from_input   input::ReadInput (src/input.cpp:167) +
 *                          ReadP3dGrid (src/plot3d.cpp:363) + procBlock ctor
 *                          geometry (src/procBlock.cpp:59) +
 *                          AssignGhostCellsGeom (src/procBlock.cpp:2160) +
 *                          GetConnectionBCs (src/boundaryConditions.cpp:500)
 *                          + HyperplaneReorder (src/utility.cpp:377)
 *   ath_batch_iterate      mgSolution::Iterate (src/mgSolution.cpp:246) with
 *                          the norm reductions of src/main.cpp:254-271
 *   ath_batch_fill_ghosts  gridLevel::GetBoundaryConditions
 *                          (src/gridLevel.cpp:287)
 *   ath_batch_residual     gridLevel::CalcResidual (src/gridLevel.cpp:372)
 *                          -> procBlock::CalcResidualNoSource
 *                          (src/procBlock.cpp:6111)
 *   ath_batch_timestep     gridLevel::CalcTimeStep (src/gridLevel.cpp:240)
 *   ath_batch_diag_invert  gridLevel::InvertDiagonal (src/gridLevel.cpp:402)
 *                          -> linearSolver::AddDiagonalTerms / Invert
 *                          (src/linearSolver.cpp:146,177)
 *   ath_batch_relax        lusgs::Relax (src/linearSolver.cpp:430) with
 *                          LUSGS_Forward / LUSGS_Backward (:341,:385)
 *   ath_batch_update       gridLevel::UpdateBlocks (src/gridLevel.cpp:418)
 *                          -> procBlock::UpdateBlock (src/procBlock.cpp:826)
 *   ath_batch_matrix_resid linearSolver::Residual (src/linearSolver.cpp:92)
 */
#ifndef AITHER_GB300_H
#define AITHER_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ATH_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
enum {
  ATH_RETIRED = 1,        /* (per-solve status) the solve had retired before
                             this iteration: converged or nonphysical */
  ATH_OK = 0,
  ATH_ERR_ARG = -1,       /* invalid argument */
  ATH_ERR_IO = -2,        /* file could not be read or parsed */
  ATH_ERR_UNSUPPORTED = -3,
  ATH_ERR_CUDA = -4,      /* a CUDA runtime call failed */
  ATH_ERR_NOMEM = -5,     /* device memory budget exceeded */
  ATH_ERR_NONPHYSICAL = -6, /* non-finite or non-positive density/pressure */
  ATH_ERR_TIMEOUT = -7    /* a bounded device-side wait gave up */
};

/* ---- enumerations mirroring the reference's string keywords ------------ */
enum { ATH_EQN_EULER = 0, ATH_EQN_NAVIER_STOKES = 1, ATH_EQN_RANS = 2 };
enum { ATH_RECON_CONSTANT = 0, ATH_RECON_MUSCL = 1, ATH_RECON_WENO = 2,
       ATH_RECON_WENOZ = 3 };
enum { ATH_LIMITER_NONE = 0, ATH_LIMITER_MINMOD = 1,
       ATH_LIMITER_VANALBADA = 2 };
enum { ATH_FLUX_ROE = 0, ATH_FLUX_AUSM = 1 };
/* linear solvers (input::AssignLinearSolver, src/input.cpp:843): LU-SGS and
 * block LU-SGS hyperplane sweeps; DP-LUR and block DP-LUR Jacobi sweeps */
enum { ATH_SOLVER_LUSGS = 0, ATH_SOLVER_BLUSGS = 1, ATH_SOLVER_DPLUR = 2,
       ATH_SOLVER_BDPLUR = 3 };
enum { ATH_TURB_NONE = 0, ATH_TURB_SST2003 = 1, ATH_TURB_KW2006 = 2 };

/* boundary condition types (reference keyword in brackets) */
enum {
  ATH_BC_SLIP_WALL = 0,           /* slipWall */
  ATH_BC_VISCOUS_WALL = 1,        /* viscousWall */
  ATH_BC_CHARACTERISTIC = 2,      /* characteristic */
  ATH_BC_STAGNATION_INLET = 3,    /* stagnationInlet */
  ATH_BC_PRESSURE_OUTLET = 4,     /* pressureOutlet */
  ATH_BC_SUPERSONIC_INFLOW = 5,   /* supersonicInflow */
  ATH_BC_SUPERSONIC_OUTFLOW = 6,  /* supersonicOutflow */
  ATH_BC_PERIODIC = 7,            /* periodic (connection) */
  ATH_BC_INTERBLOCK = 8,          /* interblock (connection) */
  ATH_BC_INLET = 9,               /* inlet (reflecting form) */
  /* block-edge ghost cells (procBlock::AssignInviscidGhostCellsEdge /
   * AssignViscousGhostCellsEdge): copy of src, average of src and src2,
   * or a slip-wall reflection of src across a ghost-layer face */
  ATH_EDGE_COPY = 20,
  ATH_EDGE_AVG = 21,
  ATH_EDGE_SLIP = 22
};

/* arithmetic of the per-iteration path */
enum {
  ATH_PREC_FP64 = 0,  /* everything in FP64 */
  ATH_PREC_MIXED = 1  /* FP32 reconstruction/fluxes/sweeps inside an FP64
                         defect-correction loop (FP64 residual assembly,
                         conserved update and norms) */
};

/* ---- host-side setup ---------------------------------------------------- */
typedef struct ath_setup ath_setup;

/* One ghost-cell assignment.  All ghost cells of a block are filled by a
 * list of these, applied in order (boundary states first, then connection
 * copies, then block-edge cells). */
typedef struct {
  int64_t dst;        /* padded cell index of the ghost cell (own block) */
  int64_t src;        /* padded cell index of the donor cell */
  int32_t src_block;  /* block of the donor (connections), else own block */
  int32_t type;       /* ATH_BC_* */
  int32_t layer;      /* 1..ng; edge ops: phase (layer3-1)*ng + layer2-1 */
  int32_t dir;        /* 0,1,2 = boundary normal direction i,j,k */
  int32_t lower;      /* 1 = lower surface (normal flipped outward) */
  int32_t state;      /* index into the solve's boundary-state table */
  int64_t face;       /* padded face index of the boundary face (dir) */
  int64_t src2;       /* edge cells: second donor; viscous-wall cells: the
                         wall-adjacent cell (-1 when unused) */
} ath_ghost_op;

/* A cell next to a nonreflecting boundary surface. */
typedef struct {
  int64_t cell;    /* padded index of the boundary-adjacent cell */
  int64_t face;    /* padded face index (direction dir) of its boundary face */
  int32_t surf;    /* block-local index of the surface */
  int32_t dir;     /* boundary normal direction */
  int32_t lower;   /* 1 = lower surface (outward normal flipped) */
  int32_t pad;
} ath_nr_cell;

/* Boundary-state data, nondimensional (reference inputStates.cpp). */
typedef struct {
  int32_t tag;
  int32_t type;
  double rho, u, v, w, p;      /* characteristic / supersonic inflow */
  double p0, t0, dir[3];       /* stagnationInlet */
  double p_out;                /* pressureOutlet */
  double wall_u, wall_v, wall_w, wall_t, wall_q; /* viscousWall; wall_q is the
                                                    heat flux over (a_ref/l_ref)^3 */
  int32_t isothermal, heat_flux;
  double turb_intensity, eddy_visc_ratio;
  /* inlet / pressureOutlet with nonreflecting=true: LODI relaxation towards
   * the specified state over lengthScale (nondimensional) */
  int32_t nonreflecting, pad_nr;
  double length_scale;
} ath_bc_state;

/* Per-solve physics and scheme constants, nondimensional. */
typedef struct {
  int32_t eqn, recon, limiter, flux, solver, turb;
  int32_t nv, ng, sweeps;
  double kappa, cfl_start, cfl_step, cfl_max, theta, zeta, relax;
  double gas_r, gas_n, gas_hf;          /* calorically perfect, one species */
  double mu_c1, mu_s, mu_ref, t_ref;    /* Sutherland viscosity constants,
                                           mu_ref = mixture reference viscosity */
  double r_ref, a_ref, l_ref;           /* dimensional reference values */
  double visc_scale;                    /* transport NondimScaling */
  double visc_cfl_coeff;                /* input::ViscousCFLCoefficient */
  double k_c1, k_s, k_ref;              /* Sutherland conductivity constants,
                                           k_ref = conductivity reference */
  int32_t nstates;
  const ath_bc_state *states;
  /* time integration (timeIntegration, src/input.cpp:259-266): theta and
   * zeta above are implicitEuler 1/0, crankNicholson 0.5/0, bdf2 1/0.5 (with
   * the time n-1 solution: multilevel = 1); dt_global is the nondimensional
   * global time step (timeStep * a_ref / l_ref; 0: local time stepping from
   * the CFL), dual_cfl the dual-time CFL (0: none), nl_iters the nonlinear
   * iterations per time step */
  double dt_global, dual_cfl;
  int32_t nl_iters, multilevel;
  /* multigrid (multigridLevels, multigridCycle; mgSolution src/mgSolution.cpp:
   * 160-207): grid levels (1: none) and the cycle index (1 V, 2 W) */
  int32_t mg_levels, mg_cycle;
} ath_solve_view;

/* Read-only view of one block of a setup; arrays are host memory owned by
 * the setup.  Padded layout: cell (i,j,k), i in [-ng, ni+ng), has index
 * (i+ng) + NI*((j+ng) + NJ*(k+ng)), NI = ni+2ng.  Face arrays of direction
 * d have one more entry along d.  Vectors are stored as separate
 * components (x plane, then y, then z). */
typedef struct {
  int32_t ni, nj, nk, ng, nv, solve;
  int64_t ncell_padded;
  int64_t nface_padded[3];
  const double *vol;        /* [ncell_padded] */
  const double *center;     /* [3][ncell_padded] */
  const double *width;      /* [3][ncell_padded] cell widths i,j,k */
  const double *farea[3];   /* [4][nface_padded[d]]: unit x,y,z, magnitude */
  const double *wall_dist;  /* [ncell_padded] */
  const double *state0;     /* initial primitive, padded AoS [cell][nv] */
  int32_t nops;
  const ath_ghost_op *ops;          /* boundary states and connections */
  int32_t nedge_ops;
  const ath_ghost_op *edge_ops;     /* block-edge ghosts, by phase */
  int32_t nvops;
  const ath_ghost_op *vops;         /* viscous-wall ghosts (viscous flux) */
  int32_t nvedge_ops;
  const ath_ghost_op *vedge_ops;    /* block-edge ghosts after vops */
  int32_t nplanes;
  const int32_t *plane_offsets; /* [nplanes+1] */
  const int32_t *plane_cells;   /* padded cell index, hyperplane order */
  /* per padded cell: bit 2d (lower face of direction d) or 2d+1 (upper
   * face) is set when the neighbour across that face enters the implicit
   * off-diagonal sums: it is a physical cell or the face lies on a
   * periodic/interblock connection (procBlock::ImplicitLower/Upper). */
  const uint8_t *nbr_mask;
  /* cells next to the block's nonreflecting boundary surfaces, surface by
   * surface, each surface in the reference's k, j, i loop order
   * (procBlock::GetGhostStates src/procBlock.cpp:6235): the average and
   * largest outward normal Mach number of each surface enter its ghost
   * states; the ghost ops of such a surface carry its index in src2 */
  int32_t n_nr;
  const ath_nr_cell *nr;
} ath_block_view;

/* Load a case from the reference's input file format (and the Plot3D grid
 * it names, read from the input file's directory).  A setup may hold many
 * independent solves: ath_setup_append() adds the blocks of another input
 * file as a new solve. */
int ath_setup_from_input(const char *inp_path, ath_setup **out);
/* The same with the physical cells' and faces' geometry (volumes,
 * centroids, face areas and centres: the procBlock constructor's
 * plot3dBlock::Volume / Centroid / FaceArea* / FaceCenter*, src/plot3d.cpp:
 * 60-360) and the physical cells' wall distance (procBlock::CalcWallDistance,
 * src/procBlock.cpp:6030) computed on CUDA device `device`, bit for bit the
 * host setup's; blocks appended later (ath_setup_append) use the device too. */
int ath_setup_from_input_dev(const char *inp_path, int device, ath_setup **out);
int ath_setup_append(ath_setup *setup, const char *inp_path);
int ath_setup_destroy(ath_setup *setup);
int ath_setup_counts(const ath_setup *setup, int *nsolves, int *nblocks,
                     int64_t *ncells);
int ath_setup_block(const ath_setup *setup, int block, ath_block_view *out);
int ath_setup_solve(const ath_setup *setup, int solve, ath_solve_view *out);
/* Replace the initial primitive state (nondimensional, AoS over physical
 * cells, k slowest, i fastest). */
int ath_setup_set_state(ath_setup *setup, int block, const double *prim);

/* Multigrid levels (multigridLevels > 1; mgSolution::ConstructMultigrids
 * src/mgSolution.cpp:86, gridLevel::Coarsen src/gridLevel.cpp:440).  Level 0
 * is the setup itself; level l holds, in the order of the solves, the l-th
 * coarser grid of every solve with more than l levels: each coarse block
 * keeps every fine node a boundary surface starts or ends on and otherwise
 * every other node (procBlock::GetCoarseMeshAndBCs src/procBlock.cpp:6471),
 * with its own geometry, boundary and connection bookkeeping.  The
 * ath_setup_level_* calls are ath_setup_counts / _block / _solve of a
 * level; views stay valid while the setup lives. */
int ath_setup_levels(const ath_setup *setup, int *nlevels);
int ath_setup_level_counts(const ath_setup *setup, int level, int *nsolves, int *nblocks,
                           int64_t *ncells);
int ath_setup_level_block(const ath_setup *setup, int level, int block, ath_block_view *out);
int ath_setup_level_solve(const ath_setup *setup, int level, int solve, ath_solve_view *out);

/* Transfer between block `block` of level `level` and its block on level
 * level+1: per fine physical cell (k, j, i order) the coarse physical cell
 * it lies in (i + ni*(j + nj*k) of the coarse block), its weight in the
 * volume-weighted restriction (fine volume over the summed volume of the
 * fine cells of that coarse cell) and its 7 trilinear prolongation
 * coefficients from the coarse cell's nodes (TrilinearInterpCoeff
 * src/utility.cpp:633), [cell][7]. */
typedef struct {
  int32_t coarse_block, pad;
  int64_t ncells;
  const int32_t *coarse_cell;
  const double *volfac;
  const double *coef;
} ath_mg_map;
int ath_setup_mg_map(const ath_setup *setup, int level, int block, ath_mg_map *out);

/* ---- device context and batches ----------------------------------------- */
typedef struct ath_ctx ath_ctx;
typedef struct ath_batch ath_batch;

typedef struct {
  double l2[7];        /* sqrt(sum over cells of R^2), per equation */
  double linf;         /* max residual entry */
  int32_t linf_block, linf_i, linf_j, linf_k, linf_eqn;
  double matrix_resid; /* linear-system residual (0 when not computed) */
  double cfl;
  int32_t status;      /* ATH_OK or ATH_ERR_NONPHYSICAL for this solve */
  /* integrated wall forces of the iteration's residual, summed over the
   * viscous-wall faces: p_w A (area vector, x y z) then tau_w |A| (x y z);
   * zero for solves without viscous walls.  The reference keeps the wall
   * data (procBlock::WallPressure / WallShearStress, include/procBlock.hpp:
   * 525-552) but does not integrate it. */
  double force[6];
} ath_norms;

int ath_ctx_create(int device, size_t hbm_budget_bytes, ath_ctx **out);
int ath_ctx_destroy(ath_ctx *ctx);
/* FP64 issue-rate peak of the context's GPU, measured: chains of
 * independent fused multiply-adds on every SM (2 FLOP each), best of
 * `reps` timed launches; *tflops receives FP64 TFLOP/s.  The second bound
 * of the solver's roofline beside HBM bandwidth (its FP64 kernels run
 * divisions and square roots as FMA sequences). */
int ath_ctx_fp64_peak(ath_ctx *ctx, int reps, double *tflops);
const char *ath_last_error(void);

/* Copy a setup to the device.  precision = ATH_PREC_*.  flags: bit 0 =
 * compute the logged matrix residual every iteration (the reference always
 * does, src/linearSolver.cpp:470); bit 1 (ATH_BATCH_FAST_FACES) = FP64
 * batches evaluate the MUSCL reconstruction and the Roe flux of solves
 * without turbulence equations in a rearranged form with fewer divisions
 * and square roots, and run the faces, the cell kernel, the scalar LU-SGS
 * hyperplane sweeps and the update with contracted multiply-adds (FP64
 * throughout; equal to the reference to roundoff, about 1e-15 per face,
 * instead of bit for bit); bit 2 (ATH_BATCH_OUTPUT_GRADS) = every residual
 * also keeps the cells' velocity, temperature, density, pressure, k and
 * omega gradients for output (ATH_FIELD_GRADS). */
enum { ATH_BATCH_MATRIX_RESID = 1, ATH_BATCH_FAST_FACES = 2, ATH_BATCH_OUTPUT_GRADS = 4 };
int ath_batch_create(ath_ctx *ctx, const ath_setup *setup, int precision,
                     int flags, ath_batch **out);
/* The flags a batch was created with. */
int ath_batch_flags(const ath_batch *batch, int *flags);
int ath_batch_destroy(ath_batch *batch);

/* Run n nonlinear iterations on every solve of the batch.  norms_h receives
 * n * nsolves entries (iteration-major) when not NULL.  The iteration
 * counter advances (CFL ramp, src/input.cpp:647). */
int ath_batch_iterate(ath_batch *batch, int n, ath_norms *norms_h);

/* Per-solve record of a run to convergence. */
typedef struct {
  int64_t iterations;  /* iterations the solve ran in this batch */
  double drop;         /* last total L2 / first-iteration total L2; the total
                          L2 is sqrt(sum over equations of l2^2) */
  double ms;           /* device time from the end of the solve's first
                          iteration in this batch to its retirement (or to
                          now while it runs) */
  int32_t converged;   /* 1: drop reached, -1: retired nonphysical, 0: running */
  int32_t pad;
} ath_converge_info;

/* Runs iterations until every solve has retired or max_iters iterations
 * have passed.  A solve retires, on the device and in the iteration where
 * it happens, when its total L2 norm falls to `drop` times that of its first
 * iteration (the reference normalises its residual history by the first
 * iteration, src/main.cpp:254-271) or when its state turns nonphysical;
 * from then on its kernels skip their work, so a solve's result does not
 * depend on what else shares the batch.  The host checks every
 * `check_every` iterations.  info: nsolves entries (may be NULL). */
int ath_batch_converge(ath_batch *batch, int max_iters, double drop, int check_every,
                       ath_converge_info *info);
/* Retirement target of one solve (0 = never), or reactivation: active = 1
 * resumes a retired solve from its current state. */
int ath_batch_set_target(ath_batch *batch, int solve, double drop, int active);
/* Current per-solve records (nsolves entries). */
int ath_batch_solve_info(ath_batch *batch, ath_converge_info *info);

/* Autotuner of the LU-SGS sweep shape: times `reps` graph-captured
 * iterations for each candidate and keeps the fastest -- one launch per
 * hyperplane with CTAs of 32, 64, 128 or 256 threads (a thread per cell or
 * lane groups; lane groups also with the solves as 2 or 4 concurrent
 * chains, and lane groups below 32,768 cells per plane with a thread per
 * cell above), the persistent
 * cluster sweep (one launch per pass; a thread-block cluster of 1, 2, 4 or
 * 8 CTAs of 256 threads per solve walks the solve's hyperplanes with
 * cluster barriers), or the persistent tile-queue sweep (one launch per
 * pass over all solves: each warp claims (solve, hyperplane) tiles of one
 * to eight warp rounds from an atomic ticket in step order, a tile waiting
 * for the tiles of the previous step that hold its cells' swept-side
 * neighbours).  Every shape gives bit-identical results.  The solution,
 * per-solve counters and CFL are restored afterwards, so tuning does not
 * advance the solves.  The chosen CTA size (tile size for the tile queue)
 * is written to *sweep_threads (may be NULL).  A new batch starts with the
 * persistent cluster sweep sized to its largest hyperplane. */
int ath_batch_autotune(ath_batch *batch, int reps, int *sweep_threads);
/* Current sweep shape: mode 1 persistent cluster sweep (cluster = CTAs per
 * solve), 0 one launch per hyperplane, 2 one launch per hyperplane with a
 * group of lanes per scalar-solve cell, one per neighbour term (modes 0 and
 * 2: cluster = the number of concurrent chains, 1, 2 or 4, the batch's
 * solves split into groups balanced by cells, each group's hyperplanes a
 * chain of launches on its own stream; 0 reads as 1), 3 persistent
 * tile-queue sweep (threads = cells per tile), 4 one
 * launch per hyperplane, lane groups (CTAs of threads) on planes of fewer
 * than cluster cells and a thread per cell (CTAs of 128) on larger ones.  Successive hyperplane launches of a pass are chained by
 * programmatic dependent launch: a plane's kernel loads what the pass does
 * not change while the previous plane's kernel runs. */
int ath_batch_sweep_shape(ath_batch *batch, int *mode, int *threads, int *cluster);
/* Sets the sweep shape (as ath_batch_sweep_shape reports it; mode 3 takes
 * tiles of 1..4096 cells, mode 4 a threshold of at least one cell);
 * the next iteration recaptures the batch's graph.  Call it outside any
 * stream capture. */
int ath_batch_set_sweep_shape(ath_batch *batch, int mode, int threads, int cluster);
/* The tile-queue sweep's waits are bounded: a wait for another tile polls
 * at most poll_limit times (default 2^24, about a second), then the sweep
 * records ATH_ERR_TIMEOUT, every CTA stops taking tiles, and the run that
 * launched it (ath_batch_iterate, _converge, _relax, _autotune) returns
 * ATH_ERR_TIMEOUT with that iteration's update incomplete; the context and
 * the batch stay usable.  wait_never = 1 makes every wait poll a flag that
 * nothing sets (for tests of the bounded wait).  No counterpart in the
 * reference (its sweeps are sequential loops). */
int ath_batch_sweep_wait_test(ath_batch *batch, long long poll_limit, int wait_never);

/* ---- serving ------------------------------------------------------------
 * A request loop over independent solves (continuous batching).  Every
 * admitted request is its own device-resident batch on its own stream, so
 * the iterations of all admitted requests overlap on the device.  Requests
 * are admitted first come, first served, while fewer than max_active are
 * resident and the estimated device memory of the resident requests plus
 * this one fits the context's budget (or, when the budget is 0, the device
 * memory free at server creation less 1 GiB).  A
 * request retires on the device in the iteration where its total L2 drop
 * reaches `drop` (or its state turns nonphysical, or after max_iters); the
 * host then copies its final state out and frees its device memory.  The
 * batches share no data, so a request's result is the same alone and in
 * any mix.  The reference has no serving layer: every run is one MPI job
 * (src/main.cpp). */
typedef struct ath_server ath_server;
typedef struct {
  int64_t id;
  int64_t iterations;
  double drop;        /* last total L2 / first total L2 */
  int32_t converged;  /* 1 drop reached, -1 nonphysical, 0 iteration cap */
  int32_t pad;
  double queue_ms;    /* submit to admission (host clock) */
  double latency_ms;  /* submit to retirement (host clock): time to convergence */
  double device_ms;   /* first iteration to retirement (device clock) */
} ath_request_status;

/* precision = ATH_PREC_*; iterations are launched `chunk` at a time (1..1024)
 * between host checks. */
int ath_server_create(ath_ctx *ctx, int precision, double drop, int64_t max_iters,
                      int chunk, int max_active, ath_server **out);
/* Parses the input file (the reference's format) and queues the request. */
int ath_server_submit(ath_server *server, const char *inp_path, int64_t *id);
/* One scheduling pass, non-blocking: requests whose last chunk finished
 * retire or get their next chunk; queued requests are admitted while slots
 * and memory allow. */
int ath_server_step(ath_server *server, int *n_active, int *n_queued);
/* Requests retired since the last poll (up to max). */
int ath_server_poll(ath_server *server, ath_request_status *out, int max, int *n);
/* Final primitive state of a retired request's block (AoS, physical cells,
 * k slowest), kept on the host until released. */
int ath_server_fetch(ath_server *server, int64_t id, int block, double *prim_out);
int ath_server_release(ath_server *server, int64_t id);
int ath_server_destroy(ath_server *server);

/* Same as one iteration but split into the reference's stages, for parity
 * tests.  Stage order: fill_ghosts, residual, timestep, diag_invert, relax,
 * update. */
int ath_batch_fill_ghosts(ath_batch *batch);
int ath_batch_residual(ath_batch *batch);
int ath_batch_timestep(ath_batch *batch);
int ath_batch_diag_invert(ath_batch *batch);
int ath_batch_relax(ath_batch *batch);
int ath_batch_update(ath_batch *batch, ath_norms *norms_h);

/* Field download/upload.  Fields are per physical cell, AoS, k slowest;
 * ATH_FIELD_STATE_GHOSTS covers the padded block. */
enum {
  ATH_FIELD_STATE = 0,        /* primitive W, nv per cell */
  ATH_FIELD_STATE_GHOSTS = 1, /* primitive W incl. ghosts, nv per cell */
  ATH_FIELD_RESID = 2,        /* residual R, nv */
  ATH_FIELD_DT = 3,           /* local time step, 1 */
  ATH_FIELD_SPECRAD = 4,      /* cell spectral radius (flow, turb), 2 */
  ATH_FIELD_DU = 5,           /* implicit update, nv */
  ATH_FIELD_AINV = 6,         /* inverse main diagonal, 1 (scalar) */
  /* auxiliary cell values as the reference holds them at output time
   * (procBlock temperature_, viscosity_, eddyViscosity_, f1_, f2_): 5 =
   * temperature and laminar viscosity of the last auxiliary update (the
   * residual of the last iteration, UpdateAuxillaryVariables
   * src/procBlock.cpp:6171; Euler solves: temperature of the current
   * state, viscosity 0), then eddy viscosity, F1, F2 of the last SST
   * residual (0 without turbulence), nondimensional */
  ATH_FIELD_AUX = 7,
  /* cell-averaged velocity gradient of the last residual (velocityGrad_),
   * 9 = d(u,v,w)/dx, d(u,v,w)/dy, d(u,v,w)/dz; block LU-SGS viscous and SST
   * solves only (others: ATH_ERR_UNSUPPORTED) */
  ATH_FIELD_VELGRAD = 8,
  /* wall distance (procBlock::CalcWallDistance src/procBlock.cpp:6030), 1;
   * 1e10 without viscous walls */
  ATH_FIELD_WALLDIST = 9,
  /* conserved state of time n and of time n-1 (procBlock consVarsN_,
   * consVarsNm1_), nv per cell (rho, rho u, rho v, rho w, rho E [, rho k,
   * rho omega]); time-accurate solves only (time n-1: bdf2 solves) */
  ATH_FIELD_CONS_N = 10,
  ATH_FIELD_CONS_NM1 = 11,
  /* cell-averaged gradients of the last residual (batches created with
   * ATH_BATCH_OUTPUT_GRADS; procBlock velocityGrad_, temperatureGrad_,
   * densityGrad_, pressureGrad_, tkeGrad_, omegaGrad_, written by
   * WriteFunFile src/output.cpp:309-395), 24 per cell: velocity gradient (9,
   * as ATH_FIELD_VELGRAD), then the temperature, density, pressure, k and
   * omega gradients (x, y, z each; k and omega zero without RANS) */
  ATH_FIELD_GRADS = 12
};
int ath_batch_get_field(ath_batch *batch, int block, int field, double *out_h);
int ath_batch_set_state(ath_batch *batch, int block, const double *prim_h);
/* Sets the conserved state of time n-1 of a bdf2 solve's block (nv per
 * cell, as ATH_FIELD_CONS_NM1; procBlock::GetSolNm1FromRestart
 * src/procBlock.cpp:6418).  The solve then keeps it through its first
 * time step instead of copying time n into it, as a restarted reference
 * run does (mgSolution::StoreOldSolution src/mgSolution.cpp:103); set every
 * block of the solve.  NULL cons_h copies the block's current state into
 * time n-1 instead (the one-level restart of a bdf2 solve, ReadRestart
 * src/output.cpp:892). */
int ath_batch_set_state_nm1(ath_batch *batch, int block, const double *cons_h);
/* Values per cell of `field` for block `block`: the block's nv (5, or 7
 * with the SST k and omega) for STATE, STATE_GHOSTS, RESID and DU. */
int ath_batch_field_width(ath_batch *batch, int block, int field);

/* Device work counters of the last ath_batch_iterate call. */
typedef struct {
  int64_t kernel_launches;   /* kernels launched (graph nodes included) */
  double device_ms;          /* CUDA-event time on the batch stream */
} ath_stats;
int ath_batch_stats(ath_batch *batch, ath_stats *out);

/* ---- output files (reference formats) ------------------------------------
 * Host fields of one block for the writers, physical cells with i fastest
 * and k slowest (AoS), nondimensional; NULL where not available (a variable
 * that needs a missing field is an ATH_ERR_ARG). */
typedef struct {
  const double *prim;      /* nv per cell: rho, u, v, w, p [, k, omega] */
  const double *dt;        /* 1 per cell: local time step */
  const double *resid;     /* nv per cell: residual */
  const double *aux;       /* 5 per cell: as ATH_FIELD_AUX */
  const double *velgrad;   /* 9 per cell: as ATH_FIELD_VELGRAD */
  const double *wall_dist; /* 1 per cell */
  const double *cons_nm1;  /* nv per cell: conserved state of time n-1 (bdf2
                              solves: the restart file's second level) */
  const double *grads;     /* 24 per cell: as ATH_FIELD_GRADS (the gradient
                              output variables; velGrad_* from here when
                              given, else from velgrad) */
} ath_block_fields;

/* Plot3D cell-centre function file (WriteFunFile, src/output.cpp:209) of
 * one solve: `variables` is a comma-separated list of the reference's
 * output variable names (NULL or "" = the input file's outputVariables),
 * written in sorted order as the reference's set keeps them; `fields` has
 * one entry per block of the solve.  Supported: density, vel_x/y/z,
 * pressure, mach, sos, dt, temperature, energy, enthalpy, cp, cv, rank,
 * globalPosition, viscosityRatio, turbulentViscosity, viscosity, tke, sdr,
 * f1, f2, wallDistance, velGrad_*, resid_*, mf_<species>, vf_<species>;
 * the temperature, density, pressure, k and omega gradients are not kept
 * and are ATH_ERR_UNSUPPORTED. */
int ath_output_function(const ath_setup *setup, int solve, const char *variables,
                        const ath_block_fields *fields, const char *path);
/* Restart file (WriteRestart, src/output.cpp:591): iteration, the L2
 * normalisation per equation (nv), dimensional primitives per cell; for a
 * bdf2 solve a second time level, the dimensional conserved state of time
 * n-1 (fields[k].cons_nm1, required). */
int ath_output_restart(const ath_setup *setup, int solve, int iteration,
                       const double *resid_first, const ath_block_fields *fields,
                       const char *path);
/* Reads a restart file (ReadRestart, src/output.cpp:756) into prim_out[k]
 * (one nv-per-cell array per block of the solve, may be NULL), checking it
 * against the solve's equations, species and block sizes.  *levels (may be
 * NULL) receives the file's time levels; with two, cons_nm1_out[k] (may be
 * NULL) receives the nondimensional conserved state of time n-1
 * (ReadSolNm1FromRestart, :1242). */
int ath_input_restart(const ath_setup *setup, int solve, const char *path, int *iteration,
                      double *resid_first, double *const *prim_out, int *levels,
                      double *const *cons_nm1_out);
/* Cell-centre grid (WriteCellCenter, src/output.cpp:57) and Paraview meta
 * file (WriteMeta, :903) naming <grid>_center.xyz and
 * <sim>_<iteration>_center.fun. */
int ath_output_center_grid(const ath_setup *setup, int solve, const char *path);
int ath_output_meta(const ath_setup *setup, int solve, const char *variables, int iteration,
                    const char *path);
/* Residual history (PrintHeaders / PrintResiduals, src/output.cpp:1007,
 * 1028): n rows from the solve's norms of nonlinear iterations
 * first_step.., each shown as time step it / nonlinearIterations and
 * nonlinear iteration it % nonlinearIterations, with the input's timeStep
 * (when given) or the CFL; a header first unless flags has
 * ATH_RESID_APPEND.  resid_first (nv) carries the normalisation: set at
 * the first time step's first nonlinear iteration and raised to each
 * equation's largest L2 over the first nonlinear iterations of time steps
 * 1-4, unless flags has ATH_RESID_RESTARTED (a run restarted from a file,
 * whose normalisation the file gave). */
enum { ATH_RESID_APPEND = 1, ATH_RESID_RESTARTED = 2 };
int ath_output_resid(const ath_setup *setup, int solve, const char *path, int flags,
                     int first_step, int n, const ath_norms *norms, double *resid_first);
/* The same from a batch's resident solution (fields gathered from the
 * device; the setup is the one the batch was created from). */
int ath_batch_write_function(ath_batch *batch, const ath_setup *setup, int solve,
                             const char *variables, const char *path);
int ath_batch_write_restart(ath_batch *batch, const ath_setup *setup, int solve,
                            int iteration, const double *resid_first, const char *path);
/* The restart read into a batch sets the state and, for a bdf2 solve, time
 * n-1: the file's second level, or the state itself when the file holds
 * one (ath_batch_set_state_nm1). */
int ath_batch_read_restart(ath_batch *batch, const ath_setup *setup, int solve,
                           const char *path, int *iteration, double *resid_first);

/* Whole-batch snapshot of the primitive state in the device layout:
 * [nv][pool cells] FP64 with nv from ath_batch_pool_vars (5, or 7 when the
 * batch holds SST solves: rho, u, v, w, p, then k, omega; k and omega are
 * 0 in the blocks of other solves), every block's padded cells back to back
 * (block b starts at the sum of the padded cell counts of blocks 0..b-1).
 * One copy per pool each way; pass page-locked host memory for full link
 * bandwidth.  to_device = 1 uploads host -> device, 0 downloads.  (Restart
 * snapshots of resident solutions, reference WriteRestart/ReadRestart
 * src/output.cpp:591,756, go through this.) */
int ath_batch_pool_cells(ath_batch *batch, int64_t *ncell);
int ath_batch_pool_vars(ath_batch *batch, int *nv);
int ath_batch_copy_state(ath_batch *batch, double *host, int to_device);

/* CUDA-event timing of each kernel class on the batch stream, averaged
 * over reps launches of one iteration's worth of work (outside the graph).
 * ms[]: 0 ghost fill, 1 i-face fluxes, 2 j-face fluxes, 3 k-face fluxes,
 * 4 residual/dt/diagonal cells, 5 forward sweep (all hyperplanes),
 * 6 backward sweep (all hyperplanes), 7 update + norms.  The batch state
 * advances by reps iterations. */
int ath_batch_profile(ath_batch *batch, int reps, double ms[8]);

/* ---- allocation-free residual of one block ------------------------------
 * No counterpart in the reference: an addition for callers that cannot
 * allocate device memory while the solver step runs (a code that records
 * the step into a CUDA graph it owns, a serving loop that has handed every
 * byte of HBM to its admission budget, a plugin host that owns the device
 * allocator).  The caller passes its own device arrays for every input and
 * output; the face-flux scratch of the stage is a fixed device array inside
 * this library of ATH_NOALLOC_MAX_CELLS padded cells (15.7 MB, held on every
 * GPU that loads the library until the process exits).  Blocks with more
 * padded cells are rejected with ATH_ERR_UNSUPPORTED.
 *
 * Computes the same residual R, cell spectral radius, local time step and
 * inverse scalar diagonal as ath_batch_residual (FP64) for a steady Euler
 * solve with MUSCL reconstruction, the Roe flux and a scalar diagonal
 * (lusgs or dplur); any other view (viscous or RANS equations, block
 * solvers, a global time step, a dual-time CFL, WENO or AUSM) is refused
 * with ATH_ERR_UNSUPPORTED.  Arrays use the
 * padded layout of ath_block_view (cell (i,j,k) at (i+ng) + NI*((j+ng) +
 * NJ*(k+ng))), all [var][cell]; face data of direction d are stored at the
 * index of the cell above the face (face i at cell i).  Ghost layers of W
 * must already be filled.
 *
 * Each call outside a stream capture looks up the scratch array's device
 * address with the calling device current (so it stays valid after a reset
 * of the device's primary context); a call inside a capture reuses the
 * address of that device's last uncaptured call, so make the first call on
 * a device before any stream capture.
 * Every call on a device shares the one scratch array, so calls that
 * overlap on the GPU (other streams, other host threads) race: serialise
 * them.  stream: a cudaStream_t (NULL = legacy default stream); the call
 * returns after enqueueing, without synchronising. */
#define ATH_NOALLOC_MAX_CELLS 131072
typedef struct {
  int32_t ni, nj, nk, ng;   /* physical cells and ghost layers (ng >= 2) */
  const double *W;          /* [5][ncell] primitive state incl. ghosts */
  const double *vol;        /* [ncell] cell volumes */
  const double *width[3];   /* [ncell] cell widths in i, j, k */
  const double *farea[3];   /* [4][ncell] unit normal x,y,z and magnitude */
  double *R;                /* out [5][ncell] residual (physical cells) */
  double *lam;              /* out [ncell] inviscid cell spectral radius */
  double *dt;               /* out [ncell] local time step */
  double *ainv;             /* out [ncell] inverse scalar main diagonal */
} ath_block_dev;
int ath_block_residual_noalloc(const ath_block_dev *blk, const ath_solve_view *phys,
                               double cfl, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* AITHER_GB300_H */
