// Kernels of the per-iteration path and their device data layout.
//
// Layout in HBM (all blocks of all solves of a batch share one pool):
//   * cell fields are structure-of-arrays, [var][pool cell], over the padded
//     cells of every block (ghost layers included), i fastest inside a
//     block;
//   * face fields of direction d are stored at the pool index of the cell
//     on the upper side of the face (face i of a block sits at cell i), so
//     faces and cells share one index space;
//   * work lists (physical cells, faces of direction d) are padded per block
//     to a multiple of the CTA size, so every CTA works inside one block and
//     reads that block's strides once.
#pragma once

#include <cstdint>
#include <type_traits>

#include "aither_gb300.h"
#include "physics.cuh"

namespace ath {

constexpr int kCta = 256;   // threads per CTA of the cell/face kernels
constexpr int kNv = 5;      // flow equations
constexpr int kNvMax = 7;   // with the k and omega equations of RANS solves

struct BlockDev {
  int32_t ni, nj, nk, ng, NI, NJ, NK, solve;
  int64_t cell0;  // pool index of padded cell (-ng,-ng,-ng)
};

struct SolveDev {
  double gas_r, gas_n, gas_hf;
  double kappa, theta, zeta, relax, cfl_start, cfl_step, cfl_max;
  double padded_values;  // sum over blocks of padded cells x nv
  double cells;          // physical cells of the solve
  // laminar transport (Sutherland), nondimensional
  double visc_scale, mu_c1, mu_s, mu_ref, t_ref, k_c1, k_s, k_ref, visc_coeff;
  int32_t viscous;
  int32_t wilcox;  // RANS with the Wilcox k-omega 2006 model instead of SST-2003
  int32_t limiter, nstates, state0, recon;
  int32_t flux;
  int32_t block;   // blusgs: 5x5 Jacobian diagonal and off-diagonals
  int32_t rans;    // SST-2003: k and omega beside the flow equations
  int32_t jacobi;  // dplur / bdplur: Jacobi sweeps instead of LU-SGS
  int32_t sweeps;  // matrixSweeps
  int32_t active;  // 0 once the solve is retired: its kernels skip their work
  // time integration: global nondimensional time step (0: local from the
  // CFL), dual-time CFL (0: none), nonlinear iterations per time step,
  // bdf2's time n-1 level, and whether the right-hand side carries the
  // time-level terms (multilevel or several nonlinear iterations)
  double dt_global, dual_cfl;
  int32_t nl_iters, multilevel, unsteady;
  int32_t store_n;  // keep the time-n state: time-accurate or nonreflecting
  // Constants derived from the ones above by SetDerived() on the host, each
  // one IEEE operation (or Gas::Set's three) so its bits are those a thread
  // would compute; kernels read them instead of dividing per thread: cv, cp
  // and gamma in double and in float, and 1 / theta
  double gas_cv, gas_cp, gas_gam, theta_inv;
  float gas_cvf, gas_cpf, gas_gamf, pad_f;
};

// Fills SolveDev's derived constants from gas_r, gas_n, gas_hf and theta
inline void SetDerived(SolveDev &x) {
  Gas<double> gd;
  gd.Set(x.gas_r, x.gas_n, x.gas_hf);
  x.gas_cv = gd.cv;
  x.gas_cp = gd.cp;
  x.gas_gam = gd.gam;
  Gas<float> gf;
  gf.Set((float)x.gas_r, (float)x.gas_n, (float)x.gas_hf);
  x.gas_cvf = gf.cv;
  x.gas_cpf = gf.cp;
  x.gas_gamf = gf.gam;
  x.pad_f = 0.0f;
  x.theta_inv = 1.0 / x.theta;
}

// Per-solve hyperplane lists of the persistent sweep: items (q index,
// block) ordered by solve, then plane; step_off[solve_step0[s] + p] .. +1
// bound plane p of solve s (solve_nsteps[s] planes)
// One pass of the persistent tile-queue sweep (k_sweep_tq): tiles in ticket
// order (x, y: range of items; z, w: range of deps), the tiles each waits on,
// per-tile done flags (one more, never set, for the forced-timeout test
// mode), the ticket counter and the batch's sweep status word.
struct TileQueueDev {
  const int2 *items;
  const int4 *tiles;
  const int32_t *deps;
  int *done;
  int *ticket;
  int *status;
  int ntiles;
  int wait_never;
  long long spin_limit;
};

struct SweepLists {
  const int2 *items;
  const int32_t *step_off, *solve_step0, *solve_nsteps;
  int nsolves;
};

// A ghost-cell assignment with pool indices.
struct GhostOpDev {
  int32_t dst, src, type, lower;
  int32_t face, dir, state, layer;
  int32_t src2, pad;
};

// A viscous-wall face: pool index of the face (cell above it), direction,
// block.  Lists are ordered by solve.
// A cell next to a nonreflecting surface: pool indices of the cell and of
// its boundary face, outward-normal sign; grouped by surface.
struct NrDev {
  int32_t cell, face, lower, dir, solve, pad;
};

struct WallFaceDev {
  int32_t face, dir, block, pad;
};

// Partial norms of one CTA of the update kernel.
struct NormPartial {
  double l2[7];     // per equation (the k and omega equations of RANS solves last)
  double linf;
  int64_t linf_pos;  // position in the solve's loop order, for ties
  int32_t linf_cell, linf_eqn;
  int32_t bad;       // nonphysical state produced
  int32_t pad;
};

// Device pointers of a batch.  Passed by value to every kernel.
//
// The LU-SGS sweeps work on a second copy of their working set stored in
// hyperplane order ("q order": block by block, plane by plane, inside a
// plane by k then j), so that the cells of one hyperplane and of its
// neighbour plane are contiguous runs: Wq, Rq, Ainvq, dUq, the face
// normals of each cell's lower and upper faces, and the q index of each
// neighbour (nbq; -1 = no off-diagonal term, <= -2 = a ghost cell across a
// connection, slot -nbq-2 of the ghost tables).
template <typename T>
struct Pools {
  double *W;        // [5][ncell] primitive state, FP64
  double *R;        // [5][ncell] residual, FP64
  double *flux[3];  // [5][ncell] F.|A| on faces of direction d (FP64 in both
                    // paths: the residual is their FP64 sum)
  T *vflux[3];      // [5][ncell] viscous F.|A| (viscous solves)
  double *mu;       // [ncell] laminar viscosity (viscous solves)
  double *lam;      // [ncell] cell spectral radius
  double *dt;       // [ncell]
  const double *vol;       // [ncell]
  const double *width[3];  // [ncell]
  const double *fa[3];     // [4][ncell] unit normal x,y,z and magnitude
  // FP64 batches, formed once from the geometry: fgeo[d] [4][ncell] at a
  // face of direction d, MUSCL's width ratios dplus and dminus of its lower
  // and of its upper side; cgeo[d] [4][ncell] at a physical cell, the
  // normalised average (fast option: sum) of its two face normals of
  // direction d and their average area (the cell spectral radius's
  // geometry).  Bit-exact batches form them with the per-face and per-cell
  // expressions, the fast option with its own
  double *fgeo[3];
  double *cgeo[3];
  const int32_t *qpos;     // [ncell] q index of a physical cell, -1 for ghosts
  // hyperplane-ordered sweep working set, nq = physical cells of the batch
  T *Wq;            // [5][nq] state in the sweep's arithmetic
  T *Rq;            // [5][nq]
  T *Ainvq;         // [nq] inverse of the scalar main diagonal; [25][nq]
                    // row-major 5x5 inverse when the batch has block solves
  T *Aq;            // the main diagonal (matrix residual), same layout
  T *muq;           // [nq] laminar viscosity, q order
  T *Npre;          // [9][nq] NbrPre of each cell (FP64 batches with scalar
                    // solves; null otherwise)
  const T *dist_lo; // [3][nq] centre-to-centre distance along the lower face normal
  const T *dist_hi; // [3][nq] same for the upper face
  T *dUq;           // [5][nq] implicit update
  const T *face_lo; // [3 dirs][4][nq] lower face of each direction
  const T *face_hi; // [3 dirs][4][nq] upper face
  const int32_t *nbq;      // [6][nq] neighbours: lower i,j,k then upper i,j,k
  const int32_t *ghost_cell;  // [nghost] pool cell of each connection ghost
  const int32_t *ghost_src;   // [nghost] q index of the partner interior cell
  T *dUg;           // [5][nghost] update of the connection ghosts
  // block (blusgs) solves only
  T *fst[3];        // [10][ncell] reconstructed face states, lower side then upper
  T *vst[3];        // [15][ncell] viscous face state, face viscosity, face
                    // velocity gradient (row = derivative axis)
  T *vgq;           // [9][nq] cell-averaged velocity gradient, q order
  // RANS (SST-2003) solves only
  double *Wt;       // [2][ncell] k, omega
  double *Rt;       // [2][ncell] turbulence residual
  double *fluxt[3]; // [2][ncell] turbulence inviscid flux F.|A|
  T *vfluxt[3];     // [2][ncell] turbulence viscous flux F.|A|
  T *rst[3];        // [18][ncell] face: velocity gradient (9), k gradient (3),
                    // omega gradient (3), eddy viscosity, F1, F2
  double *lamt;     // [ncell] turbulence spectral radius
  const double *wd; // [ncell] wall distance
  T *Rtq, *dUtq;    // [2][nq]
  T *dUtg;          // [2][nghost]
  T *Ainvtq, *Atq;  // [nq] scalar or [4][nq] 2x2 turbulence diagonal (inverse)
  T *mutq, *f1q;    // [nq] cell eddy viscosity and F1
  T *f2q;           // [nq] cell F2 (output only)
  double *Taux;     // [ncell] temperature of the last auxiliary update (viscous)
  // block solves: off-diagonal Jacobians of each cell's six neighbours,
  // [(side*3 + d)*25 + e][nq] (side 0 = lower) and the turbulence blocks
  // [(side*3 + d)*4 + e][nq]
  T *Joff, *Jtoff;
  // Jacobi (DP-LUR) solves: the second update buffer of the sweeps
  T *dUq2, *dUtq2;
  // time-accurate solves: conserved state of time levels n and n-1
  // [7][ncell] (rho, rho u, rho v, rho w, rho E, rho k, rho omega) and the
  // linear system's right-hand side in q order ([5][nq], [2][nq])
  double *Un, *Unm1;
  T *Bq, *Btq;
  double *nr_mach;  // [2][nonreflecting surfaces] average, largest Mach
  // [12][ncell] cell-averaged velocity gradient (9, d/dx rows) and pressure
  // gradient (3) of the previous residual at the cells nonreflecting
  // pressure outlets read (null without such outlets)
  double *nrg;
  // multigrid: forcing of a coarse level's linear system ([5][nq], null on
  // the finest level), the matrix residual f - (A x - b) of the level's last
  // relaxation ([5][nq], null without multigrid), and mg_accum = 1 when the
  // level's diagonal adds to the one of its previous visit in this
  // iteration (a W cycle's second visit; gridLevel::ResetDiagonal only
  // after each update, src/mgSolution.cpp:225-228)
  T *Fq, *MRq;
  int mg_accum;
  // [nq] unlimited eddy viscosity rho k / omega of the cells of Wilcox
  // k-omega 2006 solves (their turbulence radii and Jacobians; null without
  // such solves)
  T *nutq;
  // [24][ncell] cell-averaged gradients of the last residual kept for
  // output (batch flag ATH_BATCH_OUTPUT_GRADS; null otherwise)
  double *ogr;
  // FP64 batches with the fast-arithmetic option: the launchers run the
  // faces, cell, scalar sweep and update kernels built with contracted
  // multiply-adds (kernels_fp64_fast.cu); a host-side switch
  int fast_fp64;
  // solve kinds of the batch (host-side): bit 0 solves without, bit 1 with
  // turbulence equations; the cell kernel is built per kind
  int fkinds;
  const BlockDev *blocks;
  const SolveDev *solves;
  const ath_bc_state *states;
  const double *cfl;       // [nsolves] current CFL
  int64_t ncell, nq, nghost;
};

__device__ __forceinline__ int64_t StrideOf(const BlockDev &b, int d) {
  return d == 0 ? 1 : (d == 1 ? (int64_t)b.NI : (int64_t)b.NI * b.NJ);
}

template <typename T>
__device__ __forceinline__ Prim<T> LoadW(const double *W, int64_t n, int64_t c) {
  Prim<T> s;
  s.rho = (T)W[c];
  s.u = (T)W[n + c];
  s.v = (T)W[2 * n + c];
  s.w = (T)W[3 * n + c];
  s.p = (T)W[4 * n + c];
  return s;
}

// Programmatic dependent launch (sm_90 and later).  GridDependencyWait
// returns once the grid this one was launched after with the
// programmatic-serialization attribute has completed and its memory
// operations are visible (at once for a normal launch);
// GridDependentsLaunch lets the grid launched after this one with that
// attribute start (a no-op without one).
__device__ __forceinline__ void GridDependencyWait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void GridDependentsLaunch() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename T>
__device__ __forceinline__ Gas<T> GasOf(const SolveDev &s) {
  static_assert(std::is_same<T, double>::value || std::is_same<T, float>::value, "T");
  Gas<T> g;
  g.r = (T)s.gas_r;
  g.n = (T)s.gas_n;
  g.hf = (T)s.gas_hf;
  if constexpr (std::is_same<T, double>::value) {
    g.cv = s.gas_cv;
    g.cp = s.gas_cp;
    g.gam = s.gas_gam;
  } else {
    g.cv = s.gas_cvf;
    g.cp = s.gas_cpf;
    g.gam = s.gas_gamf;
  }
  return g;
}

// ---------------------------------------------------------------------------
// Ghost cells: boundary states (procBlock::AssignInviscidGhostCells,
// src/procBlock.cpp:2449, GetGhostState src/ghostStates.cpp:62) and
// connection copies (SwapStateSlice, src/procBlock.cpp:3050).
template <typename T>
__global__ void k_ghost(Pools<T> P, const GhostOpDev *ops, int nops,
                        const int32_t *op_solve);

// Face fluxes of direction D over the face list (CalcInvFluxI/J/K,
// src/procBlock.cpp:384,522,660): k_face<T, D, RANS, FAST, MR> in
// kernels_impl.cuh.

// Residual assembly, spectral radius, local time step and inverted
// diagonal of every physical cell (procBlock residual accumulation,
// CalcBlockTimeStep src/procBlock.cpp:798, AddDiagonalTerms/Invert
// src/linearSolver.cpp:146,177).
template <typename T, bool BLOCK, bool RANS>
__global__ void k_cell(Pools<T> P, const int32_t *list, const int32_t *cta_block);

// One hyperplane of the LU-SGS forward / backward sweep
// (lusgs::LUSGS_Forward/Backward, src/linearSolver.cpp:341,385); items are
// (q index, block) pairs.  FULL: some solve runs more than one sweep, so
// both triangles may enter a pass.  k_sweep (a thread per cell) and
// k_sweepg (a group of lanes per cell, one per neighbour term) serve scalar
// solves, k_sweepb block solves.
template <typename T, bool FULL, bool TURB>
__global__ void k_sweep(Pools<T> P, const int2 *items, int n, int forward, int sweep);
template <typename T, bool FULL, int MINB, bool TURB>
__global__ void k_sweepg(Pools<T> P, const int2 *items, int n, int forward, int sweep);
template <typename T>
__global__ void k_sweepb(Pools<T> P, const int2 *items, int n, int forward, int sweep,
                         int full_any);
// Initial update x = A^-1 b of solves with more than one sweep, x = 0 for
// the others (linearSolver::InitializeMatrixUpdate, src/linearSolver.cpp:111).
template <typename T>
__global__ void k_init(Pools<T> P, const int2 *items, int n);

// dU ghost copies across connections (SwapImplicitUpdate, src/utility.cpp:400).
template <typename T>
__global__ void k_conn_du(Pools<T> P);

// Per-solve reduction of the CTA partials into the norm ring, CFL of the
// next iteration, iteration counter (one warp per solve).
struct NormOut {
  double l2[7];
  double linf;
  int64_t linf_pos;
  int32_t bad;
  int32_t pad;
  double cfl;
  double matrix_resid;
};
// Per-solve iteration bookkeeping on the device: the solve's own iteration
// count (it drives the CFL ramp and the residual normalisation), the total
// L2 norm of its first iteration, its retirement target and record.
struct SolveState {
  int64_t iter;          // iterations run by this solve
  double l2_first;       // total L2 (over the equations) of its first iteration
  double target;         // retire when total L2 <= target * l2_first (0: never)
  int64_t retire_iter;   // iterations run when it retired (0: still active)
  uint64_t t_first_ns;   // device clock at the end of its first iteration
  uint64_t t_retire_ns;  // device clock at retirement
  double l2_last;        // total L2 of its last iteration
  int32_t converged;     // 1 target reached, -1 retired on a nonphysical state
  int32_t nm1_given;     // time n-1 set by the host (restart): kept at the first step
};
__global__ void k_norms(const NormPartial *partials, const double *mres_partials,
                        const int32_t *solve_cta0, int nsolves, NormOut *ring,
                        int ring_cap, int64_t *iter_counter, SolveDev *solves,
                        SolveState *sstate, double *cfl);

// Logged matrix residual r = -(A x - (L x - U x) - b) summed as r^2 per CTA
// (linearSolver::Residual / AXmB, src/linearSolver.cpp:58,92).
template <typename T, bool BLOCK>
__global__ void k_matres(Pools<T> P, const int32_t *list, const int32_t *cta_block,
                         double *mres_partials);
// Wall forces per solve: fixed-order sum of the per-face values of each
// solve's range into the forces ring (one warp per solve).
__global__ void k_wallsum(const double *wbuf, int nfaces, const int32_t *solve_face0,
                          int nsolves, double *fring, int ring_cap,
                          const int64_t *iter_counter);
// Sets the CFL of each solve's current iteration from its own iteration
// count (input::CalcCFL, src/input.cpp:647).
__global__ void k_cfl(const SolveDev *solves, int nsolves, const SolveState *sstate,
                      double *cfl);

// Host-side launchers, one instantiation per arithmetic type (defined in
// kernels_fp64.cu / kernels_fp32.cu).
// The fast FP64 faces of direction d (k_face<double, d, false, true>),
// compiled in their own unit with contracted multiply-adds: roundoff-equal
// to the reference's faces, not bit-equal.
void LaunchFastFaceFp64(int d, const Pools<double> &P, const int32_t *list,
                        const int32_t *cta_block, int ncta, bool muscl_roe, cudaStream_t s);
// The cell kernel, the scalar LU-SGS sweeps and the update of FP64 batches
// with the fast option, from the same unit (same arguments as
// Launch<double>::Cell / Sweep / Update; the sweep: scalar solves only).
void LaunchFastCellFp64(const Pools<double> &P, const int32_t *list, const int32_t *cta_block,
                        int ncta, int kinds, cudaStream_t s);
void LaunchFastSweepFp64(const Pools<double> &P, const int2 *items, int n, int forward,
                         int sweep, bool full, int threads, bool group, bool chained,
                         cudaStream_t s);
// The geometry tables (Pools::fgeo, cgeo) over the batch's face lists of
// each direction and its physical-cell list: the fast option's forms
// (kernels_fp64_fast.cu), or the bit-exact ones (kernels_fp64.cu)
void LaunchExactGeomFp64(const Pools<double> &P, const int32_t *const faces[3],
                         const int32_t *const face_cta_block[3], const int nface_cta[3],
                         const int32_t *cells, const int32_t *cell_cta_block, int ncell_cta,
                         cudaStream_t s);
void LaunchFastGeomFp64(const Pools<double> &P, const int32_t *const faces[3],
                        const int32_t *const face_cta_block[3], const int nface_cta[3],
                        const int32_t *cells, const int32_t *cell_cta_block, int ncell_cta,
                        cudaStream_t s);
void LaunchFastUpdateFp64(const Pools<double> &P, const int32_t *list, const int32_t *cta_block,
                          const int32_t *cta_pos0, NormPartial *partials, int ncta,
                          const SolveState *ss, cudaStream_t s);

// Transfer between a multigrid level (fine) and the next coarser one.
// Restriction is a gather per coarse physical cell c over its fine cells
// e in [off[c], off[c+1]), in the fine cells' k, j, i order; prolongation
// per fine physical cell from the coarse correction at the coarse nodes.
struct MgLinkDev {
  int ncoarse, nfine, nnode;
  const int32_t *off;                       // [ncoarse+1]
  const int32_t *c_pool, *c_q;              // [ncoarse] coarse pool / q index
  const int32_t *f_pool, *f_q;              // [nfine] fine pool / q index (gather order)
  const double *f_w;                        // [nfine] volume weight
  const int32_t *node_cells;                // [nnode][8] coarse q (-1: none), summing order
  const double *node_fac;                   // [nnode] 1, 1/2 or 1/8
  const int32_t *p_q;                       // [nfine] fine q (k, j, i order of each block)
  const int32_t *p_node0;                   // [nfine] node (ci, cj, ck) of its coarse cell
  const int32_t *p_sx, *p_sxy;              // [nfine] node strides of that coarse block
  const double *p_coef;                     // [7][nfine] trilinear coefficients
};

template <typename T>
struct Launch {
  static void Ghost(const Pools<T> &P, const GhostOpDev *ops, int nops,
                    const int32_t *op_solve, cudaStream_t s);
  // laminar viscosity of the listed cells (UpdateAuxillaryVariables)
  static void Aux(const Pools<T> &P, const int32_t *cells, const int32_t *cell_block,
                  int n, cudaStream_t s);
  // rkinds: bit 0 = the batch has solves without turbulence equations
  // (for ViscFace: laminar viscous solves), bit 1 = SST solves; each kind
  // has its own kernel so the laminar one keeps its register budget
  static void ViscFace(int d, const Pools<T> &P, const int32_t *list,
                       const int32_t *cta_block, int ncta, int rkinds, cudaStream_t s);
  static void Face(int d, const Pools<T> &P, const int32_t *list,
                   const int32_t *cta_block, int ncta, int rkinds, cudaStream_t s);
  // kinds: bit 0 = the batch has scalar solves, bit 1 = block solves
  static void Cell(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                   int ncta, int kinds, cudaStream_t s);
  // chained: the launch follows the same pass's previous hyperplane, so the
  // grouped sweep starts programmatically and overlaps its loads of data the
  // pass does not change with that plane's kernel
  static void Sweep(const Pools<T> &P, const int2 *items, int n, int forward, int sweep,
                    bool full, int kinds, int threads, bool group, bool chained,
                    cudaStream_t s);
  // one pass of every LU-SGS solve as one launch: a cluster of `cluster`
  // CTAs of `threads` per solve walks its hyperplanes with cluster barriers
  static void SweepCl(const Pools<T> &P, const SweepLists &L, int forward, int sweep,
                      bool full, int kinds, int threads, int cluster, cudaStream_t s);
  // clusters of that shape the device can hold at once (0 = not launchable)
  static int MaxClusters(int kinds, int threads, int cluster);
  // one pass of the LU-SGS solves of one kind (block: 5x5 block solves,
  // else scalar) as one persistent launch of `ctas` CTAs of two warps over
  // a tile work queue; the queue's done flags and ticket must be zero
  static void SweepTq(const Pools<T> &P, const TileQueueDev &Q, int forward, int sweep,
                      bool full, bool block, int ctas, cudaStream_t s);
  // CTAs of the tile-queue sweep kernel resident per SM
  static int TqOccupancy(bool full, bool block);
  // off-diagonal Jacobians of the block solves' cells, once per iteration
  static void OffJac(const Pools<T> &P, const int2 *items, int n, cudaStream_t s);
  // jacobi = 0: x0 of the LU-SGS solves, 1: of the DP-LUR solves
  static void Init(const Pools<T> &P, const int2 *items, int n, int jacobi, cudaStream_t s);
  // one DP-LUR sweep of the Jacobi solves from P.dUq into dst (kinds:
  // scalar / block solves present); solves past their sweep count carry
  // their iterate over
  static void Jacobi(const Pools<T> &P, T *dst, T *dstt, const int2 *items, int n, int sweep,
                     int kinds, cudaStream_t s);
  // the Jacobi solves' final iterate from (src, srct) into dUq, dUtq
  static void JacobiCopy(const Pools<T> &P, const T *src, const T *srct, const int2 *items,
                         int n, cudaStream_t s);
  static void ConnDu(const Pools<T> &P, cudaStream_t s);
  static void Update(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                     const int32_t *cta_pos0, NormPartial *partials, int ncta,
                     const SolveState *ss, cudaStream_t s);
  // average and largest outward normal Mach number of each nonreflecting
  // surface (items nr[off[s] .. off[s+1]) into P.nr_mach[2 s .. 2 s + 1])
  static void NrMach(const Pools<T> &P, const NrDev *nr, const int32_t *off, int nsurf,
                     cudaStream_t s);
  // cell-averaged velocity and pressure gradients of the listed cells
  // (pool index, block) into P.nrg, from the current state and ghosts
  static void NrGrads(const Pools<T> &P, const int32_t *cells, const int32_t *cell_block, int n,
                      cudaStream_t s);
  // cell-averaged gradients of every physical cell for output into P.ogr
  // (fkinds: bit 0 solves without, bit 1 with turbulence equations)
  static void OutGrads(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                       int ncta, int fkinds, cudaStream_t s);
  // StoreOldSolution of the time-accurate solves at a time step's start;
  // block >= 0: that block's current state into both time levels
  static void StoreN(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                     int ncta, const SolveState *ss, int block, cudaStream_t s);
  static void MatRes(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                     double *mres_partials, int ncta, int kinds, cudaStream_t s);
  // multigrid forcing of a coarse level: P.Fq = (A x - (L x - U x) - b) + P.Fq
  static void MgForcing(const Pools<T> &P, const int32_t *list, const int32_t *cta_block,
                        int ncta, int kinds, cudaStream_t s);
  // restrictions: the primitive state (volume-weighted, pool to pool, into a
  // zeroed coarse pool), the update (volume-weighted, q to q) and the matrix
  // residual (summed, fine MRq into coarse Fq)
  static void MgRestrictState(const MgLinkDev &k, const double *fineW, int64_t fine_n,
                              double *coarseW, int64_t coarse_n, cudaStream_t s);
  static void MgRestrictQ(const MgLinkDev &k, const T *fine, int64_t fine_nq, T *coarse,
                          int64_t coarse_nq, bool weighted, cudaStream_t s);
  // x -= x0 over [5][nq]
  static void MgSubtract(T *x, const T *x0, int64_t nq, cudaStream_t s);
  // coarse correction at the coarse nodes, then added to the fine update
  static void MgProlong(const MgLinkDev &k, const T *coarse_du, int64_t coarse_nq, T *nodes,
                        T *fine_du, int64_t fine_nq, cudaStream_t s);
  // per-face wall forces [6][n] of the viscous-wall faces
  static void Wall(const Pools<T> &P, const WallFaceDev *faces, int n, double *wbuf,
                   cudaStream_t s);
};

}  // namespace ath
