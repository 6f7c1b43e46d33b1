/* CPU oracle of the per-iteration solver step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the
 * reference solver's (aither v0.10.0) per-iteration algorithm for the
 * per-iteration path (Euler, laminar and SST-2003 RANS; scalar and block
 * LU-SGS), used by the parity tests, by smoke checks and as
 * the timed CPU baseline.  The product library never links or calls it.
 *
 * It consumes the same host setup (geometry, ghost-cell op lists, hyperplane
 * orders) as the device batch, through the ath_block_view / ath_solve_view
 * structs of include/aither_gb300.h, and keeps the reference's own loop
 * structure: face loops that scatter fluxes into the two adjacent cells,
 * sequential hyperplane sweeps, sequential norm sums.
 *
 * Parity pins: the restatement is checked against the reference built from
 * its sources (oracle/ref_build) and against golden fixtures generated from
 * that build (tests/golden/). */
#ifndef AITHER_ORACLE_H
#define AITHER_ORACLE_H

#include "aither_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_case orc_case;

orc_case *orc_create(int nblocks, const ath_block_view *blocks, int nsolves,
                     const ath_solve_view *solves);
void orc_destroy(orc_case *c);
/* Number of OpenMP threads used across blocks (0 = library default). */
void orc_set_threads(orc_case *c, int nthreads);

/* Also compute the logged matrix residual in orc_relax (the reference
 * always does, src/linearSolver.cpp:470); read it with orc_matrix_resid. */
void orc_set_matrix_resid(orc_case *c, int on);
/* Keep the cell-averaged gradients of every residual for output
 * (ATH_FIELD_GRADS of orc_get_field). */
void orc_set_output_grads(orc_case *c, int on);
/* Multigrid: link level c to its next coarser level `coarse` (cycle index 1
 * V, 2 W); maps[b] is the transfer of block b of c (ath_setup_mg_map).
 * orc_relax of the finest level then runs the cycle over the linked levels
 * (mgSolution::CycleAtLevel, src/mgSolution.cpp:160). */
void orc_set_coarse(orc_case *c, orc_case *coarse, int cycle, const ath_mg_map *maps);
double orc_matrix_resid(const orc_case *c, int solve);

/* Integrated wall forces of the last residual evaluation: sum over the
 * viscous-wall faces of p_w A (area vector, 3 values) then tau_w |A| (3). */
void orc_forces(const orc_case *c, int solve, double *out6);

/* Stages of one nonlinear iteration, in order. */
void orc_fill_ghosts(orc_case *c);
void orc_residual(orc_case *c);
void orc_timestep(orc_case *c);
void orc_diag_invert(orc_case *c);
void orc_relax(orc_case *c);
/* l2_out: nsolves*7 (sqrt taken; entries 5 and 6 are the k and omega
 * equations of RANS solves, 0 otherwise); linf_out: nsolves (may be NULL) */
int orc_update(orc_case *c, double *l2_out, double *linf_out);

/* n full iterations; l2_out receives n*nsolves*7 values (may be NULL).
 * Returns 0, or -6 when a nonphysical state appeared. */
int orc_iterate(orc_case *c, int n, double *l2_out);

/* Fields as in ath_batch_get_field (ATH_FIELD_*). */
int orc_get_field(orc_case *c, int block, int field, double *out);
int orc_set_state(orc_case *c, int block, const double *prim);
int orc_set_state_nm1(orc_case *c, int block, const double *cons);

#ifdef __cplusplus
}
#endif

#endif
