/* warp_reactor_diff.h -- C ABI of the differentiation form.
 *
 * The reference has no gradient path; these entry points have no counterpart in
 * it.  They differentiate the gridwide-independent chemistry map of one grid
 * (prepare_grid_timestep_kernel + advance_collapse_gridwide_kernel per cell,
 * reference reproducer.cpp:7696-7785) through a given outer schedule:
 *
 *   inputs   u[n][15]  per cell xn[0..13] and T (the record's other fields are
 *                      held fixed; e is recomputed from T before every burn)
 *            p[P]      log multipliers of the network's P rate coefficients
 *                      (P = wr_diff_num_multipliers())
 *   outputs  q[n][15]  per cell the final xn[0..13] and T
 *
 * The schedule dt_hist[0..nsteps) is the list of grid timesteps of a plain run of
 * the same grid (wr_grid_dt_history); the map applies it as given.  The forward
 * pass runs the reference's ROS2S controller and records the accepted step
 * sizes; the adjoint differentiates the map that takes exactly those steps.
 * With p == 0 and the plain run's schedule the forward reproduces the plain run
 * bit for bit.
 *
 * All array arguments except dt_hist are device pointers on the context's
 * device; every call is synchronous.  Status codes are the WR_* values of
 * warp_reactor.h (WR_SUCCESS = 1). */
#ifndef WARP_REACTOR_DIFF_H
#define WARP_REACTOR_DIFF_H

#include "warp_reactor.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wr_diff wr_diff;

/* Number of rate-coefficient multipliers P of the network. */
int wr_diff_num_multipliers(void);

/* Context for num_cells cells, schedules of up to max_outer_steps steps and up to
 * max_accepted_per_cell accepted ROS2S steps per cell over the whole schedule
 * (a cell that needs more fails with WR_TOO_MANY_STEPS).  Device memory:
 * 8*(18*max_outer_steps + 1.03*max_accepted_per_cell + 9600) + 5*max_outer_steps
 * bytes per cell.  NULL on bad sizes or allocation failure. */
wr_diff* wr_diff_create(int num_cells, int max_outer_steps, int max_accepted_per_cell, int device);
void wr_diff_destroy(wr_diff* d);
const char* wr_diff_last_error(wr_diff* d);

/* Forward map.  d_cells: num_cells records (device); d_u: num_cells x 15 or NULL
 * (the records' own xn and T); d_log_mult: P values or NULL (all 0); dt_hist:
 * HOST array of nsteps > 0 grid timesteps; d_q: num_cells x 15 output.  Keeps what
 * the adjoint needs.  Returns the first failing cell's code (index order). */
int wr_diff_forward(wr_diff* d, const wr_collapse_state* d_cells, const double* d_u, const double* d_log_mult,
                    const double* dt_hist, int nsteps, int perturb, double* d_q);

/* Adjoint of the last successful forward: d_qbar (num_cells x 15) -> d_ubar
 * (num_cells x 15, overwritten) and d_pbar (P, overwritten).  The multiplier
 * gradient is summed over cells in index order (reproducible bit for bit). */
int wr_diff_backward(wr_diff* d, const double* d_qbar, double* d_ubar, double* d_pbar);

/* The accepted step sizes of the last forward, HOST arrays: h_hbuf
 * num_cells x max_accepted_per_cell (row i: cell i's steps in order) and h_counts
 * num_cells x nsteps (accepted steps of each outer step's burn). */
int wr_diff_record(wr_diff* d, double* h_hbuf, int* h_counts);

#ifdef __cplusplus
}
#endif

#endif /* WARP_REACTOR_DIFF_H */
