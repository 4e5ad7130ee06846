/*
 * warp_reactor.h -- C ABI of the GB300 primordial-chemistry grid integrator.
 *
 * The integrator advances N independent chemistry cells (14 species number
 * densities + internal energy) through the free-fall collapse schedule of the
 * reference reproducer under the "gridwide-independent" policy: every outer step a
 * prepare kernel perturbs each cell and publishes its free-fall dt, the device
 * takes the grid-wide minimum, and the advance kernel integrates every cell over
 * that dt with its own ROS2S controller.
 *
 * Conventions
 *  - Every entry point returns an int status with the reference's
 *    IntegratorResult values (reproducer.cpp:30-37): WR_SUCCESS = 1 on success,
 *    a negative code on failure.  Nothing throws across this boundary.
 *  - The first failure recorded on the device wins (compare-and-swap from
 *    WR_SUCCESS), as in reproducer.cpp:7716,7724,7782.  After a failure the cell
 *    states may be partially committed, as in the reference.
 *  - A context owns all device memory it allocates; host arrays belong to the
 *    caller.  One context = one CUDA device and one stream; calls are synchronous
 *    with respect to the host and must come from one host thread at a time.
 *  - wr_collapse_state has the byte layout of the reference's CollapseState
 *    (reproducer.cpp:7455-7461, 216 bytes), so a reference caller can pass
 *    cells.data() of its std::vector<CollapseState> directly.
 */
#ifndef WARP_REACTOR_H
#define WARP_REACTOR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WR_NUM_SPECIES 14
#define WR_NEQS 15
#define WR_MAX_COLLAPSE_STEPS 1000

/* IntegratorResult codes, reproducer.cpp:30-37. */
enum {
    WR_SUCCESS = 1,
    WR_BAD_INPUTS = -1,
    WR_DT_UNDERFLOW = -2,
    WR_TOO_MANY_STEPS = -4,
    WR_TOO_MUCH_ACCURACY_REQUESTED = -5,
    WR_LU_DECOMPOSITION_ERROR = -7
};

/* IntegratorStats, reproducer.cpp:7433-7441. */
typedef struct wr_integrator_stats {
    uint64_t internal_steps;
    uint64_t rhs_calls;
    uint64_t jacobian_calls;
    uint64_t decompositions;
    uint64_t linear_solves;
    uint64_t accepted_steps;
    uint64_t rejected_steps;
} wr_integrator_stats;

/* CollapseState (burn_t current; time; density_driver; completed_steps; stats),
 * reproducer.cpp:263-268 and 7455-7461.  Species order: E, Hp, H, Hm, Dp, D, H2p,
 * Dm, H2, HDp, HD, HEpp, HEp, HE (reproducer.cpp:228-229). */
typedef struct wr_collapse_state {
    double rho;
    double T;
    double e;
    double xn[WR_NUM_SPECIES];
    double time;
    double density_driver;
    int32_t completed_steps;
    int32_t reserved_;
    wr_integrator_stats stats;
} wr_collapse_state;

/* Packed 172-byte final-state record of final_states_grid<N>_<backend>.bin,
 * reproducer.cpp:7488-7505 (little-endian, no padding). */
#pragma pack(push, 1)
typedef struct wr_packed_final_state {
    int32_t cell, i, j, k, completed_steps;
    double time, density_driver, rho, T, e;
    double xn[WR_NUM_SPECIES];
} wr_packed_final_state;
#pragma pack(pop)

/* Arithmetic used for exp/log/cbrt on the device.
 *  WR_MATH_CUDA: CUDA's libm, the arithmetic of the reference's own CUDA build
 *    (reproducer.cpp compiled by nvcc): every result, substep count included,
 *    equals the reference CUDA kernel's bit for bit.  The default of
 *    wr_run_cells, the CLI and the Python mirror.
 *  WR_MATH_PORTABLE: the project's own bit-reproducible exp/log/cbrt (integer
 *    fixed-point cores, no FP64 instructions), identical on the GPU and in the
 *    CPU oracle; within an ulp of CUDA's and glibc's, which the adaptive
 *    controller amplifies to ~1e-5 relative in final T over a collapse. */
enum { WR_MATH_PORTABLE = 0, WR_MATH_CUDA = 1 };

typedef struct wr_ctx wr_ctx;

/* Create a context for num_cells cells on CUDA device `device`.  Allocates the
 * structure-of-arrays cell state and the step scratch.  Replaces the allocation
 * half of run_cells_cuda (reproducer.cpp:7794-7828). */
int wr_create(int num_cells, int device, int math_mode, wr_ctx** out);

/* A context holding several independent grids batched in one state (the batching
 * form): grid g owns cells [sum(cells_per_grid[0..g-1]), ... + cells_per_grid[g])
 * and runs its own gridwide-independent schedule (its own grid minimum, clock,
 * completed steps and failure code), while one prepare / advance launch covers
 * every cell of every grid.  Each grid gives the same result as a one-grid
 * context of its cells.  Host-stepped wr_prepare / wr_advance need one grid; use
 * wr_run.  No reference counterpart (the reference runs one grid per process). */
int wr_create_batch(int num_grids, const int* cells_per_grid, int device, int math_mode, wr_ctx** out);

/* Completed global steps and IntegratorResult of one grid after wr_run. */
int wr_grid_result(wr_ctx* ctx, int grid, int* completed_global_steps, int* result);

/* Grid dt per outer step of one grid of the last wr_run. */
int wr_grid_dt_history(wr_ctx* ctx, int grid, double* out, int max_steps);

/* Outer-step policy of wr_run.
 *  WR_POLICY_GRIDWIDE_INDEPENDENT: one grid-wide dt per step, the minimum over
 *    cells (the reference CUDA program, reproducer.cpp:7696-7785).  Default.
 *  WR_POLICY_LEGACY_LOCAL: every cell advances with its own free-fall dt (the
 *    reference CPU program's default, advance_collapse_step, :7646-7685 and the
 *    loop at :8630-8648); its final_states_grid<N>_cpu.bin is reproduced.
 *  WR_POLICY_GRIDWIDE_CTA32: the grid-wide dt, and one ROS2S controller per tile of
 *    32 consecutive cells (tile error = maximum over its cells), the reference's
 *    structured CUDA policy (advance_collapse_gridwide_structured_kernel,
 *    structured_cuda.cuh:393-782).  One grid. */
enum { WR_POLICY_GRIDWIDE_INDEPENDENT = 0, WR_POLICY_LEGACY_LOCAL = 1, WR_POLICY_GRIDWIDE_CTA32 = 2 };
int wr_set_policy(wr_ctx* ctx, int policy);

/* Release every device buffer of the context (reproducer.cpp:7967-7973). */
void wr_destroy(wr_ctx* ctx);

/* Copy num_cells host records into the device state (AoS -> SoA transpose on the
 * device) and reset the failure code.  reproducer.cpp:7822-7834. */
int wr_upload(wr_ctx* ctx, const wr_collapse_state* cells);

/* Copy the device state back into host records (SoA -> AoS).
 * reproducer.cpp:7961-7966. */
int wr_download(wr_ctx* ctx, wr_collapse_state* cells);

/* One prepare launch plus the device grid minimum.  Replaces
 * prepare_grid_timestep_kernel (reproducer.cpp:7696-7734) and the host scan of
 * all candidates (reproducer.cpp:7865-7893).  *dt_grid_out receives the minimum
 * candidate dt, or DBL_MAX when no cell is a candidate. */
int wr_prepare(wr_ctx* ctx, int completed_global_steps, double grid_time, int step,
               int perturb, double* dt_grid_out);

/* One advance launch.  Replaces advance_collapse_gridwide_kernel
 * (reproducer.cpp:7736-7785) and the counter read-back (:7903-7956).
 * *integrated_out receives the number of cells that committed the step. */
int wr_advance(wr_ctx* ctx, int completed_global_steps, double next_grid_time,
               double dt_grid, int* integrated_out);

/* The whole outer loop (reproducer.cpp:7856-7959) on the device state: up to
 * WR_MAX_COLLAPSE_STEPS prepare/min/advance steps.  *completed_global_steps is read
 * as the starting count and receives the final count. */
int wr_run(wr_ctx* ctx, int perturb, int* completed_global_steps);

/* Copy the grid dt of each outer step of the last wr_run (the value the reference
 * computes on the host at reproducer.cpp:7888-7893) into out[0..max_steps-1]. */
int wr_dt_history(wr_ctx* ctx, double* out, int max_steps);

/* Device-time breakdown of the last wr_run, measured with CUDA events on the
 * context's stream (collected only after wr_set_profiling(ctx, 1)).  The
 * reference times the whole run on the host (reproducer.cpp:8626-8651); these
 * are the per-kernel figures behind that number. */
typedef struct wr_run_timing {
    double run_ms;        /* first launch to last launch of wr_run */
    double prepare_ms;    /* sum over prepare launches */
    double advance_ms;    /* sum over advance launches */
    int32_t prepare_launches;
    int32_t advance_launches;
    int32_t outer_steps;  /* completed global steps of the run */
    int32_t reserved_;
} wr_run_timing;

int wr_set_profiling(wr_ctx* ctx, int on);

/* Launch shape of the advance kernel (the knob the autotuner sweeps):
 *   0  one lane per cell, 128 lanes per SM, iteration matrix in shared memory
 *   1  one lane per cell, 256 lanes per SM (2 blocks of 128), matrix in global memory
 *   2  one lane per cell, 256 lanes per SM (1 block of 256), matrix in global memory
 *   3  the precision form: 256 lanes per SM, the iteration matrix factorised in
 *      FP32 with one FP64-residual refinement sweep per stage solve; RHS,
 *      exp/log, stage combination, error norm, controller and EOS stay FP64
 *   4  one lane per cell, 384 lanes per SM (1 block), matrix in global memory
 *   5  cooperative: 8 lanes per cell (4 cells per warp), 9 warps per SM
 *   6  cooperative: 16 lanes per cell (2 cells per warp), 16 warps per SM (default)
 *   7  cooperative: 32 lanes per cell (1 cell per warp), 16 warps per SM
 * The cooperative advance evaluates one cell's network, LU factorisation and
 * triangular solves with a group of lanes (generated vector programs, a
 * warp-cooperative LU with shuffle pivot search, shared-memory matrices).
 * Variants 0-2 and 4-7 give identical results (only the speed differs); variant
 * 3 approximates the FP64 result.  No reference counterpart (the reference fixes
 * one thread per cell, 128 threads per block, reproducer.cpp:7398). */
int wr_set_advance_variant(wr_ctx* ctx, int variant);

/* Autotuner: times the first `steps` outer steps of the uploaded state with each
 * exact launch shape (variants 0-2 and 4-7: lanes per cell 1, 8, 16, 32 and the
 * lane-per-cell block shapes), restores the state, selects the fastest and returns
 * it in *best_variant.  The precision form is never chosen by it. */
int wr_autotune(wr_ctx* ctx, int perturb, int steps, int* best_variant);
int wr_get_run_timing(wr_ctx* ctx, wr_run_timing* out);

/* Drop-in for run_cells_cuda (reproducer.cpp:7791-7975): create, upload, run,
 * download, destroy, on the current CUDA device, with WR_MATH_CUDA (the
 * reference CUDA build's arithmetic, so the result is the reference's). */
int wr_run_cells(wr_collapse_state* cells, int num_cells, int perturb,
                 int* completed_global_steps);

/* No-allocation advance.  Some callers cannot allocate device memory: they keep
 * their cells in device buffers owned by another framework's allocator or pool,
 * or run on a device whose memory is budgeted for them.  This entry point runs
 * one advance step on num_cells <= WR_NOALLOC_MAX_CELLS records in the caller's
 * device memory, updated in place, and allocates nothing: its scratch is one
 * fixed file-scope device array (7.9 MiB, resident on every GPU that loads the
 * library until the process exits).  Its arithmetic is WR_MATH_PORTABLE: the
 * result equals wr_advance of a WR_MATH_PORTABLE context on those cells bit for
 * bit.  Calls share the scratch array, so calls that overlap on the GPU race;
 * issue them one at a time.  The first call on a device looks up the array's
 * device address (cudaGetSymbolAddress) and caches it for the process; do not
 * use the entry point across a cudaDeviceReset of that device.  Every call runs
 * on the legacy default stream and returns after the step completes (a blocking
 * copy), with *integrated_out = cells committed: issue no call while any stream
 * capture is active, and order the caller's own writes to the cells on
 * non-blocking streams before the call (cudaStreamSynchronize or an event).
 * No counterpart in the reference. */
#define WR_NOALLOC_MAX_CELLS 4096
#define WR_NOALLOC_LANES 4096
int wr_advance_cells_noalloc(wr_collapse_state* d_cells, int num_cells, int completed_global_steps,
                             double next_grid_time, double dt_grid, int* integrated_out);

/* Text of the last error of wr_advance_cells_noalloc on this host thread. */
const char* wr_noalloc_last_error(void);

/* The reference's initial collapse cell (make_collapse_state,
 * reproducer.cpp:7533-7546). */
void wr_make_collapse_state(wr_collapse_state* out);

/* A seeded initial cell of the batching workload (no reference counterpart; the
 * reference has one initial cell): make_collapse_state with density scaled by
 * 10^(sigma_dex * N(0,1)) and T log-uniform in [10^log10_tmin, 10^log10_tmax],
 * e from the EOS.  Deterministic in (grid_id, cell). */
void wr_make_batch_state(int grid_id, int cell, double sigma_dex, double log10_tmin, double log10_tmax,
                         wr_collapse_state* out);

/* Text of the last error recorded on this host thread ("" if none). */
const char* wr_last_error(void);

/* Number of kernels this library has launched since it was loaded. */
uint64_t wr_kernel_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* WARP_REACTOR_H */
