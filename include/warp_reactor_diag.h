/*
 * warp_reactor_diag.h -- diagnostic entry points of the GB300 library.
 *
 * Each runs one piece of the device integrator on caller-supplied inputs so that
 * tests can compare it with the CPU oracle and with the reference's own test
 * fixtures.  Inputs and outputs are host arrays; the functions allocate and free
 * their own device buffers and run on the current CUDA device.  Return values are
 * IntegratorResult codes (WR_SUCCESS = 1).
 */
#ifndef WARP_REACTOR_DIAG_H
#define WARP_REACTOR_DIAG_H

#include "warp_reactor.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The network at n burn states (X: n x 14 floored number densities, T: n
 * temperatures): J (n x 225, row-major, the reference's jac(row+1, col+1)) and the
 * fused RHS f_fused (n x 15) from one evaluation, and f_rhs (n x 15) from the
 * RHS-only evaluation.  The reference computes these in actual_jac / actual_rhs
 * (reproducer.cpp:6998-7011, 1515-1535).  math_mode is WR_MATH_PORTABLE or
 * WR_MATH_CUDA. */
int wr_diag_network(int n, const double* X, const double* T, int math_mode,
                    double* J, double* f_fused, double* f_rhs);

/* n independent 15x15 systems: LU factorisation with partial pivoting and the
 * triangular solve, the device code of the advance kernel.  Replaces
 * lu_decomposition<15> / lu_solve<15> (reproducer.cpp:96-181).  A and LU are
 * n x 225 row-major, b and x are n x 15, ipvt and info are n x 15 and n.  The
 * solve runs only where info == 0 (x = b otherwise). */
int wr_diag_lu(int n, const double* A, const double* b, double* LU, int* ipvt, int* info, double* x);

/* The cooperative advance's generated vector programs (lanes_per_cell = 8, 16 or
 * 32 lanes evaluating one cell) at n ROS2S states y (n x 15: 14 number densities
 * and the internal energy): burn_state_from_y (floor, T from e) followed by the
 * fused Jacobian + RHS program (J: n x 225, f: n x 15) and by the RHS-only program
 * (f_rhs: n x 15).  The reference evaluates these in jacobian() / rhs() of its
 * ROS2S system (reproducer.cpp:7029-7049). */
int wr_diag_coop_network(int lanes_per_cell, int n, const double* y, int math_mode, double* J, double* f,
                         double* f_rhs);

/* The cooperative (lanes_per_cell = 8, 16 or 32) LU factorisation and triangular
 * solve of the advance kernel on n 15x15 systems; arguments as wr_diag_lu.
 * Replaces lu_decomposition<15> / lu_solve<15> (reproducer.cpp:96-181). */
int wr_diag_coop_lu(int lanes_per_cell, int n, const double* A, const double* b, double* LU, int* ipvt,
                    int* info, double* x);

/* Elementwise exp (fn = 0), log (fn = 1) or cbrt (fn = 2) of n values on the
 * device with the given math mode: the functions std::exp / std::log / std::cbrt
 * of the reference's network and controller (reproducer.cpp:342-6994, 7309). */
int wr_diag_math(int n, const double* x, int fn, int math_mode, double* out);

/* Elementwise a[i] / b[i] with the device's integer-pipe division (the kernels'
 * division everywhere in the integrator): must equal IEEE binary64 division bit
 * for bit.  The reference divides with the hardware operator throughout
 * (reproducer.cpp:96-181, 284-339, 7205-7347). */
int wr_diag_div(int n, const double* a, const double* b, double* out);

/* Evict the GPU's L2 cache by writing `mib` MiB of device memory (a buffer kept
 * for the life of the process), so a following timed run starts cold like the
 * reference's first launch.  No reference counterpart (benchmark hygiene). */
int wr_diag_flush_l2(int mib);

/* FP64 issue interval of one warp: one block of `warps` warps on one SM, every lane
 * running `chains` (1, 4 or 8) independent dependent-FMA chains; returns SM clock
 * cycles per FMA instruction per warp.  No reference counterpart: the
 * measurement behind the advance kernel's launch shape. */
int wr_diag_fp64_issue(int warps, int chains, double* cycles_per_instr);

/* Measured FP64 throughput of this GPU: independent FMA chains in every lane of a
 * full grid, timed with CUDA events.  *dfma_per_s receives FP64 FMA instructions
 * per second per GPU (one FMA = 2 FLOP).  No reference counterpart: the roofline
 * denominator of the reference's FP64-bound path, measured on the same device. */
int wr_diag_fp64_peak(double* dfma_per_s);

/* Phase counters of the cooperative advance.  No reference counterpart: a
 * diagnostic of where an attempt's time goes.  With on != 0 the context's
 * cooperative advance launches (wr_advance, wr_run) run an instrumented
 * instantiation of the kernel that adds, per warp, the clock64 cycles of each
 * phase of its ROS2S attempts into 16 device counters (allocated here, zeroed):
 *   [0] work queue, prologue and epilogue   [1] Jacobian+RHS program
 *   [2] output loads, Jacobian gather, diagonal, stage combinations
 *   [3] LU and the pivots' reciprocals      [4] stage solves
 *   [5] RHS programs                        [6] error norm and step-size control
 *   [7] attempts (per warp: two cells at 16 lanes per cell)
 *   [8] cycles from a warp's start to its exit   [9] warps
 * Results are unchanged; the counters cost a few percent of speed.  on = 0
 * frees them and returns to the plain kernel. */
int wr_diag_coop_phases(wr_ctx* ctx, int on);

/* Copy the 16 phase counters to out16 (host) and, with reset != 0, zero them.
 * Fails when the counters are off. */
int wr_diag_coop_phases_read(wr_ctx* ctx, unsigned long long* out16, int reset);

#ifdef __cplusplus
}
#endif

#endif /* WARP_REACTOR_DIAG_H */
