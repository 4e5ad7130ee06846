// wr_diff.cuh -- differentiation form: forward map with recorded controller and
// its hand-written discrete adjoint.
//
// The differentiable map.  One grid of cells (one record per cell, as uploaded to
// the integrator) is advanced through a given outer schedule dt_hist[0..S) -- the
// grid timesteps of a gridwide-independent run of the same grid, which depend on
// the densities only -- exactly as the gridwide kernels do it for each cell
// (prepare_grid_timestep_kernel, reproducer.cpp:7696-7734, then
// advance_collapse_gridwide_kernel, :7736-7785), with
//   * a log multiplier p[r] on each of the network's rate coefficients (the RHS is
//     evaluated with k_r * exp(p[r]); at p == 0 it is the plain RHS, bit for bit);
//   * the accepted ROS2S step sizes recorded by the forward pass and held fixed
//     by the adjoint (the "frozen controller": the adjoint differentiates the map
//     that takes exactly those steps).
// Inputs u: per cell xn[0..13] and T (e is recomputed from T before every burn;
// rho, driver and the other fields are held fixed).  Outputs q: per cell the final
// xn[0..13] and T.  With the schedule of a plain run and p == 0 the forward map
// reproduces that run bit for bit.
//
// Kernels (one thread per cell; cells are independent once the schedule is given):
//   k_diff_forward   the cell's whole schedule with the reference controller
//                    (RODAS::integrate, :7205-7347); stores per outer step the
//                    cell's state at the start of the step (18 doubles,
//                    outer-step checkpoints) and the accepted step sizes
//   k_diff_backward  reverse sweep over the outer steps: each step is recomputed
//                    from its checkpoint, its burn is replayed with a checkpoint
//                    every 32 accepted steps, and each 32-step segment is
//                    recomputed and reversed step by step (adjoint of the three
//                    ROS2S stages, the transposed LU solves, the RHS and Jacobian
//                    vector-Jacobian products of the generated network code, the
//                    EOS, normalisation, charge balance, perturbation and driver
//                    updates)
//   k_diff_reduce    per-cell multiplier adjoints summed in cell order (fixed
//                    order: the gradient is reproducible bit for bit)
//
// HBM layout (n cells, S outer steps, cap accepted steps per cell):
//   ckpt   [S][18][n]   doubles, coalesced per field
//   counts [S][n]       accepted steps of the burn at each outer step
//   kind   [S][n]       0 not live, 1 stopped in prepare (dt < 10 s), 2 stopped at
//                       the density limit, 3 burned
//   hbuf   [n][cap]     accepted step sizes in order, one row per cell
//   segck  [n][cap/32+1][15]   burn-segment checkpoints (backward scratch)
//   ys     [n][32][15]  states of the segment being reversed (backward scratch)
//   stage  [n][32][271] LU, pivots and stage vectors of those steps (backward scratch)
//   mbar   [n][P]       per-cell multiplier adjoints
//
// Source files: wr_diff.cu (forward kernel, C ABI), wr_diff_bwd.cu (adjoint
// kernel), wr_diff_net.cu (network RHS/Jacobian and RHS vector-Jacobian product),
// wr_diff_jvjp0.cu / wr_diff_jvjp1.cu (Jacobian vector-Jacobian product in
// chunks).  They are compiled as relocatable device code and device-linked: the
// generated derivative code is tens of thousands of statements, and one
// translation unit of it takes ptxas minutes; split, the pieces compile in
// parallel.
#pragma once

#include <cuda_runtime.h>

#include "../../include/warp_reactor.h"
#include "../../include/warp_reactor_diff.h"
#include "wr_kernels.cuh"

namespace wr {
namespace diff {

constexpr int NP = 44;        // rate-coefficient multipliers (WR_NUM_RATE_MULT, checked where generated code is included)
constexpr int kFields = 18;   // xn[14], T, e, rho, driver
constexpr int kSeg = 32;      // accepted steps between burn checkpoints
constexpr int kThreads = 32;  // one warp per block: a small grid spreads over all SMs
// per-step record of the adjoint's segment pass: LU (225), pivots (1), k1, k2, k3
constexpr int kStageIp = NEQ * NEQ;
constexpr int kStageK1 = kStageIp + 1;
constexpr int kStageK2 = kStageK1 + NEQ;
constexpr int kStageK3 = kStageK2 + NEQ;
constexpr int kStage = kStageK3 + NEQ;

using M = PortableMath;

struct MatL {
    double* a;
    __device__ __forceinline__ double& operator()(int r, int c) const { return a[r * NEQ + c]; }
};

struct LocalJSink {
    double* J;
    __device__ __forceinline__ void operator()(int r, int c, double v) { J[r * NEQ + c] = v; }
};

// network routines (wr_diff_net.cu, wr_diff_jvjp1.cu), one out-of-line copy each
__device__ void net_jac(const double* X, double T, double* J);
__device__ void net_rhs(const double* X, double T, const double* mult, double* f);
__device__ void net_rhs_vjp(const double* X, double T, const double* mult, const double* fbar, double* Xbar,
                            double* Tbar, double* mbar);
__device__ void net_jac_vjp(const double* X, double T, const double* Jbar, double* Xbar, double* Tbar);

struct Args {
    const wr_collapse_state* cells;
    const double* u;        // [n][15] or null
    const double* mult;     // [P] exp(p)
    const double* dt_hist;  // [S]
    int nsteps, perturb, n, cap, nseg;
    double* ckpt;
    int* counts;
    unsigned char* kind;
    double* hbuf;
    double* q;              // [n][15]
    int* status;            // [n]
    // backward
    const double* qbar;     // [n][15]
    double* ubar;           // [n][15]
    double* segck;
    double* ys;
    double* stage;          // [n][32][kStage]
    double* mbar;           // [n][P]
};

// forward pieces (wr_diff.cu)
__device__ void ros2s_stages(const double* y, double h, MatL E, uint64_t ip, const double* mult, double* ak1,
                             double* ak2, double* ak3, double* ynew, double* work);
__device__ int factor(const double* J, double h, MatL E, uint64_t& ip);
// one accepted step of the frozen controller; with st != nullptr it also stores
// the step's factorised iteration matrix, pivots and stage vectors (kStage doubles)
__device__ void step_replay(double* y, double h, const double* mult, double* st);

__global__ void k_diff_forward(Args a);
__global__ void k_diff_backward(Args a);
__global__ void k_diff_mult(const double* logm, double* mult);
__global__ void k_diff_reduce(const double* mbar, const double* mult, int n, double* pbar);

struct CellS {
    double xn[NS], T, e, rho, driver;
};

__device__ __forceinline__ void save_ckpt(const Args& a, int s, int i, const CellS& c) {
    double* p = a.ckpt + static_cast<size_t>(s) * kFields * a.n + i;
#pragma unroll
    for (int k = 0; k < NS; ++k) p[static_cast<size_t>(k) * a.n] = c.xn[k];
    p[static_cast<size_t>(14) * a.n] = c.T;
    p[static_cast<size_t>(15) * a.n] = c.e;
    p[static_cast<size_t>(16) * a.n] = c.rho;
    p[static_cast<size_t>(17) * a.n] = c.driver;
}
__device__ __forceinline__ void load_ckpt(const Args& a, int s, int i, CellS& c) {
    const double* p = a.ckpt + static_cast<size_t>(s) * kFields * a.n + i;
#pragma unroll
    for (int k = 0; k < NS; ++k) c.xn[k] = p[static_cast<size_t>(k) * a.n];
    c.T = p[static_cast<size_t>(14) * a.n];
    c.e = p[static_cast<size_t>(15) * a.n];
    c.rho = p[static_cast<size_t>(16) * a.n];
    c.driver = p[static_cast<size_t>(17) * a.n];
}

// prepare part of outer step s (perturbation, free-fall dt).  Returns the kind of
// step: 1 stopped (dt < 10 s), otherwise 3 (candidate); -1 invalid state.
__device__ __forceinline__ int prepare_part(const Args& a, int s, int i, CellS& c, double& dt) {
    if (a.perturb && s != 0 && s % kPerturbInterval == 0) {
        const double f = perturbation_factor(i, s);
        c.driver *= f;
        c.rho = c.rho * f;
#pragma unroll
        for (int k = 0; k < NS; ++k) c.xn[k] *= f;
        renormalize(c.xn, c.rho);
        c.T = eos_T_from_e(c.xn, c.e);
    }
    dt = collapse_timestep(c.xn);
    if (!valid_positive(dt) || !valid_positive(c.driver)) return -1;
    if (dt < 10.0) {
        const double tff = ddiv(dt, kTffReduc);
        c.driver += dt * ddiv(c.driver, tff);
        return 1;
    }
    return 3;
}

// advance part up to the burn.  Returns 2 when the density limit stops the cell,
// 3 when the cell burns (y holds the burn's initial state).
__device__ __forceinline__ int advance_part(double dt_grid, double dt, CellS& c, double* y) {
    const double old_density = c.driver;
    const double tff = ddiv(dt, kTffReduc);
    c.driver = old_density + dt_grid * ddiv(old_density, tff);
    if (!valid_positive(c.driver) || c.driver > kDriverLimit) return 2;
    const double ratio = ddiv(c.driver, old_density);
#pragma unroll
    for (int k = 0; k < NS; ++k) c.xn[k] *= ratio;
    c.rho = c.rho * ratio;
    c.e = eos_e_from_T(c.xn, c.T);
#pragma unroll
    for (int k = 0; k < NS; ++k) y[k] = c.xn[k];
    y[NS] = c.e;
    return 3;
}

__device__ __forceinline__ void commit_part(CellS& c, const double* y) {
#pragma unroll
    for (int k = 0; k < NS; ++k) c.xn[k] = y[k];
    renormalize(c.xn, c.rho);
    c.T = eos_T_from_e(c.xn, y[NS]);
    c.e = y[NS];
}

}  // namespace diff
}  // namespace wr
