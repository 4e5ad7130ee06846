// wr_kernels.cuh -- device kernels of the gridwide-independent integrator.
//
// Data layout in HBM (structure of arrays, one slot per cell, coalesced):
//   rho[N] T[N] e[N] xn[14][N] time[N] driver[N] steps[N] stats[7][N]
// Step control lives in one small device struct (StepCtl) so that a whole outer
// step -- prepare, grid minimum, advance, commit -- runs without a host round
// trip and can be captured in a CUDA graph.
//
// Kernels (reference counterparts in reproducer.cpp):
//   k_unpack / k_pack      AoS host records <-> SoA device state (H2D/D2H at
//                          :7822-7828, :7961-7966)
//   k_prepare              prepare_grid_timestep_kernel (:7696-7734) fused with
//                          the grid minimum (host scan at :7888-7893): each block
//                          reduces its candidates and does one 64-bit atomicMin on
//                          the bit pattern of a positive double (monotone in value)
//   k_decide               the host checks between the two kernels (:7888-7909)
//   k_advance              advance_collapse_gridwide_kernel (:7736-7785) as a
//                          persistent kernel: every lane owns one cell at a time,
//                          runs the ROS2S controller of RODAS::integrate
//                          (:7205-7347) one attempt per loop trip, and takes the
//                          next cell from a device work queue as soon as its cell
//                          is done, so lanes of a warp stay busy although cells
//                          need 1 to 10+ attempts per step
//   k_finalize             the host bookkeeping after the advance (:7930-7958)
#pragma once

#include <cfloat>
#include <stdint.h>
#include <type_traits>

#include "../../include/warp_reactor.h"
#include "wr_physics.cuh"

#ifndef WR_NET_HD
#define WR_NET_HD __device__ __forceinline__
#endif
#include "generated/network_gen.h"

namespace wr {

struct DevState {
    double* rho;
    double* T;
    double* e;
    double* xn;      // [14][n]
    double* time;
    double* driver;
    int* steps;
    uint64_t* stats;  // [7][n]
    int* cost;        // ROS2S attempts of the cell's last burn (scheduling hint)
    int* order;       // advance work queue: cells of this step, heaviest first
    int* qbucket;     // queue bucket chosen by k_prepare for this step (-1: not queued)
    const int* grid_of;    // sub-grid of each cell (nullptr: one grid)
    const int* grid_start; // first cell of each sub-grid (nullptr: one grid)
    double* local_dt;      // legacy-local policy: each cell's own dt (nullptr: gridwide)
    int n;
    // index of the cell within its own sub-grid is cell - grid_base(g): the
    // perturbation seed of the reference uses the cell's index in its grid
    __device__ __forceinline__ int grid_base(int g) const { return grid_start ? grid_start[g] : 0; }
};

// Work-queue order: cells are bucketed by last step's attempt count, heaviest
// bucket first (longest-processing-time-first list scheduling), so the cells that
// set a step's length start early instead of straggling at the end.
constexpr int kBuckets = 64;
__host__ __device__ __forceinline__ int cost_bucket(int cost) {
    return kBuckets - 1 - (cost < kBuckets - 1 ? (cost > 0 ? cost : 0) : kBuckets - 1);
}

struct StepCtl {
    unsigned long long dmin_bits;  // grid minimum of the candidates (double bits)
    int failure;                   // first failure, WR_SUCCESS otherwise
    int integrated;                // cells committed by the last advance
    int stop;                      // 1 once the outer loop has ended
    int cgs;                       // completed global steps
    int step;                      // outer-loop index (perturbation seed)
    int perturb;
    double grid_time;
    double dt_grid;
    double next_grid_time;
    unsigned int queue;            // work-queue head of k_advance (ctl[0] only)
    unsigned int queued;           // cells in the work queue of this step (ctl[0] only)
    int all_stop;                  // every sub-grid has stopped (ctl[0] only)
    int pad_;
    unsigned int hist[kBuckets];   // queued cells per cost bucket (k_prepare; ctl[0] only)
    unsigned int off[kBuckets];    // bucket start offsets in `order` (ctl[0] only)
};

constexpr unsigned long long kDblMaxBits = 0x7fefffffffffffffULL;

// ------------------------------------------------------------------ math policies
struct PortableMath {
    static __device__ __forceinline__ double exp(double x) { return wr_exp(x); }
    static __device__ __forceinline__ double log(double x) { return wr_log(x); }
    static __device__ __forceinline__ double cbrt(double x) { return wr_cbrt(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double fabs(double x) { return ::fabs(x); }
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
};

struct CudaMath {
    static __device__ __forceinline__ double exp(double x) { return ::exp(x); }
    static __device__ __forceinline__ double log(double x) { return ::log(x); }
    static __device__ __forceinline__ double cbrt(double x) { return ::cbrt(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double fabs(double x) { return ::fabs(x); }
    static __device__ __forceinline__ double div(double a, double b) { return a / b; }
};

// Out-of-line transcendentals: the generated network makes several hundred
// exp/log calls per evaluation; one shared copy keeps the kernel's instruction
// footprint small.
static __device__ __noinline__ double wr_exp_call(double x) { return wr_exp(x); }
static __device__ __noinline__ double wr_log_call(double x) { return wr_log(x); }
struct PortableMathCall {
    static __device__ __forceinline__ double exp(double x) { return wr_exp_call(x); }
    static __device__ __forceinline__ double log(double x) { return wr_log_call(x); }
    static __device__ __forceinline__ double cbrt(double x) { return wr_cbrt(x); }
    static __device__ __forceinline__ double sqrt(double x) { return ::sqrt(x); }
    static __device__ __forceinline__ double fabs(double x) { return ::fabs(x); }
    static __device__ __forceinline__ double div(double a, double b) { return wr_div_call(a, b); }
};

// Batched out-of-line exp/log: the generated network evaluates up to four
// independent exp (log) in one call; inlined side by side, the four integer
// chains interleave, so a warp has four independent instructions ready where one
// chain would stall on its own latency.
static __device__ __noinline__ WrD2 wr_exp2_call(double a, double b) { return {wr_exp(a), wr_exp(b)}; }
static __device__ __noinline__ WrD3 wr_exp3_call(double a, double b, double c) {
    return {wr_exp(a), wr_exp(b), wr_exp(c)};
}
static __device__ __noinline__ WrD4 wr_exp4_call(double a, double b, double c, double d) {
    return {wr_exp(a), wr_exp(b), wr_exp(c), wr_exp(d)};
}
static __device__ __noinline__ WrD2 wr_log2_call(double a, double b) { return {wr_log(a), wr_log(b)}; }
static __device__ __noinline__ WrD3 wr_log3_call(double a, double b, double c) {
    return {wr_log(a), wr_log(b), wr_log(c)};
}
static __device__ __noinline__ WrD4 wr_log4_call(double a, double b, double c, double d) {
    return {wr_log(a), wr_log(b), wr_log(c), wr_log(d)};
}
}  // namespace wr

template <>
struct WrBatch<wr::PortableMathCall> {
    static __device__ __forceinline__ WrD2 exp2(double a, double b) { return wr::wr_exp2_call(a, b); }
    static __device__ __forceinline__ WrD3 exp3(double a, double b, double c) { return wr::wr_exp3_call(a, b, c); }
    static __device__ __forceinline__ WrD4 exp4(double a, double b, double c, double d) {
        return wr::wr_exp4_call(a, b, c, d);
    }
    static __device__ __forceinline__ WrD2 log2(double a, double b) { return wr::wr_log2_call(a, b); }
    static __device__ __forceinline__ WrD3 log3(double a, double b, double c) { return wr::wr_log3_call(a, b, c); }
    static __device__ __forceinline__ WrD4 log4(double a, double b, double c, double d) {
        return wr::wr_log4_call(a, b, c, d);
    }
};

namespace wr {


// ------------------------------------------------------------------ prepare
__device__ __forceinline__ void record_failure(StepCtl* ctl, int code) {
    atomicCAS(&ctl->failure, WR_SUCCESS, code);
}

// One prepare pass over all cells.  With several sub-grids batched in one state
// (s.grid_of != nullptr), each cell reads and reduces into its own sub-grid's
// control block; a warp whose lanes all belong to one sub-grid reduces with
// shuffles and issues one atomic, other warps (sub-grid boundaries) issue one
// atomic per lane.  The queue histogram is global (ctl[0]).
template <int B>
__global__ void __launch_bounds__(B) k_prepare(DevState s, StepCtl* ctl) {
    __shared__ unsigned int hist[kBuckets];
    for (int i = threadIdx.x; i < kBuckets; i += B) hist[i] = 0;
    __syncthreads();
    const int cell = blockIdx.x * B + threadIdx.x;
    const int g = (s.grid_of != nullptr && cell < s.n) ? s.grid_of[cell] : 0;
    StepCtl* c = ctl + g;
    unsigned long long cand = kDblMaxBits;
    int bucket = -1;
    if (cell < s.n && !c->stop && c->failure == WR_SUCCESS) {
        const int n = s.n;
        const int cgs = c->cgs;
        const int step = c->step;
        const int cs = s.steps[cell];
        if (cs >= cgs) {
            if (cs != cgs || s.time[cell] != c->grid_time) {
                record_failure(c, WR_BAD_INPUTS);
            } else {
                double xn[NS];
#pragma unroll
                for (int k = 0; k < NS; ++k) xn[k] = s.xn[k * n + cell];
                double driver = s.driver[cell];
                // apply_perturbation, reproducer.cpp:7564-7580
                if (c->perturb && step != 0 && step % kPerturbInterval == 0) {
                    const double factor = perturbation_factor(cell - s.grid_base(g), step);
                    driver *= factor;
                    const double rho = s.rho[cell] * factor;
#pragma unroll
                    for (int k = 0; k < NS; ++k) xn[k] *= factor;
                    renormalize(xn, rho);
                    const double T = eos_T_from_e(xn, s.e[cell]);
                    s.rho[cell] = rho;
                    s.T[cell] = T;
#pragma unroll
                    for (int k = 0; k < NS; ++k) s.xn[k * n + cell] = xn[k];
                }
                const double dt = collapse_timestep(xn);
                if (!valid_positive(dt) || !valid_positive(driver)) {
                    record_failure(c, WR_BAD_INPUTS);
                } else if (dt < 10.0) {
                    const double tff = ddiv(dt, kTffReduc);
                    driver += dt * ddiv(driver, tff);
                } else {
                    cand = static_cast<unsigned long long>(__double_as_longlong(dt));
                }
                s.driver[cell] = driver;
                bucket = cost_bucket(s.cost[cell]);
                atomicAdd(&hist[bucket], 1u);
            }
        }
    }
    if (cell < s.n) s.qbucket[cell] = bucket;
    // minimum of positive-double bit patterns per sub-grid
    const int g0 = __shfl_sync(0xffffffffu, g, 0);
    if (__all_sync(0xffffffffu, g == g0)) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long o = __shfl_xor_sync(0xffffffffu, cand, off);
            cand = o < cand ? o : cand;
        }
        if ((threadIdx.x & 31) == 0 && cand != kDblMaxBits) atomicMin(&c->dmin_bits, cand);
    } else if (cand != kDblMaxBits) {
        atomicMin(&c->dmin_bits, cand);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kBuckets; i += B)
        if (hist[i]) atomicAdd(&ctl->hist[i], hist[i]);
}

// Prepare of the legacy-local policy (the reference CPU program's default,
// advance_collapse_step up to the burn, reproducer.cpp:7646-7670): each cell
// perturbs, takes its own free-fall dt and density update, and either stops
// (dt < 10 s or density limit) or is queued with its scaled state and dt.
template <int B>
__global__ void __launch_bounds__(B) k_prepare_legacy(DevState s, StepCtl* ctl) {
    __shared__ unsigned int hist[kBuckets];
    for (int i = threadIdx.x; i < kBuckets; i += B) hist[i] = 0;
    __syncthreads();
    const int cell = blockIdx.x * B + threadIdx.x;
    int bucket = -1;
    if (cell < s.n && !ctl->stop && ctl->failure == WR_SUCCESS && s.steps[cell] >= ctl->cgs) {
        const int n = s.n;
        const int step = ctl->step;
        double xn[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) xn[k] = s.xn[k * n + cell];
        double driver = s.driver[cell];
        double rho = s.rho[cell];
        bool changed = false;
        if (ctl->perturb && step != 0 && step % kPerturbInterval == 0) {
            const double factor = perturbation_factor(cell, step);
            driver *= factor;
            rho = rho * factor;
#pragma unroll
            for (int k = 0; k < NS; ++k) xn[k] *= factor;
            renormalize(xn, rho);
            s.T[cell] = eos_T_from_e(xn, s.e[cell]);
            changed = true;
        }
        const double old_density = driver;
        const double dt = collapse_timestep(xn);
        const double tff = ddiv(dt, kTffReduc);
        driver += dt * ddiv(driver, tff);
        if (!(dt < 10.0 || driver > kDriverLimit)) {
            const double ratio = ddiv(driver, old_density);
#pragma unroll
            for (int k = 0; k < NS; ++k) xn[k] *= ratio;
            rho *= ratio;
            s.e[cell] = eos_e_from_T(xn, s.T[cell]);  // burn_ros2s prologue (eos_rt)
            s.local_dt[cell] = dt;
            changed = true;
            bucket = cost_bucket(s.cost[cell]);
            atomicAdd(&hist[bucket], 1u);
        }
        s.driver[cell] = driver;
        if (changed) {
            s.rho[cell] = rho;
#pragma unroll
            for (int k = 0; k < NS; ++k) s.xn[k * n + cell] = xn[k];
        }
    }
    if (cell < s.n) s.qbucket[cell] = bucket;
    __syncthreads();
    for (int i = threadIdx.x; i < kBuckets; i += B)
        if (hist[i]) atomicAdd(&ctl->hist[i], hist[i]);
}

// bucket offsets from the histogram (one thread), resetting the histogram
__device__ __forceinline__ void build_queue_offsets(StepCtl* ctl) {
    unsigned int acc = 0;
    for (int b = 0; b < kBuckets; ++b) {
        ctl->off[b] = acc;
        acc += ctl->hist[b];
        ctl->hist[b] = 0;
    }
    ctl->queued = acc;
    ctl->queue = 0;
}




// ------------------------------------------------------------------ advance
// Per-lane 15x15 matrix storage: element (r, c) of lane l at base[(r*15 + c) * stride]
// with base pointing at the lane's first element, so 32 consecutive lanes touch 32
// consecutive doubles.  Shared memory (stride = threads per block, a compile-time
// constant) or a global per-lane slot array (stride = number of lane slots).
template <int B>
struct Mat {
    double* base;
    __device__ __forceinline__ double& operator()(int r, int c) const { return base[(r * NEQ + c) * B]; }
    __device__ __forceinline__ double& at(int idx) const { return base[idx * B]; }
};
struct MatG {
    double* base;
    int stride;
    __device__ __forceinline__ double& operator()(int r, int c) const { return base[(r * NEQ + c) * stride]; }
    __device__ __forceinline__ double& at(int idx) const { return base[idx * stride]; }
};

// J sink of the generated network: E = -J into the lane's matrix, J into the lane's
// global backup (re-read only when an attempt is retried with the same J)
template <class MT>
struct JSink {
    MT E;
    double* jb;
    int stride;
    __device__ __forceinline__ void operator()(int r, int c, double v) {
        E(r, c) = -v;
        jb[(r * NEQ + c) * stride] = v;
    }
};

// J sink of the precision form: J only into the lane's FP64 global backup
struct JBackupSink {
    double* jb;
    int stride;
    __device__ __forceinline__ void operator()(int r, int c, double v) { jb[(r * NEQ + c) * stride] = v; }
};

// burn_state_from_y (reproducer.cpp:7029-7038): floored X and T from y
__device__ __forceinline__ void state_from_y(const double* y, double* X, double& T) {
#pragma unroll
    for (int k = 0; k < NS; ++k) X[k] = smax(y[k], kFloor);
    T = eos_T_from_e(X, y[NS]);
}

// lu_decomposition<15> (reproducer.cpp:96-151) on the lane's matrix: the same
// pivot rule (first strictly larger |a_ik|), row interchange of columns k..14,
// negated multipliers and column-oriented update, with the operations in the
// reference's order.  The loops stay rolled: the matrix is in memory anyway, and
// a fully unrolled 15x15 elimination is ~20k instructions of code that the
// instruction cache then has to stream for every attempt.  Pivot indices are
// returned packed four bits each (ip = pivot row of column k at bits 4k..4k+3).
template <class MT>
__device__ __forceinline__ int lu_decompose(MT A, uint64_t& ip) {
    int info = 0;
    uint64_t piv = 0;
#pragma unroll 1
    for (int k = 0; k < NEQ - 1; ++k) {
        int p = k;
        double maxv = ::fabs(A(k, k));
#pragma unroll 1
        for (int i = k + 1; i < NEQ; ++i) {
            const double v = ::fabs(A(i, k));
            if (v > maxv) {
                maxv = v;
                p = i;
            }
        }
        piv |= static_cast<uint64_t>(p) << (4 * k);
        if (A(p, k) != 0.0) {
            if (p != k) {
#pragma unroll 1
                for (int j = k; j < NEQ; ++j) {
                    const double t = A(p, j);
                    A(p, j) = A(k, j);
                    A(k, j) = t;
                }
            }
            const double mult = ddiv(-1.0, A(k, k));
#pragma unroll 1
            for (int i = k + 1; i < NEQ; ++i) A(i, k) = A(i, k) * mult;
#pragma unroll 1
            for (int j = k + 1; j < NEQ; ++j) {
                const double t = A(k, j);
#pragma unroll 4
                for (int i = k + 1; i < NEQ; ++i) A(i, j) = A(i, j) + t * A(i, k);
            }
        } else {
            info = k + 1;
        }
    }
    piv |= static_cast<uint64_t>(NEQ - 1) << (4 * (NEQ - 1));
    if (A(NEQ - 1, NEQ - 1) == 0.0) info = NEQ;
    ip = piv;
    return info;
}

// lu_solve<15> (reproducer.cpp:154-181); x stays in registers, the pivot swap is a
// select chain instead of a dynamically indexed register array
template <class MT>
__device__ __forceinline__ void lu_solve(MT LU, const uint64_t ip, double* x) {
#pragma unroll
    for (int k = 0; k < NEQ - 1; ++k) {
        const int p = static_cast<int>((ip >> (4 * k)) & 15);
        double t = x[k];
#pragma unroll
        for (int i = k + 1; i < NEQ; ++i) t = (p == i) ? x[i] : t;
        if (p != k) {
#pragma unroll
            for (int i = k + 1; i < NEQ; ++i) x[i] = (p == i) ? x[k] : x[i];
            x[k] = t;
        }
#pragma unroll
        for (int j = k + 1; j < NEQ; ++j) x[j] = x[j] + t * LU(j, k);
    }
#pragma unroll
    for (int kb = 0; kb < NEQ; ++kb) {
        const int k = NEQ - 1 - kb;
        x[k] = ddiv(x[k], LU(k, k));
        const double t = -x[k];
#pragma unroll
        for (int j = 0; j < k; ++j) x[j] = x[j] + t * LU(j, k);
    }
}

// ---------------------------------------------------------------- precision form
// The iteration matrix factorised in FP32 (shared memory, 900 B per lane), with
// one FP64 residual refinement per stage solve; J itself stays FP64 in the lane's
// global backup, from which both the FP32 matrix and the FP64 residual are built.
template <int B>
struct MatF {
    float* base;
    __device__ __forceinline__ float& operator()(int r, int c) const { return base[(r * NEQ + c) * B]; }
};

template <class MT>
__device__ __forceinline__ int lu_decompose_f32(MT A, uint64_t& ip) {
    int info = 0;
    uint64_t piv = 0;
#pragma unroll 1
    for (int k = 0; k < NEQ - 1; ++k) {
        int p = k;
        float maxv = fabsf(A(k, k));
#pragma unroll 1
        for (int i = k + 1; i < NEQ; ++i) {
            const float v = fabsf(A(i, k));
            if (v > maxv) {
                maxv = v;
                p = i;
            }
        }
        piv |= static_cast<uint64_t>(p) << (4 * k);
        if (A(p, k) != 0.0f) {
            if (p != k) {
#pragma unroll 1
                for (int j = k; j < NEQ; ++j) {
                    const float t = A(p, j);
                    A(p, j) = A(k, j);
                    A(k, j) = t;
                }
            }
            const float mult = -1.0f / A(k, k);
#pragma unroll 1
            for (int i = k + 1; i < NEQ; ++i) A(i, k) = A(i, k) * mult;
#pragma unroll 1
            for (int j = k + 1; j < NEQ; ++j) {
                const float t = A(k, j);
#pragma unroll 4
                for (int i = k + 1; i < NEQ; ++i) A(i, j) = fmaf(t, A(i, k), A(i, j));
            }
        } else {
            info = k + 1;
        }
    }
    piv |= static_cast<uint64_t>(NEQ - 1) << (4 * (NEQ - 1));
    if (A(NEQ - 1, NEQ - 1) == 0.0f) info = NEQ;
    ip = piv;
    return info;
}

template <class MT>
__device__ __forceinline__ void lu_solve_f32(MT LU, const uint64_t ip, float* x) {
#pragma unroll
    for (int k = 0; k < NEQ - 1; ++k) {
        const int p = static_cast<int>((ip >> (4 * k)) & 15);
        float t = x[k];
#pragma unroll
        for (int i = k + 1; i < NEQ; ++i) t = (p == i) ? x[i] : t;
        if (p != k) {
#pragma unroll
            for (int i = k + 1; i < NEQ; ++i) x[i] = (p == i) ? x[k] : x[i];
            x[k] = t;
        }
#pragma unroll
        for (int j = k + 1; j < NEQ; ++j) x[j] = fmaf(t, LU(j, k), x[j]);
    }
#pragma unroll
    for (int kb = 0; kb < NEQ; ++kb) {
        const int k = NEQ - 1 - kb;
        x[k] = x[k] / LU(k, k);
        const float t = -x[k];
#pragma unroll
        for (int j = 0; j < k; ++j) x[j] = fmaf(t, LU(j, k), x[j]);
    }
}

// x <- E^-1 x with E = fac*I - J, the FP32 factors being those of W^-1 E W
// (error-weighted variables, W = diag(atol + rtol |y|)): FP32 solve of
// W^-1 E W x' = W^-1 b, x0 = W x', one FP64 residual r = b - E x0 (J from the
// lane's FP64 backup), FP32 correction solve of the scaled residual
template <class MT>
__device__ __forceinline__ void solve_refined(MT LU, const uint64_t ip, const double* jb, int stride, double fac,
                                              const double* w, double* x) {
    float xf[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) xf[i] = __double2float_rn(ddiv(x[i], w[i]));
    lu_solve_f32(LU, ip, xf);
    double x0[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) x0[i] = static_cast<double>(xf[i]) * w[i];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        double acc = 0.0;
#pragma unroll
        for (int j = 0; j < NEQ; ++j) acc = acc + jb[(i * NEQ + j) * stride] * x0[j];
        xf[i] = __double2float_rn(ddiv(x[i] - (fac * x0[i] - acc), w[i]));
    }
    lu_solve_f32(LU, ip, xf);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) x[i] = x0[i] + static_cast<double>(xf[i]) * w[i];
}

struct Lane {
    // ROS2S controller state of RODAS::integrate (reproducer.cpp:7225-7235)
    double x, h, hacc, erracc, hopt, tout;
    int n_step, n_accept, n_reject, n_jac, n_decomp, nsing;
    bool reject, last, fresh;
};

// Advance kernel configurations (lane slots = blocks x B):
//   B threads per block, MINB resident blocks per SM (register budget), SMEM_E
//   whether the per-lane iteration matrix lives in shared memory (225 doubles per
//   lane) or in the global per-lane array `ebuf`.
//   PREC 0: FP64 factorisation (the plain form); 1: FP32 factorisation in shared
//   memory with one FP64 residual refinement per stage solve (the precision form).
template <class M, int B, int MINB, bool SMEM_E, int PREC = 0>
__global__ void __launch_bounds__(B, MINB) k_advance(DevState s, StepCtl* ctl, double* __restrict__ jbackup,
                                                   double* __restrict__ ebuf) {
    extern __shared__ double smem[];
    using MT = typename std::conditional<SMEM_E && PREC == 0, Mat<B>, MatG>::type;
    MatF<B> E32{reinterpret_cast<float*>(smem) + threadIdx.x};
    if (ctl->all_stop) return;
    const int n = s.n;
    const unsigned int queued = ctl->queued;
    const int lane_slot = blockIdx.x * B + threadIdx.x;
    const int nslots = gridDim.x * B;
    MT E;
    if constexpr (SMEM_E && PREC == 0) {
        E = MT{smem + threadIdx.x};
    } else {
        E = MT{ebuf + lane_slot, nslots};
    }
    double* jb = jbackup + lane_slot;

    Lane L;
    int cell = -1;
    int g = 0;               // sub-grid of the lane's cell
    int cgs = 0;             // its completed global steps
    double next_grid_time = 0.0;
    bool alive = true;   // lane may still take cells
    bool have = false;   // lane holds a cell
    double y[NEQ], f0[NEQ];
    double wsc[PREC ? NEQ : 1];  // precision form: the error weights of the attempt
    uint64_t ip = 0;

    while (__any_sync(0xffffffffu, alive)) {
        // ---- bring the lane to "ready for an attempt"
        while (alive) {
            if (!have) {
                const unsigned int q = atomicAdd(&ctl->queue, 1u);
                if (q >= queued) { alive = false; break; }
                cell = s.order[q];
                g = s.grid_of ? s.grid_of[cell] : 0;
                const StepCtl* c = ctl + g;
                if (c->stop || c->failure != WR_SUCCESS) continue;
                cgs = c->cgs;
                if (s.steps[cell] != cgs) continue;
                s.cost[cell] = 0;
                double dt_grid;
                if (s.local_dt == nullptr) {
                    dt_grid = c->dt_grid;
                    next_grid_time = c->next_grid_time;
                    // advance_collapse_gridwide_kernel prologue, reproducer.cpp:7748-7768
                    double xn[NS];
#pragma unroll
                    for (int k = 0; k < NS; ++k) xn[k] = s.xn[k * n + cell];
                    const double local_dt = collapse_timestep(xn);
                    if (local_dt < 10.0) continue;
                    const double old_density = s.driver[cell];
                    const double tff = ddiv(local_dt, kTffReduc);
                    const double driver = old_density + dt_grid * ddiv(old_density, tff);
                    s.driver[cell] = driver;
                    if (!valid_positive(driver) || driver > kDriverLimit) continue;
                    const double ratio = ddiv(driver, old_density);
#pragma unroll
                    for (int k = 0; k < NS; ++k) xn[k] *= ratio;
                    const double rho = s.rho[cell] * ratio;
                    // burn_ros2s prologue (reproducer.cpp:7594-7606): e from T
                    const double e = eos_e_from_T(xn, s.T[cell]);
                    // the scaled pre-burn state is what a failed burn leaves behind
                    s.rho[cell] = rho;
                    s.e[cell] = e;
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        s.xn[k * n + cell] = xn[k];
                        y[k] = xn[k];
                    }
                    y[NS] = e;
                } else {
                    // legacy-local: k_prepare_legacy has scaled the cell and set its own dt
                    dt_grid = s.local_dt[cell];
                    next_grid_time = s.time[cell] + dt_grid;  // collapse.time += dt, reproducer.cpp:7682
#pragma unroll
                    for (int k = 0; k < NS; ++k) y[k] = s.xn[k * n + cell];
                    y[NS] = s.e[cell];
                }
                // RODAS::integrate prologue, reproducer.cpp:7218-7235
                L.tout = dt_grid;
                L.x = 0.0;
                double h0 = dt_grid;
                if (::fabs(h0) <= 10.0 * kUround) h0 = 1.e-6;
                L.h = smin(::fabs(h0), dt_grid);
                L.reject = false;
                L.last = false;
                L.nsing = 0;
                L.hacc = 0.0;
                L.erracc = 1.0;
                L.hopt = L.h;
                L.n_step = 0;
                L.n_accept = 0;
                L.n_reject = 0;
                L.n_jac = 0;
                L.n_decomp = 0;
                L.fresh = true;
                have = true;
            }
            if (!L.fresh) break;
            // outer-loop checks, reproducer.cpp:7236-7255
            int code = 0;
            if (L.n_step > kMaxSteps) code = WR_TOO_MANY_STEPS;
            else if (0.1 * ::fabs(L.h) <= ::fabs(L.x) * kUround) code = WR_DT_UNDERFLOW;
            else if (L.last) code = WR_SUCCESS;
            if (code != 0) {
                // burn_ros2s epilogue: counters, then commit or failure
                const uint64_t st[7] = {
                    static_cast<uint64_t>(L.n_step), static_cast<uint64_t>(3 * L.n_step),
                    static_cast<uint64_t>(L.n_jac), static_cast<uint64_t>(L.n_decomp),
                    static_cast<uint64_t>(3 * L.n_step), static_cast<uint64_t>(L.n_accept),
                    static_cast<uint64_t>(L.n_reject)};
#pragma unroll
                for (int k = 0; k < 7; ++k) s.stats[k * n + cell] += st[k];
                s.cost[cell] = L.n_step;
                if (code == WR_SUCCESS) {
                    double xn[NS];
#pragma unroll
                    for (int k = 0; k < NS; ++k) xn[k] = y[k];
                    const double rho = s.rho[cell];
                    renormalize(xn, rho);
                    s.T[cell] = eos_T_from_e(xn, y[NS]);
                    s.e[cell] = y[NS];
#pragma unroll
                    for (int k = 0; k < NS; ++k) s.xn[k * n + cell] = xn[k];
                    s.time[cell] = next_grid_time;
                    s.steps[cell] = cgs + 1;
                    atomicAdd(&ctl[g].integrated, 1);
                } else {
                    record_failure(ctl + g, code);
                }
                have = false;
                continue;
            }
            L.hopt = L.h;
            if (L.x + L.h * 1.0001 >= L.tout) {
                L.h = L.tout - L.x;
                L.last = true;
            }
            break;
        }
        // ---- fresh outer iteration: Jacobian (fused with f(y))
        if (alive && have && L.fresh) {
            double X[NS], T;
            state_from_y(y, X, T);
            if constexpr (PREC == 0) {
                JSink<MT> sink{E, jb, nslots};
                wr_net_jac_rhs<M>(X, T, f0, sink);
            } else {
                JBackupSink sink{jb, nslots};
                wr_net_jac_rhs<M>(X, T, f0, sink);
            }
            L.n_jac += 1;
            L.fresh = false;
        } else if (PREC == 0 && alive && have) {
            // retry with the same Jacobian: rebuild E = -J
#pragma unroll
            for (int r = 0; r < NEQ; ++r)
#pragma unroll
                for (int c = 0; c < NEQ; ++c) E(r, c) = -jb[(r * NEQ + c) * nslots];
        }
        // ---- one attempt of the inner loop, reproducer.cpp:7259-7345
        if (alive && have) {
            const double h = L.h;
            const double fac = ddiv(1.0, h * kGamma);
            int info;
            if constexpr (PREC == 0) {
#pragma unroll
                for (int i = 0; i < NEQ; ++i) E(i, i) = E(i, i) + fac;
                info = lu_decompose(E, ip);
            } else {
                // error-weighted variables: the controller's own scale per component
#pragma unroll
                for (int i = 0; i < NEQ; ++i)
                    wsc[i] = (i < NS ? kAtolSpec : kAtolEnergy) + (i < NS ? kRtolSpec : kRtolEnergy) * ::fabs(y[i]);
#pragma unroll 1
                for (int r = 0; r < NEQ; ++r)
#pragma unroll
                    for (int c = 0; c < NEQ; ++c) {
                        double v = -jb[(r * NEQ + c) * nslots];
                        if (r == c) v = v + fac;
                        E32(r, c) = __double2float_rn(ddiv(v * wsc[c], wsc[r]));
                    }
                info = lu_decompose_f32(E32, ip);
            }
            if (info != 0) {
                L.nsing += 1;
                if (L.nsing >= 5) {
                    // fails like the outer checks: counters then the failure code
                    const uint64_t st[7] = {
                        static_cast<uint64_t>(L.n_step), static_cast<uint64_t>(3 * L.n_step),
                        static_cast<uint64_t>(L.n_jac), static_cast<uint64_t>(L.n_decomp),
                        static_cast<uint64_t>(3 * L.n_step), static_cast<uint64_t>(L.n_accept),
                        static_cast<uint64_t>(L.n_reject)};
#pragma unroll
                    for (int k = 0; k < 7; ++k) s.stats[k * n + cell] += st[k];
                    record_failure(ctl + g, WR_LU_DECOMPOSITION_ERROR);
                    have = false;
                } else {
                    L.h = h * 0.5;
                    L.reject = true;
                    L.last = false;
                }
            } else {
                L.n_decomp += 1;
                double ak1[NEQ], ak2[NEQ], w[NEQ];
#pragma unroll
                for (int i = 0; i < NEQ; ++i) ak1[i] = f0[i];
                if constexpr (PREC == 0) lu_solve(E, ip, ak1);
                else solve_refined(E32, ip, jb, nslots, fac, wsc, ak1);
                // stages 2 and 3 share one inlined RHS evaluation
#pragma unroll 1
                for (int stage = 2; stage <= 3; ++stage) {
                    double yn[NEQ];
                    if (stage == 2) {
#pragma unroll
                        for (int i = 0; i < NEQ; ++i) {
                            yn[i] = y[i] + kA21 * ak1[i];
                            w[i] = ddiv(kC21, h) * ak1[i];
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < NEQ; ++i) {
                            yn[i] = y[i] + kA31 * ak1[i] + kA32 * ak2[i];
                            w[i] = ddiv(kC31 * ak1[i] + kC32 * ak2[i], h);
                        }
                    }
                    double X[NS], T, dy[NEQ];
                    state_from_y(yn, X, T);
                    wr_net_rhs<M>(X, T, dy);
#pragma unroll
                    for (int i = 0; i < NEQ; ++i) w[i] += dy[i];
                    if constexpr (PREC == 0) lu_solve(E, ip, w);
                    else solve_refined(E32, ip, jb, nslots, fac, wsc, w);
                    if (stage == 2) {
#pragma unroll
                        for (int i = 0; i < NEQ; ++i) ak2[i] = w[i];
                    }
                }
                // w = k3; candidate and error estimate, reproducer.cpp:7299-7304
                double ynew[NEQ];
                double err = 0.0;
#pragma unroll
                for (int i = 0; i < NEQ; ++i) {
                    const double ak3 = w[i];
                    ynew[i] = y[i] + kB1 * ak1[i] + kB2 * ak2[i] + ak3;
                    const double wi = kE1 * ak1[i] + kE2 * ak2[i] + kE3 * ak3;
                    const double rtol = i < NS ? kRtolSpec : kRtolEnergy;
                    const double atol = i < NS ? kAtolSpec : kAtolEnergy;
                    const double sk = atol + rtol * smax(::fabs(y[i]), ::fabs(ynew[i]));
                    const double term = ddiv(wi, sk);
                    err += term * term;
                }
                err = ::sqrt(ddiv(err, 15.0));
                L.n_step += 1;
                // step-size controller, reproducer.cpp:7308-7344
                const double raw_fac = ddiv(M::cbrt(err), kSafe);
                const double fac_step = smax(1.0 / kFacMax, smin(1.0 / kFacMin, raw_fac));
                double hnew = ddiv(h, fac_step);
                if (err <= 1.0) {
                    L.n_accept += 1;
                    if (L.n_accept > 1) {
                        const double facgus = smax(1.0 / kFacMax,
                            smin(1.0 / kFacMin, ddiv(ddiv(L.hacc, h) * M::cbrt(ddiv(err * err, L.erracc)), kSafe)));
                        hnew = ddiv(h, smax(fac_step, facgus));
                    }
                    L.hacc = h;
                    L.erracc = smax(1.e-2, err);
#pragma unroll
                    for (int i = 0; i < NEQ; ++i) y[i] = ynew[i];
                    L.x += h;
                    const double hmaxn = L.tout;  // tout - t with t = 0
                    if (::fabs(hnew) > hmaxn) hnew = hmaxn;
                    if (L.reject) hnew = smin(::fabs(hnew), ::fabs(h));
                    L.reject = false;
                    L.h = hnew;
                    L.fresh = true;
                } else {
                    L.reject = true;
                    L.last = false;
                    L.h = hnew;
                    if (L.n_accept >= 1) L.n_reject += 1;
                    if (hnew == 0.0) {
                        // The step size has underflowed inside the reject loop, which
                        // has no exit of its own (reproducer.cpp:7259-7345 leaves it
                        // only on an accepted attempt): with a NaN error norm (the
                        // network is undefined below ~100 K) it would retry forever.
                        // A zero step is the reference's DT_UNDERFLOW (:7240), so the
                        // cell ends with that code here instead of never ending.
                        const uint64_t st[7] = {
                            static_cast<uint64_t>(L.n_step), static_cast<uint64_t>(3 * L.n_step),
                            static_cast<uint64_t>(L.n_jac), static_cast<uint64_t>(L.n_decomp),
                            static_cast<uint64_t>(3 * L.n_step), static_cast<uint64_t>(L.n_accept),
                            static_cast<uint64_t>(L.n_reject)};
#pragma unroll
                        for (int k = 0; k < 7; ++k) s.stats[k * n + cell] += st[k];
                        record_failure(ctl + g, WR_DT_UNDERFLOW);
                        have = false;
                    }
                }
            }
        }
    }

}

}  // namespace wr
