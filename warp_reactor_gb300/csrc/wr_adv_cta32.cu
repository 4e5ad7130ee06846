// wr_adv_cta32.cu -- advance kernel of the gridwide-structured-cta32 policy.
//
// The reference's other GPU policy (advance_collapse_gridwide_structured_kernel,
// structured_cuda.cuh:393-782; selected by PRIMORDIAL_ROS2S_CUDA_STRUCTURED,
// reproducer.cpp:7845-7916): the grid is cut into tiles of 32 consecutive cells and
// each tile advances its participating cells with ONE ROS2S controller -- a common
// step h, the tile error = maximum over its participating cells of their error
// norms (a non-finite norm counts as DBL_MAX), the Jacobian kept across rejected
// trials, the common final-step truncation and the commit of every participating
// cell on success.  The prepare kernel and the grid minimum are the
// gridwide-independent ones.
//
// GB300 mapping: one warp per tile, one lane per cell.  The controller is
// warp-uniform, so a warp never diverges on accept/reject; the tile maximum is a
// shuffle reduction (fmax is exact and order-free on non-NaN values).  Per-cell
// Jacobian and iteration matrix live in global arrays [225][n] (coalesced across a
// warp's consecutive cells).  Arithmetic is the independent kernel's, operation for
// operation, plus the structured controller's rules.
#include "wr_launch.h"

namespace wr {

namespace {

constexpr int kTileCells = 32;
constexpr int kCtaThreads = 256;  // eight tiles per block

template <class M>
__device__ __forceinline__ double cbrt_nonnegative(double v) {  // structured_cuda.cuh:88-93
    if (v == 0.0) return 0.0;
    return M::exp(ddiv(M::log(v), 3.0));
}

template <class M>
__global__ void __launch_bounds__(kCtaThreads, 1) k_advance_cta32(DevState s, StepCtl* ctl, double* jall,
                                                                   double* eall) {
    const int lane = threadIdx.x & 31;
    const int tile = blockIdx.x * (kCtaThreads / 32) + (threadIdx.x >> 5);
    const int n = s.n;
    const int tile_begin = tile * kTileCells;
    if (tile_begin >= n) return;  // whole warp
    StepCtl* c = ctl;
    if (c->stop) return;  // set by k_decide before this launch: uniform over the grid
    const int cell = tile_begin + lane;
    const bool active = cell < n;
    const int cgs = c->cgs;
    const double grid_time = c->grid_time;
    const double dt_grid = c->dt_grid;
    const double next_grid_time = c->next_grid_time;

    // ---- per-cell prologue, structured_cuda.cuh:410-450
    bool part = false;
    double base[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) base[i] = 0.0;
    if (active && s.steps[cell] == cgs) {
        if (s.time[cell] != grid_time) {
            record_failure(c, WR_BAD_INPUTS);
        } else {
            double xn[NS];
#pragma unroll
            for (int k = 0; k < NS; ++k) xn[k] = s.xn[k * n + cell];
            const double local_dt = collapse_timestep(xn);
            if (local_dt >= 10.0) {
                const double old_density = s.driver[cell];
                const double driver = old_density + ddiv(dt_grid * old_density, ddiv(local_dt, kTffReduc));
                s.driver[cell] = driver;
                if (valid_positive(driver) && driver <= kDriverLimit) {
                    const double ratio = ddiv(driver, old_density);
#pragma unroll
                    for (int k = 0; k < NS; ++k) xn[k] *= ratio;
                    const double rho = s.rho[cell] * ratio;
                    const double e = eos_e_from_T(xn, s.T[cell]);
                    s.rho[cell] = rho;
                    s.e[cell] = e;
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        s.xn[k * n + cell] = xn[k];
                        base[k] = xn[k];
                    }
                    base[NS] = e;
                    part = true;
                }
            }
        }
    }
    const unsigned int pmask = __ballot_sync(0xffffffffu, part);
    const int count = __popc(pmask);
    if (count == 0) return;

    // ---- the tile's controller, structured_cuda.cuh:468-733
    double h = dt_grid, x = 0.0, hacc = 0.0, erracc = 1.0;
    bool reject = false, jac_valid = false;
    int nsing = 0, n_step = 0, n_accept = 0, n_jac = 0, n_rej = 0;
    int status = WR_SUCCESS;
    double f0[NEQ];
    MatG E{eall + cell, n};
    double* jb = jall + cell;
    while (true) {
        if (x >= dt_grid || status != WR_SUCCESS) break;
        if (n_step > kMaxSteps) {
            status = WR_TOO_MANY_STEPS;
            continue;
        }
        if (0.1 * ::fabs(h) <= ::fabs(x) * kUround) {
            status = WR_DT_UNDERFLOW;
            continue;
        }
        bool final_trial = false;
        if (x + h * 1.0001 >= dt_grid) {
            h = dt_grid - x;
            final_trial = true;
        }
        bool singular = false;
        double err = 0.0;
        double cand[NEQ];
        if (part) {
            if (!jac_valid) {
                double X[NS], T;
                state_from_y(base, X, T);
                JBackupSink sink{jb, n};
                wr_net_jac_rhs<M>(X, T, f0, sink);
            }
            const double fac = ddiv(1.0, h * kGamma);
#pragma unroll 1
            for (int r = 0; r < NEQ; ++r)
#pragma unroll 1
                for (int q = 0; q < NEQ; ++q) E(r, q) = -jb[(r * NEQ + q) * n];
#pragma unroll 1
            for (int i = 0; i < NEQ; ++i) E(i, i) = E(i, i) + fac;
            uint64_t ip = 0;
            if (lu_decompose(E, ip) != 0) {
                singular = true;
            } else {
                double ak1[NEQ], ak2[NEQ], w[NEQ];
#pragma unroll
                for (int i = 0; i < NEQ; ++i) ak1[i] = f0[i];
                lu_solve(E, ip, ak1);
#pragma unroll 1
                for (int stage = 2; stage <= 3; ++stage) {
                    double yn[NEQ];
                    if (stage == 2) {
#pragma unroll
                        for (int i = 0; i < NEQ; ++i) {
                            yn[i] = base[i] + kA21 * ak1[i];
                            w[i] = ddiv(kC21, h) * ak1[i];
                        }
                    } else {
#pragma unroll
                        for (int i = 0; i < NEQ; ++i) {
                            yn[i] = base[i] + kA31 * ak1[i] + kA32 * ak2[i];
                            w[i] = ddiv(kC31 * ak1[i] + kC32 * ak2[i], h);
                        }
                    }
                    double X[NS], T, dy[NEQ];
                    state_from_y(yn, X, T);
                    wr_net_rhs<M>(X, T, dy);
#pragma unroll
                    for (int i = 0; i < NEQ; ++i) w[i] += dy[i];
                    lu_solve(E, ip, w);
                    if (stage == 2) {
#pragma unroll
                        for (int i = 0; i < NEQ; ++i) ak2[i] = w[i];
                    }
                }
                double sum = 0.0;
#pragma unroll
                for (int i = 0; i < NEQ; ++i) {
                    const double ak3 = w[i];
                    cand[i] = base[i] + kB1 * ak1[i] + kB2 * ak2[i] + ak3;
                    const double est = kE1 * ak1[i] + kE2 * ak2[i] + kE3 * ak3;
                    const double rtol = i < NS ? kRtolSpec : kRtolEnergy;
                    const double atol = i < NS ? kAtolSpec : kAtolEnergy;
                    const double scale = atol + rtol * ::fmax(::fabs(base[i]), ::fabs(cand[i]));
                    const double term = ddiv(est, scale);
                    sum += term * term;
                }
                err = ::sqrt(ddiv(sum, 15.0));
            }
        }
        if (!jac_valid) n_jac += 1;
        jac_valid = true;
        if (__any_sync(0xffffffffu, singular)) {
            ++nsing;
            if (nsing >= 5) {
                status = WR_LU_DECOMPOSITION_ERROR;
            } else {
                h = h * 0.5;
                reject = true;
            }
            continue;
        }
        double ev = part ? (isfinite(err) ? err : DBL_MAX) : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) ev = ::fmax(ev, __shfl_xor_sync(0xffffffffu, ev, off));
        const double err_tile = ev;
        ++n_step;
        const double fac_step = ::fmax(1.0 / kFacMax, ::fmin(1.0 / kFacMin, ddiv(cbrt_nonnegative<M>(err_tile), kSafe)));
        double hnew = ddiv(h, fac_step);
        if (err_tile <= 1.0) {
            ++n_accept;
            if (n_accept > 1) {
                const double facgus = ::fmax(1.0 / kFacMax,
                    ::fmin(1.0 / kFacMin,
                           ddiv(ddiv(hacc, h) * cbrt_nonnegative<M>(ddiv(err_tile * err_tile, erracc)), kSafe)));
                hnew = ddiv(h, ::fmax(fac_step, facgus));
            }
            if (part) {
#pragma unroll
                for (int i = 0; i < NEQ; ++i) base[i] = cand[i];
            }
            hacc = h;
            erracc = ::fmax(1.0e-2, err_tile);
            x = final_trial ? dt_grid : x + h;
            hnew = ::fmin(::fabs(hnew), dt_grid);
            if (reject) hnew = ::fmin(hnew, ::fabs(h));
            reject = false;
            h = hnew;
            jac_valid = false;
        } else {
            if (n_accept >= 1) ++n_rej;
            reject = true;
            h = hnew;
        }
    }

    // ---- commit, structured_cuda.cuh:737-778
    if (status != WR_SUCCESS) {
        if (lane == 0) record_failure(c, status);
        return;
    }
    if (part) {
        double xn[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) xn[k] = base[k];
        renormalize(xn, s.rho[cell]);
        s.T[cell] = eos_T_from_e(xn, base[NS]);
        s.e[cell] = base[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) s.xn[k * n + cell] = xn[k];
        s.time[cell] = next_grid_time;
        s.steps[cell] = cgs + 1;
        const uint64_t st[7] = {static_cast<uint64_t>(n_step), static_cast<uint64_t>(3 * n_step),
                                static_cast<uint64_t>(n_jac), static_cast<uint64_t>(n_step),
                                static_cast<uint64_t>(3 * n_step), static_cast<uint64_t>(n_accept),
                                static_cast<uint64_t>(n_rej)};
#pragma unroll
        for (int k = 0; k < 7; ++k) s.stats[k * n + cell] += st[k];
    }
    if (lane == 0) atomicAdd(&c->integrated, count);
}

}  // namespace

cudaError_t launch_advance_cta32(int math_cuda, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                 double* jall, double* eall) {
    if (math_cuda)
        k_advance_cta32<CudaMath><<<blocks, kCtaThreads, 0, stream>>>(s, ctl, jall, eall);
    else
        k_advance_cta32<PortableMathCall><<<blocks, kCtaThreads, 0, stream>>>(s, ctl, jall, eall);
    return cudaGetLastError();
}

int cta32_blocks(int n) {
    const int tiles = (n + kTileCells - 1) / kTileCells;
    const int per_block = kCtaThreads / 32;
    return (tiles + per_block - 1) / per_block;
}

}  // namespace wr
