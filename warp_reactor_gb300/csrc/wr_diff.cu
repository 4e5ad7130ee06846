// wr_diff.cu -- differentiation form: forward kernel and C ABI (the map and its
// storage are described in wr_diff.cuh).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "wr_diff.cuh"

namespace wr {
namespace diff {

// ---------------------------------------------------------------- forward pieces
// ---------------------------------------------------------------- forward pieces
// One ROS2S attempt (reproducer.cpp:7259-7304) from y with step h and iteration
// matrix already factorised in E/ip; writes ynew and the error vector.
__device__ void ros2s_stages(const double* y, double h, MatL E, uint64_t ip, const double* mult,
                                             double* ak1, double* ak2, double* ak3, double* ynew, double* work) {
    double X[NS], T, dy[NEQ];
    state_from_y(y, X, T);
    net_rhs(X, T, mult, ak1);
    lu_solve(E, ip, ak1);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        ynew[i] = y[i] + kA21 * ak1[i];
        ak2[i] = ddiv(kC21, h) * ak1[i];
    }
    state_from_y(ynew, X, T);
    net_rhs(X, T, mult, dy);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) ak2[i] += dy[i];
    lu_solve(E, ip, ak2);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        ynew[i] = y[i] + kA31 * ak1[i] + kA32 * ak2[i];
        ak3[i] = ddiv(kC31 * ak1[i] + kC32 * ak2[i], h);
    }
    state_from_y(ynew, X, T);
    net_rhs(X, T, mult, dy);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) ak3[i] += dy[i];
    lu_solve(E, ip, ak3);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        ynew[i] = y[i] + kB1 * ak1[i] + kB2 * ak2[i] + ak3[i];
        work[i] = kE1 * ak1[i] + kE2 * ak2[i] + kE3 * ak3[i];
    }
}

__device__ int factor(const double* J, double h, MatL E, uint64_t& ip) {
    const double fac = ddiv(1.0, h * kGamma);
#pragma unroll 1
    for (int r = 0; r < NEQ; ++r)
#pragma unroll 1
        for (int c = 0; c < NEQ; ++c) E(r, c) = -J[r * NEQ + c];
#pragma unroll 1
    for (int i = 0; i < NEQ; ++i) E(i, i) = E(i, i) + fac;
    return lu_decompose(E, ip);
}

// RODAS::integrate with the configure_ros2s settings (:7205-7347, :7582-7590),
// appending accepted step sizes to h_out (at most cap_left).  Returns the
// IntegratorResult; *count = accepted steps.
static __device__ __noinline__ int burn_record(double* y, double tout, const double* mult, double* h_out, int cap_left, int* count) {
    double Jm[NEQ * NEQ], Em[NEQ * NEQ];
    MatL E{Em};
    uint64_t ip = 0;
    double ak1[NEQ], ak2[NEQ], ak3[NEQ], ynew[NEQ], work[NEQ];
    const double hmaxn = tout;
    double h = tout;
    if (::fabs(h) <= 10.0 * kUround) h = 1.e-6;
    h = smin(::fabs(h), hmaxn);
    bool reject = false, last = false;
    int nsing = 0, n_step = 0, n_accept = 0;
    double hacc = 0.0, erracc = 1.0, x = 0.0;
    *count = 0;
    for (;;) {
        if (n_step > kMaxSteps) return WR_TOO_MANY_STEPS;
        if (0.1 * ::fabs(h) <= ::fabs(x) * kUround) return WR_DT_UNDERFLOW;
        if (last) return WR_SUCCESS;
        if (x + h * 1.0001 >= tout) {
            h = tout - x;
            last = true;
        }
        {
            double X[NS], T;
            state_from_y(y, X, T);
            net_jac(X, T, Jm);
        }
        for (;;) {
            if (factor(Jm, h, E, ip) != 0) {
                nsing += 1;
                if (nsing >= 5) return WR_LU_DECOMPOSITION_ERROR;
                h = h * 0.5;
                reject = true;
                last = false;
                continue;
            }
            ros2s_stages(y, h, E, ip, mult, ak1, ak2, ak3, ynew, work);
            n_step += 1;
            double err = 0.0;
#pragma unroll
            for (int i = 0; i < NEQ; ++i) {
                const double rtol = i < NS ? kRtolSpec : kRtolEnergy;
                const double atol = i < NS ? kAtolSpec : kAtolEnergy;
                const double sk = atol + rtol * smax(::fabs(y[i]), ::fabs(ynew[i]));
                const double term = ddiv(work[i], sk);
                err += term * term;
            }
            err = ::sqrt(ddiv(err, 15.0));
            const double raw_fac = ddiv(M::cbrt(err), kSafe);
            const double fac_step = smax(1.0 / kFacMax, smin(1.0 / kFacMin, raw_fac));
            double hnew = ddiv(h, fac_step);
            if (err <= 1.0) {
                n_accept += 1;
                if (n_accept > 1) {
                    const double facgus = smax(1.0 / kFacMax,
                        smin(1.0 / kFacMin, ddiv(ddiv(hacc, h) * M::cbrt(ddiv(err * err, erracc)), kSafe)));
                    hnew = ddiv(h, smax(fac_step, facgus));
                }
                hacc = h;
                erracc = smax(1.e-2, err);
                if (*count >= cap_left) return WR_TOO_MANY_STEPS;
                h_out[*count] = h;
                *count += 1;
#pragma unroll
                for (int i = 0; i < NEQ; ++i) y[i] = ynew[i];
                x += h;
                if (::fabs(hnew) > hmaxn) hnew = hmaxn;
                if (reject) hnew = smin(::fabs(hnew), ::fabs(h));
                reject = false;
                h = hnew;
                break;
            }
            reject = true;
            last = false;
            h = hnew;
            if (hnew == 0.0) return WR_DT_UNDERFLOW;  // the reject loop's only other exit
        }
    }
}

// one accepted step of the frozen controller
__device__ void step_replay(double* y, double h, const double* mult, double* st) {
    double Jm[NEQ * NEQ], Em[NEQ * NEQ];
    MatL E{Em};
    uint64_t ip = 0;
    double ak1[NEQ], ak2[NEQ], ak3[NEQ], ynew[NEQ], work[NEQ];
    double X[NS], T;
    state_from_y(y, X, T);
    net_jac(X, T, Jm);
    factor(Jm, h, E, ip);
    ros2s_stages(y, h, E, ip, mult, ak1, ak2, ak3, ynew, work);
    if (st != nullptr) {
        // what the step's adjoint needs: the factorised matrix, pivots, stage vectors
#pragma unroll 1
        for (int k = 0; k < NEQ * NEQ; ++k) st[k] = Em[k];
        st[kStageIp] = __longlong_as_double(static_cast<long long>(ip));
#pragma unroll
        for (int i = 0; i < NEQ; ++i) {
            st[kStageK1 + i] = ak1[i];
            st[kStageK2 + i] = ak2[i];
            st[kStageK3 + i] = ak3[i];
        }
    }
#pragma unroll
    for (int i = 0; i < NEQ; ++i) y[i] = ynew[i];
}

__global__ void __launch_bounds__(kThreads) k_diff_forward(Args a) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.n) return;
    CellS c;
    {
        const wr_collapse_state& st = a.cells[i];
#pragma unroll
        for (int k = 0; k < NS; ++k) c.xn[k] = a.u ? a.u[15 * i + k] : st.xn[k];
        c.T = a.u ? a.u[15 * i + NS] : st.T;
        c.e = st.e;
        c.rho = st.rho;
        c.driver = st.density_driver;
    }
    double* hrow = a.hbuf + static_cast<size_t>(i) * a.cap;
    int used = 0;
    int status = WR_SUCCESS;
    bool live = true;
    for (int s = 0; s < a.nsteps; ++s) {
        unsigned char kind = 0;
        int cnt = 0;
        if (live) {
            save_ckpt(a, s, i, c);
            double dt;
            int k = prepare_part(a, s, i, c, dt);
            if (k == 3) {
                double y[NEQ];
                k = advance_part(a.dt_hist[s], dt, c, y);
                if (k == 3) {
                    const int r = burn_record(y, a.dt_hist[s], a.mult, hrow + used, a.cap - used, &cnt);
                    if (r != WR_SUCCESS) {
                        status = r;
                        live = false;
                    } else {
                        commit_part(c, y);
                        used += cnt;
                    }
                }
            }
            if (k < 0) {
                status = WR_BAD_INPUTS;
                live = false;
            } else {
                kind = static_cast<unsigned char>(k);
                if (k != 3) live = false;
            }
        }
        a.kind[static_cast<size_t>(s) * a.n + i] = kind;
        a.counts[static_cast<size_t>(s) * a.n + i] = cnt;
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) a.q[15 * i + k] = c.xn[k];
    a.q[15 * i + NS] = c.T;
    a.status[i] = status;
}

__global__ void k_diff_mult(const double* logm, double* mult) {
    const int r = threadIdx.x;
    if (r < NP) mult[r] = logm ? M::exp(logm[r]) : 1.0;
}

// pbar[r] = mult[r] * sum over cells (in cell order) of mbar[cell][r]
__global__ void k_diff_reduce(const double* mbar, const double* mult, int n, double* pbar) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= NP) return;
    double acc = 0.0;
    for (int i = 0; i < n; ++i) acc += mbar[static_cast<size_t>(i) * NP + r];
    pbar[r] = acc * mult[r];
}

}  // namespace diff
}  // namespace wr

// ------------------------------------------------------------------ C-ABI
struct wr_diff {
    int n = 0, max_steps = 0, cap = 0, nseg = 0, device = 0;
    int nsteps = 0, perturb = 0;
    bool have_forward = false;
    cudaStream_t stream = nullptr;
    double* ckpt = nullptr;
    int* counts = nullptr;
    unsigned char* kind = nullptr;
    double* hbuf = nullptr;
    double* segck = nullptr;
    double* ys = nullptr;
    double* stage = nullptr;
    double* mbar = nullptr;
    double* mult = nullptr;
    double* dt_hist = nullptr;
    int* status = nullptr;
    const wr_collapse_state* cells = nullptr;  // the caller's records of the last forward
    const double* u = nullptr;
    std::string error;
};

namespace {

int fail(wr_diff* d, const std::string& msg, int code = WR_BAD_INPUTS) {
    if (d) d->error = msg;
    return code;
}

bool cuda_ok(wr_diff* d, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    if (d) d->error = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

wr::diff::Args make_args(wr_diff* d) {
    wr::diff::Args a{};
    a.cells = d->cells;
    a.u = d->u;
    a.mult = d->mult;
    a.dt_hist = d->dt_hist;
    a.nsteps = d->nsteps;
    a.perturb = d->perturb;
    a.n = d->n;
    a.cap = d->cap;
    a.nseg = d->nseg;
    a.ckpt = d->ckpt;
    a.counts = d->counts;
    a.kind = d->kind;
    a.hbuf = d->hbuf;
    a.segck = d->segck;
    a.ys = d->ys;
    a.stage = d->stage;
    a.mbar = d->mbar;
    a.status = d->status;
    return a;
}

}  // namespace

extern "C" {

int wr_diff_num_multipliers(void) { return wr::diff::NP; }

wr_diff* wr_diff_create(int num_cells, int max_outer_steps, int max_accepted_per_cell, int device) {
    if (num_cells <= 0 || max_outer_steps <= 0 || max_accepted_per_cell <= 0) return nullptr;
    wr_diff* d = new wr_diff();
    d->n = num_cells;
    d->max_steps = max_outer_steps;
    d->cap = max_accepted_per_cell;
    d->nseg = (max_accepted_per_cell + wr::diff::kSeg - 1) / wr::diff::kSeg + 1;
    d->device = device;
    const size_t n = static_cast<size_t>(num_cells);
    const size_t S = static_cast<size_t>(max_outer_steps);
    bool ok = cuda_ok(d, cudaSetDevice(device), "cudaSetDevice") &&
              cuda_ok(d, cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking), "cudaStreamCreate") &&
              cuda_ok(d, cudaMalloc(&d->ckpt, S * wr::diff::kFields * n * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->counts, S * n * sizeof(int)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->kind, S * n), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->hbuf, n * d->cap * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->segck, n * d->nseg * wr::NEQ * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->ys, n * wr::diff::kSeg * wr::NEQ * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->stage, n * wr::diff::kSeg * wr::diff::kStage * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->mbar, n * wr::diff::NP * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->mult, wr::diff::NP * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->dt_hist, S * sizeof(double)), "cudaMalloc") &&
              cuda_ok(d, cudaMalloc(&d->status, n * sizeof(int)), "cudaMalloc");
    if (!ok) {
        fprintf(stderr, "wr_diff_create: %s\n", d->error.c_str());
        wr_diff_destroy(d);
        return nullptr;
    }
    return d;
}

void wr_diff_destroy(wr_diff* d) {
    if (!d) return;
    cudaFree(d->ckpt);
    cudaFree(d->counts);
    cudaFree(d->kind);
    cudaFree(d->hbuf);
    cudaFree(d->segck);
    cudaFree(d->ys);
    cudaFree(d->stage);
    cudaFree(d->mbar);
    cudaFree(d->mult);
    cudaFree(d->dt_hist);
    cudaFree(d->status);
    if (d->stream) cudaStreamDestroy(d->stream);
    delete d;
}

const char* wr_diff_last_error(wr_diff* d) { return d ? d->error.c_str() : "null context"; }

int wr_diff_forward(wr_diff* d, const wr_collapse_state* d_cells, const double* d_u, const double* d_log_mult,
                    const double* dt_hist, int nsteps, int perturb, double* d_q) {
    if (!d) return WR_BAD_INPUTS;
    if (!d_cells || !dt_hist || !d_q) return fail(d, "null pointer argument");
    if (nsteps <= 0 || nsteps > d->max_steps) return fail(d, "nsteps outside 1..max_outer_steps");
    for (int s = 0; s < nsteps; ++s)
        if (!(dt_hist[s] > 0.0) || !std::isfinite(dt_hist[s])) return fail(d, "dt_hist holds a non-positive step");
    if (!cuda_ok(d, cudaSetDevice(d->device), "cudaSetDevice")) return WR_BAD_INPUTS;
    d->cells = d_cells;
    d->u = d_u;
    d->nsteps = nsteps;
    d->perturb = perturb ? 1 : 0;
    d->have_forward = false;
    if (!cuda_ok(d, cudaMemcpyAsync(d->dt_hist, dt_hist, nsteps * sizeof(double), cudaMemcpyHostToDevice,
                                    d->stream), "cudaMemcpyAsync"))
        return WR_BAD_INPUTS;
    wr::diff::k_diff_mult<<<1, 64, 0, d->stream>>>(d_log_mult, d->mult);
    wr::diff::Args a = make_args(d);
    a.q = d_q;
    const int blocks = (d->n + wr::diff::kThreads - 1) / wr::diff::kThreads;
    wr::diff::k_diff_forward<<<blocks, wr::diff::kThreads, 0, d->stream>>>(a);
    if (!cuda_ok(d, cudaGetLastError(), "k_diff_forward launch")) return WR_BAD_INPUTS;
    if (!cuda_ok(d, cudaStreamSynchronize(d->stream), "k_diff_forward")) return WR_BAD_INPUTS;
    // first failing cell in index order decides the result
    int* st = new int[d->n];
    const bool got = cuda_ok(d, cudaMemcpy(st, d->status, d->n * sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy");
    int result = got ? WR_SUCCESS : WR_BAD_INPUTS;
    for (int i = 0; got && i < d->n; ++i)
        if (st[i] != WR_SUCCESS) {
            result = st[i];
            d->error = "cell " + std::to_string(i) + " failed with code " + std::to_string(st[i]);
            break;
        }
    delete[] st;
    d->have_forward = result == WR_SUCCESS;
    return result;
}

int wr_diff_backward(wr_diff* d, const double* d_qbar, double* d_ubar, double* d_pbar) {
    if (!d) return WR_BAD_INPUTS;
    if (!d->have_forward) return fail(d, "wr_diff_backward needs a successful wr_diff_forward first");
    if (!d_qbar || !d_ubar || !d_pbar) return fail(d, "null pointer argument");
    if (!cuda_ok(d, cudaSetDevice(d->device), "cudaSetDevice")) return WR_BAD_INPUTS;
    wr::diff::Args a = make_args(d);
    a.qbar = d_qbar;
    a.ubar = d_ubar;
    const int blocks = (d->n + wr::diff::kThreads - 1) / wr::diff::kThreads;
    wr::diff::k_diff_backward<<<blocks, wr::diff::kThreads, 0, d->stream>>>(a);
    if (!cuda_ok(d, cudaGetLastError(), "k_diff_backward launch")) return WR_BAD_INPUTS;
    wr::diff::k_diff_reduce<<<1, 64, 0, d->stream>>>(d->mbar, d->mult, d->n, d_pbar);
    if (!cuda_ok(d, cudaStreamSynchronize(d->stream), "k_diff_backward")) return WR_BAD_INPUTS;
    return WR_SUCCESS;
}

int wr_diff_record(wr_diff* d, double* h_hbuf, int* h_counts) {
    if (!d || !d->have_forward || !h_hbuf || !h_counts) return WR_BAD_INPUTS;
    const size_t n = static_cast<size_t>(d->n);
    if (!cuda_ok(d, cudaMemcpy(h_hbuf, d->hbuf, n * d->cap * sizeof(double), cudaMemcpyDeviceToHost), "cudaMemcpy"))
        return WR_BAD_INPUTS;
    // counts are stored [S][n]; the host copy is [n][S]
    int* tmp = new int[static_cast<size_t>(d->nsteps) * n];
    const bool ok = cuda_ok(d, cudaMemcpy(tmp, d->counts, static_cast<size_t>(d->nsteps) * n * sizeof(int),
                                          cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (ok)
        for (size_t i = 0; i < n; ++i)
            for (int s = 0; s < d->nsteps; ++s) h_counts[i * d->nsteps + s] = tmp[static_cast<size_t>(s) * n + i];
    delete[] tmp;
    return ok ? WR_SUCCESS : WR_BAD_INPUTS;
}

}  // extern "C"

