// wr_capi.cu -- the C ABI of include/warp_reactor.h and the small kernels.
//
// Host-side lifecycle of run_cells_cuda (reproducer.cpp:7791-7975), restructured
// for one GPU: device state is structure-of-arrays, the grid minimum is taken on
// the device, and a whole outer step (prepare -> decide -> advance -> finalize)
// is four launches with no host round trip.  wr_run checks the device's stop flag
// every kCheckEvery steps with one 64-byte copy instead of the reference's two
// synchronisations and a 2 MiB copy per step.
#include <cuda_runtime.h>

#include <atomic>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/warp_reactor.h"
#include "wr_launch.h"

using namespace wr;

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};

int fail(const char* what, cudaError_t e) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return WR_BAD_INPUTS;
}

int fail_msg(const std::string& msg) {
    g_last_error = msg;
    return WR_BAD_INPUTS;
}

constexpr int kCheckEvery = 16;

}  // namespace

struct wr_ctx {
    int n = 0;
    int device = 0;
    int math = WR_MATH_PORTABLE;
    int advance_blocks = 0;
    int sms = 1;
    int variant = 2;  // fastest measured shape (256 lanes per SM, matrices in global memory)
    cudaStream_t stream = nullptr;
    DevState s{};
    void* state_buf = nullptr;
    StepCtl* ctl = nullptr;
    StepCtl* host_ctl = nullptr;  // pinned mirror
    double* jbackup = nullptr;
    double* ebuf = nullptr;    // per-lane iteration matrices for the global-matrix variants
    double* dt_hist = nullptr;  // grid dt of every outer step of the last wr_run
    wr_collapse_state* staging = nullptr;  // device AoS records for upload/download
    // optional per-kernel timing of wr_run (CUDA events on the context stream)
    bool profiling = false;
    cudaEvent_t ev[4 * WR_MAX_COLLAPSE_STEPS + 2] = {};
    int ev_used = 0;
    wr_run_timing timing{};
};

namespace wr {

__global__ void k_unpack(const wr_collapse_state* __restrict__ in, DevState s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const wr_collapse_state c = in[i];
    const int n = s.n;
    s.rho[i] = c.rho;
    s.T[i] = c.T;
    s.e[i] = c.e;
#pragma unroll
    for (int k = 0; k < NS; ++k) s.xn[k * n + i] = c.xn[k];
    s.time[i] = c.time;
    s.driver[i] = c.density_driver;
    s.steps[i] = c.completed_steps;
    const uint64_t st[7] = {c.stats.internal_steps, c.stats.rhs_calls, c.stats.jacobian_calls,
                            c.stats.decompositions, c.stats.linear_solves, c.stats.accepted_steps,
                            c.stats.rejected_steps};
#pragma unroll
    for (int k = 0; k < 7; ++k) s.stats[k * n + i] = st[k];
}

__global__ void k_pack(DevState s, wr_collapse_state* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const int n = s.n;
    wr_collapse_state c;
    c.rho = s.rho[i];
    c.T = s.T[i];
    c.e = s.e[i];
#pragma unroll
    for (int k = 0; k < NS; ++k) c.xn[k] = s.xn[k * n + i];
    c.time = s.time[i];
    c.density_driver = s.driver[i];
    c.completed_steps = s.steps[i];
    c.reserved_ = 0;
    c.stats.internal_steps = s.stats[0 * n + i];
    c.stats.rhs_calls = s.stats[1 * n + i];
    c.stats.jacobian_calls = s.stats[2 * n + i];
    c.stats.decompositions = s.stats[3 * n + i];
    c.stats.linear_solves = s.stats[4 * n + i];
    c.stats.accepted_steps = s.stats[5 * n + i];
    c.stats.rejected_steps = s.stats[6 * n + i];
    out[i] = c;
}

// scatter the queued cells (those whose completed steps equal the grid's) into
// the bucket order
__global__ void k_order(DevState s, StepCtl* ctl) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= s.n || ctl->stop) return;
    if (s.steps[cell] != ctl->cgs) return;
    const unsigned int pos = atomicAdd(&ctl->off[cost_bucket(s.cost[cell])], 1u);
    if (pos < static_cast<unsigned int>(s.n)) s.order[pos] = cell;
}

// start of an outer step driven by the host (wr_prepare)
__global__ void k_begin_step(StepCtl* ctl, int cgs, double grid_time, int step, int perturb) {
    for (int b = 0; b < kBuckets; ++b) ctl->hist[b] = 0;
    ctl->cgs = cgs;
    ctl->grid_time = grid_time;
    ctl->step = step;
    ctl->perturb = perturb;
    ctl->dmin_bits = kDblMaxBits;
    ctl->stop = 0;
}

// advance arguments driven by the host (wr_advance)
__global__ void k_begin_advance(StepCtl* ctl, int cgs, double next_grid_time, double dt_grid) {
    ctl->cgs = cgs;
    ctl->next_grid_time = next_grid_time;
    ctl->dt_grid = dt_grid;
    ctl->integrated = 0;
    ctl->stop = 0;
    build_queue_offsets(ctl);
}

// host checks between prepare and advance, reproducer.cpp:7880-7909
__global__ void k_decide(StepCtl* ctl, double* dt_hist) {
    if (ctl->stop) return;
    if (ctl->failure != WR_SUCCESS) {
        ctl->stop = 1;
        return;
    }
    if (ctl->dmin_bits == kDblMaxBits) {  // no candidate: the loop ends successfully
        ctl->stop = 1;
        return;
    }
    const double dt = __longlong_as_double(static_cast<long long>(ctl->dmin_bits));
    const double next = ctl->grid_time + dt;
    if (!valid_positive(dt) || !isfinite(next)) {
        ctl->failure = WR_BAD_INPUTS;
        ctl->stop = 1;
        return;
    }
    ctl->dt_grid = dt;
    ctl->next_grid_time = next;
    ctl->integrated = 0;
    build_queue_offsets(ctl);
    if (ctl->step >= 0 && ctl->step < WR_MAX_COLLAPSE_STEPS) dt_hist[ctl->step] = dt;
}

// host bookkeeping after the advance, reproducer.cpp:7930-7958
__global__ void k_finalize(StepCtl* ctl, int max_steps) {
    if (ctl->stop) return;
    if (ctl->failure != WR_SUCCESS || ctl->integrated == 0) {
        ctl->stop = 1;
        return;
    }
    ctl->grid_time = ctl->next_grid_time;
    ctl->cgs += 1;
    ctl->step += 1;
    ctl->dmin_bits = kDblMaxBits;
    if (ctl->step >= max_steps) ctl->stop = 1;
}

}  // namespace wr

namespace {

int set_device(wr_ctx* ctx) {
    const cudaError_t e = cudaSetDevice(ctx->device);
    return e == cudaSuccess ? WR_SUCCESS : fail("cudaSetDevice", e);
}

void record(wr_ctx* ctx, int idx) {
    if (ctx->profiling) cudaEventRecord(ctx->ev[idx], ctx->stream);
}

cudaError_t launch_advance(wr_ctx* ctx) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const int blocks = ctx->sms * kAdvanceShapes[ctx->variant].blocks_per_sm;
    if (ctx->math == WR_MATH_CUDA)
        return launch_advance_cuda(ctx->variant, blocks, ctx->stream, ctx->s, ctx->ctl, ctx->jbackup, ctx->ebuf);
    return launch_advance_portable(ctx->variant, blocks, ctx->stream, ctx->s, ctx->ctl, ctx->jbackup, ctx->ebuf);
}

cudaError_t launch_order(wr_ctx* ctx) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_order<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->s, ctx->ctl);
    return cudaGetLastError();
}

cudaError_t launch_prepare(wr_ctx* ctx) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const int blocks = (ctx->n + kPrepareThreads - 1) / kPrepareThreads;
    k_prepare<kPrepareThreads><<<blocks > 0 ? blocks : 1, kPrepareThreads, 0, ctx->stream>>>(ctx->s, ctx->ctl);
    return cudaGetLastError();
}

int read_ctl(wr_ctx* ctx) {
    cudaError_t e = cudaMemcpyAsync(ctx->host_ctl, ctx->ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return fail("cudaMemcpyAsync(step control)", e);
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail("cudaStreamSynchronize", e);
    return WR_SUCCESS;
}

}  // namespace

extern "C" {

const char* wr_last_error(void) { return g_last_error.c_str(); }

uint64_t wr_kernel_launch_count(void) { return g_launches.load(); }

int wr_create(int num_cells, int device, int math_mode, wr_ctx** out) {
    if (!out) return fail_msg("wr_create: null output pointer");
    *out = nullptr;
    if (num_cells <= 0) return fail_msg("wr_create: num_cells must be positive");
    if (math_mode != WR_MATH_PORTABLE && math_mode != WR_MATH_CUDA) return fail_msg("wr_create: unknown math mode");
    wr_ctx* ctx = new (std::nothrow) wr_ctx;
    if (!ctx) return fail_msg("wr_create: out of host memory");
    ctx->n = num_cells;
    ctx->device = device;
    ctx->math = math_mode;
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) {
        delete ctx;
        return rc;
    }
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete ctx;
        return fail("cudaStreamCreate", e);
    }
    const size_t n = static_cast<size_t>(num_cells);
    const size_t bytes = n * sizeof(double) * (3 + NS + 2) + n * sizeof(uint64_t) * 7 + n * sizeof(int) * 3;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    ctx->sms = sms > 0 ? sms : 1;
    ctx->advance_blocks = ctx->sms;
    size_t nslots = 0;  // lane slots of the largest configuration
    for (const AdvanceShape& sh : kAdvanceShapes) {
        const size_t slots = static_cast<size_t>(ctx->sms) * sh.blocks_per_sm * sh.threads;
        nslots = slots > nslots ? slots : nslots;
    }
    e = cudaMalloc(&ctx->state_buf, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->ctl, sizeof(StepCtl));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->jbackup, nslots * NEQ * NEQ * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->ebuf, nslots * NEQ * NEQ * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dt_hist, WR_MAX_COLLAPSE_STEPS * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->host_ctl, sizeof(StepCtl));
    if (e == cudaSuccess) e = ctx->math == WR_MATH_CUDA ? configure_advance_cuda() : configure_advance_portable();
    if (e != cudaSuccess) {
        wr_destroy(ctx);
        return fail("wr_create allocation", e);
    }
    char* p = static_cast<char*>(ctx->state_buf);
    auto take = [&](size_t b) {
        char* q = p;
        p += b;
        return q;
    };
    ctx->s.n = num_cells;
    ctx->s.stats = reinterpret_cast<uint64_t*>(take(n * sizeof(uint64_t) * 7));
    ctx->s.rho = reinterpret_cast<double*>(take(n * sizeof(double)));
    ctx->s.T = reinterpret_cast<double*>(take(n * sizeof(double)));
    ctx->s.e = reinterpret_cast<double*>(take(n * sizeof(double)));
    ctx->s.xn = reinterpret_cast<double*>(take(n * sizeof(double) * NS));
    ctx->s.time = reinterpret_cast<double*>(take(n * sizeof(double)));
    ctx->s.driver = reinterpret_cast<double*>(take(n * sizeof(double)));
    ctx->s.steps = reinterpret_cast<int*>(take(n * sizeof(int)));
    ctx->s.cost = reinterpret_cast<int*>(take(n * sizeof(int)));
    ctx->s.order = reinterpret_cast<int*>(take(n * sizeof(int)));
    StepCtl init{};
    init.dmin_bits = kDblMaxBits;
    init.failure = WR_SUCCESS;
    e = cudaMemcpyAsync(ctx->ctl, &init, sizeof init, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        wr_destroy(ctx);
        return fail("wr_create init", e);
    }
    *out = ctx;
    return WR_SUCCESS;
}

void wr_destroy(wr_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->profiling) wr_set_profiling(ctx, 0);
    cudaFree(ctx->state_buf);
    cudaFree(ctx->ctl);
    cudaFree(ctx->jbackup);
    cudaFree(ctx->ebuf);
    cudaFree(ctx->dt_hist);
    cudaFree(ctx->staging);
    cudaFreeHost(ctx->host_ctl);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

static int ensure_staging(wr_ctx* ctx) {
    if (ctx->staging) return WR_SUCCESS;
    const cudaError_t e = cudaMalloc(&ctx->staging, static_cast<size_t>(ctx->n) * sizeof(wr_collapse_state));
    return e == cudaSuccess ? WR_SUCCESS : fail("cudaMalloc(staging)", e);
}

int wr_upload(wr_ctx* ctx, const wr_collapse_state* cells) {
    if (!ctx || !cells) return fail_msg("wr_upload: null argument");
    int rc = set_device(ctx);
    if (rc == WR_SUCCESS) rc = ensure_staging(ctx);
    if (rc != WR_SUCCESS) return rc;
    const size_t bytes = static_cast<size_t>(ctx->n) * sizeof(wr_collapse_state);
    cudaError_t e = cudaMemcpyAsync(ctx->staging, cells, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return fail("cudaMemcpyAsync(cells to device)", e);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_unpack<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->staging, ctx->s);
    e = cudaMemsetAsync(ctx->s.cost, 0, static_cast<size_t>(ctx->n) * sizeof(int), ctx->stream);
    if (e != cudaSuccess) return fail("cudaMemsetAsync(cost)", e);
    StepCtl init{};
    init.dmin_bits = kDblMaxBits;
    init.failure = WR_SUCCESS;
    e = cudaMemcpyAsync(ctx->ctl, &init, sizeof init, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? WR_SUCCESS : fail("wr_upload", e);
}

int wr_download(wr_ctx* ctx, wr_collapse_state* cells) {
    if (!ctx || !cells) return fail_msg("wr_download: null argument");
    int rc = set_device(ctx);
    if (rc == WR_SUCCESS) rc = ensure_staging(ctx);
    if (rc != WR_SUCCESS) return rc;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_pack<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->s, ctx->staging);
    const size_t bytes = static_cast<size_t>(ctx->n) * sizeof(wr_collapse_state);
    cudaError_t e = cudaMemcpyAsync(cells, ctx->staging, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? WR_SUCCESS : fail("wr_download", e);
}

int wr_prepare(wr_ctx* ctx, int completed_global_steps, double grid_time, int step, int perturb,
               double* dt_grid_out) {
    if (!ctx || !dt_grid_out) return fail_msg("wr_prepare: null argument");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_begin_step<<<1, 1, 0, ctx->stream>>>(ctx->ctl, completed_global_steps, grid_time, step, perturb ? 1 : 0);
    cudaError_t e = launch_prepare(ctx);
    if (e != cudaSuccess) return fail("prepare launch", e);
    rc = read_ctl(ctx);
    if (rc != WR_SUCCESS) return rc;
    *dt_grid_out = ctx->host_ctl->dmin_bits == kDblMaxBits
                       ? DBL_MAX
                       : [](unsigned long long b) { double d; std::memcpy(&d, &b, sizeof d); return d; }(ctx->host_ctl->dmin_bits);
    return ctx->host_ctl->failure;
}

int wr_advance(wr_ctx* ctx, int completed_global_steps, double next_grid_time, double dt_grid,
               int* integrated_out) {
    if (!ctx || !integrated_out) return fail_msg("wr_advance: null argument");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_begin_advance<<<1, 1, 0, ctx->stream>>>(ctx->ctl, completed_global_steps, next_grid_time, dt_grid);
    cudaError_t e = launch_order(ctx);
    if (e == cudaSuccess) e = launch_advance(ctx);
    if (e != cudaSuccess) return fail("advance launch", e);
    rc = read_ctl(ctx);
    if (rc != WR_SUCCESS) return rc;
    *integrated_out = ctx->host_ctl->integrated;
    return ctx->host_ctl->failure;
}

int wr_run(wr_ctx* ctx, int perturb, int* completed_global_steps) {
    if (!ctx || !completed_global_steps) return fail_msg("wr_run: null argument");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const int nev = 4 * WR_MAX_COLLAPSE_STEPS + 2;
    ctx->ev_used = 0;
    record(ctx, nev - 2);
    k_begin_step<<<1, 1, 0, ctx->stream>>>(ctx->ctl, *completed_global_steps, 0.0, 0, perturb ? 1 : 0);
    int steps_launched = 0;
    for (int step = 0; step < WR_MAX_COLLAPSE_STEPS; ++step) {
        record(ctx, 4 * step + 0);
        cudaError_t e = launch_prepare(ctx);
        record(ctx, 4 * step + 1);
        if (e == cudaSuccess) {
            g_launches.fetch_add(1, std::memory_order_relaxed);
            k_decide<<<1, 1, 0, ctx->stream>>>(ctx->ctl, ctx->dt_hist);
            e = launch_order(ctx);
            record(ctx, 4 * step + 2);
            if (e == cudaSuccess) e = launch_advance(ctx);
            record(ctx, 4 * step + 3);
        }
        steps_launched = step + 1;
        if (e == cudaSuccess) {
            g_launches.fetch_add(1, std::memory_order_relaxed);
            k_finalize<<<1, 1, 0, ctx->stream>>>(ctx->ctl, WR_MAX_COLLAPSE_STEPS);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) return fail("step launch", e);
        if ((step + 1) % kCheckEvery == 0 || step + 1 == WR_MAX_COLLAPSE_STEPS) {
            rc = read_ctl(ctx);
            if (rc != WR_SUCCESS) return rc;
            if (ctx->host_ctl->stop) break;
        }
    }
    record(ctx, nev - 1);
    rc = read_ctl(ctx);
    if (rc != WR_SUCCESS) return rc;
    if (ctx->profiling) {
        wr_run_timing t{};
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ctx->ev[nev - 2], ctx->ev[nev - 1]);
        t.run_ms = ms;
        for (int s = 0; s < steps_launched; ++s) {
            cudaEventElapsedTime(&ms, ctx->ev[4 * s + 0], ctx->ev[4 * s + 1]);
            t.prepare_ms += ms;
            cudaEventElapsedTime(&ms, ctx->ev[4 * s + 2], ctx->ev[4 * s + 3]);
            t.advance_ms += ms;
        }
        t.advance_launches = steps_launched;
        t.prepare_launches = steps_launched;
        t.outer_steps = ctx->host_ctl->cgs;
        ctx->timing = t;
    }
    *completed_global_steps = ctx->host_ctl->cgs;
    return ctx->host_ctl->failure;
}

int wr_set_advance_variant(wr_ctx* ctx, int variant) {
    if (!ctx) return fail_msg("wr_set_advance_variant: null context");
    if (variant < 0 || variant >= kAdvanceVariants) return fail_msg("wr_set_advance_variant: unknown variant");
    ctx->variant = variant;
    return WR_SUCCESS;
}

int wr_set_profiling(wr_ctx* ctx, int on) {
    if (!ctx) return fail_msg("wr_set_profiling: null context");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    if (on && !ctx->profiling) {
        for (auto& ev : ctx->ev) {
            const cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return fail("cudaEventCreate", e);
        }
    }
    if (!on && ctx->profiling) {
        for (auto& ev : ctx->ev) {
            cudaEventDestroy(ev);
            ev = nullptr;
        }
    }
    ctx->profiling = on != 0;
    return WR_SUCCESS;
}

int wr_get_run_timing(wr_ctx* ctx, wr_run_timing* out) {
    if (!ctx || !out) return fail_msg("wr_get_run_timing: null argument");
    *out = ctx->timing;
    return WR_SUCCESS;
}

int wr_dt_history(wr_ctx* ctx, double* out, int max_steps) {
    if (!ctx || !out || max_steps < 0) return fail_msg("wr_dt_history: bad argument");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    const int n = max_steps < WR_MAX_COLLAPSE_STEPS ? max_steps : WR_MAX_COLLAPSE_STEPS;
    cudaError_t e = cudaMemcpyAsync(out, ctx->dt_hist, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? WR_SUCCESS : fail("wr_dt_history", e);
}

int wr_run_cells(wr_collapse_state* cells, int num_cells, int perturb, int* completed_global_steps) {
    int device = 0;
    cudaGetDevice(&device);
    wr_ctx* ctx = nullptr;
    int rc = wr_create(num_cells, device, WR_MATH_PORTABLE, &ctx);
    if (rc != WR_SUCCESS) return rc;
    rc = wr_upload(ctx, cells);
    int result = rc;
    if (rc == WR_SUCCESS) result = wr_run(ctx, perturb, completed_global_steps);
    rc = wr_download(ctx, cells);
    if (rc != WR_SUCCESS && result == WR_SUCCESS) result = rc;
    wr_destroy(ctx);
    return result;
}

// make_initial_state / make_collapse_state, reproducer.cpp:7533-7546
void wr_make_collapse_state(wr_collapse_state* out) {
    static const double xn0[NS] = {1.0e-4, 1.0e-4, 1.0e0,  1.0e-40, 1.0e-40, 1.0e-40, 1.0e-40,
                                   1.0e-40, 1.0e-6, 1.0e-40, 1.0e-40, 1.0e-40, 1.0e-40, 0.0775};
    std::memset(out, 0, sizeof(*out));
    double xn[NS];
    double rho = 0.0;
    for (int k = 0; k < NS; ++k) {
        xn[k] = xn0[k];
        rho += xn[k] * mass(k);
    }
    double mf[NS];
    double sum = 0.0;
    for (int k = 0; k < NS; ++k) {
        mf[k] = mass(k) * xn[k] / rho;
        sum += mf[k];
    }
    for (int k = 0; k < NS; ++k) {
        mf[k] /= sum;
        xn[k] = mf[k] * rho / mass(k);
    }
    double sa = 0.0, sg = 0.0, rt = 0.0;
    for (int k = 0; k < NS; ++k) rt += xn[k] * mass(k);
    for (int k = 0; k < NS; ++k) {
        sa += xn[k];
        sg += (xn[k] * kMp / rt) * inv_gm1(k);
    }
    sa *= kMp / rt;
    sg /= sa;
    const double T = 1.0e2;
    out->rho = rho;
    out->T = T;
    out->e = sg * sa * kGasConstant * T;
    for (int k = 0; k < NS; ++k) out->xn[k] = xn[k];
    out->time = 0.0;
    out->density_driver = rho;
    out->completed_steps = 0;
}

}  // extern "C"
