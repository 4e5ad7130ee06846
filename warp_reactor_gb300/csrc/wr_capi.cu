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
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/warp_reactor.h"
#include "wr_coop.cuh"
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
    int G = 1;                    // sub-grids batched in this context
    int* grid_of = nullptr;       // device: sub-grid of each cell (G > 1)
    int* grid_start = nullptr;    // device: first cell of each sub-grid (G > 1)
    int device = 0;
    int math = WR_MATH_PORTABLE;
    int advance_blocks = 0;
    int sms = 1;
    int variant = kDefaultVariant;  // the cooperative advance, 16 lanes per cell
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
    // CUDA graph of kCheckEvery outer steps (prepare, decide, order, advance,
    // finalize per step), captured once per advance variant and replayed by wr_run
    cudaGraphExec_t graph = nullptr;
    int graph_variant = -1;
    int graph_policy = -1;
    int graph_timed = -1;  // the captured graph records the per-kernel events
    int graph_phases = -1; // the captured graph launches the phase-counting advance
    unsigned long long* phases = nullptr;  // wr_diag_coop_phases: 16 device counters
    int policy = WR_POLICY_GRIDWIDE_INDEPENDENT;
    double* local_dt = nullptr;  // legacy-local policy: each cell's own dt
    double* cta_j = nullptr;     // cta32 policy: per-cell Jacobian [225][n]
    double* cta_e = nullptr;     // cta32 policy: per-cell iteration matrix [225][n]
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

// scatter the cells k_prepare queued into the heaviest-first bucket order
__global__ void k_order(DevState s, StepCtl* ctl) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= s.n || ctl->all_stop) return;
    const int b = s.qbucket[cell];
    if (b < 0) return;
    const unsigned int pos = atomicAdd(&ctl->off[b], 1u);
    if (pos < static_cast<unsigned int>(s.n)) s.order[pos] = cell;
}

// Prologue of advance_collapse_gridwide_kernel (reproducer.cpp:7748-7768) for every
// queued cell, fused with the queue scatter: the cell's free-fall dt check, the
// driver (density) update with the grid dt, the density limit, the scaling of the
// number densities and e from T (burn_ros2s prologue, :7594-7606).  The cell is
// then marked kQBurn (the advance burns it) or kQSkip.  Legacy-local cells were
// scaled by k_prepare_legacy already.
__global__ void __launch_bounds__(256) k_order_preburn(DevState s, StepCtl* ctl) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= s.n || ctl->all_stop) return;
    const int b = s.qbucket[cell];
    if (b < 0) return;
    const unsigned int pos = atomicAdd(&ctl->off[b], 1u);
    if (pos < static_cast<unsigned int>(s.n)) s.order[pos] = cell;
    const int g = s.grid_of ? s.grid_of[cell] : 0;
    const StepCtl* c = ctl + g;
    int flag = kQSkip;
    if (!c->stop && c->failure == WR_SUCCESS && s.steps[cell] == c->cgs) {
        s.cost[cell] = 0;
        if (s.local_dt != nullptr) {
            flag = kQBurn;
        } else {
            const int n = s.n;
            double xn[NS];
#pragma unroll
            for (int k = 0; k < NS; ++k) xn[k] = s.xn[k * n + cell];
            const double local_dt = collapse_timestep(xn);
            if (!(local_dt < 10.0)) {
                const double old_density = s.driver[cell];
                const double tff = ddiv(local_dt, kTffReduc);
                const double driver = old_density + c->dt_grid * ddiv(old_density, tff);
                s.driver[cell] = driver;
                if (valid_positive(driver) && !(driver > kDriverLimit)) {
                    const double ratio = ddiv(driver, old_density);
#pragma unroll
                    for (int k = 0; k < NS; ++k) xn[k] *= ratio;
                    s.rho[cell] = s.rho[cell] * ratio;
                    s.e[cell] = eos_e_from_T(xn, s.T[cell]);
#pragma unroll
                    for (int k = 0; k < NS; ++k) s.xn[k * n + cell] = xn[k];
                    flag = kQBurn;
                }
            }
        }
    }
    s.qbucket[cell] = flag;
}

// Commit of a successful burn (advance kernel epilogue, reproducer.cpp:7774-7784):
// renormalise the number densities, T from e, the grid clock and the step count;
// the integrated count per sub-grid.
__global__ void __launch_bounds__(256) k_commit(DevState s, StepCtl* ctl) {
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    bool done = false;
    int g = 0;
    if (cell < s.n && !ctl->all_stop && s.qbucket[cell] == kQBurnOK) {
        const int n = s.n;
        g = s.grid_of ? s.grid_of[cell] : 0;
        const StepCtl* c = ctl + g;
        double xn[NS];
#pragma unroll
        for (int k = 0; k < NS; ++k) xn[k] = s.xn[k * n + cell];
        renormalize(xn, s.rho[cell]);
        s.T[cell] = eos_T_from_e(xn, s.e[cell]);
#pragma unroll
        for (int k = 0; k < NS; ++k) s.xn[k * n + cell] = xn[k];
        const double dt = s.local_dt ? s.local_dt[cell] : 0.0;
        s.time[cell] = s.local_dt ? s.time[cell] + dt : c->next_grid_time;
        s.steps[cell] = c->cgs + 1;
        s.qbucket[cell] = kQSkip;
        done = true;
    }
    // one atomic per warp when the warp's cells share a sub-grid
    const unsigned m = __ballot_sync(0xffffffffu, done);
    const int g0 = __shfl_sync(0xffffffffu, g, __ffs(m ? m : 1u) - 1);
    const bool uniform = __all_sync(0xffffffffu, !done || g == g0);
    if (uniform) {
        if ((threadIdx.x & 31) == 0 && m) atomicAdd(&ctl[g0].integrated, __popc(m));
    } else if (done) {
        atomicAdd(&ctl[g].integrated, 1);
    }
}

// start of an outer step driven by the host (wr_prepare; one grid)
__global__ void k_begin_step(StepCtl* ctl, int cgs, double grid_time, int step, int perturb) {
    for (int b = 0; b < kBuckets; ++b) ctl->hist[b] = 0;
    ctl->cgs = cgs;
    ctl->grid_time = grid_time;
    ctl->step = step;
    ctl->perturb = perturb;
    ctl->dmin_bits = kDblMaxBits;
    ctl->stop = 0;
    ctl->all_stop = 0;
}

// start of a device-driven run: every sub-grid at step 0
__global__ void k_begin_run(StepCtl* ctl, int G, int cgs, int perturb) {
    const int g = threadIdx.x;
    if (g < G) {
        StepCtl* c = ctl + g;
        c->cgs = cgs;
        c->grid_time = 0.0;
        c->step = 0;
        c->perturb = perturb;
        c->dmin_bits = kDblMaxBits;
        c->stop = 0;
        c->integrated = 0;
    }
    if (g == 0) {
        for (int b = 0; b < kBuckets; ++b) ctl->hist[b] = 0;
        ctl->all_stop = 0;
    }
}

// advance arguments driven by the host (wr_advance; one grid)
__global__ void k_begin_advance(StepCtl* ctl, int cgs, double next_grid_time, double dt_grid) {
    ctl->cgs = cgs;
    ctl->next_grid_time = next_grid_time;
    ctl->dt_grid = dt_grid;
    ctl->integrated = 0;
    ctl->stop = 0;
    ctl->all_stop = 0;
    build_queue_offsets(ctl);
}

// host checks between prepare and advance, reproducer.cpp:7880-7909, one thread
// per sub-grid
__global__ void k_decide(StepCtl* ctl, int G, double* dt_hist, int legacy) {
    const int g = threadIdx.x;
    if (g == 0) build_queue_offsets(ctl);
    if (g >= G) return;
    StepCtl* c = ctl + g;
    if (c->stop) return;
    if (c->failure != WR_SUCCESS) {
        c->stop = 1;
        return;
    }
    if (legacy) {  // every cell has its own dt: no grid minimum
        c->integrated = 0;
        return;
    }
    if (c->dmin_bits == kDblMaxBits) {  // no candidate: the loop ends successfully
        c->stop = 1;
        return;
    }
    const double dt = __longlong_as_double(static_cast<long long>(c->dmin_bits));
    const double next = c->grid_time + dt;
    if (!valid_positive(dt) || !isfinite(next)) {
        c->failure = WR_BAD_INPUTS;
        c->stop = 1;
        return;
    }
    c->dt_grid = dt;
    c->next_grid_time = next;
    c->integrated = 0;
    if (c->step >= 0 && c->step < WR_MAX_COLLAPSE_STEPS) dt_hist[g * WR_MAX_COLLAPSE_STEPS + c->step] = dt;
}

// host bookkeeping after the advance, reproducer.cpp:7930-7958, one thread per
// sub-grid; the run ends when every sub-grid has stopped
__global__ void k_finalize(StepCtl* ctl, int G, int max_steps) {
    __shared__ int running;
    const int g = threadIdx.x;
    if (g == 0) running = 0;
    __syncthreads();
    if (g < G) {
        StepCtl* c = ctl + g;
        if (!c->stop) {
            if (c->failure != WR_SUCCESS || c->integrated == 0) {
                c->stop = 1;
            } else {
                c->grid_time = c->next_grid_time;
                c->cgs += 1;
                c->step += 1;
                c->dmin_bits = kDblMaxBits;
                if (c->step >= max_steps) c->stop = 1;
            }
        }
        if (!c->stop) atomicAdd(&running, 1);
    }
    __syncthreads();
    if (g == 0) ctl->all_stop = running == 0;
}

}  // namespace wr

namespace {

int set_device(wr_ctx* ctx) {
    const cudaError_t e = cudaSetDevice(ctx->device);
    return e == cudaSuccess ? WR_SUCCESS : fail("cudaSetDevice", e);
}

// with profiling on, record event idx on the context stream; inside a stream
// capture the record becomes an event-record node of the graph (the external
// flag, valid only during capture), so the events time the replayed kernels
void record(wr_ctx* ctx, int idx) {
    if (!ctx->profiling) return;
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(ctx->stream, &st);
    if (st == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(ctx->ev[idx], ctx->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(ctx->ev[idx], ctx->stream);
}

// the cooperative advance runs between k_order_preburn and k_commit
bool coop_active(const wr_ctx* ctx) {
    return ctx->policy != WR_POLICY_GRIDWIDE_CTA32 && is_coop(ctx->variant);
}

cudaError_t launch_advance(wr_ctx* ctx) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (ctx->policy == WR_POLICY_GRIDWIDE_CTA32)
        return launch_advance_cta32(ctx->math == WR_MATH_CUDA ? 1 : 0, cta32_blocks(ctx->n), ctx->stream, ctx->s,
                                    ctx->ctl, ctx->cta_j, ctx->cta_e);
    const int blocks = ctx->sms * kAdvanceShapes[ctx->variant].blocks_per_sm;
    if (is_coop(ctx->variant)) {
        const int math_cuda = ctx->math == WR_MATH_CUDA ? 1 : 0;
        switch (kAdvanceShapes[ctx->variant].coop_lanes) {
            case 8: return launch_advance_coop8(math_cuda, blocks, ctx->stream, ctx->s, ctx->ctl, ctx->phases);
            case 32: return launch_advance_coop32(math_cuda, blocks, ctx->stream, ctx->s, ctx->ctl, ctx->phases);
            default: return launch_advance_coop16(math_cuda, blocks, ctx->stream, ctx->s, ctx->ctl, ctx->phases);
        }
    }
    if (ctx->math == WR_MATH_CUDA)
        return launch_advance_cuda(ctx->variant, blocks, ctx->stream, ctx->s, ctx->ctl, ctx->jbackup, ctx->ebuf);
    return launch_advance_portable(ctx->variant, blocks, ctx->stream, ctx->s, ctx->ctl, ctx->jbackup, ctx->ebuf);
}

cudaError_t launch_order(wr_ctx* ctx) {
    if (ctx->policy == WR_POLICY_GRIDWIDE_CTA32) return cudaSuccess;  // tiles are fixed: no work queue
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (coop_active(ctx))
        k_order_preburn<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->s, ctx->ctl);
    else
        k_order<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->s, ctx->ctl);
    return cudaGetLastError();
}

// after the cooperative advance: commit the cells it burned
cudaError_t launch_commit(wr_ctx* ctx) {
    if (!coop_active(ctx)) return cudaSuccess;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_commit<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(ctx->s, ctx->ctl);
    return cudaGetLastError();
}

cudaError_t launch_prepare(wr_ctx* ctx) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const int blocks = (ctx->n + kPrepareThreads - 1) / kPrepareThreads;
    if (ctx->policy == WR_POLICY_LEGACY_LOCAL)
        k_prepare_legacy<kPrepareThreads><<<blocks > 0 ? blocks : 1, kPrepareThreads, 0, ctx->stream>>>(ctx->s, ctx->ctl);
    else
        k_prepare<kPrepareThreads><<<blocks > 0 ? blocks : 1, kPrepareThreads, 0, ctx->stream>>>(ctx->s, ctx->ctl);
    return cudaGetLastError();
}

cudaError_t reset_ctl(wr_ctx* ctx) {
    std::vector<StepCtl> init(static_cast<size_t>(ctx->G));
    for (auto& c : init) {
        std::memset(&c, 0, sizeof c);
        c.dmin_bits = kDblMaxBits;
        c.failure = WR_SUCCESS;
    }
    cudaError_t e = cudaMemcpyAsync(ctx->ctl, init.data(), init.size() * sizeof(StepCtl), cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e;
}

int read_ctl(wr_ctx* ctx) {
    cudaError_t e = cudaMemcpyAsync(ctx->host_ctl, ctx->ctl, sizeof(StepCtl) * ctx->G, cudaMemcpyDeviceToHost,
                                    ctx->stream);
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
    return wr_create_batch(1, &num_cells, device, math_mode, out);
}

int wr_create_batch(int num_grids, const int* cells_per_grid, int device, int math_mode, wr_ctx** out) {
    if (!out) return fail_msg("wr_create: null output pointer");
    *out = nullptr;
    if (num_grids < 1 || num_grids > 1024 || !cells_per_grid) return fail_msg("wr_create_batch: 1..1024 grids");
    long long total = 0;
    for (int g = 0; g < num_grids; ++g) {
        if (cells_per_grid[g] <= 0) return fail_msg("wr_create: num_cells must be positive");
        total += cells_per_grid[g];
    }
    if (total > 0x7fffffffLL) return fail_msg("wr_create_batch: more than INT_MAX cells");
    const int num_cells = static_cast<int>(total);
    if (math_mode != WR_MATH_PORTABLE && math_mode != WR_MATH_CUDA) return fail_msg("wr_create: unknown math mode");
    wr_ctx* ctx = new (std::nothrow) wr_ctx;
    if (!ctx) return fail_msg("wr_create: out of host memory");
    ctx->n = num_cells;
    ctx->G = num_grids;
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
    if (num_grids > 1) {
        std::vector<int> of(static_cast<size_t>(num_cells)), start(static_cast<size_t>(num_grids));
        int c0 = 0;
        for (int g = 0; g < num_grids; ++g) {
            start[g] = c0;
            for (int i = 0; i < cells_per_grid[g]; ++i) of[c0 + i] = g;
            c0 += cells_per_grid[g];
        }
        e = cudaMalloc(&ctx->grid_of, of.size() * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc(&ctx->grid_start, start.size() * sizeof(int));
        if (e == cudaSuccess) e = cudaMemcpy(ctx->grid_of, of.data(), of.size() * sizeof(int), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(ctx->grid_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            wr_destroy(ctx);
            return fail("wr_create_batch grid map", e);
        }
    }
    const size_t n = static_cast<size_t>(num_cells);
    const size_t bytes = n * sizeof(double) * (3 + NS + 2) + n * sizeof(uint64_t) * 7 + n * sizeof(int) * 4;
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
    if (e == cudaSuccess) e = cudaMalloc(&ctx->ctl, sizeof(StepCtl) * ctx->G);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->jbackup, nslots * NEQ * NEQ * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->ebuf, nslots * NEQ * NEQ * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dt_hist, static_cast<size_t>(ctx->G) * WR_MAX_COLLAPSE_STEPS * sizeof(double));
    if (e == cudaSuccess) e = cudaMallocHost(&ctx->host_ctl, sizeof(StepCtl) * ctx->G);
    if (e == cudaSuccess) e = ctx->math == WR_MATH_CUDA ? configure_advance_cuda() : configure_advance_portable();
    if (e == cudaSuccess) e = configure_advance_coop8();
    if (e == cudaSuccess) e = configure_advance_coop16();
    if (e == cudaSuccess) e = configure_advance_coop32();
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
    ctx->s.qbucket = reinterpret_cast<int*>(take(n * sizeof(int)));
    ctx->s.grid_of = ctx->grid_of;
    ctx->s.grid_start = ctx->grid_start;
    e = reset_ctl(ctx);
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
    if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
    cudaFree(ctx->state_buf);
    cudaFree(ctx->ctl);
    cudaFree(ctx->grid_of);
    cudaFree(ctx->grid_start);
    cudaFree(ctx->jbackup);
    cudaFree(ctx->ebuf);
    cudaFree(ctx->local_dt);
    cudaFree(ctx->cta_j);
    cudaFree(ctx->cta_e);
    cudaFree(ctx->dt_hist);
    cudaFree(ctx->staging);
    cudaFree(ctx->phases);
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
    e = reset_ctl(ctx);
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
    if (ctx->G != 1 || ctx->policy != WR_POLICY_GRIDWIDE_INDEPENDENT)
        return fail_msg("wr_prepare: host-stepped calls need a one-grid gridwide context");
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
    if (ctx->G != 1) return fail_msg("wr_advance: host-stepped calls need a one-grid context");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_begin_advance<<<1, 1, 0, ctx->stream>>>(ctx->ctl, completed_global_steps, next_grid_time, dt_grid);
    cudaError_t e = launch_order(ctx);
    if (e == cudaSuccess) e = launch_advance(ctx);
    if (e == cudaSuccess) e = launch_commit(ctx);
    if (e != cudaSuccess) return fail("advance launch", e);
    rc = read_ctl(ctx);
    if (rc != WR_SUCCESS) return rc;
    *integrated_out = ctx->host_ctl->integrated;
    return ctx->host_ctl->failure;
}

// one outer step's launches (captured into the graph); with profiling on, the
// events of chunk step `slot` bracket the prepare and the advance launch
static cudaError_t launch_step(wr_ctx* ctx, int slot) {
    record(ctx, 4 * slot + 0);
    cudaError_t e = launch_prepare(ctx);
    record(ctx, 4 * slot + 1);
    if (e == cudaSuccess) {
        g_launches.fetch_add(1, std::memory_order_relaxed);
        k_decide<<<1, 1024, 0, ctx->stream>>>(ctx->ctl, ctx->G, ctx->dt_hist,
                                              ctx->policy == WR_POLICY_LEGACY_LOCAL);
        e = launch_order(ctx);
    }
    record(ctx, 4 * slot + 2);
    if (e == cudaSuccess) e = launch_advance(ctx);
    record(ctx, 4 * slot + 3);
    if (e == cudaSuccess) e = launch_commit(ctx);
    if (e == cudaSuccess) {
        g_launches.fetch_add(1, std::memory_order_relaxed);
        k_finalize<<<1, 1024, 0, ctx->stream>>>(ctx->ctl, ctx->G, WR_MAX_COLLAPSE_STEPS);
        e = cudaGetLastError();
    }
    return e;
}

static int ensure_graph(wr_ctx* ctx) {
    if (ctx->graph && ctx->graph_variant == ctx->variant && ctx->graph_policy == ctx->policy &&
        ctx->graph_timed == (ctx->profiling ? 1 : 0) && ctx->graph_phases == (ctx->phases ? 1 : 0))
        return WR_SUCCESS;
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    const uint64_t before = g_launches.load();
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return fail("cudaStreamBeginCapture", e);
    for (int i = 0; i < kCheckEvery && e == cudaSuccess; ++i) e = launch_step(ctx, i);
    cudaGraph_t graph = nullptr;
    const cudaError_t e2 = cudaStreamEndCapture(ctx->stream, &graph);
    g_launches.store(before);  // capture launches nothing
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return fail("graph capture", e != cudaSuccess ? e : e2);
    }
    e = cudaGraphInstantiate(&ctx->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail("cudaGraphInstantiate", e);
    ctx->graph_variant = ctx->variant;
    ctx->graph_policy = ctx->policy;
    ctx->graph_timed = ctx->profiling ? 1 : 0;
    ctx->graph_phases = ctx->phases ? 1 : 0;
    return WR_SUCCESS;
}

// wr_run: chunks of kCheckEvery outer steps replayed from a CUDA graph, one
// 64-byte-per-grid status read between chunks.  With profiling on, the graph also
// records an event pair around every prepare and advance launch, and an event
// pair brackets the whole run: the per-kernel times of the shipped path.
static int run_graph(wr_ctx* ctx, int perturb, int* completed_global_steps) {
    int rc = ensure_graph(ctx);
    if (rc != WR_SUCCESS) return rc;
    const int nev = 4 * WR_MAX_COLLAPSE_STEPS + 2;
    wr_run_timing t{};
    record(ctx, nev - 2);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    k_begin_run<<<1, 1024, 0, ctx->stream>>>(ctx->ctl, ctx->G, *completed_global_steps, perturb ? 1 : 0);
    for (int done = 0; done < WR_MAX_COLLAPSE_STEPS; done += kCheckEvery) {
        cudaError_t e = cudaGraphLaunch(ctx->graph, ctx->stream);
        if (e != cudaSuccess) return fail("cudaGraphLaunch", e);
        g_launches.fetch_add((coop_active(ctx) ? 6 : 5) * kCheckEvery, std::memory_order_relaxed);
        rc = read_ctl(ctx);
        if (rc != WR_SUCCESS) return rc;
        if (ctx->profiling) {
            for (int s = 0; s < kCheckEvery; ++s) {
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, ctx->ev[4 * s + 0], ctx->ev[4 * s + 1]);
                t.prepare_ms += ms;
                cudaEventElapsedTime(&ms, ctx->ev[4 * s + 2], ctx->ev[4 * s + 3]);
                t.advance_ms += ms;
            }
        }
        if (ctx->host_ctl->all_stop) break;
    }
    if (ctx->profiling) {
        record(ctx, nev - 1);
        const cudaError_t e = cudaEventSynchronize(ctx->ev[nev - 1]);
        if (e != cudaSuccess) return fail("cudaEventSynchronize", e);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, ctx->ev[nev - 2], ctx->ev[nev - 1]);
        t.run_ms = ms;
        int steps = 0;  // outer steps that advanced some grid
        for (int g = 0; g < ctx->G; ++g) steps = ctx->host_ctl[g].cgs > steps ? ctx->host_ctl[g].cgs : steps;
        t.advance_launches = steps;
        t.prepare_launches = steps;
        t.outer_steps = ctx->host_ctl->cgs;
        ctx->timing = t;
    }
    *completed_global_steps = ctx->host_ctl->cgs;
    for (int g = 0; g < ctx->G; ++g)
        if (ctx->host_ctl[g].failure != WR_SUCCESS) return ctx->host_ctl[g].failure;
    return WR_SUCCESS;
}

static int run_profiled(wr_ctx* ctx, int perturb, int max_steps, int* completed_global_steps);

int wr_run(wr_ctx* ctx, int perturb, int* completed_global_steps) {
    if (!ctx || !completed_global_steps) return fail_msg("wr_run: null argument");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    return run_graph(ctx, perturb, completed_global_steps);
}

// launch by launch, with CUDA events around every kernel when profiling; stops
// after max_steps outer steps (the autotuner's short runs)
static int run_profiled(wr_ctx* ctx, int perturb, int max_steps, int* completed_global_steps) {
    int rc = WR_SUCCESS;
    g_launches.fetch_add(1, std::memory_order_relaxed);
    const int nev = 4 * WR_MAX_COLLAPSE_STEPS + 2;
    ctx->ev_used = 0;
    record(ctx, nev - 2);
    k_begin_run<<<1, 1024, 0, ctx->stream>>>(ctx->ctl, ctx->G, *completed_global_steps, perturb ? 1 : 0);
    int steps_launched = 0;
    for (int step = 0; step < max_steps; ++step) {
        record(ctx, 4 * step + 0);
        cudaError_t e = launch_prepare(ctx);
        record(ctx, 4 * step + 1);
        if (e == cudaSuccess) {
            g_launches.fetch_add(1, std::memory_order_relaxed);
            k_decide<<<1, 1024, 0, ctx->stream>>>(ctx->ctl, ctx->G, ctx->dt_hist,
                                                  ctx->policy == WR_POLICY_LEGACY_LOCAL);
            e = launch_order(ctx);
            record(ctx, 4 * step + 2);
            if (e == cudaSuccess) e = launch_advance(ctx);
            record(ctx, 4 * step + 3);
            if (e == cudaSuccess) e = launch_commit(ctx);
        }
        steps_launched = step + 1;
        if (e == cudaSuccess) {
            g_launches.fetch_add(1, std::memory_order_relaxed);
            k_finalize<<<1, 1024, 0, ctx->stream>>>(ctx->ctl, ctx->G, max_steps);
            e = cudaGetLastError();
        }
        if (e != cudaSuccess) return fail("step launch", e);
        if ((step + 1) % kCheckEvery == 0 || step + 1 == max_steps) {
            rc = read_ctl(ctx);
            if (rc != WR_SUCCESS) return rc;
            if (ctx->host_ctl->all_stop) break;
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
    for (int g = 0; g < ctx->G; ++g)
        if (ctx->host_ctl[g].failure != WR_SUCCESS) return ctx->host_ctl[g].failure;
    return WR_SUCCESS;
}

int wr_grid_result(wr_ctx* ctx, int grid, int* completed_global_steps, int* result) {
    if (!ctx || !completed_global_steps || !result || grid < 0 || grid >= ctx->G)
        return fail_msg("wr_grid_result: bad argument");
    int rc = set_device(ctx);
    if (rc == WR_SUCCESS) rc = read_ctl(ctx);
    if (rc != WR_SUCCESS) return rc;
    *completed_global_steps = ctx->host_ctl[grid].cgs;
    *result = ctx->host_ctl[grid].failure;
    return WR_SUCCESS;
}

int wr_grid_dt_history(wr_ctx* ctx, int grid, double* out, int max_steps) {
    if (!ctx || !out || max_steps < 0 || grid < 0 || grid >= ctx->G) return fail_msg("wr_grid_dt_history: bad argument");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    const int n = max_steps < WR_MAX_COLLAPSE_STEPS ? max_steps : WR_MAX_COLLAPSE_STEPS;
    cudaError_t e = cudaMemcpyAsync(out, ctx->dt_hist + static_cast<size_t>(grid) * WR_MAX_COLLAPSE_STEPS,
                                    n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? WR_SUCCESS : fail("wr_grid_dt_history", e);
}

int wr_autotune(wr_ctx* ctx, int perturb, int steps, int* best_variant) {
    if (!ctx || !best_variant || steps < 1) return fail_msg("wr_autotune: bad argument");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    const size_t bytes = static_cast<size_t>(ctx->n) * ((3 + NS + 2) * sizeof(double) + 7 * sizeof(uint64_t) + 4 * sizeof(int));
    void* snap = nullptr;
    cudaError_t e = cudaMalloc(&snap, bytes);
    if (e != cudaSuccess) return fail("wr_autotune snapshot", e);
    e = cudaMemcpyAsync(snap, ctx->state_buf, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    const bool was_profiling = ctx->profiling;
    const int keep = ctx->variant;
    if (e == cudaSuccess && !was_profiling) rc = wr_set_profiling(ctx, 1);
    double best_ms = 1e300;
    int best = keep;
    // candidates: the exact (FP64) launch shapes; the precision form is a
    // different arithmetic and is chosen explicitly, never by the tuner
    for (int v = 0; e == cudaSuccess && rc == WR_SUCCESS && v < kAdvanceVariants; ++v) {
        if (v == kPrecisionVariant) continue;
        e = cudaMemcpyAsync(ctx->state_buf, snap, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
        if (e != cudaSuccess) break;
        rc = reset_ctl(ctx) == cudaSuccess ? WR_SUCCESS : WR_BAD_INPUTS;
        if (rc != WR_SUCCESS) break;
        ctx->variant = v;
        int cgs = 0;
        rc = run_profiled(ctx, perturb, steps, &cgs);
        if (rc != WR_SUCCESS) break;
        if (ctx->timing.advance_ms < best_ms) {
            best_ms = ctx->timing.advance_ms;
            best = v;
        }
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->state_buf, snap, bytes, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess) e = reset_ctl(ctx);
    cudaFree(snap);
    if (!was_profiling) wr_set_profiling(ctx, 0);
    if (e != cudaSuccess) return fail("wr_autotune", e);
    if (rc != WR_SUCCESS) {
        ctx->variant = keep;
        return rc;
    }
    ctx->variant = best;
    *best_variant = best;
    return WR_SUCCESS;
}

int wr_set_policy(wr_ctx* ctx, int policy) {
    if (!ctx) return fail_msg("wr_set_policy: null context");
    if (policy != WR_POLICY_GRIDWIDE_INDEPENDENT && policy != WR_POLICY_LEGACY_LOCAL &&
        policy != WR_POLICY_GRIDWIDE_CTA32)
        return fail_msg("wr_set_policy: unknown policy");
    if (policy == WR_POLICY_LEGACY_LOCAL && ctx->G != 1) return fail_msg("wr_set_policy: legacy-local needs one grid");
    if (policy == WR_POLICY_GRIDWIDE_CTA32 && ctx->G != 1)
        return fail_msg("wr_set_policy: gridwide-cta32 needs one grid");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    if (policy == WR_POLICY_LEGACY_LOCAL && !ctx->local_dt) {
        const cudaError_t e = cudaMalloc(&ctx->local_dt, static_cast<size_t>(ctx->n) * sizeof(double));
        if (e != cudaSuccess) return fail("cudaMalloc(local dt)", e);
    }
    if (policy == WR_POLICY_GRIDWIDE_CTA32 && !ctx->cta_j) {
        const size_t bytes = static_cast<size_t>(ctx->n) * NEQ * NEQ * sizeof(double);
        cudaError_t e = cudaMalloc(&ctx->cta_j, bytes);
        if (e == cudaSuccess) e = cudaMalloc(&ctx->cta_e, bytes);
        if (e != cudaSuccess) return fail("wr_set_policy cta32 buffers", e);
    }
    ctx->policy = policy;
    ctx->s.local_dt = policy == WR_POLICY_LEGACY_LOCAL ? ctx->local_dt : nullptr;
    return WR_SUCCESS;
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

int wr_diag_coop_phases(wr_ctx* ctx, int on) {
    if (!ctx) return fail_msg("wr_diag_coop_phases: null context");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    if (on && !ctx->phases) {
        cudaError_t e = cudaMalloc(&ctx->phases, 16 * sizeof(unsigned long long));
        if (e == cudaSuccess) e = cudaMemset(ctx->phases, 0, 16 * sizeof(unsigned long long));
        if (e != cudaSuccess) return fail("wr_diag_coop_phases", e);
    }
    if (!on && ctx->phases) {
        const cudaError_t e = cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->phases);
        ctx->phases = nullptr;
        if (e != cudaSuccess) return fail("wr_diag_coop_phases", e);
    }
    return WR_SUCCESS;
}

int wr_diag_coop_phases_read(wr_ctx* ctx, unsigned long long* out16, int reset) {
    if (!ctx || !out16) return fail_msg("wr_diag_coop_phases_read: null argument");
    if (!ctx->phases) return fail_msg("wr_diag_coop_phases_read: phase counters are off (wr_diag_coop_phases)");
    int rc = set_device(ctx);
    if (rc != WR_SUCCESS) return rc;
    cudaError_t e = cudaMemcpyAsync(out16, ctx->phases, 16 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                    ctx->stream);
    if (e == cudaSuccess && reset) e = cudaMemsetAsync(ctx->phases, 0, 16 * sizeof(unsigned long long), ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return fail("wr_diag_coop_phases_read", e);
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
    int rc = wr_create(num_cells, device, WR_MATH_CUDA, &ctx);
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

// Seeded initial cells of the batching workload: the reference's initial cell
// (make_collapse_state) with its density scaled by a log-normal factor
// 10^(sigma_dex * N(0,1)) and its temperature drawn log-uniformly in
// [10^log10_tmin, 10^log10_tmax]; the energy follows from the EOS (eos_rt,
// reproducer.cpp:306-309).  Streams: splitmix64 of (cell, grid_id), Box-Muller
// for the normal deviate.  Host code; the same array feeds the GPU and the oracle.
void wr_make_batch_state(int grid_id, int cell, double sigma_dex, double log10_tmin, double log10_tmax,
                         wr_collapse_state* out) {
    wr_make_collapse_state(out);
    const uint64_t seed = (static_cast<uint64_t>(static_cast<unsigned int>(cell)) << 32U) ^
                          (static_cast<uint64_t>(static_cast<unsigned int>(grid_id) + 1U) << 8U) ^
                          0x5bd1e9955bd1e995ULL;
    double u[3];
    for (int k = 0; k < 3; ++k) {
        const uint64_t bits = splitmix64(seed + 0x632be59bd9b4e019ULL * static_cast<uint64_t>(k + 1)) >> 11U;
        u[k] = static_cast<double>(bits) * (1.0 / 9007199254740992.0);
    }
    const double two_pi = 6.283185307179586476925286766559;
    const double normal = std::sqrt(-2.0 * std::log(1.0 - u[0])) * std::cos(two_pi * u[1]);
    const double mult = std::pow(10.0, sigma_dex * normal);
    for (int k = 0; k < NS; ++k) out->xn[k] *= mult;
    out->rho *= mult;
    out->density_driver = out->rho;
    const double T = std::pow(10.0, log10_tmin + (log10_tmax - log10_tmin) * u[2]);
    double sa = 0.0, sg = 0.0, rt = 0.0;
    for (int k = 0; k < NS; ++k) rt += out->xn[k] * mass(k);
    for (int k = 0; k < NS; ++k) {
        sa += out->xn[k];
        sg += (out->xn[k] * kMp / rt) * inv_gm1(k);
    }
    sa *= kMp / rt;
    sg /= sa;
    out->T = T;
    out->e = sg * sa * kGasConstant * T;
}

}  // extern "C"
