// wr_noalloc.cu -- wr_advance_cells_noalloc: one advance step of the gridwide
// integrator on caller-owned device memory, with no device allocation at all.
//
// Who needs it: callers that hold their cells in device memory they manage
// themselves and may not allocate -- a host code running inside another
// framework's memory pool or allocator, or a caller on a budgeted or
// pre-partitioned device -- where the context API's cudaMalloc of state,
// Jacobian backup and step control is not allowed.
//
// All scratch lives in one file-scope __device__ array of kNoallocScratchBytes
// (7.9 MiB, held on every GPU that loads the library until the process exits):
// the step control block, a structure-of-arrays copy of at most
// WR_NOALLOC_MAX_CELLS cells, and the per-lane Jacobian backup of
// WR_NOALLOC_LANES lanes (32 blocks of 128).  Calls share that array: every call
// re-initialises what must start from zero, and calls that overlap on the GPU
// (from several host threads or streams) race on it and must not be issued.
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it for the life of
// the process; do not use the entry point across a cudaDeviceReset of that
// device.  Every call launches on the legacy default stream and ends with a
// blocking copy, so no call may be issued while any stream capture is active,
// and a caller that wrote the cells on a non-blocking stream must order that
// work before the call (cudaStreamSynchronize or an event).
//
// Arithmetic: the portable exp/log/cbrt (WR_MATH_PORTABLE), one lane per cell;
// the result equals wr_advance of a WR_MATH_PORTABLE context bit for bit.
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>
#include <string>

#include "../../include/warp_reactor.h"
#include "wr_launch.h"

using namespace wr;

namespace {

constexpr size_t kCtlBytes = 4096;
constexpr size_t kStateBytesPerCell = (3 + NS + 2) * sizeof(double) + 7 * sizeof(uint64_t) + 3 * sizeof(int);
constexpr size_t kStateBytes = ((WR_NOALLOC_MAX_CELLS * kStateBytesPerCell + 255) / 256) * 256;
constexpr size_t kJacBytes = static_cast<size_t>(WR_NOALLOC_LANES) * NEQ * NEQ * sizeof(double);
constexpr size_t kNoallocScratchBytes = kCtlBytes + kStateBytes + kJacBytes;
static_assert(sizeof(StepCtl) <= kCtlBytes, "step control must fit its slot");
// the call reads failure and integrated back with one copy
static_assert(offsetof(StepCtl, integrated) == offsetof(StepCtl, failure) + sizeof(int),
              "StepCtl: integrated must follow failure");
constexpr int kNoallocThreads = 128;  // advance shape 0: 128 lanes per block, matrices in shared memory

// The scratch array.  Host code must not use this name as a device address: it
// is a host-side stand-in; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};
thread_local std::string g_noalloc_error;

int noalloc_fail(const std::string& msg) {
    g_noalloc_error = msg;
    return WR_BAD_INPUTS;
}

__global__ void k_noalloc_unpack(const wr_collapse_state* __restrict__ in, DevState s, StepCtl* ctl, int cgs,
                                 double next_grid_time, double dt_grid) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        ctl->dmin_bits = kDblMaxBits;
        ctl->failure = WR_SUCCESS;
        ctl->integrated = 0;
        ctl->stop = 0;
        ctl->cgs = cgs;
        ctl->step = cgs;
        ctl->perturb = 0;
        ctl->grid_time = 0.0;
        ctl->dt_grid = dt_grid;
        ctl->next_grid_time = next_grid_time;
        ctl->queue = 0;
        ctl->queued = static_cast<unsigned int>(s.n);
        ctl->all_stop = 0;
    }
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
    s.cost[i] = 0;
    s.order[i] = i;  // cells in index order
}

__global__ void k_noalloc_pack(DevState s, wr_collapse_state* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= s.n) return;
    const int n = s.n;
    wr_collapse_state c = out[i];
    c.rho = s.rho[i];
    c.T = s.T[i];
    c.e = s.e[i];
#pragma unroll
    for (int k = 0; k < NS; ++k) c.xn[k] = s.xn[k * n + i];
    c.time = s.time[i];
    c.density_driver = s.driver[i];
    c.completed_steps = s.steps[i];
    c.stats.internal_steps = s.stats[0 * n + i];
    c.stats.rhs_calls = s.stats[1 * n + i];
    c.stats.jacobian_calls = s.stats[2 * n + i];
    c.stats.decompositions = s.stats[3 * n + i];
    c.stats.linear_solves = s.stats[4 * n + i];
    c.stats.accepted_steps = s.stats[5 * n + i];
    c.stats.rejected_steps = s.stats[6 * n + i];
    out[i] = c;
}

// Device address of the scratch array on the current device (looked up once).
int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail("wr_advance_cells_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return noalloc_fail(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        e = configure_advance_portable();  // dynamic shared memory limit of the advance kernel
        if (e != cudaSuccess)
            return noalloc_fail(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return WR_SUCCESS;
}

}  // namespace

extern "C" {

int wr_advance_cells_noalloc(wr_collapse_state* d_cells, int num_cells, int completed_global_steps,
                             double next_grid_time, double dt_grid, int* integrated_out) {
    g_noalloc_error.clear();
    if (!d_cells || !integrated_out) return noalloc_fail("wr_advance_cells_noalloc: null argument");
    if (num_cells <= 0) return noalloc_fail("wr_advance_cells_noalloc: num_cells must be positive");
    if (num_cells > WR_NOALLOC_MAX_CELLS)
        return noalloc_fail("wr_advance_cells_noalloc: num_cells " + std::to_string(num_cells) +
                            " exceeds the no-allocation limit of " + std::to_string(WR_NOALLOC_MAX_CELLS) +
                            " cells; use the context API (wr_create/wr_advance) for larger grids");
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != WR_SUCCESS) return rc;
    char* p = static_cast<char*>(base);
    StepCtl* ctl = reinterpret_cast<StepCtl*>(p);
    char* q = p + kCtlBytes;
    const size_t n = static_cast<size_t>(num_cells);
    DevState s{};
    s.n = num_cells;
    s.stats = reinterpret_cast<uint64_t*>(q);
    q += n * sizeof(uint64_t) * 7;
    s.rho = reinterpret_cast<double*>(q);
    q += n * sizeof(double);
    s.T = reinterpret_cast<double*>(q);
    q += n * sizeof(double);
    s.e = reinterpret_cast<double*>(q);
    q += n * sizeof(double);
    s.xn = reinterpret_cast<double*>(q);
    q += n * sizeof(double) * NS;
    s.time = reinterpret_cast<double*>(q);
    q += n * sizeof(double);
    s.driver = reinterpret_cast<double*>(q);
    q += n * sizeof(double);
    s.steps = reinterpret_cast<int*>(q);
    q += n * sizeof(int);
    s.cost = reinterpret_cast<int*>(q);
    q += n * sizeof(int);
    s.order = reinterpret_cast<int*>(q);
    s.qbucket = nullptr;  // not used by the advance kernel
    s.local_dt = nullptr;
    s.grid_of = nullptr;
    s.grid_start = nullptr;
    double* jbackup = reinterpret_cast<double*>(p + kCtlBytes + kStateBytes);

    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return noalloc_fail(std::string("wr_advance_cells_noalloc: device query: ") + cudaGetErrorString(e));
    int blocks = (num_cells + kNoallocThreads - 1) / kNoallocThreads;
    const int max_blocks = WR_NOALLOC_LANES / kNoallocThreads;
    if (blocks > max_blocks) blocks = max_blocks;
    if (blocks > sms) blocks = sms;

    const int grid = (num_cells + 255) / 256;
    k_noalloc_unpack<<<grid, 256>>>(d_cells, s, ctl, completed_global_steps, next_grid_time, dt_grid);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = launch_advance_portable(0, blocks, nullptr, s, ctl, jbackup, nullptr);
    if (e == cudaSuccess) {
        k_noalloc_pack<<<grid, 256>>>(s, d_cells);
        e = cudaGetLastError();
    }
    int head[2] = {0, 0};  // failure, integrated (adjacent ints of StepCtl)
    if (e == cudaSuccess)
        e = cudaMemcpy(head, &ctl->failure, sizeof(head), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess)
        return noalloc_fail(std::string("wr_advance_cells_noalloc: ") + cudaGetErrorString(e));
    *integrated_out = head[1];
    return head[0];
}

const char* wr_noalloc_last_error(void) { return g_noalloc_error.c_str(); }

}  // extern "C"
