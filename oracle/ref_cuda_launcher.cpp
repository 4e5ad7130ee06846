// ORACLE -- test infrastructure only.
//
// Runs the reference's own CUDA kernels (oracle/_ref/ref_kernels.cubin, built from
// reproducer.cpp by oracle/build_ref.sh) through the host loop of run_cells_cuda
// (reproducer.cpp:7791-7975), and writes the packed final states of the
// reference's file format (reproducer.cpp:7488-7505, 8357-8378).  The kernels are
// found in the cubin by name with the driver API; nothing of the reference is
// modified.  Usage: ref_cuda_launcher <cubin> <grid> <out.bin> [--no-perturb] [--structured]
// --structured: the cubin holds the reference's structured (gridwide-structured-
// cta32) advance kernel, launched as the reference's host loop does in that build
// (reproducer.cpp:7843-7852, 7910-7916): one block of 256 threads per 32-cell tile,
// its shared storage, and a per-cell Jacobian cache.
#include <cuda.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../include/warp_reactor.h"

#define CK(x)                                                                  \
    do {                                                                       \
        CUresult r_ = (x);                                                     \
        if (r_ != CUDA_SUCCESS) {                                              \
            const char* s_ = nullptr;                                          \
            cuGetErrorString(r_, &s_);                                         \
            std::fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");       \
            std::exit(2);                                                      \
        }                                                                      \
    } while (0)

// wr_make_collapse_state restated: make_collapse_state, reproducer.cpp:7533-7546
static wr_collapse_state initial_cell() {
    static const double m[14] = {9.10938188e-28,   1.67262158e-24,   1.67353251819e-24, 1.67444345638e-24,
                                 3.34512158e-24,   3.34603251819e-24, 3.34615409819e-24, 3.34694345638e-24,
                                 3.34706503638e-24, 5.01865409819e-24, 5.01956503638e-24, 6.69024316e-24,
                                 6.69115409819e-24, 6.69206503638e-24};
    static const double x0[14] = {1.0e-4, 1.0e-4, 1.0e0,  1.0e-40, 1.0e-40, 1.0e-40, 1.0e-40,
                                  1.0e-40, 1.0e-6, 1.0e-40, 1.0e-40, 1.0e-40, 1.0e-40, 0.0775};
    wr_collapse_state c;
    std::memset(&c, 0, sizeof c);
    double xn[14], rho = 0.0, mf[14], sum = 0.0;
    for (int k = 0; k < 14; ++k) { xn[k] = x0[k]; rho += xn[k] * m[k]; }
    for (int k = 0; k < 14; ++k) { mf[k] = m[k] * xn[k] / rho; sum += mf[k]; }
    for (int k = 0; k < 14; ++k) { mf[k] /= sum; xn[k] = mf[k] * rho / m[k]; }
    const double mp = 1.67262192595e-24, gc = 6.02214076e+23 * 1.3806490000000002e-16;
    double sa = 0.0, sg = 0.0, rt = 0.0;
    for (int k = 0; k < 14; ++k) rt += xn[k] * m[k];
    for (int k = 0; k < 14; ++k) {
        const double g = (k == 6 || k == 8 || k == 9 || k == 10) ? 1.4 : 5.0 / 3.0;
        sa += xn[k];
        sg += (xn[k] * mp / rt) * (1.0 / (g - 1.0));
    }
    sa *= mp / rt;
    sg /= sa;
    c.rho = rho;
    c.T = 1.0e2;
    c.e = sg * sa * gc * c.T;
    for (int k = 0; k < 14; ++k) c.xn[k] = xn[k];
    c.density_driver = rho;
    return c;
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s <cubin> <grid> <out.bin> [--no-perturb] [--structured]\n", argv[0]);
        return 2;
    }
    const int grid = std::atoi(argv[2]);
    bool perturb = true, structured = false;
    for (int a = 4; a < argc; ++a) {
        const std::string opt(argv[a]);
        if (opt == "--no-perturb") perturb = false;
        else if (opt == "--structured") structured = true;
        else {
            std::fprintf(stderr, "unknown option %s\n", argv[a]);
            return 2;
        }
    }
    int n = grid * grid * grid;
    std::vector<wr_collapse_state> cells(static_cast<size_t>(n), initial_cell());
    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    CUmodule mod;
    CK(cuModuleLoad(&mod, argv[1]));
    unsigned int count = 0;
    CK(cuModuleGetFunctionCount(&count, mod));
    std::vector<CUfunction> fns(count);
    CK(cuModuleEnumerateFunctions(fns.data(), count, mod));
    CUfunction prep = nullptr, adv = nullptr;
    for (CUfunction f : fns) {
        const char* name = nullptr;
        CK(cuFuncGetName(&name, f));
        const std::string s(name);
        if (s.find("prepare_grid_timestep_kernel") != std::string::npos) prep = f;
        if (structured ? s.find("advance_collapse_gridwide_structured_kernel") != std::string::npos
                       : (s.find("advance_collapse_gridwide_kernel") != std::string::npos &&
                          s.find("structured") == std::string::npos))
            adv = f;
    }
    if (!prep || !adv) {
        std::fprintf(stderr, "reference kernels not found in %s\n", argv[1]);
        return 2;
    }
    unsigned long long shared_bytes = 0;
    if (structured) {
        CUdeviceptr sym;
        size_t sym_size = 0;
        CK(cuModuleGetGlobal(&sym, &sym_size, mod, "wr_ref_structured_shared_bytes"));
        CK(cuMemcpyDtoH(&shared_bytes, sym, sizeof shared_bytes));
        CK(cuFuncSetAttribute(adv, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, static_cast<int>(shared_bytes)));
    }
    const auto t0 = std::chrono::steady_clock::now();
    CUdeviceptr dcells, dcand, dcount, dfail, djac = 0;
    CK(cuMemAlloc(&dcells, cells.size() * sizeof(wr_collapse_state)));
    CK(cuMemAlloc(&dcand, cells.size() * sizeof(double)));
    CK(cuMemAlloc(&dcount, sizeof(int)));
    CK(cuMemAlloc(&dfail, sizeof(int)));
    if (structured) CK(cuMemAlloc(&djac, cells.size() * 225 * sizeof(double)));
    CK(cuMemcpyHtoD(dcells, cells.data(), cells.size() * sizeof(wr_collapse_state)));
    const int success = 1;
    CK(cuMemcpyHtoD(dfail, &success, sizeof(int)));
    std::vector<double> cand(cells.size());
    const int block = 128, blocks = (n + block - 1) / block;
    int cgs = 0;
    double grid_time = 0.0;
    int result = 1;
    bool p = perturb;
    for (int step = 0; result == 1 && step < WR_MAX_COLLAPSE_STEPS; ++step) {
        void* pa[] = {&dcells, &n, &cgs, &grid_time, &step, &p, &dcand, &dfail};
        CK(cuLaunchKernel(prep, blocks, 1, 1, block, 1, 1, 0, nullptr, pa, nullptr));
        CK(cuCtxSynchronize());
        int hf = 0;
        CK(cuMemcpyDtoH(&hf, dfail, sizeof(int)));
        CK(cuMemcpyDtoH(cand.data(), dcand, cand.size() * sizeof(double)));
        if (hf != 1) { result = hf; break; }
        double dtg = 1.7976931348623157e308;
        for (double c : cand) if (c < dtg) dtg = c;
        if (dtg == 1.7976931348623157e308) break;
        double next = grid_time + dtg;
        if (!(dtg > 0.0) || !(next - next == 0.0)) { result = -1; break; }
        const int zero = 0;
        CK(cuMemcpyHtoD(dcount, &zero, sizeof(int)));
        if (structured) {
            void* sa[] = {&dcells, &n, &cgs, &grid_time, &next, &dtg, &djac, &dcount, &dfail};
            const unsigned tiles = static_cast<unsigned>((n + 31) / 32);
            CK(cuLaunchKernel(adv, tiles, 1, 1, 256, 1, 1, static_cast<unsigned>(shared_bytes), nullptr, sa, nullptr));
        } else {
            void* aa[] = {&dcells, &n, &cgs, &next, &dtg, &dcount, &dfail};
            CK(cuLaunchKernel(adv, blocks, 1, 1, block, 1, 1, 0, nullptr, aa, nullptr));
        }
        CK(cuCtxSynchronize());
        int cnt = 0;
        CK(cuMemcpyDtoH(&hf, dfail, sizeof(int)));
        CK(cuMemcpyDtoH(&cnt, dcount, sizeof(int)));
        if (hf != 1) { result = hf; break; }
        if (cnt == 0) break;
        grid_time = next;
        cgs += 1;
    }
    CK(cuMemcpyDtoH(cells.data(), dcells, cells.size() * sizeof(wr_collapse_state)));
    const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // substep totals over the grid (IntegratorStats, reproducer.cpp:7433-7441)
    unsigned long long internal = 0, accepted = 0, rejected = 0, jacobians = 0;
    for (const wr_collapse_state& c : cells) {
        internal += c.stats.internal_steps;
        accepted += c.stats.accepted_steps;
        rejected += c.stats.rejected_steps;
        jacobians += c.stats.jacobian_calls;
    }
    std::printf("{\"grid\": %d, \"cells\": %d, \"result\": %d, \"completed_global_steps\": %d, \"wall_s\": %.6f, "
                "\"cells_per_s\": %.3f, \"internal_steps\": %llu, \"accepted_steps\": %llu, \"rejected_steps\": %llu, "
                "\"jacobian_calls\": %llu}\n",
                grid, n, result, cgs, wall, n / wall, internal, accepted, rejected, jacobians);
    FILE* f = std::fopen(argv[3], "wb");
    if (!f) return 2;
    for (int c = 0; c < n; ++c) {
        wr_packed_final_state r;
        r.cell = c; r.i = c % grid; r.j = (c / grid) % grid; r.k = c / (grid * grid);
        r.completed_steps = cells[c].completed_steps;
        r.time = cells[c].time; r.density_driver = cells[c].density_driver;
        r.rho = cells[c].rho; r.T = cells[c].T; r.e = cells[c].e;
        std::memcpy(r.xn, cells[c].xn, sizeof r.xn);
        std::fwrite(&r, sizeof r, 1, f);
    }
    std::fclose(f);
    return result == 1 ? 0 : 1;
}
