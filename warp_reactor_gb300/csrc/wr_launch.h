// wr_launch.h -- host-side launchers of the advance kernel, one translation unit
// per math policy (the advance kernel is the large one; compiling the policies in
// parallel keeps the build short).
#pragma once

#include <cuda_runtime.h>

#include "wr_kernels.cuh"

namespace wr {

constexpr int kPrepareThreads = 256;

// Advance kernel configurations, selected per context (wr_set_advance_variant):
//   0  128 threads x 1 block per SM, iteration matrix in shared memory (225 KiB)
//   1  128 threads x 2 blocks per SM, iteration matrix in a global lane array
//   2  256 threads x 1 block per SM, iteration matrix in a global lane array
//   3  precision form: 256 threads x 1 block per SM, FP32 factorisation in shared
//      memory (900 B per lane) with one FP64 residual refinement per stage solve
//   4  384 threads x 1 block per SM (at most 168 registers per thread: more spills,
//      twelve warps per SM to hide them)
//   5  cooperative advance (wr_coop.cuh), 8 lanes per cell
//   6  cooperative advance, 16 lanes per cell
//   7  cooperative advance, 32 lanes per cell
//   (cooperative advance: one block per SM, as many warps as the cells' slot
//   arrays fit in its shared memory, kWarps of generated/coop_prog_g<G>.h)
constexpr int kAdvanceVariants = 8;
constexpr int kPrecisionVariant = 3;
constexpr int kDefaultVariant = 6;
struct AdvanceShape {
    int threads;    // lane-per-cell shapes (0 for the cooperative advance)
    int blocks_per_sm;
    bool smem_matrix;
    int precision;  // 0 FP64 factorisation, 1 FP32 factorisation + FP64 refinement
    int coop_lanes; // lanes per cell of the cooperative advance (0: one lane per cell)
};
constexpr AdvanceShape kAdvanceShapes[kAdvanceVariants] = {
    {128, 1, true, 0, 0},  {128, 2, false, 0, 0}, {256, 1, false, 0, 0},  {256, 1, true, 1, 0},
    {384, 1, false, 0, 0}, {0, 1, false, 0, 8}, {0, 1, false, 0, 16}, {0, 1, false, 0, 32}};
constexpr bool is_coop(int variant) { return kAdvanceShapes[variant].coop_lanes != 0; }

constexpr size_t advance_smem_bytes(int variant) {
    return kAdvanceShapes[variant].smem_matrix && !is_coop(variant)
               ? static_cast<size_t>(NEQ) * NEQ * kAdvanceShapes[variant].threads *
                     (kAdvanceShapes[variant].precision ? sizeof(float) : sizeof(double))
               : 0;
}

cudaError_t launch_advance_portable(int variant, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                    double* jbackup, double* ebuf);
cudaError_t launch_advance_cuda(int variant, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                double* jbackup, double* ebuf);
cudaError_t configure_advance_portable();
// gridwide-structured-cta32 policy (wr_adv_cta32.cu): one warp per 32-cell tile;
// jall / eall are per-cell [225][n] Jacobian and iteration-matrix arrays
cudaError_t launch_advance_cta32(int math_cuda, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                 double* jall, double* eall);
int cta32_blocks(int n);
cudaError_t configure_advance_cuda();
// cooperative advance (wr_adv_coop<G>.cu): G lanes per cell, one block per SM
cudaError_t configure_advance_coop8();
cudaError_t configure_advance_coop16();
cudaError_t configure_advance_coop32();
cudaError_t launch_advance_coop8(int math_cuda, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                  unsigned long long* phases);
cudaError_t launch_advance_coop16(int math_cuda, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                  unsigned long long* phases);
cudaError_t launch_advance_coop32(int math_cuda, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                  unsigned long long* phases);
// diagnostics of the cooperative programs and LU on device buffers (wr_diag.cu)
cudaError_t diag_coop_network8(int math_cuda, int n, const double* y, double* J, double* f, double* f2);
cudaError_t diag_coop_network16(int math_cuda, int n, const double* y, double* J, double* f, double* f2);
cudaError_t diag_coop_network32(int math_cuda, int n, const double* y, double* J, double* f, double* f2);
cudaError_t diag_coop_lu8(int n, const double* A, const double* b, double* LU, int* ipvt, int* info, double* x);
cudaError_t diag_coop_lu16(int n, const double* A, const double* b, double* LU, int* ipvt, int* info, double* x);
cudaError_t diag_coop_lu32(int n, const double* A, const double* b, double* LU, int* ipvt, int* info, double* x);

}  // namespace wr
