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
constexpr int kAdvanceVariants = 5;
constexpr int kPrecisionVariant = 3;
struct AdvanceShape {
    int threads;
    int blocks_per_sm;
    bool smem_matrix;
    int precision;  // 0 FP64 factorisation, 1 FP32 factorisation + FP64 refinement
};
constexpr AdvanceShape kAdvanceShapes[kAdvanceVariants] = {
    {128, 1, true, 0}, {128, 2, false, 0}, {256, 1, false, 0}, {256, 1, true, 1}, {384, 1, false, 0}};

constexpr size_t advance_smem_bytes(int variant) {
    return kAdvanceShapes[variant].smem_matrix
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
cudaError_t launch_advance_cta32(int blocks, cudaStream_t stream, DevState s, StepCtl* ctl, double* jall,
                                 double* eall);
int cta32_blocks(int n);
cudaError_t configure_advance_cuda();

}  // namespace wr
