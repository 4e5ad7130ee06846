// wr_launch.h -- host-side launchers of the advance kernel, one translation unit
// per math policy (the advance kernel is the large one; compiling the policies in
// parallel keeps the build short).
#pragma once

#include <cuda_runtime.h>

#include "wr_kernels.cuh"

namespace wr {

constexpr int kAdvanceThreads = 128;  // one warp per SM sub-partition
constexpr int kPrepareThreads = 256;

// dynamic shared memory of k_advance: one 15x15 FP64 matrix per lane
constexpr size_t advance_smem_bytes(int threads) { return static_cast<size_t>(NEQ) * NEQ * threads * sizeof(double); }

cudaError_t launch_advance_portable(int blocks, cudaStream_t stream, DevState s, StepCtl* ctl, double* jbackup);
cudaError_t launch_advance_cuda(int blocks, cudaStream_t stream, DevState s, StepCtl* ctl, double* jbackup);
cudaError_t configure_advance_portable();
cudaError_t configure_advance_cuda();

}  // namespace wr
