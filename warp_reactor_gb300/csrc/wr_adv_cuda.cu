// Advance kernel instantiated with CUDA's libm exp/log/cbrt: the arithmetic of the
// reference's own CUDA build (reproducer.cpp compiled with nvcc --fmad=false).
#include "wr_launch.h"

namespace wr {

cudaError_t configure_advance_cuda() {
    return cudaFuncSetAttribute(k_advance<CudaMath, kAdvanceThreads>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(advance_smem_bytes(kAdvanceThreads)));
}

cudaError_t launch_advance_cuda(int blocks, cudaStream_t stream, DevState s, StepCtl* ctl, double* jbackup) {
    k_advance<CudaMath, kAdvanceThreads>
        <<<blocks, kAdvanceThreads, advance_smem_bytes(kAdvanceThreads), stream>>>(s, ctl, jbackup);
    return cudaGetLastError();
}

}  // namespace wr
