// Advance kernel instantiated with CUDA's libm exp/log/cbrt: the arithmetic of the reference's own CUDA build (reproducer.cpp compiled with nvcc --fmad=false).
#include "wr_launch.h"

namespace wr {

cudaError_t configure_advance_cuda() {
    cudaError_t e = cudaFuncSetAttribute(k_advance<CudaMath, 128, 1, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(advance_smem_bytes(0)));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_advance<CudaMath, 256, 1, true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(advance_smem_bytes(kPrecisionVariant)));
}

cudaError_t launch_advance_cuda(int variant, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                    double* jbackup, double* ebuf) {
    switch (variant) {
        case 1:
            k_advance<CudaMath, 128, 2, false><<<blocks, 128, 0, stream>>>(s, ctl, jbackup, ebuf);
            break;
        case 2:
            k_advance<CudaMath, 256, 1, false><<<blocks, 256, 0, stream>>>(s, ctl, jbackup, ebuf);
            break;
        case 4:
            k_advance<CudaMath, 384, 1, false><<<blocks, 384, 0, stream>>>(s, ctl, jbackup, ebuf);
            break;
        case 3:
            k_advance<CudaMath, 256, 1, true, 1>
                <<<blocks, 256, advance_smem_bytes(kPrecisionVariant), stream>>>(s, ctl, jbackup, ebuf);
            break;
        default:
            k_advance<CudaMath, 128, 1, true><<<blocks, 128, advance_smem_bytes(0), stream>>>(s, ctl, jbackup, ebuf);
            break;
    }
    return cudaGetLastError();
}

}  // namespace wr
