// Advance kernel instantiated with the portable (bit-reproducible) exp/log/cbrt.
#include "wr_launch.h"

namespace wr {

cudaError_t configure_advance_portable() {
    return cudaFuncSetAttribute(k_advance<PortableMathCall, kAdvanceThreads>,
                                cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(advance_smem_bytes(kAdvanceThreads)));
}

cudaError_t launch_advance_portable(int blocks, cudaStream_t stream, DevState s, StepCtl* ctl, double* jbackup) {
    k_advance<PortableMathCall, kAdvanceThreads>
        <<<blocks, kAdvanceThreads, advance_smem_bytes(kAdvanceThreads), stream>>>(s, ctl, jbackup);
    return cudaGetLastError();
}

}  // namespace wr
