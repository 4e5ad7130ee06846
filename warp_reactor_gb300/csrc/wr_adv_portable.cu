// Advance kernel instantiated with portable (bit-reproducible) exp/log/cbrt.
#include "wr_launch.h"

namespace wr {

cudaError_t configure_advance_portable() {
    return cudaFuncSetAttribute(k_advance<PortableMathCall, 128, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(advance_smem_bytes(0)));
}

cudaError_t launch_advance_portable(int variant, int blocks, cudaStream_t stream, DevState s, StepCtl* ctl,
                                    double* jbackup, double* ebuf) {
    switch (variant) {
        case 1:
            k_advance<PortableMathCall, 128, 2, false><<<blocks, 128, 0, stream>>>(s, ctl, jbackup, ebuf);
            break;
        case 2:
            k_advance<PortableMathCall, 256, 1, false><<<blocks, 256, 0, stream>>>(s, ctl, jbackup, ebuf);
            break;
        default:
            k_advance<PortableMathCall, 128, 1, true><<<blocks, 128, advance_smem_bytes(0), stream>>>(s, ctl, jbackup, ebuf);
            break;
    }
    return cudaGetLastError();
}

}  // namespace wr
