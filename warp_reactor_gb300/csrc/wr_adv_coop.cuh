// wr_adv_coop.cuh -- one translation unit per lanes-per-cell count G: the
// generated vector programs of that G (coop_prog_g<G>.h, large initialisers) and
// the cooperative advance kernel instantiated for both math policies.  The unit
// defines WR_COOP_G and includes generated/coop_prog_g<G>.h (which sets the warps
// per block: as many as the block's shared memory holds) before this file.
#include "wr_launch.h"
#include "wr_coop.cuh"

#define WR_CAT2(a, b) a##b
#define WR_CAT(a, b) WR_CAT2(a, b)

namespace wr {

namespace {
namespace cp = WR_CAT(coop, WR_COOP_G);

struct Tab {
    static constexpr int kNV = cp::kNV;
    static constexpr int kNR = cp::kNR;
    static constexpr int kNF = cp::kNF;
    static constexpr int kJSteps = cp::kJRHSSteps;
    static constexpr int kRSteps = cp::kRHSSteps;
    static __device__ __forceinline__ const ulonglong2* jprog() { return cp::kJRHSProg; }
    static __device__ __forceinline__ const uint64_t* jlit() { return cp::kJRHSLit; }
    static __device__ __forceinline__ const ulonglong2* rprog() { return cp::kRHSProg; }
    static __device__ __forceinline__ const uint64_t* rlit() { return cp::kRHSLit; }
    static __device__ __forceinline__ const uint16_t* jout() { return cp::kJRHSOut; }
    static __device__ __forceinline__ const uint16_t* jac() { return cp::kJRHSJac; }
    static __device__ __forceinline__ const uint16_t* rout() { return cp::kRHSOut; }
    static __device__ __forceinline__ const uint64_t* vconst() { return cp::kVConst; }
    static __device__ __forceinline__ const ulonglong2* vfun() { return cp::kVFun; }
};
static_assert(Tab::kJSteps % 4 == 0 && Tab::kRSteps % 4 == 0, "programs are padded to groups of four steps");
static_assert(coop::kRes + Tab::kNR + Tab::kNF <= Tab::kNV, "reserved constants lie inside the slot array");

constexpr int kG = WR_COOP_G;
constexpr int kW = cp::kWarps;
constexpr size_t kSmem = static_cast<size_t>(kW) * (32 / kG) * Tab::kNV * 8;
static_assert(kSmem <= 232448, "cooperative advance: shared memory of one block exceeds 227 KiB");
}  // namespace

cudaError_t WR_CAT(configure_advance_coop, WR_COOP_G)() {
    const void* kernels[4] = {reinterpret_cast<const void*>(k_advance_coop<PortableMathCall, kG, kW, Tab, false>),
                              reinterpret_cast<const void*>(k_advance_coop<CudaMath, kG, kW, Tab, false>),
                              reinterpret_cast<const void*>(k_advance_coop<PortableMathCall, kG, kW, Tab, true>),
                              reinterpret_cast<const void*>(k_advance_coop<CudaMath, kG, kW, Tab, true>)};
    for (const void* k : kernels) {
        const cudaError_t e =
            cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kSmem));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// phases: the 16 phase counters of the instrumented instantiation (nullptr: the
// plain kernel)
cudaError_t WR_CAT(launch_advance_coop, WR_COOP_G)(int math_cuda, int blocks, cudaStream_t stream, DevState s,
                                                   StepCtl* ctl, unsigned long long* phases) {
    if (phases) {
        if (math_cuda)
            k_advance_coop<CudaMath, kG, kW, Tab, true><<<blocks, kW * 32, kSmem, stream>>>(s, ctl, phases);
        else
            k_advance_coop<PortableMathCall, kG, kW, Tab, true><<<blocks, kW * 32, kSmem, stream>>>(s, ctl, phases);
    } else if (math_cuda) {
        k_advance_coop<CudaMath, kG, kW, Tab, false><<<blocks, kW * 32, kSmem, stream>>>(s, ctl, nullptr);
    } else {
        k_advance_coop<PortableMathCall, kG, kW, Tab, false><<<blocks, kW * 32, kSmem, stream>>>(s, ctl, nullptr);
    }
    return cudaGetLastError();
}

namespace {
constexpr int kDiagWarps = 4;
constexpr size_t kDiagNetSmem = static_cast<size_t>(kDiagWarps) * (32 / kG) * Tab::kNV * 8;
constexpr size_t kDiagLuSmem = static_cast<size_t>(kDiagWarps) * (32 / kG) * NEQ * NEQ * 8;
}  // namespace

// diagnostics on device buffers (wr_diag.cu owns the host side)
cudaError_t WR_CAT(diag_coop_network, WR_COOP_G)(int math_cuda, int n, const double* y, double* J, double* f,
                                                 double* f2) {
    const int per_block = kDiagWarps * (32 / kG);
    const int blocks = (n + per_block - 1) / per_block;
    cudaError_t e;
    if (math_cuda) {
        e = cudaFuncSetAttribute(k_diag_coop_network<CudaMath, kG, Tab>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(kDiagNetSmem));
        if (e != cudaSuccess) return e;
        k_diag_coop_network<CudaMath, kG, Tab><<<blocks, kDiagWarps * 32, kDiagNetSmem>>>(n, y, J, f, f2);
    } else {
        e = cudaFuncSetAttribute(k_diag_coop_network<PortableMathCall, kG, Tab>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kDiagNetSmem));
        if (e != cudaSuccess) return e;
        k_diag_coop_network<PortableMathCall, kG, Tab><<<blocks, kDiagWarps * 32, kDiagNetSmem>>>(n, y, J, f, f2);
    }
    return cudaGetLastError();
}

cudaError_t WR_CAT(diag_coop_lu, WR_COOP_G)(int n, const double* A, const double* b, double* LU, int* ipvt, int* info,
                                            double* x) {
    const int per_block = kDiagWarps * (32 / kG);
    k_diag_coop_lu<kG><<<(n + per_block - 1) / per_block, kDiagWarps * 32, kDiagLuSmem>>>(n, A, b, LU, ipvt, info, x);
    return cudaGetLastError();
}

}  // namespace wr
