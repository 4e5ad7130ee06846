// wr_diag.cu -- diagnostic entry points (include/warp_reactor_diag.h): the device
// network, LU and math functions on caller-supplied inputs, for parity tests.
#include <cuda_runtime.h>

#include <string>

#include "../../include/warp_reactor_diag.h"
#include "wr_launch.h"

using namespace wr;

namespace {

constexpr int kLuThreads = 32;

struct RowSink {
    double* J;
    __device__ __forceinline__ void operator()(int r, int c, double v) { J[r * NEQ + c] = v; }
};

template <class M>
__global__ void k_diag_network(int n, const double* __restrict__ X, const double* __restrict__ T,
                               double* J, double* f_fused, double* f_rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double x[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) x[k] = X[i * NS + k];
    const double t = T[i];
    double f[NEQ];
    RowSink sink{J + static_cast<size_t>(i) * NEQ * NEQ};
    wr_net_jac_rhs<M>(x, t, f, sink);
#pragma unroll
    for (int k = 0; k < NEQ; ++k) f_fused[i * NEQ + k] = f[k];
    wr_net_rhs<M>(x, t, f);
#pragma unroll
    for (int k = 0; k < NEQ; ++k) f_rhs[i * NEQ + k] = f[k];
}

__global__ void k_diag_lu(int n, const double* __restrict__ A, const double* __restrict__ b, double* LU,
                          int* ipvt, int* info, double* x) {
    extern __shared__ double smem[];
    const int i = blockIdx.x * kLuThreads + threadIdx.x;
    Mat<kLuThreads> E{smem + threadIdx.x};
    const bool live = i < n;
    if (!live) return;
#pragma unroll
    for (int r = 0; r < NEQ; ++r)
#pragma unroll
        for (int c = 0; c < NEQ; ++c) E(r, c) = A[static_cast<size_t>(i) * NEQ * NEQ + r * NEQ + c];
    uint64_t ip = 0;
    const int inf = lu_decompose(E, ip);
    double v[NEQ];
#pragma unroll
    for (int k = 0; k < NEQ; ++k) v[k] = b[i * NEQ + k];
    if (inf == 0) lu_solve(E, ip, v);
#pragma unroll
    for (int r = 0; r < NEQ; ++r)
#pragma unroll
        for (int c = 0; c < NEQ; ++c) LU[static_cast<size_t>(i) * NEQ * NEQ + r * NEQ + c] = E(r, c);
#pragma unroll
    for (int k = 0; k < NEQ; ++k) {
        ipvt[i * NEQ + k] = static_cast<int>((ip >> (4 * k)) & 15);
        x[i * NEQ + k] = v[k];
    }
    info[i] = inf;
}

template <class M>
__global__ void k_diag_math(int n, const double* __restrict__ x, int fn, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    out[i] = fn == 0 ? M::exp(v) : fn == 1 ? M::log(v) : M::cbrt(v);
}

constexpr int kPeakIters = 4096;

// eight independent FMA chains per lane
__global__ void k_fp64_peak(double* out, double a, double b) {
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < kPeakIters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_diag_div(int n, const double* __restrict__ a, const double* __restrict__ b, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = ddiv(a[i], b[i]);
}

// one block of `warps` warps, each lane running C independent dependent FMA chains;
// clock64 cycles per iteration tell the per-warp FP64 issue interval
template <int C>
__global__ void k_fp64_issue(double* out, long long* cyc, int iters) {
    double x[C];
#pragma unroll
    for (int c = 0; c < C; ++c) x[c] = threadIdx.x * 1e-3 + c;
    const long long t0 = clock64();
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < C; ++c) x[c] = fma(x[c], 0.999999, 1.0e-7);
    }
    const long long t1 = clock64();
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < C; ++c) s += x[c];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
    if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

thread_local std::string g_diag_error;

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { cudaFree(p); }
};

int diag_fail(const char* what, cudaError_t e) {
    g_diag_error = std::string(what) + ": " + cudaGetErrorString(e);
    return WR_BAD_INPUTS;
}

}  // namespace

extern "C" {

int wr_diag_network(int n, const double* X, const double* T, int math_mode, double* J, double* f_fused,
                    double* f_rhs) {
    if (n <= 0 || !X || !T || !J || !f_fused || !f_rhs) return WR_BAD_INPUTS;
    const size_t nn = static_cast<size_t>(n);
    DevBuf dX, dT, dJ, dF, dR;
    cudaError_t e = cudaMalloc(&dX.p, nn * NS * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dT.p, nn * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dJ.p, nn * NEQ * NEQ * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dF.p, nn * NEQ * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dR.p, nn * NEQ * 8);
    if (e == cudaSuccess) e = cudaMemcpy(dX.p, X, nn * NS * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dT.p, T, nn * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return diag_fail("wr_diag_network setup", e);
    const int blocks = (n + 63) / 64;
    if (math_mode == WR_MATH_CUDA)
        k_diag_network<CudaMath><<<blocks, 64>>>(n, (double*)dX.p, (double*)dT.p, (double*)dJ.p, (double*)dF.p,
                                                 (double*)dR.p);
    else
        k_diag_network<PortableMathCall><<<blocks, 64>>>(n, (double*)dX.p, (double*)dT.p, (double*)dJ.p,
                                                         (double*)dF.p, (double*)dR.p);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(J, dJ.p, nn * NEQ * NEQ * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f_fused, dF.p, nn * NEQ * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f_rhs, dR.p, nn * NEQ * 8, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WR_SUCCESS : diag_fail("wr_diag_network", e);
}

int wr_diag_lu(int n, const double* A, const double* b, double* LU, int* ipvt, int* info, double* x) {
    if (n <= 0 || !A || !b || !LU || !ipvt || !info || !x) return WR_BAD_INPUTS;
    const size_t nn = static_cast<size_t>(n);
    DevBuf dA, db, dLU, dip, dinfo, dx;
    const size_t smem = static_cast<size_t>(NEQ) * NEQ * kLuThreads * sizeof(double);
    cudaError_t e = cudaFuncSetAttribute(k_diag_lu, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e == cudaSuccess) e = cudaMalloc(&dA.p, nn * 225 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&db.p, nn * 15 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dLU.p, nn * 225 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dip.p, nn * 15 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dinfo.p, nn * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dx.p, nn * 15 * 8);
    if (e == cudaSuccess) e = cudaMemcpy(dA.p, A, nn * 225 * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db.p, b, nn * 15 * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return diag_fail("wr_diag_lu setup", e);
    k_diag_lu<<<(n + kLuThreads - 1) / kLuThreads, kLuThreads, smem>>>(
        n, (double*)dA.p, (double*)db.p, (double*)dLU.p, (int*)dip.p, (int*)dinfo.p, (double*)dx.p);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(LU, dLU.p, nn * 225 * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ipvt, dip.p, nn * 15 * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(info, dinfo.p, nn * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(x, dx.p, nn * 15 * 8, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WR_SUCCESS : diag_fail("wr_diag_lu", e);
}

int wr_diag_coop_network(int lanes_per_cell, int n, const double* y, int math_mode, double* J, double* f,
                         double* f2) {
    if (n <= 0 || !y || !J || !f || !f2) return WR_BAD_INPUTS;
    if (lanes_per_cell != 8 && lanes_per_cell != 16 && lanes_per_cell != 32) return WR_BAD_INPUTS;
    const size_t nn = static_cast<size_t>(n);
    DevBuf dy, dJ, dF, dR;
    cudaError_t e = cudaMalloc(&dy.p, nn * NEQ * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dJ.p, nn * NEQ * NEQ * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dF.p, nn * NEQ * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dR.p, nn * NEQ * 8);
    if (e == cudaSuccess) e = cudaMemcpy(dy.p, y, nn * NEQ * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return diag_fail("wr_diag_coop_network setup", e);
    const int mc = math_mode == WR_MATH_CUDA ? 1 : 0;
    const double* py = static_cast<const double*>(dy.p);
    double *pJ = static_cast<double*>(dJ.p), *pF = static_cast<double*>(dF.p), *pR = static_cast<double*>(dR.p);
    e = lanes_per_cell == 8    ? diag_coop_network8(mc, n, py, pJ, pF, pR)
        : lanes_per_cell == 16 ? diag_coop_network16(mc, n, py, pJ, pF, pR)
                               : diag_coop_network32(mc, n, py, pJ, pF, pR);
    if (e == cudaSuccess) e = cudaMemcpy(J, dJ.p, nn * NEQ * NEQ * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f, dF.p, nn * NEQ * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f2, dR.p, nn * NEQ * 8, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WR_SUCCESS : diag_fail("wr_diag_coop_network", e);
}

int wr_diag_coop_lu(int lanes_per_cell, int n, const double* A, const double* b, double* LU, int* ipvt, int* info,
                    double* x) {
    if (n <= 0 || !A || !b || !LU || !ipvt || !info || !x) return WR_BAD_INPUTS;
    if (lanes_per_cell != 8 && lanes_per_cell != 16 && lanes_per_cell != 32) return WR_BAD_INPUTS;
    const size_t nn = static_cast<size_t>(n);
    DevBuf dA, db, dLU, dip, dinfo, dx;
    cudaError_t e = cudaMalloc(&dA.p, nn * 225 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&db.p, nn * 15 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dLU.p, nn * 225 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dip.p, nn * 15 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dinfo.p, nn * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dx.p, nn * 15 * 8);
    if (e == cudaSuccess) e = cudaMemcpy(dA.p, A, nn * 225 * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db.p, b, nn * 15 * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return diag_fail("wr_diag_coop_lu setup", e);
    const double *pA = static_cast<const double*>(dA.p), *pb = static_cast<const double*>(db.p);
    double *pLU = static_cast<double*>(dLU.p), *px = static_cast<double*>(dx.p);
    int *pip = static_cast<int*>(dip.p), *pinfo = static_cast<int*>(dinfo.p);
    e = lanes_per_cell == 8    ? diag_coop_lu8(n, pA, pb, pLU, pip, pinfo, px)
        : lanes_per_cell == 16 ? diag_coop_lu16(n, pA, pb, pLU, pip, pinfo, px)
                               : diag_coop_lu32(n, pA, pb, pLU, pip, pinfo, px);
    if (e == cudaSuccess) e = cudaMemcpy(LU, dLU.p, nn * 225 * 8, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ipvt, dip.p, nn * 15 * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(info, dinfo.p, nn * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(x, dx.p, nn * 15 * 8, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WR_SUCCESS : diag_fail("wr_diag_coop_lu", e);
}

int wr_diag_math(int n, const double* x, int fn, int math_mode, double* out) {
    if (n <= 0 || !x || !out || fn < 0 || fn > 2) return WR_BAD_INPUTS;
    const size_t nn = static_cast<size_t>(n);
    DevBuf dx, dout;
    cudaError_t e = cudaMalloc(&dx.p, nn * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dout.p, nn * 8);
    if (e == cudaSuccess) e = cudaMemcpy(dx.p, x, nn * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return diag_fail("wr_diag_math setup", e);
    const int blocks = (n + 255) / 256;
    if (math_mode == WR_MATH_CUDA)
        k_diag_math<CudaMath><<<blocks, 256>>>(n, (double*)dx.p, fn, (double*)dout.p);
    else
        k_diag_math<PortableMath><<<blocks, 256>>>(n, (double*)dx.p, fn, (double*)dout.p);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, dout.p, nn * 8, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WR_SUCCESS : diag_fail("wr_diag_math", e);
}

int wr_diag_div(int n, const double* a, const double* b, double* out) {
    if (n <= 0 || !a || !b || !out) return WR_BAD_INPUTS;
    const size_t nn = static_cast<size_t>(n);
    DevBuf da, db, dout;
    cudaError_t e = cudaMalloc(&da.p, nn * 8);
    if (e == cudaSuccess) e = cudaMalloc(&db.p, nn * 8);
    if (e == cudaSuccess) e = cudaMalloc(&dout.p, nn * 8);
    if (e == cudaSuccess) e = cudaMemcpy(da.p, a, nn * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db.p, b, nn * 8, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return diag_fail("wr_diag_div setup", e);
    k_diag_div<<<(n + 255) / 256, 256>>>(n, (double*)da.p, (double*)db.p, (double*)dout.p);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(out, dout.p, nn * 8, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? WR_SUCCESS : diag_fail("wr_diag_div", e);
}

int wr_diag_flush_l2(int mib) {
    static void* buf = nullptr;
    static size_t have = 0;
    if (mib <= 0) return WR_BAD_INPUTS;
    const size_t bytes = static_cast<size_t>(mib) << 20;
    if (bytes > have) {
        cudaFree(buf);
        buf = nullptr;
        have = 0;
        const cudaError_t e = cudaMalloc(&buf, bytes);
        if (e != cudaSuccess) return diag_fail("wr_diag_flush_l2", e);
        have = bytes;
    }
    cudaError_t e = cudaMemset(buf, mib & 0xff, bytes);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? WR_SUCCESS : diag_fail("wr_diag_flush_l2", e);
}

int wr_diag_fp64_issue(int warps, int chains, double* cycles_per_instr) {
    if (warps < 1 || warps > 32 || !cycles_per_instr || (chains != 1 && chains != 4 && chains != 8)) return WR_BAD_INPUTS;
    DevBuf out, cyc;
    cudaError_t e = cudaMalloc(&out.p, static_cast<size_t>(warps) * 32 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&cyc.p, sizeof(long long));
    if (e != cudaSuccess) return diag_fail("wr_diag_fp64_issue", e);
    const int iters = 2048;
    for (int rep = 0; rep < 2; ++rep) {  // the first launch warms up
        if (chains == 1) k_fp64_issue<1><<<1, warps * 32>>>((double*)out.p, (long long*)cyc.p, iters);
        else if (chains == 4) k_fp64_issue<4><<<1, warps * 32>>>((double*)out.p, (long long*)cyc.p, iters);
        else k_fp64_issue<8><<<1, warps * 32>>>((double*)out.p, (long long*)cyc.p, iters);
    }
    long long c = 0;
    e = cudaMemcpy(&c, cyc.p, sizeof c, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return diag_fail("wr_diag_fp64_issue", e);
    *cycles_per_instr = static_cast<double>(c) / (static_cast<double>(iters) * chains);
    return WR_SUCCESS;
}

int wr_diag_fp64_peak(double* dfma_per_s) {
    if (!dfma_per_s) return WR_BAD_INPUTS;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
    const int blocks = sms * 8, threads = 256;
    DevBuf out;
    cudaError_t e = cudaMalloc(&out.p, static_cast<size_t>(blocks) * threads * sizeof(double));
    if (e != cudaSuccess) return diag_fail("wr_diag_fp64_peak", e);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    k_fp64_peak<<<blocks, threads>>>((double*)out.p, 0.999999, 1.0e-7);  // warm-up
    cudaEventRecord(a);
    k_fp64_peak<<<blocks, threads>>>((double*)out.p, 0.999999, 1.0e-7);
    cudaEventRecord(b);
    e = cudaEventSynchronize(b);
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess) return diag_fail("wr_diag_fp64_peak", e);
    *dfma_per_s = static_cast<double>(blocks) * threads * kPeakIters * 8 / (ms * 1e-3);
    return WR_SUCCESS;
}

}  // extern "C"
