// wr_diff_jvjp1.cu -- differentiation form: Jacobian vector-Jacobian product,
// the lower half of the reverse chunks and the driver (generated code).
#include "wr_diff.cuh"

#undef WR_NET_HD
#define WR_NET_HD __device__ __forceinline__
#define WR_NET_CHUNK __device__ __noinline__
#include "generated/network_adj.h"

static_assert(WR_NET_JAC_VJP_CHUNKS == 12, "chunk list below");

namespace wr {
namespace diff {

__device__ void jac_vjp_part0(const double* X, double T, const double* Jbar, double* V, double* A, double* Xbar,
                              double& Tbar);

// adjoints of X and T of sum_rc Jbar[r][c] * J[r][c](X, T), accumulated
__device__ void net_jac_vjp(const double* X, double T, const double* Jbar, double* Xbar, double* Tbar) {
    double V[WR_NET_JAC_VJP_SLOTS], A[WR_NET_JAC_VJP_SLOTS];
    double tb = 0.0;
    jac_vjp_part0(X, T, Jbar, V, A, Xbar, tb);
    wr_net_jac_vjp_r5<M>(X, T, Jbar, V, A, Xbar, tb);
    wr_net_jac_vjp_r4<M>(X, T, Jbar, V, A, Xbar, tb);
    wr_net_jac_vjp_r3<M>(X, T, Jbar, V, A, Xbar, tb);
    wr_net_jac_vjp_r2<M>(X, T, Jbar, V, A, Xbar, tb);
    wr_net_jac_vjp_r1<M>(X, T, Jbar, V, A, Xbar, tb);
    wr_net_jac_vjp_r0<M>(X, T, Jbar, V, A, Xbar, tb);
    *Tbar += tb;
}

}  // namespace diff
}  // namespace wr
