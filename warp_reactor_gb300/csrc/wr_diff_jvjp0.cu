// wr_diff_jvjp0.cu -- differentiation form: Jacobian vector-Jacobian product,
// forward chunks and the upper half of the reverse chunks (generated code,
// split over two translation units so that they compile in parallel).
#include "wr_diff.cuh"

#undef WR_NET_HD
#define WR_NET_HD __device__ __forceinline__
#define WR_NET_CHUNK __device__ __noinline__
#include "generated/network_adj.h"

static_assert(WR_NET_JAC_VJP_CHUNKS == 12, "chunk list below");

namespace wr {
namespace diff {

// forward chunks 0..C-1, then reverse chunks C-1..C/2
__device__ void jac_vjp_part0(const double* X, double T, const double* Jbar, double* V, double* A, double* Xbar,
                              double& Tbar) {
    wr_net_jac_vjp_f0<M>(X, T, V);
    wr_net_jac_vjp_f1<M>(X, T, V);
    wr_net_jac_vjp_f2<M>(X, T, V);
    wr_net_jac_vjp_f3<M>(X, T, V);
    wr_net_jac_vjp_f4<M>(X, T, V);
    wr_net_jac_vjp_f5<M>(X, T, V);
    wr_net_jac_vjp_f6<M>(X, T, V);
    wr_net_jac_vjp_f7<M>(X, T, V);
    wr_net_jac_vjp_f8<M>(X, T, V);
    wr_net_jac_vjp_f9<M>(X, T, V);
    wr_net_jac_vjp_f10<M>(X, T, V);
    wr_net_jac_vjp_f11<M>(X, T, V);
    wr_net_jac_vjp_r11<M>(X, T, Jbar, V, A, Xbar, Tbar);
    wr_net_jac_vjp_r10<M>(X, T, Jbar, V, A, Xbar, Tbar);
    wr_net_jac_vjp_r9<M>(X, T, Jbar, V, A, Xbar, Tbar);
    wr_net_jac_vjp_r8<M>(X, T, Jbar, V, A, Xbar, Tbar);
    wr_net_jac_vjp_r7<M>(X, T, Jbar, V, A, Xbar, Tbar);
    wr_net_jac_vjp_r6<M>(X, T, Jbar, V, A, Xbar, Tbar);
}

}  // namespace diff
}  // namespace wr
