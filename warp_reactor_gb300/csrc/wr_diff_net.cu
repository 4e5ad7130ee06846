// wr_diff_net.cu -- differentiation form: one out-of-line copy of the network
// routines used by the forward and adjoint kernels (generated code).
#include "wr_diff.cuh"

#undef WR_NET_HD
#define WR_NET_HD __device__ __forceinline__
#include "generated/network_adj.h"

static_assert(WR_NUM_RATE_MULT == wr::diff::NP, "rate multiplier count");

namespace wr {
namespace diff {

// One out-of-line copy of each network routine (each is thousands of instructions).
__device__ void net_jac(const double* X, double T, double* J) {
    double f[NEQ];
    LocalJSink sink{J};
    wr_net_jac_rhs<M>(X, T, f, sink);
}

__device__ void net_rhs(const double* X, double T, const double* mult, double* f) {
    wr_netp_rhs<M>(X, T, mult, f);
}

__device__ void net_rhs_vjp(const double* X, double T, const double* mult, const double* fbar,
                                         double* Xbar, double* Tbar, double* mbar) {
    double tb = 0.0;
    wr_netp_rhs_vjp<M>(X, T, mult, fbar, Xbar, tb, mbar);
    *Tbar += tb;
}

}  // namespace diff
}  // namespace wr
