// wr_diff_bwd.cu -- differentiation form: the discrete adjoint kernel (the map
// and its storage are described in wr_diff.cuh).
#include "wr_diff.cuh"

namespace wr {
namespace diff {

// ---------------------------------------------------------------- adjoint pieces
// The adjoints below differentiate the mathematical form of each operation (the
// forward values are the exact IEEE sequence; derivatives need no bit matching).

// eos_re: T = e * A / (R mp B), A = sum m x, B = sum x/(gamma-1)
__device__ __forceinline__ void eos_T_adj(const double* x, double e, double Tbar, double* xbar, double& ebar) {
    double A = 0.0, B = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        A += mass(n) * x[n];
        B += x[n] * inv_gm1(n);
    }
    const double T = e * A / (kGasConstant * kMp * B);
    ebar += Tbar * A / (kGasConstant * kMp * B);
#pragma unroll
    for (int n = 0; n < NS; ++n) xbar[n] += Tbar * T * (mass(n) / A - inv_gm1(n) / B);
}

// eos_rt: e = R mp T B / A
__device__ __forceinline__ void eos_e_adj(const double* x, double T, double ebar, double* xbar, double& Tbar) {
    double A = 0.0, B = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        A += mass(n) * x[n];
        B += x[n] * inv_gm1(n);
    }
    const double e = kGasConstant * kMp * T * B / A;
    Tbar += ebar * kGasConstant * kMp * B / A;
#pragma unroll
    for (int n = 0; n < NS; ++n) xbar[n] += ebar * e * (inv_gm1(n) / B - mass(n) / A);
}

// floor_and_normalize: out = max(x, F) * rho / S, S = sum m max(x, F)
__device__ __forceinline__ void fn_adj(const double* x, double rho, const double* obar, double* xbar, double& rhobar) {
    double xf[NS], S = 0.0, c = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        xf[n] = smax(x[n], kFloor);
        S += mass(n) * xf[n];
        c += obar[n] * xf[n];
    }
    rhobar += c / S;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        const double g = obar[n] * rho / S - mass(n) * rho * c / (S * S);
        xbar[n] = (x[n] < kFloor) ? 0.0 : g;
    }
}

// renormalize = floor_and_normalize, balance_charge, floor_and_normalize;
// xbar receives (overwrites) the adjoint of x
static __device__ __noinline__ void renorm_adj(const double* x, double rho, const double* obar, double* xbar, double& rhobar) {
    double x1[NS], l2[NS], l1[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) x1[n] = x[n];
    floor_and_normalize(x1, rho);
    balance_charge(x1);  // x1 is now x2, the input of the second normalisation
    fn_adj(x1, rho, obar, l2, rhobar);
    // balance_charge: x2[0] = -x3 - x7 + x1 + x12 + x6 + x4 + x9 + 2 x11
#pragma unroll
    for (int n = 0; n < NS; ++n) l1[n] = l2[n];
    l1[0] = 0.0;
    l1[3] -= l2[0];
    l1[7] -= l2[0];
    l1[1] += l2[0];
    l1[12] += l2[0];
    l1[6] += l2[0];
    l1[4] += l2[0];
    l1[9] += l2[0];
    l1[11] += 2.0 * l2[0];
    fn_adj(x, rho, l1, xbar, rhobar);
}

// state_from_y: X = max(y, F), T = eos_re(X, y[14])
__device__ __forceinline__ void sfy_adj(const double* y, const double* X, const double* Xbar, double Tbar,
                                        double* ybar) {
    double xb[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) xb[n] = Xbar[n];
    double eb = 0.0;
    eos_T_adj(X, y[NS], Tbar, xb, eb);
#pragma unroll
    for (int n = 0; n < NS; ++n) ybar[n] += (y[n] < kFloor) ? 0.0 : xb[n];
    ybar[NS] += eb;
}

// x <- E^-T x with the LU of E (LINPACK dgesl, transposed job)
static __device__ __noinline__ void lu_solve_t(MatL LU, uint64_t ip, double* x) {
#pragma unroll 1
    for (int k = 0; k < NEQ; ++k) {
        double t = 0.0;
#pragma unroll 1
        for (int i = 0; i < k; ++i) t += LU(i, k) * x[i];
        x[k] = (x[k] - t) / LU(k, k);
    }
#pragma unroll 1
    for (int k = NEQ - 2; k >= 0; --k) {
        double t = 0.0;
#pragma unroll 1
        for (int i = k + 1; i < NEQ; ++i) t += LU(i, k) * x[i];
        x[k] += t;
        const int l = static_cast<int>((ip >> (4 * k)) & 15);
        if (l != k) {
            const double tmp = x[l];
            x[l] = x[k];
            x[k] = tmp;
        }
    }
}

// f-VJP at state ys (X, T from state_from_y), accumulated into ybar and mbar
static __device__ __noinline__ void rhs_adj_at(const double* ys, const double* mult, const double* fbar, double* ybar,
                                           double* mbar) {
    double X[NS], T, Xb[NS], Tb = 0.0;
    state_from_y(ys, X, T);
#pragma unroll
    for (int n = 0; n < NS; ++n) Xb[n] = 0.0;
    net_rhs_vjp(X, T, mult, fbar, Xb, &Tb, mbar);
    sfy_adj(ys, X, Xb, Tb, ybar);
}

// Adjoint of one accepted step y -> ynew with step h: lam (in: adjoint of ynew,
// out: adjoint of y); multiplier adjoints accumulate into mbar.
static __device__ __noinline__ void step_adj(const double* y, double h, const double* mult, double* lam,
                                             double* mbar, double* st) {
    // the step's factorised matrix, pivots and stage vectors, stored by its replay
    MatL E{st};
    const uint64_t ip = static_cast<uint64_t>(__double_as_longlong(st[kStageIp]));
    const double* k1 = st + kStageK1;
    const double* k2 = st + kStageK2;
    const double* k3 = st + kStageK3;
    double Jb[NEQ * NEQ];
    double yb[NEQ], kb1[NEQ], kb2[NEQ], r[NEQ], ys[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        yb[i] = lam[i];
        kb1[i] = kB1 * lam[i];
        kb2[i] = kB2 * lam[i];
        r[i] = lam[i];  // kb3 (b3 = 1)
    }
    const double ih = 1.0 / h;
    // stage 3: k3 = E^-1 (f(y3) + (c31 k1 + c32 k2)/h), y3 = y + a31 k1 + a32 k2
    lu_solve_t(E, ip, r);
#pragma unroll 1
    for (int a = 0; a < NEQ; ++a)
#pragma unroll 1
        for (int b = 0; b < NEQ; ++b) Jb[a * NEQ + b] = r[a] * k3[b];
    double y3b[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        kb1[i] += kC31 * ih * r[i];
        kb2[i] += kC32 * ih * r[i];
        ys[i] = y[i] + kA31 * k1[i] + kA32 * k2[i];
        y3b[i] = 0.0;
    }
    rhs_adj_at(ys, mult, r, y3b, mbar);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        yb[i] += y3b[i];
        kb1[i] += kA31 * y3b[i];
        kb2[i] += kA32 * y3b[i];
        r[i] = kb2[i];
    }
    // stage 2: k2 = E^-1 (f(y2) + (c21/h) k1), y2 = y + a21 k1
    lu_solve_t(E, ip, r);
#pragma unroll 1
    for (int a = 0; a < NEQ; ++a)
#pragma unroll 1
        for (int b = 0; b < NEQ; ++b) Jb[a * NEQ + b] += r[a] * k2[b];
    double y2b[NEQ];
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        kb1[i] += kC21 * ih * r[i];
        ys[i] = y[i] + kA21 * k1[i];
        y2b[i] = 0.0;
    }
    rhs_adj_at(ys, mult, r, y2b, mbar);
#pragma unroll
    for (int i = 0; i < NEQ; ++i) {
        yb[i] += y2b[i];
        kb1[i] += kA21 * y2b[i];
        r[i] = kb1[i];
    }
    // stage 1: k1 = E^-1 f(y)
    lu_solve_t(E, ip, r);
#pragma unroll 1
    for (int a = 0; a < NEQ; ++a)
#pragma unroll 1
        for (int b = 0; b < NEQ; ++b) Jb[a * NEQ + b] += r[a] * k1[b];
    rhs_adj_at(y, mult, r, yb, mbar);
    // E = fac I - J(y): Jbar = sum_i rbar_i k_i^T
    {
        double X[NS], T, Xb[NS], Tb = 0.0;
        state_from_y(y, X, T);
#pragma unroll
        for (int n = 0; n < NS; ++n) Xb[n] = 0.0;
        net_jac_vjp(X, T, Jb, Xb, &Tb);
        sfy_adj(y, X, Xb, Tb, yb);
    }
#pragma unroll
    for (int i = 0; i < NEQ; ++i) lam[i] = yb[i];
}

// Burn replay for the adjoint: the state at the start of every 32-step segment
// into segck, the states before each step of the last segment into ys, the
// burn's final state into y (y holds y0 on entry).
static __device__ __noinline__ void burn_checkpoint(double* y, const double* hs, int count, const double* mult,
                                                    double* segck, double* ys, double* stage) {
    const int nseg = (count + kSeg - 1) / kSeg;
    for (int g = 0; g < nseg; ++g) {
#pragma unroll
        for (int i = 0; i < NEQ; ++i) segck[g * NEQ + i] = y[i];
        const int k0 = g * kSeg;
        const int k1 = (k0 + kSeg < count) ? k0 + kSeg : count;
        for (int k = k0; k < k1; ++k) {
            // the last segment's states and step records go straight to ys and
            // stage: it is reversed first
            const bool last = g == nseg - 1;
            if (last) {
#pragma unroll
                for (int i = 0; i < NEQ; ++i) ys[(k - k0) * NEQ + i] = y[i];
            }
            step_replay(y, hs[k], mult, last ? stage + static_cast<size_t>(k - k0) * kStage : nullptr);
        }
    }
}

// Adjoint of the burn recorded by burn_checkpoint: lam in (adjoint of the final
// state) / out (adjoint of y0); each segment but the last (already in ys) is
// recomputed into ys from its checkpoint, then reversed step by step.
static __device__ __noinline__ void burn_reverse(const double* hs, int count, const double* mult, double* lam,
                                                 double* mbar, const double* segck, double* ys, double* stage) {
    const int nseg = (count + kSeg - 1) / kSeg;
    double y[NEQ];
    for (int g = nseg - 1; g >= 0; --g) {
        const int k0 = g * kSeg;
        const int k1 = (k0 + kSeg < count) ? k0 + kSeg : count;
        if (g != nseg - 1) {
#pragma unroll
            for (int i = 0; i < NEQ; ++i) y[i] = segck[g * NEQ + i];
            for (int k = k0; k < k1; ++k) {
#pragma unroll
                for (int i = 0; i < NEQ; ++i) ys[(k - k0) * NEQ + i] = y[i];
                step_replay(y, hs[k], mult, stage + static_cast<size_t>(k - k0) * kStage);
            }
        }
        for (int k = k1 - 1; k >= k0; --k)
            step_adj(ys + (k - k0) * NEQ, hs[k], mult, lam, mbar, stage + static_cast<size_t>(k - k0) * kStage);
    }
}

struct CellAdj {
    double xn[NS], T, e, rho, driver;
};

__global__ void __launch_bounds__(kThreads) k_diff_backward(Args a) {
    const int i = blockIdx.x * kThreads + threadIdx.x;
    if (i >= a.n) return;
    double* hrow = a.hbuf + static_cast<size_t>(i) * a.cap;
    double* segck = a.segck + static_cast<size_t>(i) * a.nseg * NEQ;
    double* ys = a.ys + static_cast<size_t>(i) * kSeg * NEQ;
    double* stage = a.stage + static_cast<size_t>(i) * kSeg * kStage;
    double* mbar = a.mbar + static_cast<size_t>(i) * NP;
    for (int r = 0; r < NP; ++r) mbar[r] = 0.0;
    CellAdj L;
#pragma unroll
    for (int k = 0; k < NS; ++k) L.xn[k] = a.qbar[15 * i + k];
    L.T = a.qbar[15 * i + NS];
    L.e = 0.0;
    L.rho = 0.0;
    L.driver = 0.0;
    int hend = 0;
    for (int s = 0; s < a.nsteps; ++s) hend += a.counts[static_cast<size_t>(s) * a.n + i];
    for (int s = a.nsteps - 1; s >= 0; --s) {
        const int kind = a.kind[static_cast<size_t>(s) * a.n + i];
        if (kind == 0) continue;
        const int cnt = a.counts[static_cast<size_t>(s) * a.n + i];
        const int hbeg = hend - cnt;
        // ---- recompute the step's forward pieces from its checkpoint
        CellS c0;
        load_ckpt(a, s, i, c0);
        const bool pert = a.perturb && s != 0 && s % kPerturbInterval == 0;
        const double f = pert ? perturbation_factor(i, s) : 1.0;
        CellS c1 = c0;  // after the perturbation
        double xa[NS];
        if (pert) {
            c1.driver *= f;
            c1.rho = c1.rho * f;
#pragma unroll
            for (int k = 0; k < NS; ++k) {
                c1.xn[k] *= f;
                xa[k] = c1.xn[k];
            }
            renormalize(c1.xn, c1.rho);
            c1.T = eos_T_from_e(c1.xn, c1.e);
        }
        const double dt = collapse_timestep(c1.xn);
        double rho_n = 0.0;  // density of c1.xn
#pragma unroll
        for (int k = 0; k < NS; ++k) rho_n += mass(k) * c1.xn[k];
        double lam_dt = 0.0, lam_drv1 = 0.0;
        // adjoint of the state after the step, mapped back to c1 (and dt)
        double lx1[NS], lT1 = 0.0, le1 = 0.0, lrho1 = 0.0;
        if (kind == 1) {
            // driver += dt * driver / (dt / 0.1) ; xn, T, e, rho unchanged
            const double tff = dt / kTffReduc;
            lam_drv1 = L.driver * (1.0 + dt / tff);
            lam_dt = L.driver * c1.driver * (1.0 / tff - dt / (tff * tff * kTffReduc));
#pragma unroll
            for (int k = 0; k < NS; ++k) lx1[k] = L.xn[k];
            lT1 = L.T;
            le1 = L.e;
            lrho1 = L.rho;
        } else {
            const double dtg = a.dt_hist[s];
            const double tff = dt / kTffReduc;
            // drv2 = drv1 + dtg * drv1 / tff
            double lam_drv2 = L.driver;
            double lxc[NS], lrho2 = 0.0, le2 = 0.0;
#pragma unroll
            for (int k = 0; k < NS; ++k) lxc[k] = 0.0;
            if (kind == 2) {
#pragma unroll
                for (int k = 0; k < NS; ++k) lx1[k] = L.xn[k];
                lT1 = L.T;
                le1 = L.e;
                lrho1 = L.rho;
            } else {
                // forward: c2 = c1 scaled by the driver ratio, burn, commit
                CellS c2 = c1;
                double y0[NEQ];
                advance_part(dtg, dt, c2, y0);
                const double ratio = c2.driver / c1.driver;
                double yN[NEQ];
#pragma unroll
                for (int k = 0; k < NEQ; ++k) yN[k] = y0[k];
                burn_checkpoint(yN, hrow + hbeg, cnt, a.mult, segck, ys, stage);
                // commit: xd = renormalize(yN, rho2), e3 = yN[14], T3 = eos_re(xd, e3)
                double xd[NS];
#pragma unroll
                for (int k = 0; k < NS; ++k) xd[k] = yN[k];
                renormalize(xd, c2.rho);
                double lxd[NS], le3 = L.e;
#pragma unroll
                for (int k = 0; k < NS; ++k) lxd[k] = L.xn[k];
                eos_T_adj(xd, yN[NS], L.T, lxd, le3);
                double lam[NEQ];
                lrho2 = L.rho;
                renorm_adj(yN, c2.rho, lxd, lam, lrho2);
                lam[NS] = le3;
                burn_reverse(hrow + hbeg, cnt, a.mult, lam, mbar, segck, ys, stage);
                // y0 = (xc, e2), e2 = eos_rt(xc, T1), xc = x1 * ratio, rho2 = rho1 * ratio
                double lratio = 0.0;
#pragma unroll
                for (int k = 0; k < NS; ++k) lxc[k] = lam[k];
                le2 = lam[NS];
                eos_e_adj(y0, c1.T, le2, lxc, lT1);
#pragma unroll
                for (int k = 0; k < NS; ++k) {
                    lx1[k] = lxc[k] * ratio;
                    lratio += lxc[k] * c1.xn[k];
                }
                lrho1 = lrho2 * ratio;
                lratio += lrho2 * c1.rho;
                // ratio = drv2 / drv1
                lam_drv2 += lratio / c1.driver;
                lam_drv1 -= lratio * c2.driver / (c1.driver * c1.driver);
                le1 = 0.0;  // e is recomputed from T before the burn
            }
            lam_drv1 += lam_drv2 * (1.0 + dtg / tff);
            lam_dt += lam_drv2 * (-dtg * c1.driver / (tff * tff)) / kTffReduc;
        }
        // dt = 0.1 sqrt(3 pi / (32 G rho)), rho = sum m x1
#pragma unroll
        for (int k = 0; k < NS; ++k) lx1[k] += lam_dt * (-0.5 * dt * mass(k) / rho_n);
        // ---- through the perturbation
        if (pert) {
            // T1 = eos_re(x1, e0)
            double le0 = le1;
            eos_T_adj(c1.xn, c0.e, lT1, lx1, le0);
            double lxa[NS];
            renorm_adj(xa, c1.rho, lx1, lxa, lrho1);
#pragma unroll
            for (int k = 0; k < NS; ++k) L.xn[k] = lxa[k] * f;
            L.T = 0.0;
            L.e = le0;
            L.rho = lrho1 * f;
            L.driver = lam_drv1 * f;
        } else {
#pragma unroll
            for (int k = 0; k < NS; ++k) L.xn[k] = lx1[k];
            L.T = lT1;
            L.e = le1;
            L.rho = lrho1;
            L.driver = lam_drv1;
        }
        hend = hbeg;
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) a.ubar[15 * i + k] = L.xn[k];
    a.ubar[15 * i + NS] = L.T;
}

}  // namespace diff
}  // namespace wr
