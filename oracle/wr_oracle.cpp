// ORACLE -- test infrastructure only.
//
// CPU restatement of the reference's gridwide-independent chemistry path, used as
// the checker for the GPU library.  Only the tests, __graft_entry__.smoke() and
// bench.py's CPU-baseline leg load it; the product never does.
//
// What it restates (reference file reproducer.cpp):
//   species data and EOS              :201-339
//   ROS2S integrator + LU/solve       :96-181, :7068-7347
//   collapse driver helpers           :7406-7431, :7533-7644
//   prepare / advance kernels         :7696-7785 (as host loops over cells)
//   host outer loop                   :7856-7959
// The network RHS/Jacobian comes from the project's generated header, whose
// expressions are the reference's generated code (:342-6994) with only exact
// rewrites.  Two builds exist:
//   -DWR_ORACLE_LIBM      std::exp/std::log/std::cbrt from the C library: the
//                         arithmetic of the reference CPU build.  Pinned bit for
//                         bit against the reference compiled from its sources.
//   (default)             the project's portable exp/log/cbrt (wr_math.h): the
//                         arithmetic of the GPU library's default mode.
// Compile with -ffp-contract=off: the reference's rounding sequence has no FMAs.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../include/warp_reactor.h"

#ifdef WR_ORACLE_LIBM
struct OracleMath {
    static double exp(double x) { return std::exp(x); }
    static double log(double x) { return std::log(x); }
    static double sqrt(double x) { return std::sqrt(x); }
    static double cbrt(double x) { return std::cbrt(x); }
    static double fabs(double x) { return std::fabs(x); }
    static double div(double a, double b) { return a / b; }
};
#define WR_ORACLE_MATH_NAME "libm"
#else
#include "../warp_reactor_gb300/csrc/wr_math.h"
struct OracleMath {
    static double exp(double x) { return wr_exp(x); }
    static double log(double x) { return wr_log(x); }
    static double sqrt(double x) { return std::sqrt(x); }
    static double cbrt(double x) { return wr_cbrt(x); }
    static double fabs(double x) { return std::fabs(x); }
    static double div(double a, double b) { return a / b; }
};
#define WR_ORACLE_MATH_NAME "portable"
#endif

#define WR_NET_HD inline
#include "../warp_reactor_gb300/csrc/generated/network_gen.h"

namespace {

constexpr int NS = 14;
constexpr int NEQ = 15;

// reproducer.cpp:233-248
constexpr double kMass[NS] = {
    9.10938188e-28,   1.67262158e-24,   1.67353251819e-24, 1.67444345638e-24,
    3.34512158e-24,   3.34603251819e-24, 3.34615409819e-24, 3.34694345638e-24,
    3.34706503638e-24, 5.01865409819e-24, 5.01956503638e-24, 6.69024316e-24,
    6.69115409819e-24, 6.69206503638e-24};
// reproducer.cpp:250-252
constexpr double gamma_of(int n) { return (n == 6 || n == 8 || n == 9 || n == 10) ? 1.4 : 5.0 / 3.0; }
// reproducer.cpp:207-211
constexpr double kNA = 6.02214076e+23;
constexpr double kKB = 1.3806490000000002e-16;
constexpr double kMp = 1.67262192595e-24;
constexpr double kFloor = 1.0e-100;          // :231
constexpr double kGrav = 6.674e-8;           // :203
constexpr double kPi = 3.141592653589793238462643383279502884;  // :204
// reproducer.cpp:7406-7431
constexpr double kTffReduc = 1.0e-1;
constexpr int kMaxCollapseSteps = 1000;
constexpr double kInitialT = 1.0e2;
constexpr double kRtolSpec = 1.0e-4, kAtolSpec = 1.0e-4;
constexpr double kRtolEnergy = 1.0e-6, kAtolEnergy = 1.0e-6;
constexpr int kPerturbInterval = 20;
constexpr double kPerturbAmplitude = 0.2;
constexpr double kInitialXn[NS] = {1.0e-4, 1.0e-4, 1.0e0,  1.0e-40, 1.0e-40, 1.0e-40, 1.0e-40,
                                   1.0e-40, 1.0e-6, 1.0e-40, 1.0e-40, 1.0e-40, 1.0e-40, 0.0775};

// std::max / std::min semantics (first argument wins ties and NaN comparisons)
inline double smax(double a, double b) { return (a < b) ? b : a; }
inline double smin(double a, double b) { return (b < a) ? b : a; }

struct Burn {  // burn_t, reproducer.cpp:263-268
    double rho, T, e;
    double xn[NS];
};

// reproducer.cpp:270-276
double density(const double* xn) {
    double rho = 0.0;
    for (int n = 0; n < NS; ++n) rho += xn[n] * kMass[n];
    return rho;
}

struct EosSums { double sum_abarinv, sum_gammasinv, gasconstant; };

// reproducer.cpp:284-304
EosSums eos_sums(const double* xn) {
    const double gasconstant = kNA * kKB;
    double sum_abarinv = 0.0, sum_gammasinv = 0.0, rhotot = 0.0;
    for (int n = 0; n < NS; ++n) rhotot += xn[n] * kMass[n];
    for (int n = 0; n < NS; ++n) {
        sum_abarinv += xn[n];
        sum_gammasinv += (xn[n] * kMp / rhotot) * (1.0 / (gamma_of(n) - 1.0));
    }
    sum_abarinv *= kMp / rhotot;
    sum_gammasinv /= sum_abarinv;
    return {sum_abarinv, sum_gammasinv, gasconstant};
}

// reproducer.cpp:306-314
void eos_rt(Burn& s) {
    const EosSums q = eos_sums(s.xn);
    s.e = q.sum_gammasinv * q.sum_abarinv * q.gasconstant * s.T;
}
void eos_re(Burn& s) {
    const EosSums q = eos_sums(s.xn);
    s.T = s.e / (q.sum_gammasinv * q.gasconstant * q.sum_abarinv);
}

// reproducer.cpp:316-319
void balance_charge(Burn& s) {
    s.xn[0] = -s.xn[3] - s.xn[7] + s.xn[1] + s.xn[12] + s.xn[6] + s.xn[4] + s.xn[9] + 2.0 * s.xn[11];
}

// reproducer.cpp:321-339
void floor_and_normalize(Burn& s) {
    for (double& x : s.xn) x = smax(x, kFloor);
    double mf[NS];
    double sum = 0.0;
    for (int n = 0; n < NS; ++n) {
        mf[n] = kMass[n] * s.xn[n] / s.rho;
        sum += mf[n];
    }
    for (int n = 0; n < NS; ++n) {
        mf[n] /= sum;
        s.xn[n] = mf[n] * s.rho / kMass[n];
    }
}

// PrimordialChem::burn_state_from_y, reproducer.cpp:7029-7038: floored X and T
void state_from_y(const double* y, double* X, double& T) {
    Burn s;
    for (int n = 0; n < NS; ++n) s.xn[n] = smax(y[n], kFloor);
    s.e = y[NS];
    eos_re(s);
    for (int n = 0; n < NS; ++n) X[n] = s.xn[n];
    T = s.T;
}

// PrimordialChem::rhs, reproducer.cpp:7040-7050
void rhs(const double* y, double* dydt) {
    double X[NS], T;
    state_from_y(y, X, T);
    wr_net_rhs<OracleMath>(X, T, dydt);
}

struct MatSink {
    double (*J)[NEQ];
    void operator()(int r, int c, double v) { J[r][c] = v; }
};

// PrimordialChem::jacobian, reproducer.cpp:7052-7060 (the RHS at the same state is
// produced by the same fused evaluation and discarded here)
void jacobian(const double* y, double J[NEQ][NEQ]) {
    double X[NS], T, f[NEQ];
    state_from_y(y, X, T);
    MatSink sink{J};
    wr_net_jac_rhs<OracleMath>(X, T, f, sink);
}

// lu_decomposition<15>, reproducer.cpp:96-151
int lu_decomposition(double A[NEQ][NEQ], int* ipvt) {
    int info = 0;
    for (int k = 0; k < NEQ - 1; ++k) {
        int p = k;
        double max_val = std::fabs(A[k][k]);
        for (int i = k + 1; i < NEQ; ++i) {
            const double v = std::fabs(A[i][k]);
            if (v > max_val) { max_val = v; p = i; }
        }
        ipvt[k] = p;
        if (A[p][k] != 0.0) {
            if (p != k) {
                const double t = A[p][k]; A[p][k] = A[k][k]; A[k][k] = t;
                for (int j = k + 1; j < NEQ; ++j) {
                    const double tr = A[p][j]; A[p][j] = A[k][j]; A[k][j] = tr;
                }
            }
            const double mult = -1.0 / A[k][k];
            for (int i = k + 1; i < NEQ; ++i) A[i][k] *= mult;
            for (int j = k + 1; j < NEQ; ++j) {
                const double t = A[k][j];
                for (int i = k + 1; i < NEQ; ++i) A[i][j] += t * A[i][k];
            }
        } else {
            info = k + 1;
        }
    }
    ipvt[NEQ - 1] = NEQ - 1;
    if (A[NEQ - 1][NEQ - 1] == 0.0) info = NEQ;
    return info;
}

// lu_solve<15>, reproducer.cpp:154-181
void lu_solve(const double LU[NEQ][NEQ], const int* ipvt, double* x) {
    for (int k = 0; k < NEQ - 1; ++k) {
        const int p = ipvt[k];
        const double t = x[p];
        if (p != k) { x[p] = x[k]; x[k] = t; }
        for (int j = k + 1; j < NEQ; ++j) x[j] += t * LU[j][k];
    }
    for (int kb = 0; kb < NEQ; ++kb) {
        const int k = NEQ - 1 - kb;
        x[k] /= LU[k][k];
        const double t = -x[k];
        for (int j = 0; j < k; ++j) x[j] += t * LU[j][k];
    }
}

// ROS2SCoefficients, reproducer.cpp:7113-7128
constexpr double kGamma = 0.292893218813452;
constexpr double kCt2 = 0.585786437626905;
constexpr double kA21 = 2.0000000000000036;
constexpr double kA31 = 6.828427124746214;
constexpr double kA32 = 3.4142135623731007;
constexpr double kC21 = -6.828427124746214;
constexpr double kC31 = -10.949747468305889;
constexpr double kC32 = -7.535533905932761;
constexpr double kB1 = 6.828427124746214;
constexpr double kB2 = 3.414213562373101;
constexpr double kB3 = 1.0;
constexpr double kE1 = -0.23570226039551292;
constexpr double kE2 = -0.23570226039551567;
constexpr double kE3 = -0.13807118745769906;

struct Counters { int n_step = 0, n_rhs = 0, n_jac = 0, n_accept = 0, n_reject = 0, n_decomp = 0, n_solve = 0; };

// ---------------------------------------------------------------- precision form
// WR_ORACLE_PREC (compile-time, default 0 = plain FP64): the precision form's
// linear algebra restated from the device kernel (advance variant 3).
//  2  the precision form (libwr_oracle_prec.so): the iteration matrix in
//     error-weighted variables, E' = W^-1 E W with W = diag(atol + rtol |y|) (the
//     scale of the controller's error norm, reproducer.cpp:7194-7202), rounded to
//     FP32 and factorised in FP32 (fmaf updates); each stage solve is
//     x0 = W LU32^-1 W^-1 b followed by WR_ORACLE_PREC_SWEEPS (default 1) FP64
//     residual sweeps r = b - E x0 (E = fac I - J in FP64), x0 += W LU32^-1 W^-1 r;
//  1  the same without the weights (W = I): the unscaled variant, kept to
//     reproduce the measurement that motivated the weights.
#ifndef WR_ORACLE_PREC
#define WR_ORACLE_PREC 0
#endif
#ifndef WR_ORACLE_PREC_SWEEPS
#define WR_ORACLE_PREC_SWEEPS 1
#endif
#if WR_ORACLE_PREC
int lu_decomposition_f32(float A[NEQ][NEQ], int* ipvt) {
    int info = 0;
    for (int k = 0; k < NEQ - 1; ++k) {
        int p = k;
        float max_val = std::fabs(A[k][k]);
        for (int i = k + 1; i < NEQ; ++i) {
            const float v = std::fabs(A[i][k]);
            if (v > max_val) { max_val = v; p = i; }
        }
        ipvt[k] = p;
        if (A[p][k] != 0.0f) {
            if (p != k)
                for (int j = k; j < NEQ; ++j) { const float t = A[p][j]; A[p][j] = A[k][j]; A[k][j] = t; }
            const float mult = -1.0f / A[k][k];
            for (int i = k + 1; i < NEQ; ++i) A[i][k] = A[i][k] * mult;
            for (int j = k + 1; j < NEQ; ++j) {
                const float t = A[k][j];
                for (int i = k + 1; i < NEQ; ++i) A[i][j] = std::fmaf(t, A[i][k], A[i][j]);
            }
        } else {
            info = k + 1;
        }
    }
    ipvt[NEQ - 1] = NEQ - 1;
    if (A[NEQ - 1][NEQ - 1] == 0.0f) info = NEQ;
    return info;
}

void lu_solve_f32(const float LU[NEQ][NEQ], const int* ipvt, float* x) {
    for (int k = 0; k < NEQ - 1; ++k) {
        const int p = ipvt[k];
        const float t = x[p];
        if (p != k) { x[p] = x[k]; x[k] = t; }
        for (int j = k + 1; j < NEQ; ++j) x[j] = std::fmaf(t, LU[j][k], x[j]);
    }
    for (int kb = 0; kb < NEQ; ++kb) {
        const int k = NEQ - 1 - kb;
        x[k] = x[k] / LU[k][k];
        const float t = -x[k];
        for (int j = 0; j < k; ++j) x[j] = std::fmaf(t, LU[j][k], x[j]);
    }
}

// x <- E^-1 x (E = fac I - J) with the FP32 factors of W^-1 E W (W = I in mode 1)
void solve_refined(const float LU[NEQ][NEQ], const int* ip, const double J[NEQ][NEQ], double fac,
                   const double* w, double* x) {
    double b[NEQ], xx[NEQ];
    for (int i = 0; i < NEQ; ++i) b[i] = x[i];
    float xf[NEQ];
    for (int i = 0; i < NEQ; ++i) xf[i] = static_cast<float>(b[i] / w[i]);
    lu_solve_f32(LU, ip, xf);
    for (int i = 0; i < NEQ; ++i) xx[i] = static_cast<double>(xf[i]) * w[i];
    for (int sweep = 0; sweep < WR_ORACLE_PREC_SWEEPS; ++sweep) {
        for (int i = 0; i < NEQ; ++i) {
            double acc = 0.0;
            for (int j = 0; j < NEQ; ++j) acc = acc + J[i][j] * xx[j];
            xf[i] = static_cast<float>((b[i] - (fac * xx[i] - acc)) / w[i]);
        }
        lu_solve_f32(LU, ip, xf);
        for (int i = 0; i < NEQ; ++i) xx[i] = xx[i] + static_cast<double>(xf[i]) * w[i];
    }
    for (int i = 0; i < NEQ; ++i) x[i] = xx[i];
}
#endif

// RODAS<PrimordialChem>::integrate with configure_ros2s settings
// (reproducer.cpp:7205-7347, 7582-7590, RODASState defaults :7077-7109).
// y: in/out 15-vector; t from 0 to tout; returns IntegratorResult.
int ros2s_integrate(double* y, double tout, double dt0, Counters& c) {
    const double t0 = 0.0;
    const double uround = 1.e-16, fac_min = 0.2, fac_max = 6.0, safe = 0.9;
    const int max_steps = 10000000;
    double rtol[NEQ], atol[NEQ];
    for (int n = 0; n < NS; ++n) { rtol[n] = kRtolSpec; atol[n] = kAtolSpec; }
    rtol[NS] = kRtolEnergy; atol[NS] = kAtolEnergy;

    if (tout <= t0) return WR_BAD_INPUTS;
    const double hmaxn = tout - t0;
    double h = dt0;
    if (std::fabs(h) <= 10.0 * uround) h = 1.e-6;
    h = smin(std::fabs(h), hmaxn);

    bool reject = false, last = false;
    int nsing = 0;
    double hacc = 0.0, erracc = 1.0, hopt = h, x = t0;
    int n_step = 0, n_accept = 0;
    double fjac[NEQ][NEQ], e[NEQ][NEQ];
    int ip[NEQ];
#if WR_ORACLE_PREC
    float e32[NEQ][NEQ];
    double wsc[NEQ];
#define WR_SOLVE(v) solve_refined(e32, ip, fjac, fac, wsc, v)
#else
#define WR_SOLVE(v) lu_solve(e, ip, v)
#endif
    double ynew[NEQ], ak1[NEQ], ak2[NEQ], work[NEQ], dy[NEQ];

    for (;;) {
        if (n_step > max_steps) return WR_TOO_MANY_STEPS;
        if (0.1 * std::fabs(h) <= std::fabs(x) * uround) return WR_DT_UNDERFLOW;
        if (last) return WR_SUCCESS;
        hopt = h;
        if (x + h * 1.0001 >= tout) { h = tout - x; last = true; }
        jacobian(y, fjac);
        c.n_jac += 1;
        for (;;) {
            const double fac = 1.0 / (h * kGamma);
            for (int i = 0; i < NEQ; ++i) {
                for (int j = 0; j < NEQ; ++j) e[i][j] = -fjac[i][j];
                e[i][i] += fac;
            }
#if WR_ORACLE_PREC
            for (int i = 0; i < NEQ; ++i) wsc[i] = WR_ORACLE_PREC == 2 ? atol[i] + rtol[i] * std::fabs(y[i]) : 1.0;
            for (int i = 0; i < NEQ; ++i)
                for (int j = 0; j < NEQ; ++j) e32[i][j] = static_cast<float>(e[i][j] * wsc[j] / wsc[i]);
            const int info = lu_decomposition_f32(e32, ip);
#else
            const int info = lu_decomposition(e, ip);
#endif
            if (info != 0) {
                nsing += 1;
                if (nsing >= 5) return WR_LU_DECOMPOSITION_ERROR;
                h *= 0.5;
                reject = true;
                last = false;
                continue;
            }
            c.n_decomp += 1;
            rhs(y, ak1);
            WR_SOLVE(ak1);
            c.n_solve += 1;
            for (int i = 0; i < NEQ; ++i) {
                ynew[i] = y[i] + kA21 * ak1[i];
                ak2[i] = (kC21 / h) * ak1[i];
            }
            rhs(ynew, dy);
            for (int i = 0; i < NEQ; ++i) ak2[i] += dy[i];
            WR_SOLVE(ak2);
            c.n_solve += 1;
            for (int i = 0; i < NEQ; ++i) {
                ynew[i] = y[i] + kA31 * ak1[i] + kA32 * ak2[i];
                work[i] = (kC31 * ak1[i] + kC32 * ak2[i]) / h;
            }
            rhs(ynew, dy);
            for (int i = 0; i < NEQ; ++i) work[i] += dy[i];
            WR_SOLVE(work);
            c.n_solve += 1;
            for (int i = 0; i < NEQ; ++i) {
                const double ak3 = work[i];
                ynew[i] = y[i] + kB1 * ak1[i] + kB2 * ak2[i] + kB3 * ak3;
                work[i] = kE1 * ak1[i] + kE2 * ak2[i] + kE3 * ak3;
            }
            c.n_rhs += 3;
            n_step += 1;
            c.n_step = n_step;
            double err = 0.0;  // error_norm, reproducer.cpp:7194-7202
            for (int i = 0; i < NEQ; ++i) {
                const double sk = atol[i] + rtol[i] * smax(std::fabs(y[i]), std::fabs(ynew[i]));
                const double term = work[i] / sk;
                err += term * term;
            }
            err = std::sqrt(err / static_cast<double>(NEQ));
            const double raw_fac = OracleMath::cbrt(err) / safe;
            const double lower_fac = 1.0 / fac_max;
            const double upper_fac = 1.0 / fac_min;
            const double fac_step = smax(lower_fac, smin(upper_fac, raw_fac));
            double hnew = h / fac_step;
            if (err <= 1.0) {
                n_accept += 1;
                c.n_accept = n_accept;
                if (n_accept > 1) {
                    const double facgus = smax(1.0 / fac_max,
                        smin(1.0 / fac_min, (hacc / h) * OracleMath::cbrt((err * err) / erracc) / safe));
                    hnew = h / smax(fac_step, facgus);
                }
                hacc = h;
                erracc = smax(1.e-2, err);
                for (int i = 0; i < NEQ; ++i) y[i] = ynew[i];
                x += h;
                if (std::fabs(hnew) > hmaxn) hnew = hmaxn;
                if (reject) hnew = smin(std::fabs(hnew), std::fabs(h));
                reject = false;
                h = hnew;
                break;
            }
            reject = true;
            last = false;
            h = hnew;
            if (n_accept >= 1) c.n_reject += 1;
            // the reject loop has no exit of its own: a step size that underflowed
            // to zero ends the burn with DT_UNDERFLOW (the GPU library does the same)
            if (hnew == 0.0) return WR_DT_UNDERFLOW;
        }
    }
}

// burn_ros2s, reproducer.cpp:7592-7627
int burn_ros2s(Burn& s, double dt, wr_integrator_stats& st) {
    eos_rt(s);
    double y[NEQ];
    for (int n = 0; n < NS; ++n) y[n] = s.xn[n];
    y[NS] = s.e;
    Counters c;
    const int r = ros2s_integrate(y, dt, dt, c);
    st.internal_steps += static_cast<uint64_t>(c.n_step > 0 ? c.n_step : 0);
    st.rhs_calls += static_cast<uint64_t>(c.n_rhs > 0 ? c.n_rhs : 0);
    st.jacobian_calls += static_cast<uint64_t>(c.n_jac > 0 ? c.n_jac : 0);
    st.decompositions += static_cast<uint64_t>(c.n_decomp > 0 ? c.n_decomp : 0);
    st.linear_solves += static_cast<uint64_t>(c.n_solve > 0 ? c.n_solve : 0);
    st.accepted_steps += static_cast<uint64_t>(c.n_accept > 0 ? c.n_accept : 0);
    st.rejected_steps += static_cast<uint64_t>(c.n_reject > 0 ? c.n_reject : 0);
    if (r != WR_SUCCESS) return r;
    for (int n = 0; n < NS; ++n) s.xn[n] = y[n];
    s.e = y[NS];
    return r;
}

Burn load(const wr_collapse_state& c) {
    Burn s;
    s.rho = c.rho; s.T = c.T; s.e = c.e;
    for (int n = 0; n < NS; ++n) s.xn[n] = c.xn[n];
    return s;
}
void store(wr_collapse_state& c, const Burn& s) {
    c.rho = s.rho; c.T = s.T; c.e = s.e;
    for (int n = 0; n < NS; ++n) c.xn[n] = s.xn[n];
}

// splitmix64 / perturbation_factor / apply_perturbation, reproducer.cpp:7548-7580
uint64_t splitmix64(uint64_t v) {
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30U)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27U)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31U);
}
double perturbation_factor(int cell, int step) {
    const uint64_t seed = (static_cast<uint64_t>(static_cast<unsigned int>(cell)) << 32U) ^
                          (static_cast<uint64_t>(static_cast<unsigned int>(step)) << 16U);
    const uint64_t bits = splitmix64(seed) >> 11U;
    const double unit = static_cast<double>(bits) * (1.0 / static_cast<double>(1ULL << 53U));
    return 1.0 + kPerturbAmplitude * (2.0 * unit - 1.0);
}
void apply_perturbation(wr_collapse_state& c, int cell, int step, bool enabled) {
    if (!enabled || step == 0 || step % kPerturbInterval != 0) return;
    const double factor = perturbation_factor(cell, step);
    c.density_driver *= factor;
    Burn s = load(c);
    s.rho *= factor;
    for (double& x : s.xn) x *= factor;
    floor_and_normalize(s);
    balance_charge(s);
    floor_and_normalize(s);
    eos_re(s);
    store(c, s);
}

bool valid_positive(double v) { return v > 0.0 && std::isfinite(v); }  // :7629

// collapse_timestep, reproducer.cpp:7633-7644
double collapse_timestep(const wr_collapse_state& c) {
    const double rho = density(c.xn);
    if (!valid_positive(rho)) return -1.0;
    const double tff = std::sqrt(kPi * 3.0 / (32.0 * rho * kGrav));
    if (!valid_positive(tff)) return -1.0;
    const double dt = kTffReduc * tff;
    return valid_positive(dt) ? dt : -1.0;
}

void record_failure(std::atomic<int>& code, int value) {
    int expected = WR_SUCCESS;
    code.compare_exchange_strong(expected, value);
}

// prepare_grid_timestep_kernel, reproducer.cpp:7696-7734, for one cell
void prepare_cell(wr_collapse_state& st, int cell, int cgs, double grid_time, int step,
                  bool perturb, double& candidate, std::atomic<int>& failure) {
    candidate = DBL_MAX;
    if (failure.load() != WR_SUCCESS) return;
    if (st.completed_steps < cgs) return;
    if (st.completed_steps != cgs || st.time != grid_time) {
        record_failure(failure, WR_BAD_INPUTS);
        return;
    }
    apply_perturbation(st, cell, step, perturb);
    const double dt = collapse_timestep(st);
    if (!valid_positive(dt) || !valid_positive(st.density_driver)) {
        record_failure(failure, WR_BAD_INPUTS);
        return;
    }
    if (dt < 10.0) {
        const double tff = dt / kTffReduc;
        st.density_driver += dt * (st.density_driver / tff);
        return;
    }
    candidate = dt;
}

// advance_collapse_gridwide_kernel, reproducer.cpp:7736-7785, for one cell
int advance_cell(wr_collapse_state& st, int cgs, double next_grid_time, double dt_grid,
                 std::atomic<int>& failure) {
    if (failure.load() != WR_SUCCESS) return 0;
    if (st.completed_steps != cgs) return 0;
    const double local_dt = collapse_timestep(st);
    if (local_dt < 10.0) return 0;
    const double old_density = st.density_driver;
    const double tff = local_dt / kTffReduc;
    st.density_driver += dt_grid * (st.density_driver / tff);
    if (!valid_positive(st.density_driver) || st.density_driver > 2.0e-6) return 0;
    const double ratio = st.density_driver / old_density;
    Burn s = load(st);
    for (double& x : s.xn) x *= ratio;
    s.rho *= ratio;
    const int r = burn_ros2s(s, dt_grid, st.stats);
    if (r != WR_SUCCESS) {
        // the reference kernel keeps the pre-burn scaling of xn/rho in the cell
        // (burn_ros2s returns before copying y back; eos_rt has updated e)
        store(st, s);
        record_failure(failure, r);
        return 0;
    }
    floor_and_normalize(s);
    balance_charge(s);
    floor_and_normalize(s);
    eos_re(s);
    store(st, s);
    st.time = next_grid_time;
    st.completed_steps = cgs + 1;
    return 1;
}

// advance_collapse_step (legacy-local policy), reproducer.cpp:7646-7685: the cell's
// own free-fall dt; returns true when the cell stops (dt < 10 s or density limit)
bool legacy_step(wr_collapse_state& st, int cell, int step, bool perturb, int& failure) {
    apply_perturbation(st, cell, step, perturb);
    const double old_density = st.density_driver;
    const double dt = collapse_timestep(st);
    const double tff = dt / kTffReduc;
    st.density_driver += dt * (st.density_driver / tff);
    if (dt < 10.0 || st.density_driver > 2.0e-6) return true;
    const double ratio = st.density_driver / old_density;
    Burn s = load(st);
    for (double& x : s.xn) x *= ratio;
    s.rho *= ratio;
    const int r = burn_ros2s(s, dt, st.stats);
    if (r != WR_SUCCESS) {
        store(st, s);
        failure = r;
        return true;
    }
    floor_and_normalize(s);
    balance_charge(s);
    floor_and_normalize(s);
    eos_re(s);
    store(st, s);
    st.time += dt;
    st.completed_steps += 1;
    return false;
}

// ---------------------------------------------------------------- gridwide-cta32
// advance_collapse_gridwide_structured_kernel (structured_cuda.cuh:393-782), for
// one 32-cell tile: the per-cell prologue (:410-450), then ONE ROS2S controller for
// the tile (:468-733): a common step h, the tile error = max over participating
// cells of their error norms (non-finite -> DBL_MAX, :676-688), the Jacobian kept
// across rejected trials (:496-561), the step-size rules of :689-733, and the
// commit of :737-768.  Returns the number of cells integrated (0 on failure).
constexpr int kTile = 32;

double cbrt_nonnegative(double v) {  // structured_cuda.cuh:88-93
    if (v == 0.0) return 0.0;
    return OracleMath::exp(OracleMath::log(v) / 3.0);
}

int advance_tile(wr_collapse_state* cells, int tile_begin, int active, int cgs, double grid_time,
                 double next_grid_time, double dt_grid, std::atomic<int>& failure) {
    bool part[kTile] = {false};
    double base[kTile][NEQ];
    int count = 0;
    for (int t = 0; t < active; ++t) {
        wr_collapse_state& c = cells[tile_begin + t];
        if (c.completed_steps == cgs) {
            if (c.time != grid_time) {
                record_failure(failure, WR_BAD_INPUTS);
            } else {
                const double local_dt = collapse_timestep(c);
                if (local_dt >= 10.0) {
                    const double old_density = c.density_driver;
                    c.density_driver += (dt_grid * c.density_driver) / (local_dt / kTffReduc);
                    if (valid_positive(c.density_driver) && c.density_driver <= 2.0e-6) {
                        const double ratio = c.density_driver / old_density;
                        Burn s = load(c);
                        for (double& x : s.xn) x *= ratio;
                        s.rho *= ratio;
                        eos_rt(s);
                        store(c, s);
                        part[t] = true;
                        ++count;
                    }
                }
            }
        }
        for (int k = 0; k < NS; ++k) base[t][k] = c.xn[k];
        base[t][NS] = c.e;
    }
    if (count == 0) return 0;
    const double uround = 1.0e-16, fac_min = 0.2, fac_max = 6.0, safe = 0.9;
    const int max_steps = 10000000;
    double h = dt_grid, x = 0.0, hacc = 0.0, erracc = 1.0;
    bool reject = false, jac_valid = false;
    int nsing = 0, n_step = 0, n_accept = 0, n_jac = 0, n_rej = 0;
    int status = WR_SUCCESS;
    static thread_local double J[kTile][NEQ][NEQ];
    double f0[kTile][NEQ];
    while (true) {
        if (x >= dt_grid || status != WR_SUCCESS) break;
        if (n_step > max_steps) { status = WR_TOO_MANY_STEPS; continue; }
        if (0.1 * std::fabs(h) <= std::fabs(x) * uround) { status = WR_DT_UNDERFLOW; continue; }
        bool final_trial = false;
        if (x + h * 1.0001 >= dt_grid) {
            h = dt_grid - x;
            final_trial = true;
        }
        bool singular = false;
        double err_cell[kTile], cand[kTile][NEQ];
        for (int t = 0; t < active; ++t) {
            if (!part[t]) continue;
            if (!jac_valid) {
                double Xs[NS], T;
                state_from_y(base[t], Xs, T);
                MatSink sink{J[t]};
                wr_net_jac_rhs<OracleMath>(Xs, T, f0[t], sink);
            }
            double e[NEQ][NEQ];
            int ip[NEQ];
            for (int i = 0; i < NEQ; ++i) {
                for (int j = 0; j < NEQ; ++j) e[i][j] = -J[t][i][j];
                e[i][i] += 1.0 / (h * kGamma);
            }
            if (lu_decomposition(e, ip) != 0) { singular = true; continue; }
            double k1[NEQ], k2[NEQ], w[NEQ], ys[NEQ], dy[NEQ];
            for (int i = 0; i < NEQ; ++i) k1[i] = f0[t][i];
            lu_solve(e, ip, k1);
            for (int i = 0; i < NEQ; ++i) {
                ys[i] = base[t][i] + kA21 * k1[i];
                k2[i] = (kC21 / h) * k1[i];
            }
            rhs(ys, dy);
            for (int i = 0; i < NEQ; ++i) k2[i] = dy[i] + k2[i];
            lu_solve(e, ip, k2);
            for (int i = 0; i < NEQ; ++i) {
                ys[i] = base[t][i] + kA31 * k1[i] + kA32 * k2[i];
                w[i] = (kC31 * k1[i] + kC32 * k2[i]) / h;
            }
            rhs(ys, dy);
            for (int i = 0; i < NEQ; ++i) w[i] = dy[i] + w[i];
            lu_solve(e, ip, w);
            double sum = 0.0;
            for (int i = 0; i < NEQ; ++i) {
                const double k3 = w[i];
                cand[t][i] = base[t][i] + kB1 * k1[i] + kB2 * k2[i] + k3;
                const double est = kE1 * k1[i] + kE2 * k2[i] + kE3 * k3;
                const double rtol = i == NS ? kRtolEnergy : kRtolSpec;
                const double atol = i == NS ? kAtolEnergy : kAtolSpec;
                const double scale = atol + rtol * std::fmax(std::fabs(base[t][i]), std::fabs(cand[t][i]));
                const double term = est / scale;
                sum += term * term;
            }
            err_cell[t] = std::sqrt(sum / static_cast<double>(NEQ));
        }
        if (!jac_valid) n_jac += 1;
        jac_valid = true;
        if (singular) {
            ++nsing;
            if (nsing >= 5) status = WR_LU_DECOMPOSITION_ERROR;
            else { h *= 0.5; reject = true; }
            continue;
        }
        double err_tile = 0.0;
        for (int t = 0; t < active; ++t) {
            if (!part[t]) continue;
            double e = err_cell[t];
            if (!std::isfinite(e)) e = DBL_MAX;
            err_tile = std::fmax(err_tile, e);
        }
        ++n_step;
        const double fac_step = std::fmax(1.0 / fac_max, std::fmin(1.0 / fac_min, cbrt_nonnegative(err_tile) / safe));
        double hnew = h / fac_step;
        if (err_tile <= 1.0) {
            ++n_accept;
            if (n_accept > 1) {
                const double facgus = std::fmax(1.0 / fac_max, std::fmin(1.0 / fac_min,
                    (hacc / h) * cbrt_nonnegative((err_tile * err_tile) / erracc) / safe));
                hnew = h / std::fmax(fac_step, facgus);
            }
            for (int t = 0; t < active; ++t)
                if (part[t]) for (int i = 0; i < NEQ; ++i) base[t][i] = cand[t][i];
            hacc = h;
            erracc = std::fmax(1.0e-2, err_tile);
            x = final_trial ? dt_grid : x + h;
            hnew = std::fmin(std::fabs(hnew), dt_grid);
            if (reject) hnew = std::fmin(hnew, std::fabs(h));
            reject = false;
            h = hnew;
            jac_valid = false;
        } else {
            if (n_accept >= 1) ++n_rej;
            reject = true;
            h = hnew;
        }
    }
    if (status != WR_SUCCESS) {
        record_failure(failure, status);
        return 0;
    }
    for (int t = 0; t < active; ++t) {
        if (!part[t]) continue;
        wr_collapse_state& c = cells[tile_begin + t];
        Burn s = load(c);
        for (int k = 0; k < NS; ++k) s.xn[k] = base[t][k];
        s.e = base[t][NS];
        floor_and_normalize(s);
        balance_charge(s);
        floor_and_normalize(s);
        eos_re(s);
        store(c, s);
        c.time = next_grid_time;
        c.completed_steps = cgs + 1;
        c.stats.internal_steps += static_cast<uint64_t>(n_step);
        c.stats.rhs_calls += static_cast<uint64_t>(3 * n_step);
        c.stats.jacobian_calls += static_cast<uint64_t>(n_jac);
        c.stats.decompositions += static_cast<uint64_t>(n_step);
        c.stats.linear_solves += static_cast<uint64_t>(3 * n_step);
        c.stats.accepted_steps += static_cast<uint64_t>(n_accept);
        c.stats.rejected_steps += static_cast<uint64_t>(n_rej);
    }
    return count;
}

}  // namespace

extern "C" {

const char* wro_math_name(void) { return WR_ORACLE_MATH_NAME; }

// make_initial_state / make_collapse_state, reproducer.cpp:7533-7546
void wro_make_collapse_state(wr_collapse_state* out) {
    Burn s;
    s.T = kInitialT;
    for (int n = 0; n < NS; ++n) s.xn[n] = kInitialXn[n];
    s.rho = density(s.xn);
    // normalize_number_densities_to_density (:321-332) without the floor
    double mf[NS];
    double sum = 0.0;
    for (int n = 0; n < NS; ++n) { mf[n] = kMass[n] * s.xn[n] / s.rho; sum += mf[n]; }
    for (int n = 0; n < NS; ++n) { mf[n] /= sum; s.xn[n] = mf[n] * s.rho / kMass[n]; }
    eos_rt(s);
    std::memset(out, 0, sizeof(*out));
    store(*out, s);
    out->time = 0.0;
    out->density_driver = s.rho;
    out->completed_steps = 0;
}

void wro_rhs(const double* y, double* dydt) { rhs(y, dydt); }

void wro_jac(const double* y, double* J) {
    double M[NEQ][NEQ];
    jacobian(y, M);
    std::memcpy(J, M, sizeof(M));
}

// Raw network at a given (X, T): no flooring, no EOS.
void wro_net_rhs(const double* X, double T, double* f) { wr_net_rhs<OracleMath>(X, T, f); }
void wro_net_jac(const double* X, double T, double* J, double* f) {
    double M[NEQ][NEQ];
    MatSink sink{M};
    wr_net_jac_rhs<OracleMath>(X, T, f, sink);
    std::memcpy(J, M, sizeof(M));
}

int wro_lu(double* A, int* ipvt) {
    double M[NEQ][NEQ];
    std::memcpy(M, A, sizeof(M));
    const int info = lu_decomposition(M, ipvt);
    std::memcpy(A, M, sizeof(M));
    return info;
}

void wro_lu_solve(const double* LU, const int* ipvt, double* x) {
    double M[NEQ][NEQ];
    std::memcpy(M, LU, sizeof(M));
    lu_solve(M, ipvt, x);
}

double wro_exp(double x) { return OracleMath::exp(x); }
double wro_log(double x) { return OracleMath::log(x); }
double wro_cbrt(double x) { return OracleMath::cbrt(x); }
#ifndef WR_ORACLE_LIBM
double wro_div_int(double a, double b) { return wr_div_int(a, b); }
#endif

// burn_ros2s on one cell's burn state, stats accumulated into cell->stats
int wro_burn(wr_collapse_state* cell, double dt) {
    Burn s = load(*cell);
    const int r = burn_ros2s(s, dt, cell->stats);
    store(*cell, s);
    return r;
}

int wro_prepare(wr_collapse_state* cells, int n, int cgs, double grid_time, int step,
                int perturb, double* dt_grid_out, int nthreads) {
    std::atomic<int> failure{WR_SUCCESS};
    double* cand = new double[n > 0 ? n : 1];
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < n; ++i)
        prepare_cell(cells[i], i, cgs, grid_time, step, perturb != 0, cand[i], failure);
    double dt_grid = DBL_MAX;  // host min, reproducer.cpp:7888-7893
    for (int i = 0; i < n; ++i)
        if (cand[i] < dt_grid) dt_grid = cand[i];
    delete[] cand;
    *dt_grid_out = dt_grid;
    return failure.load();
}

int wro_advance(wr_collapse_state* cells, int n, int cgs, double next_grid_time,
                double dt_grid, int* integrated, int nthreads) {
    std::atomic<int> failure{WR_SUCCESS};
    int count = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : count) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < n; ++i) count += advance_cell(cells[i], cgs, next_grid_time, dt_grid, failure);
    *integrated = count;
    return failure.load();
}

// Host outer loop, reproducer.cpp:7856-7959 (grid_time starts at 0, steps count
// from 0, *cgs is the completed_global_steps in/out argument).  max_steps < 0 runs
// the reference's 1000 steps; a smaller positive value stops early (tests).
int wro_run(wr_collapse_state* cells, int n, int perturb, int* cgs, int max_steps, int nthreads) {
    int result = WR_SUCCESS;
    double grid_time = 0.0;
    const int steps = max_steps > 0 ? max_steps : kMaxCollapseSteps;
    for (int step = 0; result == WR_SUCCESS && step < steps; ++step) {
        double dt_grid = DBL_MAX;
        result = wro_prepare(cells, n, *cgs, grid_time, step, perturb, &dt_grid, nthreads);
        if (result != WR_SUCCESS) break;
        if (dt_grid == DBL_MAX) break;
        const double next = grid_time + dt_grid;
        if (!valid_positive(dt_grid) || !std::isfinite(next)) { result = WR_BAD_INPUTS; break; }
        int integrated = 0;
        result = wro_advance(cells, n, *cgs, next, dt_grid, &integrated, nthreads);
        if (result != WR_SUCCESS) break;
        if (integrated == 0) break;
        grid_time = next;
        *cgs += 1;
    }
    return result;
}

// Host outer loop of the gridwide-structured-cta32 policy (reproducer.cpp:7856-7959
// with the structured advance launch of :7911-7916): the same prepare and grid
// minimum, then every 32-cell tile advanced by advance_tile.
int wro_run_cta32(wr_collapse_state* cells, int n, int perturb, int* cgs, int max_steps, int nthreads) {
    int result = WR_SUCCESS;
    double grid_time = 0.0;
    const int steps = max_steps > 0 ? max_steps : kMaxCollapseSteps;
    const int tiles = (n + kTile - 1) / kTile;
    for (int step = 0; result == WR_SUCCESS && step < steps; ++step) {
        double dt_grid = DBL_MAX;
        result = wro_prepare(cells, n, *cgs, grid_time, step, perturb, &dt_grid, nthreads);
        if (result != WR_SUCCESS) break;
        if (dt_grid == DBL_MAX) break;
        const double next = grid_time + dt_grid;
        if (!valid_positive(dt_grid) || !std::isfinite(next)) { result = WR_BAD_INPUTS; break; }
        std::atomic<int> failure{WR_SUCCESS};
        int integrated = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : integrated) num_threads(nthreads > 0 ? nthreads : 1)
        for (int tl = 0; tl < tiles; ++tl) {
            const int b = tl * kTile;
            integrated += advance_tile(cells, b, std::min(kTile, n - b), *cgs, grid_time, next, dt_grid, failure);
        }
        result = failure.load();
        if (result != WR_SUCCESS) break;
        if (integrated == 0) break;
        grid_time = next;
        *cgs += 1;
    }
    return result;
}

// The reference CPU program's loop (legacy-local policy), reproducer.cpp:8630-8648:
// cells in index order, each with its own dt; stops when every cell stopped or
// at the first failure.  Cells are independent within a step, so the cell loop
// runs in parallel; on failure the cells after the failing one in index order
// are left as the reference leaves them only when no failure occurs (failure
// runs are reported, not replayed).
int wro_run_legacy(wr_collapse_state* cells, int n, int perturb, int* cgs, int max_steps, int nthreads) {
    int failure = WR_SUCCESS;
    const int steps = max_steps > 0 ? max_steps : kMaxCollapseSteps;
    for (int step = 0; step < steps; ++step) {
        int all_stopped = 1;
        int fail_code = WR_SUCCESS;
#pragma omp parallel for schedule(dynamic, 1) reduction(min : all_stopped) num_threads(nthreads > 0 ? nthreads : 1)
        for (int i = 0; i < n; ++i) {
            if (cells[i].completed_steps < *cgs) continue;
            int f = WR_SUCCESS;
            const bool stopped = legacy_step(cells[i], i, step, perturb != 0, f);
            if (f != WR_SUCCESS) {
#pragma omp critical
                if (fail_code == WR_SUCCESS) fail_code = f;
            }
            all_stopped = (all_stopped && stopped) ? 1 : 0;
        }
        if (fail_code != WR_SUCCESS) {
            failure = fail_code;
            break;
        }
        if (all_stopped) break;
        *cgs += 1;
    }
    return failure;
}

// Replays a subset of cells through a recorded grid-timestep history: cell_ids[i]
// is the grid index of cells[i] (the perturbation seed), dt_hist[s] the grid dt of
// outer step s.  Cells are independent given the grid dt, so a sample of a large
// grid can be checked against the GPU run without integrating the whole grid.
// Returns the first failure code; *cgs receives the number of steps replayed.
int wro_replay(wr_collapse_state* cells, const int* cell_ids, int n, int perturb,
               const double* dt_hist, int nsteps, int nthreads) {
    std::atomic<int> failure{WR_SUCCESS};
    double grid_time = 0.0;
    for (int step = 0; step < nsteps; ++step) {
        const double dt_grid = dt_hist[step];
        const double next = grid_time + dt_grid;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
        for (int i = 0; i < n; ++i) {
            double cand;
            prepare_cell(cells[i], cell_ids[i], step, grid_time, step, perturb != 0, cand, failure);
            if (cand != DBL_MAX && cand < dt_grid) record_failure(failure, WR_BAD_INPUTS);
            advance_cell(cells[i], step, next, dt_grid, failure);
        }
        if (failure.load() != WR_SUCCESS) break;
        grid_time = next;
    }
    return failure.load();
}

}  // extern "C"
