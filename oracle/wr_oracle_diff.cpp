// ORACLE -- test infrastructure only.
//
// CPU restatement of the differentiation form's discrete map, and its FP64
// tangent-linear, used as the checker of the GPU forward and adjoint kernels.
// Only the tests and bench.py's checks load it; the product never does.
//
// The map (one cell, the grid's outer schedule given as dt_hist):
//   for each outer step s with the cell at completed_steps == s:
//     prepare_grid_timestep_kernel for the cell (reproducer.cpp:7696-7734):
//       perturbation (:7564-7580), collapse_timestep (:7633-7644), dt < 10 s branch
//     advance_collapse_gridwide_kernel for the cell (:7736-7785):
//       driver update, density-limit exit, rescale by the driver ratio, burn_ros2s
//       (:7592-7627), floor/normalise, charge balance, floor/normalise, eos_re
// with two changes that make it a differentiable function:
//   * every rate coefficient of the RHS is multiplied by exp(p[r]) (the generated
//     wr_netp_rhs; at p == 0 the RHS is the plain one, bit for bit);
//   * the accepted ROS2S step sizes are a recorded input ("frozen controller"):
//     record mode runs the reference controller (:7205-7347) and stores the step
//     sizes it accepted; replay mode takes exactly those steps.  At the recording
//     point both give the same bits as the plain integrator.
// The inputs are each cell's xn[0..13] and T (its other fields are held fixed:
// e is recomputed from T before every burn), and the log multipliers p; the
// outputs are each cell's final xn[0..13] and T.
//
// Every function is a template over the scalar type: double for the map itself,
// Dual (value + one tangent) for the tangent-linear.  With Dual the values follow
// exactly the double operations, so a tangent run also reproduces the map.
// Portable exp/log/cbrt (wr_math.h), the GPU library's default arithmetic.
// Compile with -ffp-contract=off.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../include/warp_reactor.h"
#include "../warp_reactor_gb300/csrc/wr_math.h"

struct OracleMath {
    static double exp(double x) { return wr_exp(x); }
    static double log(double x) { return wr_log(x); }
    static double sqrt(double x) { return std::sqrt(x); }
    static double cbrt(double x) { return wr_cbrt(x); }
    static double fabs(double x) { return std::fabs(x); }
    static double div(double a, double b) { return a / b; }
};

#define WR_NET_HD inline
#include "../warp_reactor_gb300/csrc/generated/network_gen.h"
#include "../warp_reactor_gb300/csrc/generated/network_adj.h"

namespace {

constexpr int NS = 14;
constexpr int NEQ = 15;
constexpr int NP = WR_NUM_RATE_MULT;

// reproducer.cpp:233-252, :203-231, :7406-7431
constexpr double kMass[NS] = {
    9.10938188e-28,   1.67262158e-24,   1.67353251819e-24, 1.67444345638e-24,
    3.34512158e-24,   3.34603251819e-24, 3.34615409819e-24, 3.34694345638e-24,
    3.34706503638e-24, 5.01865409819e-24, 5.01956503638e-24, 6.69024316e-24,
    6.69115409819e-24, 6.69206503638e-24};
constexpr double gamma_of(int n) { return (n == 6 || n == 8 || n == 9 || n == 10) ? 1.4 : 5.0 / 3.0; }
constexpr double kNA = 6.02214076e+23;
constexpr double kKB = 1.3806490000000002e-16;
constexpr double kMp = 1.67262192595e-24;
constexpr double kFloor = 1.0e-100;
constexpr double kGrav = 6.674e-8;
constexpr double kPi = 3.141592653589793238462643383279502884;
constexpr double kTffReduc = 1.0e-1;
constexpr double kRtolSpec = 1.0e-4, kAtolSpec = 1.0e-4;
constexpr double kRtolEnergy = 1.0e-6, kAtolEnergy = 1.0e-6;
constexpr int kPerturbInterval = 20;
constexpr double kPerturbAmplitude = 0.2;
constexpr double kDriverLimit = 2.0e-6;
// ROS2SCoefficients, reproducer.cpp:7113-7128
constexpr double kGamma = 0.292893218813452;
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

// ------------------------------------------------------------------ scalar types
struct Dual {
    double v, d;
    Dual() : v(0.0), d(0.0) {}
    Dual(double x) : v(x), d(0.0) {}  // NOLINT: constants promote
    Dual(double x, double t) : v(x), d(t) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator!=(Dual a, Dual b) { return a.v != b.v; }

inline double val(double x) { return x; }
inline double val(Dual x) { return x.v; }
inline double dfabs(double x) { return std::fabs(x); }
inline Dual dfabs(Dual x) { return x.v < 0.0 ? -x : x; }
inline double dsqrt(double x) { return std::sqrt(x); }
inline Dual dsqrt(Dual x) {
    const double r = std::sqrt(x.v);
    return {r, x.d / (2.0 * r)};
}
inline double dexp(double x) { return OracleMath::exp(x); }
inline Dual dexp(Dual x) {
    const double r = OracleMath::exp(x.v);
    return {r, r * x.d};
}

// std::max / std::min semantics
template <class S> inline S smax(S a, S b) { return (a < b) ? b : a; }
template <class S> inline S smin(S a, S b) { return (b < a) ? b : a; }

// ------------------------------------------------------------------ network
struct MatSink {
    double (*J)[NEQ];
    void operator()(int r, int c, double v) { J[r][c] = v; }
};
inline void net_rhs(const double* X, double T, const double* mult, double* f) {
    wr_netp_rhs<OracleMath>(X, T, mult, f);
}
inline void net_rhs(const Dual* X, Dual T, const Dual* mult, Dual* f) {
    double x[NS], dx[NS], m[NP], dm[NP], fv[NEQ], df[NEQ];
    for (int i = 0; i < NS; ++i) { x[i] = X[i].v; dx[i] = X[i].d; }
    for (int i = 0; i < NP; ++i) { m[i] = mult[i].v; dm[i] = mult[i].d; }
    wr_netp_rhs_jvp<OracleMath>(x, T.v, m, dx, T.d, dm, fv, df);
    for (int i = 0; i < NEQ; ++i) f[i] = Dual(fv[i], df[i]);
}
inline void net_jac(const double* X, double T, double J[NEQ][NEQ]) {
    double f[NEQ];
    MatSink sink{J};
    wr_net_jac_rhs<OracleMath>(X, T, f, sink);
}
inline void net_jac(const Dual* X, Dual T, Dual J[NEQ][NEQ]) {
    double x[NS], dx[NS], jv[NEQ * NEQ], dj[NEQ * NEQ];
    for (int i = 0; i < NS; ++i) { x[i] = X[i].v; dx[i] = X[i].d; }
    wr_net_jac_jvp<OracleMath>(x, T.v, dx, T.d, jv, dj);
    for (int r = 0; r < NEQ; ++r)
        for (int c = 0; c < NEQ; ++c) J[r][c] = Dual(jv[r * NEQ + c], dj[r * NEQ + c]);
}

// ------------------------------------------------------------------ physics
template <class S> struct Cell {
    S rho, T, e, driver;
    S xn[NS];
};

template <class S> S density(const S* xn) {  // :270-276
    S rho = 0.0;
    for (int n = 0; n < NS; ++n) rho = rho + xn[n] * kMass[n];
    return rho;
}
template <class S> void eos_sums(const S* xn, S& sa, S& sg) {  // :284-304
    S rhotot = 0.0;
    sa = 0.0;
    sg = 0.0;
    for (int n = 0; n < NS; ++n) rhotot = rhotot + xn[n] * kMass[n];
    for (int n = 0; n < NS; ++n) {
        sa = sa + xn[n];
        sg = sg + (xn[n] * kMp / rhotot) * (1.0 / (gamma_of(n) - 1.0));
    }
    sa = sa * (kMp / rhotot);
    sg = sg / sa;
}
template <class S> S eos_e_from_T(const S* xn, S T) {  // eos_rt, :306-309
    S sa, sg;
    eos_sums(xn, sa, sg);
    return sg * sa * (kNA * kKB) * T;
}
template <class S> S eos_T_from_e(const S* xn, S e) {  // eos_re, :311-314
    S sa, sg;
    eos_sums(xn, sa, sg);
    return e / (sg * (kNA * kKB) * sa);
}
template <class S> void balance_charge(S* xn) {  // :316-319
    xn[0] = -xn[3] - xn[7] + xn[1] + xn[12] + xn[6] + xn[4] + xn[9] + 2.0 * xn[11];
}
template <class S> void floor_and_normalize(S* xn, S rho) {  // :321-339
    S mf[NS];
    S sum = 0.0;
    for (int n = 0; n < NS; ++n) {
        xn[n] = smax(xn[n], S(kFloor));
        mf[n] = kMass[n] * xn[n] / rho;
        sum = sum + mf[n];
    }
    for (int n = 0; n < NS; ++n) {
        mf[n] = mf[n] / sum;
        xn[n] = mf[n] * rho / kMass[n];
    }
}
template <class S> void renormalize(S* xn, S rho) {
    floor_and_normalize(xn, rho);
    balance_charge(xn);
    floor_and_normalize(xn, rho);
}
template <class S> S collapse_timestep(const S* xn) {  // :7633-7644 (validity checked by value)
    const S rho = density(xn);
    const S tff = dsqrt(kPi * 3.0 / (32.0 * rho * kGrav));
    return kTffReduc * tff;
}
inline bool valid_positive(double v) { return v > 0.0 && std::isfinite(v); }

uint64_t splitmix64(uint64_t v) {  // :7548-7562
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

template <class S> void state_from_y(const S* y, S* X, S& T) {  // :7029-7038
    for (int n = 0; n < NS; ++n) X[n] = smax(y[n], S(kFloor));
    T = eos_T_from_e(X, y[NS]);
}

template <class S> int lu_decomposition(S A[NEQ][NEQ], int* ipvt) {  // :96-151
    int info = 0;
    for (int k = 0; k < NEQ - 1; ++k) {
        int p = k;
        double max_val = std::fabs(val(A[k][k]));
        for (int i = k + 1; i < NEQ; ++i) {
            const double v = std::fabs(val(A[i][k]));
            if (v > max_val) { max_val = v; p = i; }
        }
        ipvt[k] = p;
        if (val(A[p][k]) != 0.0) {
            if (p != k) {
                for (int j = k; j < NEQ; ++j) {
                    const S t = A[p][j]; A[p][j] = A[k][j]; A[k][j] = t;
                }
            }
            const S mult = S(-1.0) / A[k][k];
            for (int i = k + 1; i < NEQ; ++i) A[i][k] = A[i][k] * mult;
            for (int j = k + 1; j < NEQ; ++j) {
                const S t = A[k][j];
                for (int i = k + 1; i < NEQ; ++i) A[i][j] = A[i][j] + t * A[i][k];
            }
        } else {
            info = k + 1;
        }
    }
    ipvt[NEQ - 1] = NEQ - 1;
    if (val(A[NEQ - 1][NEQ - 1]) == 0.0) info = NEQ;
    return info;
}
template <class S> void lu_solve(S LU[NEQ][NEQ], const int* ipvt, S* x) {  // :154-181
    for (int k = 0; k < NEQ - 1; ++k) {
        const int p = ipvt[k];
        const S t = x[p];
        if (p != k) { x[p] = x[k]; x[k] = t; }
        for (int j = k + 1; j < NEQ; ++j) x[j] = x[j] + t * LU[j][k];
    }
    for (int kb = 0; kb < NEQ; ++kb) {
        const int k = NEQ - 1 - kb;
        x[k] = x[k] / LU[k][k];
        const S t = -x[k];
        for (int j = 0; j < k; ++j) x[j] = x[j] + t * LU[j][k];
    }
}

// One ROS2S attempt from y with step h and Jacobian J (reproducer.cpp:7259-7304):
// ynew and the error-estimate vector; returns the LU info.
template <class S> int ros2s_attempt(const S* y, S h, S J[NEQ][NEQ], const S* mult, S* ynew, S* work) {
    S e[NEQ][NEQ], ak1[NEQ], ak2[NEQ], dy[NEQ], X[NS], T;
    int ip[NEQ];
    const S fac = S(1.0) / (h * kGamma);
    for (int i = 0; i < NEQ; ++i) {
        for (int j = 0; j < NEQ; ++j) e[i][j] = -J[i][j];
        e[i][i] = e[i][i] + fac;
    }
    const int info = lu_decomposition(e, ip);
    if (info != 0) return info;
    state_from_y(y, X, T);
    net_rhs(X, T, mult, ak1);
    lu_solve(e, ip, ak1);
    for (int i = 0; i < NEQ; ++i) {
        ynew[i] = y[i] + kA21 * ak1[i];
        ak2[i] = (kC21 / h) * ak1[i];
    }
    state_from_y(ynew, X, T);
    net_rhs(X, T, mult, dy);
    for (int i = 0; i < NEQ; ++i) ak2[i] = ak2[i] + dy[i];
    lu_solve(e, ip, ak2);
    for (int i = 0; i < NEQ; ++i) {
        ynew[i] = y[i] + kA31 * ak1[i] + kA32 * ak2[i];
        work[i] = (kC31 * ak1[i] + kC32 * ak2[i]) / h;
    }
    state_from_y(ynew, X, T);
    net_rhs(X, T, mult, dy);
    for (int i = 0; i < NEQ; ++i) work[i] = work[i] + dy[i];
    lu_solve(e, ip, work);
    for (int i = 0; i < NEQ; ++i) {
        const S ak3 = work[i];
        ynew[i] = y[i] + kB1 * ak1[i] + kB2 * ak2[i] + kB3 * ak3;
        work[i] = kE1 * ak1[i] + kE2 * ak2[i] + kE3 * ak3;
    }
    return 0;
}

template <class S> void jacobian(const S* y, S J[NEQ][NEQ]) {
    S X[NS], T;
    state_from_y(y, X, T);
    net_jac(X, T, J);
}

// The reference controller (RODAS::integrate, :7205-7347, configure_ros2s
// :7582-7590) on doubles, appending the accepted step sizes to hs.
int integrate_record(double* y, double tout, const double* mult, std::vector<double>& hs) {
    const double uround = 1.e-16, fac_min = 0.2, fac_max = 6.0, safe = 0.9;
    const int max_steps = 10000000;
    if (tout <= 0.0) return WR_BAD_INPUTS;
    const double hmaxn = tout;
    double h = tout;
    if (std::fabs(h) <= 10.0 * uround) h = 1.e-6;
    h = smin(std::fabs(h), hmaxn);
    bool reject = false, last = false;
    int nsing = 0, n_step = 0, n_accept = 0;
    double hacc = 0.0, erracc = 1.0, x = 0.0;
    double J[NEQ][NEQ], ynew[NEQ], work[NEQ];
    for (;;) {
        if (n_step > max_steps) return WR_TOO_MANY_STEPS;
        if (0.1 * std::fabs(h) <= std::fabs(x) * uround) return WR_DT_UNDERFLOW;
        if (last) return WR_SUCCESS;
        if (x + h * 1.0001 >= tout) { h = tout - x; last = true; }
        jacobian(y, J);
        for (;;) {
            if (ros2s_attempt(y, h, J, mult, ynew, work) != 0) {
                nsing += 1;
                if (nsing >= 5) return WR_LU_DECOMPOSITION_ERROR;
                h *= 0.5;
                reject = true;
                last = false;
                continue;
            }
            n_step += 1;
            double err = 0.0;
            for (int i = 0; i < NEQ; ++i) {
                const double rtol = i < NS ? kRtolSpec : kRtolEnergy;
                const double atol = i < NS ? kAtolSpec : kAtolEnergy;
                const double sk = atol + rtol * smax(std::fabs(y[i]), std::fabs(ynew[i]));
                const double term = work[i] / sk;
                err += term * term;
            }
            err = std::sqrt(err / static_cast<double>(NEQ));
            const double raw_fac = OracleMath::cbrt(err) / safe;
            const double fac_step = smax(1.0 / fac_max, smin(1.0 / fac_min, raw_fac));
            double hnew = h / fac_step;
            if (err <= 1.0) {
                n_accept += 1;
                if (n_accept > 1) {
                    const double facgus = smax(1.0 / fac_max,
                        smin(1.0 / fac_min, (hacc / h) * OracleMath::cbrt((err * err) / erracc) / safe));
                    hnew = h / smax(fac_step, facgus);
                }
                hacc = h;
                erracc = smax(1.e-2, err);
                hs.push_back(h);
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
            if (hnew == 0.0) return WR_DT_UNDERFLOW;  // the reject loop's only other exit
        }
    }
}

// The frozen controller: exactly the given accepted steps.
template <class S> void integrate_replay(S* y, const double* hs, int count, const S* mult) {
    S J[NEQ][NEQ], ynew[NEQ], work[NEQ];
    for (int k = 0; k < count; ++k) {
        jacobian(y, J);
        ros2s_attempt(y, S(hs[k]), J, mult, ynew, work);
        for (int i = 0; i < NEQ; ++i) y[i] = ynew[i];
    }
}

// The cell's whole schedule.  record: run the controller and fill hs / counts;
// otherwise replay them.  counts[s] = accepted steps of the burn at outer step s
// (0 without a burn).  Returns an IntegratorResult.
template <class S>
int run_cell(Cell<S>& c, int cell_id, int perturb, const double* dt_hist, int nsteps, const S* mult,
             bool record, std::vector<double>& hs, int* counts) {
    size_t hpos = 0;
    for (int s = 0; s < nsteps; ++s) {
        counts[s] = record ? 0 : counts[s];
        // prepare
        if (perturb && s != 0 && s % kPerturbInterval == 0) {
            const double factor = perturbation_factor(cell_id, s);
            c.driver = c.driver * factor;
            c.rho = c.rho * factor;
            for (int n = 0; n < NS; ++n) c.xn[n] = c.xn[n] * factor;
            renormalize(c.xn, c.rho);
            c.T = eos_T_from_e(c.xn, c.e);
        }
        const S dt = collapse_timestep(c.xn);
        if (!valid_positive(val(dt)) || !valid_positive(val(c.driver))) return WR_BAD_INPUTS;
        if (val(dt) < 10.0) {
            const S tff = dt / kTffReduc;
            c.driver = c.driver + dt * (c.driver / tff);
            return WR_SUCCESS;  // no candidate, no burn: the cell is done
        }
        // advance
        const double dt_grid = dt_hist[s];
        const S old_density = c.driver;
        const S tff = dt / kTffReduc;
        c.driver = c.driver + dt_grid * (c.driver / tff);
        if (!valid_positive(val(c.driver)) || val(c.driver) > kDriverLimit) return WR_SUCCESS;
        const S ratio = c.driver / old_density;
        for (int n = 0; n < NS; ++n) c.xn[n] = c.xn[n] * ratio;
        c.rho = c.rho * ratio;
        c.e = eos_e_from_T(c.xn, c.T);
        S y[NEQ];
        for (int n = 0; n < NS; ++n) y[n] = c.xn[n];
        y[NS] = c.e;
        if constexpr (std::is_same<S, double>::value) {
            if (record) {
                const size_t before = hs.size();
                const int r = integrate_record(y, dt_grid, mult, hs);
                if (r != WR_SUCCESS) return r;
                counts[s] = static_cast<int>(hs.size() - before);
            } else {
                integrate_replay(y, hs.data() + hpos, counts[s], mult);
            }
        } else {
            integrate_replay(y, hs.data() + hpos, counts[s], mult);
        }
        hpos += static_cast<size_t>(counts[s]);
        for (int n = 0; n < NS; ++n) c.xn[n] = y[n];
        renormalize(c.xn, c.rho);
        c.e = y[NS];
        c.T = eos_T_from_e(c.xn, c.e);
    }
    return WR_SUCCESS;
}

template <class S> Cell<S> load_cell(const wr_collapse_state& st, const double* u, const double* du) {
    Cell<S> c;
    c.rho = st.rho;
    c.e = st.e;
    c.driver = st.density_driver;
    for (int n = 0; n < NS; ++n) c.xn[n] = u ? u[n] : st.xn[n];
    c.T = u ? u[NS] : st.T;
    if constexpr (std::is_same<S, Dual>::value) {
        if (du) {
            for (int n = 0; n < NS; ++n) c.xn[n].d = du[n];
            c.T.d = du[NS];
        }
    }
    return c;
}

}  // namespace

extern "C" {

int wro_diff_num_multipliers(void) { return NP; }

// The generated derivative code itself, for tests against finite differences.
void wro_netp_rhs(const double* X, double T, const double* mult, double* f) {
    wr_netp_rhs<OracleMath>(X, T, mult, f);
}
void wro_netp_rhs_vjp(const double* X, double T, const double* mult, const double* fbar, double* Xbar,
                      double* Tbar, double* mbar) {
    wr_netp_rhs_vjp<OracleMath>(X, T, mult, fbar, Xbar, *Tbar, mbar);
}
void wro_netp_rhs_jvp(const double* X, double T, const double* mult, const double* dX, double dT,
                      const double* dmult, double* f, double* df) {
    wr_netp_rhs_jvp<OracleMath>(X, T, mult, dX, dT, dmult, f, df);
}
void wro_net_jac_vjp(const double* X, double T, const double* Jbar, double* Xbar, double* Tbar) {
    wr_net_jac_vjp<OracleMath>(X, T, Jbar, Xbar, *Tbar);
}
void wro_net_jac_jvp(const double* X, double T, const double* dX, double dT, double* J, double* dJ) {
    wr_net_jac_jvp<OracleMath>(X, T, dX, dT, J, dJ);
}

// Forward map.  cells: the n input records (AoS); cell_ids: their grid indices
// (perturbation seed); u: n x 15 overrides of (xn[0..13], T) or null; log_mult: NP
// log multipliers or null (0); record != 0 runs the controller and writes hbuf
// (n x cap step sizes) and counts (n x nsteps); record == 0 replays them.  q_out:
// n x 15 (final xn[0..13], T).  Returns the first failure (WR_SUCCESS = 1).
int wro_diff_forward(const wr_collapse_state* cells, const int* cell_ids, int n, int perturb,
                     const double* dt_hist, int nsteps, const double* u, const double* log_mult, int record,
                     double* hbuf, int cap, int* counts, double* q_out, int nthreads) {
    double mult[NP];
    for (int r = 0; r < NP; ++r) mult[r] = log_mult ? OracleMath::exp(log_mult[r]) : 1.0;
    int failure = WR_SUCCESS;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < n; ++i) {
        Cell<double> c = load_cell<double>(cells[i], u ? u + 15 * i : nullptr, nullptr);
        std::vector<double> hs;
        int* cnt = counts + static_cast<size_t>(i) * nsteps;
        if (!record) {
            int total = 0;
            for (int s = 0; s < nsteps; ++s) total += cnt[s];
            hs.assign(hbuf + static_cast<size_t>(i) * cap, hbuf + static_cast<size_t>(i) * cap + total);
        }
        int r = run_cell(c, cell_ids ? cell_ids[i] : i, perturb, dt_hist, nsteps, mult, record != 0, hs, cnt);
        if (record && r == WR_SUCCESS) {
            if (static_cast<int>(hs.size()) > cap) r = WR_TOO_MANY_STEPS;
            else std::memcpy(hbuf + static_cast<size_t>(i) * cap, hs.data(), hs.size() * sizeof(double));
        }
        for (int k = 0; k < NS; ++k) q_out[15 * i + k] = c.xn[k];
        q_out[15 * i + NS] = c.T;
        if (r != WR_SUCCESS) {
#pragma omp critical
            if (failure == WR_SUCCESS) failure = r;
        }
    }
    return failure;
}

// Tangent-linear of the frozen map along (du, dlog_mult): dq_out = dq/du du +
// dq/dp dp, n x 15, with q_out as in wro_diff_forward (replay mode).
int wro_diff_tangent(const wr_collapse_state* cells, const int* cell_ids, int n, int perturb,
                     const double* dt_hist, int nsteps, const double* u, const double* log_mult,
                     const double* du, const double* dlog_mult, const double* hbuf, int cap,
                     const int* counts, double* q_out, double* dq_out, int nthreads) {
    Dual mult[NP];
    for (int r = 0; r < NP; ++r) {
        const double p = log_mult ? log_mult[r] : 0.0;
        const double m = OracleMath::exp(p);
        mult[r] = Dual(m, dlog_mult ? m * dlog_mult[r] : 0.0);
    }
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int i = 0; i < n; ++i) {
        Cell<Dual> c = load_cell<Dual>(cells[i], u ? u + 15 * i : nullptr, du ? du + 15 * i : nullptr);
        int* cnt = const_cast<int*>(counts + static_cast<size_t>(i) * nsteps);
        int total = 0;
        for (int s = 0; s < nsteps; ++s) total += cnt[s];
        std::vector<double> hs(hbuf + static_cast<size_t>(i) * cap, hbuf + static_cast<size_t>(i) * cap + total);
        run_cell(c, cell_ids ? cell_ids[i] : i, perturb, dt_hist, nsteps, mult, false, hs, cnt);
        for (int k = 0; k < NS; ++k) {
            q_out[15 * i + k] = c.xn[k].v;
            dq_out[15 * i + k] = c.xn[k].d;
        }
        q_out[15 * i + NS] = c.T.v;
        dq_out[15 * i + NS] = c.T.d;
    }
    return WR_SUCCESS;
}

}  // extern "C"
