// wr_physics.cuh -- per-cell chemistry physics shared by the device kernels.
//
// Species data, equation of state, charge balance, normalisation, the collapse
// driver helpers and the ROS2S coefficients of the reference reproducer, restated
// for device code.  Every function performs the reference's floating-point
// operations in the reference's order (no FMA contraction: the library is built
// with --fmad=false), so results are bit-identical to the reference's rounding
// sequence given the same exp/log/cbrt.
#pragma once

#include <stdint.h>

#include "wr_math.h"

namespace wr {

// Division on the device: the IEEE quotient computed on the integer pipe
// (wr_div_int), one shared out-of-line copy.  Bit-identical to a / b.
static __device__ __noinline__ double wr_div_call(double a, double b) { return wr_div_int(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return wr_div_call(a, b); }
// a / b with b's reciprocal Y = wr_div_recip(b) already computed (several
// quotients by one divisor): the same bits as ddiv(a, b)
static __device__ __noinline__ double ddiv_recip(double a, double b, uint64_t Y) { return wr_div_finish(a, b, Y); }

constexpr int NS = 14;
constexpr int NEQ = 15;

// species masses, reproducer.cpp:233-248
__host__ __device__ constexpr double mass(int n) {
    return n == 0 ? 9.10938188e-28 : n == 1 ? 1.67262158e-24 : n == 2 ? 1.67353251819e-24 :
           n == 3 ? 1.67444345638e-24 : n == 4 ? 3.34512158e-24 : n == 5 ? 3.34603251819e-24 :
           n == 6 ? 3.34615409819e-24 : n == 7 ? 3.34694345638e-24 : n == 8 ? 3.34706503638e-24 :
           n == 9 ? 5.01865409819e-24 : n == 10 ? 5.01956503638e-24 : n == 11 ? 6.69024316e-24 :
           n == 12 ? 6.69115409819e-24 : 6.69206503638e-24;
}
// 1/(gamma_n - 1), reproducer.cpp:250-252 and :297 (folded exactly by the compiler)
__host__ __device__ constexpr double inv_gm1(int n) {
    return 1.0 / (((n == 6 || n == 8 || n == 9 || n == 10) ? 1.4 : 5.0 / 3.0) - 1.0);
}
constexpr double kNA = 6.02214076e+23;           // reproducer.cpp:207
constexpr double kKB = 1.3806490000000002e-16;   // :208
constexpr double kMp = 1.67262192595e-24;        // :209
constexpr double kGasConstant = kNA * kKB;       // :285
constexpr double kFloor = 1.0e-100;              // :231
constexpr double kGrav = 6.674e-8;               // :203
constexpr double kPi = 3.141592653589793238462643383279502884;  // :204
constexpr double kTffReduc = 1.0e-1;             // :7407
constexpr double kRtolSpec = 1.0e-4, kAtolSpec = 1.0e-4;        // :7410-7411
constexpr double kRtolEnergy = 1.0e-6, kAtolEnergy = 1.0e-6;    // :7412-7413
constexpr int kPerturbInterval = 20;             // :7418
constexpr double kPerturbAmplitude = 0.2;        // :7419
constexpr int kMaxSteps = 10000000;              // configure_ros2s, :7589
constexpr double kDriverLimit = 2.0e-6;          // :7759

// ROS2S coefficients, reproducer.cpp:7113-7128
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
constexpr double kE1 = -0.23570226039551292;
constexpr double kE2 = -0.23570226039551567;
constexpr double kE3 = -0.13807118745769906;
constexpr double kUround = 1.e-16, kFacMin = 0.2, kFacMax = 6.0, kSafe = 0.9;  // :7097-7101

// std::max / std::min semantics: (a < b) ? b : a and (b < a) ? b : a
__host__ __device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }

__device__ __forceinline__ bool valid_positive(double v) { return v > 0.0 && isfinite(v); }

// density, reproducer.cpp:270-276
__device__ __forceinline__ double density(const double* xn) {
    double rho = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) rho += xn[n] * mass(n);
    return rho;
}

// sum_gammasinv * gasconstant * sum_abarinv and friends, reproducer.cpp:284-314
struct Eos {
    double sum_abarinv, sum_gammasinv;
};
__device__ __forceinline__ Eos eos_sums(const double* xn) {
    double sa = 0.0, sg = 0.0, rhotot = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) rhotot += xn[n] * mass(n);
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        sa += xn[n];
        sg += ddiv(xn[n] * kMp, rhotot) * inv_gm1(n);
    }
    sa *= ddiv(kMp, rhotot);
    sg = ddiv(sg, sa);
    return {sa, sg};
}
// eos_rt: e from T, reproducer.cpp:306-309
__device__ __forceinline__ double eos_e_from_T(const double* xn, double T) {
    const Eos q = eos_sums(xn);
    return q.sum_gammasinv * q.sum_abarinv * kGasConstant * T;
}
// eos_re: T from e, reproducer.cpp:311-314
__device__ __forceinline__ double eos_T_from_e(const double* xn, double e) {
    const Eos q = eos_sums(xn);
    return ddiv(e, q.sum_gammasinv * kGasConstant * q.sum_abarinv);
}

// balance_charge, reproducer.cpp:316-319
__device__ __forceinline__ void balance_charge(double* xn) {
    xn[0] = -xn[3] - xn[7] + xn[1] + xn[12] + xn[6] + xn[4] + xn[9] + 2.0 * xn[11];
}

// floor_and_normalize_number_densities, reproducer.cpp:321-339
__device__ __forceinline__ void floor_and_normalize(double* xn, double rho) {
    double mf[NS];
    double sum = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        xn[n] = smax(xn[n], kFloor);
        mf[n] = ddiv(mass(n) * xn[n], rho);
        sum += mf[n];
    }
#pragma unroll
    for (int n = 0; n < NS; ++n) {
        mf[n] = ddiv(mf[n], sum);
        xn[n] = ddiv(mf[n] * rho, mass(n));
    }
}

// the post-burn / post-perturbation sequence: floor+normalise, charge, floor+normalise
__device__ __forceinline__ void renormalize(double* xn, double rho) {
    floor_and_normalize(xn, rho);
    balance_charge(xn);
    floor_and_normalize(xn, rho);
}

// splitmix64 / perturbation_factor, reproducer.cpp:7548-7562
__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t v) {
    v += 0x9e3779b97f4a7c15ULL;
    v = (v ^ (v >> 30U)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27U)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31U);
}
__host__ __device__ __forceinline__ double perturbation_factor(int cell, int step) {
    const uint64_t seed = (static_cast<uint64_t>(static_cast<unsigned int>(cell)) << 32U) ^
                          (static_cast<uint64_t>(static_cast<unsigned int>(step)) << 16U);
    const uint64_t bits = splitmix64(seed) >> 11U;
    const double unit = static_cast<double>(bits) * (1.0 / static_cast<double>(1ULL << 53U));
    return 1.0 + kPerturbAmplitude * (2.0 * unit - 1.0);
}

// collapse_timestep, reproducer.cpp:7633-7644
__device__ __forceinline__ double collapse_timestep(const double* xn) {
    const double rho = density(xn);
    if (!valid_positive(rho)) return -1.0;
    const double tff = sqrt(ddiv(kPi * 3.0, 32.0 * rho * kGrav));
    if (!valid_positive(tff)) return -1.0;
    const double dt = kTffReduc * tff;
    return valid_positive(dt) ? dt : -1.0;
}

}  // namespace wr
