// wr_math.h -- bit-reproducible exp / log / cbrt for host and device code.
//
// The same source compiles for the CPU (g++, -ffp-contract=off) and for sm_103a
// (nvcc, --fmad=false) and returns the same bits on both: exp and log are computed
// in 64/128-bit integer fixed point (only integer arithmetic, table lookups and a
// final round-to-nearest-even), and cbrt uses plain binary64 + - * / in a fixed
// order.  On GB300 the integer cores matter for speed as well as reproducibility:
// the SM issues integer multiplies at many times its FP64 rate, so moving the
// transcendental work off the FP64 pipe frees it for the network's own + - * /.
//
// Accuracy (checked against 200-bit mpmath in tests/test_math.py):
//   exp: |error| < 0.51 ulp for normal results; underflow to subnormals rounds
//        once from the fixed-point value.
//   log: |error| < 0.51 ulp.
//   cbrt: |error| <= 1 ulp (Newton iteration in binary64).
//
// Methods (textbook, restated here):
//   exp(x) = 2^k * 2^f, t = x*log2(e) = k + f computed as a 128-bit product of the
//     53-bit mantissa with a 128-bit log2(e); 2^f = T1[f>>58] * T2[(f>>52)&63] *
//     e^u with |u| < 2^-12.5 and e^u - 1 = u + u^2/2 + u^3/6 + u^4/24 (table-driven
//     reduction in the manner of Tang, ACM TOMS 15(2), 1989).
//   log(x) = E*ln2 - log(r_i/2048) + log1p(z), z = m*r_i/2048 - 1 exactly in integers,
//     |z| < 2^-9, log1p(z) = z*(1 - z/2 + z^2/3 - ... + z^6/7) (Tang's reduction
//     with a 512-entry reciprocal table, ACM TOMS 16(4), 1990).  The two
//     intervals adjacent to 1 use the product z*h directly, which keeps full
//     relative precision for results near zero.
//   cbrt(x): exponent-divided initial guess and four Newton steps
//     y <- y + (x/y^2 - y)/3.
#pragma once

#include <stdint.h>

#include "wr_math_tables.h"

#if defined(__CUDACC__)
#define WR_MHD __host__ __device__ __forceinline__
#else
#include <string.h>
#define WR_MHD static inline
#endif

#if defined(__CUDACC__)
static __device__ const uint64_t wr_d_exp_t1[64] = WR_EXP_T1_INIT;
static __device__ const uint64_t wr_d_exp_t2[64] = WR_EXP_T2_INIT;
static __device__ const uint16_t wr_d_log_r[512] = WR_LOG_R_INIT;
static __device__ const uint64_t wr_d_log_nl[1024] = WR_LOG_NL_INIT;
#endif
static const uint64_t wr_h_exp_t1[64] = WR_EXP_T1_INIT;
static const uint64_t wr_h_exp_t2[64] = WR_EXP_T2_INIT;
static const uint16_t wr_h_log_r[512] = WR_LOG_R_INIT;
static const uint64_t wr_h_log_nl[1024] = WR_LOG_NL_INIT;

#if defined(__CUDA_ARCH__)
#define WR_TAB(name) wr_d_##name
#else
#define WR_TAB(name) wr_h_##name
#endif

WR_MHD uint64_t wr_bits(double x) {
#if defined(__CUDA_ARCH__)
    return static_cast<uint64_t>(__double_as_longlong(x));
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

WR_MHD double wr_from_bits(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double(static_cast<long long>(u));
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

WR_MHD uint64_t wr_umulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return static_cast<uint64_t>((static_cast<unsigned __int128>(a) * b) >> 64);
#endif
}

WR_MHD int64_t wr_smulhi(int64_t a, int64_t b) {
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return static_cast<int64_t>((static_cast<__int128>(a) * b) >> 64);
#endif
}

WR_MHD int wr_clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll(static_cast<long long>(x));
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

// Round a signed 128-bit fixed-point value (hi:lo, q fractional bits) to the
// nearest binary64 (ties to even).  The value must be in the normal range.
WR_MHD double wr_fixed_to_double(int64_t hi, uint64_t lo, int q) {
    uint64_t sign = 0;
    uint64_t h = static_cast<uint64_t>(hi);
    if (hi < 0) {
        sign = 0x8000000000000000ULL;
        lo = ~lo + 1;
        h = ~h + (lo == 0 ? 1 : 0);
    }
    if (h == 0 && lo == 0) return 0.0;
    const int n = h ? wr_clz64(h) : 64 + wr_clz64(lo);
    uint64_t top, rest;
    if (n == 0) {
        top = h;
        rest = lo;
    } else if (n < 64) {
        top = (h << n) | (lo >> (64 - n));
        rest = lo << n;
    } else {
        top = lo << (n - 64);
        rest = 0;
    }
    uint64_t mant = top >> 11;
    const uint64_t rem = top & 0x7ff;
    const bool up = rem > 0x400 || (rem == 0x400 && (rest != 0 || (mant & 1)));
    mant += up ? 1 : 0;
    int e2 = (127 - n) - q;
    if (mant >> 53) {
        mant >>= 1;
        e2 += 1;
    }
    return wr_from_bits(sign | (static_cast<uint64_t>(e2 + 1023) << 52) | (mant & 0x000fffffffffffffULL));
}

// Correctly rounded binary64 quotient a/b from integer arithmetic: the result is
// the IEEE quotient (which is unique), so it can replace a/b anywhere without
// changing a bit.  Method: Newton-Raphson reciprocal iteration followed by an
// exact remainder correction of the quotient (the Newton-Raphson-based division of
// J.-M. Muller et al., Handbook of Floating-Point Arithmetic, 2nd ed., Birkhauser
// 2018), carried out in fixed point.  Normal operands with a normal quotient take
// the integer path: a float reciprocal of the divisor's top 24 bits, two
// fixed-point Newton steps (Q63), a 54-bit quotient, an exact remainder check and
// round-to-nearest-even.
// Everything else (zeros, subnormals, inf/NaN, overflow/underflow) uses a / b.
// On GB300 this keeps divisions off the FP64 pipe (a native double division
// issues about eight FP64 instructions).  wr_div_int (below) is
// wr_div_finish(a, b, wr_div_recip(b)).

// The divisor's part of wr_div_int: Y ~ 1/b_m in Q63 (b_m = b's significand in
// [1, 2)) from a float seed and two fixed-point Newton steps.  Any value for a
// zero, subnormal, infinite or NaN b (wr_div_finish then divides by a / b).  A
// quotient needs only wr_div_finish with this Y, so several divisions by one b
// share it.
WR_MHD uint64_t wr_div_recip(double b) {
    const uint64_t ub = wr_bits(b);
    const uint64_t mb = (ub & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const float bf = static_cast<float>(static_cast<uint32_t>(mb >> 29));  // exact, 24 bits
#if defined(__CUDA_ARCH__)
    const float rf = __frcp_rn(bf);
#else
    const float rf = 1.0f / bf;
#endif
    uint64_t Y = static_cast<uint64_t>(static_cast<uint32_t>(rf * 18014398509481984.0f)) << 32;
    const uint64_t B = mb << 10;  // b_m * 2^62
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const int64_t e = static_cast<int64_t>(0x2000000000000000ULL - wr_umulhi(B, Y));  // (1 - b y) * 2^61
        const uint64_t c = e >= 0 ? wr_umulhi(Y, static_cast<uint64_t>(e)) : 0 - wr_umulhi(Y, static_cast<uint64_t>(-e));
        Y += c << 3;
    }
    return Y;
}

// a / b given Y = wr_div_recip(b): a 54-bit quotient Q ~ floor(a_m * 2^(53+adj) /
// b_m), its exact remainder, at most two corrections each way, round to nearest
// even.  Operands or quotients outside the normal range divide by a / b.
WR_MHD double wr_div_finish(double a, double b, uint64_t Y) {
    const uint64_t ua = wr_bits(a), ub = wr_bits(b);
    const uint32_t ea = static_cast<uint32_t>(ua >> 52) & 0x7ff;
    const uint32_t eb = static_cast<uint32_t>(ub >> 52) & 0x7ff;
    if (ea - 1u >= 2046u || eb - 1u >= 2046u) return a / b;
    const uint64_t ma = (ua & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const uint64_t mb = (ub & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const int adj = ma < mb ? 1 : 0;
    const int be = static_cast<int>(ea) - static_cast<int>(eb) - adj + 1023;
    if (be < 1 || be > 2046) return a / b;
    uint64_t Q = wr_umulhi(ma << (2 + adj), Y);
    int64_t R = static_cast<int64_t>((ma << (53 + adj)) - Q * mb);
    const int64_t smb = static_cast<int64_t>(mb);
    if (R < 0) { Q -= 1; R += smb; }
    if (R < 0) { Q -= 1; R += smb; }
    if (R >= smb) { Q += 1; R -= smb; }
    if (R >= smb) { Q += 1; R -= smb; }
    uint64_t mant = Q >> 1;
    const bool up = (Q & 1) && (R != 0 || (mant & 1));
    mant += up ? 1 : 0;
    int e2 = be;
    if (mant >> 53) {
        mant >>= 1;
        e2 += 1;
        if (e2 > 2046) return a / b;
    }
    return wr_from_bits(((ua ^ ub) & 0x8000000000000000ULL) | (static_cast<uint64_t>(e2) << 52) |
                        (mant & 0x000fffffffffffffULL));
}

WR_MHD double wr_div_int(double a, double b) { return wr_div_finish(a, b, wr_div_recip(b)); }

WR_MHD double wr_exp(double x) {
    const uint64_t u = wr_bits(x);
    const uint64_t ax = u & 0x7fffffffffffffffULL;
    const bool neg = (u >> 63) != 0;
    if (ax < 0x3c90000000000000ULL) return 1.0 + x;  // |x| < 2^-54
    if (ax >= 0x4087500000000000ULL) {                // |x| >= 746, inf, NaN
        if (ax > 0x7ff0000000000000ULL) return x + x;
        return neg ? 0.0 : wr_from_bits(0x7ff0000000000000ULL);
    }
    // |x| = M * 2^e with e in [-106, -43]
    const int e = static_cast<int>(ax >> 52) - 1075;
    const uint64_t M = (ax & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    // Q = (M * log2(e) * 2^127) >> 64, the low partial product's low word dropped
    const uint64_t a_hi = wr_umulhi(M, WR_L2E_Q127_HI);
    const uint64_t a_lo = M * WR_L2E_Q127_HI;
    const uint64_t b_hi = wr_umulhi(M, WR_L2E_Q127_LO);
    const uint64_t q_lo = a_lo + b_hi;
    const uint64_t q_hi = a_hi + (q_lo < a_lo ? 1 : 0);
    // |t| * 2^64 = Q * 2^(e+1): shift right by s in [42, 105]
    const int s = -(e + 1);
    uint64_t r_hi, r_lo;
    if (s >= 64) {
        r_lo = q_hi >> (s - 64);
        r_hi = 0;
    } else {
        r_lo = (q_lo >> s) | (q_hi << (64 - s));
        r_hi = q_hi >> s;
    }
    int k = static_cast<int>(r_hi);
    uint64_t F = r_lo;
    if (neg) {
        if (F != 0) {
            F = 0 - F;
            k = -k - 1;
        } else {
            k = -k;
        }
    }
    // 2^(F * 2^-64) in Q63
    const int i1 = static_cast<int>(F >> 58);
    const int i2 = static_cast<int>((F >> 52) & 63);
    const uint64_t G = F & 0x000fffffffffffffULL;
    const uint64_t U = wr_umulhi(G << 11, WR_LN2_Q64);  // u * 2^75
    const uint64_t u2 = wr_umulhi(U, U);                // u^2 * 2^86
    const uint64_t u3 = wr_umulhi(u2, U);               // u^3 * 2^97
    const uint64_t u4 = wr_umulhi(u2, u2);              // u^4 * 2^108
    const uint64_t inv6 = static_cast<uint64_t>(WR_INV6_Q62);
    const uint64_t p = (U >> 11) + (u2 >> 23) + (wr_umulhi(u3, inv6) >> 31) + (wr_umulhi(u4, inv6) >> 44);
    const uint64_t t1 = WR_TAB(exp_t1)[i1];
    const uint64_t t2 = WR_TAB(exp_t2)[i2];
    const uint64_t s12 = (wr_umulhi(t1, t2) << 1) | ((t1 * t2) >> 63);
    uint64_t R = s12 + wr_umulhi(s12, p);
    if (R < s12) R = 0xffffffffffffffffULL;  // 2^f within a few units of 2
    const int be = k + 1023;
    if (be >= 1) {
        uint64_t mant = R >> 11;
        const uint64_t rem = R & 0x7ff;
        mant += (rem > 0x400 || (rem == 0x400 && (mant & 1))) ? 1 : 0;
        int b = be;
        if (mant >> 53) {
            mant >>= 1;
            b += 1;
        }
        if (b >= 2047) return wr_from_bits(0x7ff0000000000000ULL);
        return wr_from_bits((static_cast<uint64_t>(b) << 52) | (mant & 0x000fffffffffffffULL));
    }
    // subnormal or zero: value = R * 2^(k-63) = (R >> sh) units of 2^-1074
    const int sh = -(k + 1011);
    if (sh > 64) return 0.0;
    uint64_t qv, rm, half;
    if (sh == 64) {
        qv = 0;
        rm = R;
        half = 0x8000000000000000ULL;
    } else {
        qv = R >> sh;
        rm = R & ((1ULL << sh) - 1);
        half = 1ULL << (sh - 1);
    }
    qv += (rm > half || (rm == half && (qv & 1))) ? 1 : 0;
    return wr_from_bits(qv);
}

WR_MHD double wr_log(double x) {
    const uint64_t u = wr_bits(x);
    if (u >= 0x7ff0000000000000ULL || u == 0) {
        const uint64_t ax = u & 0x7fffffffffffffffULL;
        if (ax > 0x7ff0000000000000ULL) return x + x;                   // NaN
        if (ax == 0) return wr_from_bits(0xfff0000000000000ULL);         // +-0 -> -inf
        if (u == 0x7ff0000000000000ULL) return x;                        // +inf
        return wr_from_bits(0x7ff8000000000000ULL);                      // x < 0
    }
    int E;
    uint64_t M;
    if (u < 0x0010000000000000ULL) {  // subnormal
        const int n = wr_clz64(u) - 11;
        M = u << n;
        E = -1022 - n;
    } else {
        E = static_cast<int>(u >> 52) - 1023;
        M = (u & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    }
    const int i = static_cast<int>((M >> 43) & 511);
    const uint64_t r = WR_TAB(log_r)[i];
    const int64_t Z = static_cast<int64_t>(M * r - 0x8000000000000000ULL);  // z * 2^63
    const int64_t Z1 = Z * 512;                                             // z * 2^72
    int64_t h = WR_INV6_Q62 - (wr_smulhi(Z1, WR_INV7_Q62) >> 8);
    h = WR_INV5_Q62 - (wr_smulhi(Z1, h) >> 8);
    h = WR_INV4_Q62 - (wr_smulhi(Z1, h) >> 8);
    h = WR_INV3_Q62 - (wr_smulhi(Z1, h) >> 8);
    h = WR_INV2_Q62 - (wr_smulhi(Z1, h) >> 8);
    h = WR_INV1_Q62 - (wr_smulhi(Z1, h) >> 8);
    // log1p(z) = z * h as signed Q125
    const int64_t p_hi = wr_smulhi(Z, h);
    const uint64_t p_lo = static_cast<uint64_t>(Z) * static_cast<uint64_t>(h);
    if ((E == 0 && i == 0) || (E == -1 && i == 511)) return wr_fixed_to_double(p_hi, p_lo, 125);
    // S = E*ln2 - log(r/2048) + log1p(z) in signed Q96
    const uint64_t ae = static_cast<uint64_t>(E < 0 ? -E : E);
    uint64_t e_lo = ae * WR_LN2_Q96_LO;
    uint64_t e_hi = wr_umulhi(ae, WR_LN2_Q96_LO) + ae * WR_LN2_Q96_HI;
    if (E < 0) {
        e_lo = ~e_lo + 1;
        e_hi = ~e_hi + (e_lo == 0 ? 1 : 0);
    }
    const uint64_t n_hi = WR_TAB(log_nl)[2 * i];
    const uint64_t n_lo = WR_TAB(log_nl)[2 * i + 1];
    const uint64_t l_lo = (p_lo >> 29) | (static_cast<uint64_t>(p_hi) << 35);
    const uint64_t l_hi = static_cast<uint64_t>(p_hi >> 29);
    uint64_t s_lo = e_lo + n_lo;
    uint64_t s_hi = e_hi + n_hi + (s_lo < e_lo ? 1 : 0);
    const uint64_t s2 = s_lo + l_lo;
    s_hi += l_hi + (s2 < s_lo ? 1 : 0);
    return wr_fixed_to_double(static_cast<int64_t>(s_hi), s2, 96);
}

WR_MHD double wr_cbrt(double x) {
    const uint64_t u = wr_bits(x);
    const uint64_t ax = u & 0x7fffffffffffffffULL;
    if (ax >= 0x7ff0000000000000ULL || ax == 0) return x + x;  // inf, NaN, +-0
    double a = wr_from_bits(ax);
    double scale = 1.0;
    if (ax < 0x0010000000000000ULL) {  // subnormal: cbrt(a * 2^54) = cbrt(a) * 2^18
        a = a * 18014398509481984.0;
        scale = 1.0 / 262144.0;
    }
    const uint64_t b = wr_bits(a);
    double y = wr_from_bits(b / 3 + 0x2a9f800000000000ULL);
    const double third = 1.0 / 3.0;
    for (int it = 0; it < 4; ++it) y = y + (wr_div_int(a, y * y) - y) * third;
    y = y * scale;
    return (u >> 63) ? -y : y;
}
