// wr_coop.cuh -- the cooperative advance: G lanes per cell (G = 8, 16 or 32).
//
// advance_collapse_gridwide_kernel (reproducer.cpp:7736-7785) runs one thread per
// cell.  On GB300 a warp issues one FP64 instruction every ~64-76 cycles, so an
// FP64 instruction executed with few active lanes wastes the scarce pipe, and a
// lane-per-cell kernel whose lanes sit in different phases, or idle at the end of
// an outer step while the stiffest cells still iterate, runs far below the FP64
// rate.  Here a group of G lanes owns one cell and every lane of the warp executes
// the same instruction stream:
//
//  * the network (burn_state_from_y, the analytic Jacobian and the RHS) is a
//    generated vector program (gen/coop.py): each step every lane computes one DAG
//    node from operands in the cell's shared-memory slot array V; all add/sub/mul
//    are one fused-multiply-add class with exact neutral operands, so one FP64
//    instruction serves G nodes; comparisons, selects and boolean logic ride on
//    the integer pipe in the same steps;
//  * the 15x15 factorisation (lu_decomposition, reproducer.cpp:96-151) is
//    warp-cooperative: pivot search by a __shfl_xor_sync argmax over the group,
//    row interchange, scaling and the rank-1 update spread over the G lanes, the
//    matrix staged in shared memory (V[0..225));
//  * the triangular solves (lu_solve, :154-181) keep the vector distributed over
//    the group's lanes and broadcast each pivot element with __shfl_sync;
//  * stage combinations, the error norm and the step-size controller
//    (RODAS::integrate, :7205-7347) run per component on the lanes; scalars are
//    replicated in every lane of the group.
//
// A rejected attempt recomputes the Jacobian at the same state: the values are
// identical (same operations on the same operands), and the warp stays in one
// instruction stream; the Jacobian counter follows the reference's rule.  Every
// value is the same binary64 operation on the same operands as in the reference
// and the CPU oracle, so results are bit-identical.
//
// The prologue of the advance (driver update, density scaling, e from T) and the
// commit after a successful burn (renormalisation, T from e) are cell-parallel
// kernels around the burn (k_order_preburn, k_commit): lane-per-cell work at full
// SIMD width, out of the cooperative kernel's instruction stream.
#pragma once

#include <climits>

#include "wr_kernels.cuh"

namespace wr {

// qbucket states after k_order_preburn (>= 0 is a queue bucket, -1 not queued)
constexpr int kQSkip = -2;     // queued, but the prologue ended the cell's step
constexpr int kQBurn = -3;     // to be burned by the advance
constexpr int kQBurnOK = -4;   // burned successfully: k_commit commits it

namespace coop {

enum { C_NONE = 0, C_FMA = 1, C_EXP = 2, C_LOG = 3, C_SQRT = 4, C_DIV = 5 };
enum { I_SEL = 0, I_LE = 1, I_LT = 2, I_SGN = 3 };
// flags in the low three bits of the 16-bit byte-offset fields of a step
enum : uint32_t {
    FL_NEG = 1u, FL_ABS = 2u, FL_SWAP = 4u,  // X, Y: argument modifiers; Y: divide V[Y] ^ L by V[X]
    FL_INT = 1u, FL_SPECIAL = 2u,            // Z: integer nodes / comparisons or sign ops in the step
    FL_SABS = 4u                             // integer destination of I_SGN: clear the sign (else flip)
};
constexpr int kE = 0;        // iteration matrix slots [0, 225)
constexpr int kY = 225;      // program inputs y[0..14]
constexpr int kRes = 240;    // reserved constants [240, 240 + Tab::kNR + Tab::kNF)
constexpr uint32_t kOff = 0xfff8u;
constexpr uint64_t kSign = 0x8000000000000000ULL;
constexpr uint64_t kAbs = 0x7fffffffffffffffULL;
constexpr uint64_t kInfBits = 0x7ff0000000000000ULL;

__device__ __forceinline__ double dbl(uint64_t u) { return __longlong_as_double(static_cast<long long>(u)); }
__device__ __forceinline__ uint64_t bits(double d) { return static_cast<uint64_t>(__double_as_longlong(d)); }

// output operand (the RHS and Jacobian tables): slot (12 bits) | negate (bit 13) |
// abs (bit 14); constants sit in reserved slots
__device__ __forceinline__ uint64_t fetch(const uint64_t* V, uint32_t op) {
    uint64_t v = V[op & 0xfffu];
    v = (op & 0x4000u) ? (v & kAbs) : v;
    v = (op & 0x2000u) ? (v ^ kSign) : v;
    return v;
}

// Shared-memory access by 32-bit shared-window addresses (the interpreter runs out
// of line, where generic pointers would lose their address space).
__device__ __forceinline__ uint64_t lds64(uint32_t addr) {
    uint64_t v;
    asm volatile("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
    return v;
}
__device__ __forceinline__ void sts64(uint32_t addr, uint64_t v) {
    asm volatile("st.shared.b64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}
__device__ __forceinline__ void group_sync(unsigned gmask) {
    asm volatile("bar.warp.sync %0;" ::"r"(gmask) : "memory");
}
// sign modifiers of an exp/log/sqrt/div argument (abs, then negate)
__device__ __forceinline__ uint64_t modify(uint64_t v, uint32_t fl) {
    v = (fl & FL_ABS) ? (v & kAbs) : v;
    return (fl & FL_NEG) ? (v ^ kSign) : v;
}

// IEEE a <= b and a < b on bit patterns: false when either is NaN, -0 == +0
__device__ __forceinline__ uint64_t ble(uint64_t a, uint64_t b) {
    const uint64_t ma = a & kAbs, mb = b & kAbs;
    const bool nan = (ma > kInfBits) | (mb > kInfBits);
    const bool zero = (ma | mb) == 0;
    const bool sa = (a >> 63) != 0, sb = (b >> 63) != 0;
    const bool same = sa ? (ma >= mb) : (ma <= mb);
    return (!nan && (zero || (sa != sb ? sa : same))) ? 1ULL : 0ULL;
}
__device__ __forceinline__ uint64_t blt(uint64_t a, uint64_t b) {
    const uint64_t ma = a & kAbs, mb = b & kAbs;
    const bool nan = (ma > kInfBits) | (mb > kInfBits);
    const bool zero = (ma | mb) == 0;
    const bool sa = (a >> 63) != 0, sb = (b >> 63) != 0;
    const bool same = sa ? (ma > mb) : (ma < mb);
    return (!nan && !zero && (sa != sb ? sa : same)) ? 1ULL : 0ULL;
}

// Transcendental steps call one out-of-line copy each, so the interpreter loop
// stays small (CUDA's own functions inside for CudaMath).
template <class M>
struct StepMath {
    static __device__ __noinline__ double exp(double x) { return M::exp(x); }
    static __device__ __noinline__ double log(double x) { return M::log(x); }
    static __device__ __noinline__ double sqrt(double x) { return M::sqrt(x); }
};

// One step of one lane.  e.x: main word X | Y | Z | D (16-bit byte offsets into
// the cell's slot array at shared address vb, flags in their low three bits);
// e.y: integer word A | B | C | D2; lit: the lane's literal, XOR-ed into V[Y].
// An FMA step's operand offsets carry no flags (the generator guarantees it), so
// they are added to vb as they are.
template <class M>
__device__ __forceinline__ void exec_step(const ulonglong2 e, const uint64_t lit, uint32_t vb) {
    const uint32_t w0 = static_cast<uint32_t>(e.x), w1 = static_cast<uint32_t>(e.x >> 32);
    const uint32_t cls = (w1 >> 16) & 7u;
    const uint32_t dst = vb + ((w1 >> 16) & kOff);
    if (cls == C_FMA) {
        const double a = dbl(lds64(vb + (w0 & 0xffffu)));
        const double b = dbl(lds64(vb + (w0 >> 16)) ^ lit);
        const double c = dbl(lds64(vb + (w1 & kOff)));
        sts64(dst, bits(__fma_rn(a, b, c)));
    } else if (cls != C_NONE) {
        const uint32_t yf = w0 >> 16;
        const uint64_t y = modify(lds64(vb + (yf & kOff)) ^ lit, yf);
        double r;
        if (cls == C_DIV) {
            const uint64_t x = modify(lds64(vb + (w0 & kOff)), w0);
            const bool sw = (yf & FL_SWAP) != 0;
            r = ddiv(dbl(sw ? y : x), dbl(sw ? x : y));
        } else if (cls == C_EXP) {
            r = StepMath<M>::exp(dbl(y));
        } else if (cls == C_LOG) {
            r = StepMath<M>::log(dbl(y));
        } else {
            r = StepMath<M>::sqrt(dbl(y));
        }
        sts64(dst, bits(r));
    }
    if (w1 & FL_INT) {  // the step carries integer nodes (uniform over the warp)
        const uint32_t i0 = static_cast<uint32_t>(e.y), i1 = static_cast<uint32_t>(e.y >> 32);
        const uint64_t A = lds64(vb + (i0 & 0xffffu));
        const uint64_t B = lds64(vb + (i0 >> 16));
        const uint64_t C = lds64(vb + (i1 & 0xffffu));
        uint64_t r = A != 0 ? B : C;
        if (w1 & FL_SPECIAL) {  // comparisons or sign operations (uniform over the warp)
            const uint32_t iop = (i1 >> 16) & 3u;
            r = iop == I_LE ? ble(A, B) : r;
            r = iop == I_LT ? blt(A, B) : r;
            r = iop == I_SGN ? (((i1 >> 16) & FL_SABS) ? (A & kAbs) : (A ^ kSign)) : r;
        }
        sts64(vb + ((i1 >> 16) & kOff), r);
    }
}

// One generated program on the group's cell: the steps' words per lane; the group
// synchronises after every step.  One out-of-line copy serves every call site (the
// instruction cache holds one loop).  The step count is a multiple of four and the
// tables carry four idle steps more, so the loop runs four steps per iteration and
// loads each step's words four steps before it executes them (the tables, ~100-200
// KB per G, live mostly in L2: shared memory takes most of L1).
template <class M, int G>
__device__ __noinline__ void run_prog(const ulonglong2* __restrict__ prog, const uint64_t* __restrict__ lits,
                                      int nsteps, int gl, uint64_t* V, unsigned gmask) {
    const uint32_t vb = static_cast<uint32_t>(__cvta_generic_to_shared(V));
    const ulonglong2* p = prog + gl;
    const uint64_t* q = lits + gl;
    ulonglong2 e0 = __ldg(p), e1 = __ldg(p + G), e2 = __ldg(p + 2 * G), e3 = __ldg(p + 3 * G);
    uint64_t l0 = __ldg(q), l1 = __ldg(q + G), l2 = __ldg(q + 2 * G), l3 = __ldg(q + 3 * G);
#pragma unroll 1
    for (int s = 0; s < nsteps; s += 4) {
        p += 4 * G;
        q += 4 * G;
        exec_step<M>(e0, l0, vb);
        e0 = __ldg(p);
        l0 = __ldg(q);
        group_sync(gmask);
        exec_step<M>(e1, l1, vb);
        e1 = __ldg(p + G);
        l1 = __ldg(q + G);
        group_sync(gmask);
        exec_step<M>(e2, l2, vb);
        e2 = __ldg(p + 2 * G);
        l2 = __ldg(q + 2 * G);
        group_sync(gmask);
        exec_step<M>(e3, l3, vb);
        e3 = __ldg(p + 3 * G);
        l3 = __ldg(q + 3 * G);
        group_sync(gmask);
    }
}

// the reserved constants of the programs into the group's slot array (once per
// launch: no program writes them), then the exp/log/sqrt of constants, evaluated
// here with the kernel's own functions so that they are the bits a program step
// would compute
template <class M, int G, class Tab>
__device__ __forceinline__ void init_reserved(uint64_t* V, int gl, unsigned gmask) {
    for (int i = gl; i < Tab::kNR; i += G) V[kRes + i] = Tab::vconst()[i];
    for (int i = gl; i < Tab::kNF; i += G) {
        const ulonglong2 f = Tab::vfun()[i];
        const double a = dbl(f.y);
        const double r = f.x == C_EXP ? StepMath<M>::exp(a) : f.x == C_LOG ? StepMath<M>::log(a) : StepMath<M>::sqrt(a);
        V[kRes + Tab::kNR + i] = bits(r);
    }
    __syncwarp(gmask);
}

// lu_decomposition<15> (reproducer.cpp:96-151) by the G lanes of a group on the
// matrix E[r*15 + c] in shared memory: the same pivot (first strictly largest
// |a_ik|, a NaN diagonal keeps its row), the same row interchange, negated
// multipliers and rank-1 update, each element the same two roundings.
template <int G>
__device__ __forceinline__ int lu_coop(double* E, int gl, unsigned gmask, uint64_t& ip) {
    constexpr int K = (NEQ + G - 1) / G;
    int info = 0;
    uint64_t piv = 0;
#pragma unroll 1
    for (int k = 0; k < NEQ - 1; ++k) {
        long long key = -1;
        int idx = NEQ;
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int r = gl + t * G;
            if (r >= k && r < NEQ) {
                const uint64_t u = bits(E[r * NEQ + k]) & kAbs;
                const long long kk = u > kInfBits ? (r == k ? LLONG_MAX : -1LL) : static_cast<long long>(u);
                if (kk > key) {
                    key = kk;
                    idx = r;
                }
            }
        }
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) {
            const long long ok = __shfl_xor_sync(gmask, key, off, G);
            const int oi = __shfl_xor_sync(gmask, idx, off, G);
            if (ok > key || (ok == key && oi < idx)) {
                key = ok;
                idx = oi;
            }
        }
        const int p = idx;
        piv |= static_cast<uint64_t>(p) << (4 * k);
        if (E[p * NEQ + k] != 0.0) {
            if (p != k) {
#pragma unroll
                for (int t = 0; t < K; ++t) {
                    const int j = k + gl + t * G;
                    if (j < NEQ) {
                        const double tmp = E[p * NEQ + j];
                        E[p * NEQ + j] = E[k * NEQ + j];
                        E[k * NEQ + j] = tmp;
                    }
                }
                __syncwarp(gmask);
            }
            const double mult = ddiv(-1.0, E[k * NEQ + k]);
#pragma unroll
            for (int t = 0; t < K; ++t) {
                const int i = k + 1 + gl + t * G;
                if (i < NEQ) E[i * NEQ + k] = E[i * NEQ + k] * mult;
            }
            __syncwarp(gmask);
            const int m = NEQ - 1 - k;
            const unsigned cm = (65536u + static_cast<unsigned>(m) - 1u) / static_cast<unsigned>(m);
#pragma unroll 1
            for (int e = gl; e < m * m; e += G) {
                const int ii = static_cast<int>((static_cast<unsigned>(e) * cm) >> 16);
                const int i = k + 1 + ii;
                const int j = k + 1 + (e - ii * m);
                E[i * NEQ + j] = E[i * NEQ + j] + E[k * NEQ + j] * E[i * NEQ + k];
            }
        } else {
            info = k + 1;
        }
        __syncwarp(gmask);
    }
    piv |= static_cast<uint64_t>(NEQ - 1) << (4 * (NEQ - 1));
    if (E[(NEQ - 1) * NEQ + NEQ - 1] == 0.0) info = NEQ;
    ip = piv;
    return info;
}

// component c of a vector distributed over the group: lane c % G, register c / G
// (c is uniform over the group; the register is picked by a select, so the
// array stays in registers)
template <int G, int K, class T>
__device__ __forceinline__ T get(const T (&x)[K], int c, unsigned gmask) {
    T v = x[0];
#pragma unroll
    for (int t = 1; t < K; ++t) v = (c / G == t) ? x[t] : v;
    return __shfl_sync(gmask, v, c % G, G);
}

// the reciprocals of the factorisation's diagonal for the back substitutions
// (wr_div_recip of U(c, c), distributed like a vector): the three stage solves
// of an attempt divide by the same 15 pivots
template <int G, int K>
__device__ __forceinline__ void diag_recips(const double* LU, uint64_t (&rY)[K], int gl) {
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        rY[t] = c < NEQ ? wr_div_recip(LU[c * NEQ + c]) : 0;
    }
}

// lu_solve<15> (reproducer.cpp:154-181) with x distributed over the group; the
// back substitution's quotients use the pivots' precomputed reciprocals (the same
// IEEE quotients as a division)
template <int G, int K>
__device__ __forceinline__ void solve_coop(const double* LU, uint64_t ip, const uint64_t (&rY)[K], double (&x)[K],
                                           int gl, unsigned gmask) {
#pragma unroll 1
    for (int k = 0; k < NEQ - 1; ++k) {
        const int p = static_cast<int>((ip >> (4 * k)) & 15);
        if (p != k) {
            const double xk = get<G, K>(x, k, gmask);
            const double xp = get<G, K>(x, p, gmask);
#pragma unroll
            for (int t = 0; t < K; ++t) {
                const int c = gl + t * G;
                x[t] = c == k ? xp : (c == p ? xk : x[t]);
            }
        }
        const double tk = get<G, K>(x, k, gmask);
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int c = gl + t * G;
            if (c > k && c < NEQ) x[t] = x[t] + tk * LU[c * NEQ + k];
        }
    }
#pragma unroll 1
    for (int k = NEQ - 1; k >= 0; --k) {
        const uint64_t yk = get<G, K>(rY, k, gmask);
        const double q = ddiv_recip(get<G, K>(x, k, gmask), LU[k * NEQ + k], yk);
        const double tk = -q;
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int c = gl + t * G;
            if (c == k) x[t] = q;
            if (c < k) x[t] = x[t] + tk * LU[c * NEQ + k];
        }
    }
}

template <int G, int K>
__device__ __forceinline__ void store_inputs(uint64_t* V, const double (&v)[K], int gl) {
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        if (c < NEQ) V[kY + c] = bits(v[t]);
    }
}

template <int G, int K>
__device__ __forceinline__ void load_outputs(const uint64_t* V, const uint16_t* out, double (&v)[K], int gl) {
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        v[t] = c < NEQ ? dbl(fetch(V, out[c])) : 0.0;
    }
}

// E = -J into the matrix slots after the Jacobian program.  The program uses the
// matrix slots as scratch and keeps its results (the Jacobian entries and the
// RHS) above them; the generated table names, per matrix entry r * 15 + c, the
// slot (a reserved one for a constant entry) that holds J(r, c) with the negation
// as an operand modifier.
template <int G>
__device__ __forceinline__ void gather_matrix(uint64_t* V, const uint16_t* jac, int gl, unsigned gmask) {
#pragma unroll 1
    for (int i = gl; i < NEQ * NEQ; i += G) V[kE + i] = fetch(V, jac[i]);
    __syncwarp(gmask);
}

// Generated tables of one G, supplied by the translation unit that includes the
// generated header (one unit per G keeps the large initialisers apart).
//   Tab::kNV, Tab::kNR, Tab::kNF, Tab::kJSteps, Tab::kRSteps and device accessors
//   jprog(), jlit(), rprog(), rlit(), jout(), jac(), rout(), vconst(), vfun().

}  // namespace coop

// Phase counters (a diagnostic, wr_diag_coop_phases): the instrumented
// instantiation adds, per warp, the clock64 cycles of each phase of its attempts
// into 16 device counters: [0] queue, prologue and epilogue, [1] Jacobian+RHS
// program, [2] output loads, Jacobian gather, diagonal and stage combinations,
// [3] LU, [4] stage solves, [5] RHS programs, [6] error norm and controller,
// [7] attempts, [8] cycles from start to exit, [9] warps.  The plain
// instantiation compiles every call to nothing.
enum { PH_QUEUE = 0, PH_JPROG = 1, PH_MISC = 2, PH_LU = 3, PH_SOLVE = 4, PH_RPROG = 5, PH_CTL = 6 };
__device__ __forceinline__ long long phase_now() {
#if defined(__CUDA_ARCH__)
    return clock64();
#else
    return 0;
#endif
}
template <bool ON>
struct PhaseClock {
    __device__ __forceinline__ void mark(int) {}
    __device__ __forceinline__ void attempt() {}
    __device__ __forceinline__ void flush(unsigned long long*, int) {}
};
template <>
struct PhaseClock<true> {
    long long acc[7] = {0, 0, 0, 0, 0, 0, 0};
    long long t0, t, attempts = 0;
    __device__ __forceinline__ PhaseClock() : t0(phase_now()), t(t0) {}
    __device__ __forceinline__ void mark(int k) {
        const long long now = phase_now();
        acc[k] += now - t;
        t = now;
    }
    __device__ __forceinline__ void attempt() { ++attempts; }
    __device__ __forceinline__ void flush(unsigned long long* out, int lane) {
        mark(PH_QUEUE);
        if (lane != 0 || out == nullptr) return;
#pragma unroll
        for (int k = 0; k < 7; ++k) atomicAdd(out + k, static_cast<unsigned long long>(acc[k]));
        atomicAdd(out + 7, static_cast<unsigned long long>(attempts));
        atomicAdd(out + 8, static_cast<unsigned long long>(phase_now() - t0));
        atomicAdd(out + 9, 1ULL);
    }
};

// The cooperative burn: persistent blocks of W warps, G lanes per cell, each group
// taking cells from the work queue until it is empty.  PH: the phase-counting
// instantiation (phases: its 16 counters).
template <class M, int G, int W, class Tab, bool PH = false>
__global__ void __launch_bounds__(W * 32, 1) k_advance_coop(DevState s, StepCtl* ctl, unsigned long long* phases) {
    using namespace coop;
    constexpr int K = (NEQ + G - 1) / G;
    constexpr int SLOTS = 32 / G;
    extern __shared__ uint64_t sm[];
    if (ctl->all_stop) return;
    const int lane = threadIdx.x & 31;
    const int slot = lane / G;
    const int gl = lane % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (slot * G));
    uint64_t* V = sm + static_cast<size_t>((threadIdx.x >> 5) * SLOTS + slot) * Tab::kNV;
    double* E = reinterpret_cast<double*>(V + kE);
    init_reserved<M, G, Tab>(V, gl, gmask);
    const int n = s.n;
    const unsigned int queued = ctl->queued;

    PhaseClock<PH> pc;
    Lane L;
    int cell = -1, g = 0;
    bool have = false;
    double y[K], f0[K], ak1[K], ak2[K], w[K];
#pragma unroll
    for (int t = 0; t < K; ++t) y[t] = f0[t] = ak1[t] = ak2[t] = w[t] = 0.0;
    uint64_t ip = 0;

#pragma unroll 1
    while (true) {
        // ---- bring the group's cell to "ready for an attempt" (per group)
        bool exhausted = false;
#pragma unroll 1
        while (true) {
            if (!have) {
                unsigned int q = 0;
                if (gl == 0) q = atomicAdd(&ctl->queue, 1u);
                q = __shfl_sync(gmask, q, 0, G);
                if (q >= queued) {
                    exhausted = true;
                    break;
                }
                cell = s.order[q];
                if (s.qbucket[cell] != kQBurn) continue;
                g = s.grid_of ? s.grid_of[cell] : 0;
                const double dt_grid = s.local_dt ? s.local_dt[cell] : ctl[g].dt_grid;
#pragma unroll
                for (int t = 0; t < K; ++t) {
                    const int c = gl + t * G;
                    y[t] = c < NS ? s.xn[c * n + cell] : (c == NS ? s.e[cell] : 0.0);
                }
                // RODAS::integrate prologue, reproducer.cpp:7218-7235
                L.tout = dt_grid;
                L.x = 0.0;
                double h0 = dt_grid;
                if (::fabs(h0) <= 10.0 * kUround) h0 = 1.e-6;
                L.h = smin(::fabs(h0), dt_grid);
                L.reject = false;
                L.last = false;
                L.nsing = 0;
                L.hacc = 0.0;
                L.erracc = 1.0;
                L.hopt = L.h;
                L.n_step = L.n_accept = L.n_reject = L.n_jac = L.n_decomp = 0;
                L.fresh = true;
                have = true;
            }
            if (!L.fresh) break;
            // outer-loop checks, reproducer.cpp:7236-7255
            int code = 0;
            if (L.n_step > kMaxSteps) code = WR_TOO_MANY_STEPS;
            else if (0.1 * ::fabs(L.h) <= ::fabs(L.x) * kUround) code = WR_DT_UNDERFLOW;
            else if (L.last) code = WR_SUCCESS;
            if (code != 0) {
                // burn_ros2s epilogue: counters, then the state (success) or the code
                if (gl == 0) {
                    const uint64_t st[7] = {
                        static_cast<uint64_t>(L.n_step), static_cast<uint64_t>(3 * L.n_step),
                        static_cast<uint64_t>(L.n_jac), static_cast<uint64_t>(L.n_decomp),
                        static_cast<uint64_t>(3 * L.n_step), static_cast<uint64_t>(L.n_accept),
                        static_cast<uint64_t>(L.n_reject)};
#pragma unroll
                    for (int k = 0; k < 7; ++k) s.stats[k * n + cell] += st[k];
                    s.cost[cell] = L.n_step;
                    if (code != WR_SUCCESS) record_failure(ctl + g, code);
                }
                if (code == WR_SUCCESS) {
#pragma unroll
                    for (int t = 0; t < K; ++t) {
                        const int c = gl + t * G;
                        if (c < NS) s.xn[c * n + cell] = y[t];
                        else if (c == NS) s.e[cell] = y[t];
                    }
                    if (gl == 0) s.qbucket[cell] = kQBurnOK;
                }
                have = false;
                continue;
            }
            L.hopt = L.h;
            if (L.x + L.h * 1.0001 >= L.tout) {
                L.h = L.tout - L.x;
                L.last = true;
            }
            break;
        }
        if (exhausted) break;
        pc.mark(PH_QUEUE);
        pc.attempt();

        // ---- one ROS2S attempt, reproducer.cpp:7259-7345
        store_inputs<G, K>(V, y, gl);
        __syncwarp(gmask);
        run_prog<M, G>(Tab::jprog(), Tab::jlit(), Tab::kJSteps, gl, V, gmask);
        pc.mark(PH_JPROG);
        load_outputs<G, K>(V, Tab::jout(), f0, gl);
        gather_matrix<G>(V, Tab::jac(), gl, gmask);
        if (L.fresh) L.n_jac += 1;
        L.fresh = false;
        const double h = L.h;
        const double fac = ddiv(1.0, h * kGamma);
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int c = gl + t * G;
            if (c < NEQ) E[c * NEQ + c] = E[c * NEQ + c] + fac;
        }
        __syncwarp(gmask);
        pc.mark(PH_MISC);
        const int info = lu_coop<G>(E, gl, gmask, ip);
        if (info != 0) {
            L.nsing += 1;
            if (L.nsing >= 5) {
                if (gl == 0) {
                    const uint64_t st[7] = {
                        static_cast<uint64_t>(L.n_step), static_cast<uint64_t>(3 * L.n_step),
                        static_cast<uint64_t>(L.n_jac), static_cast<uint64_t>(L.n_decomp),
                        static_cast<uint64_t>(3 * L.n_step), static_cast<uint64_t>(L.n_accept),
                        static_cast<uint64_t>(L.n_reject)};
#pragma unroll
                    for (int k = 0; k < 7; ++k) s.stats[k * n + cell] += st[k];
                    s.cost[cell] = L.n_step;
                    record_failure(ctl + g, WR_LU_DECOMPOSITION_ERROR);
                }
                have = false;
            } else {
                L.h = h * 0.5;
                L.reject = true;
                L.last = false;
            }
            __syncwarp(gmask);
            continue;
        }
        L.n_decomp += 1;
        uint64_t rY[K];
        diag_recips<G, K>(E, rY, gl);
        pc.mark(PH_LU);
#pragma unroll
        for (int t = 0; t < K; ++t) ak1[t] = f0[t];
        solve_coop<G, K>(E, ip, rY, ak1, gl, gmask);
        pc.mark(PH_SOLVE);
        // stage 2
        {
            double yn[K];
            const double c21h = ddiv(kC21, h);
#pragma unroll
            for (int t = 0; t < K; ++t) {
                yn[t] = y[t] + kA21 * ak1[t];
                w[t] = c21h * ak1[t];
            }
            store_inputs<G, K>(V, yn, gl);
            __syncwarp(gmask);
            pc.mark(PH_MISC);
            run_prog<M, G>(Tab::rprog(), Tab::rlit(), Tab::kRSteps, gl, V, gmask);
            pc.mark(PH_RPROG);
            double dy[K];
            load_outputs<G, K>(V, Tab::rout(), dy, gl);
#pragma unroll
            for (int t = 0; t < K; ++t) w[t] += dy[t];
            pc.mark(PH_MISC);
            solve_coop<G, K>(E, ip, rY, w, gl, gmask);
            pc.mark(PH_SOLVE);
#pragma unroll
            for (int t = 0; t < K; ++t) ak2[t] = w[t];
        }
        // stage 3
        {
            double yn[K];
#pragma unroll
            for (int t = 0; t < K; ++t) {
                yn[t] = y[t] + kA31 * ak1[t] + kA32 * ak2[t];
                w[t] = ddiv(kC31 * ak1[t] + kC32 * ak2[t], h);
            }
            __syncwarp(gmask);  // every lane has read the stage-2 outputs
            store_inputs<G, K>(V, yn, gl);
            __syncwarp(gmask);
            pc.mark(PH_MISC);
            run_prog<M, G>(Tab::rprog(), Tab::rlit(), Tab::kRSteps, gl, V, gmask);
            pc.mark(PH_RPROG);
            double dy[K];
            load_outputs<G, K>(V, Tab::rout(), dy, gl);
#pragma unroll
            for (int t = 0; t < K; ++t) w[t] += dy[t];
            pc.mark(PH_MISC);
            solve_coop<G, K>(E, ip, rY, w, gl, gmask);
            pc.mark(PH_SOLVE);
        }
        // w = k3: candidate and error estimate, reproducer.cpp:7299-7304
        double ynew[K], sq[K];
#pragma unroll
        for (int t = 0; t < K; ++t) {
            const int c = gl + t * G;
            const double ak3 = w[t];
            ynew[t] = y[t] + kB1 * ak1[t] + kB2 * ak2[t] + ak3;
            const double wi = kE1 * ak1[t] + kE2 * ak2[t] + kE3 * ak3;
            const double rtol = c < NS ? kRtolSpec : kRtolEnergy;
            const double atol = c < NS ? kAtolSpec : kAtolEnergy;
            const double sk = atol + rtol * smax(::fabs(y[t]), ::fabs(ynew[t]));
            const double term = ddiv(wi, sk);
            sq[t] = term * term;
        }
        // err = sum over components in index order (0.0 + sq[0] == sq[0]: a square)
        double err = get<G, K>(sq, 0, gmask);
#pragma unroll
        for (int c = 1; c < NEQ; ++c) err = err + get<G, K>(sq, c, gmask);
        err = ::sqrt(ddiv(err, 15.0));
        L.n_step += 1;
        // step-size controller, reproducer.cpp:7308-7344
        const double raw_fac = ddiv(M::cbrt(err), kSafe);
        const double fac_step = smax(1.0 / kFacMax, smin(1.0 / kFacMin, raw_fac));
        double hnew = ddiv(h, fac_step);
        if (err <= 1.0) {
            L.n_accept += 1;
            if (L.n_accept > 1) {
                const double facgus = smax(1.0 / kFacMax,
                    smin(1.0 / kFacMin, ddiv(ddiv(L.hacc, h) * M::cbrt(ddiv(err * err, L.erracc)), kSafe)));
                hnew = ddiv(h, smax(fac_step, facgus));
            }
            L.hacc = h;
            L.erracc = smax(1.e-2, err);
#pragma unroll
            for (int t = 0; t < K; ++t) y[t] = ynew[t];
            L.x += h;
            const double hmaxn = L.tout;
            if (::fabs(hnew) > hmaxn) hnew = hmaxn;
            if (L.reject) hnew = smin(::fabs(hnew), ::fabs(h));
            L.reject = false;
            L.h = hnew;
            L.fresh = true;
        } else {
            L.reject = true;
            L.last = false;
            L.h = hnew;
            if (L.n_accept >= 1) L.n_reject += 1;
            if (hnew == 0.0) {
                // the reject loop's only exit besides acceptance: a step size that
                // has underflowed to zero ends the cell with the reference's
                // DT_UNDERFLOW (reproducer.cpp:7240) instead of retrying forever
                if (gl == 0) {
                    const uint64_t st[7] = {
                        static_cast<uint64_t>(L.n_step), static_cast<uint64_t>(3 * L.n_step),
                        static_cast<uint64_t>(L.n_jac), static_cast<uint64_t>(L.n_decomp),
                        static_cast<uint64_t>(3 * L.n_step), static_cast<uint64_t>(L.n_accept),
                        static_cast<uint64_t>(L.n_reject)};
#pragma unroll
                    for (int k = 0; k < 7; ++k) s.stats[k * n + cell] += st[k];
                    s.cost[cell] = L.n_step;
                    record_failure(ctl + g, WR_DT_UNDERFLOW);
                }
                have = false;
            }
        }
        __syncwarp(gmask);  // the next attempt overwrites V: every lane is done with it
        pc.mark(PH_CTL);
    }
    pc.flush(phases, lane);
}

// ---------------------------------------------------------------- diagnostics
// The generated programs and the cooperative LU/solve on caller-supplied inputs
// (include/warp_reactor_diag.h), one group of G lanes per case.
template <class M, int G, class Tab>
__global__ void k_diag_coop_network(int n, const double* __restrict__ y, double* J, double* f, double* f2) {
    using namespace coop;
    constexpr int K = (NEQ + G - 1) / G;
    constexpr int SLOTS = 32 / G;
    extern __shared__ uint64_t sm[];
    const int lane = threadIdx.x & 31, slot = lane / G, gl = lane % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (slot * G));
    const int warp = threadIdx.x >> 5;
    const int cell = (blockIdx.x * (blockDim.x >> 5) + warp) * SLOTS + slot;
    if (cell >= n) return;
    uint64_t* V = sm + static_cast<size_t>(warp * SLOTS + slot) * Tab::kNV;
    const double* E = reinterpret_cast<const double*>(V + kE);
    init_reserved<M, G, Tab>(V, gl, gmask);
    double yy[K], out[K];
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        yy[t] = c < NEQ ? y[static_cast<size_t>(cell) * NEQ + c] : 0.0;
    }
    store_inputs<G, K>(V, yy, gl);
    __syncwarp(gmask);
    run_prog<M, G>(Tab::jprog(), Tab::jlit(), Tab::kJSteps, gl, V, gmask);
    load_outputs<G, K>(V, Tab::jout(), out, gl);
    gather_matrix<G>(V, Tab::jac(), gl, gmask);
    for (int i = gl; i < NEQ * NEQ; i += G) J[static_cast<size_t>(cell) * NEQ * NEQ + i] = -E[i];
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        if (c < NEQ) f[static_cast<size_t>(cell) * NEQ + c] = out[t];
    }
    __syncwarp(gmask);
    store_inputs<G, K>(V, yy, gl);
    __syncwarp(gmask);
    run_prog<M, G>(Tab::rprog(), Tab::rlit(), Tab::kRSteps, gl, V, gmask);
    load_outputs<G, K>(V, Tab::rout(), out, gl);
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        if (c < NEQ) f2[static_cast<size_t>(cell) * NEQ + c] = out[t];
    }
}

template <int G>
__global__ void k_diag_coop_lu(int n, const double* __restrict__ A, const double* __restrict__ b, double* LU,
                               int* ipvt, int* info, double* x) {
    using namespace coop;
    constexpr int K = (NEQ + G - 1) / G;
    constexpr int SLOTS = 32 / G;
    extern __shared__ uint64_t sm[];
    const int lane = threadIdx.x & 31, slot = lane / G, gl = lane % G;
    const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (slot * G));
    const int warp = threadIdx.x >> 5;
    const int cell = (blockIdx.x * (blockDim.x >> 5) + warp) * SLOTS + slot;
    if (cell >= n) return;
    double* E = reinterpret_cast<double*>(sm) + static_cast<size_t>(warp * SLOTS + slot) * NEQ * NEQ;
    for (int i = gl; i < NEQ * NEQ; i += G) E[i] = A[static_cast<size_t>(cell) * NEQ * NEQ + i];
    __syncwarp(gmask);
    uint64_t ip = 0;
    const int inf = lu_coop<G>(E, gl, gmask, ip);
    double v[K];
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        v[t] = c < NEQ ? b[static_cast<size_t>(cell) * NEQ + c] : 0.0;
    }
    if (inf == 0) {
        uint64_t rY[K];
        diag_recips<G, K>(E, rY, gl);
        solve_coop<G, K>(E, ip, rY, v, gl, gmask);
    }
    __syncwarp(gmask);
    for (int i = gl; i < NEQ * NEQ; i += G) LU[static_cast<size_t>(cell) * NEQ * NEQ + i] = E[i];
#pragma unroll
    for (int t = 0; t < K; ++t) {
        const int c = gl + t * G;
        if (c < NEQ) {
            x[static_cast<size_t>(cell) * NEQ + c] = v[t];
            ipvt[static_cast<size_t>(cell) * NEQ + c] = static_cast<int>((ip >> (4 * c)) & 15);
        }
    }
    if (gl == 0) info[cell] = inf;
}

}  // namespace wr
