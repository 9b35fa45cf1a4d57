// One exact step of rebop's direct method for the thread-per-trajectory
// kernels: binary64 work in exact integer emulation (b64.cuh), running sums
// and the clock add on the FP64 pipe, comparisons of non-negative doubles as
// integer comparisons, and a per-lane fallback to native binary64 for anything
// outside the emulation's domain.  Results equal rebop's, bit for bit:
//   propensity  rate * x_1 * x_2 ... (gillespie.rs:73-86), or the macro's
//               rate * ff_1 * ff_2 ... (gillespie_macro.rs:106, :133-146)
//   cumulative  cum_r = total + a_r (gillespie.rs:357-364)
//   absorb      !(0 < total): no draw, the step records (gillespie.rs:323-326)
//   clock       t + Exp1 / total; past the sample time the draw is discarded
//               (gillespie.rs:327-331)
//   choice      #{r : cum_r < total * U} (gillespie.rs:402-407), or the
//               macro's first r with total * U < cum_r (gillespie_macro.rs:159)
#pragma once

#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#endif

#include "b64.cuh"
#include "rng.cuh"
#include "ssa_args.hpp"

namespace rbg {

constexpr uint64_t kOneBits = 0x3FF0000000000000ull;

// Block-wide tables in shared memory.
struct ExactTables {
    const ulonglong2 *zxk;  // [256] {x[i] bits, K_i}
    const uint64_t *zf;     // [257] f bits
    const uint64_t *zd;     // [256] |f[i] - f[i+1]| bits
    const int32_t *fac;     // [R*P] species | order << 16
    const int32_t *jsp;     // [R*Q]
    const int64_t *jd;      // [R*Q]
};

// Truncated float32 of a positive normal double (bits) in float range.
__device__ __forceinline__ float f32_rz(uint64_t v) {
    const uint32_t e = (uint32_t)(v >> 52) - 1023u + 127u;
    return __uint_as_float((e << 23) | ((uint32_t)(v >> 29) & 0x7FFFFFu));
}

// +0 or positive normal: the integer emulation's domain.
__device__ __forceinline__ bool emul_domain(uint64_t v) {
    const uint64_t e = v >> 52;
    return v == 0 || (e >= 1 && e <= 2046);
}

// Wedge test of the ziggurat, f[i+1] + (f[i] - f[i+1]) U < exp(-x) with
// f[i] < f[i+1], decided in float32 unless the operands fall within 2^-17 of
// each other (float32 errors here stay below 2e-6 relative); inside that band
// the exact binary64 operands decide.  `x` is the exact candidate abscissa.
__device__ __forceinline__ bool wedge_accept(const ExactTables &m, int i, uint64_t x, uint64_t mu, bool &bad) {
    const uint64_t w = b64::sub(m.zf[i + 1], b64::mul_u64(m.zd[i], mu, 53, bad), bad);
    const float wf = f32_rz(w), ef = expf(-f32_rz(x));
    if (wf < ef * (1.0f - 0x1p-17f)) return true;
    if (wf > ef * (1.0f + 0x1p-17f)) return false;
    return __longlong_as_double((long long)w) < exp(-__longlong_as_double((long long)x));
}

// Exp1 draw (ziggurat, rng.cuh) with exact integer arithmetic.
__device__ __forceinline__ uint64_t exp1_emul(Xoshiro &g, const ExactTables &m, bool &bad) {
    for (;;) {
        const uint64_t b = xo_next(g);
        const int i = (int)(b & 0xff);
        const uint64_t k = b >> 12;
        const ulonglong2 e = m.zxk[i];
        const uint64_t x = b64::mul_u64(e.x, 2 * k + 1, 53, bad);
        if (k < e.y) return x;
        if (i == 0) return (uint64_t)__double_as_longlong(__dsub_rn(kZigR, log(xo_uniform(g))));
        if (wedge_accept(m, i, x, xo_next(g) >> 11, bad)) return x;
    }
}

// One step in native binary64 from the committed state.  Returns true when a
// reaction fires (index and new clock out); commits the draws it consumes.
template <int MAXR, bool MACRO>
__device__ __noinline__ bool native_step(const SsaArgs &a, const ExactTables &m, Xoshiro &g, const int64_t *sp,
                                         const uint64_t *rl, int RS, int BD, uint64_t t_bits, uint64_t T_bits, int &idx,
                                         uint64_t &tn_bits) {
    double cum[MAXR];
    double total = 0.0;
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        if (r < a.R) {
            double acc = __longlong_as_double((long long)rl[r * RS]);
            for (int p = 0; p < a.P; ++p) {
                const int f = m.fac[r * a.P + p];
                const int o = f >> 16;
                if (o == 0) continue;
                const int64_t n = sp[(f & 0xFFFF) * BD];
                if (MACRO) {
                    int64_t ff = n;
                    for (int j = 1; j < o; ++j) ff *= n - j;
                    acc = __dmul_rn(acc, (double)ff);
                } else {
                    for (int j = o - 1; j >= 0; --j) acc = __dmul_rn(acc, (double)(n - j));
                }
            }
            total = __dadd_rn(total, acc);
            cum[r] = total;
        }
    }
    if (!(0.0 < total)) return false;
    const double t = __longlong_as_double((long long)t_bits), T = __longlong_as_double((long long)T_bits);
    const double tn = __dadd_rn(t, __ddiv_rn(xo_exp1(g, a.zig, a.zig + kZigOffF), total));
    if (tn > T) return false;
    const double chosen = __dmul_rn(total, xo_uniform(g));
    if (MACRO) {
        idx = a.R;
#pragma unroll
        for (int r = MAXR - 1; r >= 0; --r)
            if (r < a.R && chosen < cum[r]) idx = r;
    } else {
        idx = 0;
#pragma unroll
        for (int r = 0; r < MAXR; ++r)
            if (r < a.R) idx += (cum[r] < chosen) ? 1 : 0;
    }
    tn_bits = (uint64_t)__double_as_longlong(tn);
    return true;
}

// a + b in binary64 on the FP64 pipe (ADD_NATIVE) or on the integer pipes.
template <bool ADD_NATIVE>
__device__ __forceinline__ uint64_t hot_add(uint64_t a, uint64_t b, bool &bad) {
    if (ADD_NATIVE)
        return (uint64_t)__double_as_longlong(
            __dadd_rn(__longlong_as_double((long long)a), __longlong_as_double((long long)b)));
    return b64::add_bf(a, b, bad);
}

// One exact step from the committed state (g, t) towards the sample time T.
// Returns true when a reaction fires (its index in idx, the new clock in tn);
// false when the step records the sample (total vanished, or the clock passed
// T).  Commits exactly the draws the reference consumes; the caller applies
// the jump and the clock.  `nat` forces native binary64.
template <int MAXR, bool MACRO, bool ADDN>
__device__ __forceinline__ bool exact_step(const SsaArgs &a, const ExactTables &m, const int64_t *sp,
                                           const uint64_t *rl, int RS, int BD, Xoshiro &g, uint64_t t, uint64_t T, bool nat,
                                           int &idx, uint64_t &tn) {
    const int R = a.R, P = a.P;
    uint64_t cum[MAXR];
    uint64_t tot = 0;
    bool bad = nat;
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        if (r < R) {
            uint64_t acc = rl[r * RS];
            for (int p = 0; p < P; ++p) {
                const int f = m.fac[r * P + p];
                const int o = f >> 16;
                if (o == 0) continue;
                const int64_t n = sp[(f & 0xFFFF) * BD];
                if (MACRO) {
                    int64_t ff = n;
                    for (int j = 1; j < o; ++j) ff *= n - j;
                    bad |= (uint64_t)ff >= 0x100000000ull;
                    acc = b64::mul_u32(acc, (uint32_t)ff, bad);
                } else {
                    for (int j = o - 1; j >= 0; --j) {
                        const int64_t x = n - j;
                        bad |= (uint64_t)x >= 0x100000000ull;
                        acc = b64::mul_u32(acc, (uint32_t)x, bad);
                    }
                }
            }
            tot = hot_add<ADDN>(tot, acc, bad);
            cum[r] = tot;
        }
    }
    bad |= !emul_domain(tot);
    const bool pos = tot != 0;
    Xoshiro g2 = g;
    bool bad_t = false, bad_c = false;
    const uint64_t x = exp1_emul(g2, m, bad_t);
    const uint64_t q = b64::div_bf(x, pos ? tot : kOneBits, bad_t);
    tn = hot_add<ADDN>(t, q, bad_t);
    bad_t |= !emul_domain(tn);
    bool fire = pos && tn <= T;
    Xoshiro g3 = g2;
    const uint64_t chosen = b64::mul_u64(tot, xo_next(g3) >> 11, 53, bad_c);
    if (MACRO) {
        idx = R;
#pragma unroll
        for (int r = MAXR - 1; r >= 0; --r)
            if (r < R && chosen < cum[r]) idx = r;
    } else {
        idx = 0;
#pragma unroll
        for (int r = 0; r < MAXR; ++r)
            if (r < R) idx += (cum[r] < chosen) ? 1 : 0;
    }
    bad = bad || (pos && bad_t) || (fire && bad_c);
    if (bad) return native_step<MAXR, MACRO>(a, m, g, sp, rl, RS, BD, t, T, idx, tn);
    g = fire ? g3 : (pos ? g2 : g);
    return fire;
}

// Fill the block-wide tables from the device descriptor and ziggurat tables.
__device__ __forceinline__ void load_exact_tables(const SsaArgs &a, ulonglong2 *zxk, uint64_t *zf, uint64_t *zd,
                                                  int32_t *fac, int32_t *jsp, int64_t *jd) {
    const int BD = blockDim.x, tid = threadIdx.x;
    for (int k = tid; k < 256; k += BD) {
        zxk[k] = make_ulonglong2((uint64_t)__double_as_longlong(a.zig[k]),
                                 (uint64_t)__double_as_longlong(a.zig[kZigOffK + k]));
        zd[k] = (uint64_t)__double_as_longlong(a.zig[kZigOffD + k]) & ~(1ull << 63);
    }
    for (int k = tid; k < 257; k += BD) zf[k] = (uint64_t)__double_as_longlong(a.zig[kZigOffF + k]);
    for (int k = tid; k < a.R * a.P; k += BD) fac[k] = a.fac_sp[k] | (a.fac_ord[k] << 16);
    for (int k = tid; k < a.R * a.Q; k += BD) {
        jsp[k] = a.jmp_sp[k];
        jd[k] = a.jmp_d[k];
    }
}

}  // namespace rbg
