// Exact IEEE-754 binary64 arithmetic on the integer pipes.
//
// GB300 retires about 1.9 binary64 FMA per clock per SM but several dozen
// 32-bit integer operations, so the SSA hot loop does its binary64 work here,
// in integer arithmetic, with results identical bit for bit to the hardware's
// round-to-nearest-even operations.  Operands are raw bit patterns of
// non-negative doubles that are normal or +0 (the hot loop's domain: rates,
// propensities, their running sums, the clock, Exp1 draws).  Anything else --
// a subnormal or non-finite input, a result that would overflow or fall below
// the normal range -- sets `bad`, and the caller redoes the step with native
// binary64 instructions.
//
// Every function is __host__ __device__ so the CPU test suite checks it against
// the host FPU on random and constructed operands.
#pragma once

#include "rtc_types.hpp"

#if defined(__CUDACC__)
#define B64_HD __host__ __device__ __forceinline__
#else
#define B64_HD inline
#endif

namespace rbg {
namespace b64 {

constexpr uint64_t kMant = (1ull << 52) - 1;
constexpr uint64_t kHidden = 1ull << 52;

B64_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

B64_HD void mul64(uint64_t a, uint64_t b, uint64_t &hi, uint64_t &lo) {
#if defined(__CUDA_ARCH__)
    lo = a * b;
    hi = __umul64hi(a, b);
#else
    unsigned __int128 p = (unsigned __int128)a * b;
    lo = (uint64_t)p;
    hi = (uint64_t)(p >> 64);
#endif
}

// Pack a significand m in [2^52, 2^53] (2^53 = a rounding carry) with biased
// exponent E: ((E - 1) << 52) + m lets the carry bump the exponent.
B64_HD uint64_t pack(int E, uint64_t m, bool &bad) {
    if (E < 1 || E + (int)(m >> 53) > 2046) {
        bad = true;
        return 0;
    }
    return ((uint64_t)(E - 1) << 52) + m;
}

// Exact double of an integer 0 <= n < 2^53.
B64_HD uint64_t from_u53(uint64_t n) {
    if (n == 0) return 0;
    const int L = 63 - clz64(n);  // position of the leading bit
    return ((uint64_t)(1022 + L) << 52) + (n << (52 - L));
}

// RN(a * n * 2^-down) for a non-negative double a (normal or +0) and an
// integer 0 <= n < 2^63.
B64_HD uint64_t mul_int(uint64_t a, uint64_t n, int down, bool &bad) {
    if (a == 0 || n == 0) return 0;
    const int ea = (int)(a >> 52);
    if (ea == 0 || ea >= 2047) {
        bad = true;
        return 0;
    }
    uint64_t hi, lo;
    mul64((a & kMant) | kHidden, n, hi, lo);
    int s;  // left shift that puts the product's leading bit at bit 127
    if (hi) {
        s = clz64(hi);
        if (s) {
            hi = (hi << s) | (lo >> (64 - s));
            lo <<= s;
        }
    } else {
        s = 64 + clz64(lo);
        hi = lo << (s - 64);
        lo = 0;
    }
    uint64_t m = hi >> 11;
    const uint64_t rest = hi & 0x7FF;  // bit 10 = round bit, below it the sticky bits
    m += ((rest >> 10) & ((rest & 0x3FF) != 0 || lo != 0 || (m & 1))) ? 1 : 0;
    return pack(ea + 75 - s - down, m, bad);
}

// Branch-free forms for the kernels' hot loop (no data-dependent branches, so
// the lanes of a warp stay converged; 32-bit limbs where the operands allow).

// RN(a * n) for a non-negative double a (normal or +0) and 0 <= n < 2^32.
// The 85-bit product is formed from two 32x32 -> 64 multiplies.
B64_HD uint64_t mul_u32(uint64_t a, uint32_t n, bool &bad) {
    const int ea = (int)(a >> 52);
    const uint32_t ml = (uint32_t)a, mh = ((uint32_t)(a >> 32) & 0xFFFFFu) | 0x100000u;
    const uint64_t lo = (uint64_t)ml * n;
    const uint64_t hi = (uint64_t)mh * n + (lo >> 32);  // product = hi * 2^32 + (uint32)lo
    const uint32_t w0 = (uint32_t)lo;
    const int z = clz64(hi | 1);                        // in [10, 43] when n > 0
    const uint64_t top = z < 32 ? (hi << z) | ((uint64_t)w0 >> (32 - z)) : (hi << z) | ((uint64_t)w0 << (z - 32));
    const uint32_t rest = z < 32 ? (w0 << z) : 0u;
    uint64_t m = top >> 11;
    m += ((top >> 10) & (((top & 0x3FF) | rest) != 0 || (m & 1))) ? 1 : 0;
    const int E = ea + 43 - z;
    const bool zero = (a == 0) | (n == 0);
    bad |= !zero && (ea == 0 || ea >= 2047 || E < 1 || E + (int)(m >> 53) > 2046);
    return zero ? 0 : ((uint64_t)(E - 1) << 52) + m;
}

// RN(a * n * 2^-down) for a non-negative double a (normal or +0) and
// 0 <= n < 2^63; branch-free 128-bit normalisation.
B64_HD uint64_t mul_u64(uint64_t a, uint64_t n, int down, bool &bad) {
    const int ea = (int)(a >> 52);
    uint64_t hi, lo;
    mul64((a & kMant) | kHidden, n, hi, lo);
    const bool big = hi != 0;
    const int s = big ? clz64(hi) : 64 + clz64(lo | 1);
    const int sl = s & 63;
    const uint64_t H = big ? (sl ? (hi << sl) | (lo >> (64 - sl)) : hi) : (lo << sl);
    const uint64_t L = big ? (lo << sl) : 0;
    uint64_t m = H >> 11;
    const uint64_t rest = H & 0x7FF;
    m += ((rest >> 10) & ((rest & 0x3FF) != 0 || L != 0 || (m & 1))) ? 1 : 0;
    const int E = ea + 75 - s - down;
    const bool zero = (a == 0) | (n == 0);
    bad |= !zero && (ea == 0 || ea >= 2047 || E < 1 || E + (int)(m >> 53) > 2046);
    return zero ? 0 : ((uint64_t)(E - 1) << 52) + m;
}

// RN(a + b) for non-negative doubles a, b (normal or +0), branch-free.
B64_HD uint64_t add_bf(uint64_t a, uint64_t b, bool &bad) {
    const uint64_t x = a > b ? a : b, y = a > b ? b : a;  // x >= y
    const int ex = (int)(x >> 52), ey = (int)(y >> 52);
    const uint64_t A = ((x & kMant) | kHidden) << 10;
    const uint64_t B = ((y & kMant) | kHidden) << 10;
    const int d = ex - ey;
    const int dd = d < 63 ? d : 63;
    const uint64_t Bs = B >> dd;
    uint64_t sticky = (B & ((1ull << dd) - 1)) != 0;
    uint64_t S = A + Bs;
    const uint64_t carry = S >> 63;
    sticky |= S & carry;
    S >>= carry;
    uint64_t m = S >> 10;
    const uint64_t r = S & 0x3FF;
    m += (r > 0x200 || (r == 0x200 && (sticky || (m & 1)))) ? 1 : 0;
    const int E = ex + (int)carry;
    const bool trivial = y == 0;  // x + 0 = x (also covers 0 + 0)
    bad |= !trivial && (ey == 0 || ex >= 2047 || E + (int)(m >> 53) > 2046);
    return trivial ? x : ((uint64_t)(E - 1) << 52) + m;
}

// RN(a / b) for a >= 0 (normal or +0) and b > 0 normal, branch-free; same
// radix-2^11 long division as div() below.
B64_HD uint64_t div_bf(uint64_t a, uint64_t b, bool &bad);

// RN(a + b) for non-negative doubles a, b (normal or +0).
B64_HD uint64_t add(uint64_t a, uint64_t b, bool &bad) {
    if (a == 0) return b;
    if (b == 0) return a;
    if (a < b) {
        const uint64_t t = a;
        a = b;
        b = t;
    }
    const int ea = (int)(a >> 52), eb = (int)(b >> 52);
    if (eb == 0 || ea >= 2047) {
        bad = true;
        return 0;
    }
    const uint64_t A = ((a & kMant) | kHidden) << 10;
    uint64_t B = ((b & kMant) | kHidden) << 10;
    const int d = ea - eb;
    uint64_t sticky = 0;
    if (d >= 64) {
        sticky = 1;
        B = 0;
    } else if (d > 0) {
        sticky = (B << (64 - d)) != 0;
        B >>= d;
    }
    uint64_t S = A + B;
    int E = ea;
    if (S >> 63) {
        sticky |= S & 1;
        S >>= 1;
        E += 1;
    }
    uint64_t m = S >> 10;
    const uint64_t r = S & 0x3FF;
    m += (r > 0x200 || (r == 0x200 && (sticky || (m & 1)))) ? 1 : 0;
    return pack(E, m, bad);
}

// RN(a - b) for doubles a >= b >= 0 (normal or +0).  The subtrahend is aligned
// with 10 guard bits and its shifted-out bits folded into the lowest bit (the
// sticky bit), which preserves the rounding of the difference; cancellation is
// renormalised with a leading-zero count.
B64_HD uint64_t sub(uint64_t a, uint64_t b, bool &bad) {
    if (b == 0) return a;
    if (a == b) return 0;
    const int ea = (int)(a >> 52), eb = (int)(b >> 52);
    if (eb == 0 || ea >= 2047 || a < b) {
        bad = true;
        return 0;
    }
    const uint64_t A = ((a & kMant) | kHidden) << 10;
    uint64_t B = ((b & kMant) | kHidden) << 10;
    const int d = ea - eb;
    if (d >= 64) {
        B = 1;
    } else if (d > 0) {
        B = (B >> d) | ((B << (64 - d)) != 0 ? 1 : 0);
    }
    uint64_t S = A - B;                 // > 0, leading bit at or below bit 62
    const int z = clz64(S) - 1;         // left shift that puts it at bit 62
    S <<= z;
    const int E = ea - z;
    uint64_t m = S >> 10;
    const uint64_t r = S & 0x3FF;
    m += (r > 0x200 || (r == 0x200 && (m & 1))) ? 1 : 0;
    return pack(E, m, bad);
}

// inv with 2^83/mb * (1 - 2^-21) <= inv <= 2^83/mb for a significand mb in
// [2^52, 2^53): the float reciprocal of mt = (mb >> 21) + 1 >= mb/2^21, with
// mt rounded up and the reciprocal rounded down, scaled by 2^62.  The host
// branch computes the same integer exactly (floats in [2^31, 2^32] are the
// multiples of 256, those in [2^30, 2^31) the multiples of 128).
B64_HD uint32_t recip_estimate(uint64_t mb) {
    const uint64_t mt = (mb >> 21) + 1;
#if defined(__CUDA_ARCH__)
    const float r = __frcp_rd(__ull2float_ru(mt));
    return __float2uint_rz(r * 0x1p62f);
#else
    const uint64_t f = (mt + 255) & ~255ull;
    return (uint32_t)(((1ull << 62) / f) & ~127ull);
#endif
}

// RN(a / b) for a >= 0 (normal or +0) and b > 0 normal.  The 55-bit quotient
// floor(ma * 2^55 / mb) of the significands is built from five 11-bit digits
// (long division in radix 2^11).  Each digit is estimated as
// ((R >> 32) * inv) >> 51, which never exceeds floor(R / mb) (inv <= 2^83/mb)
// and falls short by at most one (R/2^32 and inv lose < 2^-10 of a digit), so
// one comparison against the exact 64-bit remainder fixes it.
B64_HD uint64_t div(uint64_t a, uint64_t b, bool &bad) {
    if (a == 0) return 0;
    const int ea = (int)(a >> 52), eb = (int)(b >> 52);
    if (ea == 0 || ea >= 2047 || eb == 0 || eb >= 2047) {
        bad = true;
        return 0;
    }
    const uint64_t ma = (a & kMant) | kHidden, mb = (b & kMant) | kHidden;
    const uint32_t inv = recip_estimate(mb);
    uint64_t R = ma, Q = 0;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int j = 0; j < 5; ++j) {
        R <<= 11;  // R < mb * 2^11 < 2^64
        uint64_t q = ((R >> 32) * (uint64_t)inv) >> 51;
        R -= q * mb;
        if (R >= mb) {
            R -= mb;
            q += 1;
        }
        Q = (Q << 11) | q;
    }
    // Q = floor(ma * 2^55 / mb) in [2^54, 2^56); R = the remainder
    int E;
    uint64_t m, g, half;
    if (Q >> 55) {
        m = Q >> 3;
        g = Q & 7;
        half = 4;
        E = ea - eb + 1023;
    } else {
        m = Q >> 2;
        g = Q & 3;
        half = 2;
        E = ea - eb + 1022;
    }
    const bool sticky = (g & (half - 1)) != 0 || R != 0;
    m += ((g & half) && (sticky || (m & 1))) ? 1 : 0;
    return pack(E, m, bad);
}

// Branch-free RN(a / b); see the declaration above.
B64_HD uint64_t div_bf(uint64_t a, uint64_t b, bool &bad) {
    const int ea = (int)(a >> 52), eb = (int)(b >> 52);
    const uint64_t ma = (a & kMant) | kHidden, mb = (b & kMant) | kHidden;
    const uint32_t inv = recip_estimate(mb);
    const uint32_t mb_lo = (uint32_t)mb, mb_hi = (uint32_t)(mb >> 32);
    uint64_t R = ma, Q = 0;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int j = 0; j < 5; ++j) {
        R <<= 11;
        const uint32_t q = (uint32_t)(((R >> 32) * (uint64_t)inv) >> 51);
        R -= (uint64_t)mb_lo * q + ((uint64_t)(mb_hi * q) << 32);
        const uint32_t c = R >= mb ? 1u : 0u;
        R -= c ? mb : 0;
        Q = (Q << 11) | (q + c);
    }
    const uint64_t top = Q >> 55;  // 1 when ma >= mb
    const uint64_t m0 = Q >> (2 + top);
    const uint64_t g = Q & ((4ull << top) - 1);
    const uint64_t half = 2ull << top;
    const bool sticky = (g & (half - 1)) != 0 || R != 0;
    const uint64_t m = m0 + (((g & half) != 0 && (sticky || (m0 & 1))) ? 1 : 0);
    const int E = ea - eb + 1022 + (int)top;
    const bool zero = a == 0;
    bad |= !zero && (ea == 0 || ea >= 2047 || eb == 0 || eb >= 2047 || E < 1 || E + (int)(m >> 53) > 2046);
    return zero ? 0 : ((uint64_t)(E - 1) << 52) + m;
}

}  // namespace b64
}  // namespace rbg
