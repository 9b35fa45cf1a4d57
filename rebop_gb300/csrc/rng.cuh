// Device random stream: the generator stack of rebop's run-time API, so that
// a trajectory seeded with s draws exactly the numbers the reference's
// `SmallRng::seed_from_u64(s)` gives it (src/gillespie.rs:184, 285-286,
// 327, 332).  The pieces are written from their published descriptions:
//   * xoshiro256++ (Blackman & Vigna 2018): 256-bit state, output
//     rotl(s0 + s3, 23) + s0, then the xorshift/rotate state update;
//   * seeding by four successive SplitMix64 outputs (Steele, Lea & Flood 2014);
//   * uniform [0,1): the top 53 bits of one 64-bit output times 2^-53;
//   * Exp1: 256-layer ziggurat (Marsaglia & Tsang 2000) over the ZIGNOR
//     layer table (Doornik 2005).  One 64-bit draw gives the layer i from its
//     low 8 bits and the abscissa fraction u in (0,1) from its top 52 bits;
//     x = u * X[i] is accepted when below X[i+1]; layer 0 falls back to the
//     tail R - ln(U); otherwise a second uniform decides the wedge test
//     F[i+1] + (F[i] - F[i+1]) * U < exp(-x).
// The wedge test is written with explicit round-to-nearest intrinsics so the
// compiler cannot fuse it into an FMA.
#pragma once

#include "rtc_types.hpp"

namespace rbg {

struct Xoshiro {
    uint64_t s0, s1, s2, s3;
};

__device__ __forceinline__ uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

__device__ __forceinline__ uint64_t splitmix64_next(uint64_t &state) {
    state += 0x9E3779B97F4A7C15ull;
    uint64_t z = state;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ void xo_seed(Xoshiro &g, uint64_t seed) {
    uint64_t st = seed;
    g.s0 = splitmix64_next(st);
    g.s1 = splitmix64_next(st);
    g.s2 = splitmix64_next(st);
    g.s3 = splitmix64_next(st);
}

__device__ __forceinline__ uint64_t xo_next(Xoshiro &g) {
    const uint64_t out = rotl64(g.s0 + g.s3, 23) + g.s0;
    const uint64_t t = g.s1 << 17;
    g.s2 ^= g.s0;
    g.s3 ^= g.s1;
    g.s1 ^= g.s2;
    g.s0 ^= g.s3;
    g.s2 ^= t;
    g.s3 = rotl64(g.s3, 45);
    return out;
}

// The state before the last xo_next: the update is invertible; s1 ^ s2 after
// it is b ^ (b << 17) of the old s1 = b, undone by three more shifts.
__device__ __forceinline__ void xo_prev(Xoshiro &g) {
    const uint64_t d1 = rotl64(g.s3, 19);
    const uint64_t y = g.s1 ^ g.s2;
    const uint64_t b = y ^ (y << 17) ^ (y << 34) ^ (y << 51);
    const uint64_t a = g.s0 ^ d1;
    g.s2 = g.s1 ^ b ^ a;
    g.s0 = a;
    g.s1 = b;
    g.s3 = d1 ^ b;
}

// k * 2^-53 for the top 53 bits k of a draw (exact: k < 2^53).
__device__ __forceinline__ double uniform53(uint64_t bits) {
    return __dmul_rn((double)(bits >> 11), 0x1.0p-53);
}

__device__ __forceinline__ double xo_uniform(Xoshiro &g) { return uniform53(xo_next(g)); }

// Nanosecond wall clock of the GPU.
__device__ __forceinline__ int64_t global_ns() {
    int64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

constexpr double kZigR = 7.69711747013104972;  // start of the exponential tail

// zx/zf: the 257-entry abscissa and density tables (shared memory).
__device__ __forceinline__ double xo_exp1(Xoshiro &g, const double *__restrict__ zx,
                                          const double *__restrict__ zf) {
    for (;;) {
        const uint64_t bits = xo_next(g);
        const int i = (int)(bits & 0xff);
        // (bits >> 12) as the mantissa of a number in [1, 2), minus (1 - 2^-53):
        // an exact odd multiple of 2^-53 in (0, 1).
        const double one_two = __longlong_as_double((long long)((bits >> 12) | 0x3FF0000000000000ull));
        const double u = __dsub_rn(one_two, 0x1.fffffffffffffp-1);
        const double x = __dmul_rn(u, zx[i]);
        if (x < zx[i + 1]) return x;
        if (i == 0) return __dsub_rn(kZigR, log(xo_uniform(g)));
        const double f1 = zf[i + 1];
        const double w = __dadd_rn(f1, __dmul_rn(__dsub_rn(zf[i], f1), xo_uniform(g)));
        if (w < exp(-x)) return x;
    }
}

}  // namespace rbg
