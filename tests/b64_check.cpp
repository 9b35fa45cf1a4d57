// Bit-exact check of the integer binary64 primitives (rebop_gb300/csrc/b64.cuh)
// against the host FPU (IEEE round-to-nearest-even), on random and constructed
// operands.  Prints one line per operation: "<op> <cases> <mismatches> <bad>".
// `bad` counts cases the primitive refused (they must all be cases whose result
// is not a normal number or whose inputs are outside the primitive's domain).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

#include "b64.cuh"

using namespace rbg::b64;

static uint64_t bits(double d) {
    uint64_t u;
    std::memcpy(&u, &d, 8);
    return u;
}
static double dbl(uint64_t u) {
    double d;
    std::memcpy(&d, &u, 8);
    return d;
}
// A refusal is legitimate when the rounded result is not comfortably inside
// the normal range: zero by underflow, subnormal, infinite, or within an ulp of
// the smallest normal (where the 53-bit rounding would differ from IEEE's).
static bool refusal_ok(double ref) {
    const double r = std::fabs(ref);
    return !(r > 0x1.0000000000001p-1022 && std::isfinite(r));
}

static std::mt19937_64 rng(20261203);

// Significands with varied bit patterns: random, sparse, dense, near powers of two.
static uint64_t mantissa() {
    switch (rng() % 6) {
        case 0: return rng() & kMant;
        case 1: return (1ull << (rng() % 52)) | (1ull << (rng() % 52));
        case 2: return kMant ^ (1ull << (rng() % 52));
        case 3: return rng() % 8;
        case 4: return kMant - rng() % 8;
        default: return (rng() & kMant) & ~((1ull << (rng() % 40)) - 1);
    }
}
static uint64_t rnd_double(int emin, int emax) {
    const int e = emin + (int)(rng() % (uint64_t)(emax - emin + 1));
    return ((uint64_t)e << 52) | mantissa();
}
static uint64_t rnd_int() {
    switch (rng() % 6) {
        case 0: return rng() % 16;
        case 1: return rng() % 5000;
        case 2: return rng() & 0xFFFFFFFFull;
        case 3: return rng() >> 11;                       // 53 bits
        case 4: return ((rng() >> 11) | 1) & ((1ull << 53) - 1);
        default: return (1ull << (rng() % 53)) + (rng() % 3);
    }
}

int main(int argc, char **argv) {
    const long N = argc > 1 ? std::atol(argv[1]) : 1000000;
    long fail, bad;

    // from_u53
    fail = 0;
    for (long i = 0; i < N; i++) {
        uint64_t n = rnd_int() & ((1ull << 53) - 1);
        if (from_u53(n) != bits((double)n)) fail++;
    }
    std::printf("from_u53 %ld %ld 0\n", N, fail);

    // mul_int, with and without the 2^-53 scale
    fail = bad = 0;
    for (long i = 0; i < N; i++) {
        const uint64_t a = (i % 17 == 0) ? 0 : rnd_double(i % 5 == 0 ? 1 : 600, i % 7 == 0 ? 2046 : 1400);
        const uint64_t n = rnd_int() & ((1ull << 53) - 1);
        const int down = (i & 1) ? 53 : 0;
        bool b = false;
        const uint64_t got = mul_int(a, n, down, b);
        // the kernel's operation: a times an exact double n * 2^-down, one rounding
        const double ref = dbl(a) * ((double)n * (down ? 0x1p-53 : 1.0));
        if (b) {
            bad++;
            if (!refusal_ok(ref)) fail++;
        } else if (got != bits(ref)) {
            fail++;
        }
    }
    std::printf("mul_int %ld %ld %ld\n", N, fail, bad);

    // mul_u32 (counts) and mul_u64 (53-bit integers, optional 2^-53 scale), branch-free
    long f32 = 0, b32 = 0, f64 = 0, b64c = 0;
    for (long i = 0; i < N; i++) {
        const uint64_t a = (i % 17 == 0) ? 0 : rnd_double(i % 5 == 0 ? 1 : 600, i % 7 == 0 ? 2046 : 1400);
        const uint32_t n32 = (uint32_t)(rnd_int() & 0xFFFFFFFFull);
        bool b = false;
        uint64_t got = mul_u32(a, n32, b);
        double ref = dbl(a) * (double)n32;
        if (b) {
            b32++;
            if (!refusal_ok(ref)) f32++;
        } else if (got != bits(ref)) {
            f32++;
        }
        const uint64_t n = rnd_int() & ((1ull << 53) - 1);
        const int down = (i & 1) ? 53 : 0;
        b = false;
        got = mul_u64(a, n, down, b);
        ref = dbl(a) * ((double)n * (down ? 0x1p-53 : 1.0));
        if (b) {
            b64c++;
            if (!refusal_ok(ref)) f64++;
        } else if (got != bits(ref)) {
            f64++;
        }
    }
    std::printf("mul_u32 %ld %ld %ld\n", N, f32, b32);
    std::printf("mul_u64 %ld %ld %ld\n", N, f64, b64c);

    // add
    fail = bad = 0;
    for (long i = 0; i < N; i++) {
        const uint64_t a = (i % 19 == 0) ? 0 : rnd_double(i % 11 == 0 ? 1 : 900, i % 13 == 0 ? 2046 : 1200);
        uint64_t b;
        if (i % 3 == 0) {
            const int d = (int)(rng() % 80);
            const int ea = (int)(a >> 52);
            b = ea - d >= 1 ? (((uint64_t)(ea - d)) << 52) | mantissa() : rnd_double(900, 1200);
        } else {
            b = (i % 23 == 0) ? 0 : rnd_double(900, 1200);
        }
        bool bb = false;
        const uint64_t got = add(a, b, bb);
        const double ref = dbl(a) + dbl(b);
        if (bb) {
            bad++;
            if (!refusal_ok(ref)) fail++;
        } else if (got != bits(ref)) {
            fail++;
        }
        bool bb2 = false;
        const uint64_t got2 = add_bf(a, b, bb2);
        if (bb2) {
            if (!refusal_ok(ref)) fail++;
        } else if (got2 != bits(ref)) {
            fail++;
        }
    }
    std::printf("add %ld %ld %ld\n", N, fail, bad);

    // sub (a >= b >= 0), including heavy cancellation
    fail = bad = 0;
    for (long i = 0; i < N; i++) {
        uint64_t a = rnd_double(i % 11 == 0 ? 1 : 900, 1200), b;
        const int kind = (int)(i % 4);
        if (kind == 0) {
            b = a - (rng() % 64);                        // a few ulps apart
        } else if (kind == 1) {
            const int d = (int)(rng() % 80);
            const int ea = (int)(a >> 52);
            b = ea - d >= 1 ? (((uint64_t)(ea - d)) << 52) | mantissa() : 0;
        } else if (kind == 2) {
            b = (i % 7 == 0) ? 0 : rnd_double(900, 1200);
        } else {
            b = (a & ~kMant) | mantissa();              // same binade
        }
        if (b > a) {
            const uint64_t t = a;
            a = b;
            b = t;
        }
        bool bb = false;
        const uint64_t got = sub(a, b, bb);
        const double ref = dbl(a) - dbl(b);
        if (bb) {
            bad++;
            if (!refusal_ok(ref) && ref != 0.0) fail++;
        } else if (got != bits(ref)) {
            fail++;
        }
    }
    std::printf("sub %ld %ld %ld\n", N, fail, bad);

    // div
    fail = bad = 0;
    for (long i = 0; i < N; i++) {
        const uint64_t a = (i % 29 == 0) ? 0 : rnd_double(i % 9 == 0 ? 1 : 700, i % 10 == 0 ? 2046 : 1400);
        const uint64_t b = rnd_double(i % 8 == 0 ? 1 : 700, i % 12 == 0 ? 2046 : 1400);
        bool bb = false;
        const uint64_t got = div(a, b, bb);
        const double ref = dbl(a) / dbl(b);
        if (bb) {
            bad++;
            if (!refusal_ok(ref)) fail++;
        } else if (got != bits(ref)) {
            fail++;
        }
        bool bb2 = false;
        const uint64_t got2 = div_bf(a, b, bb2);
        if (bb2) {
            if (!refusal_ok(ref)) fail++;
        } else if (got2 != bits(ref)) {
            fail++;
        }
    }
    std::printf("div %ld %ld %ld\n", N, fail, bad);

    // div with quotients that are exact or exactly half-way: (q * b) / b and ties
    fail = 0;
    long n_tie = 0;
    for (long i = 0; i < N / 4; i++) {
        const uint64_t b = rnd_double(1000, 1050);
        const uint64_t q = rnd_double(1000, 1050);
        const double prod = dbl(q) * dbl(b);
        bool bb = false;
        const uint64_t got = div(bits(prod), b, bb);
        if (!bb && got != bits(prod / dbl(b))) fail++;
        // half-way: a = (2k+1) * b * 2^-54 style constructions through integers
        const uint64_t k = (rng() >> 12) | 1;
        const double num = (double)(2 * k + 1);
        const double den = 2.0;
        const uint64_t g2 = div(bits(num), bits(den), bb);
        if (!bb && g2 != bits(num / den)) fail++;
        n_tie++;
    }
    std::printf("div_exact %ld %ld 0\n", n_tie, fail);
    return 0;
}
