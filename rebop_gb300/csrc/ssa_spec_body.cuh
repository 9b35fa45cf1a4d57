// Speculative thread-per-trajectory SSA kernel: float-pair arithmetic with
// rigorous error bounds, exact re-run of undecidable sample intervals.
//
// What an SSA trajectory records depends on its binary64 arithmetic only
// through decisions: which reaction fires (#{r : cum_r < total * U}) and
// whether the next event falls before the sample time (t + Exp1/total <= T).
// The random stream consumed follows from those decisions too.  And at every
// sample time the clock is reset to T exactly (gillespie.rs:328-330).
//
// So each step here evaluates propensities and their total in float pairs
// (hi + lo, about 46 bits), the clock as a float triple, Exp1/total in float
// pairs and the choice in float32, all on the FP32 and integer pipes,
// together with a bound on the distance of every quantity from the value
// rebop's binary64 arithmetic produces.  A decision whose operands lie farther
// apart than their bounds is the reference's decision:
//   * a float32 choice comparison inside its margin ((R + M + 6) 2^-24 of
//     the total) is redone in binary64 for that step alone
//     (Ops::exact_choice);
//   * a clock comparison inside its margin, a count outside [0, 2^23) or a
//     total outside 2^-90 .. 2^90 makes the lane restore the state it saved at
//     the start of the sample interval and re-run that interval with the exact
//     step of ssa_exact.cuh.
// So every recorded count, event count and random draw equals rebop's bit for
// bit.  Trajectories whose rates lie outside 2^-60 .. 2^60 run exactly.
//
// Error model: every float-pair operation (including the reference's own
// binary64 rounding of the same operation) moves a value by at most
// gamma = 2^-44 relative (the float-pair errors are near 2^-46, binary64's
// 2^-53).  With M reactant factors per reaction at most and R reactions, the
// total (a float32 running sum of the high parts plus a float32 sum of the
// two-sum errors and low parts) is within G = (M + R + 2 + (R (R + 1) / 2 +
// R (M + 2)) / 16) gamma of the reference's and Exp1/total
// within (G + 6 gamma) q plus the Exp1 abscissa's absolute error over the
// total.  The triple-float clock add is exact up to its low part's rounding,
// and the reference's own rounding of t + q adds at most 2^-53 (t + q): the
// bound grows by 2^-52 t per event, accumulated with upward rounding.
//
// This header holds the device side, templated on the network operations of
// the float-pair step: TableOps below walks the packed descriptor; a network
// compiled at run time supplies the same members unrolled, with its counts in
// registers.
#pragma once

#include "ssa_exact.cuh"

namespace rbg {

extern __shared__ __align__(16) unsigned char g_spec_smem[];

constexpr float kGamma = 0x1p-44f;

struct DF {
    float h, l;
};

__device__ __forceinline__ DF fast2sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}

// a * f for a float pair a and an exact float f >= 0.
__device__ __forceinline__ DF df_mul_f(DF a, float f) {
    const float p = __fmul_rn(a.h, f);
    const float e = __fmaf_rn(a.h, f, -p);
    return fast2sum(p, __fmaf_rn(a.l, f, e));
}

// a * f without the final renormalisation: the low part stays below 2^-20 of
// the high part for up to eight successive factors, which df_add accepts.
__device__ __forceinline__ DF df_mul_fu(DF a, float f) {
    const float p = __fmul_rn(a.h, f);
    return DF{p, __fmaf_rn(a.l, f, __fmaf_rn(a.h, f, -p))};
}

__device__ __forceinline__ DF df_mul(DF a, DF b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast2sum(p, e);
}

// a + b for non-negative float pairs.
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = __fadd_rn(a.h, b.h);
    const float bb = __fsub_rn(s, a.h);
    float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    return fast2sum(s, e);
}

// Running sum of non-negative float pairs: s is the float32 running sum of the
// high parts, e collects the two-sum errors and the low parts, so s + e is
// the pair.  After r terms of at most M factors each, s is within
// (r + M + 2) 2^-24 of the exact running sum (a rate's low part is below
// 2^-23 of its high part, each factor adds 2^-24; one rounding per add).
struct RunSum {
    float s, e;
};

__device__ __forceinline__ void rs_add(RunSum &a, DF b) {
    const float s = __fadd_rn(a.s, b.h);
    const float bb = __fsub_rn(s, a.s);
    const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
    a.e = __fadd_rn(a.e, __fadd_rn(err, b.l));
    a.s = s;
}

__device__ __forceinline__ DF rs_total(RunSum a) { return fast2sum(a.s, a.e); }

__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// a / b for b > 0: one reciprocal estimate, one residual correction.
__device__ __forceinline__ DF df_div(DF a, DF b, float r) {
    const float q1 = __fmul_rn(a.h, r);
    const float p = __fmul_rn(q1, b.h);
    const float pe = __fmaf_rn(q1, b.h, -p);
    float res = __fsub_rn(__fsub_rn(a.h, p), pe);
    res = __fadd_rn(res, a.l);
    res = __fmaf_rn(-q1, b.l, res);
    return fast2sum(q1, __fmul_rn(res, r));
}

// Exact float of an integer 0 <= x < 2^23.
__device__ __forceinline__ float f23(uint32_t x) { return __fsub_rn(__uint_as_float(0x4B000000u | x), 8388608.0f); }

// u * 2^-53 for 0 <= u < 2^53, keeping the top 46 bits of u (absolute error < 2^-46).
__device__ __forceinline__ DF df_u53(uint64_t u) {
    return DF{__fmul_rn(f23((uint32_t)(u >> 30)), 0x1p-23f),
              __fmul_rn(f23((uint32_t)(u >> 7) & 0x7FFFFFu), 0x1p-46f)};
}

// Float pair of a double (rare paths: interval starts, rates, the Exp1 tail).
__device__ __forceinline__ DF df_from_double(double v) {
    const float h = __double2float_rz(v);
    return DF{h, __double2float_rn(__dsub_rn(v, (double)h))};
}

// Clock as an unevaluated sum of three floats.  Adding a float pair is exact
// up to the rounding of the smallest part, so the clock keeps the reference's
// binary64 clock to within that binary64 arithmetic's own rounding.
struct TF {
    float h, m, l;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Exact triple of a double v = 0 or 2^-60 <= v < 2^60.
__device__ __forceinline__ TF tf_from_double(double v) {
    const float h = __double2float_rz(v);
    const double r1 = __dsub_rn(v, (double)h);
    const float m = __double2float_rz(r1);
    return TF{h, m, __double2float_rn(__dsub_rn(r1, (double)m))};
}

// t + q for t, q >= 0 (t with |m| <= ulp(h)/2, q normalised).  Every step is
// an error-free transformation except the two roundings into the low part,
// which are bounded by 2^-24 (|l| + |e2 + e3|).
__device__ __forceinline__ TF tf_add(TF t, DF q) {
    float s, e1, m, e2, m2, e3;
    two_sum(t.h, q.h, s, e1);
    two_sum(t.m, q.l, m, e2);
    two_sum(m, e1, m2, e3);
    const float l = __fadd_rn(t.l, __fadd_rn(e2, e3));
    const float h = __fadd_rn(s, m2);  // |m2| <= |s|: fast two-sum
    return TF{h, __fsub_rn(m2, __fsub_rn(h, s)), l};
}

// Wedge test of the ziggurat, f[i+1] - |f[i] - f[i+1]| U < exp(-x), for the
// candidate x = X_i (2k + 1) 2^-53 (xh its float within 2^-24 x) and U = mu
// 2^-53.  First in float32: the float copies of the tables and U are within
// 2^-23 (2^-20.2 of the left side at the steepest layer, f[2]/f[1] < 2.2),
// xh within 2^-24 x (x < 7.7: 2^-21 on exp(-x)) and expf within 2 ulp, so a
// side more than 2^-17 apart decides as binary64 would; inside that band the
// exact operands decide (wedge_accept).
__device__ __forceinline__ bool wedge_df(const ExactTables &ex, int i, uint64_t k, float xh, uint64_t mu) {
    const float u = __fmul_rn(f23((uint32_t)(mu >> 30)), 0x1p-23f);
    const float wf = __fmaf_rn(-f32_rz(ex.zd[i]), u, f32_rz(ex.zf[i + 1]));
    const float ef = expf(-xh);
    if (wf < __fmul_rn(ef, 1.0f - 0x1p-17f)) return true;
    if (wf > __fmul_rn(ef, 1.0f + 0x1p-17f)) return false;
    bool bad = false;
    return wedge_accept(ex, i, b64::mul_u64(ex.zxk[i].x, 2 * k + 1, 53, bad), mu, bad);
}

// Exp1 draw as a float pair, consuming the stream exactly as the reference
// does: every accept/reject decision is the binary64 one.  xerr bounds
// |x - rebop's binary64 draw|.
__device__ __forceinline__ DF exp1_df(Xoshiro &g, const ExactTables &ex, const float2 *xdf, float &xerr) {
    for (;;) {
        const uint64_t b = xo_next(g);
        const int i = (int)(b & 0xff);
        const uint64_t k = b >> 12;
        const float2 X = xdf[i];
        const DF x = df_mul(df_u53(2 * k + 1), DF{X.x, X.y});
        if (k < ex.zxk[i].y) {
            xerr = kGamma * X.x;
            return x;
        }
        if (i == 0) {
            const DF t = df_from_double(__dsub_rn(kZigR, log(xo_uniform(g))));
            xerr = kGamma * t.h;
            return t;
        }
        if (wedge_df(ex, i, k, x.h, xo_next(g) >> 11)) {
            xerr = kGamma * X.x;
            return x;
        }
    }
}

// Exp1 draw whose first candidate (draw b, float pair x) failed the fast
// test, when the next draw b2 is already taken (g is past it): b2 is the
// wedge's or the tail's uniform, as in the reference.
__device__ __forceinline__ DF exp1_df_cont(Xoshiro &g, uint64_t b, uint64_t b2, DF x, const ExactTables &ex,
                                           const float2 *xdf, float &xerr) {
    const int i = (int)(b & 0xff);
    if (i == 0) {
        const DF t = df_from_double(__dsub_rn(kZigR, log(uniform53(b2))));
        xerr = kGamma * t.h;
        return t;
    }
    if (wedge_df(ex, i, b >> 12, x.h, b2 >> 11)) {
        xerr = kGamma * xdf[i].x;
        return x;
    }
    return exp1_df(g, ex, xdf, xerr);
}

// Rate in the float-pair range (0, or 2^-60 .. 2^60), also inside the exact
// engine's integer domain.
__device__ __forceinline__ bool spec_rate_ok(uint64_t v) {
    const uint64_t e = v >> 52;
    return v == 0 || (e >= 1023 - 60 && e <= 1023 + 60);
}

constexpr int kSpecBlock = 512;   // lanes per block; one block per SM
constexpr int kSpecPhase = 128;   // default steps between two compactions of a warp
constexpr int kSpecMaxSlots = 2048;

// Shared memory: block tables, then per-slot columns [field][slots].  A slot
// holds one trajectory's whole state between phases; a lane works on the
// slot the last compaction gave it.  A block may hold more slots than lanes:
// then the lanes rotate over the live slots, so every resident trajectory
// advances at the same pace and no second wave of late starters is left to
// run on a nearly empty SM.
constexpr int kSpecSampleCache = 256;  // sample times kept in shared memory

__host__ __device__ inline int spec_sample_cache(const SsaArgs &a) {
    return a.n_samples <= kSpecSampleCache ? (int)a.n_samples : 0;
}

// Rates live in per-slot columns when every trajectory has its own, else
// once for the block.
__host__ __device__ inline size_t spec_smem_bytes(const SsaArgs &a, int slots) {
    const int S = a.S, R = a.R, P = a.P, Q = a.Q;
    const bool rate_per_traj = a.rate_stride != 0;
    size_t b = 16 * 256 + 8 * 257 + 8 * 256 + 8 * 256;  // zxk, zf, zd, xdf
    b += 24 * (size_t)spec_sample_cache(a);             // sample times: bits, float triple
    b += 4 * (size_t)a.n_save + 16;                     // saved species
    b += 8 * (size_t)R * Q;                             // jd
    b += 16 * (size_t)R * (rate_per_traj ? slots : 1);  // exact rate bits, float-pair rates
    b += 16 * (size_t)S * slots;                        // counts, counts at interval start
    b += 32 * (size_t)slots;                            // generator at interval start
    b += 80 * (size_t)slots;                            // 10 state words
    b += 32 * (size_t)slots;                            // 7 float state words, flags
    b += 4 * (size_t)slots + 512;                       // slot list, block counters
    b += 8 * (size_t)slots;                             // rows recorded, not yet counted
    b += 4 * ((size_t)R * P + (size_t)R * Q);           // fac, jsp
    return (b + 15) & ~(size_t)15;
}

// Exact re-run of one sample interval from its saved start (counts in sps,
// generator in gsv, event count ev0, clock t0) up to the step that records
// the sample at T.  Kept out of line so the float-pair loop keeps its
// registers; the generator state after the interval goes back to gsv.
// Returns the event count, or ~0 if the time budget ran out.
template <int MAXR, bool MACRO>
__device__ __noinline__ unsigned long long replay_interval(const SsaArgs &a, const ExactTables &ex, int64_t *sp,
                                                           const int64_t *sps, uint64_t *gsv, const uint64_t *rl,
                                                           int RS, int BD, uint64_t t0, uint64_t T, bool nat,
                                                           unsigned long long ev0, int64_t t_start) {
    for (int s = 0; s < a.S; ++s) sp[s * BD] = sps[s * BD];
    Xoshiro h{gsv[0], gsv[BD], gsv[2 * BD], gsv[3 * BD]};
    unsigned long long e = ev0;
    uint64_t t = t0;
    for (unsigned int n = 1;; ++n) {
        if ((n & 255u) == 0 && global_ns() - t_start > a.budget_ns) return ~0ull;
        int ix;
        uint64_t tx;
        if (!exact_step<MAXR, MACRO, true>(a, ex, sp, rl, RS, BD, h, t, T, nat, ix, tx)) break;
        t = tx;
        ++e;
        if (ix < a.R)
            for (int k = 0; k < a.Q; ++k) sp[ex.jsp[ix * a.Q + k] * BD] += ex.jd[ix * a.Q + k];
    }
    gsv[0] = h.s0;
    gsv[BD] = h.s1;
    gsv[2 * BD] = h.s2;
    gsv[3 * BD] = h.s3;
    return e;
}

// The reference's choice #{r : cum_r < total * U} (or the macro's first r with
// total * U < cum_r) in native binary64 from the counts in the slot column:
// the rare steps whose float choice falls within its error margin.
template <int MAXR, bool MACRO>
__device__ __noinline__ int exact_choice_table(const SsaArgs &a, const ExactTables &m, const int64_t *sp, int NS,
                                               const uint64_t *rl, int RS, uint64_t u53) {
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
                const int64_t n = sp[(f & 0xFFFF) * NS];
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
    const double chosen = __dmul_rn(total, (double)u53 * 0x1p-53);
    int idx;
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
    return idx;
}

// Slot flags.
constexpr uint32_t kLive = 1, kNat = 2, kExactTraj = 4, kBegin = 8, kHave = 16;

// Rows [lo, hi) of `out` hold this lane's trajectory's samples: count them in
// a.row_done, after a fence that makes the sample stores visible device-wide
// first (the host copies a row once its count reaches n_traj).
__device__ __forceinline__ void count_rows_nofence(const SsaArgs &a, uint32_t lo, uint32_t hi) {
    for (uint32_t r = lo; r < hi; ++r) atomicAdd(a.row_done + r, 1u);
}
static __device__ __noinline__ void count_rows(const SsaArgs &a, uint32_t lo, uint32_t hi) {
    __threadfence();
    count_rows_nofence(a, lo, hi);
}

// Live-slot entries per lane that the lag scheduler keeps in registers (it
// covers warps of up to 128 live slots; beyond that the lanes rotate).
constexpr int kSpecSchedPerLane = 4;

// Slot for this lane among a warp's n_live > 32 live slots (wlist[0 ..
// n_live)): the 32 whose clocks lag furthest behind.  A slot that holds no
// trajectory yet counts as time 0.  Keys are the clock's float bits (monotone
// for t >= 0) with the low bits replaced by the list position, so they are
// unique; a radix search finds tau, the 33rd smallest key, and the keys below
// it go to the lanes in list order.  stf[0 .. NS) holds each slot's clock.
static __device__ __noinline__ int lag_select(const float *stf, const uint32_t *stflag, int32_t *wlist, int n_live, int lane) {
    const int nb = 32 - __clz(n_live - 1);  // bits of a list position
    const uint32_t low = (1u << nb) - 1u;
    uint32_t key[kSpecSchedPerLane];
    int32_t sl[kSpecSchedPerLane];
#pragma unroll
    for (int c = 0; c < kSpecSchedPerLane; ++c) {
        const int e = c * 32 + lane;
        key[c] = 0xFFFFFFFFu;
        sl[c] = -1;
        if (e < n_live) {
            const int32_t s = wlist[e];
            const uint32_t t = (stflag[s] & kHave) ? __float_as_uint(stf[s]) : 0u;
            key[c] = (t & ~low) | (uint32_t)e;
            sl[c] = s;
        }
    }
    uint32_t tau = 0;
    for (int b = 31; b >= 0; --b) {
        const uint32_t cand = tau | (1u << b);
        unsigned int cnt = 0;
#pragma unroll
        for (int c = 0; c < kSpecSchedPerLane; ++c) cnt += key[c] < cand ? 1u : 0u;
        if (__reduce_add_sync(0xffffffffu, cnt) <= 32u) tau = cand;
    }
    __syncwarp();  // every lane has read its list entries
    int n_sel = 0;
#pragma unroll
    for (int c = 0; c < kSpecSchedPerLane; ++c) {
        const bool sel = key[c] < tau;
        const unsigned int bal = __ballot_sync(0xffffffffu, sel);
        if (sel) wlist[n_sel + __popc(bal & ((1u << lane) - 1u))] = sl[c];
        n_sel += __popc(bal);
    }
    __syncwarp();
    return wlist[lane];
}

// Network operations of the float-pair step over a data-driven descriptor:
// the counts stay in the slot's shared-memory column and every reaction walks
// its (species, order) factor list.  A generated network (see ssa_jit.cpp)
// supplies the same members with the network unrolled and the counts held in
// registers.
template <int MAXR, bool MACRO>
struct TableOps {
    static constexpr int kMaxR = MAXR;
    static constexpr bool kMacro = MACRO;
    struct Counts {};
    __device__ static int nr(const SsaArgs &a) { return a.R; }
    // registers <- column; false if a count is outside [0, 2^23)
    __device__ static bool load(Counts &, const SsaArgs &, const int64_t *, int) { return true; }
    // column <- registers
    __device__ static void store(const Counts &, const SsaArgs &, int64_t *, int) {}
    // interval-start copy of the counts
    __device__ static void save(const Counts &, const SsaArgs &a, const int64_t *sp, int64_t *sps, int NS) {
        for (int s = 0; s < a.S; ++s) sps[s * NS] = sp[s * NS];
    }
    // Float-pair propensities: the total as a float pair, the running sums'
    // high parts; true if a count leaves the float-pair range (then the step
    // is undecided).
    __device__ static bool props(const SsaArgs &a, const ExactTables &ex, const Counts &, const int64_t *sp,
                                 int NS, const float2 *rf, int RS, float *cum, DF &tot) {
        bool amb = false;
        RunSum sum{0.f, 0.f};
#pragma unroll
        for (int r = 0; r < MAXR; ++r) {
            if (r < a.R) {
                const float2 k = rf[r * RS];
                DF acc{k.x, k.y};
                for (int p = 0; p < a.P; ++p) {
                    const int f = ex.fac[r * a.P + p];
                    const int o = f >> 16;
                    if (o == 0) continue;
                    const int64_t n = sp[(f & 0xFFFF) * NS];
                    // counts in [0, 2^23); for n < o the factors n, n-1, ...
                    // reach 0 before going negative, so the product is 0 (the
                    // reference's +-0 leaves every running sum unchanged):
                    // clamp at 0.
                    amb |= (uint64_t)n >= (1ull << 23);
                    for (int j = 0; j < o; ++j) {
                        const int64_t x = n - j > 0 ? n - j : 0;
                        acc = df_mul_fu(acc, f23((uint32_t)x & 0x7FFFFFu));
                    }
                }
                rs_add(sum, acc);
                cum[r] = sum.s;
            }
        }
        tot = rs_total(sum);
        return amb;
    }
    // The reference's choice for this state and uniform draw, in binary64.
    __device__ static int exact_choice(const SsaArgs &a, const ExactTables &ex, const Counts &, const int64_t *sp,
                                       int NS, const uint64_t *rl, int RS, uint64_t u53) {
        return exact_choice_table<MAXR, MACRO>(a, ex, sp, NS, rl, RS, u53);
    }
    __device__ static void jump(Counts &, const SsaArgs &a, const ExactTables &ex, int64_t *sp, int NS, int idx) {
        if (idx < a.R)
            for (int k = 0; k < a.Q; ++k) sp[ex.jsp[idx * a.Q + k] * NS] += ex.jd[idx * a.Q + k];
    }
};

// The kernel body: one block per SM; each warp rotates its lanes over its own
// `a.n_slots / warps` trajectory slots in phases of `a.phase_steps` steps.
template <class Ops>
__device__ __forceinline__ void spec_body(const SsaArgs &a) {
    constexpr int MAXR = Ops::kMaxR;
    constexpr bool MACRO = Ops::kMacro;
    const int BD = blockDim.x, tid = threadIdx.x;
    const int NS = a.n_slots;  // slots per block: a multiple of the warps, >= 32 per warp
    const int warp = tid >> 5, lane = tid & 31;
    const int SPW = NS / (BD >> 5);  // slots per warp
    const int wbase = warp * SPW;
    const int S = a.S, R = Ops::nr(a), P = a.P, Q = a.Q;

    // ---- shared memory: block tables, then per-slot columns
    ulonglong2 *zxk = reinterpret_cast<ulonglong2 *>(g_spec_smem);
    uint64_t *zf = reinterpret_cast<uint64_t *>(zxk + 256);
    uint64_t *zd = zf + 257;
    float2 *xdf = reinterpret_cast<float2 *>(zd + 256);
    int64_t *jd = reinterpret_cast<int64_t *>(xdf + 256);
    const bool rate_cols = a.rate_stride != 0;  // per-slot rate columns
    const int RS = rate_cols ? NS : 1;           // stride between two reactions' rates
    uint64_t *rate = reinterpret_cast<uint64_t *>(jd + (size_t)R * Q);
    float2 *rdf = reinterpret_cast<float2 *>(rate + (size_t)R * RS);
    int64_t *spa = reinterpret_cast<int64_t *>(rdf + (size_t)R * RS);
    int64_t *spsa = spa + (size_t)S * NS;
    uint64_t *gsva = reinterpret_cast<uint64_t *>(spsa + (size_t)S * NS);
    uint64_t *stw = gsva + 4 * (size_t)NS;                         // [10][NS]
    float *stf = reinterpret_cast<float *>(stw + 10 * (size_t)NS);  // [7][NS]
    uint32_t *stflag = reinterpret_cast<uint32_t *>(stf + 7 * (size_t)NS);
    int32_t *slot_list = reinterpret_cast<int32_t *>(stflag + NS);
    int32_t *ctr = slot_list + NS;  // [1] abort flag
    // rows a slot's trajectories recorded since the last count (a.row_done):
    // spend = lo | hi << 16 for rows [lo, hi) of the trajectory it holds (0:
    // none), sfin = lo + 1 for rows [lo, n_samples) of one that ended (0: none)
    uint32_t *spend = reinterpret_cast<uint32_t *>(ctr + 128);
    uint32_t *sfin = spend + NS;
    int32_t *fac = reinterpret_cast<int32_t *>(sfin + NS);
    int32_t *jsp = fac + (size_t)R * P;
    int32_t *ssave = jsp + (size_t)R * Q;  // saved species indices
    const int n_cache = spec_sample_cache(a);
    uint64_t *sTb = reinterpret_cast<uint64_t *>(
        (reinterpret_cast<uintptr_t>(ssave + a.n_save) + 15) & ~(uintptr_t)15);  // sample time bits
    float *sTf = reinterpret_cast<float *>(sTb + n_cache);                         // as float triples
    load_exact_tables(a, zxk, zf, zd, fac, jsp, jd);
    for (int k = tid; k < a.n_save; k += BD) ssave[k] = a.save_idx[k];
    for (int k = tid; k < n_cache; k += BD) {
        const double v = a.sample_t[k];
        sTb[k] = (uint64_t)__double_as_longlong(v);
        const TF f = tf_from_double(v);
        sTf[3 * k] = f.h;
        sTf[3 * k + 1] = f.m;
        sTf[3 * k + 2] = f.l;
    }
    for (int k = tid; k < 256; k += BD) {
        const double v = a.zig[kZigOffXdf + k];
        xdf[k] = *reinterpret_cast<const float2 *>(&v);
    }
    if (!a.rate_stride)
        for (int r = tid; r < R; r += BD) {
            const uint64_t rb = (uint64_t)__double_as_longlong(a.rate[r]);
            rate[r] = rb;
            const DF d = spec_rate_ok(rb) ? df_from_double(__longlong_as_double((long long)rb)) : DF{0.f, 0.f};
            rdf[r] = make_float2(d.h, d.l);
        }
    // every slot a lane may hold starts live and empty (no trajectory taken yet)
    const int lanes = a.lanes > 0 && a.lanes < 32 ? a.lanes : 32;
    for (int k = tid; k < NS; k += BD) {
        stflag[k] = lanes == 32 || (k % SPW) < lanes ? kLive : 0u;
        spend[k] = 0;
        sfin[k] = 0;
    }
    if (tid < 128) ctr[tid] = 0;
    __syncthreads();
    const ExactTables ex{zxk, zf, zd, fac, jsp, jd};

    // running-sum bound: the products and the reference's own roundings
    // (M + R + 2 gamma), plus the float32 accumulation of the low parts,
    // (r + M + 2) 2^-48 of the total at add r (1/16 gamma each)
    const float G = ((float)(a.max_mults + R + 2) +
                     (float)(R * (R + 1) / 2 + R * (a.max_mults + 2)) * 0.0625f) * kGamma;
    const float c_q = G + 6.0f * kGamma;                     // relative bound of Exp1/total
    // float32 choice margin / total: running sums within (R + M + 2) 2^-24,
    // U truncated to 2^-23, the product rounded (2^-24), the total's high
    // part within 2^-24
    const float c_sel = (float)(a.max_mults + R + 6) * 0x1p-24f * 1.001f;
    const int64_t t_start = global_ns();
    const int phase_steps = a.phase_steps > 0 ? a.phase_steps : kSpecPhase;
    unsigned int rot = 0;
    unsigned long long lane_events = 0;

    // ---- this lane's slot; the hot state sits in registers during a phase,
    // the cold words (interval start t0, sample time T, trajectory, event
    // count at the interval start, sample index) stay in the slot's columns
    int slot = lane < lanes ? wbase + lane : -1;
    int32_t *const wlist = slot_list + wbase;
    typename Ops::Counts c{};
    Xoshiro g{0, 0, 0, 0};
    TF Tc{0.f, 0.f, 0.f}, tc{0.f, 0.f, 0.f};  // sample time, clock
    float err_t = 0.f;                         // bound on |clock - reference clock|
    unsigned long long ev = 0;
    bool live = slot >= 0, have = false, nat = false, exact_traj = false, begin = false, abort_run = false;

    for (;;) {
        // rows this lane's slot recorded in the phase, counted after it by the
        // whole warp: rows [cnt_pw & 0xFFFF, cnt_pw >> 16) of its trajectory,
        // and for a trajectory that ended, rows [cnt_fw - 1, n_samples)
        uint32_t cnt_pw = 0, cnt_fw = 0;
        // ---------------------------------------------------------- phase
        if (slot >= 0) {
            int64_t *const sp = spa + slot;
            int64_t *const sps = spsa + slot;
            uint64_t *const gsv = gsva + slot;
            uint64_t *const st = stw + slot;  // cold words: st[k * NS]
            uint64_t *const rl = rate + (rate_cols ? slot : 0);
            float2 *const rf = rdf + (rate_cols ? slot : 0);
            for (int step = 0; step < phase_steps && live; ++step) {
                if (!have || begin) {  // rare: one branch for both
                    if (!have) {
                        // take the next trajectory into this slot
                        const long long traj = (long long)atomicAdd(a.work, 1ull);
                        if (traj >= a.n_traj) {
                            live = false;
                            break;
                        }
                        uint64_t t0;
                        if (a.in_species) {
                            for (int s = 0; s < S; ++s) sp[s * NS] = a.in_species[traj * S + s];
                            t0 = (uint64_t)__double_as_longlong(a.in_t[traj]);
                            g.s0 = a.in_rng[traj * 4 + 0];
                            g.s1 = a.in_rng[traj * 4 + 1];
                            g.s2 = a.in_rng[traj * 4 + 2];
                            g.s3 = a.in_rng[traj * 4 + 3];
                        } else {
                            for (int s = 0; s < S; ++s) sp[s * NS] = a.x0[traj * a.x0_stride + s];
                            t0 = 0;
                            xo_seed(g, a.seeds[traj]);
                        }
                        nat = !emul_domain(t0);
                        exact_traj = (t0 >> 52) > 1023 + 60;
                        for (int r = 0; r < R; ++r) {
                            const uint64_t rb = (uint64_t)__double_as_longlong(a.rate[traj * a.rate_stride + r]);
                            nat |= !emul_domain(rb);
                            exact_traj |= !spec_rate_ok(rb);
                            if (rate_cols) {
                                rl[r * RS] = rb;
                                const DF d = df_from_double(__longlong_as_double((long long)rb));
                                rf[r * RS] = make_float2(d.h, d.l);
                            }
                        }
                        exact_traj |= nat;
                        exact_traj |= !Ops::load(c, a, sp, NS);
                        tc = tf_from_double(__longlong_as_double((long long)t0));
                        st[4 * NS] = t0;
                        st[6 * NS] = (uint64_t)traj;
                        st[9 * NS] = 0;
                        ev = 0;
                        have = true;
                        begin = true;
                    }
                    if (begin) {
                        // a sample interval starts at t0 (the clock tc holds t0
                        // exactly): save what a re-run needs
                        const int si = (int)st[9 * NS];
                        if (si < n_cache) {
                            st[5 * NS] = sTb[si];
                            Tc = TF{sTf[3 * si], sTf[3 * si + 1], sTf[3 * si + 2]};
                        } else {
                            const double T = a.sample_t[si];
                            st[5 * NS] = (uint64_t)__double_as_longlong(T);
                            Tc = tf_from_double(T);
                        }
                        err_t = 0.f;
                        if (exact_traj)
                            for (int s = 0; s < S; ++s) sps[s * NS] = sp[s * NS];
                        else
                            Ops::save(c, a, sp, sps, NS);
                        gsv[0] = g.s0;
                        gsv[NS] = g.s1;
                        gsv[2 * NS] = g.s2;
                        gsv[3 * NS] = g.s3;
                        st[8 * NS] = ev;
                        begin = false;
                    }
                }

                bool fire = false, replay = exact_traj;
                int idx = 0;
                if (!replay) {
                    // Float-pair step.  Both draws the step may make are taken
                    // ahead (the reference draws Exp1 only when total > 0 and
                    // the uniform only when the reaction fires), so they
                    // overlap the propensities; a step that commits fewer
                    // draws steps the generator back.  An undecided step
                    // re-runs the interval from its saved state.
                    const uint64_t b1 = xo_next(g);
                    const uint64_t b2 = xo_next(g);
                    const int i1 = (int)(b1 & 0xff);
                    const uint64_t k1 = b1 >> 12;
                    const uint64_t K1 = ex.zxk[i1].y;
                    const float2 X1 = xdf[i1];
                    DF x = df_mul(df_u53(2 * k1 + 1), DF{X1.x, X1.y});
                    float xerr = kGamma * X1.x;
                    float cum[MAXR];
                    DF tot;
                    bool amb = Ops::props(a, ex, c, sp, NS, rf, RS, cum, tot);
                    const bool slow = !(k1 < K1);
                    uint64_t bu = b2;
                    if (tot.h > 0.0f) {
                        if (slow) {
                            // wedge or tail: b2 was its uniform, the choice
                            // takes the draw after the Exp1 is settled
                            x = exp1_df_cont(g, b1, b2, x, ex, xdf, xerr);
                            bu = xo_next(g);
                        }
                        amb |= tot.h < 0x1p-90f || tot.h > 0x1p90f;
                        const float r = rcp_approx(tot.h);
                        const DF q = df_div(x, tot, r);
                        const TF tn = tf_add(tc, q);
                        // error bound, rounded up: previous bound, Exp1/total
                        // against the reference's quotient, the reference's
                        // rounding of its clock add, the low part's roundings
                        float err_tn = __fadd_ru(err_t, __fmul_ru(c_q, q.h));
                        err_tn = __fadd_ru(err_tn, __fmul_ru(__fmul_ru(xerr, r), 1.001f));
                        err_tn = __fadd_ru(err_tn, __fmul_ru(0x1p-52f, tn.h));
                        err_tn = __fadd_ru(err_tn, __fmul_ru(0x1p-23f, fabsf(tn.l)));
                        // T - tn: the high difference is exact near T, the
                        // rest is below 2^-46 max(T, tn) off
                        const float d = __fadd_rn(__fsub_rn(Tc.h, tn.h),
                                                  __fadd_rn(__fsub_rn(Tc.m, tn.m), __fsub_rn(Tc.l, tn.l)));
                        const float mt = __fadd_ru(err_tn, __fmul_ru(0x1p-44f, fmaxf(Tc.h, tn.h)));
                        const float dd = __fmul_rn(d, 1.0f - 0x1p-22f);
                        fire = dd > mt;
                        amb |= !(fire || dd < -mt) || !(err_tn < 1.0e30f) || q.h < 0x1p-100f;
                        // choice #{r : cum_r < total * U} in float32: the high
                        // parts are within 2^-23.9 of the exact sums, U and the
                        // product add 2^-23 each; a comparison inside that
                        // margin is redone exactly in binary64
                        const float ch = __fmul_rn(tot.h, f23((uint32_t)(bu >> 41)) * 0x1p-23f);
                        const float msel = c_sel * tot.h;
                        bool close = false;
#pragma unroll
                        for (int rr = 0; rr < MAXR; ++rr) {
                            if (rr < R) {
                                const float dr = __fsub_rn(cum[rr], ch);
                                idx += dr < 0.0f ? 1 : 0;
                                close |= fabsf(dr) <= msel;
                            }
                        }
                        if (!amb && fire && !close) {
                            // the common step, decided in float32: commit the
                            // clock and fire the reaction
                            tc = tn;
                            err_t = err_tn;
                            ++ev;
                            Ops::jump(c, a, ex, sp, NS, idx);
                            continue;
                        }
                        if (!amb) {
                            if (fire) {
                                if (close) idx = Ops::exact_choice(a, ex, c, sp, NS, rl, RS, bu >> 11);
                                tc = tn;
                                err_t = err_tn;
                            } else {
                                // the sample records: the Exp1 draw alone was made
                                xo_prev(g);
                            }
                        }
                    } else {
                        // no reaction can fire: no draw is made
                        xo_prev(g);
                        xo_prev(g);
                    }
                    replay = amb;
                }
                if (replay) {
                    if (!exact_traj) atomicAdd(a.work + 3, 1ull);  // speculation undecided
                    const unsigned long long ev0 = st[8 * NS];
                    ev = replay_interval<MAXR, MACRO>(a, ex, sp, sps, gsv, rl, RS, NS, st[4 * NS], st[5 * NS], nat,
                                                      ev0, t_start);
                    if (ev == ~0ull) {
                        ev = ev0;
                        abort_run = true;
                        break;
                    }
                    g = Xoshiro{gsv[0], gsv[NS], gsv[2 * NS], gsv[3 * NS]};
                    exact_traj |= !Ops::load(c, a, sp, NS);
                    fire = false;
                }
                if (fire) {
                    ++ev;
                    Ops::jump(c, a, ex, sp, NS, idx);
                } else {
                    // record sample i at t = T
                    if (!replay) Ops::store(c, a, sp, NS);
                    const long long traj = (long long)st[6 * NS];
                    const uint64_t i = st[9 * NS];
                    int64_t *o = a.out + (size_t)i * a.n_save * a.n_traj + traj;
                    for (int k = 0; k < a.n_save; ++k) o[(size_t)k * a.n_traj] = sp[ssave[k] * NS];
                    if (a.row_done) {
                        const uint32_t pw = spend[slot];
                        spend[slot] = (pw ? (pw & 0xFFFFu) : (uint32_t)i) | ((uint32_t)(i + 1) << 16);
                    }
                    if ((long long)i + 1 < a.n_samples) {
                        st[9 * NS] = i + 1;
                        st[4 * NS] = st[5 * NS];  // next interval starts at T
                        tc = Tc;
                        begin = true;
                    } else {
                        const uint64_t T = st[5 * NS];
                        if (a.fin_species)
                            for (int s = 0; s < S; ++s) a.fin_species[traj * S + s] = sp[s * NS];
                        if (a.fin_t) a.fin_t[traj] = __longlong_as_double((long long)T);
                        if (a.fin_rng) {
                            a.fin_rng[traj * 4 + 0] = g.s0;
                            a.fin_rng[traj * 4 + 1] = g.s1;
                            a.fin_rng[traj * 4 + 2] = g.s2;
                            a.fin_rng[traj * 4 + 3] = g.s3;
                        }
                        if (a.events) a.events[traj] = ev;
                        lane_events += ev;
                        have = false;
                        if (a.row_done) {
                            // a second trajectory ending in one phase counts
                            // the first one's rows now
                            if (sfin[slot]) count_rows(a, sfin[slot] - 1u, (uint32_t)a.n_samples);
                            sfin[slot] = (spend[slot] & 0xFFFFu) + 1u;
                            spend[slot] = 0;
                        }
                    }
                }
            }
            // ---- the wall-clock budget, once per phase (a phase is at most
            // phase_steps steps, and an interval re-run checks it itself)
            if (global_ns() - t_start > a.budget_ns) abort_run = true;
            // ---- the rows recorded in this phase, counted below by the warp
            if (a.row_done) {
                cnt_pw = spend[slot];
                cnt_fw = sfin[slot];
                spend[slot] = 0;
                sfin[slot] = 0;
            }
            // ---- park the slot's hot state
            if (live) {
                if (have && !exact_traj) Ops::store(c, a, sp, NS);
                st[0 * NS] = g.s0;
                st[1 * NS] = g.s1;
                st[2 * NS] = g.s2;
                st[3 * NS] = g.s3;
                st[7 * NS] = ev;
                stf[0 * NS + slot] = tc.h;
                stf[1 * NS + slot] = tc.m;
                stf[2 * NS + slot] = tc.l;
                stf[3 * NS + slot] = err_t;
                stf[4 * NS + slot] = Tc.h;
                stf[5 * NS + slot] = Tc.m;
                stf[6 * NS + slot] = Tc.l;
            }
            stflag[slot] = (live ? kLive : 0u) | (have ? kHave : 0u) | (nat ? kNat : 0u) |
                           (exact_traj ? kExactTraj : 0u) | (begin ? kBegin : 0u);
            if (abort_run) ctr[1] = 1;
        }
        __syncwarp();
        // ---- count the phase's rows: one fence per lane (its sample stores
        // visible device-wide before any count), then per row one atomic add
        // of the number of the warp's lanes that completed it
        if (a.row_done && __any_sync(0xffffffffu, (cnt_pw | cnt_fw) != 0)) {
            __threadfence();
            const uint32_t plo = cnt_pw ? (cnt_pw & 0xFFFFu) : 0xFFFFFFFFu, phi = cnt_pw ? (cnt_pw >> 16) : 0u;
            const uint32_t flo = cnt_fw ? cnt_fw - 1u : 0xFFFFFFFFu, fhi = cnt_fw ? (uint32_t)a.n_samples : 0u;
            const uint32_t rlo = __reduce_min_sync(0xffffffffu, min(plo, flo));
            const uint32_t rhi = __reduce_max_sync(0xffffffffu, max(phi, fhi));
            for (uint32_t r = rlo; r < rhi; ++r) {
                const uint32_t n = __reduce_add_sync(0xffffffffu, (uint32_t)(r >= plo && r < phi) +
                                                                      (uint32_t)(r >= flo && r < fhi));
                if (lane == 0 && n) atomicAdd(a.row_done + r, n);
            }
        }
        // ---------------------------------------------------------- compaction
        // Each warp owns slots [wbase, wbase + SPW) and never waits for
        // another warp: its live slots, in slot order, go to its list, so the
        // warp stays full while trajectories end at different times.  With
        // more live slots than lanes the lanes take the 32 slots whose clocks
        // lag furthest behind (a.sched == 0), or the starting entry rotates by
        // 32 per phase (a.sched == 1).
        int n_live = 0;
        for (int c0 = 0; c0 < SPW; c0 += 32) {
            const int j = c0 + lane;
            const bool alive = j < SPW && (stflag[wbase + j] & kLive) != 0;
            const unsigned int bal = __ballot_sync(0xffffffffu, alive);
            if (alive) wlist[n_live + __popc(bal & ((1u << lane) - 1u))] = wbase + j;
            n_live += __popc(bal);
        }
        __syncwarp();
        const bool aborted = *reinterpret_cast<volatile int32_t *>(ctr + 1) != 0;
        if (n_live == 0 || aborted) {
            if (aborted && lane == 0) atomicExch(a.work + 2, 1ull);
            break;
        }
        if (n_live <= 32) {
            slot = lane < n_live ? wlist[lane] : -1;
            rot = 0;
        } else if (a.sched != 0 || n_live > 32 * kSpecSchedPerLane) {
            rot %= (unsigned int)n_live;
            unsigned int k = rot + (unsigned int)lane;
            if (k >= (unsigned int)n_live) k -= (unsigned int)n_live;
            slot = wlist[k];
            rot += 32u;
        } else {
            slot = lag_select(stf, stflag, wlist, n_live, lane);
        }
        live = slot >= 0;
        if (live) {
            const uint32_t fl = stflag[slot];
            have = (fl & kHave) != 0;
            nat = (fl & kNat) != 0;
            exact_traj = (fl & kExactTraj) != 0;
            begin = (fl & kBegin) != 0;
            g = Xoshiro{stw[0 * NS + slot], stw[1 * NS + slot], stw[2 * NS + slot], stw[3 * NS + slot]};
            ev = stw[7 * NS + slot];
            tc = TF{stf[0 * NS + slot], stf[1 * NS + slot], stf[2 * NS + slot]};
            err_t = stf[3 * NS + slot];
            Tc = TF{stf[4 * NS + slot], stf[5 * NS + slot], stf[6 * NS + slot]};
            if (have && !exact_traj) Ops::load(c, a, spa + slot, NS);
        }
        __syncwarp();  // slot flags are rewritten by the next phase
    }
    for (int off = 16; off > 0; off >>= 1) lane_events += __shfl_down_sync(0xffffffffu, lane_events, off);
    if ((tid & 31) == 0 && lane_events) atomicAdd(a.work + 1, lane_events);
}

}  // namespace rbg
