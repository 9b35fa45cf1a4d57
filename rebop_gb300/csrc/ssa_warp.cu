// Warp-per-trajectory SSA kernel for large networks (hundreds of species,
// thousands of reactions), where one trajectory's propensity pass is itself
// data-parallel work.
//
// Each step of rebop's direct method (gillespie.rs:315-344) recomputes every
// propensity and folds them left to right into cumulative sums
// (make_cumrates, gillespie.rs:357-364).  Here the 32 lanes of a warp own
// contiguous chunks of the reaction list: each lane evaluates its chunk's
// propensities in float pairs and sums them, a shuffle scan of the lane sums
// gives every chunk's prefix and the total, lane 0 holds the random stream,
// the triple-float clock and its error bound (as in ssa_spec_body.cuh), and
// the lane whose prefix range holds total * U walks its chunk to the chosen
// reaction.
//
// The reference's sums are a sequential binary64 fold, within (R + M + 2)
// 2^-53 of the exact sums; the float pairs are within a few 2^-44 of them.
// A decision whose operands lie farther apart than both bounds together is
// the reference's decision.  A close choice is redone for that step alone
// with the exact fold below; anything else -- a close clock comparison, a
// count outside [0, 2^23), a rate outside 2^-60 .. 2^60 -- re-runs the sample
// interval from its saved start with the exact step: lanes compute the
// binary64 propensities in the reference's multiply order and fold them in
// order lane after lane, lane 0 draws in native binary64, so counts, event
// numbers and the random stream equal rebop's bit for bit.
//
// After a reaction fires only the propensities reading a species it changed
// are re-evaluated (SsaArgs::dep_tab); a lane's chunk is summed in groups, so
// only the groups holding them are re-summed.
#include <cuda_runtime.h>

#include <algorithm>

#include "ssa_spec_body.cuh"

namespace rbg {

namespace {

constexpr int kWarpMaxWarps = 16;
// batch launches: small per-warp regions, so registers set the warps per SM
constexpr int kWarpMaxWarpsBatch = 24;

struct WarpLayout {
    size_t block_bytes, warp_bytes;
};

// Lane l owns the C = ceil(R / 32) reactions l*C .. l*C + C - 1.  Arrays the
// lanes walk together are stored lane-major -- reaction l*C + i at position
// i*32 + l -- so one step of the walk touches 32 consecutive words.
__host__ __device__ inline int warp_chunk(int R) { return (R + 31) / 32; }

// A lane's chunk is summed in groups of warp_group(C) reactions (at most 32
// groups), so that re-evaluating a few propensities re-sums only their groups.
__host__ __device__ inline int warp_group(int C) { return C > 256 ? (C + 31) / 32 : 8; }
__host__ __device__ inline int warp_ngroups(int C) { return (C + warp_group(C) - 1) / warp_group(C); }

// Every reaction of order <= 2 over fewer than 32767 species: propensities
// come from two-slot shapes (shape_word) and the factor list is not needed.
__host__ __device__ inline bool warp_shape2(const SsaArgs &a) { return a.max_mults <= 2 && a.S < 32767; }

// Shared memory: block tables (Exp1 tables, float-pair rates when shared,
// reactant factors in both layouts, jumps), then per warp: counts,
// float-pair propensities (and float-pair rates when per trajectory).  The
// counts at the interval start go to global memory (SsaArgs::warp_cnt0).
__host__ __device__ inline WarpLayout warp_layout(const SsaArgs &a) {
    WarpLayout l;
    const size_t RP = 32 * (size_t)warp_chunk(a.R);     // lane-major positions
    size_t b = 16 * 256 + 8 * 257 + 8 * 256 + 8 * 256;  // zxk, zf, zd, xdf
    if (!a.batch) {  // a batch's networks stay in global memory
        b += 8 * RP;                                        // shared float-pair rates (lane-major)
        if (!warp_shape2(a)) b += 4 * RP * a.P;             // factors (lane-major), when shapes do not cover
        b += 4 * RP;                                        // two-slot reaction shapes (lane-major)
        b += 2 * (size_t)a.R * a.Q + 2 * (size_t)a.R * a.Q; // jumps: species, deltas (16 bit each)
        b += 16;                                            // alignment of the jump deltas
    }
    l.block_bytes = (b + 15) & ~(size_t)15;
    size_t w = 8 * (size_t)a.S;                         // counts
    w += 4 * ((size_t)a.S + 1);                         // counts as floats, plus the constant 1
    w += 8 * RP + 8;                                    // propensities (lane-major), alignment
    if (a.rate_stride) w += 8 * RP;                     // per-trajectory float-pair rates
    if (!a.batch) w += 8 * 32 * (size_t)warp_ngroups(warp_chunk(a.R)) + 4 * 32;  // group sums, dirty masks
    const size_t wt = 8 * 32 * (2 * (size_t)a.tbatch_S + 4);  // a thread unit's counts, their copy, generator
    if (a.batch && wt > w) w = wt;
    l.warp_bytes = (w + 15) & ~(size_t)15;
    return l;
}

// Physical slot of the float-pair propensity at lane-major position pos
// (reaction l*C + i at i*32 + l): the lane bits are XORed with the row, so a
// row read by the 32 lanes (the chunk sums) and a column read by the 32 lanes
// (the walk through one lane's chunk to the chosen reaction) both touch 32
// distinct banks.  Without it every lane of the walk hit the same bank.
__device__ __forceinline__ int pz(int pos) { return pos ^ ((pos >> 5) & 31); }

__device__ __forceinline__ DF shfl_df(DF v, int src) {
    return DF{__shfl_sync(0xffffffffu, v.h, src), __shfl_sync(0xffffffffu, v.l, src)};
}

__device__ __forceinline__ DF shfl_up_df(DF v, int d) {
    return DF{__shfl_up_sync(0xffffffffu, v.h, d), __shfl_up_sync(0xffffffffu, v.l, d)};
}

__device__ __forceinline__ double shfl_d(double v, int src) {
    return __longlong_as_double(__shfl_sync(0xffffffffu, __double_as_longlong(v), src));
}

// Exact binary64 propensity of reaction r in the reference's multiply order:
// Rate::rate's fold (gillespie.rs:71-90), or the macro's integer falling
// factorials (gillespie_macro.rs:133-146).
template <bool MACRO>
__device__ __forceinline__ double exact_propensity(const SsaArgs &it, const int64_t *cnt, double rate, int r) {
    double acc = rate;
    for (int p = 0; p < it.P; ++p) {
        const int o = it.fac_ord[r * it.P + p];
        if (o == 0) continue;
        const int64_t n = cnt[it.fac_sp[r * it.P + p]];
        if (MACRO) {
            int64_t ff = n;
            for (int j = 1; j < o; ++j) ff *= n - j;
            acc = __dmul_rn(acc, (double)ff);
        } else {
            for (int j = o - 1; j >= 0; --j) acc = __dmul_rn(acc, (double)(n - j));
        }
    }
    return acc;
}

// Exact binary64 propensities and their running sums, in scr: this warp's
// shared-memory scratch of 32 * ceil(R / 32) doubles, lane-major like the
// chunks.  Lane l evaluates and folds its own reactions l*C .. l*C + C - 1, in
// order, starting from the running sum lane l - 1 hands over, so the sums are
// the reference's sequential fold (make_cumrates, gillespie.rs:357-364) while
// every lane reads only its own column.  Returns the total on every lane.
template <bool MACRO>
__device__ __forceinline__ double warp_exact_fold(const SsaArgs &it, const int64_t *cnt, const double *rates,
                                                  double *scr) {
    const int lane = threadIdx.x & 31, R = it.R, C = warp_chunk(R);
    const int r_lo = min(R, lane * C), n_own = min(R, r_lo + C) - r_lo;
    for (int i = 0; i < n_own; ++i) scr[i * 32 + lane] = exact_propensity<MACRO>(it, cnt, rates[r_lo + i], r_lo + i);
    // one lane's chunk after the other; loads go ahead in blocks of 8
    double run = 0.0;
    for (int l = 0; l < 32; ++l) {
        if (lane == l) {
            for (int i0 = 0; i0 < n_own; i0 += 8) {
                double v[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) v[j] = i0 + j < n_own ? scr[(i0 + j) * 32 + lane] : 0.0;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (i0 + j < n_own) {
                        run = __dadd_rn(run, v[j]);
                        scr[(i0 + j) * 32 + lane] = run;
                    }
            }
        }
        run = shfl_d(run, l);
    }
    return run;
}

// The reaction the reference picks for `chosen` from the running sums in scr:
// #{r : cum_r < chosen} (gillespie.rs:402-407), or for define_system! the
// first r with chosen < cum_r (gillespie_macro.rs:150-171); R if none.
template <bool MACRO>
__device__ __forceinline__ int warp_exact_pick(const SsaArgs &it, const double *scr, double chosen) {
    const int lane = threadIdx.x & 31, R = it.R, C = warp_chunk(R);
    const int r_lo = min(R, lane * C), n_own = min(R, r_lo + C) - r_lo;
    if (MACRO) {
        int first = n_own;
        for (int i = n_own - 1; i >= 0; --i)
            if (chosen < scr[i * 32 + lane]) first = i;
        const unsigned int has = __ballot_sync(0xffffffffu, first < n_own);
        if (!has) return R;
        const int l = __ffs((int)has) - 1;
        return l * C + __shfl_sync(0xffffffffu, first, l);
    }
    int c = 0;
    for (int i = 0; i < n_own; ++i) c += scr[i * 32 + lane] < chosen ? 1 : 0;
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
    return c;
}

// One exact step of the whole warp from the committed state (lane 0 holds the
// generator).  Returns 1 when a reaction fires (its index in idx, the clock in
// t), 0 when the step records the sample.
template <bool MACRO>
__device__ __noinline__ int warp_exact_step(const SsaArgs &it, const int64_t *cnt, const double *rates,
                                            const double *zig, double *scr, Xoshiro &g, double &t, double T,
                                            int &idx) {
    const int lane = threadIdx.x & 31;
    const double total = warp_exact_fold<MACRO>(it, cnt, rates, scr);
    int fire = 0;
    double chosen = 0.0;
    if (lane == 0 && 0.0 < total) {
        const double tn = __dadd_rn(t, __ddiv_rn(xo_exp1(g, zig, zig + kZigOffF), total));
        if (!(tn > T)) {
            fire = 1;
            t = tn;
            chosen = __dmul_rn(total, xo_uniform(g));
        }
    }
    fire = __shfl_sync(0xffffffffu, fire, 0);
    t = shfl_d(t, 0);
    if (!fire) return 0;
    idx = warp_exact_pick<MACRO>(it, scr, shfl_d(chosen, 0));
    return 1;
}

// The exact choice alone, for a step whose clock the float pairs decided
// (the reaction fires) but whose choice they left close: the reference's
// total, chosen = total * U for the uniform's top 53 bits u53, and the pick.
// Overwrites scr.
template <bool MACRO>
__device__ __noinline__ int warp_exact_choice(const SsaArgs &it, const int64_t *cnt, const double *rates,
                                              double *scr, uint64_t u53) {
    const double total = warp_exact_fold<MACRO>(it, cnt, rates, scr);
    const double chosen = __dmul_rn(total, __dmul_rn((double)u53, 0x1.0p-53));
    return warp_exact_pick<MACRO>(it, scr, chosen);
}

// Two-slot shape of reaction r (reactant order <= 2): slots (species, offset)
// 2A -> (A,0)(A,1); A+B -> (A,0)(B,0); A -> (A,0)(one); none -> (one)(one),
// species S standing for a constant 1.  The propensity is then
// rate * max(n1 - o1, 0) * max(n2 - o2, 0), without branches.
__host__ __device__ inline uint32_t shape_word(const int32_t *fac_sp, const int32_t *fac_ord, int P, int S, int r) {
    uint32_t sl[2] = {(uint32_t)S, (uint32_t)S}, of[2] = {0, 0};
    int k = 0;
    for (int p = 0; p < P; ++p) {
        const int o = fac_ord[r * P + p];
        for (int j = 0; j < o && k < 2; ++j, ++k) {
            sl[k] = (uint32_t)fac_sp[r * P + p];
            of[k] = (uint32_t)j;
        }
    }
    return sl[0] | of[0] << 15 | sl[1] << 16 | of[1] << 31;
}

// One thread unit of a persistent batch: lane l runs trajectory first + l of
// the small-network item `it` (if it has one) from start to end with the
// speculative float-pair step of the thread kernels (ssa_spec_body.cuh):
// propensities as float pairs summed into a float32 running sum, the clock as
// a float triple with a rigorous error bound, the choice in float32 with an
// exact binary64 decision when it is close, and an exact re-run of any sample
// interval whose clock decision the bound leaves open -- so its counts,
// events and draws are rebop's.  wreg is this warp's region: counts [S][32],
// counts at the interval start [S][32] and the generator there [4][32].
// Returns the lane's event count; sets `late` if the wall-clock budget ran
// out (the trajectory is then incomplete).
// MAXR bounds the item's reactions (4, 8 or 16): the per-reaction loops are
// unrolled to it.
template <bool MACRO, int MAXR>
__device__ __noinline__ unsigned long long thread_unit(const SsaArgs &it, const ExactTables &zt, const float2 *xdf,
                                                       unsigned char *wreg, long long first, int64_t t_start,
                                                       bool &late) {
    using Ops = TableOps<MAXR, MACRO>;
    constexpr int NS = 32;  // column stride of the per-lane arrays
    const int lane = threadIdx.x & 31;
    const long long traj = first + lane;
    if (traj >= it.n_traj) return 0;
    const int S = it.S, R = it.R;
    int64_t *sp = reinterpret_cast<int64_t *>(wreg) + lane;
    int64_t *sps = sp + NS * S;
    uint64_t *gsv = reinterpret_cast<uint64_t *>(sps + NS * S);
    const ExactTables ex{zt.zxk, zt.zf, zt.zd, it.fac_packed, it.jmp_sp, it.jmp_d};
    for (int s = 0; s < S; ++s) sp[s * NS] = it.x0[traj * it.x0_stride + s];
    Xoshiro g;
    xo_seed(g, it.seeds[traj]);
    const uint64_t *rl = reinterpret_cast<const uint64_t *>(it.rate + traj * it.rate_stride);
    const float2 *rf = it.lm_rdf + traj * it.rate_stride;
    bool nat = false, exact_traj = false;
    for (int r = 0; r < R; ++r) {
        nat |= !emul_domain(rl[r]);
        exact_traj |= !spec_rate_ok(rl[r]);
    }
    exact_traj |= nat;
    // error model of the float-pair step (ssa_spec_body.cuh)
    const float G = ((float)(it.max_mults + R + 2) + (float)(R * (R + 1) / 2 + R * (it.max_mults + 2)) * 0.0625f) *
                    kGamma;
    const float c_q = G + 6.0f * kGamma;
    const float c_sel = (float)(it.max_mults + R + 6) * 0x1p-24f * 1.001f;
    typename Ops::Counts c{};
    unsigned long long ev = 0;
    uint64_t t0 = 0;  // clock at the interval start (bits)
    unsigned int tick = 0;
    for (long long i = 0; i < it.n_samples; ++i) {
        const double Td = it.sample_t[i];
        const uint64_t T = (uint64_t)__double_as_longlong(Td);
        const TF Tc = tf_from_double(Td);
        TF tc = tf_from_double(__longlong_as_double((long long)t0));
        float err_t = 0.0f;
        for (int s = 0; s < S; ++s) sps[s * NS] = sp[s * NS];
        gsv[0] = g.s0;
        gsv[NS] = g.s1;
        gsv[2 * NS] = g.s2;
        gsv[3 * NS] = g.s3;
        const unsigned long long ev0 = ev;
        bool replay = exact_traj;
        while (!replay) {
            if ((++tick & 1023u) == 0 && global_ns() - t_start > it.budget_ns) {
                late = true;
                return ev;
            }
            // both draws the step may make, taken ahead (stepped back when fewer
            // are committed)
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
            bool amb = Ops::props(it, ex, c, sp, NS, rf, 1, cum, tot);
            const bool slow = !(k1 < K1);
            uint64_t bu = b2;
            if (!(tot.h > 0.0f)) {
                xo_prev(g);  // no reaction can fire: no draw is made
                xo_prev(g);
                if (amb) replay = true;
                break;  // the sample records
            }
            if (slow) {
                x = exp1_df_cont(g, b1, b2, x, ex, xdf, xerr);
                bu = xo_next(g);
            }
            amb |= tot.h < 0x1p-90f || tot.h > 0x1p90f;
            const float rr = rcp_approx(tot.h);
            const DF q = df_div(x, tot, rr);
            const TF tn = tf_add(tc, q);
            float err_tn = __fadd_ru(err_t, __fmul_ru(c_q, q.h));
            err_tn = __fadd_ru(err_tn, __fmul_ru(__fmul_ru(xerr, rr), 1.001f));
            err_tn = __fadd_ru(err_tn, __fmul_ru(0x1p-52f, tn.h));
            err_tn = __fadd_ru(err_tn, __fmul_ru(0x1p-23f, fabsf(tn.l)));
            const float d = __fadd_rn(__fsub_rn(Tc.h, tn.h), __fadd_rn(__fsub_rn(Tc.m, tn.m), __fsub_rn(Tc.l, tn.l)));
            const float mt = __fadd_ru(err_tn, __fmul_ru(0x1p-44f, fmaxf(Tc.h, tn.h)));
            const float dd = __fmul_rn(d, 1.0f - 0x1p-22f);
            const bool fire = dd > mt;
            amb |= !(fire || dd < -mt) || !(err_tn < 1.0e30f) || q.h < 0x1p-100f;
            if (amb) {
                replay = true;
                break;
            }
            if (!fire) {
                xo_prev(g);  // the sample records: the Exp1 draw alone was made
                break;
            }
            const float ch = __fmul_rn(tot.h, f23((uint32_t)(bu >> 41)) * 0x1p-23f);
            const float msel = c_sel * tot.h;
            bool close = false;
            int idx = 0;
#pragma unroll
            for (int r = 0; r < MAXR; ++r) {
                if (r < R) {
                    const float dr = __fsub_rn(cum[r], ch);
                    idx += dr < 0.0f ? 1 : 0;
                    close |= fabsf(dr) <= msel;
                }
            }
            if (close) idx = Ops::exact_choice(it, ex, c, sp, NS, rl, 1, bu >> 11);
            tc = tn;
            err_t = err_tn;
            ++ev;
            Ops::jump(c, it, ex, sp, NS, idx);
        }
        if (replay) {
            // the interval again, exactly, from its saved start
            ev = replay_interval<MAXR, MACRO>(it, ex, sp, sps, gsv, rl, 1, NS, t0, T, nat, ev0, t_start);
            if (ev == ~0ull) {
                late = true;
                return ev0;
            }
            g = Xoshiro{gsv[0], gsv[NS], gsv[2 * NS], gsv[3 * NS]};
        }
        int64_t *o = it.out + (size_t)i * it.n_save * it.n_traj + traj;
        for (int k = 0; k < it.n_save; ++k) o[(size_t)k * it.n_traj] = sp[it.save_idx[k] * NS];
        t0 = T;  // the sample records at T (gillespie.rs:328-330)
    }
    if (it.events) it.events[traj] = ev;
    return ev;
}

// BATCH: the launch runs a.batch's networks (each item's tables in global
// memory, lane-major) and a.tbatch's thread units; otherwise the one network
// of `a`, whose tables the block copies to shared memory.
template <bool MACRO, bool BATCH>
__global__ void __launch_bounds__(32 * (BATCH ? kWarpMaxWarpsBatch : kWarpMaxWarps), 1)
    ssa_warp_kernel(const __grid_constant__ SsaArgs a) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const WarpLayout L = warp_layout(a);  // sized for the largest network of the launch

    // ---- block tables: Exp1 tables; in single-network mode also the
    // network's lane-major rates, factors, shapes and its jumps
    ulonglong2 *zxk = reinterpret_cast<ulonglong2 *>(g_spec_smem);
    uint64_t *zf = reinterpret_cast<uint64_t *>(zxk + 256);
    uint64_t *zd = zf + 257;
    float2 *xdf = reinterpret_cast<float2 *>(zd + 256);
    float2 *rdf_sh = xdf + 256;
    const int C0 = warp_chunk(a.R), RP0 = 32 * C0;
    const bool shape2 = warp_shape2(a);
    int32_t *facl_sh = reinterpret_cast<int32_t *>(rdf_sh + RP0);  // absent (size 0) when shape2
    uint32_t *shape_sh = reinterpret_cast<uint32_t *>(facl_sh + (shape2 ? 0 : (size_t)RP0 * a.P));
    // jumps of the one network: species as 16-bit indices (S < 65536), deltas
    // as 16-bit values when every one fits (else read from the descriptor)
    uint16_t *jsp_sh = reinterpret_cast<uint16_t *>(shape_sh + RP0);
    int16_t *jd_sh = reinterpret_cast<int16_t *>(
        (reinterpret_cast<uintptr_t>(jsp_sh + (size_t)a.R * a.Q) + 15) & ~(uintptr_t)15);
    for (int k = tid; k < 256; k += blockDim.x) {
        zxk[k] = make_ulonglong2((uint64_t)__double_as_longlong(a.zig[k]),
                                 (uint64_t)__double_as_longlong(a.zig[kZigOffK + k]));
        zd[k] = (uint64_t)__double_as_longlong(a.zig[kZigOffD + k]) & ~(1ull << 63);
    }
    for (int k = tid; k < 257; k += blockDim.x) zf[k] = (uint64_t)__double_as_longlong(a.zig[kZigOffF + k]);
    bool jd_wide = false;
    if (!BATCH) {
        for (int k = tid; k < a.R * a.Q; k += blockDim.x) {
            const int64_t dlt = a.jmp_d[k];
            jsp_sh[k] = (uint16_t)a.jmp_sp[k];
            jd_sh[k] = (int16_t)dlt;
            jd_wide |= dlt != (int64_t)(int16_t)dlt;
        }
        for (int q = tid; q < RP0; q += blockDim.x) {
            const int i = q >> 5, l = q & 31, r = l * C0 + i;
            if (!a.rate_stride) {
                const DF d = r < a.R ? df_from_double(a.rate[r]) : DF{0.f, 0.f};
                rdf_sh[q] = make_float2(d.h, d.l);
            }
            if (shape2) {
                shape_sh[q] = r < a.R ? shape_word(a.fac_sp, a.fac_ord, a.P, a.S, r) : (uint32_t)a.S << 16 | a.S;
            } else {
                for (int p = 0; p < a.P; ++p)
                    facl_sh[(i * a.P + p) * 32 + l] =
                        r < a.R ? (a.fac_sp[r * a.P + p] | (a.fac_ord[r * a.P + p] << 16)) : 0;
            }
        }
    }
    for (int k = tid; k < 256; k += blockDim.x) {
        const double v = a.zig[kZigOffXdf + k];
        xdf[k] = *reinterpret_cast<const float2 *>(&v);
    }
    jd_wide = __syncthreads_or(jd_wide);
    // the Exp1 draws use the ziggurat tables only
    const ExactTables ex{zxk, zf, zd, nullptr, nullptr, nullptr};

    // ---- this warp's region (sized for the largest network)
    unsigned char *wbase = g_spec_smem + L.block_bytes + (size_t)warp * L.warp_bytes;
    int64_t *cnt = reinterpret_cast<int64_t *>(wbase);
    int64_t *cnt0 = a.warp_cnt0 + ((size_t)blockIdx.x * nw + warp) * (size_t)a.S;  // global
    float *cntf = reinterpret_cast<float *>(cnt + a.S);  // [S + 1]
    float2 *prop = reinterpret_cast<float2 *>((reinterpret_cast<uintptr_t>(cntf + a.S + 1) + 7) & ~(uintptr_t)7);
    float2 *rdf_w = prop + RP0;  // per-trajectory float-pair rates (single-network mode)
    float2 *gsum = rdf_w + (a.rate_stride ? RP0 : 0);  // group sums [NG][32] (one network only)
    uint32_t *dmask = reinterpret_cast<uint32_t *>(gsum + 32 * (size_t)warp_ngroups(C0));  // dirty groups per lane
    // exact steps use the propensity array as their scratch (32 * C doubles)
    double *scr = reinterpret_cast<double *>(prop);
    const int64_t t_start = global_ns();
    unsigned long long warp_events = 0;
    bool abort_run = false;

    for (;;) {
        long long ticket = 0;
        if (lane == 0) ticket = (long long)atomicAdd(a.work, 1ull);
        ticket = __shfl_sync(0xffffffffu, ticket, 0);
        if (ticket >= a.n_traj) break;

        // ---- a thread unit: 32 trajectories of a small network, one per lane
        if (BATCH && ticket >= a.n_warp_tickets) {
            const long long u = ticket - a.n_warp_tickets;
            int lo = 0, hi = a.tbatch_n - 1;  // last item with tbatch_unit <= u
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (a.tbatch_unit[mid] <= u) lo = mid;
                else hi = mid - 1;
            }
            bool late = false;
            const SsaArgs &ti = a.tbatch[lo];
            const long long first = (u - a.tbatch_unit[lo]) * 32;
            unsigned long long ev = ti.R <= 4   ? thread_unit<MACRO, 4>(ti, ex, xdf, wbase, first, t_start, late)
                                    : ti.R <= 8 ? thread_unit<MACRO, 8>(ti, ex, xdf, wbase, first, t_start, late)
                                                : thread_unit<MACRO, 16>(ti, ex, xdf, wbase, first, t_start, late);
            for (int off = 16; off > 0; off >>= 1) ev += __shfl_xor_sync(0xffffffffu, ev, off);
            warp_events += ev;
            if (__any_sync(0xffffffffu, late)) {
                if (lane == 0) atomicExch(a.work + 2, 1ull);
                break;
            }
            __syncwarp();
            continue;
        }

        // ---- the trajectory's network and run
        long long traj = ticket;
        const SsaArgs *itp = &a;
        if (BATCH) {
            int lo = 0, hi = a.batch_n - 1;  // last item with batch_start <= ticket
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (a.batch_start[mid] <= ticket) lo = mid;
                else hi = mid - 1;
            }
            itp = a.batch + lo;
            traj = ticket - a.batch_start[lo];
        }
        const SsaArgs &it = *itp;
        const int S = it.S, R = it.R, P = it.P, Q = it.Q;
        const int C = warp_chunk(R);
        const float2 *rdf = BATCH ? it.lm_rdf : (it.rate_stride ? rdf_w : rdf_sh);
        const int32_t *facl = BATCH ? it.lm_fac : facl_sh;
        const uint32_t *shape = BATCH ? it.lm_shape : shape_sh;
        const bool use_shape = BATCH ? it.lm_shape != nullptr : (it.max_mults <= 2 && it.S < 32767);
        // reaction j's k-th jump entry: species, delta
        auto jump_sp = [&](int e) -> int { return BATCH ? it.jmp_sp[e] : (int)jsp_sh[e]; };
        auto jump_d = [&](int e) -> int64_t { return BATCH || jd_wide ? it.jmp_d[e] : (int64_t)jd_sh[e]; };
        // lane l owns reactions [l * C, min(R, (l + 1) * C)); local index i sits at i*32 + l
        const int r_lo = min(R, lane * C), r_hi = min(R, r_lo + C);
        const int n_own = r_hi - r_lo;
        const int mm = use_shape ? 2 : it.max_mults;  // multiplies per propensity
        const int GS = warp_group(C), NG = warp_ngroups(C);
        // dependency table (one network only: a batch's small networks gain
        // nothing from it); a reaction with more than 31 dependents
        // re-evaluates everything after it fires
        const bool deps = !BATCH && a.dep_tab != nullptr;
        // adds on the way to a chunk sum: a batch sums its chunk in order (C),
        // one network sums groups and then their sums (at most GS + NG)
        const int depth = BATCH ? C : GS + NG;
        const float c_tot = (float)(mm + 1 + depth + 5) * kGamma + (float)(R + mm + 4) * 0x1p-53f;
        const float c_q = c_tot + 6.0f * kGamma;
        const float c_sel = 2.0f * (c_tot + (float)(C + 4) * kGamma);
        // float-pair propensity of the reaction at lane-major position pos;
        // bad is set when a count it reads lies outside [0, 2^23)
        auto eval_prop = [&](int pos, bool &bad) -> DF {
            const float2 k = rdf[pos];
            if (use_shape) {
                const uint32_t w = shape[pos];
                const float n1 = cntf[w & 0x7FFFu], n2 = cntf[(w >> 16) & 0x7FFFu];
                bad |= !(n1 >= 0.0f && n1 < 8388608.0f && n2 >= 0.0f && n2 < 8388608.0f);
                const float f1 = fmaxf(__fsub_rn(n1, (float)((w >> 15) & 1u)), 0.0f);
                const float f2 = fmaxf(__fsub_rn(n2, (float)(w >> 31)), 0.0f);
                return df_mul_fu(df_mul_fu(DF{k.x, k.y}, f1), f2);
            }
            const int i2 = pos >> 5, l = pos & 31;
            DF acc{k.x, k.y};
            for (int p = 0; p < P; ++p) {
                const int f = facl[(i2 * P + p) * 32 + l];
                const int o = f >> 16;
                if (o == 0) continue;
                const int64_t n = cnt[f & 0xFFFF];
                bad |= (uint64_t)n >= (1ull << 23);
                for (int j = 0; j < o; ++j) {
                    const int64_t x = n - j > 0 ? n - j : 0;
                    acc = df_mul_fu(acc, f23((uint32_t)x & 0x7FFFFFu));
                }
            }
            return acc;
        };
        // sum of this lane's group g (its propensities already in prop), as
        // a pairwise tree for groups of 8
        auto group_sum = [&](int g) -> DF {
            const int b = g * GS, e = min(n_own, b + GS);
            if (GS == 8) {
                DF v[8];
#pragma unroll
                for (int t = 0; t < 8; ++t) {
                    const float2 q = b + t < e ? prop[pz((b + t) * 32 + lane)] : make_float2(0.f, 0.f);
                    v[t] = DF{q.x, q.y};
                }
                return df_add(df_add(df_add(v[0], v[1]), df_add(v[2], v[3])),
                              df_add(df_add(v[4], v[5]), df_add(v[6], v[7])));
            }
            DF s{0.f, 0.f};
            for (int i2 = b; i2 < e; ++i2) {
                const float2 q = prop[pz(i2 * 32 + lane)];
                s = df_add(s, DF{q.x, q.y});
            }
            return s;
        };
        // this lane's chunk sum from its group sums (pairwise up to 4 groups)
        auto chunk_sum = [&]() -> DF {
            if (NG <= 4) {
                DF v[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const float2 q = t < NG ? gsum[t * 32 + lane] : make_float2(0.f, 0.f);
                    v[t] = DF{q.x, q.y};
                }
                return df_add(df_add(v[0], v[1]), df_add(v[2], v[3]));
            }
            DF s{0.f, 0.f};
            for (int g = 0; g < NG; ++g) {
                const float2 q = gsum[g * 32 + lane];
                s = df_add(s, DF{q.x, q.y});
            }
            return s;
        };
        bool need_full = true;  // every propensity to be evaluated
        bool amb_next = false;  // a re-evaluated propensity read a count out of range
        DF ls{0.f, 0.f};        // this lane's chunk sum

        // ---- start (or resume) the trajectory
        Xoshiro g{0, 0, 0, 0};
        double t;
        if (it.in_species) {
            for (int s = lane; s < S; s += 32) cnt[s] = it.in_species[traj * S + s];
            t = it.in_t[traj];
            if (lane == 0)
                g = Xoshiro{it.in_rng[traj * 4], it.in_rng[traj * 4 + 1], it.in_rng[traj * 4 + 2],
                            it.in_rng[traj * 4 + 3]};
        } else {
            for (int s = lane; s < S; s += 32) cnt[s] = it.x0[traj * it.x0_stride + s];
            t = 0.0;
            if (lane == 0) xo_seed(g, it.seeds[traj]);
        }
        const double *rates = it.rate + traj * it.rate_stride;
        bool exact_traj = !spec_rate_ok((uint64_t)__double_as_longlong(t)) || !(t < 0x1p60);
        for (int r = lane; r < R; r += 32) exact_traj |= !spec_rate_ok((uint64_t)__double_as_longlong(rates[r]));
        if (!BATCH && it.rate_stride)
            for (int q = lane; q < 32 * C; q += 32) {
                const int r = (q & 31) * C + (q >> 5);
                const DF d = r < R ? df_from_double(rates[r]) : DF{0.f, 0.f};
                rdf_w[q] = make_float2(d.h, d.l);
            }
        exact_traj = __any_sync(0xffffffffu, exact_traj);
        for (int s = lane; s <= S; s += 32) cntf[s] = s < S ? (float)cnt[s] : 1.0f;
        __syncwarp();
        unsigned long long ev = 0;

        for (long long i = 0; i < it.n_samples && !abort_run; ++i) {
            const double T = it.sample_t[i];
            // ---- interval start: save what an exact re-run needs
            for (int s = lane; s < S; s += 32) cnt0[s] = cnt[s];
            const Xoshiro g0 = g;
            const double t0 = t;
            const unsigned long long ev0 = ev;
            const TF Tc = tf_from_double(T);
            TF tc = tf_from_double(t0);
            float err_t = 0.0f;
            bool replay = exact_traj || !(T < 0x1p60) || (T != 0.0 && !(T >= 0x1p-60));
            __syncwarp();
            unsigned int steps = 0;
            while (!replay) {
                if ((++steps & 255u) == 0) {
                    int late = lane == 0 && global_ns() - t_start > a.budget_ns;
                    if (__shfl_sync(0xffffffffu, late, 0)) {
                        abort_run = true;
                        break;
                    }
                }
                // ---- float-pair propensities of this lane's chunk and their sum
                bool amb = amb_next;
                amb_next = false;
                if (BATCH) {
                    ls = DF{0.f, 0.f};
                    for (int i2 = 0; i2 < n_own; ++i2) {
                        const DF acc = eval_prop(i2 * 32 + lane, amb);
                        prop[pz(i2 * 32 + lane)] = make_float2(acc.h, acc.l);
                        ls = df_add(ls, acc);
                    }
                } else if (need_full) {
                    for (int g = 0; g < NG; ++g) {
                        const int e = min(n_own, (g + 1) * GS);
                        for (int i2 = g * GS; i2 < e; ++i2) {
                            const DF acc = eval_prop(i2 * 32 + lane, amb);
                            prop[pz(i2 * 32 + lane)] = make_float2(acc.h, acc.l);
                        }
                        const DF gs = group_sum(g);
                        gsum[g * 32 + lane] = make_float2(gs.h, gs.l);
                    }
                    ls = chunk_sum();
                    dmask[lane] = 0u;
                    need_full = !deps;
                    __syncwarp();
                }
                // inclusive scan of the chunk sums
                DF incl = ls;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const DF o = shfl_up_df(incl, d);
                    if (lane >= d) incl = df_add(o, incl);
                }
                const DF tot = shfl_df(incl, 31);
                amb = __any_sync(0xffffffffu, amb) || tot.h > 0x1p90f || (tot.h > 0.0f && tot.h < 0x1p-90f);

                // ---- lane 0: Exp1 draw, clock, decision; then the uniform
                int state = 0;  // 0 record, 1 fire, 2 undecided
                DF ch{0.f, 0.f};
                uint64_t u53 = 0;  // the choice uniform's top 53 bits (lane 0)
                if (lane == 0 && !amb && tot.h > 0.0f) {
                    float xerr;
                    Xoshiro gt = g;
                    const DF x = exp1_df(gt, ex, xdf, xerr);
                    const float rr = rcp_approx(tot.h);
                    const DF q = df_div(x, tot, rr);
                    const TF tn = tf_add(tc, q);
                    float err_tn = __fadd_ru(err_t, __fmul_ru(c_q, q.h));
                    err_tn = __fadd_ru(err_tn, __fmul_ru(__fmul_ru(xerr, rr), 1.001f));
                    err_tn = __fadd_ru(err_tn, __fmul_ru(0x1p-52f, tn.h));
                    err_tn = __fadd_ru(err_tn, __fmul_ru(0x1p-23f, fabsf(tn.l)));
                    const float d = __fadd_rn(__fsub_rn(Tc.h, tn.h),
                                              __fadd_rn(__fsub_rn(Tc.m, tn.m), __fsub_rn(Tc.l, tn.l)));
                    const float mt = __fadd_ru(err_tn, __fmul_ru(0x1p-44f, fmaxf(Tc.h, tn.h)));
                    const float dd = __fmul_rn(d, 1.0f - 0x1p-22f);
                    if (!(err_tn < 1.0e30f) || q.h < 0x1p-100f) {
                        state = 2;
                    } else if (dd > mt) {
                        state = 1;
                        u53 = xo_next(gt) >> 11;
                        ch = df_mul(tot, df_u53(u53));
                        g = gt;
                        tc = tn;
                        err_t = err_tn;
                    } else if (dd < -mt) {
                        state = 0;
                        g = gt;  // the sample records; the Exp1 draw was made
                    } else {
                        state = 2;
                    }
                }
                if (amb) state = 2;
                state = __shfl_sync(0xffffffffu, state, 0);
                if (state == 2) {
                    replay = true;
                    break;
                }
                if (state == 0) break;  // record
                // ---- the choice: #{r : cum_r < total * U}
                ch = shfl_df(ch, 0);
                DF excl = shfl_up_df(incl, 1);  // this chunk's exclusive prefix
                if (lane == 0) excl = DF{0.f, 0.f};
                const float msel = c_sel * tot.h;
                const float di = __fadd_rn(__fsub_rn(incl.h, ch.h), __fsub_rn(incl.l, ch.l));
                const unsigned int below = __ballot_sync(0xffffffffu, di < 0.0f);
                bool close = fabsf(di) <= msel;
                const int k = __popc(below);  // chunks entirely below the choice
                // walk chunk k with the whole warp: lane j takes its reaction k*C + j
                int idx = R;
                if (k < 32) {
                    DF carry = shfl_df(excl, k);
                    int count = 0;
                    for (int seg = 0; seg < C; seg += 32) {
                        const int j = seg + lane;
                        const bool valid = j < C && k * C + j < R;
                        DF v{0.f, 0.f};
                        if (valid) {
                            const float2 pa = prop[pz(j * 32 + k)];
                            v = DF{pa.x, pa.y};
                        }
#pragma unroll
                        for (int d2 = 1; d2 < 32; d2 <<= 1) {
                            const DF o = shfl_up_df(v, d2);
                            if (lane >= d2) v = df_add(o, v);
                        }
                        const DF cum = df_add(carry, v);
                        const float dr = __fadd_rn(__fsub_rn(cum.h, ch.h), __fsub_rn(cum.l, ch.l));
                        count += __popc(__ballot_sync(0xffffffffu, valid && dr < 0.0f));
                        close |= valid && fabsf(dr) <= msel;
                        carry = shfl_df(cum, 31);
                    }
                    idx = k * C + count;
                }
                if (__any_sync(0xffffffffu, close) || a.exact_choice) {
                    // the clock is decided: only the choice is redone, exactly
                    // (the float-pair propensities are overwritten)
                    idx = warp_exact_choice<MACRO>(it, cnt, rates, scr, __shfl_sync(0xffffffffu, u53, 0));
                    need_full = true;
                }
                // ---- jump
                ++ev;
                if (idx < R)
                    for (int q = lane; q < Q; q += 32) {
                        const int64_t dlt = jump_d(idx * Q + q);
                        if (dlt != 0) {
                            const int sp = jump_sp(idx * Q + q);
                            cnt[sp] += dlt;
                            cntf[sp] = __fadd_rn(cntf[sp], (float)dlt);
                        }
                    }
                __syncwarp();
                // ---- re-evaluate the propensities the jump touched, re-sum
                // their groups and the chunks holding them
                if (deps && idx < R && !need_full) {
                    const int v = a.dep_tab[(size_t)idx * 32 + lane];
                    const int nd = __shfl_sync(0xffffffffu, v, 0);
                    if (nd > 31) {
                        need_full = true;
                    } else {
                        if (lane >= 1 && lane <= nd) {
                            const DF acc = eval_prop(v, amb_next);
                            prop[pz(v)] = make_float2(acc.h, acc.l);
                            atomicOr(&dmask[v & 31], 1u << ((v >> 5) / GS));
                        }
                        __syncwarp();
                        uint32_t m = dmask[lane];
                        if (m) {
                            dmask[lane] = 0u;
                            while (m) {
                                const int g = __ffs((int)m) - 1;
                                m &= m - 1u;
                                const DF gs = group_sum(g);
                                gsum[g * 32 + lane] = make_float2(gs.h, gs.l);
                            }
                            ls = chunk_sum();
                        }
                        __syncwarp();
                    }
                }
            }
            if (abort_run) break;
            if (replay) {
                // ---- exact re-run of the interval from its saved start
                if (!exact_traj && lane == 0) atomicAdd(a.work + 3, 1ull);
                for (int s = lane; s < S; s += 32) cnt[s] = cnt0[s];
                g = g0;
                t = t0;
                ev = ev0;
                __syncwarp();
                for (unsigned int n = 1;; ++n) {
                    if ((n & 255u) == 0) {
                        int late = lane == 0 && global_ns() - t_start > a.budget_ns;
                        if (__shfl_sync(0xffffffffu, late, 0)) {
                            abort_run = true;
                            break;
                        }
                    }
                    int idx = 0;
                    if (!warp_exact_step<MACRO>(it, cnt, rates, a.zig, scr, g, t, T, idx)) break;
                    ++ev;
                    if (idx < R)
                        for (int q = lane; q < Q; q += 32) {
                            const int64_t dlt = jump_d(idx * Q + q);
                            if (dlt != 0) cnt[jump_sp(idx * Q + q)] += dlt;
                        }
                    __syncwarp();
                }
                if (abort_run) break;
                for (int s = lane; s < S; s += 32) cntf[s] = (float)cnt[s];
                need_full = true;
                amb_next = false;
                __syncwarp();
            }
            // ---- record sample i at t = T
            t = T;
            int64_t *o = it.out + (size_t)i * it.n_save * it.n_traj + traj;
            for (int k = lane; k < it.n_save; k += 32) o[(size_t)k * it.n_traj] = cnt[it.save_idx[k]];
            __syncwarp();
        }
        if (abort_run) {
            if (lane == 0) atomicExch(a.work + 2, 1ull);
            break;
        }
        if (it.fin_species)
            for (int s = lane; s < S; s += 32) it.fin_species[traj * S + s] = cnt[s];
        if (lane == 0) {
            if (it.fin_t) it.fin_t[traj] = t;
            if (it.fin_rng) {
                it.fin_rng[traj * 4 + 0] = g.s0;
                it.fin_rng[traj * 4 + 1] = g.s1;
                it.fin_rng[traj * 4 + 2] = g.s2;
                it.fin_rng[traj * 4 + 3] = g.s3;
            }
            if (it.events) it.events[traj] = ev;
        }
        warp_events += ev;
        __syncwarp();
    }
    if (lane == 0 && warp_events) atomicAdd(a.work + 1, warp_events);
}

template <bool MACRO, bool BATCH>
int warp_launch(const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st) {
    auto kern = ssa_warp_kernel<MACRO, BATCH>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    kern<<<grid, block, smem, st>>>(a);
    return (int)cudaGetLastError();
}

}  // namespace

int ssa_warp_warps(const SsaArgs &a, size_t smem_limit) {
    const WarpLayout l = warp_layout(a);
    if (l.block_bytes + l.warp_bytes > smem_limit) return 0;
    return (int)std::min<size_t>(a.batch ? kWarpMaxWarpsBatch : kWarpMaxWarps, (smem_limit - l.block_bytes) / l.warp_bytes);
}

size_t ssa_warp_smem(const SsaArgs &a, int warps) {
    const WarpLayout l = warp_layout(a);
    return l.block_bytes + (size_t)warps * l.warp_bytes;
}

bool ssa_warp_supported(const SsaArgs &a, int max_order) {
    return a.ex_off == nullptr && a.S < 65536 && max_order < 32768 && a.R >= 1;
}

int ssa_warp_occupancy(const SsaArgs &a, int warps, size_t smem) {
    int n = 0;
    // the arithmetic variants share the block shape and shared memory use;
    // batch launches have their own register budget
    const auto k = a.batch ? ssa_warp_kernel<false, true> : ssa_warp_kernel<false, false>;
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, 32 * warps, smem);
    return n;
}

int launch_ssa_warp(const SsaArgs &a, int warps, int grid, size_t smem, void *stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const bool batch = a.batch != nullptr;
    if (a.macro_mode)
        return batch ? warp_launch<true, true>(a, 32 * warps, grid, smem, st)
                     : warp_launch<true, false>(a, 32 * warps, grid, smem, st);
    return batch ? warp_launch<false, true>(a, 32 * warps, grid, smem, st)
                 : warp_launch<false, false>(a, 32 * warps, grid, smem, st);
}

uint32_t warp_shape_word(const int32_t *fac_sp, const int32_t *fac_ord, int P, int S, int r) {
    return shape_word(fac_sp, fac_ord, P, S, r);
}

}  // namespace rbg
