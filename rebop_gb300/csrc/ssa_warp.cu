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
// the reference's decision.  Anything else -- a close choice or clock
// comparison, a count outside [0, 2^23), a rate outside 2^-60 .. 2^60 --
// re-runs the sample interval from its saved start with the exact step below:
// lanes compute the binary64 propensities in the reference's multiply order,
// lane 0 folds them in order and draws in native binary64, so counts, event
// numbers and the random stream equal rebop's bit for bit.
#include <cuda_runtime.h>

#include <algorithm>

#include "ssa_spec_body.cuh"

namespace rbg {

namespace {

constexpr int kWarpMaxWarps = 16;

struct WarpLayout {
    size_t block_bytes, warp_bytes;
};

// Lane l owns the C = ceil(R / 32) reactions l*C .. l*C + C - 1.  Arrays the
// lanes walk together are stored lane-major -- reaction l*C + i at position
// i*32 + l -- so one step of the walk touches 32 consecutive words.
__host__ __device__ inline int warp_chunk(int R) { return (R + 31) / 32; }

// Shared memory: block tables (Exp1 tables, float-pair rates when shared,
// reactant factors in both layouts, jumps), then per warp: counts, counts at
// the interval start, float-pair propensities (and float-pair rates when per
// trajectory).
__host__ __device__ inline WarpLayout warp_layout(const SsaArgs &a) {
    WarpLayout l;
    const size_t RP = 32 * (size_t)warp_chunk(a.R);     // lane-major positions
    size_t b = 16 * 256 + 8 * 257 + 8 * 256 + 8 * 256;  // zxk, zf, zd, xdf
    b += 8 * RP;                                        // shared float-pair rates (lane-major)
    b += 4 * (size_t)a.R * a.P + 4 * RP * a.P;          // factors: reaction-major, lane-major
    b += 4 * RP;                                        // two-slot reaction shapes (lane-major)
    b += 4 * (size_t)a.R * a.Q + 8 * (size_t)a.R * a.Q; // jumps (exact tables' layout)
    b += 16;                                            // alignment of the jump deltas
    l.block_bytes = (b + 15) & ~(size_t)15;
    size_t w = 16 * (size_t)a.S;                        // counts, interval-start counts
    w += 4 * ((size_t)a.S + 1);                         // counts as floats, plus the constant 1
    w += 8 * RP + 8;                                    // propensities (lane-major), alignment
    if (a.rate_stride) w += 8 * RP;                     // per-trajectory float-pair rates
    l.warp_bytes = (w + 15) & ~(size_t)15;
    return l;
}

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
__device__ __forceinline__ double exact_propensity(const SsaArgs &a, const int32_t *fac, const int64_t *cnt,
                                                   double rate, int r) {
    double acc = rate;
    for (int p = 0; p < a.P; ++p) {
        const int f = fac[r * a.P + p];
        const int o = f >> 16;
        if (o == 0) continue;
        const int64_t n = cnt[f & 0xFFFF];
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

// One exact step of the whole warp from the committed state (lane 0 holds the
// generator).  Returns 1 when a reaction fires (its index in idx, the clock in
// t), 0 when the step records the sample.  scr is this warp's [R] scratch.
template <bool MACRO>
__device__ __noinline__ int warp_exact_step(const SsaArgs &a, const int32_t *fac, int64_t *cnt, const double *rates,
                                            double *scr, Xoshiro &g, double &t, double T, int &idx) {
    const int lane = threadIdx.x & 31, R = a.R;
    for (int r = lane; r < R; r += 32) scr[r] = exact_propensity<MACRO>(a, fac, cnt, rates[r], r);
    __syncwarp();
    int fire = 0;
    double chosen = 0.0;
    int midx = R;
    if (lane == 0) {
        double total = 0.0;
        for (int r = 0; r < R; ++r) {
            total = __dadd_rn(total, scr[r]);
            scr[r] = total;
        }
        if (0.0 < total) {
            const double tn = __dadd_rn(t, __ddiv_rn(xo_exp1(g, a.zig, a.zig + kZigOffF), total));
            if (!(tn > T)) {
                fire = 1;
                t = tn;
                chosen = __dmul_rn(total, xo_uniform(g));
                if (MACRO)  // first r with chosen < cum_r (gillespie_macro.rs:150-171)
                    for (int r = 0; r < R; ++r)
                        if (chosen < scr[r]) {
                            midx = r;
                            break;
                        }
            }
        }
    }
    __syncwarp();
    fire = __shfl_sync(0xffffffffu, fire, 0);
    t = shfl_d(t, 0);
    if (!fire) return 0;
    if (MACRO) {
        idx = __shfl_sync(0xffffffffu, midx, 0);
    } else {
        // #{r : cum_r < chosen} (gillespie.rs:402-407), counted by all lanes
        chosen = shfl_d(chosen, 0);
        int c = 0;
        for (int r = lane; r < R; r += 32) c += scr[r] < chosen ? 1 : 0;
        for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
        idx = c;
    }
    return 1;
}

// SHAPE2: every reaction has reactant order <= 2, so its propensity is
// rate * max(n1 - o1, 0) * max(n2 - o2, 0) over two (species, offset) slots
// -- species S is a constant 1 -- and the propensity pass has no branches.
template <bool MACRO, bool SHAPE2>
__global__ void __launch_bounds__(32 * kWarpMaxWarps) ssa_warp_kernel(const __grid_constant__ SsaArgs a) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const int S = a.S, R = a.R, P = a.P, Q = a.Q;
    const WarpLayout L = warp_layout(a);

    // ---- block tables
    ulonglong2 *zxk = reinterpret_cast<ulonglong2 *>(g_spec_smem);
    uint64_t *zf = reinterpret_cast<uint64_t *>(zxk + 256);
    uint64_t *zd = zf + 257;
    float2 *xdf = reinterpret_cast<float2 *>(zd + 256);
    const int C = warp_chunk(R), RP = 32 * C;
    float2 *rdf_sh = xdf + 256;
    int32_t *facl = reinterpret_cast<int32_t *>(rdf_sh + RP);  // [C][P][32] lane-major factors
    uint32_t *shape = reinterpret_cast<uint32_t *>(facl + (size_t)RP * P);  // [RP] lane-major
    int32_t *fac = reinterpret_cast<int32_t *>(shape + RP);
    int32_t *jsp = fac + (size_t)R * P;
    int64_t *jd = reinterpret_cast<int64_t *>(
        (reinterpret_cast<uintptr_t>(jsp + (size_t)R * Q) + 7) & ~(uintptr_t)7);
    load_exact_tables(a, zxk, zf, zd, fac, jsp, jd);
    for (int k = tid; k < 256; k += blockDim.x) {
        const double v = a.zig[kZigOffXdf + k];
        xdf[k] = *reinterpret_cast<const float2 *>(&v);
    }
    // lane-major copies: reaction r = l*C + i at position i*32 + l (padding
    // positions hold rate 0 and no factors)
    for (int q = tid; q < RP; q += blockDim.x) {
        const int i = q >> 5, l = q & 31, r = l * C + i;
        if (!a.rate_stride) {
            const DF d = r < R ? df_from_double(a.rate[r]) : DF{0.f, 0.f};
            rdf_sh[q] = make_float2(d.h, d.l);
        }
        for (int p = 0; p < P; ++p)
            facl[(i * P + p) * 32 + l] = r < R ? (a.fac_sp[r * P + p] | (a.fac_ord[r * P + p] << 16)) : 0;
        if (SHAPE2) {
            // slots (species, offset): 2A -> (A,0)(A,1); A+B -> (A,0)(B,0); A -> (A,0)(1); none -> (1)(1)
            uint32_t sl[2] = {(uint32_t)S, (uint32_t)S}, of[2] = {0, 0};
            int k = 0;
            for (int p = 0; r < R && p < P; ++p) {
                const int o = a.fac_ord[r * P + p];
                for (int j = 0; j < o && k < 2; ++j, ++k) {
                    sl[k] = (uint32_t)a.fac_sp[r * P + p];
                    of[k] = (uint32_t)j;
                }
            }
            shape[q] = sl[0] | of[0] << 15 | sl[1] << 16 | of[1] << 31;
        }
    }
    __syncthreads();
    const ExactTables ex{zxk, zf, zd, fac, jsp, jd};

    // ---- this warp's region
    unsigned char *wbase = g_spec_smem + L.block_bytes + (size_t)warp * L.warp_bytes;
    int64_t *cnt = reinterpret_cast<int64_t *>(wbase);
    int64_t *cnt0 = cnt + S;
    float *cntf = reinterpret_cast<float *>(cnt0 + S);                                  // [S + 1]
    float2 *prop = reinterpret_cast<float2 *>((reinterpret_cast<uintptr_t>(cntf + S + 1) + 7) & ~(uintptr_t)7);
    float2 *rdf = a.rate_stride ? prop + RP : rdf_sh;      // lane-major
    double *scr = a.warp_scratch + ((size_t)blockIdx.x * nw + warp) * (size_t)R;

    // lane l owns reactions [l * C, min(R, (l + 1) * C)); local index i sits at i*32 + l
    const int r_lo = min(R, lane * C), r_hi = min(R, r_lo + C);
    const int n_own = r_hi - r_lo;
    const float gam = kGamma;
    const int mm = SHAPE2 ? 2 : a.max_mults;  // multiplies per propensity
    const float c_tot = (float)(mm + 1 + C + 5) * gam + (float)(R + mm + 4) * 0x1p-53f;
    const float c_q = c_tot + 6.0f * gam;
    const float c_sel = 2.0f * (c_tot + (float)(C + 4) * gam);
    const int64_t t_start = global_ns();
    unsigned long long warp_events = 0;
    bool abort_run = false;

    for (;;) {
        long long traj = 0;
        if (lane == 0) traj = (long long)atomicAdd(a.work, 1ull);
        traj = __shfl_sync(0xffffffffu, traj, 0);
        if (traj >= a.n_traj) break;

        // ---- start (or resume) the trajectory
        Xoshiro g{0, 0, 0, 0};
        double t;
        if (a.in_species) {
            for (int s = lane; s < S; s += 32) cnt[s] = a.in_species[traj * S + s];
            t = a.in_t[traj];
            if (lane == 0)
                g = Xoshiro{a.in_rng[traj * 4], a.in_rng[traj * 4 + 1], a.in_rng[traj * 4 + 2],
                            a.in_rng[traj * 4 + 3]};
        } else {
            for (int s = lane; s < S; s += 32) cnt[s] = a.x0[traj * a.x0_stride + s];
            t = 0.0;
            if (lane == 0) xo_seed(g, a.seeds[traj]);
        }
        const double *rates = a.rate + traj * a.rate_stride;
        bool exact_traj = !spec_rate_ok((uint64_t)__double_as_longlong(t)) || !(t < 0x1p60);
        for (int r = lane; r < R; r += 32) exact_traj |= !spec_rate_ok((uint64_t)__double_as_longlong(rates[r]));
        if (a.rate_stride)
            for (int q = lane; q < RP; q += 32) {
                const int r = (q & 31) * C + (q >> 5);
                const DF d = r < R ? df_from_double(rates[r]) : DF{0.f, 0.f};
                rdf[q] = make_float2(d.h, d.l);
            }
        exact_traj = __any_sync(0xffffffffu, exact_traj);
        for (int s = lane; s <= S; s += 32) cntf[s] = s < S ? (float)cnt[s] : 1.0f;
        __syncwarp();
        unsigned long long ev = 0;

        for (long long i = 0; i < a.n_samples && !abort_run; ++i) {
            const double T = a.sample_t[i];
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
                DF ls{0.f, 0.f};
                bool amb = false;
                if (SHAPE2) {
                    for (int i = 0; i < n_own; ++i) {
                        const float2 k = rdf[i * 32 + lane];
                        const uint32_t w = shape[i * 32 + lane];
                        const float n1 = cntf[w & 0x7FFFu], n2 = cntf[(w >> 16) & 0x7FFFu];
                        amb |= !(n1 >= 0.0f && n1 < 8388608.0f && n2 >= 0.0f && n2 < 8388608.0f);
                        const float f1 = fmaxf(__fsub_rn(n1, (float)((w >> 15) & 1u)), 0.0f);
                        const float f2 = fmaxf(__fsub_rn(n2, (float)(w >> 31)), 0.0f);
                        const DF acc = df_mul_fu(df_mul_fu(DF{k.x, k.y}, f1), f2);
                        prop[i * 32 + lane] = make_float2(acc.h, acc.l);
                        ls = df_add(ls, acc);
                    }
                } else
                for (int i = 0; i < n_own; ++i) {
                    const float2 k = rdf[i * 32 + lane];
                    DF acc{k.x, k.y};
                    for (int p = 0; p < P; ++p) {
                        const int f = facl[(i * P + p) * 32 + lane];
                        const int o = f >> 16;
                        if (o == 0) continue;
                        const int64_t n = cnt[f & 0xFFFF];
                        amb |= (uint64_t)n >= (1ull << 23);
                        for (int j = 0; j < o; ++j) {
                            const int64_t x = n - j > 0 ? n - j : 0;
                            acc = df_mul_fu(acc, f23((uint32_t)x & 0x7FFFFFu));
                        }
                    }
                    prop[i * 32 + lane] = make_float2(acc.h, acc.l);
                    ls = df_add(ls, acc);
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
                        ch = df_mul(tot, df_u53(xo_next(gt) >> 11));
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
                            const float2 pa = prop[j * 32 + k];
                            v = DF{pa.x, pa.y};
                        }
#pragma unroll
                        for (int dd2 = 1; dd2 < 32; dd2 <<= 1) {
                            const DF o = shfl_up_df(v, dd2);
                            if (lane >= dd2) v = df_add(o, v);
                        }
                        const DF cum = df_add(carry, v);
                        const float dr = __fadd_rn(__fsub_rn(cum.h, ch.h), __fsub_rn(cum.l, ch.l));
                        count += __popc(__ballot_sync(0xffffffffu, valid && dr < 0.0f));
                        close |= valid && fabsf(dr) <= msel;
                        carry = shfl_df(cum, 31);
                    }
                    idx = k * C + count;
                }
                if (__any_sync(0xffffffffu, close)) {
                    replay = true;
                    break;
                }
                // ---- jump
                ++ev;
                if (idx < R)
                    for (int q = lane; q < Q; q += 32) {
                        const int64_t dlt = jd[idx * Q + q];
                        if (dlt != 0) {
                            const int sp = jsp[idx * Q + q];
                            cnt[sp] += dlt;
                            cntf[sp] = __fadd_rn(cntf[sp], (float)dlt);
                        }
                    }
                __syncwarp();
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
                    if (!warp_exact_step<MACRO>(a, fac, cnt, rates, scr, g, t, T, idx)) break;
                    ++ev;
                    if (idx < R)
                        for (int q = lane; q < Q; q += 32) {
                            const int64_t dlt = jd[idx * Q + q];
                            if (dlt != 0) cnt[jsp[idx * Q + q]] += dlt;
                        }
                    __syncwarp();
                }
                if (abort_run) break;
                for (int s = lane; s < S; s += 32) cntf[s] = (float)cnt[s];
                __syncwarp();
            }
            // ---- record sample i at t = T
            t = T;
            int64_t *o = a.out + (size_t)i * a.n_save * a.n_traj + traj;
            for (int k = lane; k < a.n_save; k += 32) o[(size_t)k * a.n_traj] = cnt[a.save_idx[k]];
            __syncwarp();
        }
        if (abort_run) {
            if (lane == 0) atomicExch(a.work + 2, 1ull);
            break;
        }
        if (a.fin_species)
            for (int s = lane; s < S; s += 32) a.fin_species[traj * S + s] = cnt[s];
        if (lane == 0) {
            if (a.fin_t) a.fin_t[traj] = t;
            if (a.fin_rng) {
                a.fin_rng[traj * 4 + 0] = g.s0;
                a.fin_rng[traj * 4 + 1] = g.s1;
                a.fin_rng[traj * 4 + 2] = g.s2;
                a.fin_rng[traj * 4 + 3] = g.s3;
            }
            if (a.events) a.events[traj] = ev;
        }
        warp_events += ev;
        __syncwarp();
    }
    if (lane == 0 && warp_events) atomicAdd(a.work + 1, warp_events);
}

template <bool MACRO, bool SHAPE2>
int warp_launch(const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st) {
    auto kern = ssa_warp_kernel<MACRO, SHAPE2>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    kern<<<grid, block, smem, st>>>(a);
    return (int)cudaGetLastError();
}

}  // namespace

int ssa_warp_warps(const SsaArgs &a, size_t smem_limit) {
    const WarpLayout l = warp_layout(a);
    if (l.block_bytes + l.warp_bytes > smem_limit) return 0;
    return (int)std::min<size_t>(kWarpMaxWarps, (smem_limit - l.block_bytes) / l.warp_bytes);
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
    // all instances share the block shape and shared memory use
    cudaFuncSetAttribute(ssa_warp_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssa_warp_kernel<false, true>, 32 * warps, smem);
    return n;
}

int launch_ssa_warp(const SsaArgs &a, int warps, int grid, size_t smem, void *stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // two-slot shapes need reactant order <= 2 and species indices below 2^15
    const bool shape2 = a.max_mults <= 2 && a.S < 32767;
    if (a.macro_mode)
        return shape2 ? warp_launch<true, true>(a, 32 * warps, grid, smem, st)
                      : warp_launch<true, false>(a, 32 * warps, grid, smem, st);
    return shape2 ? warp_launch<false, true>(a, 32 * warps, grid, smem, st)
                  : warp_launch<false, false>(a, 32 * warps, grid, smem, st);
}

}  // namespace rbg
