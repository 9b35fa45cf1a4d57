// Lockstep thread-per-trajectory SSA kernel with binary64 on the integer pipes.
//
// Same contract and results as ssa_thread_kernel (one thread per trajectory,
// ticket refill, rebop's direct method and sampling loop), built for GB300:
//
// * Binary64 work runs in exact integer emulation (b64.cuh): the propensity
//   products, their running sum, the Exp1 abscissa, Exp1 / total, the clock
//   update and total * U, with results identical to the FPU's.  Comparisons
//   of non-negative doubles are integer comparisons of their bit patterns.
//   GB300's FP64 pipe (about 1.9 results per clock per SM) would otherwise
//   bound the loop; the integer pipes are some 40x wider.
// * Every lane executes the same instruction stream for each step: it always
//   computes the propensities, the Exp1 draw, the candidate clock and the
//   choice, then either fires the reaction or records a sample.  Random draws
//   are made on copies of the generator state and committed only in the
//   order the reference consumes them (no draw when the total propensity
//   vanishes; the uniform only when the reaction fires).
// * The ziggurat's fast test x < x[i+1] is an integer comparison of the
//   52-bit fraction against a per-layer threshold; its wedge test compares in
//   float32 with a proven margin and falls back to binary64 only inside it.
// * Steps the emulation does not cover (negative or non-finite rates,
//   negative counts, results outside the normal range) are detected per lane
//   and redone with native binary64 instructions from the committed state.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "b64.cuh"
#include "rng.cuh"
#include "ssa_args.hpp"

namespace rbg {

extern __shared__ __align__(16) unsigned char g_fast_smem[];

namespace {

constexpr uint64_t kOneBits = 0x3FF0000000000000ull;
constexpr uint64_t kLimit53 = 1ull << 53;

struct FastSmem {
    ulonglong2 *zxk;  // [256] {x bits, K}
    uint64_t *zf;     // [257] f bits
    uint64_t *zd;     // [256] |f[i] - f[i+1]| bits
    int64_t *jd;      // [R*Q]
    uint64_t *rate;   // [R][block] per-lane rate bits
    int64_t *sp;      // [S][block] per-lane counts
    int32_t *fac;     // [R*P] species | order << 16
    int32_t *jsp;     // [R*Q]
};

__host__ __device__ inline size_t fast_smem_bytes(int S, int R, int P, int Q, int block) {
    size_t b = 16 * 256 + 8 * 257 + 8 * 256;
    b += 8 * (size_t)R * Q;
    b += 8 * (size_t)R * block;
    b += 8 * (size_t)S * block;
    b += 4 * ((size_t)R * P + (size_t)R * Q);
    return (b + 15) & ~(size_t)15;
}

__device__ inline FastSmem fast_layout(int S, int R, int P, int Q, int block) {
    FastSmem m;
    m.zxk = reinterpret_cast<ulonglong2 *>(g_fast_smem);
    m.zf = reinterpret_cast<uint64_t *>(m.zxk + 256);
    m.zd = m.zf + 257;
    m.jd = reinterpret_cast<int64_t *>(m.zd + 256);
    m.rate = reinterpret_cast<uint64_t *>(m.jd + (size_t)R * Q);
    m.sp = reinterpret_cast<int64_t *>(m.rate + (size_t)R * block);
    m.fac = reinterpret_cast<int32_t *>(m.sp + (size_t)S * block);
    m.jsp = m.fac + (size_t)R * P;
    return m;
}

// Truncated float32 of a positive normal double (bits), for the wedge pre-test.
__device__ __forceinline__ float f32_rz(uint64_t v) {
    const uint32_t e = (uint32_t)(v >> 52) - 1023u + 127u;
    return __uint_as_float((e << 23) | ((uint32_t)(v >> 29) & 0x7FFFFFu));
}

// A double is in the emulation's domain when it is +0 or positive normal.
__device__ __forceinline__ bool emul_domain(uint64_t v) {
    const uint64_t e = v >> 52;
    return v == 0 || (e >= 1 && e <= 2046);
}

// Exp1 draw (ziggurat) on the integer pipes; see rng.cuh for the algorithm.
__device__ __forceinline__ uint64_t exp1_emul(Xoshiro &g, const FastSmem &m, bool &bad) {
    for (;;) {
        const uint64_t b = xo_next(g);
        const int i = (int)(b & 0xff);
        const uint64_t k = b >> 12;
        const ulonglong2 e = m.zxk[i];
        const uint64_t x = b64::mul_u64(e.x, 2 * k + 1, 53, bad);
        if (k < e.y) return x;
        if (i == 0) {  // tail: R - ln U in binary64
            const double u = xo_uniform(g);
            return (uint64_t)__double_as_longlong(__dsub_rn(kZigR, log(u)));
        }
        // wedge: f[i+1] + (f[i] - f[i+1]) U < exp(-x), with f[i] < f[i+1]
        const uint64_t mu = xo_next(g) >> 11;
        const uint64_t w = b64::sub(m.zf[i + 1], b64::mul_u64(m.zd[i], mu, 53, bad), bad);
        const float wf = f32_rz(w), ef = expf(-f32_rz(x));
        // |wf - w| and |ef - exp(-x)| are below 1.5e-6 relative; the margin is 7.6e-6.
        bool accept;
        if (wf < ef * (1.0f - 0x1p-17f)) accept = true;
        else if (wf > ef * (1.0f + 0x1p-17f)) accept = false;
        else accept = __longlong_as_double((long long)w) < exp(-__longlong_as_double((long long)x));
        if (accept) return x;
    }
}

// One step of rebop's advance_until in native binary64 from the committed
// state (the emulation's fallback).  Returns true when a reaction fires, with
// its index and the new clock; commits the draws it consumes.
template <int MAXR, bool MACRO>
__device__ __noinline__ bool native_step(const SsaArgs &a, Xoshiro &g, const int64_t *sp, const uint64_t *rl,
                                         int BD, uint64_t t_bits, uint64_t T_bits, int &idx, uint64_t &tn_bits,
                                         const FastSmem &m) {
    double cum[MAXR];
    double total = 0.0;
#pragma unroll
    for (int r = 0; r < MAXR; ++r) {
        if (r < a.R) {
            double acc = __longlong_as_double((long long)rl[r * BD]);
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

}  // namespace

// Exact binary64 a + b of the hot loop: on the FP64 pipe (ADD_NATIVE), or on
// the integer pipes.  Either way the bits are the FPU's.
template <bool ADD_NATIVE>
__device__ __forceinline__ uint64_t hot_add(uint64_t a, uint64_t b, bool &bad) {
    if (ADD_NATIVE) return (uint64_t)__double_as_longlong(__dadd_rn(__longlong_as_double((long long)a),
                                                                     __longlong_as_double((long long)b)));
    return b64::add_bf(a, b, bad);
}

template <int MAXR, bool MACRO, bool ADD_NATIVE>
__global__ void __launch_bounds__(128, 6) ssa_fast_kernel(const __grid_constant__ SsaArgs a) {
    const int BD = blockDim.x, tid = threadIdx.x;
    const int S = a.S, R = a.R, P = a.P, Q = a.Q;
    const FastSmem m = fast_layout(S, R, P, Q, BD);

    for (int k = tid; k < 256; k += BD) {
        m.zxk[k] = make_ulonglong2((uint64_t)__double_as_longlong(a.zig[k]),
                                   (uint64_t)__double_as_longlong(a.zig[kZigOffK + k]));
        m.zd[k] = (uint64_t)__double_as_longlong(a.zig[kZigOffD + k]) & ~(1ull << 63);
    }
    for (int k = tid; k < 257; k += BD) m.zf[k] = (uint64_t)__double_as_longlong(a.zig[kZigOffF + k]);
    for (int k = tid; k < R * P; k += BD) m.fac[k] = a.fac_sp[k] | (a.fac_ord[k] << 16);
    for (int k = tid; k < R * Q; k += BD) {
        m.jsp[k] = a.jmp_sp[k];
        m.jd[k] = a.jmp_d[k];
    }
    __syncthreads();

    int64_t *const sp = m.sp + tid;     // count of species s: sp[s * BD]
    uint64_t *const rl = m.rate + tid;  // rate bits of reaction r: rl[r * BD]
    const int64_t t_start = global_ns();
    unsigned int tick = 0;
    unsigned long long lane_events = 0;

    Xoshiro g{0, 0, 0, 0};
    uint64_t t = 0, T = 0;
    long long i = 0, traj = -1;
    unsigned long long ev = 0;
    bool nat = false;

    for (;;) {
        if (traj < 0) {
            // ---- take the next trajectory (fresh, or resumed from a state)
            traj = (long long)atomicAdd(a.work, 1ull);
            if (traj >= a.n_traj) break;
            if (a.in_species) {
                for (int s = 0; s < S; ++s) sp[s * BD] = a.in_species[traj * S + s];
                t = (uint64_t)__double_as_longlong(a.in_t[traj]);
                g.s0 = a.in_rng[traj * 4 + 0];
                g.s1 = a.in_rng[traj * 4 + 1];
                g.s2 = a.in_rng[traj * 4 + 2];
                g.s3 = a.in_rng[traj * 4 + 3];
            } else {
                for (int s = 0; s < S; ++s) sp[s * BD] = a.x0[traj * a.x0_stride + s];
                t = 0;
                xo_seed(g, a.seeds[traj]);
            }
            nat = !emul_domain(t);
            for (int r = 0; r < R; ++r) {
                const uint64_t rb = (uint64_t)__double_as_longlong(a.rate[traj * a.rate_stride + r]);
                rl[r * BD] = rb;
                nat |= !emul_domain(rb);
            }
            i = 0;
            ev = 0;
            T = (uint64_t)__double_as_longlong(a.sample_t[0]);
        }
        if ((++tick & 1023u) == 0 && global_ns() - t_start > a.budget_ns) {
            lane_events += ev;
            atomicExch(a.work + 2, 1ull);
            break;
        }
        // ---- propensities and their running sum
        uint64_t cum[MAXR];
        uint64_t tot = 0;
        bool bad = nat;
#pragma unroll
        for (int r = 0; r < MAXR; ++r) {
            if (r < R) {
                uint64_t acc = rl[r * BD];
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
                tot = hot_add<ADD_NATIVE>(tot, acc, bad);
                cum[r] = tot;
            }
        }
        bad |= !emul_domain(tot);
        // ---- Exp1 draw, candidate clock, choice (on copies of the generator)
        const bool pos = tot != 0;
        Xoshiro g2 = g;
        bool bad_t = false, bad_c = false;
        const uint64_t x = exp1_emul(g2, m, bad_t);
        const uint64_t q = b64::div_bf(x, pos ? tot : kOneBits, bad_t);
        uint64_t tn = hot_add<ADD_NATIVE>(t, q, bad_t);
        bad_t |= !emul_domain(tn);
        bool fire = pos && tn <= T;
        Xoshiro g3 = g2;
        const uint64_t chosen = b64::mul_u64(tot, xo_next(g3) >> 11, 53, bad_c);
        int idx;
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
        if (bad) {
            fire = native_step<MAXR, MACRO>(a, g, sp, rl, BD, t, T, idx, tn, m);
        } else {
            g = fire ? g3 : (pos ? g2 : g);
        }
        // ---- fire the reaction, or record the sample and move to the next
        if (fire) {
            t = tn;
            ++ev;
            if (idx < R)
                for (int k = 0; k < Q; ++k) sp[m.jsp[idx * Q + k] * BD] += m.jd[idx * Q + k];
        } else {
            t = T;
            int64_t *o = a.out + (size_t)i * a.n_save * a.n_traj + traj;
            for (int k = 0; k < a.n_save; ++k) o[(size_t)k * a.n_traj] = sp[a.save_idx[k] * BD];
            if (++i < a.n_samples) {
                T = (uint64_t)__double_as_longlong(a.sample_t[i]);
            } else {
                if (a.fin_species)
                    for (int s = 0; s < S; ++s) a.fin_species[traj * S + s] = sp[s * BD];
                if (a.fin_t) a.fin_t[traj] = __longlong_as_double((long long)t);
                if (a.fin_rng) {
                    a.fin_rng[traj * 4 + 0] = g.s0;
                    a.fin_rng[traj * 4 + 1] = g.s1;
                    a.fin_rng[traj * 4 + 2] = g.s2;
                    a.fin_rng[traj * 4 + 3] = g.s3;
                }
                if (a.events) a.events[traj] = ev;
                lane_events += ev;
                traj = -1;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) lane_events += __shfl_down_sync(0xffffffffu, lane_events, off);
    if ((tid & 31) == 0 && lane_events) atomicAdd(a.work + 1, lane_events);
}

// ------------------------------------------------------------------ host side

namespace {

// Placement of the hot loop's binary64 adds: the FP64 pipe (default) or the
// integer pipes (RB_FAST_ADD=int); both give the same bits.
bool add_native() {
    const char *v = std::getenv("RB_FAST_ADD");
    return !(v && std::strcmp(v, "int") == 0);
}

template <int MAXR, bool MACRO, bool ADDN>
int fast_launch_v(const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st) {
    auto kern = ssa_fast_kernel<MAXR, MACRO, ADDN>;
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    kern<<<grid, block, smem, st>>>(a);
    return (int)cudaGetLastError();
}

template <int MAXR, bool MACRO>
int fast_launch(const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st) {
    return add_native() ? fast_launch_v<MAXR, MACRO, true>(a, block, grid, smem, st)
                        : fast_launch_v<MAXR, MACRO, false>(a, block, grid, smem, st);
}

template <int MAXR, bool MACRO>
int fast_occupancy(int block, size_t smem) {
    int n = 0;
    auto kern = add_native() ? ssa_fast_kernel<MAXR, MACRO, true> : ssa_fast_kernel<MAXR, MACRO, false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, block, smem);
    return n;
}

template <bool MACRO>
int fast_dispatch(const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st, bool occupancy_only,
                  int *occ) {
    if (a.R <= 8) {
        if (occupancy_only) return *occ = fast_occupancy<8, MACRO>(block, smem), 0;
        return fast_launch<8, MACRO>(a, block, grid, smem, st);
    }
    if (a.R <= 16) {
        if (occupancy_only) return *occ = fast_occupancy<16, MACRO>(block, smem), 0;
        return fast_launch<16, MACRO>(a, block, grid, smem, st);
    }
    if (occupancy_only) return *occ = fast_occupancy<32, MACRO>(block, smem), 0;
    return fast_launch<32, MACRO>(a, block, grid, smem, st);
}

}  // namespace

bool ssa_fast_supported(const SsaArgs &a, int max_order) {
    return a.R <= 32 && a.S < 65536 && max_order < 32768;
}

size_t ssa_fast_smem(const SsaArgs &a, int block) { return fast_smem_bytes(a.S, a.R, a.P, a.Q, block); }

int ssa_fast_occupancy(const SsaArgs &a, int block, size_t smem) {
    int occ = 0;
    if (a.macro_mode) fast_dispatch<true>(a, block, 0, smem, nullptr, true, &occ);
    else fast_dispatch<false>(a, block, 0, smem, nullptr, true, &occ);
    return occ;
}

int launch_ssa_fast(const SsaArgs &a, int block, int grid, size_t smem, void *stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return a.macro_mode ? fast_dispatch<true>(a, block, grid, smem, st, false, nullptr)
                        : fast_dispatch<false>(a, block, grid, smem, st, false, nullptr);
}

}  // namespace rbg
