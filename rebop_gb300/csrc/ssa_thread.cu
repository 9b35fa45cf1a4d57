// Thread-per-trajectory SSA kernel for small networks.
//
// One thread runs one trajectory of rebop's direct method at a time
// (src/gillespie.rs:315-344 driven by the sampling loop of
// src/pyo3_gillespie.rs:200-208) and pulls the next trajectory from a global
// ticket counter when it is done, so lanes of a warp never wait for a
// sibling's longer trajectory.  The per-lane loop is flattened: each pass
// either fires one reaction or records one sample, and propensities are
// recomputed only after a reaction (the reference recomputes identical
// values at the start of each advance_until call).
//
// Shared memory holds the ziggurat tables, the network descriptor and the
// per-lane state: species counts [S][blockDim] (int64) and cumulative
// propensities [R][blockDim] (f64).  The descriptor index of every access is
// warp-uniform except the chosen reaction's jump, and with blockDim a multiple
// of 32 the state columns make every access bank-conflict free.
//
// Arithmetic is the reference's, operation for operation, in binary64 with
// explicit round-to-nearest intrinsics (no FMA contraction):
//   propensity  rate * x_1 * x_2 ... (gillespie.rs:73-86), or the macro's
//               rate * ff_1 * ff_2 ... (gillespie_macro.rs:106, :133-146)
//   cumulative  cum_r = total + a_r; total = cum_r (gillespie.rs:357-364)
//   absorb      !(0 < total) -> clock to the sample time (gillespie.rs:323-326)
//   clock       t + Exp1 / total, overshoot past the sample time discards the
//               draw (gillespie.rs:327-331)
//   choice      #{r : cum_r < total * U} (gillespie.rs:402-407), or the
//               macro's first r with total * U < cum_r (gillespie_macro.rs:159)
#include <cuda_runtime.h>

#include "rng.cuh"
#include "ssa_args.hpp"

namespace rbg {

extern __shared__ __align__(16) unsigned char g_smem[];

struct ThreadSmem {
    double *zx, *zf, *rate;
    int64_t *jd, *sp;
    double *cum;
    int32_t *fsp, *ford, *jsp;
};

__host__ __device__ inline size_t thread_smem_bytes(int S, int R, int P, int Q, int block) {
    size_t b = sizeof(double) * 2 * kZigTable;
    b += sizeof(double) * (size_t)R;
    b += sizeof(int64_t) * (size_t)R * Q;
    b += sizeof(int64_t) * (size_t)S * block;
    b += sizeof(double) * (size_t)R * block;
    b += sizeof(int32_t) * ((size_t)2 * R * P + (size_t)R * Q);
    return (b + 15) & ~(size_t)15;
}

__device__ inline ThreadSmem thread_smem_layout(int S, int R, int P, int Q, int block) {
    ThreadSmem m;
    m.zx = reinterpret_cast<double *>(g_smem);
    m.zf = m.zx + kZigTable;
    m.rate = m.zf + kZigTable;
    m.jd = reinterpret_cast<int64_t *>(m.rate + R);
    m.sp = m.jd + (size_t)R * Q;
    m.cum = reinterpret_cast<double *>(m.sp + (size_t)S * block);
    m.fsp = reinterpret_cast<int32_t *>(m.cum + (size_t)R * block);
    m.ford = m.fsp + (size_t)R * P;
    m.jsp = m.ford + (size_t)R * P;
    return m;
}

template <bool MACRO>
__global__ void __launch_bounds__(256) ssa_thread_kernel(const __grid_constant__ SsaArgs a) {
    const int BD = blockDim.x, tid = threadIdx.x;
    const int S = a.S, R = a.R, P = a.P, Q = a.Q;
    ThreadSmem m = thread_smem_layout(S, R, P, Q, BD);

    for (int k = tid; k < 2 * kZigTable; k += BD) m.zx[k] = a.zig[k];
    for (int k = tid; k < R; k += BD) m.rate[k] = a.rate_stride == 0 ? a.rate[k] : 0.0;
    for (int k = tid; k < R * Q; k += BD) {
        m.jd[k] = a.jmp_d[k];
        m.jsp[k] = a.jmp_sp[k];
    }
    for (int k = tid; k < R * P; k += BD) {
        m.fsp[k] = a.fac_sp[k];
        m.ford[k] = a.fac_ord[k];
    }
    __syncthreads();

    int64_t *const sp = m.sp + tid;    // species s of this lane: sp[s * BD]
    double *const cum = m.cum + tid;   // cumulative propensity r: cum[r * BD]
    unsigned long long lane_events = 0;
    const int64_t t_start = global_ns();
    bool out_of_time = false;
    unsigned int tick = 0;

    long long traj = (long long)atomicAdd(a.work, 1ull);
    while (traj < a.n_traj) {
        // ---- start (or resume) trajectory `traj`
        Xoshiro g;
        double t;
        if (a.in_species) {
            for (int s = 0; s < S; ++s) sp[s * BD] = a.in_species[traj * S + s];
            t = a.in_t[traj];
            g.s0 = a.in_rng[traj * 4 + 0];
            g.s1 = a.in_rng[traj * 4 + 1];
            g.s2 = a.in_rng[traj * 4 + 2];
            g.s3 = a.in_rng[traj * 4 + 3];
        } else {
            for (int s = 0; s < S; ++s) sp[s * BD] = a.x0[traj * a.x0_stride + s];
            t = 0.0;
            xo_seed(g, a.seeds[traj]);
        }
        const double *rates = a.rate_stride ? a.rate + traj * a.rate_stride : m.rate;
        unsigned long long ev = 0;
        long long i = 0;
        double T = a.sample_t[0];
        bool stale = true;
        double total = 0.0;

        for (;;) {
            if ((++tick & 1023u) == 0 && global_ns() - t_start > a.budget_ns) {
                out_of_time = true;
                break;
            }
            if (stale) {
                // make_cumrates with the LMA (or macro) propensity of every reaction
                total = 0.0;
                for (int r = 0; r < R; ++r) {
                    double acc = rates[r];
                    for (int p = 0; p < P; ++p) {
                        const int o = m.ford[r * P + p];
                        if (o == 0) continue;
                        const int64_t n = sp[m.fsp[r * P + p] * BD];
                        if (MACRO) {
                            int64_t ff = n;
                            for (int j = 1; j < o; ++j) ff *= n - j;
                            acc = __dmul_rn(acc, (double)ff);
                        } else {
                            for (int j = o - 1; j >= 0; --j) acc = __dmul_rn(acc, (double)(n - j));
                        }
                    }
                    total = __dadd_rn(total, acc);
                    cum[r * BD] = total;
                }
                stale = false;
            }
            bool record = true;
            if (0.0 < total) {
                const double e = xo_exp1(g, m.zx, m.zf);
                const double tn = __dadd_rn(t, __ddiv_rn(e, total));
                if (!(tn > T)) {
                    t = tn;
                    const double chosen = __dmul_rn(total, xo_uniform(g));
                    int idx;
                    if (MACRO) {
                        idx = R;
                        for (int r = R - 1; r >= 0; --r)
                            if (chosen < cum[r * BD]) idx = r;
                    } else {
                        idx = 0;
                        for (int r = 0; r < R; ++r) idx += (cum[r * BD] < chosen) ? 1 : 0;
                    }
                    if (idx < R) {
                        for (int q = 0; q < Q; ++q) sp[m.jsp[idx * Q + q] * BD] += m.jd[idx * Q + q];
                    }
                    stale = true;
                    ++ev;
                    record = false;
                }
            }
            if (record) {
                t = T;
                int64_t *o = a.out + (size_t)i * a.n_save * a.n_traj + traj;
                for (int k = 0; k < a.n_save; ++k) o[(size_t)k * a.n_traj] = sp[a.save_idx[k] * BD];
                if (++i == a.n_samples) break;
                T = a.sample_t[i];
            }
        }

        // ---- trajectory done
        if (a.fin_species)
            for (int s = 0; s < S; ++s) a.fin_species[traj * S + s] = sp[s * BD];
        if (a.fin_t) a.fin_t[traj] = t;
        if (a.fin_rng) {
            a.fin_rng[traj * 4 + 0] = g.s0;
            a.fin_rng[traj * 4 + 1] = g.s1;
            a.fin_rng[traj * 4 + 2] = g.s2;
            a.fin_rng[traj * 4 + 3] = g.s3;
        }
        if (a.events) a.events[traj] = ev;
        lane_events += ev;
        if (out_of_time) {
            atomicExch(a.work + 2, 1ull);
            break;
        }
        traj = (long long)atomicAdd(a.work, 1ull);
    }

    // total events: warp reduction, one atomic per warp
    for (int off = 16; off > 0; off >>= 1) lane_events += __shfl_down_sync(0xffffffffu, lane_events, off);
    if ((tid & 31) == 0 && lane_events) atomicAdd(a.work + 1, lane_events);
}

size_t ssa_thread_smem(const SsaArgs &a, int block) { return thread_smem_bytes(a.S, a.R, a.P, a.Q, block); }

int ssa_thread_max_block(const SsaArgs &a, size_t smem_limit) {
    for (int b = 128; b >= 32; b >>= 1)
        if (thread_smem_bytes(a.S, a.R, a.P, a.Q, b) <= smem_limit) return b;
    return 0;
}

int launch_ssa_thread(const SsaArgs &a, int block, int grid, size_t smem, void *stream) {
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t err;
    if (a.macro_mode) {
        err = cudaFuncSetAttribute(ssa_thread_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return (int)err;
        ssa_thread_kernel<true><<<grid, block, smem, st>>>(a);
    } else {
        err = cudaFuncSetAttribute(ssa_thread_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return (int)err;
        ssa_thread_kernel<false><<<grid, block, smem, st>>>(a);
    }
    return (int)cudaGetLastError();
}

}  // namespace rbg

namespace rbg {

int ssa_thread_occupancy(const SsaArgs &a, int block, size_t smem) {
    int n = 0;
    if (a.macro_mode) {
        cudaFuncSetAttribute(ssa_thread_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssa_thread_kernel<true>, block, smem);
    } else {
        cudaFuncSetAttribute(ssa_thread_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, ssa_thread_kernel<false>, block, smem);
    }
    return n;
}

// Propensity of reaction r at counts sp (API fold or macro factorials).
template <bool MACRO>
__device__ __forceinline__ double event_propensity(const EventArgs &a, const int64_t *sp, int r) {
    double acc = a.rate[r];
    for (int p = 0; p < a.P; ++p) {
        const int o = a.fac_ord[r * a.P + p];
        if (o == 0) continue;
        const int64_t n = sp[a.fac_sp[r * a.P + p]];
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

// _advance_one_reaction in a loop.  The cumulative propensities are not
// stored: the choice pass recomputes the same running sum, which gives the
// same binary64 values as the first pass.
template <bool MACRO>
__global__ void __launch_bounds__(128) ssa_events_kernel(const __grid_constant__ EventArgs a) {
    __shared__ double zt[2 * kZigTable];
    for (int k = threadIdx.x; k < 2 * kZigTable; k += blockDim.x) zt[k] = a.zig[k];
    __syncthreads();
    const long long traj = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (traj >= a.n_traj) return;
    int64_t *sp = a.species + traj * a.S;
    double t = a.t[traj];
    Xoshiro g{a.rng[traj * 4 + 0], a.rng[traj * 4 + 1], a.rng[traj * 4 + 2], a.rng[traj * 4 + 3]};
    long long n = 0;
    auto record = [&]() {
        if (n < a.cap) {
            a.rec_t[traj * a.cap + n] = t;
            for (int k = 0; k < a.n_save; ++k) a.rec_out[(traj * a.cap + n) * a.n_save + k] = sp[a.save_idx[k]];
        }
        ++n;
    };
    if (a.record_initial) record();
    long long steps = 0;
    const int64_t t_start = global_ns();
    while ((!a.gate || t < a.tmax) && (a.max_steps < 0 || steps < a.max_steps)) {
        if ((steps & 1023) == 1023 && global_ns() - t_start > a.budget_ns) {
            atomicExch(a.flag, 1ull);
            break;
        }
        double total = 0.0;
        for (int r = 0; r < a.R; ++r) total = __dadd_rn(total, event_propensity<MACRO>(a, sp, r));
        if (!(0.0 < total)) {
            t = __longlong_as_double(0x7FF0000000000000ll);  // +inf
        } else {
            t = __dadd_rn(t, __ddiv_rn(xo_exp1(g, zt, zt + kZigTable), total));
            const double chosen = __dmul_rn(total, xo_uniform(g));
            double c = 0.0;
            int idx = MACRO ? a.R : 0;
            for (int r = 0; r < a.R; ++r) {
                c = __dadd_rn(c, event_propensity<MACRO>(a, sp, r));
                if (MACRO) {
                    if (idx == a.R && chosen < c) idx = r;
                } else {
                    idx += (c < chosen) ? 1 : 0;
                }
            }
            if (idx < a.R)
                for (int q = 0; q < a.Q; ++q) sp[a.jmp_sp[idx * a.Q + q]] += a.jmp_d[idx * a.Q + q];
        }
        ++steps;
        record();
    }
    a.t[traj] = t;
    a.rng[traj * 4 + 0] = g.s0;
    a.rng[traj * 4 + 1] = g.s1;
    a.rng[traj * 4 + 2] = g.s2;
    a.rng[traj * 4 + 3] = g.s3;
    if (a.n_rec) a.n_rec[traj] = n;
}

int launch_ssa_events(const EventArgs &a, void *stream) {
    if (a.n_traj == 0) return 0;
    const int block = 128;
    const int grid = (int)((a.n_traj + block - 1) / block);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (a.macro_mode)
        ssa_events_kernel<true><<<grid, block, 0, st>>>(a);
    else
        ssa_events_kernel<false><<<grid, block, 0, st>>>(a);
    return (int)cudaGetLastError();
}

}  // namespace rbg
