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

// Rate::Expr propensity (expr.rs:23-39, gillespie.rs:88) in native binary64:
// IEEE operations, powf and exp from CUDA's math library, max/min returning
// the operand that is not NaN.  Counts are read at sp[s * stride].
__device__ __noinline__ double expr_eval(const int32_t *code, int32_t b, int32_t e, const double *consts,
                                         const int64_t *sp, int stride) {
    double st[kExprMaxDepth];
    int top = 0;
    for (int32_t k = b; k < e; ++k) {
        const int32_t w = code[k];
        const int op = w & 0xff, arg = w >> 8;
        if (op == 0) {
            st[top++] = consts[arg];
        } else if (op == 1) {
            st[top++] = (double)sp[(size_t)arg * stride];
        } else if (op == 2) {
            st[top - 1] = -st[top - 1];
        } else if (op == 10) {
            st[top - 1] = exp(st[top - 1]);
        } else {
            const double y = st[--top], x = st[top - 1];
            double v;
            switch (op) {
                case 3: v = __dadd_rn(x, y); break;
                case 4: v = __dsub_rn(x, y); break;
                case 5: v = __dmul_rn(x, y); break;
                case 6: v = __ddiv_rn(x, y); break;
                case 7: v = pow(x, y); break;
                case 8: v = fmax(x, y); break;
                default: v = fmin(x, y); break;
            }
            st[top - 1] = v;
        }
    }
    return st[0];
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
                    if (a.ex_off && a.ex_off[r] < a.ex_off[r + 1])
                        acc = expr_eval(a.ex_code, a.ex_off[r], a.ex_off[r + 1], a.ex_const, sp, BD);
                    else
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
    if (a.ex_off && a.ex_off[r] < a.ex_off[r + 1])
        return expr_eval(a.ex_code, a.ex_off[r], a.ex_off[r + 1], a.ex_const, sp, 1);
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

// ---------------------------------------------------------------------------
// Ensemble run without device allocation.
//
// Some hosts cannot let a library call cudaMalloc: an application whose own
// pool allocator owns all GPU memory and forbids allocations outside it after
// start-up, or a latency-critical caller that cannot take cudaMalloc's implicit
// device-wide synchronisation in the middle of its work.  For them the run
// below keeps everything the engine itself needs on the device -- the counters
// the kernel updates, the Exp1 tables, the packed reaction descriptor, the
// sample times and the saved-species list -- in one fixed array compiled into
// this library, so no device memory is allocated by the call.  The caller
// still owns and passes every input and output buffer.
//
// The array is kNoAllocScratchBytes (64 KiB) per GPU; every GPU that loads
// the library keeps it until the process exits.  A run whose descriptor,
// sample grid and saved list do not fit is rejected with RB_ERR_INVALID.
// All calls share the one array: each call clears the counters and rewrites
// the rest before its kernel starts, and two calls whose work overlaps on the
// GPU (for instance on two streams) overwrite each other's data and race.
//
// The call's own data reaches the array as the by-value parameters of small
// staging kernels (at most kNoAllocStageChunk bytes each), which the launch
// itself copies; no host buffer is read after the call returns.
// ---------------------------------------------------------------------------

#include <cstring>
#include <mutex>

#include "engine.hpp"
#include "network.hpp"

namespace rbg {

constexpr size_t kNoAllocScratchBytes = 64 * 1024;
constexpr size_t kNoAllocCounterBytes = 256;  // [0] ticket, [1] events, [2] timeout flag
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// One staging launch: `nbytes` (a multiple of 16) bytes of `data` go to the
// array at `offset`.  The struct travels as the kernel's parameter block
// (below the 32 764-byte parameter limit).
constexpr uint32_t kNoAllocStageChunk = 30720;
struct NoAllocChunk {
    uint32_t offset, nbytes;
    alignas(16) unsigned char data[kNoAllocStageChunk];
};

__global__ void noalloc_stage_kernel(const __grid_constant__ NoAllocChunk c) {
    const uint4 *src = reinterpret_cast<const uint4 *>(c.data);
    uint4 *dst = reinterpret_cast<uint4 *>(g_noalloc_scratch + c.offset);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < c.nbytes / 16; i += gridDim.x * blockDim.x)
        dst[i] = src[i];
}

namespace {

std::mutex g_na_mu;
unsigned char *g_na_dev[kNoAllocMaxDevices];      // device address of the array, per device
alignas(16) unsigned char g_na_host[kNoAllocScratchBytes];  // host image, built under g_na_mu
NoAllocChunk g_na_chunk;                                    // parameter block, filled under g_na_mu

size_t na_align(size_t v) { return (v + 15) & ~(size_t)15; }

}  // namespace

int noalloc_ensemble_run(const Network &net, int64_t n_traj, const int64_t *d_x0, int32_t x0_per_traj,
                         const double *d_rates, int32_t rates_per_traj, const uint64_t *d_seeds, double tmax,
                         int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *d_out,
                         uint64_t *d_events, uint64_t *d_status, void *stream, std::string &err) {
    const int64_t S = net.n_species, R = (int64_t)net.reactions.size();
    if (n_traj < 0) return err = "negative number of trajectories", 1;
    if (nb_steps < 1) return err = "nb_steps must be >= 1", 1;
    if (nb_steps >= (int64_t)(kNoAllocScratchBytes / 8))
        return err = "the no-allocation scratch holds " + std::to_string(kNoAllocScratchBytes) +
                     " bytes, too few for " + std::to_string(nb_steps + 1) + " sample times",
               1;
    const int64_t NS = (n_save < 0 || !save_idx) ? S : n_save;
    for (int64_t k = 0; k < NS && n_save >= 0 && save_idx; k++)
        if (save_idx[k] < 0 || save_idx[k] >= S) return err = "save index out of range", 1;
    if (n_traj && S && !d_x0) return err = "null x0", 1;
    if (n_traj && !d_seeds) return err = "null seeds", 1;
    if (n_traj && NS && !d_out) return err = "null out", 1;
    for (const Reaction &r : net.reactions)
        if (!r.ex_code.empty()) return err = "rate expressions need the allocating entry points", 5;
    int64_t P = 1, Q = 1;
    for (const Reaction &r : net.reactions) {
        P = std::max<int64_t>(P, (int64_t)r.factors.size());
        Q = std::max<int64_t>(Q, (int64_t)r.jump.size());
    }
    // Layout of the array: counters | Exp1 tables | descriptor | sample times | saved list.
    const size_t o_zig = kNoAllocCounterBytes;
    const size_t o_rate = na_align(o_zig + sizeof(double) * 2 * kZigTable);
    const size_t o_jd = na_align(o_rate + 8 * (size_t)std::max<int64_t>(R, 1));
    const size_t o_fsp = na_align(o_jd + 8 * (size_t)std::max<int64_t>(R * Q, 1));
    const size_t o_ford = na_align(o_fsp + 4 * (size_t)std::max<int64_t>(R * P, 1));
    const size_t o_jsp = na_align(o_ford + 4 * (size_t)std::max<int64_t>(R * P, 1));
    const size_t o_st = na_align(o_jsp + 4 * (size_t)std::max<int64_t>(R * Q, 1));
    const size_t o_save = na_align(o_st + 8 * (size_t)(nb_steps + 1));
    const size_t used = na_align(o_save + 4 * (size_t)std::max<int64_t>(NS, 1));
    if (used > kNoAllocScratchBytes)
        return err = "the no-allocation scratch holds " + std::to_string(kNoAllocScratchBytes) +
                     " bytes; this network (" + std::to_string(R) + " reactions) with " +
                     std::to_string(nb_steps + 1) + " sample times and " + std::to_string(NS) +
                     " saved species needs " + std::to_string(used),
               1;

    int dev = 0, sms = 0, smem_optin = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return err = std::string("cudaGetDevice: ") + cudaGetErrorString(ce), 2;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return err = "device ordinal out of range", 1;
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_dev[dev]) {
        // Once per device, with that device current: the host-side name of
        // the array is not a device address; ask the runtime for it.  The
        // address is kept for the life of the process, so it is stale after a
        // cudaDeviceReset of that device.
        void *p = nullptr;
        ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (ce != cudaSuccess) return err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(ce), 2;
        g_na_dev[dev] = static_cast<unsigned char *>(p);
    }
    unsigned char *dbase = g_na_dev[dev];
    ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (ce != cudaSuccess) return err = std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(ce), 2;

    unsigned char *h = g_na_host;
    zig_tables_host(reinterpret_cast<double *>(h + o_zig), reinterpret_cast<double *>(h + o_zig) + kZigTable);
    double *rate = reinterpret_cast<double *>(h + o_rate);
    int64_t *jd = reinterpret_cast<int64_t *>(h + o_jd);
    int32_t *fsp = reinterpret_cast<int32_t *>(h + o_fsp), *ford = reinterpret_cast<int32_t *>(h + o_ford);
    int32_t *jsp = reinterpret_cast<int32_t *>(h + o_jsp);
    std::memset(h + o_rate, 0, o_st - o_rate);
    int32_t max_order = 0;
    for (int64_t i = 0; i < R; i++) {
        const Reaction &r = net.reactions[i];
        rate[i] = r.rate;
        for (size_t k = 0; k < r.factors.size(); k++) {
            fsp[i * P + k] = r.factors[k].species;
            ford[i * P + k] = r.factors[k].order;
            max_order = std::max(max_order, r.factors[k].order);
        }
        for (size_t k = 0; k < r.jump.size(); k++) {
            jsp[i * Q + k] = r.jump[k].species;
            jd[i * Q + k] = r.jump[k].delta;
        }
    }
    double *st = reinterpret_cast<double *>(h + o_st);
    for (int64_t i = 0; i <= nb_steps; i++) st[i] = tmax * (double)i / (double)nb_steps;
    int32_t *sv = reinterpret_cast<int32_t *>(h + o_save);
    for (int64_t k = 0; k < NS; k++) sv[k] = (n_save < 0 || !save_idx) ? (int32_t)k : save_idx[k];

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    ce = cudaMemsetAsync(dbase, 0, kNoAllocCounterBytes, s);
    if (ce != cudaSuccess) return err = std::string("counter reset: ") + cudaGetErrorString(ce), 2;
    // The image goes over as launch parameters, copied when each staging
    // kernel is launched, so g_na_host is free for the next call on return.
    for (size_t off = o_zig; off < used; off += kNoAllocStageChunk) {
        const size_t nb = std::min<size_t>(kNoAllocStageChunk, used - off);
        g_na_chunk.offset = (uint32_t)off;
        g_na_chunk.nbytes = (uint32_t)nb;
        std::memcpy(g_na_chunk.data, h + off, nb);
        noalloc_stage_kernel<<<8, 128, 0, s>>>(g_na_chunk);
        ce = cudaGetLastError();
        if (ce != cudaSuccess) return err = std::string("staging launch: ") + cudaGetErrorString(ce), 2;
    }

    SsaArgs a{};
    a.S = (int32_t)S;
    a.R = (int32_t)R;
    a.P = (int32_t)P;
    a.Q = (int32_t)Q;
    a.macro_mode = net.macro_mode ? 1 : 0;
    a.rate = d_rates ? d_rates : reinterpret_cast<const double *>(dbase + o_rate);
    a.rate_stride = d_rates && rates_per_traj ? R : 0;
    a.fac_sp = reinterpret_cast<const int32_t *>(dbase + o_fsp);
    a.fac_ord = reinterpret_cast<const int32_t *>(dbase + o_ford);
    a.jmp_sp = reinterpret_cast<const int32_t *>(dbase + o_jsp);
    a.jmp_d = reinterpret_cast<const int64_t *>(dbase + o_jd);
    a.n_traj = n_traj;
    a.x0 = d_x0;
    a.x0_stride = x0_per_traj ? S : 0;
    a.seeds = d_seeds;
    a.sample_t = reinterpret_cast<const double *>(dbase + o_st);
    a.n_samples = nb_steps + 1;
    a.save_idx = reinterpret_cast<const int32_t *>(dbase + o_save);
    a.n_save = (int32_t)NS;
    a.out = d_out;
    a.events = d_events;
    a.work = reinterpret_cast<unsigned long long *>(dbase);
    a.zig = reinterpret_cast<const double *>(dbase + o_zig);
    a.budget_ns = kernel_budget_ns();
    (void)max_order;
    if (n_traj > 0) {
        const int block = ssa_thread_max_block(a, (size_t)smem_optin);
        if (block == 0) return err = "network too large for the thread-per-trajectory kernel", 5;
        const size_t smem = ssa_thread_smem(a, block);
        int per_sm = std::max(1, ssa_thread_occupancy(a, block, smem));
        const int64_t want = (n_traj + block - 1) / block;
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
        int le = launch_ssa_thread(a, block, grid, smem, stream);
        if (le != 0) return err = std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)le), 2;
    }
    if (d_status) {
        ce = cudaMemcpyAsync(d_status, dbase + 8, 16, cudaMemcpyDeviceToDevice, s);
        if (ce != cudaSuccess) return err = std::string("status copy: ") + cudaGetErrorString(ce), 2;
    }
    return 0;
}

}  // namespace rbg
