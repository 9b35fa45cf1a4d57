// Lockstep thread-per-trajectory SSA kernel with exact binary64 emulation.
//
// Same contract and results as ssa_thread_kernel (one thread per trajectory,
// ticket refill, rebop's direct method and sampling loop), built for GB300:
// every step runs ssa_exact.cuh's exact_step, whose binary64 products and
// division run as exact integer arithmetic and whose adds use the FP64 pipe
// (RB_FAST_ADD=int moves them to the integer pipes too).  All lanes execute
// the same instruction stream per step: propensities, the Exp1 draw, the
// candidate clock and the choice, then either fire or record.  The same exact
// step re-runs the sample intervals that ssa_spec.cu cannot decide.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "ssa_exact.cuh"

namespace rbg {

extern __shared__ __align__(16) unsigned char g_fast_smem[];

namespace {

struct FastSmem {
    ExactTables ex;
    uint64_t *rate;  // [R][block] per-lane rate bits
    int64_t *sp;     // [S][block] per-lane counts
};

__host__ __device__ inline size_t fast_smem_bytes(int S, int R, int P, int Q, int block) {
    size_t b = 16 * 256 + 8 * 257 + 8 * 256;
    b += 8 * (size_t)R * Q;
    b += 8 * (size_t)R * block;
    b += 8 * (size_t)S * block;
    b += 4 * ((size_t)R * P + (size_t)R * Q);
    return (b + 15) & ~(size_t)15;
}

__device__ inline FastSmem fast_layout(const SsaArgs &a, int block, ulonglong2 *&zxk, uint64_t *&zf, uint64_t *&zd,
                                       int32_t *&fac, int32_t *&jsp, int64_t *&jd) {
    FastSmem m;
    zxk = reinterpret_cast<ulonglong2 *>(g_fast_smem);
    zf = reinterpret_cast<uint64_t *>(zxk + 256);
    zd = zf + 257;
    jd = reinterpret_cast<int64_t *>(zd + 256);
    m.rate = reinterpret_cast<uint64_t *>(jd + (size_t)a.R * a.Q);
    m.sp = reinterpret_cast<int64_t *>(m.rate + (size_t)a.R * block);
    fac = reinterpret_cast<int32_t *>(m.sp + (size_t)a.S * block);
    jsp = fac + (size_t)a.R * a.P;
    m.ex = ExactTables{zxk, zf, zd, fac, jsp, jd};
    return m;
}

}  // namespace

template <int MAXR, bool MACRO, bool ADD_NATIVE>
__global__ void __launch_bounds__(128, 6) ssa_fast_kernel(const __grid_constant__ SsaArgs a) {
    const int BD = blockDim.x, tid = threadIdx.x;
    const int S = a.S, R = a.R, Q = a.Q;
    ulonglong2 *zxk;
    uint64_t *zf, *zd;
    int32_t *fac, *jsp;
    int64_t *jd;
    const FastSmem m = fast_layout(a, BD, zxk, zf, zd, fac, jsp, jd);
    load_exact_tables(a, zxk, zf, zd, fac, jsp, jd);
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
        int idx;
        uint64_t tn;
        const bool fire = exact_step<MAXR, MACRO, ADD_NATIVE>(a, m.ex, sp, rl, BD, BD, g, t, T, nat, idx, tn);
        if (fire) {
            t = tn;
            ++ev;
            if (idx < R)
                for (int k = 0; k < Q; ++k) sp[jsp[idx * Q + k] * BD] += jd[idx * Q + k];
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
