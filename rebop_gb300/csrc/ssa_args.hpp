// Kernel argument block of the SSA kernels (plain C++, shared by the CUDA
// translation units and the host glue).  All pointers are device pointers.
#pragma once

#include "rtc_types.hpp"

namespace rbg {

constexpr int kExprMaxDepth = 16;  // evaluation stack of Rate::Expr programs
constexpr int kZigLayers = 256;            // ziggurat layers of the Exp1 sampler
constexpr int kZigTable = kZigLayers + 1;  // abscissae x[0..256] / f(x) values
// Device table layout (doubles / u64 words): x[257] | f[257] | k[256] | d[256]
// where k[i] is the number of 52-bit fractions u accepted without the wedge
// test in layer i and d[i] = f[i] - f[i+1] (see zig_fast_tables_host).
// The last block, xdf[256], holds each x[i] as a float pair (hi, lo) with
// hi + lo = x[i] to 2^-48, for the float-pair approximation of a draw.
constexpr int kZigOffF = kZigTable;
constexpr int kZigOffK = 2 * kZigTable;
constexpr int kZigOffD = 2 * kZigTable + kZigLayers;
constexpr int kZigOffXdf = 2 * kZigTable + 2 * kZigLayers;
constexpr int kZigWords = 2 * kZigTable + 3 * kZigLayers;

struct SsaArgs {
    // packed network (see network.hpp: Packed)
    int32_t S, R, P, Q;
    int32_t macro_mode;
    const double *rate;      // [R] shared, or [n_traj][R] when rate_stride == R
    int64_t rate_stride;     // 0 or R
    const int32_t *fac_sp;   // [R*P]
    const int32_t *fac_ord;  // [R*P]
    const int32_t *jmp_sp;   // [R*Q]
    const int64_t *jmp_d;    // [R*Q]
    // Rate::Expr programs (null ex_off: none): reaction r's postfix words are
    // ex_code[ex_off[r] .. ex_off[r+1]), empty for mass-action reactions
    const int32_t *ex_off;
    const int32_t *ex_code;
    const double *ex_const;

    // trajectories
    int64_t n_traj;
    const int64_t *x0;       // fresh start: [S] or [n_traj][S]
    int64_t x0_stride;       // 0 or S
    const uint64_t *seeds;   // fresh start: [n_traj]
    const int64_t *in_species;  // resume: [n_traj][S]   (non-null = resume mode)
    const double *in_t;         // resume: [n_traj]
    const uint64_t *in_rng;     // resume: [n_traj][4]

    // sampling
    const double *sample_t;  // [n_samples] advance_until targets
    int64_t n_samples;
    const int32_t *save_idx; // [n_save]
    int32_t n_save;
    int64_t *out;            // [n_samples][n_save][n_traj]

    // outputs (nullable)
    int64_t *fin_species;    // [n_traj][S]
    double *fin_t;           // [n_traj]
    uint64_t *fin_rng;       // [n_traj][4]
    uint64_t *events;        // [n_traj]

    // scratch: [0] trajectory ticket, [1] total accepted events,
    // [2] set to 1 when the time budget ran out, [3] exact interval re-runs
    unsigned long long *work;
    // Speculative kernels, nullable: [n_samples] per sample row, the number of
    // trajectories whose row of `out` is written and visible device-wide (the
    // host copies finished rows while the launch runs).  n_samples < 65536.
    unsigned int *row_done;

    // Exp1 ziggurat tables: x[257] then f[257]
    const double *zig;

    // Wall-clock budget per launch (ns of %globaltimer from each block's
    // start).  A clock increment below one ulp of t never reaches the next
    // sample time; the budget turns that endless loop into RB_ERR_TIMEOUT.
    int64_t budget_ns;

    // Largest sum of reactant orders over the reactions (float-pair error bound).
    int32_t max_mults;

    // Speculative kernel: trajectory slots per block (the same number for
    // every warp, at least one per lane).
    int32_t n_slots;
    // Speculative kernel: steps between two compactions of a warp's slots
    // (0: the default).
    int32_t phase_steps;
    // Speculative kernel: lanes of a warp that hold trajectories (0: all 32).
    // Small ensembles spread over more warps and SMs with fewer lanes each,
    // which shortens every trajectory's step latency.
    int32_t lanes;
    // Speculative kernel: which live slots a warp's lanes take at a phase
    // boundary when there are more than 32.  0: the 32 whose clocks lag
    // furthest behind (every trajectory advances through simulated time at
    // about the same pace, so the ones with the most events get the most steps
    // and the warp's trajectories end together); 1: rotation over the live
    // slots (every trajectory gets the same number of steps).
    int32_t sched;

    // Warp-per-trajectory kernel, one network: row j of dep_tab ([R][32])
    // holds the number n of reactions whose propensity reads a species that
    // reaction j changes, then their lane-major positions (see batch below)
    // in entries 1 .. n; n = 0xFFFF when there are more than 31.  After j
    // fires only those are re-evaluated (one coalesced load per step).  Null:
    // every propensity is re-evaluated at every step.
    const uint16_t *dep_tab;
    // Warp-per-trajectory kernel: [blocks x warps per block][S] counts at the
    // start of each warp's current sample interval (read only by an exact
    // re-run of the interval, so they stay out of shared memory).
    int64_t *warp_cnt0;
    // Warp-per-trajectory kernel: decide every choice with the exact fold, as
    // for a close float-pair comparison (RB_WARP_EXACT_CHOICE=1; tests).
    int32_t exact_choice;

    // Warp kernel over a batch of networks (batch != null): item k is
    // batch[k], its trajectories are the tickets batch_start[k] ..
    // batch_start[k+1] - 1; the launch's own S, R, P, Q are the largest of the
    // items'.  An item's lm_* fields point to its lane-major tables (reaction
    // l*C + i at position i*32 + l, C = ceil(R/32)): float-pair rates,
    // two-slot shapes (null unless every reaction has order <= 2) and factors
    // ([C][P][32], species | order << 16).
    const SsaArgs *batch;
    const int64_t *batch_start;
    int32_t batch_n;
    const float2 *lm_rdf;
    const uint32_t *lm_shape;
    const int32_t *lm_fac;
    // The same launch also runs thread units (batch != null): tickets below
    // n_warp_tickets are the warp items' trajectories, ticket
    // n_warp_tickets + u is thread unit u -- up to 32 trajectories of one
    // small-network item, one per lane, each run by the exact per-lane step.
    // Thread item k is tbatch[k]; its units are tbatch_unit[k] ..
    // tbatch_unit[k + 1] - 1, 32 trajectories each (the last one partial);
    // tbatch_S is the largest species count of the thread items.
    const SsaArgs *tbatch;
    const int64_t *tbatch_unit;
    int32_t tbatch_n, tbatch_S;
    int64_t n_warp_tickets;
    // A thread item's reactant factors [R][P], species | order << 16.
    const int32_t *fac_packed;
};

// Launch the thread-per-trajectory kernel; returns a cudaError_t value.
int launch_ssa_thread(const SsaArgs &a, int block, int grid, size_t smem, void *stream);
size_t ssa_thread_smem(const SsaArgs &a, int block);
int ssa_thread_max_block(const SsaArgs &a, size_t smem_limit);
int ssa_thread_occupancy(const SsaArgs &a, int block, size_t smem);

// Lockstep kernel with integer binary64 (ssa_fast.cu): networks with at most
// 32 reactions, reactant orders below 2^15 and finite non-negative sample times.
bool ssa_fast_supported(const SsaArgs &a, int max_order);
size_t ssa_fast_smem(const SsaArgs &a, int block);
int ssa_fast_occupancy(const SsaArgs &a, int block, size_t smem);
int launch_ssa_fast(const SsaArgs &a, int block, int grid, size_t smem, void *stream);

// Speculative float-pair kernel with exact interval re-runs (ssa_spec.cu):
// networks with at most 16 reactions and finite sample times in [0, 2^60).
bool ssa_spec_supported(const SsaArgs &a, int max_order);
int ssa_spec_block();
size_t ssa_spec_smem(const SsaArgs &a, int slots);
// Slots per block for a launch of `grid` blocks of `block` lanes: enough for
// every trajectory to be resident at once when shared memory allows; 0 if not
// even one slot per lane fits in smem_limit bytes.
int ssa_spec_slots(const SsaArgs &a, int grid, size_t smem_limit, int block);
int ssa_spec_occupancy(const SsaArgs &a, int block, size_t smem);
int launch_ssa_spec(const SsaArgs &a, int block, int grid, size_t smem, void *stream);

// Warp-per-trajectory kernel for large networks (ssa_warp.cu): any network
// without rate expressions.  ssa_warp_warps gives the warps per block that fit
// in smem_limit (0: none).
bool ssa_warp_supported(const SsaArgs &a, int max_order);
int ssa_warp_warps(const SsaArgs &a, size_t smem_limit);
size_t ssa_warp_smem(const SsaArgs &a, int warps);
int ssa_warp_occupancy(const SsaArgs &a, int warps, size_t smem);
int launch_ssa_warp(const SsaArgs &a, int warps, int grid, size_t smem, void *stream);
// Two-slot shape word of reaction r for the lane-major tables of a batch item.
uint32_t warp_shape_word(const int32_t *fac_sp, const int32_t *fac_ord, int P, int S, int r);

// Every-event runs (src/pyo3_gillespie.rs:209-223) and single
// _advance_one_reaction steps (src/gillespie.rs:269-297): one thread per
// trajectory, state in place in global memory.
struct EventArgs {
    int32_t S, R, P, Q;
    int32_t macro_mode;
    const double *rate;      // [R]
    const int32_t *fac_sp, *fac_ord, *jmp_sp;
    const int64_t *jmp_d;
    const int32_t *ex_off, *ex_code;  // as in SsaArgs
    const double *ex_const;
    int64_t n_traj;
    int64_t *species;        // [n_traj][S] in/out
    double *t;               // [n_traj] in/out
    uint64_t *rng;           // [n_traj][4] in/out
    double tmax;
    int32_t gate;            // 1: step while t < tmax; 0: no horizon
    int64_t max_steps;       // < 0: unlimited
    int32_t record_initial;  // record the state before the first step
    const int32_t *save_idx;
    int32_t n_save;
    int64_t cap;             // records kept per trajectory
    double *rec_t;           // [n_traj][cap]
    int64_t *rec_out;        // [n_traj][cap][n_save]
    int64_t *n_rec;          // [n_traj] records produced (may exceed cap)
    const double *zig;
    unsigned long long *flag;  // set to 1 when the time budget ran out
    int64_t budget_ns;
};
int launch_ssa_events(const EventArgs &a, void *stream);

}  // namespace rbg
