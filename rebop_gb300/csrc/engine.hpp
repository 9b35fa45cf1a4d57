// Host engine: per-device context, descriptor upload, kernel launches.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "network.hpp"
#include "ssa_args.hpp"

namespace rbg {

// Thread-local error channel of the C ABI.
void set_error(const std::string &msg);
const std::string &last_error();
// true for cudaSuccess; otherwise sets the error ("<what>: <CUDA message>").
bool cuda_ok(cudaError_t e, const char *what);

// Per-device immutable state: ziggurat tables and device properties.
struct DeviceCtx {
    int device = -1;
    int sm_count = 0;
    size_t smem_optin = 0;
    std::string name;       // device name (the autotuner's cache key)
    double *zig = nullptr;  // device [2][257]
};
// Context of the current device (created on first use); nullptr + error on failure.
DeviceCtx *device_ctx();
// Host copy of the Exp1 ziggurat tables (x[257], f[257]).
void zig_tables_host(double *x, double *f);
// Acceptance thresholds K[256] and wedge differences d[256] of those tables.
void zig_fast_tables_host(const double *x, const double *f, uint64_t *K, double *d);

// Device copy of one network's packed descriptor, its scratch words and the
// staging buffers of host-pointer calls.
struct DeviceNet {
    int device = -1;
    uint64_t version = 0;
    Packed packed;
    void *desc = nullptr;               // rate | jmp_d | fac_sp | fac_ord | jmp_sp
    double *rate = nullptr;
    int64_t *jmp_d = nullptr;
    int32_t *fac_sp = nullptr, *fac_ord = nullptr, *jmp_sp = nullptr;
    int32_t *ex_off = nullptr, *ex_code = nullptr;  // ex_off null: no Rate::Expr reaction
    double *ex_const = nullptr;
    unsigned long long *scratch = nullptr;  // [4]: trajectory ticket, event total, timeout flag
    void *io = nullptr;                 // staging for rb_ensemble_run & friends
    size_t io_bytes = 0;
    cudaStream_t stream = nullptr;      // library stream of host-pointer calls
    cudaStream_t copy_stream = nullptr; // result rows copied back while the kernel runs
    unsigned int *pin_rows = nullptr;   // page-locked copy of the row counters
    size_t pin_rows_n = 0;
    cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
    cudaStream_t last_stream = nullptr; // stream of the last device-pointer run
    int64_t runs = 0;                   // sampled launches of this network
    double out_gbs = 0;                 // sample bytes / kernel time of the last host-pointer run
    int64_t *warp_cnt0 = nullptr;       // warp kernel interval-start counts
    size_t warp_cnt0_n = 0;             //   (entries)
    uint16_t *dep = nullptr;            // warp kernel dependency table [R][32]
    uint64_t dep_version = 0;           //   for this descriptor version (0: none built)
    bool dep_ok = false;                //   false: the network is beyond the lists' reach
    const void *jit_k = nullptr;        // generated kernel last used, for
    int jit_block = 0;                  //   blocks of jit_block lanes and
    uint64_t jit_version = 0;           //   descriptor version jit_version
    ~DeviceNet();
};

// Dependency table of the warp kernel for a packed network ([R][32], see
// SsaArgs::dep_tab): row j lists the lane-major positions (reaction l*C + i
// at i*32 + l, C = ceil(R / 32)) of the reactions whose propensity reads a
// species reaction j changes.  False when the kernel's update groups cannot
// cover the network (more than 8192 reactions).
bool warp_dep_table(const Packed &p, std::vector<uint16_t> &tab);

// Make net.dev current for the active device and descriptor version.
// Caller holds net.mu.  Returns false (error set) on failure.
bool ensure_device(const Network &net);
// Grow net.dev->io to at least `bytes`.
bool ensure_io(DeviceNet &dn, size_t bytes);

// Device-side request of one sampled run (all pointers device pointers).
struct RunDev {
    int64_t n_traj = 0;
    const int64_t *x0 = nullptr;
    int64_t x0_stride = 0;
    const double *rates = nullptr;  // nullptr: network rates
    int64_t rate_stride = 0;
    const uint64_t *seeds = nullptr;
    const int64_t *in_species = nullptr;
    const double *in_t = nullptr;
    const uint64_t *in_rng = nullptr;
    const double *sample_t = nullptr;
    int64_t n_samples = 0;
    const int32_t *save_idx = nullptr;
    int32_t n_save = 0;
    int64_t *out = nullptr;
    int64_t *fin_species = nullptr;
    double *fin_t = nullptr;
    uint64_t *fin_rng = nullptr;
    uint64_t *events = nullptr;
    unsigned int *row_done = nullptr;  // [n_samples] row counters (speculative kernels)
    bool times_ok = false;  // every sample time finite and >= 0 (lets the fast kernels run)
    double t_last = 0.0;    // largest sample time
};

// Kernel and launch shape of a sampled run.  kernel is a mapping code
// (rb_run_stats.mapping: 0 generic, 2 lockstep exact, 3 speculative over the
// descriptor, 4 generated for the network, 5 warp per trajectory) or -1 for
// the built-in choice; block (generated kernel: lanes per block), phase
// (speculative kernels: steps per phase) and sched (their slot scheduler)
// are 0 / 0 / -1 for the defaults.
struct LaunchShape {
    int kernel = -1;
    int block = 0;
    int phase = 0;
    int sched = -1;
};

// Enqueue the sampled-run kernel on `stream` (scratch reset included).
// Records ev_start/ev_stop around the kernel when `timed`.  `force` fixes the
// kernel and launch shape (an error if it does not cover the run); without
// it the autotuner's choice for networks of this shape is used when it has
// one (tune.cpp), else the built-in choice.  RB_SSA_KERNEL, RB_JIT_BLOCK,
// RB_SPEC_PHASE and RB_SPEC_SCHED override both.
bool launch_sampled(const Network &net, DeviceNet &dn, const RunDev &r, cudaStream_t stream, bool timed,
                    int *mapping, const LaunchShape *force = nullptr);

// Which kernels can run a sampled run of this network (no GPU work).
struct Feasible {
    bool spec = false;     // speculative float-pair kernels (descriptor; generated when jit)
    bool jit = false;      // a kernel generated for the network
    bool fast = false;     // lockstep exact kernel
    bool warp = false;     // warp per trajectory
    bool generic = false;  // generic exact thread kernel
    bool spread = false;   // the ensemble is spread over fewer lanes per warp
    int reactions = 0;
};
Feasible feasible_kernels(const Packed &p, const DeviceCtx &ctx, int64_t n_traj, int64_t n_samples, bool times_ok,
                          double t_last, bool rates_per_traj);

// Ensemble run whose engine-side device data lives in a fixed array compiled
// into the library (ssa_thread.cu); returns 0, or 1 (invalid), 2 (CUDA),
// 5 (unsupported) with `err` set.
int noalloc_ensemble_run(const Network &net, int64_t n_traj, const int64_t *d_x0, int32_t x0_per_traj,
                         const double *d_rates, int32_t rates_per_traj, const uint64_t *d_seeds, double tmax,
                         int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *d_out,
                         uint64_t *d_events, uint64_t *d_status, void *stream, std::string &err);

// Per-launch wall-clock budget of the SSA kernels (RB_KERNEL_BUDGET_S, default 120 s).
int64_t kernel_budget_ns();

// Sample times t_i = tmax * i / nb_steps, i = 0..nb_steps (pyo3_gillespie.rs:202).
std::vector<double> sample_times(double tmax, int64_t nb_steps);

}  // namespace rbg
