// Autotuner of the sampled-run kernels: for a network and ensemble it times
// short pilot runs of every kernel that covers them and of the launch shapes
// of the fastest one, and remembers the winner for networks of that shape on
// that GPU (in memory and in a cache file).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "engine.hpp"

namespace rbg {

// Cache key: species, reactions, largest summed reactant order, largest
// order, macro arithmetic, log2 of the trajectory count, per-trajectory
// rates, SM count and device name.
std::string tune_key(const Packed &p, int sm_count, const std::string &gpu, int64_t n_traj, bool rates_per_traj);

// The remembered shape for this run, if any (false: none, shape untouched).
// RB_TUNE=0 turns lookups off.
bool tune_lookup(const Packed &p, const DeviceCtx &ctx, int64_t n_traj, bool rates_per_traj, LaunchShape &shape);

// Cache file: $RB_TUNE_CACHE, else $HOME/.cache/rebop_gb300/tune_cache.txt.
// One line per key: "<key>|kernel block phase sched ms".
std::string tune_cache_path();
// Record a choice (memory and file).
void tune_store(const std::string &key, const LaunchShape &s, double ms);
// Forget every choice held in memory (the next lookup reads the cache file
// again), and delete the file too when `file`.
void tune_clear(bool file);
bool tune_get(const std::string &key, LaunchShape &s, double *ms);

// Whether a kernel choice covers a run with these feasible kernels.
bool tune_shape_feasible(const Feasible &f, const LaunchShape &s);

// Candidate shapes of one tuning stage for the given feasibility and the
// best shape so far (stage 0: kernels; 1: block sizes of the generated
// kernel; 2: phase lengths and schedulers of the speculative kernels).
std::vector<LaunchShape> tune_candidates(const Feasible &f, int stage, const LaunchShape &best);

struct TuneTrial {
    LaunchShape shape;
    double ms;  // best of the timed pilot runs; < 0: the shape failed
};

// Run the tuner for one ensemble (host inputs as for rb_ensemble_run; fixed
// internal seeds).  Stores and returns the winner; false with the error set.
bool tune_ensemble(const Network &net, int64_t n_traj, const int64_t *x0, bool x0_per_traj, const double *rates,
                   bool rates_per_traj, double tmax, int64_t nb_steps, LaunchShape &best, double &best_ms,
                   std::vector<TuneTrial> &trials);

}  // namespace rbg
