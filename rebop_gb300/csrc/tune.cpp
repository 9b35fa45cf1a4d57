// Autotuner of the sampled-run kernels (see tune.hpp).
//
// The kernels differ in how they map trajectories to the GPU: a thread per
// trajectory (a kernel generated for the network, the speculative kernel over
// the packed descriptor, the lockstep exact kernel) or a warp per trajectory.
// Which is fastest, and with which block size, phase length and slot
// scheduler, depends on the network's size and on the ensemble: the tuner
// measures rather than guesses.  Pilot runs are whole ensemble runs of the
// caller's workload (its counts, rates, horizon and sample grid) with fixed
// internal seeds, timed with CUDA events; every kernel gives the same
// trajectories, so only the time differs.  Stages: the kernels that cover the
// run; then, for the generated kernel, its block size; then, for the
// speculative kernels, the phase length and the scheduler.
#include "tune.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <sys/stat.h>
#include <unistd.h>

namespace rbg {

namespace {

std::mutex g_tune_mu;
bool g_loaded = false;
struct Entry {
    LaunchShape s;
    double ms = 0;
};
std::map<std::string, Entry> g_cache;

void mkdirs(const std::string &path) {
    for (size_t i = 1; i <= path.size(); i++)
        if (i == path.size() || path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

void load_locked() {
    if (g_loaded) return;
    g_loaded = true;
    std::ifstream f(tune_cache_path());
    std::string line;
    while (std::getline(f, line)) {
        const size_t bar = line.rfind('|');
        if (bar == std::string::npos) continue;
        Entry e;
        std::istringstream in(line.substr(bar + 1));
        if (in >> e.s.kernel >> e.s.block >> e.s.phase >> e.s.sched >> e.ms) g_cache[line.substr(0, bar)] = e;
    }
}

void save_locked() {
    const std::string path = tune_cache_path();
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos) mkdirs(path.substr(0, slash));
    const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
    {
        std::ofstream f(tmp);
        if (!f) return;
        for (const auto &kv : g_cache)
            f << kv.first << '|' << kv.second.s.kernel << ' ' << kv.second.s.block << ' ' << kv.second.s.phase << ' '
              << kv.second.s.sched << ' ' << kv.second.ms << '\n';
        if (!f) return;
    }
    std::rename(tmp.c_str(), path.c_str());
}

uint64_t splitmix(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

bool tune_shape_feasible(const Feasible &f, const LaunchShape &s) {
    switch (s.kernel) {
        case 0: return f.generic;
        case 2: return f.fast;
        case 3: return f.spec;
        case 4: return f.jit;
        case 5: return f.warp;
        default: return false;
    }
}

std::string tune_key(const Packed &p, int sm_count, const std::string &gpu, int64_t n_traj, bool rates_per_traj) {
    int mm = 0;
    for (int32_t r = 0; r < p.R; r++) {
        int s = 0;
        for (int32_t k = 0; k < p.P; k++) s += p.fac_ord[(size_t)r * p.P + k];
        mm = std::max(mm, s);
    }
    int lg = 0;
    while (lg < 62 && (int64_t(1) << (lg + 1)) <= n_traj) ++lg;
    std::ostringstream o;
    o << "S=" << p.S << " R=" << p.R << " M=" << mm << " O=" << p.max_order << " macro=" << p.macro_mode
      << " expr=" << (p.has_expr ? 1 : 0) << " log2n=" << lg << " rpt=" << (rates_per_traj ? 1 : 0)
      << " sm=" << sm_count << " gpu=" << gpu;
    return o.str();
}

std::string tune_cache_path() {
    if (const char *e = std::getenv("RB_TUNE_CACHE")) return e;
    const char *home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/rebop_gb300/tune_cache.txt";
}

void tune_store(const std::string &key, const LaunchShape &s, double ms) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_locked();
    g_cache[key] = Entry{s, ms};
    save_locked();
}

bool tune_get(const std::string &key, LaunchShape &s, double *ms) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    load_locked();
    auto it = g_cache.find(key);
    if (it == g_cache.end()) return false;
    s = it->second.s;
    if (ms) *ms = it->second.ms;
    return true;
}

void tune_clear(bool file) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_cache.clear();
    g_loaded = false;  // the next lookup reads the file again
    if (file) std::remove(tune_cache_path().c_str());
}

bool tune_lookup(const Packed &p, const DeviceCtx &ctx, int64_t n_traj, bool rates_per_traj, LaunchShape &shape) {
    const char *e = std::getenv("RB_TUNE");
    if (e && std::strcmp(e, "0") == 0) return false;
    LaunchShape s;
    if (!tune_get(tune_key(p, ctx.sm_count, ctx.name, n_traj, rates_per_traj), s, nullptr)) return false;
    shape = s;
    return true;
}

std::vector<LaunchShape> tune_candidates(const Feasible &f, int stage, const LaunchShape &best) {
    std::vector<LaunchShape> out;
    auto add = [&](int kernel, int block, int phase, int sched) {
        LaunchShape s;
        s.kernel = kernel;
        s.block = block;
        s.phase = phase;
        s.sched = sched;
        if (tune_shape_feasible(f, s)) out.push_back(s);
    };
    if (stage == 0) {
        add(4, 0, 0, -1);
        add(3, 0, 0, -1);
        add(2, 0, 0, -1);
        // a warp per trajectory pays off only when a step has many reactions
        // to spread over the lanes
        if (f.reactions >= 16 || (!f.spec && !f.fast)) add(5, 0, 0, -1);
        if (!f.spec && !f.fast) add(0, 0, 0, -1);
    } else if (stage == 1) {
        // lanes per block of the generated kernel (one block per SM: 12 warps
        // at 384 lanes leave up to 168 registers a lane, 16 at 512 leave 128)
        if (best.kernel == 4 && !f.spread)
            for (int b : {256, 320, 416, 448, 512}) add(4, b, best.phase, best.sched);
    } else if (stage == 2) {
        if (best.kernel == 3 || best.kernel == 4) {
            for (int ph : {64, 256}) add(best.kernel, best.block, ph, best.sched);
            add(best.kernel, best.block, best.phase, best.sched > 0 ? 0 : 1);
        }
    }
    return out;
}

bool tune_ensemble(const Network &net, int64_t n_traj, const int64_t *x0, bool x0_per_traj, const double *rates,
                   bool rates_per_traj, double tmax, int64_t nb_steps, LaunchShape &best, double &best_ms,
                   std::vector<TuneTrial> &trials) {
    DeviceCtx *ctx = device_ctx();
    if (!ctx || !ensure_device(net)) return false;
    DeviceNet &dn = *net.dev;
    const Packed &p = dn.packed;
    const size_t S = (size_t)p.S, R = (size_t)p.R, N = (size_t)n_traj, NT = (size_t)nb_steps + 1;
    const size_t n_x0 = x0_per_traj ? N : 1, n_rates = rates ? (rates_per_traj ? N : 1) : 0;
    // one device allocation: x0 | rates | seeds | sample times | saved list | out
    const size_t o_x0 = 0, o_rates = (o_x0 + 8 * n_x0 * S + 255) / 256 * 256;
    const size_t o_seed = (o_rates + 8 * n_rates * R + 255) / 256 * 256;
    const size_t o_st = (o_seed + 8 * N + 255) / 256 * 256, o_save = (o_st + 8 * NT + 255) / 256 * 256;
    const size_t o_out = (o_save + 4 * S + 255) / 256 * 256, total = o_out + 8 * NT * S * N;
    unsigned char *b = nullptr;
    if (!cuda_ok(cudaMalloc(&b, total), "cudaMalloc(tuner)")) return false;
    struct Free {
        unsigned char *p;
        ~Free() { cudaFree(p); }
    } guard{b};
    std::vector<uint64_t> seeds(N);
    uint64_t sm = 0x5EED0F7u;
    for (auto &v : seeds) v = splitmix(sm);
    std::vector<double> st = sample_times(tmax, nb_steps);
    std::vector<int32_t> save(S);
    for (size_t k = 0; k < S; k++) save[k] = (int32_t)k;
    if (!cuda_ok(cudaMemcpy(b + o_x0, x0, 8 * n_x0 * S, cudaMemcpyHostToDevice), "cudaMemcpy") ||
        (n_rates && !cuda_ok(cudaMemcpy(b + o_rates, rates, 8 * n_rates * R, cudaMemcpyHostToDevice), "cudaMemcpy")) ||
        !cuda_ok(cudaMemcpy(b + o_seed, seeds.data(), 8 * N, cudaMemcpyHostToDevice), "cudaMemcpy") ||
        !cuda_ok(cudaMemcpy(b + o_st, st.data(), 8 * NT, cudaMemcpyHostToDevice), "cudaMemcpy") ||
        !cuda_ok(cudaMemcpy(b + o_save, save.data(), 4 * S, cudaMemcpyHostToDevice), "cudaMemcpy"))
        return false;
    RunDev r;
    r.n_traj = n_traj;
    r.x0 = reinterpret_cast<int64_t *>(b + o_x0);
    r.x0_stride = x0_per_traj ? (int64_t)S : 0;
    r.rates = n_rates ? reinterpret_cast<double *>(b + o_rates) : nullptr;
    r.rate_stride = rates && rates_per_traj ? (int64_t)R : 0;
    r.seeds = reinterpret_cast<uint64_t *>(b + o_seed);
    r.sample_t = reinterpret_cast<double *>(b + o_st);
    r.n_samples = (int64_t)NT;
    r.save_idx = reinterpret_cast<int32_t *>(b + o_save);
    r.n_save = (int32_t)S;
    r.out = reinterpret_cast<int64_t *>(b + o_out);
    r.times_ok = std::isfinite(tmax) && tmax >= 0;
    r.t_last = tmax;
    const Feasible f = feasible_kernels(p, *ctx, n_traj, (int64_t)NT, r.times_ok, tmax, rates && rates_per_traj);

    // One untimed run (it compiles a generated kernel), then the best of two
    // timed runs; a shape that fails (e.g. no run-time compiler) is skipped.
    auto time_shape = [&](const LaunchShape &s) -> double {
        int mapping = 0;
        double ms_best = -1.0;
        for (int rep = 0; rep < 3; rep++) {
            if (!launch_sampled(net, dn, r, dn.stream, rep > 0, &mapping, &s)) {
                cudaGetLastError();
                return -1.0;
            }
            if (cudaStreamSynchronize(dn.stream) != cudaSuccess) return -2.0;
            if (rep == 0) continue;
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, dn.ev_start, dn.ev_stop) != cudaSuccess) return -2.0;
            if (ms_best < 0 || ms < ms_best) ms_best = ms;
        }
        return ms_best;
    };
    best = LaunchShape{};
    best_ms = -1.0;
    trials.clear();
    // one kernel and nothing to tune about it: no pilot run needed
    const std::vector<LaunchShape> only = tune_candidates(f, 0, best);
    if (only.size() == 1 && tune_candidates(f, 1, only[0]).empty() && tune_candidates(f, 2, only[0]).empty()) {
        best = only[0];
        best_ms = 0.0;
        trials.push_back(TuneTrial{best, 0.0});
        tune_store(tune_key(p, ctx->sm_count, ctx->name, n_traj, rates && rates_per_traj), best, best_ms);
        return true;
    }
    for (int stage = 0; stage < 3; stage++) {
        for (const LaunchShape &s : tune_candidates(f, stage, best)) {
            const double ms = time_shape(s);
            if (ms == -2.0) {
                cuda_ok(cudaGetLastError(), "pilot run");
                return false;
            }
            trials.push_back(TuneTrial{s, ms});
            if (ms >= 0 && (best_ms < 0 || ms < best_ms)) {
                best = s;
                best_ms = ms;
            }
        }
        if (best_ms < 0) break;
    }
    if (best_ms < 0) {
        set_error("no kernel covers this network and sample grid");
        return false;
    }
    tune_store(tune_key(p, ctx->sm_count, ctx->name, n_traj, rates && rates_per_traj), best, best_ms);
    return true;
}

}  // namespace rbg
