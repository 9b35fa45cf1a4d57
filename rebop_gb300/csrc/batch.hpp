// Heterogeneous batches run by one CUDA graph (batch.cpp).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "engine.hpp"
#include "network.hpp"
#include "ssa_args.hpp"

namespace rbg {

struct rb_stats_out {
    uint64_t events = 0;
    float graph_ms = 0.f;
    size_t h2d = 0, d2h = 0;
    int launches = 0;
    bool replayed = false, timeout = false;
};

struct Batch {
    // One item: a network and one ensemble of it (host buffers, kept by pointer).
    struct ItemIn {
        int64_t n_traj = 0;
        const int64_t *x0 = nullptr;
        int32_t x0_per_traj = 0;
        const double *rates = nullptr;  // null: the network's rates
        int32_t rates_per_traj = 0;
        const uint64_t *seeds = nullptr;
        double tmax = 0.0;
        int64_t nb_steps = 1;
        const int32_t *save_idx = nullptr;
        int32_t n_save = -1;            // < 0: every species
        int64_t *out = nullptr;         // [nb_steps + 1][n_save][n_traj]; null: the results stay with the batch
        uint64_t *events = nullptr;     // [n_traj] or null
    };
    struct Item {
        const Network *net = nullptr;
        uint64_t version = 0;
        Packed packed;
        ItemIn in;
        std::vector<int32_t> save;
        int mapping = -1;
        // results of an item added without an output buffer when its rows are
        // not contiguous in the staging buffer (merged classes)
        std::vector<int64_t> own_out;
        size_t o_x0 = 0, o_seeds = 0, o_times = 0, o_save = 0, o_rates = 0, o_fsp = 0, o_ford = 0, o_jsp = 0,
               o_jd = 0, o_rdf = 0, o_lfac = 0, o_shape = 0, o_fpk = 0, o_out = 0, o_events = 0;
    };
    // A launch of the thread-per-trajectory kernels: items of one structure
    // and sample grid merged (Merged), or one item alone (Single).
    struct Class {
        enum Kind { Merged, Single } kind = Merged;
        std::vector<int> items;
        int64_t n_traj = 0;
        int32_t S = 0, R = 0, n_save = 0;
        int64_t n_samples = 0;
        size_t o_x0 = 0, o_rates = 0, o_seeds = 0, o_times = 0, o_save = 0, o_out = 0, o_events = 0;
        unsigned long long *scratch = nullptr;
    };

    std::vector<Item> items;
    std::vector<Class> classes;
    std::vector<int> warp_items;    // warp-per-trajectory items of the persistent launch, most work first
    std::vector<int> thread_items;  // its thread-unit items (32 trajectories a unit, one per lane)
    int macro_mode = 0;             // arithmetic of the persistent launch's items
    bool planned = false;

    // device state of the captured graph
    void *host = nullptr, *dev = nullptr;
    int64_t *warp_cnt0 = nullptr;  // the warp kernel's interval-start counts
    size_t in_bytes = 0, total_bytes = 0, o_items = 0, o_start = 0, o_work = 0, o_titems = 0, o_tunit = 0;
    SsaArgs warp_args{};
    int warp_warps = 0, warp_grid = 0;
    int64_t warp_traj = 0;
    cudaStream_t stream = nullptr, side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, t0 = nullptr, t1 = nullptr;
    cudaEvent_t e_in = nullptr, e_kern = nullptr;  // inside the graph: inputs copied, kernels done
    float last_in_ms = 0.f, last_kern_ms = 0.f, last_out_ms = 0.f;
    cudaGraphExec_t exec = nullptr;

    std::string add(const Network *net, const ItemIn &in);
    // Adding an item invalidates the captured graph.
    void free_device_if_built() {
        if (exec || dev) free_device();
        planned = false;
    }
    bool plan();
    bool run(rb_stats_out &st);
    // After a run: item k's results where they lie (the page-locked staging
    // buffer, or the batch's own copy); valid until the next run, add or
    // destruction.  False before the first run.
    bool item_results(int k, const int64_t **out, const uint64_t **events) const;
    ~Batch();

  private:
    bool build(cudaStream_t st);
    void stage_inputs();
    void unstage_outputs(uint64_t &events);
    void free_device();
};

}  // namespace rbg
