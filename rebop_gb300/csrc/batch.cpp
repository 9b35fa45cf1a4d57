// Heterogeneous batches: many networks, parameter sets and trajectory counts
// run by one CUDA graph.
//
// Planning groups the items into classes of equal network structure, sample
// grid and saved species.  A class the thread-per-trajectory kernels cover
// becomes one ensemble whose trajectories carry their own rate constants and
// initial counts (so thousands of parameter sets of one network are one
// launch); every other item joins the warp-per-trajectory kernel's batch
// mode, where warps pull (item, trajectory) tickets from one queue, items
// with the most estimated work first.  The graph holds one host-to-device
// copy of all inputs, the kernels on concurrent branches, and one copy of all
// results back; it is captured on the first run and replayed while the batch
// is unchanged.
#include "batch.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <map>
#include <thread>

#include "ssa_jit.hpp"

namespace rbg {

namespace {

size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

// Float pair (hi truncated toward zero, lo rounded) of a rate, as the
// device's df_from_double makes it; 0 for a rate the float pairs do not cover.
void float_pair(double v, float *out) {
    float hi = (float)v;
    if ((double)hi > v && v > 0) hi = std::nextafter(hi, 0.0f);
    out[0] = std::isfinite(v) ? hi : 0.0f;
    out[1] = std::isfinite(v) ? (float)(v - (double)hi) : 0.0f;
}

// Structure of a network: everything but the rate constants.
std::string structure_key(const Packed &p) {
    std::string k;
    auto put = [&](const void *d, size_t n) { k.append(static_cast<const char *>(d), n); };
    put(&p.S, sizeof p.S);
    put(&p.R, sizeof p.R);
    put(&p.P, sizeof p.P);
    put(&p.Q, sizeof p.Q);
    put(&p.macro_mode, sizeof p.macro_mode);
    put(p.fac_sp.data(), p.fac_sp.size() * 4);
    put(p.fac_ord.data(), p.fac_ord.size() * 4);
    put(p.jmp_sp.data(), p.jmp_sp.size() * 4);
    put(p.jmp_d.data(), p.jmp_d.size() * 8);
    put(&p.has_expr, sizeof p.has_expr);
    put(p.ex_code.data(), p.ex_code.size() * 4);
    put(p.ex_const.data(), p.ex_const.size() * 8);
    return k;
}

// Rough work of one trajectory: initial total propensity * horizon (events)
// times the reactions touched per event.
double work_estimate(const Packed &p, const int64_t *x0, const double *rates, double tmax) {
    double tot = 0.0;
    for (int r = 0; r < p.R; r++) {
        double a = rates ? rates[r] : p.rate[r];
        for (int f = 0; f < p.P; f++) {
            const int o = p.fac_ord[(size_t)r * p.P + f];
            const double n = (double)x0[p.fac_sp[(size_t)r * p.P + f]];
            for (int j = 0; j < o; j++) a *= std::max(0.0, n - j);
        }
        if (std::isfinite(a) && a > 0) tot += a;
    }
    const double ev = std::min(1e9, tot * (std::isfinite(tmax) ? std::max(tmax, 0.0) : 0.0)) + 1.0;
    return ev * (double)std::max(p.R, 1);
}

}  // namespace

std::string Batch::add(const Network *net, const ItemIn &in) {
    if (!net) return "null network";
    if (in.n_traj < 0) return "negative number of trajectories";
    if (in.nb_steps < 1) return "nb_steps must be >= 1";
    Item it;
    it.net = net;
    it.in = in;
    {
        std::lock_guard<std::mutex> lk(net->mu);
        it.packed = net->pack();
        it.version = net->version;
    }
    const Packed &p = it.packed;
    if (in.n_traj > 0 && p.S > 0 && !in.x0) return "null x0";
    if (in.n_traj > 0 && !in.seeds) return "null seeds";
    if (in.n_save < 0) {
        for (int32_t s = 0; s < p.S; s++) it.save.push_back(s);
    } else {
        if (in.n_save > 0 && !in.save_idx) return "null save_idx";
        for (int32_t k = 0; k < in.n_save; k++) {
            if (in.save_idx[k] < 0 || in.save_idx[k] >= p.S) return "save index out of range";
            it.save.push_back(in.save_idx[k]);
        }
    }
    items.push_back(std::move(it));
    planned = false;
    return "";
}

// Choose each item's mapping.  By default one persistent launch runs every
// mass-action item of the launch's arithmetic: items of at most 16 species
// and 16 reactions as thread units (32 trajectories of one item, one per
// lane), the others a warp per trajectory, all from one queue -- warp items
// with the most estimated work first, thread units after them, filling the
// tail.  Rate expressions, define_system! items whose arithmetic differs
// from the launch's, and per-trajectory rates on networks too large for a
// thread unit run as launches of their own.  RB_BATCH_MODE=merged keeps the
// earlier plan: items of one structure and sample grid merged into one
// thread-per-trajectory launch, the rest in the warp launch.
bool Batch::plan() {
    classes.clear();
    warp_items.clear();
    thread_items.clear();
    const char *mode = std::getenv("RB_BATCH_MODE");
    const bool merged_mode = mode && std::strcmp(mode, "merged") == 0;
    // the persistent launch's arithmetic: the items' majority
    int64_t n_macro = 0, n_plain = 0;
    for (const Item &it : items)
        if (!it.packed.has_expr) (it.packed.macro_mode ? n_macro : n_plain) += 1;
    macro_mode = n_macro > n_plain ? 1 : 0;
    std::map<std::string, int> by_key;
    auto single = [&](int i) {
        items[i].mapping = 0;  // a launch of its own (launch_sampled picks the kernel)
        Class c;
        c.kind = Class::Single;
        c.items.push_back(i);
        c.n_traj = items[i].in.n_traj;
        classes.push_back(c);
    };
    for (size_t i = 0; i < items.size(); i++) {
        Item &it = items[i];
        const Packed &p = it.packed;
        SsaArgs probe{};
        probe.S = p.S;
        probe.R = p.R;
        probe.P = p.P;
        probe.Q = p.Q;
        const bool times_ok = std::isfinite(it.in.tmax) && it.in.tmax >= 0 && it.in.tmax < 0x1p60;
        if (!merged_mode) {
            if (p.has_expr || p.macro_mode != macro_mode) {
                single((int)i);
            } else if (p.S <= 16 && p.R <= 16 && times_ok) {
                it.mapping = 7;
                thread_items.push_back((int)i);
            } else if (it.in.rates_per_traj) {
                single((int)i);
            } else {
                it.mapping = 5;
                warp_items.push_back((int)i);
            }
            continue;
        }
        // thread-per-trajectory classes: networks the generated kernels cover
        const bool thread_ok = !p.has_expr && jit_supported(p) && ssa_spec_supported(probe, p.max_order) && times_ok;
        if (!thread_ok) {
            if (p.has_expr || it.in.rates_per_traj || p.macro_mode != macro_mode) {
                single((int)i);
            } else {
                it.mapping = 5;
                warp_items.push_back((int)i);
            }
            continue;
        }
        std::string key = structure_key(p);
        key.append(reinterpret_cast<const char *>(&it.in.tmax), sizeof(double));
        key.append(reinterpret_cast<const char *>(&it.in.nb_steps), sizeof(int64_t));
        key.append(reinterpret_cast<const char *>(it.save.data()), it.save.size() * 4);
        auto f = by_key.find(key);
        if (f == by_key.end()) {
            Class c;
            c.kind = Class::Merged;
            by_key[key] = (int)classes.size();
            classes.push_back(c);
            f = by_key.find(key);
        }
        Class &c = classes[f->second];
        c.items.push_back((int)i);
        c.n_traj += it.in.n_traj;
        it.mapping = 4;
    }
    if (merged_mode) {
        // a thread launch for a handful of trajectories wastes the GPU: small
        // classes join the warp batch (RB_BATCH_MIN_THREAD trajectories,
        // default 2048, make a class worth its own launch)
        int64_t min_thread = 2048;
        if (const char *e = std::getenv("RB_BATCH_MIN_THREAD")) min_thread = std::max<int64_t>(1, std::atoll(e));
        std::vector<Class> kept;
        for (Class &c : classes) {
            bool movable = c.kind == Class::Merged && c.n_traj < min_thread;
            for (int i : c.items) movable = movable && !items[i].in.rates_per_traj;
            if (!movable) {
                kept.push_back(c);
                continue;
            }
            for (int i : c.items) {
                items[i].mapping = 5;
                warp_items.push_back(i);
            }
        }
        classes.swap(kept);
    }
    // warp items: most work first; thread units follow in item order
    std::vector<std::pair<double, int>> order;
    for (int i : warp_items) {
        const Item &it = items[i];
        order.push_back({-work_estimate(it.packed, it.in.x0, it.in.rates, it.in.tmax) * (double)it.in.n_traj, i});
    }
    std::sort(order.begin(), order.end());
    warp_items.clear();
    for (auto &o : order) warp_items.push_back(o.second);
    planned = true;
    return true;
}

bool Batch::build(cudaStream_t st) {
    DeviceCtx *ctx = device_ctx();
    if (!ctx) return false;
    free_device();
    // ---------------- host staging layout: inputs | outputs (same offsets on the device)
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align16(off + bytes);
        return o;
    };
    // merged thread classes
    for (Class &c : classes) {
        const Item &it0 = items[c.items[0]];
        const Packed &p = it0.packed;
        c.S = p.S;
        c.R = p.R;
        c.n_samples = it0.in.nb_steps + 1;
        c.n_save = (int32_t)it0.save.size();
        if (c.kind == Class::Merged) {
            c.o_x0 = take(8 * (size_t)c.n_traj * p.S);
            c.o_rates = take(8 * (size_t)c.n_traj * std::max(p.R, 1));
        } else {
            c.o_x0 = take(8 * (size_t)(it0.in.x0_per_traj ? c.n_traj : 1) * p.S);
            c.o_rates = take(8 * (size_t)(it0.in.rates ? (it0.in.rates_per_traj ? c.n_traj : 1) : 1) *
                             std::max(p.R, 1));
        }
        c.o_seeds = take(8 * (size_t)c.n_traj);
        c.o_times = take(8 * (size_t)c.n_samples);
        c.o_save = take(4 * (size_t)std::max(c.n_save, 1));
    }
    // warp batch items
    int32_t maxS = 1, maxR = 1, maxP = 1, maxQ = 1;
    for (int i : warp_items) {
        Item &it = items[i];
        const Packed &p = it.packed;
        maxS = std::max(maxS, p.S);
        maxR = std::max(maxR, p.R);
        maxP = std::max(maxP, p.P);
        maxQ = std::max(maxQ, p.Q);
        const size_t RP = 32 * (size_t)((p.R + 31) / 32);
        it.o_x0 = take(8 * (size_t)(it.in.x0_per_traj ? it.in.n_traj : 1) * p.S);
        it.o_seeds = take(8 * (size_t)it.in.n_traj);
        it.o_times = take(8 * (size_t)(it.in.nb_steps + 1));
        it.o_save = take(4 * (size_t)std::max<size_t>(it.save.size(), 1));
        it.o_rates = take(8 * (size_t)std::max(p.R, 1));
        it.o_fsp = take(4 * (size_t)p.R * p.P);
        it.o_ford = take(4 * (size_t)p.R * p.P);
        it.o_jsp = take(4 * (size_t)p.R * p.Q);
        it.o_jd = take(8 * (size_t)p.R * p.Q);
        it.o_rdf = take(8 * RP);
        it.o_lfac = take(4 * RP * p.P);
        it.o_shape = take(4 * RP);
    }
    // thread-unit items
    int32_t maxTS = 1;
    for (int i : thread_items) {
        Item &it = items[i];
        const Packed &p = it.packed;
        maxTS = std::max(maxTS, p.S);
        it.o_x0 = take(8 * (size_t)(it.in.x0_per_traj ? it.in.n_traj : 1) * p.S);
        it.o_seeds = take(8 * (size_t)it.in.n_traj);
        it.o_times = take(8 * (size_t)(it.in.nb_steps + 1));
        it.o_save = take(4 * (size_t)std::max<size_t>(it.save.size(), 1));
        it.o_rates = take(8 * (size_t)(it.in.rates && it.in.rates_per_traj ? it.in.n_traj : 1) * std::max(p.R, 1));
        it.o_rdf = take(8 * (size_t)(it.in.rates && it.in.rates_per_traj ? it.in.n_traj : 1) * std::max(p.R, 1));
        it.o_fpk = take(4 * (size_t)std::max(p.R * p.P, 1));
        it.o_jsp = take(4 * (size_t)std::max(p.R * p.Q, 1));
        it.o_jd = take(8 * (size_t)std::max(p.R * p.Q, 1));
    }
    o_items = take(sizeof(SsaArgs) * std::max<size_t>(warp_items.size(), 1));
    o_start = take(8 * (warp_items.size() + 1));
    o_titems = take(sizeof(SsaArgs) * std::max<size_t>(thread_items.size(), 1));
    o_tunit = take(8 * (thread_items.size() + 1));
    in_bytes = off;
    // outputs
    for (Class &c : classes) {
        c.o_out = take(8 * (size_t)c.n_samples * c.n_save * c.n_traj);
        c.o_events = take(8 * (size_t)std::max<int64_t>(c.n_traj, 1));
    }
    for (int i : warp_items) {
        Item &it = items[i];
        it.o_out = take(8 * (size_t)(it.in.nb_steps + 1) * it.save.size() * it.in.n_traj);
        it.o_events = take(8 * (size_t)std::max<int64_t>(it.in.n_traj, 1));
    }
    for (int i : thread_items) {
        Item &it = items[i];
        it.o_out = take(8 * (size_t)(it.in.nb_steps + 1) * it.save.size() * it.in.n_traj);
        it.o_events = take(8 * (size_t)std::max<int64_t>(it.in.n_traj, 1));
    }
    o_work = take(8 * 4);
    total_bytes = off;
    if (!cuda_ok(cudaMallocHost(&host, total_bytes), "cudaMallocHost(batch staging)") ||
        !cuda_ok(cudaMalloc(&dev, total_bytes), "cudaMalloc(batch arena)"))
        return false;
    std::memset(host, 0, total_bytes);
    unsigned char *h = static_cast<unsigned char *>(host);
    unsigned char *d = static_cast<unsigned char *>(dev);

    // ---------------- static parts of the staging (sample grids, tables, item args)
    for (Class &c : classes) {
        const Item &it0 = items[c.items[0]];
        const std::vector<double> ts = sample_times(it0.in.tmax, it0.in.nb_steps);
        std::memcpy(h + c.o_times, ts.data(), 8 * ts.size());
        std::memcpy(h + c.o_save, it0.save.data(), 4 * it0.save.size());
    }
    warp_warps = 0;
    if (!warp_items.empty() || !thread_items.empty()) {
        SsaArgs la{};
        la.S = maxS;
        la.R = maxR;
        la.P = maxP;
        la.Q = maxQ;
        la.batch = reinterpret_cast<const SsaArgs *>(d + o_items);
        la.tbatch_S = maxTS;
        warp_warps = ssa_warp_warps(la, ctx->smem_optin);
        if (warp_warps < 1) {
            set_error("the largest network of the batch does not fit the warp kernel");
            return false;
        }
        int64_t *start = reinterpret_cast<int64_t *>(h + o_start);
        SsaArgs *args = reinterpret_cast<SsaArgs *>(h + o_items);
        int64_t acc = 0;
        for (size_t k = 0; k < warp_items.size(); k++) {
            Item &it = items[warp_items[k]];
            const Packed &p = it.packed;
            start[k] = acc;
            acc += it.in.n_traj;
            const std::vector<double> ts = sample_times(it.in.tmax, it.in.nb_steps);
            std::memcpy(h + it.o_times, ts.data(), 8 * ts.size());
            std::memcpy(h + it.o_save, it.save.data(), 4 * it.save.size());
            std::memcpy(h + it.o_fsp, p.fac_sp.data(), 4 * p.fac_sp.size());
            std::memcpy(h + it.o_ford, p.fac_ord.data(), 4 * p.fac_ord.size());
            std::memcpy(h + it.o_jsp, p.jmp_sp.data(), 4 * p.jmp_sp.size());
            std::memcpy(h + it.o_jd, p.jmp_d.data(), 8 * p.jmp_d.size());
            int mm = 0;
            for (int32_t r = 0; r < p.R; r++) {
                int s = 0;
                for (int32_t f = 0; f < p.P; f++) s += p.fac_ord[(size_t)r * p.P + f];
                mm = std::max(mm, s);
            }
            SsaArgs &x = args[k];
            x = SsaArgs{};
            x.S = p.S;
            x.R = p.R;
            x.P = p.P;
            x.Q = p.Q;
            x.macro_mode = p.macro_mode;
            x.rate = reinterpret_cast<const double *>(d + it.o_rates);
            x.fac_sp = reinterpret_cast<const int32_t *>(d + it.o_fsp);
            x.fac_ord = reinterpret_cast<const int32_t *>(d + it.o_ford);
            x.jmp_sp = reinterpret_cast<const int32_t *>(d + it.o_jsp);
            x.jmp_d = reinterpret_cast<const int64_t *>(d + it.o_jd);
            x.n_traj = it.in.n_traj;
            x.x0 = reinterpret_cast<const int64_t *>(d + it.o_x0);
            x.x0_stride = it.in.x0_per_traj ? p.S : 0;
            x.seeds = reinterpret_cast<const uint64_t *>(d + it.o_seeds);
            x.sample_t = reinterpret_cast<const double *>(d + it.o_times);
            x.n_samples = it.in.nb_steps + 1;
            x.save_idx = reinterpret_cast<const int32_t *>(d + it.o_save);
            x.n_save = (int32_t)it.save.size();
            x.out = reinterpret_cast<int64_t *>(d + it.o_out);
            x.events = reinterpret_cast<uint64_t *>(d + it.o_events);
            x.max_mults = mm;
            x.lm_rdf = reinterpret_cast<const float2 *>(d + it.o_rdf);
            x.lm_fac = reinterpret_cast<const int32_t *>(d + it.o_lfac);
            x.lm_shape = (mm <= 2 && p.S < 32767) ? reinterpret_cast<const uint32_t *>(d + it.o_shape) : nullptr;
            // lane-major factor and shape tables
            const int C = (p.R + 31) / 32, RP = 32 * C;
            int32_t *lf = reinterpret_cast<int32_t *>(h + it.o_lfac);
            uint32_t *sh = reinterpret_cast<uint32_t *>(h + it.o_shape);
            for (int q = 0; q < RP; q++) {
                const int i2 = q >> 5, l = q & 31, r = l * C + i2;
                for (int f = 0; f < p.P; f++)
                    lf[(i2 * p.P + f) * 32 + l] =
                        r < p.R ? (p.fac_sp[(size_t)r * p.P + f] | (p.fac_ord[(size_t)r * p.P + f] << 16)) : 0;
                sh[q] = r < p.R ? warp_shape_word(p.fac_sp.data(), p.fac_ord.data(), p.P, p.S, r)
                                : ((uint32_t)p.S << 16 | (uint32_t)p.S);
            }
        }
        start[warp_items.size()] = acc;
        // thread units: 32 trajectories of one item each
        int64_t *unit = reinterpret_cast<int64_t *>(h + o_tunit);
        SsaArgs *targs = reinterpret_cast<SsaArgs *>(h + o_titems);
        int64_t units = 0;
        for (size_t k = 0; k < thread_items.size(); k++) {
            Item &it = items[thread_items[k]];
            const Packed &p = it.packed;
            unit[k] = units;
            units += (it.in.n_traj + 31) / 32;
            const std::vector<double> ts = sample_times(it.in.tmax, it.in.nb_steps);
            std::memcpy(h + it.o_times, ts.data(), 8 * ts.size());
            std::memcpy(h + it.o_save, it.save.data(), 4 * it.save.size());
            int32_t *fpk = reinterpret_cast<int32_t *>(h + it.o_fpk);
            for (size_t f = 0; f < p.fac_sp.size(); f++) fpk[f] = p.fac_sp[f] | (p.fac_ord[f] << 16);
            std::memcpy(h + it.o_jsp, p.jmp_sp.data(), 4 * p.jmp_sp.size());
            std::memcpy(h + it.o_jd, p.jmp_d.data(), 8 * p.jmp_d.size());
            SsaArgs &x = targs[k];
            x = SsaArgs{};
            x.S = p.S;
            x.R = p.R;
            x.P = p.P;
            x.Q = p.Q;
            x.macro_mode = p.macro_mode;
            x.rate = reinterpret_cast<const double *>(d + it.o_rates);
            x.rate_stride = it.in.rates && it.in.rates_per_traj ? p.R : 0;
            x.fac_packed = reinterpret_cast<const int32_t *>(d + it.o_fpk);
            x.jmp_sp = reinterpret_cast<const int32_t *>(d + it.o_jsp);
            x.jmp_d = reinterpret_cast<const int64_t *>(d + it.o_jd);
            x.n_traj = it.in.n_traj;
            x.x0 = reinterpret_cast<const int64_t *>(d + it.o_x0);
            x.x0_stride = it.in.x0_per_traj ? p.S : 0;
            x.seeds = reinterpret_cast<const uint64_t *>(d + it.o_seeds);
            x.sample_t = reinterpret_cast<const double *>(d + it.o_times);
            x.n_samples = it.in.nb_steps + 1;
            x.save_idx = reinterpret_cast<const int32_t *>(d + it.o_save);
            x.n_save = (int32_t)it.save.size();
            x.out = reinterpret_cast<int64_t *>(d + it.o_out);
            x.events = reinterpret_cast<uint64_t *>(d + it.o_events);
            x.zig = ctx->zig;
            x.lm_rdf = reinterpret_cast<const float2 *>(d + it.o_rdf);
            x.budget_ns = kernel_budget_ns();
            for (int32_t r = 0; r < p.R; r++) {
                int m = 0;
                for (int32_t f = 0; f < p.P; f++) m += p.fac_ord[(size_t)r * p.P + f];
                x.max_mults = std::max(x.max_mults, m);
            }
        }
        unit[thread_items.size()] = units;
        warp_traj = acc;
        warp_args = SsaArgs{};
        warp_args.S = maxS;
        warp_args.R = maxR;
        warp_args.P = maxP;
        warp_args.Q = maxQ;
        warp_args.macro_mode = macro_mode;
        warp_args.n_traj = acc + units;
        warp_args.n_warp_tickets = acc;
        warp_args.batch = reinterpret_cast<const SsaArgs *>(d + o_items);
        warp_args.batch_start = reinterpret_cast<const int64_t *>(d + o_start);
        warp_args.batch_n = (int32_t)warp_items.size();
        warp_args.tbatch = reinterpret_cast<const SsaArgs *>(d + o_titems);
        warp_args.tbatch_unit = reinterpret_cast<const int64_t *>(d + o_tunit);
        warp_args.tbatch_n = (int32_t)thread_items.size();
        warp_args.tbatch_S = maxTS;
        warp_args.work = reinterpret_cast<unsigned long long *>(d + o_work);
        warp_args.zig = ctx->zig;
        warp_args.budget_ns = kernel_budget_ns();
        const int per_sm = std::max(1, ssa_warp_occupancy(warp_args, warp_warps, ssa_warp_smem(warp_args, warp_warps)));
        warp_grid = (int)std::max<int64_t>(
            1, std::min<int64_t>((acc + units + warp_warps - 1) / warp_warps, (int64_t)ctx->sm_count * per_sm));
        if (warp_cnt0) cudaFree(warp_cnt0);
        warp_cnt0 = nullptr;
        if (!cuda_ok(cudaMalloc(&warp_cnt0, 8 * (size_t)warp_grid * warp_warps * std::max(maxS, 1)),
                     "cudaMalloc(interval-start counts)"))
            return false;
        warp_args.warp_cnt0 = warp_cnt0;
    }

    // ---------------- every class's network on the device, kernels compiled
    for (Class &c : classes) {
        const Item &it0 = items[c.items[0]];
        std::lock_guard<std::mutex> lk(it0.net->mu);
        if (!ensure_device(*it0.net)) return false;
        if (c.kind == Class::Merged && jit_supported(it0.packed) && !jit_kernel(it0.packed, jit_block()))
            cudaGetLastError();  // the descriptor kernel runs instead
    }
    if (!cuda_ok(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "cudaEventCreate") ||
        !cuda_ok(cudaEventCreateWithFlags(&join, cudaEventDisableTiming), "cudaEventCreate") ||
        !cuda_ok(cudaEventCreate(&t0), "cudaEventCreate") || !cuda_ok(cudaEventCreate(&t1), "cudaEventCreate") ||
        !cuda_ok(cudaEventCreate(&e_in), "cudaEventCreate") || !cuda_ok(cudaEventCreate(&e_kern), "cudaEventCreate"))
        return false;

    // ---------------- capture: inputs in, kernels on two branches, results out
    if (!cuda_ok(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture")) return false;
    bool ok = cuda_ok(cudaMemcpyAsync(dev, host, in_bytes, cudaMemcpyHostToDevice, st), "cudaMemcpyAsync(in)");
    ok = ok && cuda_ok(cudaMemsetAsync(d + o_work, 0, 32, st), "cudaMemsetAsync");
    // external record nodes: the events record as plain timed events on replay
    ok = ok && cuda_ok(cudaEventRecordWithFlags(e_in, st, cudaEventRecordExternal), "cudaEventRecordWithFlags");
    ok = ok && cuda_ok(cudaEventRecord(fork, st), "cudaEventRecord") &&
         cuda_ok(cudaStreamWaitEvent(side, fork, 0), "cudaStreamWaitEvent");
    if (ok && (!warp_items.empty() || !thread_items.empty())) {
        const int err = launch_ssa_warp(warp_args, warp_warps, warp_grid, ssa_warp_smem(warp_args, warp_warps), side);
        ok = err == 0 || cuda_ok((cudaError_t)err, "warp batch launch");
    }
    for (Class &c : classes) {
        if (!ok) break;
        const Item &it0 = items[c.items[0]];
        RunDev r;
        r.n_traj = c.n_traj;
        r.x0 = reinterpret_cast<const int64_t *>(d + c.o_x0);
        r.seeds = reinterpret_cast<const uint64_t *>(d + c.o_seeds);
        r.sample_t = reinterpret_cast<const double *>(d + c.o_times);
        r.n_samples = c.n_samples;
        r.save_idx = reinterpret_cast<const int32_t *>(d + c.o_save);
        r.n_save = c.n_save;
        r.out = reinterpret_cast<int64_t *>(d + c.o_out);
        r.events = reinterpret_cast<uint64_t *>(d + c.o_events);
        r.times_ok = std::isfinite(it0.in.tmax) && it0.in.tmax >= 0;
        r.t_last = it0.in.tmax;
        if (c.kind == Class::Merged) {
            r.x0_stride = c.S;
            r.rates = reinterpret_cast<const double *>(d + c.o_rates);
            r.rate_stride = c.R;
        } else {
            r.x0_stride = it0.in.x0_per_traj ? c.S : 0;
            if (it0.in.rates) {
                r.rates = reinterpret_cast<const double *>(d + c.o_rates);
                r.rate_stride = it0.in.rates_per_traj ? c.R : 0;
            }
        }
        std::lock_guard<std::mutex> lk(it0.net->mu);
        int mapping = 0;
        ok = launch_sampled(*it0.net, *it0.net->dev, r, st, false, &mapping);
        for (int i : c.items) items[i].mapping = mapping;
        c.scratch = it0.net->dev->scratch;
    }
    ok = ok && cuda_ok(cudaEventRecord(join, side), "cudaEventRecord") &&
         cuda_ok(cudaStreamWaitEvent(st, join, 0), "cudaStreamWaitEvent");
    ok = ok && cuda_ok(cudaEventRecordWithFlags(e_kern, st, cudaEventRecordExternal), "cudaEventRecordWithFlags");
    ok = ok && cuda_ok(cudaMemcpyAsync(h + in_bytes, d + in_bytes, total_bytes - in_bytes, cudaMemcpyDeviceToHost, st),
                       "cudaMemcpyAsync(out)");
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (!ok || !cuda_ok(ce, "cudaStreamEndCapture")) {
        if (graph) cudaGraphDestroy(graph);
        return false;
    }
    const bool inst = cuda_ok(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
    cudaGraphDestroy(graph);
    return inst;
}

// Pack this run's inputs into the staging buffer.
void Batch::stage_inputs() {
    unsigned char *h = static_cast<unsigned char *>(host);
    for (Class &c : classes) {
        int64_t base = 0;
        for (int i : c.items) {
            const Item &it = items[i];
            const Packed &p = it.packed;
            const int64_t n = it.in.n_traj;
            std::memcpy(h + c.o_seeds + 8 * base, it.in.seeds, 8 * (size_t)n);
            if (c.kind == Class::Merged) {
                int64_t *x0 = reinterpret_cast<int64_t *>(h + c.o_x0) + base * p.S;
                double *rt = reinterpret_cast<double *>(h + c.o_rates) + base * p.R;
                for (int64_t k = 0; k < n; k++) {
                    std::memcpy(x0 + k * p.S, it.in.x0 + (it.in.x0_per_traj ? k * p.S : 0), 8 * (size_t)p.S);
                    const double *src = it.in.rates ? it.in.rates + (it.in.rates_per_traj ? k * p.R : 0) : p.rate.data();
                    std::memcpy(rt + k * p.R, src, 8 * (size_t)p.R);
                }
            } else {
                std::memcpy(h + c.o_x0, it.in.x0, 8 * (size_t)(it.in.x0_per_traj ? n : 1) * p.S);
                if (it.in.rates)
                    std::memcpy(h + c.o_rates, it.in.rates, 8 * (size_t)(it.in.rates_per_traj ? n : 1) * p.R);
            }
            base += n;
        }
    }
    for (int i : warp_items) {
        const Item &it = items[i];
        const Packed &p = it.packed;
        const int64_t n = it.in.n_traj;
        if (n == 0) continue;
        std::memcpy(h + it.o_x0, it.in.x0, 8 * (size_t)(it.in.x0_per_traj ? n : 1) * p.S);
        std::memcpy(h + it.o_seeds, it.in.seeds, 8 * (size_t)n);
        const double *rt = it.in.rates ? it.in.rates : p.rate.data();
        std::memcpy(h + it.o_rates, rt, 8 * (size_t)p.R);
        const int C = (p.R + 31) / 32, RP = 32 * C;
        float *rdf = reinterpret_cast<float *>(h + it.o_rdf);
        for (int q = 0; q < RP; q++) {
            const int r = (q & 31) * C + (q >> 5);
            float_pair(r < p.R ? rt[r] : 0.0, rdf + 2 * q);
        }
    }
    for (int i : thread_items) {
        const Item &it = items[i];
        const Packed &p = it.packed;
        const int64_t n = it.in.n_traj;
        if (n == 0) continue;
        std::memcpy(h + it.o_x0, it.in.x0, 8 * (size_t)(it.in.x0_per_traj ? n : 1) * p.S);
        std::memcpy(h + it.o_seeds, it.in.seeds, 8 * (size_t)n);
        const size_t nr = (size_t)(it.in.rates && it.in.rates_per_traj ? n : 1) * p.R;
        const double *rt = it.in.rates ? it.in.rates : p.rate.data();
        std::memcpy(h + it.o_rates, rt, 8 * nr);
        float *rdf = reinterpret_cast<float *>(h + it.o_rdf);
        for (size_t q = 0; q < nr; q++) float_pair(rt[q], rdf + 2 * q);
    }
}

namespace {

struct CopyTask {
    void *dst;
    const void *src;
    size_t bytes;
};

// Copy every task's bytes; above 64 MB in total the tasks are cut into 16 MB
// pieces shared out to up to 16 host threads (the page-locked staging buffer
// is read at the host's memory bandwidth, not at one core's copy rate).
void parallel_copy(const std::vector<CopyTask> &tasks) {
    size_t total = 0;
    for (const CopyTask &t : tasks) total += t.bytes;
    const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (total < ((size_t)64 << 20) || hw == 1) {
        for (const CopyTask &t : tasks)
            if (t.bytes) std::memcpy(t.dst, t.src, t.bytes);
        return;
    }
    constexpr size_t kPiece = (size_t)16 << 20;
    std::vector<CopyTask> pieces;
    for (const CopyTask &t : tasks)
        for (size_t o = 0; o < t.bytes; o += kPiece)
            pieces.push_back({static_cast<unsigned char *>(t.dst) + o, static_cast<const unsigned char *>(t.src) + o,
                              std::min(kPiece, t.bytes - o)});
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < pieces.size();) std::memcpy(pieces[i].dst, pieces[i].src, pieces[i].bytes);
    };
    std::vector<std::thread> th;
    for (unsigned k = 1; k < hw; ++k) th.emplace_back(work);
    work();
    for (std::thread &t : th) t.join();
}

}  // namespace

void Batch::unstage_outputs(uint64_t &events) {
    const unsigned char *h = static_cast<const unsigned char *>(host);
    events = 0;
    std::vector<CopyTask> tasks;
    for (Class &c : classes) {
        int64_t base = 0;
        const int64_t *out = reinterpret_cast<const int64_t *>(h + c.o_out);
        const uint64_t *ev = reinterpret_cast<const uint64_t *>(h + c.o_events);
        for (int i : c.items) {
            Item &it = items[i];
            const int64_t n = it.in.n_traj;
            // a merged class interleaves its items' rows: an item without an
            // output buffer gets the batch's own copy
            int64_t *dst = it.in.out;
            if (!dst) {
                it.own_out.resize((size_t)c.n_samples * c.n_save * n);
                dst = it.own_out.data();
            }
            for (int64_t s = 0; s < c.n_samples; s++)
                for (int32_t k = 0; k < c.n_save; k++)
                    tasks.push_back({dst + (s * c.n_save + k) * n, out + (s * c.n_save + k) * c.n_traj + base,
                                     8 * (size_t)n});
            for (int64_t k = 0; k < n; k++) events += ev[base + k];
            if (it.in.events) tasks.push_back({it.in.events, ev + base, 8 * (size_t)n});
            base += n;
        }
    }
    for (const std::vector<int> *list : {&warp_items, &thread_items})
    for (int i : *list) {
        const Item &it = items[i];
        const int64_t n = it.in.n_traj;
        const size_t ob = 8 * (size_t)(it.in.nb_steps + 1) * it.save.size() * n;
        if (it.in.out && ob) tasks.push_back({it.in.out, h + it.o_out, ob});
        const uint64_t *ev = reinterpret_cast<const uint64_t *>(h + it.o_events);
        for (int64_t k = 0; k < n; k++) events += ev[k];
        if (it.in.events) tasks.push_back({it.in.events, ev, 8 * (size_t)n});
    }
    parallel_copy(tasks);
}

bool Batch::item_results(int k, const int64_t **out, const uint64_t **events) const {
    if (k < 0 || k >= (int)items.size() || !host || !exec) return false;
    const Item &it = items[k];
    const unsigned char *h = static_cast<const unsigned char *>(host);
    for (const Class &c : classes) {
        int64_t base = 0;
        for (int i : c.items) {
            if (i == k) {
                *out = it.in.out ? it.in.out : it.own_out.data();
                *events = reinterpret_cast<const uint64_t *>(h + c.o_events) + base;
                return true;
            }
            base += items[i].in.n_traj;
        }
    }
    *out = it.in.out ? it.in.out : reinterpret_cast<const int64_t *>(h + it.o_out);
    *events = reinterpret_cast<const uint64_t *>(h + it.o_events);
    return true;
}

bool Batch::run(rb_stats_out &st_out) {
    for (const Item &it : items) {
        std::lock_guard<std::mutex> lk(it.net->mu);
        if (it.net->version != it.version) {
            set_error("a network of the batch changed after it was added");
            return false;
        }
    }
    DeviceCtx *ctx = device_ctx();
    if (!ctx) return false;
    if (!stream && !cuda_ok(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate"))
        return false;
    const bool first = !planned || !exec;
    if (!planned) plan();
    if (first && !build(stream)) return false;
    stage_inputs();
    if (!cuda_ok(cudaEventRecord(t0, stream), "cudaEventRecord") ||
        !cuda_ok(cudaGraphLaunch(exec, stream), "cudaGraphLaunch") ||
        !cuda_ok(cudaEventRecord(t1, stream), "cudaEventRecord") ||
        !cuda_ok(cudaStreamSynchronize(stream), "cudaStreamSynchronize"))
        return false;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, t1);
    if (cudaEventElapsedTime(&last_in_ms, t0, e_in) != cudaSuccess ||
        cudaEventElapsedTime(&last_kern_ms, e_in, e_kern) != cudaSuccess ||
        cudaEventElapsedTime(&last_out_ms, e_kern, t1) != cudaSuccess) {
        cudaGetLastError();
        last_in_ms = last_kern_ms = last_out_ms = -1.f;
    }
    // timeout flags of every launch
    unsigned long long flag = 0;
    const unsigned long long *wk =
        reinterpret_cast<const unsigned long long *>(static_cast<unsigned char *>(host) + o_work);
    flag |= warp_items.empty() && thread_items.empty() ? 0 : wk[2];
    for (Class &c : classes) {
        unsigned long long sc[4] = {0, 0, 0, 0};
        if (c.scratch && cudaMemcpy(sc, c.scratch, sizeof sc, cudaMemcpyDeviceToHost) == cudaSuccess) flag |= sc[2];
    }
    if (flag) {
        set_error("kernel time budget exceeded (RB_KERNEL_BUDGET_S)");
        st_out.timeout = true;
    }
    uint64_t events = 0;
    unstage_outputs(events);
    st_out.events = events;
    st_out.graph_ms = ms;
    st_out.h2d = in_bytes;
    st_out.d2h = total_bytes - in_bytes;
    st_out.launches = (int)classes.size() + (warp_items.empty() && thread_items.empty() ? 0 : 1);
    st_out.replayed = !first;
    return !flag;
}

void Batch::free_device() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    if (dev) cudaFree(dev);
    dev = nullptr;
    if (warp_cnt0) cudaFree(warp_cnt0);
    warp_cnt0 = nullptr;
    if (host) cudaFreeHost(host);
    host = nullptr;
    if (side) cudaStreamDestroy(side);
    side = nullptr;
    for (cudaEvent_t *e : {&fork, &join, &t0, &t1, &e_in, &e_kern})
        if (*e) {
            cudaEventDestroy(*e);
            *e = nullptr;
        }
}

Batch::~Batch() {
    free_device();
    if (stream) cudaStreamDestroy(stream);
}

}  // namespace rbg
