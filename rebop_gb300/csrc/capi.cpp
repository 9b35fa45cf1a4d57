// extern "C" entry points (include/rebop_gb300.h).
#include "rebop_gb300.h"

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <random>
#include <thread>

#include "engine.hpp"
#include "batch.hpp"
#include "ssa_jit.hpp"
#include "network.hpp"
#include "tune.hpp"

using rbg::set_error;

struct rb_network {
    rbg::Network net;
};

// The Rust API's Gillespie object: the network plus one trajectory's state
// (species, t and the 256-bit generator state), src/gillespie.rs:157-163.
struct rb_gillespie {
    rbg::Network net;
    std::vector<int64_t> species;
    double t = 0.0;
    uint64_t rng[4] = {0, 0, 0, 0};
    int32_t sparse = 0;
};

namespace {

// SmallRng::seed_from_u64: four SplitMix64 outputs (same construction as the
// device generator's seeding).
void splitmix_state(uint64_t seed, uint64_t st[4]) {
    uint64_t s = seed;
    for (int i = 0; i < 4; i++) {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        st[i] = z ^ (z >> 31);
    }
}

int fail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

bool cuda_check(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    return false;
}

size_t align16(size_t v) { return (v + 15) & ~(size_t)15; }

// Bump allocator over a DeviceNet's staging buffer.
struct Carve {
    size_t off = 0;
    template <class T>
    size_t take(size_t n) {
        size_t o = off;
        off = align16(off + sizeof(T) * std::max<size_t>(n, 1));
        return o;
    }
};

int check_save(const rbg::Network &net, const int32_t *save_idx, int32_t n_save, std::vector<int32_t> &save) {
    save.clear();
    if (n_save < 0 || !save_idx) {
        for (int32_t s = 0; s < net.n_species; s++) save.push_back(s);
        return RB_OK;
    }
    for (int32_t k = 0; k < n_save; k++) {
        if (save_idx[k] < 0 || save_idx[k] >= net.n_species)
            return fail(RB_ERR_INVALID, "save index " + std::to_string(save_idx[k]) + " out of range for " +
                                            std::to_string(net.n_species) + " species");
        save.push_back(save_idx[k]);
    }
    return RB_OK;
}

// One GPU advance of a single stateful trajectory (resume mode).
int single_advance(const rbg::Network &net, int64_t *species, double *t, uint64_t *rng, double tmax) {
    std::lock_guard<std::mutex> lk(net.mu);
    if (!rbg::ensure_device(net)) return RB_ERR_CUDA;
    rbg::DeviceNet &dn = *net.dev;
    const size_t S = (size_t)net.n_species;
    Carve c;
    size_t o_sp = c.take<int64_t>(S), o_t = c.take<double>(1), o_rng = c.take<uint64_t>(4);
    size_t o_samp = c.take<double>(1), o_save = c.take<int32_t>(S), o_out = c.take<int64_t>(S);
    size_t o_fsp = c.take<int64_t>(S), o_ft = c.take<double>(1), o_frng = c.take<uint64_t>(4);
    if (!rbg::ensure_io(dn, c.off)) return RB_ERR_NOMEM;
    unsigned char *b = static_cast<unsigned char *>(dn.io);
    std::vector<unsigned char> h(c.off, 0);
    if (S) std::memcpy(h.data() + o_sp, species, S * 8);
    std::memcpy(h.data() + o_t, t, 8);
    std::memcpy(h.data() + o_rng, rng, 32);
    std::memcpy(h.data() + o_samp, &tmax, 8);
    for (size_t s = 0; s < S; s++) {
        int32_t v = (int32_t)s;
        std::memcpy(h.data() + o_save + 4 * s, &v, 4);
    }
    if (!cuda_check(cudaMemcpyAsync(b, h.data(), o_out, cudaMemcpyHostToDevice, dn.stream), "cudaMemcpyAsync"))
        return RB_ERR_CUDA;
    rbg::RunDev r;
    r.n_traj = 1;
    r.in_species = reinterpret_cast<int64_t *>(b + o_sp);
    r.in_t = reinterpret_cast<double *>(b + o_t);
    r.in_rng = reinterpret_cast<uint64_t *>(b + o_rng);
    r.sample_t = reinterpret_cast<double *>(b + o_samp);
    r.n_samples = 1;
    r.save_idx = reinterpret_cast<int32_t *>(b + o_save);
    r.n_save = (int32_t)S;
    r.out = reinterpret_cast<int64_t *>(b + o_out);
    r.fin_species = reinterpret_cast<int64_t *>(b + o_fsp);
    r.fin_t = reinterpret_cast<double *>(b + o_ft);
    r.fin_rng = reinterpret_cast<uint64_t *>(b + o_frng);
    r.times_ok = std::isfinite(tmax) && tmax >= 0;
    r.t_last = tmax;
    if (!rbg::launch_sampled(net, dn, r, dn.stream, false, nullptr)) return RB_ERR_CUDA;
    unsigned long long flag = 0;
    if (!cuda_check(cudaMemcpyAsync(h.data() + o_fsp, b + o_fsp, c.off - o_fsp, cudaMemcpyDeviceToHost, dn.stream),
                    "cudaMemcpyAsync") ||
        !cuda_check(cudaMemcpyAsync(&flag, dn.scratch + 2, 8, cudaMemcpyDeviceToHost, dn.stream), "cudaMemcpyAsync") ||
        !cuda_check(cudaStreamSynchronize(dn.stream), "ssa_thread_kernel"))
        return RB_ERR_CUDA;
    if (flag) return fail(RB_ERR_TIMEOUT, "advance_until ran out of its time budget (RB_KERNEL_BUDGET_S)");
    if (S) std::memcpy(species, h.data() + o_fsp, S * 8);
    std::memcpy(t, h.data() + o_ft, 8);
    std::memcpy(rng, h.data() + o_frng, 32);
    return RB_OK;
}

// Every-event / one-step runs of single trajectories.
int events_run(const rbg::Network &net, int64_t *species, double *t, uint64_t *rng, double tmax, int gate,
               int64_t max_steps, int record_initial, const std::vector<int32_t> &save, double *times,
               int64_t *out, int64_t cap, int64_t *n_records) {
    std::lock_guard<std::mutex> lk(net.mu);
    if (!rbg::ensure_device(net)) return RB_ERR_CUDA;
    rbg::DeviceCtx *ctx = rbg::device_ctx();
    if (!ctx) return RB_ERR_CUDA;
    rbg::DeviceNet &dn = *net.dev;
    const size_t S = (size_t)net.n_species, NS = save.size(), K = (size_t)std::max<int64_t>(cap, 0);
    Carve c;
    size_t o_sp = c.take<int64_t>(S), o_t = c.take<double>(1), o_rng = c.take<uint64_t>(4);
    size_t o_save = c.take<int32_t>(NS), o_rt = c.take<double>(K), o_ro = c.take<int64_t>(K * NS);
    size_t o_n = c.take<int64_t>(1);
    if (!rbg::ensure_io(dn, c.off)) return RB_ERR_NOMEM;
    unsigned char *b = static_cast<unsigned char *>(dn.io);
    std::vector<unsigned char> h(o_rt, 0);
    if (S) std::memcpy(h.data() + o_sp, species, S * 8);
    std::memcpy(h.data() + o_t, t, 8);
    std::memcpy(h.data() + o_rng, rng, 32);
    if (NS) std::memcpy(h.data() + o_save, save.data(), NS * 4);
    if (!cuda_check(cudaMemcpyAsync(b, h.data(), o_rt, cudaMemcpyHostToDevice, dn.stream), "cudaMemcpyAsync"))
        return RB_ERR_CUDA;
    const rbg::Packed &p = dn.packed;
    rbg::EventArgs a{};
    a.S = p.S;
    a.R = p.R;
    a.P = p.P;
    a.Q = p.Q;
    a.macro_mode = p.macro_mode;
    a.rate = dn.rate;
    a.fac_sp = dn.fac_sp;
    a.fac_ord = dn.fac_ord;
    a.jmp_sp = dn.jmp_sp;
    a.jmp_d = dn.jmp_d;
    a.ex_off = dn.ex_off;
    a.ex_code = dn.ex_code;
    a.ex_const = dn.ex_const;
    a.n_traj = 1;
    a.species = reinterpret_cast<int64_t *>(b + o_sp);
    a.t = reinterpret_cast<double *>(b + o_t);
    a.rng = reinterpret_cast<uint64_t *>(b + o_rng);
    a.tmax = tmax;
    a.gate = gate;
    a.max_steps = max_steps;
    a.record_initial = record_initial;
    a.save_idx = reinterpret_cast<int32_t *>(b + o_save);
    a.n_save = (int32_t)NS;
    a.cap = (int64_t)K;
    a.rec_t = reinterpret_cast<double *>(b + o_rt);
    a.rec_out = reinterpret_cast<int64_t *>(b + o_ro);
    a.n_rec = reinterpret_cast<int64_t *>(b + o_n);
    a.zig = ctx->zig;
    a.flag = dn.scratch + 2;
    a.budget_ns = rbg::kernel_budget_ns();
    if (!cuda_check(cudaMemsetAsync(dn.scratch, 0, 4 * sizeof(unsigned long long), dn.stream), "cudaMemsetAsync"))
        return RB_ERR_CUDA;
    int err = rbg::launch_ssa_events(a, dn.stream);
    if (err) return cuda_check((cudaError_t)err, "ssa_events_kernel launch") ? RB_OK : RB_ERR_CUDA;
    int64_t n = 0;
    unsigned long long flag = 0;
    std::vector<unsigned char> st(o_save, 0);
    if (!cuda_check(cudaMemcpyAsync(st.data(), b, o_save, cudaMemcpyDeviceToHost, dn.stream), "cudaMemcpyAsync") ||
        !cuda_check(cudaMemcpyAsync(&n, b + o_n, 8, cudaMemcpyDeviceToHost, dn.stream), "cudaMemcpyAsync") ||
        !cuda_check(cudaMemcpyAsync(&flag, dn.scratch + 2, 8, cudaMemcpyDeviceToHost, dn.stream), "cudaMemcpyAsync") ||
        !cuda_check(cudaStreamSynchronize(dn.stream), "ssa_events_kernel"))
        return RB_ERR_CUDA;
    if (flag) return fail(RB_ERR_TIMEOUT, "every-event run ran out of its time budget (RB_KERNEL_BUDGET_S)");
    int64_t kept = std::min<int64_t>(n, (int64_t)K);
    if (kept > 0 && times &&
        !cuda_check(cudaMemcpy(times, b + o_rt, (size_t)kept * 8, cudaMemcpyDeviceToHost), "cudaMemcpy"))
        return RB_ERR_CUDA;
    if (kept > 0 && out && NS &&
        !cuda_check(cudaMemcpy(out, b + o_ro, (size_t)kept * NS * 8, cudaMemcpyDeviceToHost), "cudaMemcpy"))
        return RB_ERR_CUDA;
    if (S) std::memcpy(species, st.data() + o_sp, S * 8);
    std::memcpy(t, st.data() + o_t, 8);
    std::memcpy(rng, st.data() + o_rng, 32);
    if (n_records) *n_records = n;
    return RB_OK;
}

}  // namespace

extern "C" {

const char *rb_version(void) { return "0.1.0"; }

size_t rb_last_error(char *buf, size_t len) {
    const std::string &e = rbg::last_error();
    if (buf && len > 0) {
        size_t n = std::min(len - 1, e.size());
        std::memcpy(buf, e.data(), n);
        buf[n] = '\0';
    }
    return e.size();
}

// ----------------------------------------------------------------- network
int rb_network_create(int32_t n_species, rb_network **out) {
    if (!out) return fail(RB_ERR_INVALID, "null output pointer");
    if (n_species < 0) return fail(RB_ERR_INVALID, "negative number of species");
    auto *n = new (std::nothrow) rb_network();
    if (!n) return fail(RB_ERR_NOMEM, "out of host memory");
    n->net.n_species = n_species;
    for (int32_t s = 0; s < n_species; s++) n->net.species_names.push_back("x" + std::to_string(s));
    *out = n;
    return RB_OK;
}

void rb_network_destroy(rb_network *net) { delete net; }

int32_t rb_network_nb_species(const rb_network *net) { return net ? net->net.n_species : -1; }
int32_t rb_network_nb_reactions(const rb_network *net) { return net ? (int32_t)net->net.reactions.size() : -1; }

int rb_network_add_reaction_lma(rb_network *net, double rate, const uint32_t *exponents, int32_t n_exponents,
                                const int64_t *differences, int32_t n_differences) {
    if (!net) return fail(RB_ERR_INVALID, "null network");
    std::lock_guard<std::mutex> lk(net->net.mu);
    std::string e = net->net.add_lma(rate, exponents, n_exponents, differences, n_differences);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

int rb_network_add_reaction_lma_sparse(rb_network *net, double rate, const uint32_t *species,
                                       const uint32_t *exponents, int32_t n_pairs, const int64_t *differences,
                                       int32_t n_differences) {
    if (!net) return fail(RB_ERR_INVALID, "null network");
    std::lock_guard<std::mutex> lk(net->net.mu);
    std::string e = net->net.add_lma_sparse(rate, species, exponents, n_pairs, differences, n_differences);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

int rb_network_add_reaction_expr(rb_network *net, const int32_t *code, int32_t n_code, const double *consts,
                                 int32_t n_consts, const int64_t *differences, int32_t n_differences) {
    if (!net) return fail(RB_ERR_INVALID, "null network");
    std::lock_guard<std::mutex> lk(net->net.mu);
    std::string e = net->net.add_expr(code, n_code, consts, n_consts, differences, n_differences);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

int rb_network_from_dsl(const char *text, rb_network **out) {
    if (!text || !out) return fail(RB_ERR_INVALID, "null argument");
    auto *n = new (std::nothrow) rb_network();
    if (!n) return fail(RB_ERR_NOMEM, "out of host memory");
    std::string e = rbg::parse_dsl(text, n->net);
    if (!e.empty()) {
        delete n;
        return fail(RB_ERR_PARSE, e);
    }
    *out = n;
    return RB_OK;
}

int rb_network_set_param(rb_network *net, const char *name, double value) {
    if (!net || !name) return fail(RB_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(net->net.mu);
    std::string e = net->net.set_param(name, value);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

int32_t rb_network_nb_params(const rb_network *net) { return net ? (int32_t)net->net.param_names.size() : -1; }

static int copy_name(const std::string &s, char *buf, size_t len) {
    if (!buf || len == 0) return fail(RB_ERR_INVALID, "null buffer");
    size_t n = std::min(len - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
    return s.size() < len ? RB_OK : fail(RB_ERR_INVALID, "buffer too small");
}

int rb_network_param_name(const rb_network *net, int32_t idx, char *buf, size_t len) {
    if (!net || idx < 0 || idx >= (int32_t)net->net.param_names.size())
        return fail(RB_ERR_INVALID, "parameter index out of range");
    return copy_name(net->net.param_names[idx], buf, len);
}

int rb_network_species_name(const rb_network *net, int32_t idx, char *buf, size_t len) {
    if (!net || idx < 0 || idx >= net->net.n_species) return fail(RB_ERR_INVALID, "species index out of range");
    return copy_name(net->net.species_names[idx], buf, len);
}

int rb_network_name(const rb_network *net, char *buf, size_t len) {
    if (!net) return fail(RB_ERR_INVALID, "null network");
    return copy_name(net->net.name, buf, len);
}

int rb_network_reaction_rate(const rb_network *net, int32_t r, double *rate) {
    if (!net || !rate || r < 0 || r >= (int32_t)net->net.reactions.size())
        return fail(RB_ERR_INVALID, "reaction index out of range");
    *rate = net->net.reactions[r].rate;
    return RB_OK;
}

// ---------------------------------------------------------------- ensemble
// Device address of a page-locked host buffer, or null for any other memory.
static void *mapped_host(void *h) {
    if (!h) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int rb_ensemble_run(const rb_network *netp, int64_t n_traj, const int64_t *x0, int32_t x0_per_traj,
                    const double *rates, int32_t rates_per_traj, const uint64_t *seeds, double tmax,
                    int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *out, double *times,
                    uint64_t *events, int64_t *final_species, rb_run_stats *stats) {
    auto wall0 = std::chrono::steady_clock::now();
    if (!netp) return fail(RB_ERR_INVALID, "null network");
    const rbg::Network &net = netp->net;
    if (n_traj < 0) return fail(RB_ERR_INVALID, "negative number of trajectories");
    if (nb_steps < 1) return fail(RB_ERR_INVALID, "nb_steps must be >= 1 (use rb_run_all_events for 0)");
    std::vector<int32_t> save;
    int rc = check_save(net, save_idx, n_save, save);
    if (rc) return rc;
    const size_t S = (size_t)net.n_species, NS = save.size(), N = (size_t)n_traj;
    const size_t NT = (size_t)nb_steps + 1;
    if (N && S && !x0) return fail(RB_ERR_INVALID, "null x0");
    if (N && !seeds) return fail(RB_ERR_INVALID, "null seeds");
    if (N && NS && !out) return fail(RB_ERR_INVALID, "null out");
    std::vector<double> st = rbg::sample_times(tmax, nb_steps);
    if (times) std::memcpy(times, st.data(), NT * 8);
    std::lock_guard<std::mutex> lk(net.mu);
    if (!rbg::ensure_device(net)) return RB_ERR_CUDA;
    rbg::DeviceNet &dn = *net.dev;
    const size_t R = (size_t)dn.packed.R;
    const size_t n_x0 = x0_per_traj ? N : 1;
    const size_t n_rates = rates ? (rates_per_traj ? N : 1) : 0;
    Carve c;
    size_t o_x0 = c.take<int64_t>(n_x0 * S), o_rates = c.take<double>(n_rates * R), o_seed = c.take<uint64_t>(N);
    size_t o_st = c.take<double>(NT), o_save = c.take<int32_t>(NS), o_out = c.take<int64_t>(NT * NS * N);
    size_t o_ev = c.take<uint64_t>(N), o_fin = c.take<int64_t>(final_species ? N * S : 0);
    size_t o_rows = c.take<uint32_t>(NT);
    if (!rbg::ensure_io(dn, c.off)) return RB_ERR_NOMEM;
    unsigned char *b = static_cast<unsigned char *>(dn.io);
    uint64_t h2d = 0, d2h = 0;
    auto h2d_copy = [&](size_t off, const void *src, size_t bytes) {
        if (!bytes) return true;
        h2d += bytes;
        return cuda_check(cudaMemcpyAsync(b + off, src, bytes, cudaMemcpyHostToDevice, dn.stream), "cudaMemcpyAsync");
    };
    if (!h2d_copy(o_x0, x0, n_x0 * S * 8) || !h2d_copy(o_rates, rates, n_rates * R * 8) ||
        !h2d_copy(o_seed, seeds, N * 8) || !h2d_copy(o_st, st.data(), NT * 8) ||
        !h2d_copy(o_save, save.data(), NS * 4))
        return RB_ERR_CUDA;
    rbg::RunDev r;
    r.n_traj = n_traj;
    r.x0 = reinterpret_cast<int64_t *>(b + o_x0);
    r.x0_stride = x0_per_traj ? (int64_t)S : 0;
    r.rates = rates ? reinterpret_cast<double *>(b + o_rates) : nullptr;
    r.rate_stride = rates && rates_per_traj ? (int64_t)R : 0;
    r.seeds = reinterpret_cast<uint64_t *>(b + o_seed);
    r.sample_t = reinterpret_cast<double *>(b + o_st);
    r.n_samples = (int64_t)NT;
    r.save_idx = reinterpret_cast<int32_t *>(b + o_save);
    r.n_save = (int32_t)NS;
    // Page-locked result buffers can be written by the kernel itself, over
    // the host link, while it runs.  That pays when the samples trickle out
    // (a few GB/s at most: the kernel's scattered 8-byte stores then cost
    // nothing), while a launch that writes faster runs better against device
    // memory and one copy back at the end; the network's previous run
    // decides (RB_ZERO_COPY=1 always, 0 never).
    const char *zc = std::getenv("RB_ZERO_COPY");
    const bool zero_copy = zc ? std::strcmp(zc, "0") != 0 : dn.out_gbs > 0 && dn.out_gbs < 4.0;
    int64_t *out_host = zero_copy ? static_cast<int64_t *>(mapped_host(out)) : nullptr;
    uint64_t *ev_host = zero_copy ? static_cast<uint64_t *>(mapped_host(events)) : nullptr;
    r.out = out_host ? out_host : reinterpret_cast<int64_t *>(b + o_out);
    r.events = ev_host ? ev_host : reinterpret_cast<uint64_t *>(b + o_ev);
    r.fin_species = final_species ? reinterpret_cast<int64_t *>(b + o_fin) : nullptr;
    r.times_ok = std::isfinite(tmax) && tmax >= 0;
    r.t_last = tmax;
    // Sample rows stream back while the kernel runs: the speculative kernels
    // count, per row, the trajectories whose samples are written (after a
    // fence), and rows every trajectory has written are copied on a second
    // stream; the rest follow the kernel.
    const char *srows = std::getenv("RB_STREAM_ROWS");  // 0: copy every row after the kernel
    const bool stream_rows = !out_host && N && NS && NT < 65536 && !(srows && std::strcmp(srows, "0") == 0);
    unsigned int *row_done = reinterpret_cast<unsigned int *>(b + o_rows);
    if (stream_rows) {
        r.row_done = row_done;
        if (!cuda_check(cudaMemsetAsync(row_done, 0, NT * 4, dn.stream), "cudaMemsetAsync")) return RB_ERR_CUDA;
        if (dn.pin_rows_n < NT) {
            if (dn.pin_rows) cudaFreeHost(dn.pin_rows);
            dn.pin_rows = nullptr;
            dn.pin_rows_n = 0;
            if (!cuda_check(cudaHostAlloc(reinterpret_cast<void **>(&dn.pin_rows), NT * 4, cudaHostAllocDefault),
                            "cudaHostAlloc"))
                return RB_ERR_NOMEM;
            dn.pin_rows_n = NT;
        }
    }
    int mapping = 0;
    if (!rbg::launch_sampled(net, dn, r, dn.stream, true, &mapping)) return RB_ERR_CUDA;
    if (out_host) d2h += NT * NS * N * 8;
    if (ev_host) d2h += N * 8;
    auto d2h_copy = [&](void *dst, size_t off, size_t bytes) {
        if (!bytes || !dst) return true;
        d2h += bytes;
        return cuda_check(cudaMemcpyAsync(dst, b + off, bytes, cudaMemcpyDeviceToHost, dn.stream), "cudaMemcpyAsync");
    };
    // only the speculative kernels (mappings 3, 4) count rows
    const bool streaming = stream_rows && (mapping == 3 || mapping == 4);
    size_t rows_copied = 0;
    if (streaming) {
        const size_t row_bytes = NS * N * 8;
        char *hout = reinterpret_cast<char *>(out);
        while (rows_copied < NT) {
            // the kernel's end first: once it is over every row is final
            const cudaError_t q = cudaEventQuery(dn.ev_stop);
            if (q != cudaSuccess && q != cudaErrorNotReady) {
                cuda_check(q, "SSA kernel");
                return RB_ERR_CUDA;
            }
            size_t k = rows_copied;
            if (q == cudaSuccess) {
                k = NT;
            } else {
                if (!cuda_check(cudaMemcpyAsync(dn.pin_rows, row_done, NT * 4, cudaMemcpyDeviceToHost, dn.copy_stream),
                                "cudaMemcpyAsync") ||
                    !cuda_check(cudaStreamSynchronize(dn.copy_stream), "cudaStreamSynchronize"))
                    return RB_ERR_CUDA;
                while (k < NT && dn.pin_rows[k] >= (unsigned int)N) ++k;
            }
            if (k > rows_copied) {
                cudaStream_t cs = q == cudaSuccess ? dn.stream : dn.copy_stream;
                if (!cuda_check(cudaMemcpyAsync(hout + rows_copied * row_bytes, b + o_out + rows_copied * row_bytes,
                                                (k - rows_copied) * row_bytes, cudaMemcpyDeviceToHost, cs),
                                "cudaMemcpyAsync"))
                    return RB_ERR_CUDA;
                d2h += (k - rows_copied) * row_bytes;
                rows_copied = k;
            } else {
                std::this_thread::sleep_for(std::chrono::microseconds(50));
            }
        }
    }
    unsigned long long sc[3] = {0, 0, 0};  // total events, timeout flag, exact re-runs
    if ((!out_host && !streaming && !d2h_copy(out, o_out, NT * NS * N * 8)) ||
        (!ev_host && !d2h_copy(events, o_ev, N * 8)) ||
        !d2h_copy(final_species, o_fin, final_species ? N * S * 8 : 0) ||
        !cuda_check(cudaMemcpyAsync(sc, dn.scratch + 1, 24, cudaMemcpyDeviceToHost, dn.stream), "cudaMemcpyAsync") ||
        !cuda_check(cudaStreamSynchronize(dn.stream), "ssa_thread_kernel") ||
        (streaming && !cuda_check(cudaStreamSynchronize(dn.copy_stream), "cudaStreamSynchronize")))
        return RB_ERR_CUDA;
    if (sc[1]) return fail(RB_ERR_TIMEOUT, "ensemble run ran out of its time budget (RB_KERNEL_BUDGET_S)");
    const uint64_t total_events = sc[0];
    float ms = 0.f;
    if (N) cudaEventElapsedTime(&ms, dn.ev_start, dn.ev_stop);
    if (ms > 0.f) dn.out_gbs = (double)(NT * NS * N * 8) / ((double)ms * 1e6);
    if (stats) {
        stats->events = total_events;
        stats->kernel_ms = ms;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h + 24;
        stats->exact_reruns = sc[2];
        stats->kernel_launches = N ? 1 : 0;
        stats->mapping = mapping;
    }
    return RB_OK;
}

int rb_ensemble_run_device(const rb_network *netp, int64_t n_traj, const int64_t *d_x0, int32_t x0_per_traj,
                           const double *d_rates, int32_t rates_per_traj, const uint64_t *d_seeds, double tmax,
                           int64_t nb_steps, const int32_t *save_idx, int32_t n_save, int64_t *d_out,
                           uint64_t *d_events, int64_t *d_final_species, void *stream) {
    if (!netp) return fail(RB_ERR_INVALID, "null network");
    const rbg::Network &net = netp->net;
    if (n_traj < 0) return fail(RB_ERR_INVALID, "negative number of trajectories");
    if (nb_steps < 1) return fail(RB_ERR_INVALID, "nb_steps must be >= 1");
    std::vector<int32_t> save;
    int rc = check_save(net, save_idx, n_save, save);
    if (rc) return rc;
    const size_t S = (size_t)net.n_species, NS = save.size(), NT = (size_t)nb_steps + 1;
    if (n_traj && S && !d_x0) return fail(RB_ERR_INVALID, "null x0");
    if (n_traj && !d_seeds) return fail(RB_ERR_INVALID, "null seeds");
    if (n_traj && NS && !d_out) return fail(RB_ERR_INVALID, "null out");
    std::lock_guard<std::mutex> lk(net.mu);
    if (!rbg::ensure_device(net)) return RB_ERR_CUDA;
    rbg::DeviceNet &dn = *net.dev;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // Sample times and saved indices live in the network's staging buffer;
    // the previous run that may still read them is waited for first.
    std::vector<double> st = rbg::sample_times(tmax, nb_steps);
    Carve c;
    size_t o_st = c.take<double>(NT), o_save = c.take<int32_t>(NS);
    if (dn.last_stream && !cuda_check(cudaStreamSynchronize(dn.last_stream), "cudaStreamSynchronize"))
        return RB_ERR_CUDA;
    if (!rbg::ensure_io(dn, c.off)) return RB_ERR_NOMEM;
    unsigned char *b = static_cast<unsigned char *>(dn.io);
    if (!cuda_check(cudaMemcpyAsync(b + o_st, st.data(), NT * 8, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync") ||
        (NS && !cuda_check(cudaMemcpyAsync(b + o_save, save.data(), NS * 4, cudaMemcpyHostToDevice, s),
                           "cudaMemcpyAsync")))
        return RB_ERR_CUDA;
    rbg::RunDev r;
    r.n_traj = n_traj;
    r.x0 = d_x0;
    r.x0_stride = x0_per_traj ? (int64_t)S : 0;
    r.rates = d_rates;
    r.rate_stride = d_rates && rates_per_traj ? (int64_t)dn.packed.R : 0;
    r.seeds = d_seeds;
    r.sample_t = reinterpret_cast<double *>(b + o_st);
    r.n_samples = (int64_t)NT;
    r.save_idx = reinterpret_cast<int32_t *>(b + o_save);
    r.n_save = (int32_t)NS;
    r.out = d_out;
    r.events = d_events;
    r.fin_species = d_final_species;
    r.times_ok = std::isfinite(tmax) && tmax >= 0;
    r.t_last = tmax;
    if (!rbg::launch_sampled(net, dn, r, s, false, nullptr)) return RB_ERR_CUDA;
    dn.last_stream = s;
    return RB_OK;
}

int rb_ensemble_run_device_noalloc(const rb_network *netp, int64_t n_traj, const int64_t *d_x0, int32_t x0_per_traj,
                                   const double *d_rates, int32_t rates_per_traj, const uint64_t *d_seeds,
                                   double tmax, int64_t nb_steps, const int32_t *save_idx, int32_t n_save,
                                   int64_t *d_out, uint64_t *d_events, uint64_t *d_status, void *stream) {
    if (!netp) return fail(RB_ERR_INVALID, "null network");
    std::lock_guard<std::mutex> lk(netp->net.mu);
    std::string err;
    int rc = rbg::noalloc_ensemble_run(netp->net, n_traj, d_x0, x0_per_traj, d_rates, rates_per_traj, d_seeds, tmax,
                                       nb_steps, save_idx, n_save, d_out, d_events, d_status, stream, err);
    if (rc == 0) return RB_OK;
    return fail(rc == 1 ? RB_ERR_INVALID : rc == 5 ? RB_ERR_UNSUPPORTED : RB_ERR_CUDA, err);
}

int rb_ensemble_last_events(const rb_network *netp, uint64_t *events) {
    if (!netp || !events) return fail(RB_ERR_INVALID, "null argument");
    const rbg::Network &net = netp->net;
    std::lock_guard<std::mutex> lk(net.mu);
    if (!net.dev) return fail(RB_ERR_INVALID, "no run on this network yet");
    rbg::DeviceNet &dn = *net.dev;
    unsigned long long sc[2] = {0, 0};
    if (!cuda_check(cudaStreamSynchronize(dn.last_stream), "cudaStreamSynchronize") ||
        !cuda_check(cudaMemcpy(sc, dn.scratch + 1, 16, cudaMemcpyDeviceToHost), "cudaMemcpy"))
        return RB_ERR_CUDA;
    *events = sc[0];
    if (sc[1]) return fail(RB_ERR_TIMEOUT, "ensemble run ran out of its time budget (RB_KERNEL_BUDGET_S)");
    return RB_OK;
}

int rb_run_all_events(const rb_network *netp, const int64_t *x0, uint64_t seed, double tmax,
                      const int32_t *save_idx, int32_t n_save, double *times, int64_t *out, int64_t cap,
                      int64_t *n_records) {
    if (!netp) return fail(RB_ERR_INVALID, "null network");
    const rbg::Network &net = netp->net;
    std::vector<int32_t> save;
    int rc = check_save(net, save_idx, n_save, save);
    if (rc) return rc;
    if (net.n_species && !x0) return fail(RB_ERR_INVALID, "null x0");
    if (cap < 0) return fail(RB_ERR_INVALID, "negative capacity");
    std::vector<int64_t> sp(x0, x0 + net.n_species);
    double t = 0.0;
    uint64_t rng[4];
    splitmix_state(seed, rng);
    return events_run(net, sp.data(), &t, rng, tmax, 1, -1, 1, save, times, out, cap, n_records);
}

// ------------------------------------------------------ single trajectory
int rb_gillespie_new_with_seed(const int64_t *species, int32_t n_species, int32_t sparse, uint64_t seed,
                               rb_gillespie **out) {
    if (!out) return fail(RB_ERR_INVALID, "null output pointer");
    if (n_species < 0 || (n_species > 0 && !species)) return fail(RB_ERR_INVALID, "bad species array");
    auto *g = new (std::nothrow) rb_gillespie();
    if (!g) return fail(RB_ERR_NOMEM, "out of host memory");
    g->net.n_species = n_species;
    for (int32_t s = 0; s < n_species; s++) g->net.species_names.push_back("x" + std::to_string(s));
    g->species.assign(species, species + n_species);
    g->sparse = sparse;
    splitmix_state(seed, g->rng);
    *out = g;
    return RB_OK;
}

int rb_gillespie_new(const int64_t *species, int32_t n_species, int32_t sparse, rb_gillespie **out) {
    std::random_device rd;
    uint64_t seed = ((uint64_t)rd() << 32) ^ (uint64_t)rd();
    return rb_gillespie_new_with_seed(species, n_species, sparse, seed, out);
}

void rb_gillespie_free(rb_gillespie *g) { delete g; }

int rb_gillespie_seed(rb_gillespie *g, uint64_t seed) {
    if (!g) return fail(RB_ERR_INVALID, "null handle");
    splitmix_state(seed, g->rng);
    return RB_OK;
}

int32_t rb_gillespie_nb_species(const rb_gillespie *g) { return g ? (int32_t)g->species.size() : -1; }
int32_t rb_gillespie_nb_reactions(const rb_gillespie *g) { return g ? (int32_t)g->net.reactions.size() : -1; }

int rb_gillespie_add_reaction_lma(rb_gillespie *g, double rate, const uint32_t *exponents, int32_t n_exponents,
                                  const int64_t *differences, int32_t n_differences) {
    if (!g) return fail(RB_ERR_INVALID, "null handle");
    std::lock_guard<std::mutex> lk(g->net.mu);
    std::string e = g->net.add_lma(rate, exponents, n_exponents, differences, n_differences);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

int rb_gillespie_add_reaction_lma_sparse(rb_gillespie *g, double rate, const uint32_t *species,
                                         const uint32_t *exponents, int32_t n_pairs, const int64_t *differences,
                                         int32_t n_differences) {
    if (!g) return fail(RB_ERR_INVALID, "null handle");
    std::lock_guard<std::mutex> lk(g->net.mu);
    std::string e = g->net.add_lma_sparse(rate, species, exponents, n_pairs, differences, n_differences);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

int rb_gillespie_add_reaction_expr(rb_gillespie *g, const int32_t *code, int32_t n_code, const double *consts,
                                   int32_t n_consts, const int64_t *differences, int32_t n_differences) {
    if (!g) return fail(RB_ERR_INVALID, "null handle");
    std::lock_guard<std::mutex> lk(g->net.mu);
    std::string e = g->net.add_expr(code, n_code, consts, n_consts, differences, n_differences);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

double rb_gillespie_get_time(const rb_gillespie *g) { return g ? g->t : NAN; }
void rb_gillespie_set_time(rb_gillespie *g, double t) {
    if (g) g->t = t;
}

int rb_gillespie_get_species(const rb_gillespie *g, int32_t s, int64_t *value) {
    if (!g || !value) return fail(RB_ERR_INVALID, "null argument");
    if (s < 0 || s >= (int32_t)g->species.size())
        return fail(RB_ERR_INVALID, "index out of bounds: the len is " + std::to_string(g->species.size()) +
                                        " but the index is " + std::to_string(s));
    *value = g->species[s];
    return RB_OK;
}

int rb_gillespie_set_species(rb_gillespie *g, const int64_t *species, int32_t n) {
    if (!g) return fail(RB_ERR_INVALID, "null handle");
    if (n != (int32_t)g->species.size())
        return fail(RB_ERR_INVALID, "assertion failed: species length " + std::to_string(n) +
                                        " != number of species " + std::to_string(g->species.size()));
    if (n && !species) return fail(RB_ERR_INVALID, "null species");
    g->species.assign(species, species + n);
    return RB_OK;
}

int rb_gillespie_advance_until(rb_gillespie *g, double tmax) {
    if (!g) return fail(RB_ERR_INVALID, "null handle");
    return single_advance(g->net, g->species.data(), &g->t, g->rng, tmax);
}

int rb_gillespie_advance_one_reaction(rb_gillespie *g) {
    if (!g) return fail(RB_ERR_INVALID, "null handle");
    std::vector<int32_t> none;
    return events_run(g->net, g->species.data(), &g->t, g->rng, 0.0, 0, 1, 0, none, nullptr, nullptr, 0, nullptr);
}

int rb_trajectory_advance_until(const rb_network *net, int64_t *species, double *t, uint64_t *rng_state,
                                double tmax) {
    if (!net || !t || !rng_state || (net->net.n_species && !species)) return fail(RB_ERR_INVALID, "null argument");
    return single_advance(net->net, species, t, rng_state, tmax);
}

void rb_rng_state_from_seed(uint64_t seed, uint64_t *state) {
    if (state) splitmix_state(seed, state);
}

// Test hook (not part of the public header): the Exp1 ziggurat tables the
// device copy is made from.
void rbg_internal_zig_tables(double *x, double *f) { rbg::zig_tables_host(x, f); }

// Test hooks: the generated source of a network's kernel, and its compilation
// by NVRTC (no GPU needed).  Return RB_ERR_UNSUPPORTED when the generator does
// not cover the network.
int rbg_internal_jit_source(const rb_network *net, char *buf, size_t len) {
    if (!net) return fail(RB_ERR_INVALID, "null network");
    std::lock_guard<std::mutex> lk(net->net.mu);
    const rbg::Packed p = net->net.pack();
    if (!rbg::jit_supported(p)) return fail(RB_ERR_UNSUPPORTED, "network not covered by the generator");
    return copy_name(rbg::jit_net_source(p, rbg::jit_block()), buf, len);
}

// The warp kernel's dependency table for the network ([R][32] entries into
// out, which holds cap entries); RB_ERR_UNSUPPORTED beyond its reach.
int rbg_internal_warp_dep_table(const rb_network *net, uint16_t *out, size_t cap) {
    if (!net || !out) return fail(RB_ERR_INVALID, "null argument");
    std::vector<uint16_t> tab;
    bool ok;
    {
        std::lock_guard<std::mutex> lk(net->net.mu);
        ok = rbg::warp_dep_table(net->net.pack(), tab);
    }
    if (!ok) return fail(RB_ERR_UNSUPPORTED, "network beyond the dependency table's reach");
    if (tab.size() > cap) return fail(RB_ERR_INVALID, "buffer too small");
    std::memcpy(out, tab.data(), 2 * tab.size());
    return RB_OK;
}

int rbg_internal_jit_compile(const rb_network *net, uint64_t *image_bytes) {
    if (!net) return fail(RB_ERR_INVALID, "null network");
    rbg::Packed p;
    {
        std::lock_guard<std::mutex> lk(net->net.mu);
        p = net->net.pack();
    }
    if (!rbg::jit_supported(p)) return fail(RB_ERR_UNSUPPORTED, "network not covered by the generator");
    size_t n = 0;
    if (!rbg::jit_compile(p, rbg::jit_block(), &n)) return RB_ERR_UNSUPPORTED;
    if (image_bytes) *image_bytes = n;
    return RB_OK;
}

// ---------------------------------------------------------------- batch
struct rb_batch {
    rbg::Batch b;
};

int rb_batch_create(rb_batch **out) {
    if (!out) return fail(RB_ERR_INVALID, "null argument");
    *out = new (std::nothrow) rb_batch();
    return *out ? RB_OK : fail(RB_ERR_NOMEM, "out of host memory");
}

void rb_batch_destroy(rb_batch *b) { delete b; }

int rb_batch_add(rb_batch *b, const rb_network *net, int64_t n_traj, const int64_t *x0, int32_t x0_per_traj,
                 const double *rates, int32_t rates_per_traj, const uint64_t *seeds, double tmax, int64_t nb_steps,
                 const int32_t *save_idx, int32_t n_save, int64_t *out, uint64_t *events) {
    if (!b || !net) return fail(RB_ERR_INVALID, "null argument");
    rbg::Batch::ItemIn in;
    in.n_traj = n_traj;
    in.x0 = x0;
    in.x0_per_traj = x0_per_traj;
    in.rates = rates;
    in.rates_per_traj = rates_per_traj;
    in.seeds = seeds;
    in.tmax = tmax;
    in.nb_steps = nb_steps;
    in.save_idx = save_idx;
    in.n_save = n_save;
    in.out = out;
    in.events = events;
    b->b.free_device_if_built();
    const std::string e = b->b.add(&net->net, in);
    return e.empty() ? RB_OK : fail(RB_ERR_INVALID, e);
}

int rb_batch_run(rb_batch *b, rb_run_stats *stats) {
    if (!b) return fail(RB_ERR_INVALID, "null batch");
    const auto t0 = std::chrono::steady_clock::now();
    rbg::rb_stats_out st;
    const bool ok = b->b.run(st);
    if (stats) {
        std::memset(stats, 0, sizeof *stats);
        stats->events = st.events;
        stats->kernel_ms = st.graph_ms;
        stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->h2d_bytes = st.h2d;
        stats->d2h_bytes = st.d2h;
        stats->kernel_launches = st.launches;
        stats->mapping = 6;
    }
    if (ok) return RB_OK;
    return st.timeout ? RB_ERR_TIMEOUT : RB_ERR_CUDA;
}

// Device time of the last run's graph in three parts: the input copy, the
// kernels, the result copy (ms; -1 if not available).
int rbg_internal_batch_times(const rb_batch *b, float *in_ms, float *kern_ms, float *out_ms) {
    if (!b || !in_ms || !kern_ms || !out_ms) return fail(RB_ERR_INVALID, "null argument");
    *in_ms = b->b.last_in_ms;
    *kern_ms = b->b.last_kern_ms;
    *out_ms = b->b.last_out_ms;
    return RB_OK;
}

int rb_batch_plan(rb_batch *b, int32_t *n_own_launches, int32_t *n_persistent_items) {
    if (!b) return fail(RB_ERR_INVALID, "null batch");
    if (!b->b.planned) b->b.plan();
    if (n_own_launches) *n_own_launches = (int32_t)b->b.classes.size();
    if (n_persistent_items) *n_persistent_items = (int32_t)(b->b.warp_items.size() + b->b.thread_items.size());
    return RB_OK;
}

int rb_batch_item_results(const rb_batch *b, int32_t item, const int64_t **out, const uint64_t **events) {
    if (!b || !out || !events) return fail(RB_ERR_INVALID, "null argument");
    if (item < 0 || item >= (int32_t)b->b.items.size()) return fail(RB_ERR_INVALID, "item index out of range");
    if (!b->b.item_results(item, out, events)) return fail(RB_ERR_INVALID, "the batch has not run yet");
    return RB_OK;
}

int rb_batch_item_mapping(const rb_batch *b, int32_t item, int32_t *mapping) {
    if (!b || !mapping || item < 0 || item >= (int32_t)b->b.items.size())
        return fail(RB_ERR_INVALID, "item index out of range");
    *mapping = b->b.items[item].mapping;
    return RB_OK;
}

// ---------------------------------------------------------------- autotuner
static void shape_out(const rbg::LaunchShape &s, double ms, rb_tune_result *o) {
    o->mapping = s.kernel;
    o->block = s.block;
    o->phase_steps = s.phase;
    o->sched = s.sched;
    o->ms = ms;
}

int rb_ensemble_tune(const rb_network *netp, int64_t n_traj, const int64_t *x0, int32_t x0_per_traj,
                     const double *rates, int32_t rates_per_traj, double tmax, int64_t nb_steps,
                     rb_tune_result *best, rb_tune_result *trials, int32_t max_trials, int32_t *n_trials) {
    if (!netp) return fail(RB_ERR_INVALID, "null network");
    const rbg::Network &net = netp->net;
    if (n_traj < 1) return fail(RB_ERR_INVALID, "tuning needs at least one trajectory");
    if (nb_steps < 1) return fail(RB_ERR_INVALID, "nb_steps must be >= 1");
    if (net.n_species && !x0) return fail(RB_ERR_INVALID, "null x0");
    if (max_trials > 0 && !trials) return fail(RB_ERR_INVALID, "null trials");
    std::lock_guard<std::mutex> lk(net.mu);
    rbg::LaunchShape b;
    double ms = 0;
    std::vector<rbg::TuneTrial> tr;
    if (!rbg::tune_ensemble(net, n_traj, x0, x0_per_traj != 0, rates, rates_per_traj != 0, tmax, nb_steps, b, ms, tr))
        return RB_ERR_CUDA;
    if (best) shape_out(b, ms, best);
    for (int32_t k = 0; k < max_trials && k < (int32_t)tr.size(); k++) shape_out(tr[k].shape, tr[k].ms, trials + k);
    if (n_trials) *n_trials = (int32_t)tr.size();
    return RB_OK;
}

int rb_tune_lookup(const rb_network *netp, int64_t n_traj, int32_t rates_per_traj, rb_tune_result *out) {
    if (!netp || !out) return fail(RB_ERR_INVALID, "null argument");
    rbg::DeviceCtx *ctx = rbg::device_ctx();
    if (!ctx) return RB_ERR_CUDA;
    rbg::Packed p;
    {
        std::lock_guard<std::mutex> lk(netp->net.mu);
        p = netp->net.pack();
    }
    rbg::LaunchShape s;
    double ms = 0;
    if (!rbg::tune_get(rbg::tune_key(p, ctx->sm_count, ctx->name, n_traj, rates_per_traj != 0), s, &ms))
        return fail(RB_ERR_INVALID, "no tuned shape for this network and ensemble size");
    shape_out(s, ms, out);
    return RB_OK;
}

size_t rb_tune_cache_path(char *buf, size_t len) {
    const std::string path = rbg::tune_cache_path();
    if (buf && len) {
        const size_t n = std::min(len - 1, path.size());
        std::memcpy(buf, path.data(), n);
        buf[n] = 0;
    }
    return path.size();
}

void rb_tune_clear(int32_t remove_file) { rbg::tune_clear(remove_file != 0); }

// The tuner's cache key and the candidate shapes of one stage, for a device
// with `sm_count` SMs and `smem_optin` bytes of shared memory per block named
// `gpu` (no GPU needed).  best: the best shape so far (stages 1, 2).
int rbg_internal_tune_key(const rb_network *netp, int32_t sm_count, const char *gpu, int64_t n_traj,
                          int32_t rates_per_traj, char *buf, size_t len) {
    if (!netp || !gpu) return fail(RB_ERR_INVALID, "null argument");
    rbg::Packed p;
    {
        std::lock_guard<std::mutex> lk(netp->net.mu);
        p = netp->net.pack();
    }
    return copy_name(rbg::tune_key(p, sm_count, gpu, n_traj, rates_per_traj != 0), buf, len);
}

int rbg_internal_tune_candidates(const rb_network *netp, int32_t sm_count, size_t smem_optin, int64_t n_traj,
                                 int64_t nb_steps, double tmax, int32_t rates_per_traj, int32_t stage,
                                 const rb_tune_result *best, rb_tune_result *out, int32_t cap, int32_t *n_out) {
    if (!netp || !n_out) return fail(RB_ERR_INVALID, "null argument");
    rbg::Packed p;
    {
        std::lock_guard<std::mutex> lk(netp->net.mu);
        p = netp->net.pack();
    }
    rbg::DeviceCtx ctx;
    ctx.sm_count = sm_count;
    ctx.smem_optin = smem_optin;
    const rbg::Feasible f = rbg::feasible_kernels(p, ctx, n_traj, nb_steps + 1, std::isfinite(tmax) && tmax >= 0,
                                                   tmax, rates_per_traj != 0);
    rbg::LaunchShape b;
    if (best) {
        b.kernel = best->mapping;
        b.block = best->block;
        b.phase = best->phase_steps;
        b.sched = best->sched;
    }
    const auto c = rbg::tune_candidates(f, stage, b);
    for (int32_t k = 0; k < cap && k < (int32_t)c.size(); k++) shape_out(c[k], 0, out + k);
    *n_out = (int32_t)c.size();
    return RB_OK;
}

// Record a tuned shape under a key (tests of the cache file).
int rbg_internal_tune_store(const char *key, const rb_tune_result *s) {
    if (!key || !s) return fail(RB_ERR_INVALID, "null argument");
    rbg::LaunchShape l;
    l.kernel = s->mapping;
    l.block = s->block;
    l.phase = s->phase_steps;
    l.sched = s->sched;
    rbg::tune_store(key, l, s->ms);
    return RB_OK;
}

int rbg_internal_tune_get(const char *key, rb_tune_result *out) {
    if (!key || !out) return fail(RB_ERR_INVALID, "null argument");
    rbg::LaunchShape l;
    double ms = 0;
    if (!rbg::tune_get(key, l, &ms)) return fail(RB_ERR_INVALID, "no entry");
    shape_out(l, ms, out);
    return RB_OK;
}

}  // extern "C"
