// Host engine implementation.
#include "engine.hpp"
#include "ssa_jit.hpp"
#include "tune.hpp"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

namespace rbg {

static thread_local std::string g_last_error;
void set_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

bool cuda_ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_error(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
    return false;
}

// ZIGNOR construction (Doornik 2005) of the 256-layer exponential ziggurat:
// x[0] = v / f(r), x[1] = r, x[i] = f^-1(v / x[i-1] + f(x[i-1])), x[256] = 0,
// f(x) = exp(-x); r and v are the tail start and the common layer area.
void zig_tables_host(double *x, double *f) {
    const double r = 7.69711747013104972;
    const double v = 0.0039496598225815571993;
    x[0] = v / std::exp(-r);
    x[1] = r;
    for (int i = 2; i < kZigLayers; i++) x[i] = -std::log(v / x[i - 1] + std::exp(-x[i - 1]));
    x[kZigLayers] = 0.0;
    for (int i = 0; i < kZigTable; i++) f[i] = std::exp(-x[i]);
}

// Fast-path companions of the tables.  Layer i draws u = (2k+1) 2^-53 from a
// 52-bit k and accepts x = RN(u * x[i]) when x < x[i+1].  RN(u * x[i]) is
// non-decreasing in k, so the accepted k form a prefix [0, K_i): K_i replaces
// the comparison with an integer one.  d[i] = RN(f[i] - f[i+1]) is the
// wedge test's difference, computed once here exactly as the draw would.
void zig_fast_tables_host(const double *x, const double *f, uint64_t *K, double *d) {
    for (int i = 0; i < kZigLayers; i++) {
        uint64_t lo = 0, hi = 1ull << 52;  // first k in [lo, hi] with !(x < x[i+1])
        while (lo < hi) {
            const uint64_t mid = lo + (hi - lo) / 2;
            const double u = (double)(2 * mid + 1) * 0x1p-53;
            if (u * x[i] < x[i + 1]) lo = mid + 1;
            else hi = mid;
        }
        K[i] = lo;
        d[i] = f[i] - f[i + 1];
    }
}

static std::mutex g_ctx_mu;
static std::map<int, DeviceCtx *> g_ctx;

DeviceCtx *device_ctx() {
    int dev = 0;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
    std::lock_guard<std::mutex> lk(g_ctx_mu);
    auto it = g_ctx.find(dev);
    if (it != g_ctx.end()) return it->second;
    auto *c = new DeviceCtx();
    c->device = dev;
    cudaDeviceProp prop;
    if (!cuda_ok(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties")) {
        delete c;
        return nullptr;
    }
    if (prop.major < 10) {
        set_error(std::string("device ") + prop.name + " is not a Blackwell-class GPU (sm_103a build)");
        delete c;
        return nullptr;
    }
    c->sm_count = prop.multiProcessorCount;
    c->smem_optin = prop.sharedMemPerBlockOptin;
    c->name = prop.name;
    std::vector<double> tab(kZigWords);
    zig_tables_host(tab.data(), tab.data() + kZigOffF);
    zig_fast_tables_host(tab.data(), tab.data() + kZigOffF, reinterpret_cast<uint64_t *>(tab.data() + kZigOffK),
                         tab.data() + kZigOffD);
    for (int i = 0; i < kZigLayers; i++) {
        float pair[2];
        pair[0] = (float)tab[i];
        pair[1] = (float)(tab[i] - (double)pair[0]);
        std::memcpy(&tab[kZigOffXdf + i], pair, sizeof pair);
    }
    if (!cuda_ok(cudaMalloc(&c->zig, sizeof(double) * kZigWords), "cudaMalloc(zig)") ||
        !cuda_ok(cudaMemcpy(c->zig, tab.data(), sizeof(double) * kZigWords, cudaMemcpyHostToDevice),
                 "cudaMemcpy(zig)")) {
        delete c;
        return nullptr;
    }
    g_ctx[dev] = c;
    return c;
}

DeviceNet::~DeviceNet() {
    // Teardown after the CUDA runtime has shut down must not fault; errors
    // are ignored here.
    if (desc) cudaFree(desc);
    if (scratch) cudaFree(scratch);
    if (dep) cudaFree(dep);
    if (warp_cnt0) cudaFree(warp_cnt0);
    if (io) cudaFree(io);
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_stop) cudaEventDestroy(ev_stop);
    if (stream) cudaStreamDestroy(stream);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (pin_rows) cudaFreeHost(pin_rows);
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

bool warp_dep_table(const Packed &p, std::vector<uint16_t> &tab) {
    const int R = p.R, P = p.P, Q = p.Q;
    const int C = (R + 31) / 32;
    tab.clear();
    if (R < 1 || C > 256) return false;
    tab.assign((size_t)R * 32, 0);
    // reactions reading each species
    std::vector<std::vector<int32_t>> readers((size_t)p.S);
    for (int r = 0; r < R; r++)
        for (int k = 0; k < P; k++)
            if (p.fac_ord[(size_t)r * P + k] > 0) {
                auto &v = readers[(size_t)p.fac_sp[(size_t)r * P + k]];
                if (v.empty() || v.back() != r) v.push_back(r);
            }
    std::vector<int32_t> mark((size_t)R, -1);
    for (int j = 0; j < R; j++) {
        int n = 0;
        uint16_t *row = tab.data() + (size_t)j * 32;
        for (int k = 0; k < Q; k++) {
            if (p.jmp_d[(size_t)j * Q + k] == 0) continue;
            for (int32_t r : readers[(size_t)p.jmp_sp[(size_t)j * Q + k]])
                if (mark[(size_t)r] != j) {
                    mark[(size_t)r] = j;
                    if (++n <= 31) row[n] = (uint16_t)((r % C) * 32 + r / C);
                }
        }
        row[0] = n <= 31 ? (uint16_t)n : (uint16_t)0xFFFF;
    }
    return true;
}

bool ensure_device(const Network &net) {
    DeviceCtx *ctx = device_ctx();
    if (!ctx) return false;
    if (net.dev && net.dev->device != ctx->device) net.dev.reset();
    if (!net.dev) {
        auto dn = std::make_unique<DeviceNet>();
        dn->device = ctx->device;
        if (!cuda_ok(cudaStreamCreateWithFlags(&dn->stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
            !cuda_ok(cudaStreamCreateWithFlags(&dn->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate") ||
            !cuda_ok(cudaEventCreate(&dn->ev_start), "cudaEventCreate") ||
            !cuda_ok(cudaEventCreate(&dn->ev_stop), "cudaEventCreate") ||
            !cuda_ok(cudaMalloc(&dn->scratch, 4 * sizeof(unsigned long long)), "cudaMalloc(scratch)"))
            return false;
        net.dev = std::move(dn);
    }
    DeviceNet &dn = *net.dev;
    if (dn.version == net.version) return true;
    Packed p = net.pack();
    const size_t R = p.R, P = p.P, Q = p.Q;
    size_t off_rate = 0;
    size_t off_jd = align_up(off_rate + sizeof(double) * std::max<size_t>(R, 1), 16);
    size_t off_fsp = align_up(off_jd + sizeof(int64_t) * std::max<size_t>(R * Q, 1), 16);
    size_t off_ford = align_up(off_fsp + sizeof(int32_t) * std::max<size_t>(R * P, 1), 16);
    size_t off_jsp = align_up(off_ford + sizeof(int32_t) * std::max<size_t>(R * P, 1), 16);
    size_t off_exo = align_up(off_jsp + sizeof(int32_t) * std::max<size_t>(R * Q, 1), 16);
    size_t off_exc = align_up(off_exo + sizeof(int32_t) * (R + 1), 16);
    size_t off_exk = align_up(off_exc + sizeof(int32_t) * std::max<size_t>(p.ex_code.size(), 1), 16);
    size_t total = align_up(off_exk + sizeof(double) * std::max<size_t>(p.ex_const.size(), 1), 16);
    if (dn.desc) {
        cudaFree(dn.desc);
        dn.desc = nullptr;
    }
    if (!cuda_ok(cudaMalloc(&dn.desc, total), "cudaMalloc(descriptor)")) return false;
    std::vector<unsigned char> img(total, 0);
    if (R) {
        std::memcpy(img.data() + off_rate, p.rate.data(), sizeof(double) * R);
        std::memcpy(img.data() + off_jd, p.jmp_d.data(), sizeof(int64_t) * R * Q);
        std::memcpy(img.data() + off_fsp, p.fac_sp.data(), sizeof(int32_t) * R * P);
        std::memcpy(img.data() + off_ford, p.fac_ord.data(), sizeof(int32_t) * R * P);
        std::memcpy(img.data() + off_jsp, p.jmp_sp.data(), sizeof(int32_t) * R * Q);
        std::memcpy(img.data() + off_exo, p.ex_off.data(), sizeof(int32_t) * (R + 1));
    }
    if (!p.ex_code.empty()) std::memcpy(img.data() + off_exc, p.ex_code.data(), sizeof(int32_t) * p.ex_code.size());
    if (!p.ex_const.empty())
        std::memcpy(img.data() + off_exk, p.ex_const.data(), sizeof(double) * p.ex_const.size());
    if (!cuda_ok(cudaMemcpy(dn.desc, img.data(), total, cudaMemcpyHostToDevice), "cudaMemcpy(descriptor)"))
        return false;
    unsigned char *b = static_cast<unsigned char *>(dn.desc);
    dn.rate = reinterpret_cast<double *>(b + off_rate);
    dn.jmp_d = reinterpret_cast<int64_t *>(b + off_jd);
    dn.fac_sp = reinterpret_cast<int32_t *>(b + off_fsp);
    dn.fac_ord = reinterpret_cast<int32_t *>(b + off_ford);
    dn.jmp_sp = reinterpret_cast<int32_t *>(b + off_jsp);
    dn.ex_off = p.has_expr ? reinterpret_cast<int32_t *>(b + off_exo) : nullptr;
    dn.ex_code = reinterpret_cast<int32_t *>(b + off_exc);
    dn.ex_const = reinterpret_cast<double *>(b + off_exk);
    dn.packed = std::move(p);
    dn.version = net.version;
    return true;
}

bool ensure_io(DeviceNet &dn, size_t bytes) {
    if (dn.io_bytes >= bytes) return true;
    if (dn.io) {
        cudaStreamSynchronize(dn.stream);
        cudaFree(dn.io);
        dn.io = nullptr;
        dn.io_bytes = 0;
    }
    size_t want = std::max(bytes, dn.io_bytes * 3 / 2);
    if (!cuda_ok(cudaMalloc(&dn.io, want), "cudaMalloc(staging)")) return false;
    dn.io_bytes = want;
    return true;
}

int64_t kernel_budget_ns() {
    const char *env = std::getenv("RB_KERNEL_BUDGET_S");
    double sec = env ? std::atof(env) : 120.0;
    if (!(sec > 0)) sec = 120.0;
    return (int64_t)(sec * 1e9);
}

std::vector<double> sample_times(double tmax, int64_t nb_steps) {
    std::vector<double> t((size_t)nb_steps + 1);
    for (int64_t i = 0; i <= nb_steps; i++) t[(size_t)i] = tmax * (double)i / (double)nb_steps;
    return t;
}

static SsaArgs base_args(const Packed &p) {
    SsaArgs a{};
    a.S = p.S;
    a.R = p.R;
    a.P = p.P;
    a.Q = p.Q;
    a.macro_mode = p.macro_mode;
    int mm = 0;
    for (int32_t rr = 0; rr < p.R; rr++) {
        int s = 0;
        for (int32_t k = 0; k < p.P; k++) s += p.fac_ord[(size_t)rr * p.P + k];
        mm = std::max(mm, s);
    }
    a.max_mults = mm;
    return a;
}

Feasible feasible_kernels(const Packed &p, const DeviceCtx &ctx, int64_t n_traj, int64_t n_samples, bool times_ok,
                          double t_last, bool rates_per_traj) {
    SsaArgs a = base_args(p);
    a.n_traj = n_traj;
    a.n_samples = n_samples;
    a.n_save = p.S;
    a.rate_stride = rates_per_traj ? p.R : 0;
    Feasible f;
    const int spec_grid = (int)std::max<int64_t>(
        1, std::min<int64_t>(ctx.sm_count, (n_traj + ssa_spec_block() - 1) / ssa_spec_block()));
    f.spec = !p.has_expr && times_ok && t_last < 0x1p60 && ssa_spec_supported(a, p.max_order) &&
             ssa_spec_slots(a, spec_grid, ctx.smem_optin, ssa_spec_block()) > 0;
    f.jit = f.spec && jit_supported(p);
    f.warp = !p.has_expr && ssa_warp_supported(a, p.max_order) && ssa_warp_warps(a, ctx.smem_optin) > 0;
    f.fast = !p.has_expr && times_ok && ssa_fast_supported(a, p.max_order) && ssa_fast_smem(a, 128) <= ctx.smem_optin;
    f.generic = p.R <= 32 && ssa_thread_max_block(a, ctx.smem_optin) > 0;
    f.spread = n_traj < (int64_t)ctx.sm_count * 4 * 32;
    f.reactions = p.R;
    return f;
}

bool launch_sampled(const Network &net, DeviceNet &dn, const RunDev &r, cudaStream_t stream, bool timed,
                    int *mapping, const LaunchShape *force) {
    DeviceCtx *ctx = device_ctx();
    if (!ctx) return false;
    const Packed &p = dn.packed;
    SsaArgs a = base_args(p);
    a.rate = r.rates ? r.rates : dn.rate;
    a.rate_stride = r.rates ? r.rate_stride : 0;
    a.fac_sp = dn.fac_sp;
    a.fac_ord = dn.fac_ord;
    a.jmp_sp = dn.jmp_sp;
    a.jmp_d = dn.jmp_d;
    a.ex_off = dn.ex_off;
    a.ex_code = dn.ex_code;
    a.ex_const = dn.ex_const;
    a.n_traj = r.n_traj;
    a.x0 = r.x0;
    a.x0_stride = r.x0_stride;
    a.seeds = r.seeds;
    a.in_species = r.in_species;
    a.in_t = r.in_t;
    a.in_rng = r.in_rng;
    a.sample_t = r.sample_t;
    a.n_samples = r.n_samples;
    a.save_idx = r.save_idx;
    a.n_save = r.n_save;
    a.out = r.out;
    a.fin_species = r.fin_species;
    a.fin_t = r.fin_t;
    a.fin_rng = r.fin_rng;
    a.events = r.events;
    a.work = dn.scratch;
    a.zig = ctx->zig;
    a.budget_ns = kernel_budget_ns();
    if (!cuda_ok(cudaMemsetAsync(dn.scratch, 0, 4 * sizeof(unsigned long long), stream), "cudaMemsetAsync"))
        return false;
    if (r.n_traj == 0) return true;
    // Kernel choice: a forced shape, else the autotuner's choice for this
    // network shape, else the speculative float-pair kernel, the lockstep
    // exact kernel, the generic shared-memory kernel (RB_SSA_KERNEL=
    // spec|fast|generic|warp overrides).
    const char *pref = std::getenv("RB_SSA_KERNEL");
    LaunchShape shape;
    if (force) shape = *force;
    else if (!pref && !r.in_species && tune_lookup(p, *ctx, r.n_traj, r.rate_stride != 0, shape) &&
             !tune_shape_feasible(feasible_kernels(p, *ctx, r.n_traj, r.n_samples, r.times_ok, r.t_last,
                                                   r.rate_stride != 0),
                                  shape))
        shape = LaunchShape{};
    const int k = pref ? -1 : shape.kernel;
    const bool want_generic = (pref && std::strcmp(pref, "generic") == 0) || k == 0;
    const bool want_fast = (pref && std::strcmp(pref, "fast") == 0) || k == 2;
    const bool want_desc = (pref && std::strcmp(pref, "spec") == 0) || k == 3;  // descriptor, not generated
    const bool want_jit = k == 4;
    const bool want_warp = (pref && std::strcmp(pref, "warp") == 0) || k == 5;
    const int spec_grid = (int)std::max<int64_t>(
        1, std::min<int64_t>(ctx->sm_count, (r.n_traj + ssa_spec_block() - 1) / ssa_spec_block()));
    const int spec_slots = ssa_spec_slots(a, spec_grid, ctx->smem_optin, ssa_spec_block());
    // Rate::Expr networks run on the generic kernel (native binary64 programs).
    const bool spec = !p.has_expr && !want_generic && !want_fast && !want_warp && r.times_ok && r.t_last < 0x1p60 &&
                      ssa_spec_supported(a, p.max_order) && spec_slots > 0;
    // Networks beyond the thread kernels' reach (more than 32 reactions, or
    // too large for their shared memory) take a warp per trajectory.
    const int warp_w = ssa_warp_supported(a, p.max_order) ? ssa_warp_warps(a, ctx->smem_optin) : 0;
    const bool warp = warp_w > 0 && !want_generic && !want_fast && !p.has_expr &&
                      (want_warp || (!spec && !(p.R <= 32 && ssa_thread_max_block(a, ctx->smem_optin) > 0)));
    const bool fast = !warp && !spec && !p.has_expr && !want_generic && r.times_ok && ssa_fast_supported(a, p.max_order) &&
                      ssa_fast_smem(a, 128) <= ctx->smem_optin;
    const bool strict = pref || force;  // a kernel asked for must run
    if (strict && ((want_fast && !fast) || (want_warp && !warp) || ((want_desc || want_jit) && !spec))) {
        set_error(std::string("kernel ") + (pref ? pref : std::to_string(k).c_str()) +
                  " does not cover this network or sample grid");
        return false;
    }
    // Ensembles too small to fill every SM scheduler with a full warp spread
    // out: `lanes` trajectories per warp, one 4-warp block per SM, so each
    // trajectory's step latency is close to a lone lane's (RB_SPEC_LANES=k
    // sets k lanes per warp; 32 turns the spreading off).
    int lanes = 0;
    if (spec) {
        const int64_t sched = (int64_t)ctx->sm_count * 4;
        if (const char *e = std::getenv("RB_SPEC_LANES")) lanes = std::max(1, std::min(32, std::atoi(e)));
        else if (r.n_traj < sched * 32) lanes = (int)((r.n_traj + sched - 1) / sched);
        if (lanes >= 32) lanes = 0;
    }
    int block, per_sm;
    size_t smem;
    if (warp) {
        block = 32 * warp_w;
        smem = ssa_warp_smem(a, warp_w);
        per_sm = std::max(1, ssa_warp_occupancy(a, warp_w, smem));
        const int64_t blocks = std::max<int64_t>(
            1, std::min<int64_t>((r.n_traj + warp_w - 1) / warp_w, (int64_t)ctx->sm_count * per_sm));
        // dependency lists: only the propensities a reaction's jump touches
        // are re-evaluated after it fires (RB_WARP_DEPS=0: all, every step)
        if (dn.dep_version != dn.version) {
            if (dn.dep) cudaFree(dn.dep);
            dn.dep = nullptr;
            std::vector<uint16_t> tab;
            dn.dep_ok = warp_dep_table(p, tab);
            if (dn.dep_ok &&
                (!cuda_ok(cudaMalloc(&dn.dep, sizeof(uint16_t) * tab.size()), "cudaMalloc(dependency table)") ||
                 !cuda_ok(cudaMemcpy(dn.dep, tab.data(), sizeof(uint16_t) * tab.size(), cudaMemcpyHostToDevice),
                          "cudaMemcpy(dependency table)")))
                return false;
            dn.dep_version = dn.version;
        }
        const size_t n_cnt0 = (size_t)blocks * warp_w * std::max(p.S, 1);
        if (dn.warp_cnt0_n < n_cnt0) {
            if (dn.warp_cnt0) {
                cudaStreamSynchronize(stream);
                cudaFree(dn.warp_cnt0);
            }
            dn.warp_cnt0 = nullptr;
            dn.warp_cnt0_n = 0;
            if (!cuda_ok(cudaMalloc(&dn.warp_cnt0, 8 * n_cnt0), "cudaMalloc(interval-start counts)")) return false;
            dn.warp_cnt0_n = n_cnt0;
        }
        a.warp_cnt0 = dn.warp_cnt0;
        const char *wd = std::getenv("RB_WARP_DEPS");
        if (dn.dep_ok && !(wd && std::strcmp(wd, "0") == 0)) a.dep_tab = dn.dep;
        if (const char *xc = std::getenv("RB_WARP_EXACT_CHOICE")) a.exact_choice = std::strcmp(xc, "0") != 0;
        if (timed && !cuda_ok(cudaEventRecord(dn.ev_start, stream), "cudaEventRecord")) return false;
        const int err = launch_ssa_warp(a, warp_w, (int)blocks, smem, stream);
        if (err != 0) return cuda_ok((cudaError_t)err, "SSA kernel launch");
        if (timed && !cuda_ok(cudaEventRecord(dn.ev_stop, stream), "cudaEventRecord")) return false;
        if (mapping) *mapping = 5;
        return true;
    }
    if (spec) {
        a.row_done = r.n_samples < 65536 ? r.row_done : nullptr;
        block = lanes ? 128 : ssa_spec_block();
        a.n_slots = lanes ? 128 : spec_slots;
        a.lanes = lanes;
        a.phase_steps = shape.phase;
        a.sched = shape.sched > 0 ? 1 : 0;
        if (const char *ph = std::getenv("RB_SPEC_PHASE")) a.phase_steps = std::atoi(ph);
        if (const char *sc = std::getenv("RB_SPEC_SCHED")) a.sched = std::strcmp(sc, "rot") == 0 ? 1 : 0;
        smem = ssa_spec_smem(a, a.n_slots);
        per_sm = ssa_spec_occupancy(a, block, smem);
    } else if (fast) {
        block = 128;
        smem = ssa_fast_smem(a, block);
        per_sm = ssa_fast_occupancy(a, block, smem);
    } else {
        block = ssa_thread_max_block(a, ctx->smem_optin);
        if (block == 0) {
            set_error("network too large for the thread-per-trajectory kernel (" + std::to_string(p.S) +
                      " species, " + std::to_string(p.R) + " reactions)");
            return false;
        }
        smem = ssa_thread_smem(a, block);
        per_sm = ssa_thread_occupancy(a, block, smem);
    }
    if (per_sm < 1) per_sm = 1;
    int64_t want = lanes ? (r.n_traj + 4 * lanes - 1) / (4 * lanes) : (r.n_traj + block - 1) / block;
    int64_t cap = (int64_t)ctx->sm_count * per_sm;
    int grid = (int)std::max<int64_t>(1, std::min(want, cap));
    // A network the generator covers runs on its own compiled kernel (RB_JIT=0
    // never, RB_JIT=1 always; results are the same either way).  By default
    // the kernel is compiled when the ensemble is large enough to repay the
    // compilation or the network runs a second time, and used whenever it is
    // already loaded or in the disk cache.
    const void *jk = nullptr;
    const int64_t run_no = ++dn.runs;
    if (spec && jit_supported(p)) {
        const char *jit = std::getenv("RB_JIT");
        // RB_SSA_KERNEL=spec (or a shape of kernel 3) asks for the
        // packed-descriptor kernel itself
        const bool off = (jit && std::strcmp(jit, "0") == 0) || want_desc;
        const bool compile = jit ? !off : (want_jit || r.n_traj >= 4096 || run_no >= 2);
        if (!off) {
            // generated kernels may run larger blocks (fewer registers per lane)
            int kb = shape.block > 0 && !std::getenv("RB_JIT_BLOCK") ? shape.block : jit_block();
            // spread launches run 128 lanes of a kernel built for 128 (all
            // registers to the few lanes that hold trajectories)
            const bool spread = lanes != 0;
            if (spread) kb = 128;
            const int jb = kb;
            const int jgrid = spread ? grid
                                     : (int)std::max<int64_t>(1, std::min<int64_t>(ctx->sm_count, (r.n_traj + jb - 1) / jb));
            const int jslots = spread ? 128 : ssa_spec_slots(a, jgrid, ctx->smem_optin, jb);
            if (jslots > 0) {
                if (dn.jit_k && dn.jit_block == kb && dn.jit_version == dn.version) {
                    jk = dn.jit_k;
                } else {
                    jk = jit_kernel(p, kb, compile);
                    if (jk) {
                        dn.jit_k = jk;
                        dn.jit_block = kb;
                        dn.jit_version = dn.version;
                    } else if (!compile) {
                        // this run takes the descriptor kernel; the generated
                        // one compiles meanwhile, for the next run to find
                        jit_compile_async(p, kb);
                    }
                }
                if (!jk && ((jit && std::strcmp(jit, "1") == 0) || (want_jit && force))) return false;
                if (jk) {
                    block = jb;
                    grid = jgrid;
                    a.n_slots = jslots;
                    a.lanes = spread ? lanes : 0;
                    smem = ssa_spec_smem(a, jslots);
                }
            }
        }
    }
    if (timed && !cuda_ok(cudaEventRecord(dn.ev_start, stream), "cudaEventRecord")) return false;
    int err = jk     ? launch_ssa_jit(jk, a, block, grid, smem, stream)
              : spec ? launch_ssa_spec(a, block, grid, smem, stream)
              : fast ? launch_ssa_fast(a, block, grid, smem, stream)
                     : launch_ssa_thread(a, block, grid, smem, stream);
    if (err != 0) return cuda_ok((cudaError_t)err, "SSA kernel launch");
    if (timed && !cuda_ok(cudaEventRecord(dn.ev_stop, stream), "cudaEventRecord")) return false;
    if (mapping) *mapping = jk ? 4 : spec ? 3 : fast ? 2 : 0;
    return true;
}

}  // namespace rbg
