// Networks compiled at run time: the float-pair step of the speculative kernel
// (ssa_spec_body.cuh) generated for one network, with every reaction unrolled,
// the counts in registers and the jumps as straight-line selects, compiled by
// NVRTC for sm_103a and loaded through the runtime's library API.
//
// This is the GPU counterpart of rebop's define_system! macro, which
// specialises the same loop for one network at Rust compile time
// (src/gillespie_macro.rs:50-171): the generated kernel's results are the
// packed-descriptor kernel's, bit for bit, since both decide every step the
// same way and both re-run undecided intervals with the same exact step.
//
// NVRTC is opened with dlopen on first use, so the library loads (and the
// descriptor kernels run) on machines without it.  Compiled images are kept in
// memory per device and on disk under $RB_JIT_CACHE (default
// $HOME/.cache/rebop_gb300), keyed by a hash of the generated source, the
// embedded headers, the options and the NVRTC version.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <set>
#include <thread>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <unistd.h>
#include <vector>

#include "engine.hpp"
#include "ssa_jit.hpp"

namespace rbg {

// Embedded device headers (generated by build.py from csrc/).
extern const char *const kJitHeaderNames[];
extern const char *const kJitHeaderSources[];
extern const int kJitHeaderCount;

namespace {

constexpr int kJitMaxSpecies = 16;
constexpr int kJitMaxReactions = 32;

struct Nvrtc {
    bool tried = false, ok = false;
    std::string why;
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
    decltype(&nvrtcVersion) version = nullptr;
};

std::mutex g_mu;
Nvrtc g_nvrtc;

Nvrtc *nvrtc() {
    if (g_nvrtc.tried) return g_nvrtc.ok ? &g_nvrtc : nullptr;
    g_nvrtc.tried = true;
    std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
    for (const char *env : {"CUDA_HOME", "CUDA_PATH"}) {
        const char *v = std::getenv(env);
        if (v && *v) names.push_back(std::string(v) + "/lib64/libnvrtc.so.13");
    }
    names.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
    void *h = nullptr;
    for (const std::string &n : names)
        if ((h = dlopen(n.c_str(), RTLD_NOW | RTLD_LOCAL))) break;
    if (!h) {
        g_nvrtc.why = "libnvrtc.so.13 not found";
        return nullptr;
    }
    auto sym = [&](const char *n) { return dlsym(h, n); };
    g_nvrtc.create = (decltype(g_nvrtc.create))sym("nvrtcCreateProgram");
    g_nvrtc.compile = (decltype(g_nvrtc.compile))sym("nvrtcCompileProgram");
    g_nvrtc.log_size = (decltype(g_nvrtc.log_size))sym("nvrtcGetProgramLogSize");
    g_nvrtc.log = (decltype(g_nvrtc.log))sym("nvrtcGetProgramLog");
    g_nvrtc.cubin_size = (decltype(g_nvrtc.cubin_size))sym("nvrtcGetCUBINSize");
    g_nvrtc.cubin = (decltype(g_nvrtc.cubin))sym("nvrtcGetCUBIN");
    g_nvrtc.destroy = (decltype(g_nvrtc.destroy))sym("nvrtcDestroyProgram");
    g_nvrtc.version = (decltype(g_nvrtc.version))sym("nvrtcVersion");
    g_nvrtc.ok = g_nvrtc.create && g_nvrtc.compile && g_nvrtc.log_size && g_nvrtc.log && g_nvrtc.cubin_size &&
                 g_nvrtc.cubin && g_nvrtc.destroy && g_nvrtc.version;
    if (!g_nvrtc.ok) g_nvrtc.why = "libnvrtc lacks a required symbol";
    return g_nvrtc.ok ? &g_nvrtc : nullptr;
}

uint64_t fnv1a(const std::string &s, uint64_t h = 0xcbf29ce484222325ull) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 0x100000001b3ull;
    }
    return h;
}

const std::vector<std::string> &compile_options() {
    // never destroyed: a background compile may still read it at exit
    static const std::vector<std::string> *opts = new std::vector<std::string>{
        "-arch=sm_103a", "-std=c++17", "-fmad=false", "-lineinfo", "-default-device", "-DRBG_JIT=1"};
    return *opts;
}

std::string cache_dir() {
    if (const char *d = std::getenv("RB_JIT_CACHE")) return d;
    const char *home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/rebop_gb300";
}

void mkdirs(const std::string &path) {
    for (size_t i = 1; i <= path.size(); i++)
        if (i == path.size() || path[i] == '/') mkdir(path.substr(0, i).c_str(), 0755);
}

bool read_file(const std::string &path, std::string &out) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return false;
    std::ostringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return !out.empty();
}

void write_file_atomic(const std::string &path, const std::string &data) {
    const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
    {
        std::ofstream f(tmp, std::ios::binary);
        if (!f) return;
        f.write(data.data(), (std::streamsize)data.size());
        if (!f) return;
    }
    std::rename(tmp.c_str(), path.c_str());
}

struct Loaded {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kern = nullptr;
};
std::map<std::pair<int, uint64_t>, Loaded> g_loaded;

}  // namespace

bool jit_supported(const Packed &p) {
    if (p.S < 1 || p.S > kJitMaxSpecies || p.R < 1 || p.R > kJitMaxReactions) return false;
    // the summed change of each species by each reaction is exact in float
    for (int r = 0; r < p.R; r++)
        for (int sp = 0; sp < p.S; sp++) {
            int64_t d = 0;
            for (int k = 0; k < p.Q; k++) {
                if (p.jmp_sp[(size_t)r * p.Q + k] != sp) continue;
                const int64_t v = p.jmp_d[(size_t)r * p.Q + k];
                if (v <= -(1 << 23) || v >= (1 << 23)) return false;
                d += v;
            }
            if (d <= -(1 << 23) || d >= (1 << 23)) return false;
        }
    return true;
}

std::string jit_net_source(const Packed &p, int block) {
    const int S = p.S, R = p.R;
    std::ostringstream o;
    o << "// generated network operations: " << S << " species, " << R << " reactions\n";
    o << "#include \"ssa_spec_body.cuh\"\n\nnamespace rbg {\n\n";
    // exact binary64 choice for the rare close float comparisons
    o << "__device__ __noinline__ int net_exact_choice(float cn[" << S
      << "], const uint64_t *rl, int RS, uint64_t u53) {\n";
    o << "    double cum[" << R << "];\n    double total = 0.0, acc;\n";
    for (int r = 0; r < R; r++) {
        o << "    acc = __longlong_as_double((long long)rl[" << r << " * RS]);\n";
        for (int f = 0; f < p.P; f++) {
            const int32_t ord = p.fac_ord[(size_t)r * p.P + f];
            const int32_t sp = p.fac_sp[(size_t)r * p.P + f];
            if (ord == 0) continue;
            if (p.macro_mode) {
                o << "    { long long ff = (long long)cn[" << sp << "];";
                for (int j = 1; j < ord; j++) o << " ff *= (long long)cn[" << sp << "] - " << j << ";";
                o << " acc = __dmul_rn(acc, (double)ff); }\n";
            } else {
                for (int j = ord - 1; j >= 0; j--)
                    o << "    acc = __dmul_rn(acc, (double)((long long)cn[" << sp << "] - " << j << "));\n";
            }
        }
        o << "    total = __dadd_rn(total, acc);\n    cum[" << r << "] = total;\n";
    }
    o << "    const double chosen = __dmul_rn(total, (double)u53 * 0x1p-53);\n";
    if (p.macro_mode) {
        o << "    int idx = " << R << ";\n";
        for (int r = R - 1; r >= 0; r--) o << "    if (chosen < cum[" << r << "]) idx = " << r << ";\n";
    } else {
        o << "    int idx = 0;\n";
        for (int r = 0; r < R; r++) o << "    idx += cum[" << r << "] < chosen ? 1 : 0;\n";
    }
    o << "    return idx;\n}\n\n";

    o << "struct NetOps {\n";
    o << "    static constexpr int kMaxR = " << R << ";\n";
    o << "    static constexpr bool kMacro = " << (p.macro_mode ? "true" : "false") << ";\n";
    // counts as exact floats in registers (|n| < 2^24)
    o << "    struct Counts { float n[" << S << "]; };\n";
    o << "    __device__ static int nr(const SsaArgs &) { return " << R << "; }\n";
    // load: column -> registers, all counts in [0, 2^23)
    o << "    __device__ static bool load(Counts &c, const SsaArgs &, const int64_t *sp, int NS) {\n";
    o << "        uint64_t m = 0;\n";
    for (int s = 0; s < S; s++)
        o << "        { const int64_t v = sp[" << s << " * NS]; m |= (uint64_t)v; c.n[" << s
          << "] = __int2float_rn((int)(v & 0x7FFFFF)); }\n";
    o << "        return m < (1ull << 23);\n    }\n";
    o << "    __device__ static void store(const Counts &c, const SsaArgs &, int64_t *sp, int NS) {\n";
    for (int s = 0; s < S; s++) o << "        sp[" << s << " * NS] = __float2int_rn(c.n[" << s << "]);\n";
    o << "    }\n";
    o << "    __device__ static void save(const Counts &c, const SsaArgs &, const int64_t *, int64_t *sps, int NS) "
         "{\n";
    for (int s = 0; s < S; s++) o << "        sps[" << s << " * NS] = __float2int_rn(c.n[" << s << "]);\n";
    o << "    }\n";
    // props: every reaction unrolled; every count must lie in [0, 2^23)
    // (a jump moves it by less than 2^23, so floats stay exact in between)
    o << "    __device__ static bool props(const SsaArgs &, const ExactTables &, const Counts &c, const int64_t *, int,\n"
         "                                 const float2 *rf, int RS, float *cum, DF &tot) {\n";
    o << "        RunSum sum;\n";
    o << "        float lo = c.n[0], hi = c.n[0];\n";
    for (int s = 1; s < S; s++) o << "        lo = fminf(lo, c.n[" << s << "]); hi = fmaxf(hi, c.n[" << s << "]);\n";
    for (int r = 0; r < R; r++) {
        o << "        {\n            const float2 k = rf[" << r << " * RS];\n            DF acc{k.x, k.y};\n";
        for (int f = 0; f < p.P; f++) {
            const int32_t ord = p.fac_ord[(size_t)r * p.P + f];
            const int32_t sp = p.fac_sp[(size_t)r * p.P + f];
            for (int j = 0; j < ord; j++) {
                if (j == 0)
                    o << "            acc = df_mul_fu(acc, c.n[" << sp << "]);\n";
                else
                    o << "            acc = df_mul_fu(acc, fmaxf(__fadd_rn(c.n[" << sp << "], -" << j
                      << ".0f), 0.0f));\n";
            }
        }
        if (r == 0)
            o << "            sum = RunSum{acc.h, acc.l};\n";
        else
            o << "            rs_add(sum, acc);\n";
        o << "            cum[" << r << "] = sum.s;\n        }\n";
    }
    o << "        tot = rs_total(sum);\n";
    o << "        return !(lo >= 0.0f && hi < 8388608.0f);\n    }\n";
    o << "    __device__ static int exact_choice(const SsaArgs &, const ExactTables &, const Counts &c, const int64_t "
         "*, int,\n                                       const uint64_t *rl, int RS, uint64_t u53) {\n";
    o << "        float cn[" << S << "];\n";
    for (int s = 0; s < S; s++) o << "        cn[" << s << "] = c.n[" << s << "];\n";
    o << "        return net_exact_choice(cn, rl, RS, u53);\n    }\n";
    // jump: per species, the sum of the deltas of the reaction that fired
    o << "    __device__ static void jump(Counts &c, const SsaArgs &, const ExactTables &, int64_t *, int, int idx) "
         "{\n";
    for (int s = 0; s < S; s++) {
        std::vector<std::pair<int, int64_t>> terms;
        for (int r = 0; r < R; r++) {
            int64_t d = 0;
            for (int k = 0; k < p.Q; k++)
                if (p.jmp_sp[(size_t)r * p.Q + k] == s) d += p.jmp_d[(size_t)r * p.Q + k];
            if (d != 0) terms.push_back({r, d});
        }
        if (terms.empty()) continue;
        o << "        c.n[" << s << "] +=";
        for (size_t k = 0; k < terms.size(); k++)
            o << (k ? " +" : "") << " (idx == " << terms[k].first << " ? " << terms[k].second << ".0f : 0.0f)";
        o << ";\n";
    }
    o << "    }\n};\n\n}  // namespace rbg\n\n";
    o << "extern \"C\" __global__ void __launch_bounds__(" << block << ", 1)\n"
         "rbg_net_kernel(const __grid_constant__ rbg::SsaArgs a) {\n    rbg::spec_body<rbg::NetOps>(a);\n}\n";
    return o.str();
}

namespace {

uint64_t image_key(const std::string &src, Nvrtc *nv) {
    int major = 0, minor = 0;
    if (nv) nv->version(&major, &minor);
    std::string keytext = src;
    for (int k = 0; k < kJitHeaderCount; k++) keytext += kJitHeaderSources[k];
    for (const std::string &opt : compile_options()) keytext += opt;
    keytext += std::to_string(major) + "." + std::to_string(minor);
    return fnv1a(keytext);
}

// Compiled image of the network's kernel, from the disk cache or NVRTC.
bool compile_image(const std::string &src, uint64_t key, Nvrtc *nv, std::string &image, bool compile = true) {
    char hex[17];
    std::snprintf(hex, sizeof hex, "%016llx", (unsigned long long)key);
    const std::string dir = cache_dir(), path = dir + "/net_" + hex + ".cubin";
    if (read_file(path, image)) return true;
    if (!compile) return false;
    if (!nv) {
        set_error("run-time network compilation unavailable: " + g_nvrtc.why);
        return false;
    }
    nvrtcProgram prog;
    if (nv->create(&prog, src.c_str(), "rbg_net.cu", kJitHeaderCount, kJitHeaderSources, kJitHeaderNames) !=
        NVRTC_SUCCESS) {
        set_error("nvrtcCreateProgram failed");
        return false;
    }
    std::vector<const char *> opts;
    for (const std::string &opt : compile_options()) opts.push_back(opt.c_str());
    const nvrtcResult rc = nv->compile(prog, (int)opts.size(), opts.data());
    if (rc != NVRTC_SUCCESS) {
        size_t n = 0;
        nv->log_size(prog, &n);
        std::string log(n, '\0');
        if (n) nv->log(prog, &log[0]);
        nv->destroy(&prog);
        set_error("network kernel compilation failed: " + log.substr(0, 4000));
        return false;
    }
    size_t n = 0;
    nv->cubin_size(prog, &n);
    image.assign(n, '\0');
    nv->cubin(prog, &image[0]);
    nv->destroy(&prog);
    mkdirs(dir);
    write_file_atomic(path, image);
    return true;
}

}  // namespace

bool jit_compile(const Packed &p, int block, size_t *image_bytes) {
    std::lock_guard<std::mutex> lk(g_mu);
    const std::string src = jit_net_source(p, block);
    Nvrtc *nv = nvrtc();
    std::string image;
    if (!compile_image(src, image_key(src, nv), nv, image)) return false;
    if (image_bytes) *image_bytes = image.size();
    return true;
}

namespace {
// Background compiles, joined when the library unloads (this object is
// destroyed before the statics the compiles use, which are defined above).
struct Background {
    std::mutex mu;
    std::set<uint64_t> started;
    std::vector<std::thread> threads;
    ~Background() {
        for (std::thread &t : threads)
            if (t.joinable()) t.join();
    }
} g_background;
}  // namespace

void jit_compile_async(const Packed &p, int block) {
    const uint64_t key = fnv1a(jit_net_source(p, block));
    std::lock_guard<std::mutex> lk(g_background.mu);
    if (!g_background.started.insert(key).second) return;
    g_background.threads.emplace_back([p, block]() {
        size_t n = 0;
        jit_compile(p, block, &n);  // failures leave the descriptor kernel in use
    });
}

const void *jit_kernel(const Packed &p, int block, bool compile) {
    std::lock_guard<std::mutex> lk(g_mu);
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaGetDevice failed");
        return nullptr;
    }
    const std::string src = jit_net_source(p, block);
    Nvrtc *nv = nvrtc();
    const uint64_t key = image_key(src, nv);
    auto it = g_loaded.find({dev, key});
    if (it != g_loaded.end()) return (const void *)it->second.kern;
    std::string image;
    if (!compile_image(src, key, nv, image, compile)) return nullptr;
    Loaded l;
    if (cudaLibraryLoadData(&l.lib, image.data(), nullptr, nullptr, 0, nullptr, nullptr, 0) != cudaSuccess ||
        cudaLibraryGetKernel(&l.kern, l.lib, "rbg_net_kernel") != cudaSuccess) {
        cudaGetLastError();
        set_error("loading the compiled network kernel failed");
        return nullptr;
    }
    g_loaded[{dev, key}] = l;
    return (const void *)l.kern;
}

int jit_block() {
    if (const char *e = std::getenv("RB_JIT_BLOCK")) return std::max(32, std::min(1024, std::atoi(e) / 32 * 32));
    return 384;
}

int launch_ssa_jit(const void *kern, const SsaArgs &a, int block, int grid, size_t smem, cudaStream_t st) {
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return (int)err;
    void *args[] = {(void *)&a};
    err = cudaLaunchKernel(kern, dim3(grid), dim3(block), args, smem, st);
    return (int)err;
}

}  // namespace rbg
