// Run-time specialised sweep kernels (see jit_dev.cuh for the device side).
//
// A planned sweep is written out as a CUDA source whose gates are calls of
// the jit_dev.cuh templates with every structural property as a template
// argument, compiled by NVRTC straight to an sm_103a cubin, loaded with the
// runtime's library API (cudaLibraryLoadData / cudaLibraryGetKernel) and
// launched like k_sweep, directly or inside the sweep's CUDA graph.  NVRTC is
// opened with dlopen: where it is missing, flushes keep the interpreted
// k_sweep (also CUDA) and jit_last_error() says why.
//
// The engine's device headers travel inside the library (jit_sources.inc,
// written by the build from csrc/), so the source tree need not exist where
// the library runs.  NVRTC has no C library headers; it gets a stdint.h of
// its own below, and the headers leave their host-only parts out under
// __CUDACC_RTC__.
#include "jit.h"

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <exception>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "jit_sources.inc"  // kJitHeaderNames[], kJitHeaderSources[], kJitHeaderCount (build output)

namespace kbwg {
namespace {

// ---- NVRTC, opened at run time ----------------------------------------------------
typedef int nvrtcResult;
typedef struct _nvrtcProgram *nvrtcProgram;

struct Nvrtc {
    nvrtcResult (*create)(nvrtcProgram *, const char *, const char *, int, const char *const *,
                          const char *const *) = nullptr;
    nvrtcResult (*compile)(nvrtcProgram, int, const char *const *) = nullptr;
    nvrtcResult (*destroy)(nvrtcProgram *) = nullptr;
    nvrtcResult (*log_size)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*log)(nvrtcProgram, char *) = nullptr;
    nvrtcResult (*cubin_size)(nvrtcProgram, size_t *) = nullptr;
    nvrtcResult (*cubin)(nvrtcProgram, char *) = nullptr;
    bool ok = false;
    std::string why;
};

const Nvrtc &nvrtc() {
    static Nvrtc n = [] {
        Nvrtc r;
        std::vector<std::string> names = {"libnvrtc.so.13", "libnvrtc.so"};
        for (const char *env : {"CUDA_HOME", "CUDA_PATH"}) {
            const char *d = getenv(env);
            if (d && *d) names.push_back(std::string(d) + "/lib64/libnvrtc.so.13");
        }
        names.push_back("/usr/local/cuda/lib64/libnvrtc.so.13");
        names.push_back("/usr/local/cuda/targets/sbsa-linux/lib/libnvrtc.so.13");
        void *h = nullptr;
        for (const std::string &nm : names)
            if ((h = dlopen(nm.c_str(), RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
        if (!h) {
            r.why = "NVRTC (libnvrtc.so.13) not found";
            return r;
        }
        auto sym = [&](const char *s) { return dlsym(h, s); };
        r.create = (decltype(r.create))sym("nvrtcCreateProgram");
        r.compile = (decltype(r.compile))sym("nvrtcCompileProgram");
        r.destroy = (decltype(r.destroy))sym("nvrtcDestroyProgram");
        r.log_size = (decltype(r.log_size))sym("nvrtcGetProgramLogSize");
        r.log = (decltype(r.log))sym("nvrtcGetProgramLog");
        r.cubin_size = (decltype(r.cubin_size))sym("nvrtcGetCUBINSize");
        r.cubin = (decltype(r.cubin))sym("nvrtcGetCUBIN");
        r.ok = r.create && r.compile && r.destroy && r.log_size && r.log && r.cubin_size && r.cubin;
        if (!r.ok) r.why = "NVRTC lacks an expected entry point";
        return r;
    }();
    return n;
}

// C library types for the device headers (LP64, as on the host)
const char kStdint[] =
    "#pragma once\n"
    "typedef signed char int8_t; typedef unsigned char uint8_t;\n"
    "typedef short int16_t; typedef unsigned short uint16_t;\n"
    "typedef int int32_t; typedef unsigned int uint32_t;\n"
    "typedef long int64_t; typedef unsigned long uint64_t;\n"
    "typedef unsigned long uintptr_t;\n";

struct Compiled {
    cudaLibrary_t lib = nullptr;
    cudaKernel_t kernel = nullptr;
};

std::mutex g_mu;
std::unordered_map<std::string, Compiled> g_cache;     // full source (+ entry) -> loaded kernel
std::unordered_map<std::string, std::string> g_cubins;  // source -> cubin compiled in the background
std::string g_last_error;
JitStats g_stats;

void note_error(const std::string &e) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_last_error = e;
    g_stats.failed++;
}

std::string program_log(const Nvrtc &nv, nvrtcProgram prog) {
    size_t n = 0;
    nv.log_size(prog, &n);
    std::string log(n, '\0');
    if (n) nv.log(prog, &log[0]);
    return log;
}

// Compile one source to a cubin; empty on failure (error noted).
std::string compile_cubin(const std::string &src) {
    const Nvrtc &nv = nvrtc();
    if (!nv.ok) {
        note_error(nv.why);
        return std::string();
    }
    std::vector<const char *> names, bodies;
    names.push_back("stdint.h");
    bodies.push_back(kStdint);
    for (int i = 0; i < kJitHeaderCount; i++) {
        names.push_back(kJitHeaderNames[i]);
        bodies.push_back(kJitHeaderSources[i]);
    }
    nvrtcProgram prog = nullptr;
    if (nv.create(&prog, src.c_str(), "kbwg_jit.cu", (int)names.size(), bodies.data(), names.data()) != 0) {
        note_error("nvrtcCreateProgram failed");
        return std::string();
    }
    // KBWG_JIT_DUMP=<dir>: keep each source there (for reading);
    // KBWG_JIT_VERBOSE=1: print ptxas' register and spill counts to stderr;
    // KBWG_JIT_OPTS: extra NVRTC options, separated by spaces
    const char *dump = getenv("KBWG_JIT_DUMP");
    if (dump && *dump) {
        char path[4096];
        snprintf(path, sizeof path, "%s/kbwg_jit_%016llx.cu", dump,
                 (unsigned long long)std::hash<std::string>()(src));
        if (FILE *f = fopen(path, "w")) {
            fwrite(src.data(), 1, src.size(), f);
            fclose(f);
        }
    }
    const char *verbose = getenv("KBWG_JIT_VERBOSE");
    const bool info = verbose && *verbose && *verbose != '0';
    std::vector<const char *> opts = {"--gpu-architecture=sm_103a", "-std=c++17", "-DKBWG_JIT_KERNEL=1"};
    if (info) opts.push_back("--ptxas-options=-v");
    std::vector<std::string> extra;
    if (const char *xo = getenv("KBWG_JIT_OPTS")) {
        std::string cur;
        for (const char *c = xo;; c++) {
            if (*c == ' ' || *c == '\0') {
                if (!cur.empty()) extra.push_back(cur);
                cur.clear();
                if (*c == '\0') break;
            } else {
                cur += *c;
            }
        }
    }
    for (const std::string &x : extra) opts.push_back(x.c_str());
    const nvrtcResult rc = nv.compile(prog, (int)opts.size(), opts.data());
    std::string cubin;
    if (rc != 0) {
        note_error("NVRTC compilation failed: " + program_log(nv, prog).substr(0, 4000));
    } else {
        if (info) fprintf(stderr, "kbwg jit: %s\n", program_log(nv, prog).c_str());
        size_t n = 0;
        nv.cubin_size(prog, &n);
        cubin.resize(n);
        if (n) nv.cubin(prog, &cubin[0]);
    }
    nv.destroy(&prog);
    return cubin;
}

const void *load_kernel(const std::string &cubin, const char *entry, Compiled &c) {
    cudaError_t e = cudaLibraryLoadData(&c.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&c.kernel, c.lib, entry);
    if (e != cudaSuccess) {
        note_error(std::string("loading a compiled sweep kernel failed: ") + cudaGetErrorString(e));
        if (c.lib) cudaLibraryUnload(c.lib);
        c = Compiled();
        return nullptr;
    }
    return (const void *)c.kernel;
}

int env_int(const char *name, int dflt) {
    const char *v = getenv(name);
    if (!v || !*v) return dflt;
    return atoi(v);
}

const char *kClassName[] = {"TG_X", "TG_Y", "TG_H", "TG_RX", "TG_RY", "TG_Z", "TG_P", "TG_RZ", "TG_PI", "TG_SCALE"};

// fn(w) for w in [0, count) on up to 32 threads.  An exception in an item
// (an allocation failing) stops the remaining items and is rethrown on the
// calling thread once every worker has joined.
void run_parallel(size_t count, const std::function<void(size_t)> &fn, bool on_device = true) {
    const size_t hw = std::max<size_t>(1, std::thread::hardware_concurrency());
    const size_t nthreads = std::min<size_t>(count, std::min<size_t>(hw, 32));
    std::atomic<size_t> next{0};
    int dev = 0;
    const bool have_dev = on_device && cudaGetDevice(&dev) == cudaSuccess;
    std::mutex emu;
    std::exception_ptr first;
    auto worker = [&]() {
        if (have_dev) cudaSetDevice(dev);  // library loads happen on the caller's device
        try {
            for (size_t w; (w = next.fetch_add(1)) < count;) fn(w);
        } catch (...) {
            std::lock_guard<std::mutex> lk(emu);
            if (!first) first = std::current_exception();
            next.store(count);
        }
    };
    std::vector<std::thread> pool;
    try {
        for (size_t t = 1; t < nthreads; t++) pool.emplace_back(worker);
    } catch (...) {  // fewer threads than asked: the ones started and this one share the items
    }
    worker();
    for (std::thread &t : pool) t.join();
    if (first) std::rethrow_exception(first);
}

}  // namespace

bool jit_available() { return nvrtc().ok; }

std::string jit_last_error() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_last_error;
}

JitStats jit_stats() {
    std::lock_guard<std::mutex> lk(g_mu);
    return g_stats;
}

int jit_default_mode() {
    static const int m = std::min(std::max(env_int("KBWG_JIT", 1), 0), 2);
    return m;
}

uint32_t jit_min_qubits() {
    static const uint32_t q = (uint32_t)std::max(env_int("KBWG_JIT_MIN_QUBITS", 20), 0);
    return q;
}

namespace {

// The constants expression of gate i (a load of its program entry, or the
// zero constants for a gate that needs none).
std::string constants_of(const TileGate &t, size_t i) {
    const bool needs_k = !(t.cls == TG_X || t.cls == TG_Y || t.cls == TG_Z || t.cls == TG_PI ||
                           (t.cls == TG_H && t.sub == 1));
    if (!needs_k) return "kz";
    char buf[64];
    snprintf(buf, sizeof buf, "P::load(sg[%zu])", i);
    return buf;
}

// Predicate of the controls on this stage's lane/warp bits ("true" if none).
std::string fok_of(const TileGate &t) {
    if (!t.fneed) return "true";
    char buf[96];
    snprintf(buf, sizeof buf, "((F & 0x%xu) == 0x%xu)", t.fneed, t.fneed);
    return buf;
}

// Side of a diagonal gate's target that is fixed per thread (DFIX gates).
std::string side_of(const TileGate &t) {
    char buf[96];
    if (t.cls == TG_SCALE)
        snprintf(buf, sizeof buf, "true");
    else if (t.tb == TG_OUTER)
        snprintf(buf, sizeof buf, "((base >> %u) & 1u) != 0u", (unsigned)t.tout);
    else
        snprintf(buf, sizeof buf, "((F >> %u) & 1u) != 0u", (unsigned)t.tb);
    return buf;
}

// Condition of a gate's controls outside the tile ("" if none).
std::string outer_cond(const TileGate &t, bool wide) {
    if (!t.co) return "";
    char buf[96];
    if (wide)
        snprintf(buf, sizeof buf, "((base & 0x%llxull) == 0x%llxull)", (unsigned long long)t.co,
                 (unsigned long long)t.co);
    else
        snprintf(buf, sizeof buf, "((base & 0x%xu) == 0x%xu)", (uint32_t)t.co, (uint32_t)t.co);
    return buf;
}

// Statement applying gate t (constants in `k`) to the registers `v`, with
// its controls on lane/warp bits and the condition `outer` of its controls
// outside the tile ("": none, or left to the caller).  Lane-bit gates,
// register-bit X and diagonal gates take the condition as a per-register
// select; other register-bit gates run under a branch.
std::string gate_stmt(const TileGate &t, const char *v, const char *k, const std::string &outer) {
    char buf[512];
    const char *cls = kClassName[t.cls];
    const int q = (t.cls == TG_PI) ? (int)t.c[0] : 0;
    std::string cond;
    if (t.fneed) cond = fok_of(t);
    if (!outer.empty()) cond = cond.empty() ? outer : cond + " && " + outer;
    const std::string c = cond.empty() ? "true" : cond;
    if (t.op < OP_REG) {
        snprintf(buf, sizeof buf, "jit::lane<P, R, %d, %s, 0x%xu, %d>(%s, %s, %s, F);", (int)t.tb, cls, t.creg,
                 (int)t.sub, v, k, c.c_str());
        return buf;
    }
    if (t.op < OP_DREG) {
        if (!cond.empty() && t.cls == TG_X) {
            snprintf(buf, sizeof buf, "jit::cswap<P, R, %d, 0x%xu>(%s, %s);", (int)t.rb, (unsigned)t.jm, v, c.c_str());
            return buf;
        }
        snprintf(buf, sizeof buf, "jit::reg<P, R, %d, %s, 0x%xu, %d>(%s, %s);", (int)t.rb, cls, (unsigned)t.jm,
                 (int)t.sub, v, k);
        return cond.empty() ? std::string(buf) : "if (" + cond + ") { " + buf + " }";
    }
    if (t.op < OP_DFIX)
        snprintf(buf, sizeof buf, "jit::dreg<P, R, %d, %s, 0x%xu, %d>(%s, %s, %s);", (int)t.rb, cls, (unsigned)t.jm, q,
                 v, k, c.c_str());
    else
        snprintf(buf, sizeof buf, "jit::dfix<P, R, %s, 0x%xu, %d>(%s, %s, %s, %s);", cls, (unsigned)t.jm, q, v, k,
                 side_of(t).c_str(), c.c_str());
    return buf;
}

// Guard of a gate with controls outside the tile (uniform over the tile).
std::string outer_guard(const TileGate &t, const std::string &body, bool wide) {
    if (!t.co) return body;
    char buf[128];
    if (wide)
        snprintf(buf, sizeof buf, "if ((base & 0x%llxull) == 0x%llxull) { ", (unsigned long long)t.co,
                 (unsigned long long)t.co);
    else
        snprintf(buf, sizeof buf, "if ((base & 0x%xu) == 0x%xu) { ", (uint32_t)t.co, (uint32_t)t.co);
    return std::string(buf) + body + " }";
}

}  // namespace

std::string jit_sweep_source(const JitGeometry &geo, const PlannedSweep &sw) {
    std::string s;
    s.reserve(4096 + 160 * sw.gates.size());
    char buf[512];
    const int first = sw.stage_layout.empty() ? (int)LAYOUT_A : (int)sw.stage_layout.front();
    const int last = sw.stage_layout.empty() ? (int)LAYOUT_A : (int)sw.stage_layout.back();
    s += "#include \"jit_dev.cuh\"\n"
         "using namespace kbwg;\n"
         "namespace {\n";
    s += geo.wide ? "typedef uint64_t BaseT;\n" : "typedef uint32_t BaseT;\n";
    s += "struct Body {\n";
    s += "  static constexpr int kFirst = " + std::to_string(first) + ", kLast = " + std::to_string(last) + ";\n";
    s += "  template <class P, int K, int R>\n"
         "  static __device__ __forceinline__ void run(typename P::Amp (&v)[1 << R], typename P::Amp *tile,\n"
         "      uint32_t FA, uint32_t FB, BaseT base, const TileGate *sg) {\n"
         "    const typename P::K4 kz{};\n";
    s += std::string("    uint32_t F = ") + (first == LAYOUT_A ? "FA" : "FB") + ";\n";
    s += "    (void)tile; (void)base; (void)sg; (void)kz; (void)F;\n";
    int layout = first;
    size_t g0 = 0;
    for (size_t st = 0; st < sw.stage_layout.size(); st++) {
        const int nl = sw.stage_layout[st];
        if (nl != layout) {
            snprintf(buf, sizeof buf, "    jit::relayout<P, K, R, %d, %d>(v, tile, FA, FB); F = %s;\n", layout, nl,
                     nl == LAYOUT_A ? "FA" : "FB");
            s += buf;
            layout = nl;
        }
        const size_t g1 = sw.stage_end[st];
        for (size_t i = g0; i < g1; i++) {
            const TileGate &t = sw.gates[i];
            s += "    " + gate_stmt(t, "v", constants_of(t, i).c_str(), outer_cond(t, geo.wide)) + "\n";
        }
        g0 = g1;
    }
    s += "  }\n};\n}  // namespace\n";
    snprintf(buf, sizeof buf,
             "extern \"C\" __global__ void __launch_bounds__(%d, %d)\n"
             "kbwg_jit_sweep(%s::Mem *__restrict__ st, const __grid_constant__ SweepParams p) {\n"
             "  jit::sweep<%s, %d, %d, Body, %s>(st, p);\n}\n",
             geo.threads, geo.ctas_per_sm, geo.policy, geo.policy, geo.K, geo.R, geo.wide ? "true" : "false");
    s += buf;
    return s;
}

std::string jit_adjoint_source(const JitGeometry &geo, const PlannedSweep &sw, const std::vector<uint32_t> &ginfo) {
    std::string s;
    s.reserve(4096 + 320 * sw.gates.size());
    char buf[512];
    const int first = sw.stage_layout.empty() ? (int)LAYOUT_A : (int)sw.stage_layout.front();
    const int last = sw.stage_layout.empty() ? (int)LAYOUT_A : (int)sw.stage_layout.back();
    s += "#include \"adjoint_dev.cuh\"\n"
         "using namespace kbwg;\n"
         "namespace {\n"
         "struct Body {\n";
    s += "  static constexpr int kFirst = " + std::to_string(first) + ", kLast = " + std::to_string(last) + ";\n";
    s += "  template <class P, int K, int R>\n"
         "  static __device__ __forceinline__ void run(typename P::Amp (&vp)[1 << R], typename P::Amp (&vl)[1 << R],\n"
         "      typename P::Amp *tp, typename P::Amp *tl, uint32_t FA, uint32_t FB, uint64_t base,\n"
         "      const TileGate *sg, typename Grad<P>::Wacc *acc) {\n"
         "    using G = Grad<P>;\n"
         "    const typename P::K4 kz{};\n";
    s += std::string("    uint32_t F = ") + (first == LAYOUT_A ? "FA" : "FB") + ";\n";
    s += "    (void)tp; (void)tl; (void)base; (void)sg; (void)kz; (void)F; (void)acc;\n";
    static const char *kGradName[] = {"GT_NONE", "GT_X", "GT_Y", "GT_Z", "GT_P1"};
    int layout = first;
    size_t g0 = 0;
    for (size_t st = 0; st < sw.stage_layout.size(); st++) {
        const int nl = sw.stage_layout[st];
        if (nl != layout) {
            snprintf(buf, sizeof buf, "    jit::relayout2<P, K, R, %d, %d>(vp, vl, tp, tl, FA, FB); F = %s;\n", layout,
                     nl, nl == LAYOUT_A ? "FA" : "FB");
            s += buf;
            layout = nl;
        }
        const size_t g1 = sw.stage_end[st];
        for (size_t i = g0; i < g1; i++) {
            const TileGate &t = sw.gates[i];
            const int gt = (int)(ginfo[i] & 15u);
            const unsigned slot = ginfo[i] >> 4;
            std::string body;
            if (gt != GT_NONE) {
                const char *gn = kGradName[gt];
                std::string expr;
                if (gt == GT_Z || gt == GT_P1) {
                    if (t.op >= OP_DREG && t.op < OP_DFIX)
                        snprintf(buf, sizeof buf, "jit::grad_dreg<P, R, %s, %d, 0x%xu>(vp, vl)", gn, (int)t.rb, t.creg);
                    else
                        snprintf(buf, sizeof buf, "jit::grad_dfix<P, R, %s, 0x%xu>(vp, vl, %s)", gn, t.creg,
                                 side_of(t).c_str());
                    expr = "if (" + fok_of(t) + ") part = " + std::string(buf) + ";";
                } else if (t.op < OP_REG) {
                    snprintf(buf, sizeof buf, "part = jit::grad_lane<P, R, %s, %d, 0x%xu>(vp, vl, %s, F);", gn,
                             (int)t.tb, t.creg, fok_of(t).c_str());
                    expr = buf;
                } else {
                    snprintf(buf, sizeof buf, "jit::grad_reg<P, R, %s, %d, 0x%xu>(vp, vl)", gn, (int)t.rb, t.creg);
                    expr = "if (" + fok_of(t) + ") part = " + std::string(buf) + ";";
                }
                snprintf(buf, sizeof buf, " jit::grad_store<P, %u>(acc, part);", slot);
                body += "{ typename G::Acc part = G::zero(); " + expr + buf + " } ";
            }
            const std::string k = constants_of(t, i);
            if (k != "kz") body += "const typename P::K4 k = " + k + "; ";
            const char *kv = (k != "kz") ? "k" : "kz";
            body += gate_stmt(t, "vp", kv, "") + " " + gate_stmt(t, "vl", kv, "");
            s += "    " + outer_guard(t, "{ " + body + " }", true) + "\n";
        }
        g0 = g1;
    }
    s += "  }\n};\n}  // namespace\n";
    snprintf(buf, sizeof buf,
             "extern \"C\" __global__ void __launch_bounds__(%d, %d)\n"
             "kbwg_jit_adjoint(%s::Mem *__restrict__ phi, %s::Mem *__restrict__ lam, const __grid_constant__ AdjParams a) {\n"
             "  jit::adjoint_sweep<%s, %d, %d, Body>(phi, lam, a);\n}\n",
             geo.threads, geo.ctas_per_sm, geo.policy, geo.policy, geo.policy, geo.K, geo.R);
    s += buf;
    return s;
}

const void *jit_kernel(const std::string &src, const char *entry) {
    const std::string key = src + '\0' + entry;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_cache.find(key);
        if (it != g_cache.end()) {
            g_stats.reused++;
            return (const void *)it->second.kernel;
        }
    }
    std::string cubin;
    bool fresh = false;
    double dt = 0.0;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_cubins.find(src);
        if (it != g_cubins.end()) {
            cubin.swap(it->second);
            g_cubins.erase(it);
        }
    }
    if (cubin.empty()) {
        const auto t0 = std::chrono::steady_clock::now();
        cubin = compile_cubin(src);
        dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        fresh = true;
    }
    if (cubin.empty()) return nullptr;
    Compiled c;
    const void *k = load_kernel(cubin, entry, c);
    std::lock_guard<std::mutex> lk(g_mu);
    g_stats.compile_s += dt;
    if (!k) return nullptr;
    if (fresh) g_stats.compiled++;
    auto ins = g_cache.emplace(key, c);
    if (!ins.second) {  // another thread loaded the same source meanwhile: keep one
        cudaLibraryUnload(c.lib);
        return (const void *)ins.first->second.kernel;
    }
    return k;
}

size_t jit_compile_only(const std::vector<std::string> &srcs) {
    if (!jit_available()) {
        note_error(nvrtc().why);
        return srcs.size();
    }
    std::atomic<size_t> failed{0};
    run_parallel(srcs.size(), [&](size_t w) {
        const auto t0 = std::chrono::steady_clock::now();
        const bool ok = !compile_cubin(srcs[w]).empty();
        const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::lock_guard<std::mutex> lk(g_mu);
        g_stats.compile_s += dt;
        if (ok)
            g_stats.compiled++;
        else
            failed++;
    });
    return failed.load();
}

// ---- background compilation -----------------------------------------------------
struct JitJob {
    std::vector<std::string> srcs;
    std::atomic<bool> done{false};
    std::mutex mu;
    std::condition_variable cv;
};

namespace {
// Worker threads of the background jobs.  Defined after the caches it fills,
// so it is destroyed first at exit: the destructor stops the jobs between
// compilations and joins them while the caches still exist.
struct Runner {
    std::mutex mu;
    std::vector<std::pair<std::thread, std::shared_ptr<JitJob>>> threads;
    std::atomic<bool> stop{false};
    ~Runner() {
        stop = true;
        std::lock_guard<std::mutex> lk(mu);
        for (auto &t : threads)
            if (t.first.joinable()) t.first.join();
    }
};
Runner g_runner;

// Stop the background jobs between compilations and join them.  A job still
// inside NVRTC when the process runs its exit handlers would crash the exit:
// NVRTC registers its own teardown lazily, during its first compilations, so
// it can run before any handler registered earlier.  Callers therefore stop
// the jobs before exit (kbwg_jit_shutdown; the Python binding registers it
// with Python's atexit, which runs before the C exit handlers); the atexit
// registration below is a best effort for hosts that do not.
void stop_jobs() {
    g_runner.stop = true;
    std::vector<std::thread> ts;
    {
        std::lock_guard<std::mutex> lk(g_runner.mu);
        for (auto &t : g_runner.threads)
            if (t.first.joinable()) ts.push_back(std::move(t.first));
    }
    for (std::thread &t : ts) t.join();
}

void run_job_body(const std::shared_ptr<JitJob> &job) {
    std::vector<size_t> todo;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        for (size_t i = 0; i < job->srcs.size(); i++) {
            const std::string &src = job->srcs[i];
            if (g_cubins.count(src) || g_cache.count(src + '\0' + "kbwg_jit_sweep")) continue;
            bool dup = false;
            for (size_t j : todo) dup = dup || job->srcs[j] == src;
            if (!dup) todo.push_back(i);
        }
    }
    run_parallel(
        todo.size(),
        [&](size_t w) {
            if (g_runner.stop) return;
            const std::string &src = job->srcs[todo[w]];
            const auto t0 = std::chrono::steady_clock::now();
            std::string cubin = compile_cubin(src);
            const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            std::lock_guard<std::mutex> lk(g_mu);
            g_stats.compile_s += dt;
            if (cubin.empty()) return;
            g_stats.compiled++;
            g_cubins.emplace(src, std::move(cubin));
        },
        false);
}

// A background job: its kernels compiled into the cubin cache.  Whatever
// happens (an allocation failing), the job ends done, so that waiters return;
// structures without a cubin then keep their interpreted kernels.
void run_job(std::shared_ptr<JitJob> job) {
    try {
        run_job_body(job);
    } catch (...) {
        note_error("background compilation stopped: host allocation failed");
    }
    {
        std::lock_guard<std::mutex> lk(job->mu);
        job->srcs.clear();  // the cubins are in the cache; the sources are no longer needed
        job->srcs.shrink_to_fit();
        job->done = true;
    }
    job->cv.notify_all();
}
}  // namespace

void jit_shutdown() { stop_jobs(); }

std::shared_ptr<JitJob> jit_prefetch(std::vector<std::string> srcs) {
    auto job = std::make_shared<JitJob>();
    job->srcs = std::move(srcs);
    if (g_runner.stop) {  // shut down: nothing more is compiled in the background
        job->done = true;
        return job;
    }
    if (!jit_available()) {
        note_error(nvrtc().why);
        job->done = true;
        return job;
    }
    static std::once_flag registered;
    std::call_once(registered, [] { std::atexit(stop_jobs); });
    std::lock_guard<std::mutex> lk(g_runner.mu);
    // join the workers of finished jobs
    for (size_t i = 0; i < g_runner.threads.size();) {
        if (g_runner.threads[i].second->done && g_runner.threads[i].first.joinable()) {
            g_runner.threads[i].first.join();
            g_runner.threads.erase(g_runner.threads.begin() + (std::ptrdiff_t)i);
        } else {
            i++;
        }
    }
    g_runner.threads.emplace_back(std::thread(run_job, job), job);
    return job;
}

bool jit_job_done(const JitJob &job) { return job.done.load(); }

void jit_job_wait(JitJob &job) {
    std::unique_lock<std::mutex> lk(job.mu);
    job.cv.wait(lk, [&] { return job.done.load(); });
}

bool jit_sweep_kernels(const JitGeometry &geo, const std::vector<PlannedSweep> &plan, std::vector<const void *> &out) {
    out.assign(plan.size(), nullptr);
    if (!jit_available()) {
        note_error(nvrtc().why);
        return false;
    }
    std::vector<std::string> srcs(plan.size());
    for (size_t i = 0; i < plan.size(); i++) srcs[i] = jit_sweep_source(geo, plan[i]);
    // distinct sources not compiled yet are compiled in parallel
    std::vector<size_t> todo;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        for (size_t i = 0; i < plan.size(); i++) {
            auto it = g_cache.find(srcs[i] + '\0' + "kbwg_jit_sweep");
            if (it != g_cache.end()) {
                out[i] = (const void *)it->second.kernel;
                g_stats.reused++;
            } else {
                bool dup = false;
                for (size_t j : todo) dup = dup || srcs[j] == srcs[i];
                if (!dup) todo.push_back(i);
            }
        }
    }
    if (!todo.empty()) run_parallel(todo.size(), [&](size_t w) { jit_kernel(srcs[todo[w]], "kbwg_jit_sweep"); });
    bool all = true;
    for (size_t i = 0; i < plan.size(); i++) {
        if (!out[i]) out[i] = jit_kernel(srcs[i], "kbwg_jit_sweep");
        all = all && out[i] != nullptr;
    }
    return all;
}

}  // namespace kbwg
