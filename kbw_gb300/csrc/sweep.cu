// Fused tile sweep: one pass over the state applies every gate of a sweep.
//
// A tile is 2^K amplitudes: its local bits 0..l-1 are the global qubits
// 0..l-1 (a contiguous chunk of 2^l amplitudes) and its local bits l..K-1 are
// m = K-l arbitrary higher qubits, so a tile is 2^m chunks.  Persistent CTAs
// (two or three per SM, by the register budget of the geometry) walk the
// tiles; per CTA:
//   * once per launch the sweep's gate program and the chunk-offset table are
//     staged in shared memory;
//   * per tile, warp 0 issues one TMA bulk copy (cp.async.bulk ... mbarrier::
//     complete_tx) per chunk into the CTA's shared-memory tile, waited on an
//     mbarrier with a bounded try_wait loop;
//   * each thread takes 2^R amplitudes into registers: local bits 0..4 map to
//     the lane, R contiguous local bits to the register index, the remaining
//     bits to the warp (layout A holds bits [5,5+R), layout B [K-R,K));
//   * gates run in program order of their stage: targets on register bits as
//     in-thread pairs, on bits 0..4 through warp shuffles, diagonal gates on
//     any bit (even outside the tile) in place; controls outside the tile are
//     one predicate per tile; a stage change re-distributes the tile through
//     shared memory;
//   * as soon as the tile buffer is no longer read, the next tile's TMA load
//     is issued, and the finished amplitudes are stored straight from
//     registers with coalesced 32-amplitude warp stores.
#include <string.h>

#include <algorithm>
#include <memory>
#include <type_traits>

#include <math.h>

#include "../../include/kbwg.h"
#include "jit.h"
#include "kernels.h"
#include "sim.h"
#include "sweep_dev.cuh"

namespace kbwg {

// C++ names of the arithmetic policies, for the run-time specialised kernels.
template <class P> struct PolicyName;
template <> struct PolicyName<Exact<float>> { static constexpr const char *s = "kbwg::Exact<float>"; };
template <> struct PolicyName<Exact<double>> { static constexpr const char *s = "kbwg::Exact<double>"; };
template <> struct PolicyName<Fast<double>> { static constexpr const char *s = "kbwg::Fast<double>"; };
template <> struct PolicyName<FastP> { static constexpr const char *s = "kbwg::FastP"; };
template <> struct PolicyName<FF2> { static constexpr const char *s = "kbwg::FF2"; };

template <class P, int K, int R>
struct SweepKernel {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    static_assert(sizeof(Amp) == sizeof(Mem), "register and memory amplitudes share the tile buffer");
    static constexpr int kThreads = 32 << (K - kLaneBits - R);
    static constexpr size_t kTileBytes = sizeof(Mem) << K;
    static constexpr size_t kChunkTable = 256 * sizeof(uint64_t);
    static constexpr size_t kSmem = kTileBytes + kChunkTable + kMaxSweepGates * sizeof(TileGate) + 16;
    static constexpr int kCtasPerSm = (R == 3) ? 3 : 2;  // register budget: 80 resp. 128 (c128) / 64 (c64)
    // register layouts A = bits [5, 5+R) and B = [K-R, K) must cover every
    // local bit above the lanes, or a gate on the gap could never run
    static_assert(K <= kLaneBits + 2 * R, "tile geometry leaves local bits no layout holds in registers");
};

// W: 64-bit state indices (registers above 32 qubits); the 32-bit form keeps
// registers free for the amplitudes.
template <class P, int K, int R, bool W>
__global__ void __launch_bounds__(SweepKernel<P, K, R>::kThreads, SweepKernel<P, K, R>::kCtasPerSm)
    k_sweep(typename P::Mem *__restrict__ st, const __grid_constant__ SweepParams p) {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    using SK = SweepKernel<P, K, R>;
    using B = typename pick_t<W, uint64_t, uint32_t>::type;
    constexpr int NR = 1 << R;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Amp *tile = reinterpret_cast<Amp *>(smem_raw);
    Mem *tile_mem = reinterpret_cast<Mem *>(smem_raw);
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(smem_raw + SK::kTileBytes);
    TileGate *sg = reinterpret_cast<TileGate *>(smem_raw + SK::kTileBytes + SK::kChunkTable);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + SK::kTileBytes + SK::kChunkTable +
                                                 kMaxSweepGates * sizeof(TileGate));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t l = p.l, m = p.m;
    const uint32_t chunk = 1u << l, nchunks = 1u << m;
    const uint32_t chunk_bytes = chunk * (uint32_t)sizeof(Mem);
    const uint64_t lowmask = chunk - 1;

    // --- prologue: program, chunk table, barrier ---
    for (uint32_t i = threadIdx.x; i < p.gate_count; i += blockDim.x) sg[i] = p.prog[i];
    for (uint32_t c = threadIdx.x; c < nchunks; c += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
        chunk_off[c] = off;
    }
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto tile_base = [&](uint32_t tau) {
        B b = (B)tau << l;
        for (uint32_t j = 0; j < m; j++) b = (B)insert_zero_at(b, p.hq[j]);
        return b;
    };
    auto issue_load = [&](uint32_t tau) {
        if (warp == 0) {
            const uint64_t b = tile_base(tau);
            if (lane == 0) mbar_expect_tx(bar, (uint32_t)SK::kTileBytes);
            __syncwarp();
            for (uint32_t c = lane; c < nchunks; c += 32)
                tma_load(tile_mem + (size_t)c * chunk, st + b + chunk_off[c], chunk_bytes, bar);
        }
    };

    uint32_t tau = blockIdx.x;
    if (tau < p.tiles) issue_load(tau);
    const uint32_t FA = (uint32_t)lane | ((uint32_t)warp << (kLaneBits + R));
    const uint32_t FB = (uint32_t)lane | ((uint32_t)warp << kLaneBits);
    for (uint32_t it = 0; tau < p.tiles; tau += gridDim.x, it++) {
        const B base = tile_base(tau);
        if (!tile_wait(bar, it & 1u, p.err)) return;
        Amp v[NR];
        int layout = p.stage_layout[0];
        int R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
        uint32_t F = (layout == LAYOUT_A) ? FA : FB;
#pragma unroll
        for (int j = 0; j < NR; j++) v[j] = P::from_mem(tile_mem[F | ((uint32_t)j << R0)]);
        // (each position is read and later rewritten by the same thread, so
        // register-format data may replace memory-format data without a barrier)
        uint32_t g0 = 0;
        for (uint32_t s = 0; s < p.nstages; s++) {
            const int nl = p.stage_layout[s];
            if (nl != layout) {
#pragma unroll
                for (int j = 0; j < NR; j++) tile[F | ((uint32_t)j << R0)] = v[j];
                __syncthreads();
                layout = nl;
                R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
                F = (layout == LAYOUT_A) ? FA : FB;
#pragma unroll
                for (int j = 0; j < NR; j++) v[j] = tile[F | ((uint32_t)j << R0)];
            }
            const uint32_t g1 = p.stage_end[s];
            for (uint32_t gi = g0; gi < g1; gi++) tile_gate<P, K, R, B>(sg[gi], v, R0, F, base);
            g0 = g1;
        }
        // the tile buffer is free: start the next tile's load, then store this one
        fence_proxy_async();
        __syncthreads();
        const uint32_t next = tau + gridDim.x;
        if (next < p.tiles) issue_load(next);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t u = F | ((uint32_t)j << R0);
            st[base + chunk_off[u >> l] + (u & lowmask)] = P::to_mem(v[j]);
        }
    }
}

// Diagnostic of the failure path: one CTA waits through tile_wait on an
// mbarrier nothing arrives on, so its polls run out and it sets the error
// flag and returns, as a tile kernel whose copies never completed would.
__global__ void k_wait_probe(int *err, uint32_t spins) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    tile_wait(&bar, 0, err, spins);
}

cudaError_t launch_wait_probe(int *err, uint32_t spins, cudaStream_t s) {
    k_wait_probe<<<1, 64, 0, s>>>(err, spins);
    count_launch();
    return cudaGetLastError();
}

// ---- replay cache ------------------------------------------------------------------
// A flush whose gate structure (kinds, targets and controls, after the
// float-float rewrite) matches an earlier flush of the handle reuses that
// flush's plan, its device program buffer and an instantiated CUDA graph of
// its sweep launches: only the gate constants are re-packed and uploaded.
// Parameter sweeps (VQE, parameter shift) and repeated circuits skip the
// planner and the per-launch host overhead.
struct SweepGraph {
    const void *kernel = nullptr;   // which k_sweep instantiation
    size_t specialised = 0;         // sweeps that run a run-time specialised kernel
    std::vector<uint64_t> sig;      // structure of the flushed gate list
    std::vector<uint32_t> src;      // program slot -> index in the flushed list
    std::vector<TileGate> planned;  // program with unpacked constants
    void *dprog = nullptr;
    cudaGraphExec_t exec = nullptr;
    size_t sweeps = 0;
    uint64_t last_use = 0;
};
// A background compilation of the specialised kernels of one structure
// (auto mode), started on its second flush.
struct SpecialisedJob {
    uint64_t key = 0;                 // structure hash (with kernel and depth)
    std::shared_ptr<JitJob> job;
    bool used = false;                // its kernels were loaded into a flush once
};
struct GraphCache {
    std::vector<SweepGraph> entries;
    std::vector<uint64_t> seen;  // structure hashes flushed once (a graph is built on the second time)
    std::vector<SpecialisedJob> jobs;
    uint64_t clock = 0;
};
// (an adjoint gradient alone brings two structures per checkpoint segment:
// its forward and its reverse sweeps)
constexpr size_t kJobEntries = 128;
constexpr size_t kSeenEntries = 256;
constexpr size_t kGraphCacheEntries = 64;  // (an adjoint's forward pass flushes one structure per segment)

static void free_entry(SweepGraph &g) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    if (g.dprog) cudaFree(g.dprog);
    g.exec = nullptr;
    g.dprog = nullptr;
}

void release_graphs(Sim &s) {
    GraphCache *c = (GraphCache *)s.graphs;
    if (!c) return;
    for (SweepGraph &g : c->entries) free_entry(g);
    delete c;
    s.graphs = nullptr;
}

static uint64_t hash_of(const std::vector<uint64_t> &sig) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a over the words
    for (uint64_t w : sig) {
        h ^= w;
        h *= 1099511628211ull;
    }
    return h;
}

// Kind, target and controls of every gate; for the float-float path's
// |1> * i^q gates also q, which the specialised kernels compile in.
static std::vector<uint64_t> structure_of(const GateDesc *gates, size_t count) {
    std::vector<uint64_t> sig(2 * count);
    for (size_t i = 0; i < count; i++) {
        sig[2 * i] = (uint64_t)gates[i].kind | ((uint64_t)gates[i].target << 8);
        if (gates[i].kind == G_PI) sig[2 * i] |= (uint64_t)(int)gates[i].c[0] << 40;
        sig[2 * i + 1] = gates[i].ctrl;
    }
    return sig;
}

// Pack the planned program with the constants of `gates` and upload it.
template <class P>
static cudaError_t upload_program(Sim &s, const std::vector<TileGate> &planned, const std::vector<uint32_t> &src,
                                  const GateDesc *gates, void *dst) {
    std::vector<TileGate> prog = planned;
    for (size_t i = 0; i < prog.size(); i++) {
        memcpy(prog[i].c, gates[src[i]].c, sizeof prog[i].c);
        P::pack_host(prog[i]);
    }
    // pageable source: the call returns once the host buffer is consumed
    return copy_async(dst, prog.data(), prog.size() * sizeof(TileGate), cudaMemcpyHostToDevice, s.stream);
}

template <class P, int K, int R, bool W = false>
static cudaError_t run_fused_p(Sim &s, const GateDesc *gates, size_t count) {
    using SK = SweepKernel<P, K, R>;
    using Mem = typename P::Mem;
    int num_sms = 0;
    {
        cudaError_t e = ensure_smem_limit((const void *)k_sweep<P, K, R, W>, SK::kSmem);
        if (e == cudaSuccess) e = current_sm_count(num_sms);
        if (e != cudaSuccess) return e;
    }
    const void *kid = (const void *)k_sweep<P, K, R, W>;
    const size_t depth = s.fusion_depth ? s.fusion_depth : (size_t)kMaxSweepGates;
    // timed profiling marks every launch with events, which a graph replay cannot
    const bool graphs_ok = !s.prof.on && !(s.flags & KBWG_FLAG_NO_GRAPHS);
    // auto mode: specialised kernels come from a background compilation
    // started on a structure's second flush; until it is done the
    // interpreted kernel runs (same amplitudes), then the structure's graph is
    // rebuilt once with the specialised kernels
    const bool auto_jit = s.jit_mode == KBWG_JIT_AUTO && s.n >= jit_min_qubits();
    bool repeat = false;  // this gate structure was flushed before on the handle
    SpecialisedJob *job = nullptr;
    std::vector<uint64_t> sig;
    uint64_t h = 0;
    if (graphs_ok || s.jit_mode == KBWG_JIT_AUTO) {
        if (!s.graphs) s.graphs = new GraphCache();
        GraphCache &gc = *(GraphCache *)s.graphs;
        sig = structure_of(gates, count);
        sig.push_back((uint64_t)(uintptr_t)kid);
        sig.push_back(depth);
        h = hash_of(sig);
        for (uint64_t x : gc.seen) repeat = repeat || x == h;
        if (!repeat) {  // first sight of this structure: launch directly, remember it
            if (gc.seen.size() >= kSeenEntries) gc.seen.erase(gc.seen.begin());
            gc.seen.push_back(h);
        }
        if (auto_jit)
            for (SpecialisedJob &j : gc.jobs)
                if (j.key == h) job = &j;
        const bool jit_ready = job && !job->used && jit_job_done(*job->job);
        if (graphs_ok)
            for (size_t gi = 0; gi < gc.entries.size(); gi++) {
                SweepGraph &g = gc.entries[gi];
                if (g.kernel != kid || g.sig != sig) continue;
                if (jit_ready && g.specialised == 0) {  // rebuild it with the specialised kernels
                    cudaStreamSynchronize(s.stream);    // its program buffer may still be read
                    free_entry(g);
                    gc.entries.erase(gc.entries.begin() + (long)gi);
                    break;
                }
                cudaError_t e = upload_program<P>(s, g.planned, g.src, gates, g.dprog);
                if (e != cudaSuccess) return e;
                e = cudaGraphLaunch(g.exec, s.stream);
                if (e != cudaSuccess) return e;
                for (size_t i = 0; i < g.sweeps; i++) count_launch();
                g.last_use = ++gc.clock;
                s.last_passes = g.sweeps;
                s.last_specialised = g.specialised;
                return cudaSuccess;
            }
    }
    const bool graphs = graphs_ok && repeat;  // a graph is built on the second sight
    std::vector<PlannedSweep> plan =
        plan_sweeps(s.n, K, R, gates, count, (s.flags & KBWG_FLAG_EXACT_ORDER) != 0, depth);
    std::vector<TileGate> planned;
    std::vector<uint32_t> src;
    for (const PlannedSweep &sw : plan) {
        planned.insert(planned.end(), sw.gates.begin(), sw.gates.end());
        src.insert(src.end(), sw.src.begin(), sw.src.end());
    }
    const size_t total = planned.size();
    if (total != count) return cudaErrorInvalidValue;  // the planner could not place every gate
    void *dbuf = nullptr;
    cudaError_t e;
    if (graphs) {
        e = cudaMalloc(&dbuf, std::max<size_t>(total, 1) * sizeof(TileGate));
        if (e != cudaSuccess) return e;
    } else {
        e = s.tmp4.ensure(total * sizeof(TileGate));
        if (e != cudaSuccess) return e;
        dbuf = s.tmp4.ptr;
    }
    e = upload_program<P>(s, planned, src, gates, dbuf);
    if (e != cudaSuccess) {
        if (graphs) cudaFree(dbuf);
        return e;
    }
    const TileGate *dprog = (const TileGate *)dbuf;
    const uint64_t tiles = 1ull << (s.n - K);
    const uint64_t grid = std::min<uint64_t>(tiles, (uint64_t)num_sms * SK::kCtasPerSm);
    // Run-time specialised kernels (jit.cpp): for a structure flushed before
    // on a large enough state (from its second flush, which also builds its
    // graph), or on every flush in KBWG_JIT_ALWAYS mode.  A sweep whose kernel
    // could not be built runs the interpreted k_sweep.
    std::vector<const void *> jk;
    const JitGeometry geo{PolicyName<P>::s, K, R, SK::kThreads, SK::kCtasPerSm, W};
    bool load_jit = s.jit_mode == KBWG_JIT_ALWAYS;
    if (auto_jit && repeat) {
        if (!job) {  // start compiling this structure's kernels in the background
            std::vector<std::string> srcs;
            for (const PlannedSweep &sw : plan) srcs.push_back(jit_sweep_source(geo, sw));
            GraphCache &gc = *(GraphCache *)s.graphs;
            if (gc.jobs.size() >= kJobEntries) gc.jobs.erase(gc.jobs.begin());
            SpecialisedJob nj;
            nj.key = h;
            nj.job = jit_prefetch(std::move(srcs));
            gc.jobs.push_back(nj);
        } else if (jit_job_done(*job->job)) {
            load_jit = true;
            job->used = true;
        }
    }
    if (load_jit) {
        jit_sweep_kernels(geo, plan, jk);
        for (const void *f : jk) {
            if (!f) continue;
            e = ensure_smem_limit(f, SK::kSmem);
            if (e != cudaSuccess) {
                if (graphs) cudaFree(dbuf);
                return e;
            }
        }
    }
    size_t specialised = 0;
    if (graphs) {
        e = cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) {
            cudaFree(dbuf);
            return e;
        }
    }
    size_t off = 0;
    for (const PlannedSweep &sw : plan) {
        SweepParams p;
        memset(&p, 0, sizeof p);
        p.hmask = sw.hmask;
        p.l = sw.l;
        p.m = sw.m;
        memcpy(p.hq, sw.hq, sizeof p.hq);
        p.nstages = (uint32_t)sw.stage_layout.size();
        p.gate_count = (uint32_t)sw.gates.size();
        for (uint32_t i = 0; i < p.nstages; i++) {
            p.stage_layout[i] = sw.stage_layout[i];
            p.stage_end[i] = sw.stage_end[i];
        }
        p.prog = dprog + off;
        p.err = s.d_err;
        p.tiles = tiles;
        off += sw.gates.size();
        if (s.prof.on) s.prof.mark(s.stream);
        const void *spec = jk.empty() ? nullptr : jk[(size_t)(&sw - plan.data())];
        if (spec) {
            Mem *stp = (Mem *)s.state;
            void *args[] = {(void *)&stp, (void *)&p};
            cudaLaunchKernel(spec, dim3((unsigned)grid), dim3(SK::kThreads), args, SK::kSmem, s.stream);
            specialised++;
        } else {
            k_sweep<P, K, R, W><<<(unsigned)grid, SK::kThreads, SK::kSmem, s.stream>>>((Mem *)s.state, p);
        }
        if (!graphs) count_launch();
        e = cudaGetLastError();
        if (s.prof.on) {
            s.prof.mark(s.stream);
            s.prof.bytes += 2.0 * (double)s.elem * (double)s.ns;
        }
        if (e != cudaSuccess) break;
    }
    s.last_passes = plan.size();
    s.last_specialised = specialised;
    if (!graphs) return e;
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s.stream, &graph);
    if (e == cudaSuccess) e = ec;
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e == cudaSuccess) e = cudaGraphLaunch(exec, s.stream);
    if (e != cudaSuccess) {
        if (exec) cudaGraphExecDestroy(exec);
        cudaStreamSynchronize(s.stream);
        cudaFree(dbuf);
        return e;
    }
    for (size_t i = 0; i < plan.size(); i++) count_launch();
    GraphCache &gc = *(GraphCache *)s.graphs;
    if (gc.entries.size() >= kGraphCacheEntries) {  // evict the least recently used
        size_t lru = 0;
        for (size_t i = 1; i < gc.entries.size(); i++)
            if (gc.entries[i].last_use < gc.entries[lru].last_use) lru = i;
        cudaStreamSynchronize(s.stream);  // its program buffer may still be read
        free_entry(gc.entries[lru]);
        gc.entries.erase(gc.entries.begin() + (long)lru);
    }
    SweepGraph g;
    g.kernel = kid;
    g.specialised = specialised;
    g.sig = std::move(sig);
    g.src = std::move(src);
    g.planned = std::move(planned);
    g.dprog = dbuf;
    g.exec = exec;
    g.sweeps = plan.size();
    g.last_use = ++gc.clock;
    gc.entries.push_back(std::move(g));
    return cudaSuccess;
}

// Tile sizes with a compiled sweep kernel, per arithmetic, default first:
// complex64 13 (16 amplitudes per thread, 512 threads), 12 (16, 256) and 11
// (8, 256); binary64 complex128 12 (16) and 11 (8); float-float complex128
// 11 (8) and 12 (16).  The order-preserving mode has the default only.
std::vector<uint32_t> compiled_tiles(const Sim &s) {
    if (s.flags & KBWG_FLAG_EXACT_ORDER) return {(uint32_t)(s.prec ? TileCfg<double>::K : TileCfg<float>::K)};
    // registers above 32 qubits: the default geometry, with 64-bit state indices
    if (s.n > 32) {
        if (ff_capable(s)) return {(uint32_t)TileCfgFF::K};
        return {(uint32_t)(s.prec ? TileCfg<double>::K : TileCfg<float>::K)};
    }
    if (ff_capable(s)) return {(uint32_t)TileCfgFF::K, 12u};
    if (s.prec) return {(uint32_t)TileCfg<double>::K, 11u};
    return {(uint32_t)TileCfg<float>::K, 12u, 11u};
}

// The default tile: the arithmetic's default, or for a state smaller than
// that the largest tile that fits (below every tile: one kernel per gate).
// A whole small state in one tile is not preferred: one CTA on one SM ran the
// 12-qubit Grover circuit slower (2.8 ms) than two 11-qubit tiles on two SMs
// in five times as many sweeps (1.8 ms).
uint32_t tile_register_bits(const Sim &s, uint32_t k) {
    const std::vector<uint32_t> ks = compiled_tiles(s);
    bool found = false;
    for (uint32_t x : ks) found = found || x == k;
    if (!found) return 0;
    if (s.flags & KBWG_FLAG_EXACT_ORDER) return (uint32_t)(s.prec ? TileCfg<double>::R : TileCfg<float>::R);
    return k == 11 ? 3u : 4u;  // the 2^11 tiles hold 8 amplitudes per thread, the larger ones 16
}

uint32_t default_tile_k(const Sim &s) {
    const std::vector<uint32_t> ks = compiled_tiles(s);
    if (ks[0] <= s.n) return ks[0];
    uint32_t fit = 0;
    for (uint32_t k : ks)
        if (k <= s.n && k > fit) fit = k;
    return fit ? fit : ks[0];
}

std::vector<uint32_t> tile_options(const Sim &s) {
    std::vector<uint32_t> out;
    if (s.flags & KBWG_FLAG_NO_FUSION) return out;
    const uint32_t def = default_tile_k(s);
    if (def <= s.n) out.push_back(def);
    for (uint32_t k : compiled_tiles(s))
        if (k <= s.n && k != def) out.push_back(k);
    return out;
}

// The handle's tile size: its setting when a kernel exists for it and the
// state is at least one tile, else the default.
static uint32_t chosen_tile(const Sim &s) {
    if (s.tile_k)
        for (uint32_t k : tile_options(s))
            if (k == s.tile_k) return k;
    return default_tile_k(s);
}

uint32_t effective_tile_k(const Sim &s) {
    if (s.flags & KBWG_FLAG_NO_FUSION) return 0;
    const uint32_t k = chosen_tile(s);
    return k <= s.n ? k : 0;
}

template <class T>
static cudaError_t run_fused_t(Sim &s, const GateDesc *gates, size_t count) {
    constexpr int K = TileCfg<T>::K, R = TileCfg<T>::R;
    if (s.n > 32) {  // 64-bit state indices, default geometry
        if (s.flags & KBWG_FLAG_EXACT_ORDER) return run_fused_p<Exact<T>, K, R, true>(s, gates, count);
        if constexpr (std::is_same<T, float>::value) return run_fused_p<FastP, K, R, true>(s, gates, count);
        else return run_fused_p<Fast<T>, K, R, true>(s, gates, count);
    }
    const uint32_t tk = chosen_tile(s);
    if (tk != (uint32_t)K && !(s.flags & KBWG_FLAG_EXACT_ORDER)) {
        if constexpr (std::is_same<T, float>::value) {
            if (tk == 12) return run_fused_p<FastP, 12, 4>(s, gates, count);
            if (tk == 11) return run_fused_p<FastP, 11, 3>(s, gates, count);
        } else {
            if (tk == 11) return run_fused_p<Fast<T>, 11, 3>(s, gates, count);
        }
    }
    if (s.n < (uint32_t)K) {
        for (size_t i = 0; i < count; i++) {
            if (s.prof.on) s.prof.mark(s.stream);
            cudaError_t e = launch_gate1<T>(s.state, s.n, gates[i], s.stream);
            if (s.prof.on) {
                s.prof.mark(s.stream);
                s.prof.bytes += 2.0 * (double)s.elem * (double)s.ns;
            }
            if (e != cudaSuccess) return e;
        }
        s.last_passes = count;
        return cudaSuccess;
    }
    if (s.flags & KBWG_FLAG_EXACT_ORDER) return run_fused_p<Exact<T>, K, R>(s, gates, count);
    if constexpr (std::is_same<T, float>::value) return run_fused_p<FastP, K, R>(s, gates, count);
    else return run_fused_p<Fast<T>, K, R>(s, gates, count);
}

// Complex128 float-float path: rewrite the queue so that uncontrolled H
// drops its 1/sqrt(2) and uncontrolled RZ(t) becomes the phase gate
// diag(1, e^{it}), collecting the dropped factors 2^{-1/2} and e^{-it/2} in
// one complex scale g, applied as a final gate (and earlier if |g| would
// leave float range).  P(+-pi/2) and P(pi) become exact multiplications by
// i^q.  Everything else keeps the binary64 constants of Dense<f64>.
static std::vector<GateDesc> ff_rewrite(const GateDesc *gates, size_t count) {
    std::vector<GateDesc> out;
    out.reserve(count + 2);
    double gr = 1.0, gi = 0.0;
    int unscaled = 0;
    auto emit_scale = [&]() {
        GateDesc sc;
        memset(&sc, 0, sizeof sc);
        sc.kind = G_SCALE;
        sc.target = 0;
        sc.c[0] = gr;
        sc.c[1] = gi;
        out.push_back(sc);
        gr = 1.0;
        gi = 0.0;
        unscaled = 0;
    };
    for (size_t i = 0; i < count; i++) {
        GateDesc x = gates[i];
        if (x.kind == G_H && x.ctrl == 0) {
            x.kind = G_HN;
            gr *= 0.70710678118654752440;
            gi *= 0.70710678118654752440;
            if (++unscaled >= 100) {
                out.push_back(x);
                emit_scale();
                continue;
            }
        } else if (x.kind == G_RZ && x.ctrl == 0) {
            // diag(u0, u1) = u0 diag(1, u1 conj(u0)) for unit u0 (for RZ(t):
            // u1 conj(u0) = e^{it}; also a folded general diagonal)
            const double c = x.c[2] * x.c[0] + x.c[3] * x.c[1], sn = x.c[3] * x.c[0] - x.c[2] * x.c[1];
            const double nr = gr * x.c[0] - gi * x.c[1], ni = gr * x.c[1] + gi * x.c[0];
            gr = nr;
            gi = ni;
            x.kind = G_P;
            x.c[0] = c;
            x.c[1] = sn;
            x.c[2] = x.c[3] = 0.0;
        }
        if (x.kind == G_P) {
            const double c = x.c[0], sn = x.c[1], t = 1e-15;
            int q = 0;
            if (fabs(c) < t && fabs(sn - 1.0) < t) q = 1;
            else if (fabs(c + 1.0) < t && fabs(sn) < t) q = 2;
            else if (fabs(c) < t && fabs(sn + 1.0) < t) q = 3;
            if (q) {
                x.kind = G_PI;
                x.c[0] = (double)q;
                x.c[1] = 0.0;
            }
        }
        out.push_back(x);
    }
    if (gr != 1.0 || gi != 0.0) emit_scale();
    return out;
}

std::vector<const void *> specialised_kernels(Sim &s, const std::vector<std::string> &srcs, const char *entry,
                                              bool *final) {
    std::vector<const void *> out(srcs.size(), nullptr);
    if (final) *final = false;
    if (s.jit_mode == KBWG_JIT_OFF || srcs.empty()) return out;
    if (s.jit_mode == KBWG_JIT_AUTO && s.n < jit_min_qubits()) return out;
    if (s.jit_mode == KBWG_JIT_AUTO) {
        if (!s.graphs) s.graphs = new GraphCache();
        GraphCache &gc = *(GraphCache *)s.graphs;
        uint64_t h = 1469598103934665603ull;  // FNV-1a over the sources
        for (const std::string &src : srcs)
            for (unsigned char c : src) {
                h ^= c;
                h *= 1099511628211ull;
            }
        SpecialisedJob *job = nullptr;
        for (SpecialisedJob &j : gc.jobs)
            if (j.key == h) job = &j;
        if (!job) {
            bool repeat = false;
            for (uint64_t x : gc.seen) repeat = repeat || x == h;
            if (!repeat) {  // first sight: remember it
                if (gc.seen.size() >= kSeenEntries) gc.seen.erase(gc.seen.begin());
                gc.seen.push_back(h);
                return out;
            }
            if (gc.jobs.size() >= kJobEntries) gc.jobs.erase(gc.jobs.begin());
            SpecialisedJob nj;
            nj.key = h;
            nj.job = jit_prefetch(srcs);
            gc.jobs.push_back(nj);
            return out;
        }
        if (!jit_job_done(*job->job)) return out;
        job->used = true;
    }
    for (size_t i = 0; i < srcs.size(); i++) out[i] = jit_kernel(srcs[i], entry);
    if (final) *final = true;
    return out;
}

bool wait_specialised(Sim &s) {
    GraphCache *gc = (GraphCache *)s.graphs;
    if (!gc) return false;
    bool waited = false;
    for (SpecialisedJob &j : gc->jobs)
        if (!j.used) {
            jit_job_wait(*j.job);
            waited = true;
        }
    return waited;
}

bool ff_capable(const Sim &s) {
    // (one kernel per gate, KBWG_FLAG_NO_FUSION, runs on binary64)
    return s.prec && (s.flags & KBWG_FLAG_FAST_C128) && !(s.flags & KBWG_FLAG_NO_FUSION) &&
           s.n >= (uint32_t)TileCfgFF::K;
}

cudaError_t ensure_binary64(Sim &s) {
    if (!s.ff_resident) return cudaSuccess;
    s.ff_resident = false;
    return launch_ff_convert(s.state, s.n, false, s.stream);
}

cudaError_t init_state(Sim &s) {
    if (ff_capable(s)) {
        s.ff_resident = true;
        return launch_init_ff(s.state, s.n, s.stream);
    }
    s.ff_resident = false;
    return s.prec ? launch_init<double>(s.state, s.n, s.stream) : launch_init<float>(s.state, s.n, s.stream);
}

// ---- compile-only check of the specialised kernels (no GPU) --------------------
template <class P, int K, int R>
static size_t check_p(const Sim &s, const GateDesc *gates, size_t count, size_t &sweeps) {
    using SK = SweepKernel<P, K, R>;
    const size_t depth = s.fusion_depth ? s.fusion_depth : (size_t)kMaxSweepGates;
    const std::vector<PlannedSweep> plan =
        plan_sweeps(s.n, K, R, gates, count, (s.flags & KBWG_FLAG_EXACT_ORDER) != 0, depth);
    const JitGeometry geo{PolicyName<P>::s, K, R, SK::kThreads, SK::kCtasPerSm, s.n > 32};
    std::vector<std::string> srcs;
    for (const PlannedSweep &sw : plan) srcs.push_back(jit_sweep_source(geo, sw));
    sweeps = plan.size();
    return jit_compile_only(srcs);
}

template <class T>
static size_t check_t(const Sim &s, const GateDesc *gates, size_t count, size_t &sweeps) {
    constexpr int K = TileCfg<T>::K, R = TileCfg<T>::R;
    const uint32_t tk = chosen_tile(s);
    if (tk != (uint32_t)K && !(s.flags & KBWG_FLAG_EXACT_ORDER)) {
        if constexpr (std::is_same<T, float>::value) {
            if (tk == 12) return check_p<FastP, 12, 4>(s, gates, count, sweeps);
            if (tk == 11) return check_p<FastP, 11, 3>(s, gates, count, sweeps);
        } else {
            if (tk == 11) return check_p<Fast<T>, 11, 3>(s, gates, count, sweeps);
        }
    }
    sweeps = 0;
    if (s.n < (uint32_t)K) return 0;
    if (s.flags & KBWG_FLAG_EXACT_ORDER) return check_p<Exact<T>, K, R>(s, gates, count, sweeps);
    if constexpr (std::is_same<T, float>::value) return check_p<FastP, K, R>(s, gates, count, sweeps);
    else return check_p<Fast<T>, K, R>(s, gates, count, sweeps);
}

size_t jit_check(const Sim &s, const GateDesc *gates, size_t count, size_t &sweeps) {
    std::vector<GateDesc> folded;
    if (!(s.flags & (KBWG_FLAG_EXACT_ORDER | KBWG_FLAG_NO_FOLD))) {
        folded = fold_diagonals(gates, count);
        gates = folded.data();
        count = folded.size();
    }
    if (ff_capable(s)) {
        std::vector<GateDesc> g = ff_rewrite(gates, count);
        if (chosen_tile(s) == 12) return check_p<FF2, 12, 4>(s, g.data(), g.size(), sweeps);
        return check_p<FF2, TileCfgFF::K, TileCfgFF::R>(s, g.data(), g.size(), sweeps);
    }
    return s.prec ? check_t<double>(s, gates, count, sweeps) : check_t<float>(s, gates, count, sweeps);
}

cudaError_t run_fused(Sim &s, const GateDesc *gates, size_t count) {
    std::vector<GateDesc> folded;
    if (!(s.flags & (KBWG_FLAG_EXACT_ORDER | KBWG_FLAG_NO_FOLD))) {
        folded = fold_diagonals(gates, count);
        gates = folded.data();
        count = folded.size();
    }
    if (ff_capable(s)) {
        // float-float sweeps read and write the float-float form; the state
        // stays in it until an operation needs binary64
        if (!s.ff_resident) {
            cudaError_t e = launch_ff_convert(s.state, s.n, true, s.stream);
            if (e != cudaSuccess) return e;
            s.ff_resident = true;
        }
        std::vector<GateDesc> g = ff_rewrite(gates, count);
        if (s.n > 32) return run_fused_p<FF2, TileCfgFF::K, TileCfgFF::R, true>(s, g.data(), g.size());
        if (chosen_tile(s) == 12) return run_fused_p<FF2, 12, 4>(s, g.data(), g.size());
        return run_fused_p<FF2, TileCfgFF::K, TileCfgFF::R>(s, g.data(), g.size());
    }
    return s.prec ? run_fused_t<double>(s, gates, count) : run_fused_t<float>(s, gates, count);
}

}  // namespace kbwg
