// Many independent circuits in one persistent launch, each with its own
// gate list and Pauli-string Hamiltonian: the <H> of every circuit.
//
// The reference answers each request of BatchExecution::exp_value with a
// fresh simulator that replays the gates and sums the strings
// (kbw src/quantum_execution.rs:392-405, 109-158).  Here the host plans
// every circuit with the sweep planner (planner.cpp) into the gate programs
// the tile kernels run, and persistent CTAs take circuits from a queue
// sorted by cost (largest first):
//   * n <= K: the circuit runs on a K-qubit tile that never leaves the SM
//     (qubits n..K-1 stay |0>), its sweeps applied to the tile in registers
//     and shared memory;
//   * n > K: the state lives in the CTA's slot of a global buffer; every
//     planned sweep walks the slot tile by tile (TMA bulk loads, bounded
//     waits, coalesced stores), as k_sweep walks a handle's state.
// <H> = sum_k c_k <P_k> with P = i^{ny} X^x Z^z: the strings are grouped by
// flip mask x, and for each group one loop over the amplitudes forms
// conj(a_s) a_{s^x} once and adds every string's signed share, accumulated
// FP64-grade.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <exception>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/kbwg.h"
#include "kernels.h"
#include "sim.h"
#include "sweep_dev.cuh"

namespace kbwg {

struct BatchSweep {
    uint32_t l, m, nstages, gate_count;
    uint32_t gate_off, pad;
    uint8_t hq[16];
    uint8_t stage_layout[kMaxStages];
    uint16_t stage_end[kMaxStages];
};

struct BatchJob {
    uint32_t n, nsweeps, sweep_off, nterms;
    uint32_t term_off, id, pad;
    uint32_t pass_off, npasses;  // tiled <H> passes (registers larger than a tile)
};

struct BatchTerm {
    uint64_t x, z;
    double cr, ci;  // c_k * i^{ny}: the string's share of conj(a_s) a_{s^x} is sign * (cr p.re - ci p.im)
};

// One tiled <H> pass of a register larger than a tile: tiles of 2^K
// amplitudes (2^l contiguous ones per chunk, the chunks picked by the m
// qubits hq) hold both a_s and a_{s^x} for every string of the pass.
struct BatchPass {
    uint32_t l, m, term_off, nterms;
    uint8_t hq[16];
};
// A string of a pass: flip and phase masks on the tile's local bits, phase
// mask on the qubits outside it; `last` closes a run of strings with the
// same flip mask and coefficient (their signs are counted, the coefficient
// applied once); `newx`: the first string of a flip mask.
struct BatchTileTerm {
    uint32_t xl, zl;
    uint64_t zo;
    double cr, ci;
    uint32_t last, newx;
};

struct BatchArgs {
    const BatchJob *jobs;
    uint32_t njobs;
    unsigned *next;
    const BatchSweep *sweeps;
    const TileGate *prog;
    const BatchTerm *terms;
    const BatchPass *passes;
    const BatchTileTerm *tterms;
    double *energies;
    void *slots;
    uint64_t slot_elems;
    int *err;
};

template <class P, int K, int R>
struct BatchKernel {
    using Mem = typename P::Mem;
    static constexpr int kThreads = 32 << (K - kLaneBits - R);
    static constexpr size_t kTileBytes = sizeof(Mem) << K;
    static constexpr size_t kSmem = kTileBytes + 256 * sizeof(uint64_t) + kMaxSweepGates * sizeof(TileGate) + 64 +
                                    32 * 8 + 64;
};

// FP64-grade sum of float shares (short float runs, then widened) or of
// double shares
template <class T> struct BatchAcc {
    double v = 0.0;
    T part = (T)0;
    int cnt = 0;
    __device__ __forceinline__ void add(T x) {
        part += x;
        if (++cnt == 16) {
            v += (double)part;
            part = (T)0;
            cnt = 0;
        }
    }
    __device__ __forceinline__ double value() { return v + (double)part; }
};

template <class Mem>
__device__ __forceinline__ Mem batch_basis(bool one) {
    Mem m;
    m.re = one ? 1 : 0;
    m.im = 0;
    return m;
}

// <H> of a register larger than a tile, in tiled passes: each tile staged
// once per pass (TMA), every string of the pass summed from shared memory.
// (Its own function: the sweep loop keeps its register allocation.)
template <class P, int K, int R>
__device__ __noinline__ bool batch_energy_passes(const BatchArgs &a, const BatchJob &job, typename P::Mem *slot,
                                                 typename P::Mem *tile_mem, uint64_t *chunk_off, uint64_t *bar,
                                                 uint32_t &phase, double &sum) {
    using Mem = typename P::Mem;
    using T = decltype(Mem{}.re);
    BatchAcc<T> acc;  // (local: the caller's accumulator would live in memory across the call)
    using BK = BatchKernel<P, K, R>;
    constexpr int NR = 1 << R;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t n = job.n;
    for (uint32_t pi = 0; pi < job.npasses; pi++) {
        const BatchPass &bp = a.passes[job.pass_off + pi];
        const uint32_t l = bp.l, m = bp.m;
        const uint32_t chunk = 1u << l, nchunks = 1u << m;
        for (uint32_t c = threadIdx.x; c < nchunks; c += blockDim.x) {
            uint64_t off = 0;
            for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << bp.hq[j];
            chunk_off[c] = off;
        }
        __syncthreads();
        const uint64_t tiles = 1ull << (n - K);
        const BatchTileTerm *tt = a.tterms + bp.term_off;
        for (uint64_t tau = 0; tau < tiles; tau++) {
            uint64_t base = tau << l;
            for (uint32_t j = 0; j < m; j++) base = insert_zero_at(base, bp.hq[j]);
            if (warp == 0) {
                if (lane == 0) mbar_expect_tx(bar, (uint32_t)BK::kTileBytes);
                __syncwarp();
                for (uint32_t c = lane; c < nchunks; c += 32)
                    tma_load(tile_mem + (size_t)c * chunk, slot + base + chunk_off[c], chunk * (uint32_t)sizeof(Mem),
                             bar);
            }
            if (!tile_wait(bar, phase & 1u, a.err)) return false;
            phase++;
            // each thread's NR amplitudes u = tid + i * threads in registers;
            // strings outer (their fields read once per tile), signs counted
            // per amplitude, the product formed once per run
            T ar[NR], ai[NR];
            int cnt[NR];
#pragma unroll
            for (int i = 0; i < NR; i++) {
                const Mem m2 = tile_mem[threadIdx.x + (uint32_t)i * BK::kThreads];
                ar[i] = m2.re;
                ai[i] = m2.im;
                cnt[i] = 0;
            }
            for (uint32_t k = 0; k < bp.nterms; k++) {
                const BatchTileTerm t = tt[k];
                const uint32_t op = (uint32_t)__popcll(base & t.zo) & 1u;
#pragma unroll
                for (int i = 0; i < NR; i++) {
                    const uint32_t u = threadIdx.x + (uint32_t)i * BK::kThreads;
                    cnt[i] += (((uint32_t)__popc((u ^ t.xl) & t.zl) + op) & 1u) ? -1 : 1;
                }
                if (t.last) {  // (uniform)
#pragma unroll
                    for (int i = 0; i < NR; i++) {
                        const uint32_t u = threadIdx.x + (uint32_t)i * BK::kThreads;
                        T pr, pim;  // conj(a_u) a_{u^x}
                        if (t.xl == 0u) {
                            pr = ar[i] * ar[i] + ai[i] * ai[i];
                            pim = (T)0;
                        } else {
                            const Mem ax = tile_mem[u ^ t.xl];
                            pr = ar[i] * ax.re + ai[i] * ax.im;
                            pim = ar[i] * ax.im - ai[i] * ax.re;
                        }
                        acc.add((T)cnt[i] * ((T)t.cr * pr - (T)t.ci * pim));
                        cnt[i] = 0;
                    }
                }
            }
            __syncthreads();  // the tile is read no more: the next load may land
        }
    }
    sum = acc.value();
    return true;
}

template <class P, int K, int R>
__global__ void __launch_bounds__(BatchKernel<P, K, R>::kThreads, 2) k_batch_circuits(const __grid_constant__ BatchArgs a) {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    using T = decltype(Mem{}.re);
    using BK = BatchKernel<P, K, R>;
    constexpr int NR = 1 << R;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Amp *tile = reinterpret_cast<Amp *>(smem_raw);
    Mem *tile_mem = reinterpret_cast<Mem *>(smem_raw);
    unsigned char *q = smem_raw + BK::kTileBytes;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(q);
    q += 256 * sizeof(uint64_t);
    TileGate *sg = reinterpret_cast<TileGate *>(q);
    q += kMaxSweepGates * sizeof(TileGate);
    uint32_t *meta = reinterpret_cast<uint32_t *>(q);
    q += 64;
    double *red = reinterpret_cast<double *>(q);
    q += 32 * 8;
    uint64_t *bar = reinterpret_cast<uint64_t *>(q);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t FA = (uint32_t)lane | ((uint32_t)warp << (kLaneBits + R));
    const uint32_t FB = (uint32_t)lane | ((uint32_t)warp << kLaneBits);
    Mem *slot = reinterpret_cast<Mem *>(a.slots) + (size_t)blockIdx.x * a.slot_elems;
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    uint32_t phase = 0;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) meta[0] = atomicAdd(a.next, 1u);
        __syncthreads();
        const uint32_t jix = meta[0];
        if (jix >= a.njobs) break;
        const BatchJob job = a.jobs[jix];
        const uint32_t n = job.n;
        const bool in_tile = n <= (uint32_t)K;
        // ---- |0...0> ----
        if (in_tile) {
            for (uint32_t u = threadIdx.x; u < (1u << K); u += blockDim.x) tile[u] = P::from_mem(batch_basis<Mem>(u == 0));
        } else {
            for (uint64_t s = threadIdx.x; s < (1ull << n); s += blockDim.x) slot[s] = batch_basis<Mem>(s == 0);
            asm volatile("fence.proxy.async;" ::: "memory");  // generic stores before the sweeps' TMA reads
        }
        __syncthreads();
        // ---- the planned sweeps ----
        for (uint32_t sw = 0; sw < job.nsweeps; sw++) {
            const BatchSweep &bs = a.sweeps[job.sweep_off + sw];
            const uint32_t l = bs.l, m = bs.m, nst = bs.nstages;
            for (uint32_t i = threadIdx.x; i < bs.gate_count; i += blockDim.x) sg[i] = a.prog[bs.gate_off + i];
            for (uint32_t c = threadIdx.x; c < (1u << m); c += blockDim.x) {
                uint64_t off = 0;
                for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << bs.hq[j];
                chunk_off[c] = off;
            }
            __syncthreads();
            const uint64_t tiles = in_tile ? 1ull : (1ull << (n - K));
            const uint32_t chunk = 1u << l, nchunks = 1u << m;
            const uint64_t lowmask = chunk - 1;
            auto tile_base = [&](uint64_t t) {
                uint64_t b = t << l;
                for (uint32_t j = 0; j < m; j++) b = insert_zero_at(b, bs.hq[j]);
                return b;
            };
            // the slot's tiles: tile tau + 1's load is issued before tile tau's
            // stores (the tiles of a sweep are disjoint)
            auto issue_load = [&](uint64_t t) {
                if (warp == 0) {
                    const uint64_t b = tile_base(t);
                    if (lane == 0) mbar_expect_tx(bar, (uint32_t)BK::kTileBytes);
                    __syncwarp();
                    for (uint32_t c = lane; c < nchunks; c += 32)
                        tma_load(tile_mem + (size_t)c * chunk, slot + b + chunk_off[c], chunk * (uint32_t)sizeof(Mem),
                                 bar);
                }
            };
            if (!in_tile) issue_load(0);
            for (uint64_t tau = 0; tau < tiles; tau++) {
                const uint64_t base = tile_base(tau);
                int layout = bs.stage_layout[0];
                int R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
                uint32_t F = (layout == LAYOUT_A) ? FA : FB;
                Amp v[NR];
                if (in_tile) {
#pragma unroll
                    for (int j = 0; j < NR; j++) v[j] = tile[F | ((uint32_t)j << R0)];
                } else {
                    if (!tile_wait(bar, phase & 1u, a.err)) return;
                    phase++;
#pragma unroll
                    for (int j = 0; j < NR; j++) v[j] = P::from_mem(tile_mem[F | ((uint32_t)j << R0)]);
                }
                uint32_t g0 = 0;
                for (uint32_t s = 0; s < nst; s++) {
                    const int nl = bs.stage_layout[s];
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
                    const uint32_t g1 = bs.stage_end[s];
                    for (uint32_t gi = g0; gi < g1; gi++) tile_gate<P, K, R, uint64_t>(sg[gi], v, R0, F, base);
                    g0 = g1;
                }
                if (in_tile) {
                    // every thread rewrites the positions it read in this layout
#pragma unroll
                    for (int j = 0; j < NR; j++) tile[F | ((uint32_t)j << R0)] = v[j];
                } else {
                    // the tile buffer is read no more (next tile's load) once all threads pass here
                    fence_proxy_async();
                    __syncthreads();
                    if (tau + 1 < tiles) issue_load(tau + 1);
#pragma unroll
                    for (int j = 0; j < NR; j++) {
                        const uint32_t u = F | ((uint32_t)j << R0);
                        slot[base + chunk_off[u >> l] + (u & lowmask)] = P::to_mem(v[j]);
                    }
                }
            }
            if (!in_tile) asm volatile("fence.proxy.async;" ::: "memory");  // this sweep's stores before the next's loads
            __syncthreads();
        }
        // ---- <H> ----
        BatchAcc<T> acc;
        // tiled passes (registers larger than a tile)
        double tiled = 0.0;
        if (job.npasses && !batch_energy_passes<P, K, R>(a, job, slot, tile_mem, chunk_off, bar, phase, tiled)) return;
        const uint64_t ns = 1ull << n;
        for (uint32_t t0 = 0; t0 < job.nterms;) {
            const uint64_t x = a.terms[job.term_off + t0].x;
            uint32_t t1 = t0 + 1;
            while (t1 < job.nterms && a.terms[job.term_off + t1].x == x) t1++;
            for (uint64_t s = threadIdx.x; s < ns; s += blockDim.x) {
                Mem as, ax;
                if (in_tile) {
                    as = P::to_mem(tile[s]);
                    ax = P::to_mem(tile[s ^ x]);
                } else {
                    as = slot[s];
                    ax = slot[s ^ x];
                }
                // conj(a_s) a_{s^x}
                const T pr = as.re * ax.re + as.im * ax.im, pi = as.re * ax.im - as.im * ax.re;
                T share = (T)0;
                for (uint32_t k = t0; k < t1; k++) {
                    const BatchTerm &tk = a.terms[job.term_off + k];
                    const T w = (T)tk.cr * pr - (T)tk.ci * pi;
                    share += (__popcll((s ^ x) & tk.z) & 1) ? -w : w;
                }
                acc.add(share);
            }
            t0 = t1;
        }
        double e = acc.value() + tiled;
        for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
        if (lane == 0) red[warp] = e;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w2 = 0; w2 < (int)(blockDim.x >> 5); w2++) t += red[w2];
            a.energies[job.id] = t;
        }
    }
}

// ---- host side -----------------------------------------------------------------------
struct BatchCircuitIn {
    uint32_t n;
    std::vector<GateDesc> gates;
    std::vector<BatchTerm> terms;  // sorted by flip mask
    // the circuit's plan (batch_run)
    std::vector<BatchSweep> sweeps;
    std::vector<TileGate> prog;
    std::vector<BatchPass> passes;       // tiled <H> passes (n > K); then `terms`
    std::vector<BatchTileTerm> tterms;   // holds only the strings too wide for a tile
    bool placed = true;
    // validation result
    int32_t status = KBWG_OK;
    const char *error = nullptr;
};

// fn(i) for i in [0, n) on all host cores (items taken one at a time).  An
// exception in any item (an allocation failing) stops the remaining items and
// is rethrown here, on the calling thread, after every worker has joined.
template <class F>
static void batch_parallel_for(size_t n, F &&fn) {
    const size_t nt = std::min<size_t>(n, std::max(1u, std::thread::hardware_concurrency()));
    std::atomic<size_t> next{0};
    std::mutex mu;
    std::exception_ptr first;
    auto worker = [&]() {
        try {
            for (size_t i; (i = next.fetch_add(1, std::memory_order_relaxed)) < n;) fn(i);
        } catch (...) {
            std::lock_guard<std::mutex> lk(mu);
            if (!first) first = std::current_exception();
            next.store(n);
        }
    };
    std::vector<std::thread> pool;
    try {
        for (size_t t = 1; t < nt; t++) pool.emplace_back(worker);
    } catch (...) {  // fewer threads than asked: the ones started and this one share the items
    }
    worker();
    for (std::thread &t : pool) t.join();
    if (first) std::rethrow_exception(first);
}

template <class P, int K, int R>
static int32_t batch_run(int prec, std::vector<BatchCircuitIn> &circs, double *energies) {
    using BK = BatchKernel<P, K, R>;
    using Mem = typename P::Mem;
    auto fail = [](cudaError_t e, const char *what) {
        cudaGetLastError();
        set_error(e == cudaErrorMemoryAllocation ? KBWG_ENOMEM : KBWG_ECUDA,
                  std::string("batch circuits: ") + what + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? (int32_t)KBWG_ENOMEM : (int32_t)KBWG_ECUDA;
    };
    (void)prec;
    // plan every circuit (in parallel: the circuits are independent)
    batch_parallel_for(circs.size(), [&](size_t c) {
        BatchCircuitIn &ci = circs[c];
        const uint32_t nplan = std::max<uint32_t>(ci.n, (uint32_t)K);  // small registers padded with |0> qubits
        const std::vector<PlannedSweep> plan =
            plan_sweeps(nplan, K, R, ci.gates.data(), ci.gates.size(), false, kMaxSweepGates);
        size_t placed = 0;
        for (const PlannedSweep &sw : plan) {
            BatchSweep b;
            memset(&b, 0, sizeof b);
            b.l = sw.l;
            b.m = sw.m;
            memcpy(b.hq, sw.hq, sizeof b.hq);
            b.nstages = (uint32_t)sw.stage_layout.size();
            b.gate_count = (uint32_t)sw.gates.size();
            b.gate_off = (uint32_t)ci.prog.size();  // within the circuit; rebased below
            for (uint32_t i = 0; i < b.nstages; i++) {
                b.stage_layout[i] = sw.stage_layout[i];
                b.stage_end[i] = sw.stage_end[i];
            }
            for (TileGate t : sw.gates) {
                P::pack_host(t);
                ci.prog.push_back(t);
            }
            placed += sw.gates.size();
            ci.sweeps.push_back(b);
        }
        ci.placed = placed == ci.gates.size();
        if (ci.n > (uint32_t)K && !ci.terms.empty()) {
            std::vector<uint64_t> xm;
            for (const BatchTerm &t : ci.terms) xm.push_back(t.x);
            std::vector<size_t> wide;
            const std::vector<PauliPass> pp = plan_pauli_passes(ci.n, K, xm, (size_t)-1, wide);
            for (const PauliPass &ps : pp) {
                BatchPass b;
                memset(&b, 0, sizeof b);
                b.l = ps.l;
                b.m = ps.m;
                memcpy(b.hq, ps.hq, sizeof b.hq);
                b.term_off = (uint32_t)ci.tterms.size();  // within the circuit; rebased below
                std::vector<BatchTileTerm> ts;
                for (size_t k : ps.members) {
                    const BatchTerm &t = ci.terms[k];
                    BatchTileTerm q;
                    memset(&q, 0, sizeof q);
                    q.xl = ps.local(t.x);
                    q.zl = ps.local(t.z & ps.tile_mask);
                    q.zo = t.z & ~ps.tile_mask;
                    q.cr = t.cr;
                    q.ci = t.ci;
                    ts.push_back(q);
                }
                std::stable_sort(ts.begin(), ts.end(), [](const BatchTileTerm &x, const BatchTileTerm &y) {
                    if (x.xl != y.xl) return x.xl < y.xl;
                    if (x.cr != y.cr) return x.cr < y.cr;
                    return x.ci < y.ci;
                });
                for (size_t j = 0; j < ts.size(); j++) {
                    ts[j].newx = (j == 0 || ts[j - 1].xl != ts[j].xl) ? 1u : 0u;
                    const bool end = j + 1 == ts.size() || ts[j + 1].xl != ts[j].xl || ts[j + 1].cr != ts[j].cr ||
                                     ts[j + 1].ci != ts[j].ci;
                    ts[j].last = end ? 1u : 0u;
                }
                b.nterms = (uint32_t)ts.size();
                ci.tterms.insert(ci.tterms.end(), ts.begin(), ts.end());
                ci.passes.push_back(b);
            }
            std::vector<BatchTerm> rest;  // (wide keeps the flip-mask order)
            for (size_t k : wide) rest.push_back(ci.terms[k]);
            ci.terms.swap(rest);
        }
    });
    // lay the programs out one after another: offsets first, then the copies
    // (in parallel again) into arrays sized once
    std::vector<BatchJob> jobs(circs.size());
    size_t nsweeps = 0, nprog = 0, nterms = 0, npass = 0, ntt = 0;
    std::vector<uint32_t> tt_off(circs.size());
    uint32_t nmax = 0;
    for (size_t c = 0; c < circs.size(); c++) {
        const BatchCircuitIn &ci = circs[c];
        if (!ci.placed) {
            set_error(KBWG_EINVAL, "batch circuits: the planner could not place a circuit's gates");
            return KBWG_EINVAL;
        }
        BatchJob &j = jobs[c];
        memset(&j, 0, sizeof j);
        j.n = ci.n;
        j.id = (uint32_t)c;
        j.sweep_off = (uint32_t)nsweeps;
        j.nsweeps = (uint32_t)ci.sweeps.size();
        j.term_off = (uint32_t)nterms;
        j.nterms = (uint32_t)ci.terms.size();
        j.pad = (uint32_t)nprog;  // the circuit's first gate, for the copies below
        j.pass_off = (uint32_t)npass;
        j.npasses = (uint32_t)ci.passes.size();
        tt_off[c] = (uint32_t)ntt;
        nsweeps += ci.sweeps.size();
        nprog += ci.prog.size();
        nterms += ci.terms.size();
        npass += ci.passes.size();
        ntt += ci.tterms.size();
        nmax = std::max(nmax, ci.n);
    }
    if (nprog > UINT32_MAX || nsweeps > UINT32_MAX || nterms > UINT32_MAX || ntt > UINT32_MAX) {
        set_error(KBWG_EINVAL, "batch circuits: more than 2^32 planned gates, sweeps or strings");
        return KBWG_EINVAL;
    }
    std::unique_ptr<BatchSweep[]> sweeps(new BatchSweep[std::max<size_t>(nsweeps, 1)]);
    std::unique_ptr<TileGate[]> prog(new TileGate[std::max<size_t>(nprog, 1)]);
    std::unique_ptr<BatchTerm[]> terms(new BatchTerm[std::max<size_t>(nterms, 1)]);
    std::unique_ptr<BatchPass[]> passes(new BatchPass[std::max<size_t>(npass, 1)]);
    std::unique_ptr<BatchTileTerm[]> tterms(new BatchTileTerm[std::max<size_t>(ntt, 1)]);
    batch_parallel_for(circs.size(), [&](size_t c) {
        BatchCircuitIn &ci = circs[c];
        BatchJob &j = jobs[c];
        const uint32_t base = j.pad;
        j.pad = 0;
        for (size_t i = 0; i < ci.sweeps.size(); i++) {
            BatchSweep b = ci.sweeps[i];
            b.gate_off += base;
            sweeps[j.sweep_off + i] = b;
        }
        if (!ci.prog.empty()) memcpy(&prog[base], ci.prog.data(), ci.prog.size() * sizeof(TileGate));
        if (!ci.terms.empty()) memcpy(&terms[j.term_off], ci.terms.data(), ci.terms.size() * sizeof(BatchTerm));
        for (size_t i = 0; i < ci.passes.size(); i++) {
            BatchPass b = ci.passes[i];
            b.term_off += tt_off[c];
            passes[j.pass_off + i] = b;
        }
        if (!ci.tterms.empty())
            memcpy(&tterms[tt_off[c]], ci.tterms.data(), ci.tterms.size() * sizeof(BatchTileTerm));
    });
    // largest first: the persistent CTAs then finish together
    std::stable_sort(jobs.begin(), jobs.end(), [&](const BatchJob &x, const BatchJob &y) {
        const double cx = (double)(1ull << x.n) * (1.0 + x.nsweeps + 0.25 * x.nterms);
        const double cy = (double)(1ull << y.n) * (1.0 + y.nsweeps + 0.25 * y.nterms);
        return cx > cy;
    });
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = ensure_smem_limit((const void *)k_batch_circuits<P, K, R>, BK::kSmem);
    if (e != cudaSuccess) return fail(e, "setup");
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_circuits<P, K, R>, BK::kThreads, BK::kSmem);
    if (e != cudaSuccess) return fail(e, "occupancy");
    const uint32_t grid = (uint32_t)std::min<size_t>(jobs.size(), (size_t)sms * std::max(occ, 1));
    const uint64_t slot_elems = nmax > (uint32_t)K ? (1ull << nmax) : 0;
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t jb = jobs.size() * sizeof(BatchJob), swb = std::max<size_t>(nsweeps, 1) * sizeof(BatchSweep),
                 pb = std::max<size_t>(nprog, 1) * sizeof(TileGate),
                 tb = std::max<size_t>(nterms, 1) * sizeof(BatchTerm), eb = circs.size() * sizeof(double),
                 pab = std::max<size_t>(npass, 1) * sizeof(BatchPass),
                 ttb = std::max<size_t>(ntt, 1) * sizeof(BatchTileTerm),
                 sb = (size_t)grid * slot_elems * sizeof(Mem);
    const size_t o_sw = up(jb), o_p = o_sw + up(swb), o_t = o_p + up(pb), o_pa = o_t + up(tb), o_tt = o_pa + up(pab),
                 o_e = o_tt + up(ttb), o_c = o_e + up(eb), o_err = o_c + 256, o_s = o_err + 256;
    cudaStream_t st = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(e, "stream");
    char *dbuf = nullptr;
    e = cudaMalloc(&dbuf, o_s + sb);
    if (e != cudaSuccess) {
        cudaStreamDestroy(st);
        return fail(e, "buffers");
    }
    BatchArgs a;
    memset(&a, 0, sizeof a);
    a.jobs = (const BatchJob *)dbuf;
    a.njobs = (uint32_t)jobs.size();
    a.next = (unsigned *)(dbuf + o_c);
    a.sweeps = (const BatchSweep *)(dbuf + o_sw);
    a.prog = (const TileGate *)(dbuf + o_p);
    a.terms = (const BatchTerm *)(dbuf + o_t);
    a.energies = (double *)(dbuf + o_e);
    a.slots = dbuf + o_s;
    a.slot_elems = slot_elems;
    a.err = (int *)(dbuf + o_err);
    a.passes = (const BatchPass *)(dbuf + o_pa);
    a.tterms = (const BatchTileTerm *)(dbuf + o_tt);
    int err_flag = 0;
    e = copy_async(dbuf, jobs.data(), jb, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nsweeps)
        e = copy_async(dbuf + o_sw, sweeps.get(), nsweeps * sizeof(BatchSweep), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nprog)
        e = copy_async(dbuf + o_p, prog.get(), nprog * sizeof(TileGate), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && nterms)
        e = copy_async(dbuf + o_t, terms.get(), nterms * sizeof(BatchTerm), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && npass)
        e = copy_async(dbuf + o_pa, passes.get(), npass * sizeof(BatchPass), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && ntt)
        e = copy_async(dbuf + o_tt, tterms.get(), ntt * sizeof(BatchTileTerm), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dbuf + o_c, 0, 512, st);
    if (e == cudaSuccess) {
        k_batch_circuits<P, K, R><<<grid, BK::kThreads, BK::kSmem, st>>>(a);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = copy_async(energies, a.energies, eb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = copy_async(&err_flag, a.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dbuf);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(e, "run");
    if (err_flag) {
        set_error(KBWG_ETIMEOUT, "batch circuits: a bounded device-side wait ran out");
        return KBWG_ETIMEOUT;
    }
    return KBWG_OK;
}

constexpr uint32_t kBatchMaxQubits = 24;

int32_t batch_circuits(int precision, uint32_t flags, size_t ncirc, const uint32_t *num_qubits, const kbwg_gate *gates,
                       const uintptr_t *gate_offsets, const uint8_t *paulis, const uintptr_t *qubits,
                       const uintptr_t *term_offsets, const double *coefficients, const uintptr_t *ham_offsets,
                       double *energies) {
    std::vector<BatchCircuitIn> circs(ncirc);
    batch_parallel_for(ncirc, [&](size_t c) {
        BatchCircuitIn &ci = circs[c];
        auto bad = [&](int32_t code, const char *msg) {
            ci.status = code;
            ci.error = msg;
        };
        const uint32_t n = num_qubits[c];
        if (n < 1 || n > kBatchMaxQubits) return bad(KBWG_EQUBITS, "batch circuits: every circuit needs 1..24 qubits");
        ci.n = n;
        if (gate_offsets[c + 1] < gate_offsets[c] || ham_offsets[c + 1] < ham_offsets[c])
            return bad(KBWG_EINVAL, "batch circuits: offsets must not decrease");
        ci.gates.reserve(gate_offsets[c + 1] - gate_offsets[c]);
        for (uintptr_t i = gate_offsets[c]; i < gate_offsets[c + 1]; i++) {
            const kbwg_gate &g = gates[i];
            if (g.kind > KBWG_RZ || g.target >= n || (g.control_mask >> n) || (g.control_mask & (1ull << g.target)))
                return bad(KBWG_EINVAL, "batch circuits: bad gate (kind, target or controls)");
            ci.gates.push_back(make_gate_desc(precision, g.kind, g.target, g.control_mask, g.angle));
        }
        ci.terms.reserve(ham_offsets[c + 1] - ham_offsets[c]);
        for (uintptr_t k = ham_offsets[c]; k < ham_offsets[c + 1]; k++) {
            BatchTerm t;
            memset(&t, 0, sizeof t);
            int ny = 0;
            if (term_offsets[k + 1] < term_offsets[k]) return bad(KBWG_EINVAL, "batch circuits: offsets must not decrease");
            for (uintptr_t i = term_offsets[k]; i < term_offsets[k + 1]; i++) {
                if (qubits[i] >= n || paulis[i] < 1 || paulis[i] > 3)
                    return bad(KBWG_EINVAL, "batch circuits: bad Pauli code or qubit");
                const uint64_t b = 1ull << qubits[i];
                if ((t.x | t.z) & b) return bad(KBWG_EINVAL, "batch circuits: a string names a qubit twice");
                if (paulis[i] == 1) t.x |= b;
                else if (paulis[i] == 2) t.x |= b, t.z |= b, ny++;
                else t.z |= b;
            }
            static const double re[4] = {1, 0, -1, 0}, im[4] = {0, 1, 0, -1};
            t.cr = coefficients[k] * re[ny & 3];
            t.ci = coefficients[k] * im[ny & 3];
            ci.terms.push_back(t);
        }
        std::stable_sort(ci.terms.begin(), ci.terms.end(),
                         [](const BatchTerm &x, const BatchTerm &y) { return x.x < y.x; });
    });
    for (const BatchCircuitIn &ci : circs)  // the first bad circuit's error
        if (ci.status != KBWG_OK) {
            set_error(ci.status, ci.error);
            return ci.status;
        }
    if (ncirc == 0) return KBWG_OK;
    if (precision == KBWG_C64) return batch_run<FastP, 12, 4>(precision, circs, energies);
    if (flags & KBWG_FLAG_FAST_C128) return batch_run<FF2B, 11, 3>(precision, circs, energies);
    return batch_run<Fast<double>, 11, 3>(precision, circs, energies);
}

}  // namespace kbwg
