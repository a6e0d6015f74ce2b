// Fused tile sweep: one pass over the state applies every gate of a sweep.
//
// A tile is 2^K amplitudes: its local bits 0..l-1 are the global qubits
// 0..l-1 (a contiguous chunk of 2^l amplitudes) and its local bits l..K-1 are
// m = K-l arbitrary higher qubits, so a tile is 2^m chunks.  Persistent CTAs
// (two per SM) walk the tiles; per CTA:
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
#include <type_traits>

#include <math.h>

#include "../../include/kbwg.h"
#include "kernels.h"
#include "sim.h"
#include "sweep_dev.cuh"

namespace kbwg {

template <class P, int K, int R>
struct SweepKernel {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    static_assert(sizeof(Amp) == sizeof(Mem), "register and memory amplitudes share the tile buffer");
    static constexpr int kThreads = 32 << (K - kLaneBits - R);
    static constexpr size_t kTileBytes = sizeof(Mem) << K;
    static constexpr size_t kChunkTable = 256 * sizeof(uint64_t);
    static constexpr size_t kSmem = kTileBytes + kChunkTable + kMaxSweepGates * sizeof(TileGate) + 16;
};

template <class P, int K, int R>
__global__ void __launch_bounds__(SweepKernel<P, K, R>::kThreads, 2)
    k_sweep(typename P::Mem *__restrict__ st, const __grid_constant__ SweepParams p) {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    using SK = SweepKernel<P, K, R>;
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

    auto tile_base = [&](uint64_t tau) {
        uint64_t b = tau << l;
        for (uint32_t j = 0; j < m; j++) b = insert_zero_at(b, p.hq[j]);
        return b;
    };
    auto issue_load = [&](uint64_t tau) {
        if (warp == 0) {
            const uint64_t b = tile_base(tau);
            if (lane == 0) mbar_expect_tx(bar, (uint32_t)SK::kTileBytes);
            __syncwarp();
            for (uint32_t c = lane; c < nchunks; c += 32)
                tma_load(tile_mem + (size_t)c * chunk, st + b + chunk_off[c], chunk_bytes, bar);
        }
    };

    uint64_t tau = blockIdx.x;
    if (tau < p.tiles) issue_load(tau);
    const uint32_t FA = (uint32_t)lane | ((uint32_t)warp << (kLaneBits + R));
    const uint32_t FB = (uint32_t)lane | ((uint32_t)warp << kLaneBits);
    for (uint32_t it = 0; tau < p.tiles; tau += gridDim.x, it++) {
        const uint64_t base = tile_base(tau);
        bool ok = false;
        for (uint32_t spin = 0; spin < (1u << 22); spin++)
            if (mbar_try_wait(bar, it & 1u)) {
                ok = true;
                break;
            }
        if (__syncthreads_or(!ok)) {
            if (threadIdx.x == 0) atomicExch(p.err, 1);
            return;
        }
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
            for (uint32_t gi = g0; gi < g1; gi++) tile_gate<P, K, R>(sg[gi], v, R0, F, base);
            g0 = g1;
        }
        // the tile buffer is free: start the next tile's load, then store this one
        fence_proxy_async();
        __syncthreads();
        const uint64_t next = tau + gridDim.x;
        if (next < p.tiles) issue_load(next);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t u = F | ((uint32_t)j << R0);
            st[base + chunk_off[u >> l] + (u & lowmask)] = P::to_mem(v[j]);
        }
    }
}

template <class P, int K, int R>
static cudaError_t run_fused_p(Sim &s, const GateDesc *gates, size_t count) {
    using SK = SweepKernel<P, K, R>;
    using Mem = typename P::Mem;
    static bool attr_set = false;
    static int num_sms = 0;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_sweep<P, K, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)SK::kSmem);
        if (e != cudaSuccess) return e;
        int dev = 0;
        e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    std::vector<PlannedSweep> plan =
        plan_sweeps(s.n, K, R, gates, count, (s.flags & KBWG_FLAG_EXACT_ORDER) != 0);
    size_t total = 0;
    for (const PlannedSweep &sw : plan) total += sw.gates.size();
    std::vector<TileGate> prog;
    prog.reserve(total);
    for (const PlannedSweep &sw : plan) prog.insert(prog.end(), sw.gates.begin(), sw.gates.end());
    for (TileGate &t : prog) P::pack_host(t);
    cudaError_t e = s.tmp4.ensure(total * sizeof(TileGate));
    if (e != cudaSuccess) return e;
    // pageable source: the call returns once the host buffer is consumed
    e = copy_async(s.tmp4.ptr, prog.data(), total * sizeof(TileGate), cudaMemcpyHostToDevice, s.stream);
    if (e != cudaSuccess) return e;
    const TileGate *dprog = (const TileGate *)s.tmp4.ptr;
    const uint64_t tiles = 1ull << (s.n - K);
    const uint64_t grid = std::min<uint64_t>(tiles, (uint64_t)num_sms * 2);
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
        k_sweep<P, K, R><<<(unsigned)grid, SK::kThreads, SK::kSmem, s.stream>>>((Mem *)s.state, p);
        count_launch();
        e = cudaGetLastError();
        if (s.prof.on) {
            s.prof.mark(s.stream);
            s.prof.bytes += 2.0 * (double)s.elem * (double)s.ns;
        }
        if (e != cudaSuccess) return e;
    }
    s.last_passes = plan.size();
    return cudaSuccess;
}

template <class T>
static cudaError_t run_fused_t(Sim &s, const GateDesc *gates, size_t count) {
    constexpr int K = TileCfg<T>::K, R = TileCfg<T>::R;
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
            // e^{-it/2} diag(1, e^{it}): e^{it} = (c2 + i c3)^2
            const double c = x.c[2] * x.c[2] - x.c[3] * x.c[3], sn = 2.0 * x.c[2] * x.c[3];
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

bool ff_capable(const Sim &s) {
    return s.prec && (s.flags & KBWG_FLAG_FAST_C128) && s.n >= (uint32_t)TileCfg<double>::K;
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

cudaError_t run_fused(Sim &s, const GateDesc *gates, size_t count) {
    if (ff_capable(s)) {
        // float-float sweeps read and write the float-float form; the state
        // stays in it until an operation needs binary64
        if (!s.ff_resident) {
            cudaError_t e = launch_ff_convert(s.state, s.n, true, s.stream);
            if (e != cudaSuccess) return e;
            s.ff_resident = true;
        }
        std::vector<GateDesc> g = ff_rewrite(gates, count);
        return run_fused_p<FF2, TileCfg<double>::K, TileCfg<double>::R>(s, g.data(), g.size());
    }
    return s.prec ? run_fused_t<double>(s, gates, count) : run_fused_t<float>(s, gates, count);
}

}  // namespace kbwg
