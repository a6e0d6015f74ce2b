// Device side of the run-time-specialised sweep kernels.
//
// jit.cpp writes one kernel per planned sweep: the gate sequence of the
// sweep becomes straight-line code in which every structural property of a
// gate -- class, target bit, which registers its register-bit controls
// select, its control masks on lane/warp bits and outside the tile -- is a
// compile-time constant; only the gate constants (angles) are read at run
// time, from the sweep's program in shared memory, so one compiled kernel
// serves every call with the same structure.  Compared with the interpreted
// k_sweep this removes the per-gate header loads, the dispatch branch, the
// register moves its jump table forces at the join, the per-register
// predicates of controlled gates, and the shuffles of registers a control
// excludes; a register-bit X is a renaming of registers and costs nothing.
//
// The arithmetic of each gate is the policy's (sweep_dev.cuh), called in the
// same order as k_sweep calls it, and the tile load/store path is k_sweep's.
#pragma once

#include "sweep_dev.cuh"

namespace kbwg {
namespace jit {

// Non-diagonal gate whose target is register bit B; bit j of JM: register j
// passes the gate's controls on register bits.
template <class P, int R, int B, int CLS, uint32_t JM, int SUB>
__device__ __forceinline__ void reg(typename P::Amp (&v)[1 << R], const typename P::K4 &k) {
#pragma unroll
    for (int jj = 0; jj < (1 << (R - 1)); jj++) {
        const int j0 = ((jj >> B) << (B + 1)) | (jj & ((1 << B) - 1));
        const int j1 = j0 | (1 << B);
        if (((JM >> j0) & 1u) == 0u) continue;
        if constexpr (CLS == TG_X) {
            const typename P::Amp t = v[j0];
            v[j0] = v[j1];
            v[j1] = t;
        } else if constexpr (CLS == TG_Y) {
            P::y_pair(v[j0], v[j1]);
        } else if constexpr (CLS == TG_H) {
            P::h_pair(SUB, k, v[j0], v[j1]);
        } else if constexpr (CLS == TG_RX) {
            P::rx_pair(k, v[j0], v[j1]);
        } else {
            P::ry_pair(k, v[j0], v[j1]);
        }
    }
}

template <class A>
__device__ __forceinline__ A sel(bool c, const A &x, const A &y) {
    return c ? x : y;
}

// Register-bit X when `c` holds (controls on lane/warp bits or outside the
// tile): per-pair selects rather than a branch around the block, so both
// sides keep one register assignment (a branch made the compiler carry two
// copies of the registers and spill).
template <class P, int R, int B, uint32_t JM>
__device__ __forceinline__ void cswap(typename P::Amp (&v)[1 << R], bool c) {
#pragma unroll
    for (int jj = 0; jj < (1 << (R - 1)); jj++) {
        const int j0 = ((jj >> B) << (B + 1)) | (jj & ((1 << B) - 1));
        const int j1 = j0 | (1 << B);
        if (((JM >> j0) & 1u) == 0u) continue;
        const typename P::Amp a = v[j0], b = v[j1];
        v[j0] = sel(c, b, a);
        v[j1] = sel(c, a, b);
    }
}

// Non-diagonal gate whose target is lane bit TB: the partner amplitude comes
// from lane ^ (1 << TB).  Registers whose register-bit controls fail (CREG)
// take no part, in any lane; `fok` (controls on lane/warp bits) selects per
// thread after the shuffle, so every lane still joins it.
template <class P, int R, int TB, int CLS, uint32_t CREG, int SUB>
__device__ __forceinline__ void lane(typename P::Amp (&v)[1 << R], const typename P::K4 &k, bool fok, uint32_t F) {
    const bool one = ((F >> TB) & 1u) != 0u;
#pragma unroll
    for (int j = 0; j < (1 << R); j++) {
        if (((uint32_t)j & CREG) != CREG) continue;
        const typename P::Amp o = P::shfl(v[j], 1 << TB);
        if (!fok) continue;
        if constexpr (CLS == TG_X) {
            v[j] = o;
        } else if constexpr (CLS == TG_Y) {
            v[j] = P::y_half(o, one);
        } else if constexpr (CLS == TG_H) {
            v[j] = P::h_half(SUB, k, v[j], o, P::sign(one));
        } else if constexpr (CLS == TG_RX) {
            v[j] = P::rx_half(k, v[j], o);
        } else {
            v[j] = P::ry_half(k, v[j], o, P::signed_s(k, one));
        }
    }
}

// Diagonal gate whose target is register bit B (Q: the power of i of a PI
// gate), applied where `c` holds (its controls off the registers).
template <class P, int R, int B, int CLS, uint32_t JM, int Q>
__device__ __forceinline__ void dreg(typename P::Amp (&v)[1 << R], const typename P::K4 &k, bool c = true) {
#pragma unroll
    for (int j = 0; j < (1 << R); j++) {
        if (((JM >> j) & 1u) == 0u) continue;
        const bool hi = ((j >> B) & 1) != 0;
        if constexpr (CLS == TG_Z) {
            if (hi) v[j] = sel(c, P::neg(v[j]), v[j]);
        } else if constexpr (CLS == TG_P) {
            if (hi) v[j] = sel(c, P::cmul(v[j], k.c0, k.c1), v[j]);
        } else if constexpr (CLS == TG_RZ) {
            v[j] = sel(c, hi ? P::cmul(v[j], k.c2, k.c3) : P::cmul(v[j], k.c0, k.c1), v[j]);
        } else {  // TG_PI
            if (hi) v[j] = sel(c, P::pi_mul(v[j], Q), v[j]);
        }
    }
}

// Diagonal gate whose target side `one` is the same for all of a thread's
// registers (a lane or warp bit, a qubit outside the tile; SCALE: always),
// applied where `c` holds.  Per-register selects (RZ: of the constants)
// rather than a branch around the block; each amplitude gets the
// arithmetic the branch would give it.
template <class P, int R, int CLS, uint32_t JM, int Q>
__device__ __forceinline__ void dfix(typename P::Amp (&v)[1 << R], const typename P::K4 &k, bool one, bool c = true) {
    if constexpr (CLS == TG_RZ) {
        const auto cr = one ? k.c2 : k.c0;
        const auto ci = one ? k.c3 : k.c1;
#pragma unroll
        for (int j = 0; j < (1 << R); j++)
            if ((JM >> j) & 1u) v[j] = sel(c, P::cmul(v[j], cr, ci), v[j]);
    } else {
        const bool on = (CLS == TG_SCALE || one) && c;
#pragma unroll
        for (int j = 0; j < (1 << R); j++) {
            if (((JM >> j) & 1u) == 0u) continue;
            if constexpr (CLS == TG_Z) {
                v[j] = sel(on, P::neg(v[j]), v[j]);
            } else if constexpr (CLS == TG_PI) {
                v[j] = sel(on, P::pi_mul(v[j], Q), v[j]);
            } else {  // P (|1> side only) and SCALE
                v[j] = sel(on, P::cmul(v[j], k.c0, k.c1), v[j]);
            }
        }
    }
}

// Register layout change through the shared-memory tile (one round trip):
// layout A holds local bits [5, 5+R) in registers, layout B [K-R, K).  Each
// thread rewrites only the positions it read in the old layout, so one
// barrier suffices.
template <class P, int K, int R, int FROM, int TO>
__device__ __forceinline__ void relayout(typename P::Amp (&v)[1 << R], typename P::Amp *tile, uint32_t FA, uint32_t FB) {
    constexpr int R0f = (FROM == LAYOUT_A) ? kLaneBits : (K - R);
    constexpr int R0t = (TO == LAYOUT_A) ? kLaneBits : (K - R);
    const uint32_t Ff = (FROM == LAYOUT_A) ? FA : FB;
    const uint32_t Ft = (TO == LAYOUT_A) ? FA : FB;
#pragma unroll
    for (int j = 0; j < (1 << R); j++) tile[Ff | ((uint32_t)j << R0f)] = v[j];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < (1 << R); j++) v[j] = tile[Ft | ((uint32_t)j << R0t)];
}

// The sweep: k_sweep's persistent tile loop (TMA bulk loads on an mbarrier
// with a bounded wait, registers in layout Body::kFirst, coalesced stores
// from registers in layout Body::kLast) with the gate program replaced by
// Body::run, the sweep's gates as straight-line code.
template <class P, int K, int R, class Body, bool W = false>
__device__ __forceinline__ void sweep(typename P::Mem *__restrict__ st, const SweepParams &p) {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    using B = typename pick_t<W, uint64_t, uint32_t>::type;  // state index width
    constexpr int NR = 1 << R;
    constexpr size_t kTileBytes = sizeof(Mem) << K;
    constexpr size_t kChunkTable = 256 * sizeof(uint64_t);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Amp *tile = reinterpret_cast<Amp *>(smem_raw);
    Mem *tile_mem = reinterpret_cast<Mem *>(smem_raw);
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(smem_raw + kTileBytes);
    TileGate *sg = reinterpret_cast<TileGate *>(smem_raw + kTileBytes + kChunkTable);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + kTileBytes + kChunkTable + kMaxSweepGates * sizeof(TileGate));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t l = p.l, m = p.m;
    const uint32_t chunk = 1u << l, nchunks = 1u << m;
    const uint32_t chunk_bytes = chunk * (uint32_t)sizeof(Mem);
    const uint64_t lowmask = chunk - 1;

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
            if (lane == 0) mbar_expect_tx(bar, (uint32_t)kTileBytes);
            __syncwarp();
            for (uint32_t c = lane; c < nchunks; c += 32)
                tma_load(tile_mem + (size_t)c * chunk, st + b + chunk_off[c], chunk_bytes, bar);
        }
    };

    uint32_t tau = blockIdx.x;
    if (tau < p.tiles) issue_load(tau);
    const uint32_t FA = (uint32_t)lane | ((uint32_t)warp << (kLaneBits + R));
    const uint32_t FB = (uint32_t)lane | ((uint32_t)warp << kLaneBits);
    constexpr int R0first = (Body::kFirst == LAYOUT_A) ? kLaneBits : (K - R);
    constexpr int R0last = (Body::kLast == LAYOUT_A) ? kLaneBits : (K - R);
    const uint32_t Ffirst = (Body::kFirst == LAYOUT_A) ? FA : FB;
    const uint32_t Flast = (Body::kLast == LAYOUT_A) ? FA : FB;
    for (uint32_t it = 0; tau < p.tiles; tau += gridDim.x, it++) {
        const B base = tile_base(tau);
        if (!tile_wait(bar, it & 1u, p.err)) return;
        Amp v[NR];
#pragma unroll
        for (int j = 0; j < NR; j++) v[j] = P::from_mem(tile_mem[Ffirst | ((uint32_t)j << R0first)]);
        Body::template run<P, K, R>(v, tile, FA, FB, base, sg);
        // the tile buffer is free: start the next tile's load, then store this one
        fence_proxy_async();
        __syncthreads();
        const uint32_t next = tau + gridDim.x;
        if (next < p.tiles) issue_load(next);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t u = Flast | ((uint32_t)j << R0last);
            st[base + chunk_off[u >> l] + (u & lowmask)] = P::to_mem(v[j]);
        }
    }
}

}  // namespace jit
}  // namespace kbwg
