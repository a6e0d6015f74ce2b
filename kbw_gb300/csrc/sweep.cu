// Fused tile sweep: one pass over the state applies every gate of a sweep.
//
// A tile is 2^K amplitudes: its local bits 0..l-1 are the global qubits
// 0..l-1 (a contiguous chunk of 2^l amplitudes) and its local bits l..K-1 are
// m = K-l arbitrary higher qubits, so a tile is 2^m chunks.  One CTA per tile:
//   1. warp 0 issues one TMA bulk copy (cp.async.bulk) per chunk into shared
//      memory, completing on an mbarrier (bounded wait);
//   2. each thread takes 2^R amplitudes into registers: local bits 0..4 map to
//      the lane, R contiguous local bits to the register index, the rest to
//      the warp (layout A holds bits [5,5+R), layout B bits [K-R,K));
//   3. gates run in order: on register bits as in-thread pairs, on bits 0..4
//      through warp shuffles, diagonal gates (Z, P, RZ) on any bit in place;
//      a stage change re-distributes the tile through shared memory;
//   4. the tile goes back to shared memory and out by TMA bulk stores.
// Controls on qubits outside the tile are one predicate per tile.
#include <string.h>

#include "../../include/kbwg.h"
#include "kernels.h"
#include "sim.h"
#include "sweep.h"

namespace kbwg {

// ---- PTX wrappers: mbarrier + TMA bulk copies ---------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void tma_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tma_store(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void tma_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__device__ __forceinline__ uint64_t insert_zero_at(uint64_t i, uint32_t m) {
    const uint64_t low = (1ull << m) - 1;
    return ((i & ~low) << 1) | (i & low);
}

// ---- single-amplitude gate forms (same operations as apply_pair) -------------
template <class T>
__device__ __forceinline__ cx<T> diag_apply(uint32_t kind, const GateK<T> &k, cx<T> a, bool one) {
    if (kind == G_Z) {
        if (one) {
            a.re = xneg(a.re);
            a.im = xneg(a.im);
        }
        return a;
    }
    if (kind == G_P) return one ? cmul_exact(a, k.c0, k.c1) : a;
    return one ? cmul_exact(a, k.c2, k.c3) : cmul_exact(a, k.c0, k.c1);  // RZ
}

// New value of `self` from the pair (self, partner); `one` = self is the |1> side.
template <class T>
__device__ __forceinline__ cx<T> half_apply(uint32_t kind, const GateK<T> &k, cx<T> self, cx<T> o, bool one) {
    cx<T> r;
    switch (kind) {
    case G_X: return o;
    case G_Y:
        if (one) {
            r.re = xneg(o.im);
            r.im = o.re;
        } else {
            r.re = o.im;
            r.im = xneg(o.re);
        }
        return r;
    case G_H:
        if (one) {
            r.re = xmul(xsub(o.re, self.re), k.c0);
            r.im = xmul(xsub(o.im, self.im), k.c0);
        } else {
            r.re = xmul(xadd(self.re, o.re), k.c0);
            r.im = xmul(xadd(self.im, o.im), k.c0);
        }
        return r;
    case G_RX:
        r.re = xadd(xmul(k.c0, self.re), xmul(k.c1, o.im));
        r.im = xsub(xmul(k.c0, self.im), xmul(k.c1, o.re));
        return r;
    case G_RY:
        if (one) {
            r.re = xadd(xmul(k.c0, self.re), xmul(k.c1, o.re));
            r.im = xadd(xmul(k.c0, self.im), xmul(k.c1, o.im));
        } else {
            r.re = xsub(xmul(k.c0, self.re), xmul(k.c1, o.re));
            r.im = xsub(xmul(k.c0, self.im), xmul(k.c1, o.im));
        }
        return r;
    default: return diag_apply(kind, k, self, one);
    }
}

template <class T>
__device__ __forceinline__ cx<T> shfl_xor_cx(cx<T> v, int m) {
    cx<T> r;
    r.re = __shfl_xor_sync(0xffffffffu, v.re, m);
    r.im = __shfl_xor_sync(0xffffffffu, v.im, m);
    return r;
}

template <class T, int R, int B>
__device__ __forceinline__ void reg_pairs(cx<T> (&v)[1 << R], uint32_t kind, const GateK<T> &k, bool fixed_ok,
                                          uint32_t creg) {
#pragma unroll
    for (int jj = 0; jj < (1 << (R - 1)); jj++) {
        const int j0 = ((jj >> B) << (B + 1)) | (jj & ((1 << B) - 1));
        const int j1 = j0 | (1 << B);
        if (fixed_ok && ((uint32_t)j0 & creg) == creg) apply_pair<T>(kind, k, v[j0], v[j1]);
    }
}

template <class T, int K, int R>
__device__ __forceinline__ void tile_gate(const TileGate &g, cx<T> (&v)[1 << R], int layout, uint32_t F,
                                          uint64_t base) {
    constexpr int NR = 1 << R;
    if ((base & g.co) != g.co) return;  // a control outside the tile is 0 for the whole tile
    GateK<T> k;
    k.c0 = (T)g.c[0];
    k.c1 = (T)g.c[1];
    k.c2 = (T)g.c[2];
    k.c3 = (T)g.c[3];
    const int R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
    const uint32_t regmask = (uint32_t)(NR - 1) << R0;
    const uint32_t fixed_need = g.cl & ~regmask;
    const bool fixed_ok = (F & fixed_need) == fixed_need;
    const uint32_t creg = (g.cl & regmask) >> R0;
    const uint32_t kind = g.kind;
    if (is_diag_kind(kind)) {
        if (g.flags & TG_OUTER_TARGET) {
            const bool one = (base & g.tout) != 0;
#pragma unroll
            for (int j = 0; j < NR; j++)
                if (fixed_ok && ((uint32_t)j & creg) == creg) v[j] = diag_apply(kind, k, v[j], one);
        } else {
            const uint32_t tb = g.tb;
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const bool one = (((F | ((uint32_t)j << R0)) >> tb) & 1u) != 0;
                if (fixed_ok && ((uint32_t)j & creg) == creg) v[j] = diag_apply(kind, k, v[j], one);
            }
        }
        return;
    }
    const uint32_t tb = g.tb;
    if (tb < (uint32_t)kLaneBits) {
        const bool one = ((F >> tb) & 1u) != 0;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const cx<T> o = shfl_xor_cx(v[j], 1 << tb);
            if (fixed_ok && ((uint32_t)j & creg) == creg) v[j] = half_apply(kind, k, v[j], o, one);
        }
        return;
    }
    switch ((int)tb - R0) {
    case 0: reg_pairs<T, R, 0>(v, kind, k, fixed_ok, creg); break;
    case 1: reg_pairs<T, R, 1>(v, kind, k, fixed_ok, creg); break;
    case 2: reg_pairs<T, R, 2>(v, kind, k, fixed_ok, creg); break;
    case 3: reg_pairs<T, R, 3>(v, kind, k, fixed_ok, creg); break;
    default:
        if constexpr (R > 4) reg_pairs<T, R, (R > 4 ? 4 : 0)>(v, kind, k, fixed_ok, creg);
        break;
    }
}

template <class T, int K, int R>
__device__ __forceinline__ void regs_from_smem(const cx<T> *tile, cx<T> (&v)[1 << R], int layout, int lane,
                                               int warp) {
    if (layout == LAYOUT_A) {
        const cx<T> *p = tile + lane + (warp << (kLaneBits + R));
#pragma unroll
        for (int j = 0; j < (1 << R); j++) v[j] = p[j << kLaneBits];
    } else {
        const cx<T> *p = tile + lane + (warp << kLaneBits);
#pragma unroll
        for (int j = 0; j < (1 << R); j++) v[j] = p[j << (K - R)];
    }
}

template <class T, int K, int R>
__device__ __forceinline__ void regs_to_smem(cx<T> *tile, const cx<T> (&v)[1 << R], int layout, int lane, int warp) {
    if (layout == LAYOUT_A) {
        cx<T> *p = tile + lane + (warp << (kLaneBits + R));
#pragma unroll
        for (int j = 0; j < (1 << R); j++) p[j << kLaneBits] = v[j];
    } else {
        cx<T> *p = tile + lane + (warp << kLaneBits);
#pragma unroll
        for (int j = 0; j < (1 << R); j++) p[j << (K - R)] = v[j];
    }
}

template <class T>
__global__ void __launch_bounds__(32 << (TileCfg<T>::K - kLaneBits - TileCfg<T>::R), 2)
    k_sweep(cx<T> *__restrict__ st, const __grid_constant__ SweepParams p) {
    constexpr int K = TileCfg<T>::K, R = TileCfg<T>::R;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    cx<T> *tile = reinterpret_cast<cx<T> *>(smem_raw);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_raw + (sizeof(cx<T>) << K));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint64_t tau = blockIdx.x;
    uint64_t base = tau << p.l;
    for (uint32_t j = 0; j < p.m; j++) base = insert_zero_at(base, p.hq[j]);
    const uint32_t chunk = 1u << p.l;
    const uint32_t nchunks = 1u << p.m;
    const uint32_t chunk_bytes = chunk * (uint32_t)sizeof(cx<T>);

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (warp == 0) {
        if (lane == 0) mbar_expect_tx(bar, (uint32_t)(sizeof(cx<T>) << K));
        __syncwarp();
        for (uint32_t c = lane; c < nchunks; c += 32) {
            uint64_t off = 0;
            for (uint32_t j = 0; j < p.m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
            tma_load(tile + (size_t)c * chunk, st + base + off, chunk_bytes, bar);
        }
    }
    bool ok = false;
    for (uint32_t it = 0; it < (1u << 22); it++)
        if (mbar_try_wait(bar, 0)) {
            ok = true;
            break;
        }
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(p.err, 1);
        return;
    }

    cx<T> v[1 << R];
    int layout = p.stage_layout[0];
    const uint32_t FA = (uint32_t)lane | ((uint32_t)warp << (kLaneBits + R));
    const uint32_t FB = (uint32_t)lane | ((uint32_t)warp << kLaneBits);
    regs_from_smem<T, K, R>(tile, v, layout, lane, warp);
    uint32_t g0 = 0;
    for (uint32_t s = 0; s < p.nstages; s++) {
        const int nl = p.stage_layout[s];
        if (nl != layout) {
            regs_to_smem<T, K, R>(tile, v, layout, lane, warp);
            __syncthreads();
            regs_from_smem<T, K, R>(tile, v, nl, lane, warp);
            layout = nl;
        }
        const uint32_t g1 = p.stage_end[s];
        const uint32_t F = (layout == LAYOUT_A) ? FA : FB;
        for (uint32_t gi = g0; gi < g1; gi++) tile_gate<T, K, R>(p.prog[gi], v, layout, F, base);
        g0 = g1;
    }
    regs_to_smem<T, K, R>(tile, v, layout, lane, warp);
    fence_proxy_async();
    __syncthreads();
    if (warp == 0) {
        for (uint32_t c = lane; c < nchunks; c += 32) {
            uint64_t off = 0;
            for (uint32_t j = 0; j < p.m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
            tma_store(st + base + off, tile + (size_t)c * chunk, chunk_bytes);
        }
        tma_commit();
        tma_wait_all();
    }
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
    static bool attr_set[2] = {false, false};
    const size_t smem = (sizeof(cx<T>) << K) + 16;
    const int pi = sizeof(T) == 8 ? 1 : 0;
    if (!attr_set[pi]) {
        cudaError_t e = cudaFuncSetAttribute(k_sweep<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        attr_set[pi] = true;
    }
    std::vector<PlannedSweep> plan =
        plan_sweeps(s.n, K, R, gates, count, (s.flags & KBWG_FLAG_EXACT_ORDER) != 0);
    size_t total = 0;
    for (const PlannedSweep &sw : plan) total += sw.gates.size();
    std::vector<TileGate> prog;
    prog.reserve(total);
    for (const PlannedSweep &sw : plan) prog.insert(prog.end(), sw.gates.begin(), sw.gates.end());
    cudaError_t e = s.tmp4.ensure(total * sizeof(TileGate));
    if (e != cudaSuccess) return e;
    // pageable source: the call returns once the host buffer is consumed
    e = copy_async(s.tmp4.ptr, prog.data(), total * sizeof(TileGate), cudaMemcpyHostToDevice, s.stream);
    if (e != cudaSuccess) return e;
    const TileGate *dprog = (const TileGate *)s.tmp4.ptr;
    const unsigned threads = 32u << (K - kLaneBits - R);
    const uint64_t tiles = 1ull << (s.n - K);
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
        off += sw.gates.size();
        if (s.prof.on) s.prof.mark(s.stream);
        k_sweep<T><<<(unsigned)tiles, threads, smem, s.stream>>>((cx<T> *)s.state, p);
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

cudaError_t run_fused(Sim &s, const GateDesc *gates, size_t count) {
    return s.prec ? run_fused_t<double>(s, gates, count) : run_fused_t<float>(s, gates, count);
}

}  // namespace kbwg
