// Batched forward of many small variational circuits in one persistent
// launch: the hardware-efficient ansatz (per layer RY then RZ on every qubit,
// then CZ on the ring (i, i+1 mod n)) followed by <H> for the ring transverse
// field Ising Hamiltonian H = zz sum Z_i Z_{i+1} + x sum X_i.
//
// The reference runs one circuit per fresh simulator (BatchExecution,
// kbw src/quantum_execution.rs:368-418).  Here persistent CTAs take circuits
// from a work queue sorted by cost (largest first).  A CTA builds the
// circuit's gate program in shared memory (angles -> constants on the device)
// and runs it with the register-tile machinery of the sweep kernel:
//   * n <= K: the whole state is one tile that never leaves the SM; the
//     circuit is one program of 2L register-layout stages;
//   * n > K (K = 13 complex64, 12 complex128): the state lives in the CTA's
//     slot of a global buffer; each layer is two tiled passes (qubits 0..K-1,
//     then the K-h low + h high qubits with the CZ ring), TMA-loaded tile by
//     tile; a final read-only pass completes <X_q>.
// <H> accumulates in FP64-grade (float-float per thread for complex64).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/kbwg.h"
#include "kernels.h"
#include "sim.h"
#include "sweep_dev.cuh"

namespace kbwg {

constexpr int kHeaMaxGates = 512;

struct HeaJob {
    uint32_t n, L;
    uint32_t id, pad;
    uint64_t poff;  // first angle of the circuit in params[]
};

struct HeaArgs {
    const HeaJob *jobs;
    uint32_t njobs;
    unsigned *next;  // work-queue counter (0 at launch)
    const double *params;
    double zz, xc;
    double *energies;
    void *slots;  // per-CTA state slots of slot_elems amplitudes
    uint64_t slot_elems;
    int *err;
};

// per-thread FP64-grade accumulator matching the policy
template <class P> struct HeaAcc;
template <class T> struct HeaAcc<Fast<T>> {
    double v = 0.0;
    T part = (T)0;
    int cnt = 0;
    __device__ __forceinline__ void add(T x) {  // short float runs, then widen
        part += x;
        if (++cnt == 16) flush();
    }
    __device__ __forceinline__ void flush() {
        v += (double)part;
        part = (T)0;
        cnt = 0;
    }
    __device__ __forceinline__ double value() {
        flush();
        return v;
    }
};
template <> struct HeaAcc<FFPol> {
    ff::f2 v{0.f, 0.f};
    __device__ __forceinline__ void add(ff::f2 x) { v = ff::add(v, x); }
    __device__ __forceinline__ double value() { return (double)v.h + (double)v.l; }
};

// |0...0> amplitude in memory format
template <class Mem>
__device__ __forceinline__ Mem mem_basis(bool one) {
    Mem m;
    m.re = one ? 1 : 0;
    m.im = 0;
    return m;
}

// |a|^2 and 2 Re(conj(a) b) in the policy's arithmetic
template <class T>
__device__ __forceinline__ T hea_norm2(const cx<T> &a) {
    return fma(a.re, a.re, a.im * a.im);
}
template <class T>
__device__ __forceinline__ T hea_re2(const cx<T> &a, const cx<T> &b) {
    return (T)2 * fma(a.re, b.re, a.im * b.im);
}
__device__ __forceinline__ ff::f2 hea_norm2(const FFPol::Amp &a) { return ff::dot2(a.re, a.re, a.im, a.im); }
__device__ __forceinline__ ff::f2 hea_re2(const FFPol::Amp &a, const FFPol::Amp &b) {
    const ff::f2 r = ff::dot2(a.re, b.re, a.im, b.im);
    return ff::f2{2.f * r.h, 2.f * r.l};
}
template <class T>
__device__ __forceinline__ T hea_scale(T x, double c) {
    return x * (T)c;
}
__device__ __forceinline__ ff::f2 hea_scale(ff::f2 x, double c) { return ff::mul(x, ff::split_constant(c)); }

// cos, sin of x in the policy's precision (complex64: as Dense<f32> does,
// in float)
template <class P>
__device__ __forceinline__ void hea_sincos(double x, double *s, double *c) {
    sincos(x, s, c);
}
template <>
__device__ __forceinline__ void hea_sincos<Fast<float>>(double x, double *s, double *c) {
    float fs, fc;
    sincosf((float)x, &fs, &fc);
    *s = fs;
    *c = fc;
}

// constants of one gate into a TileGate, in the policy's packing
template <class P> struct HeaConst;
template <class T> struct HeaConst<Fast<T>> {
    static __device__ void set(TileGate &g, double a, double b, double c, double d) {
        T *v = reinterpret_cast<T *>(g.c);
        v[0] = (T)a;
        v[1] = (T)b;
        v[2] = (T)c;
        v[3] = (T)d;
    }
};
template <> struct HeaConst<FFPol> {
    static __device__ void set(TileGate &g, double a, double b, double c, double d) {
        float *f = reinterpret_cast<float *>(g.c);
        const double in[4] = {a, b, c, d};
        for (int i = 0; i < 4; i++) {
            const float h = (float)in[i];
            f[2 * i] = h;
            f[2 * i + 1] = (float)(in[i] - (double)h);
        }
    }
};

// Program of one pass, built by thread 0.  `qmin..qmax` are the qubits whose
// RY/RZ the pass applies for layer `layer` (angles at params[poff + ...]);
// `with_cz` appends the CZ ring.  local(q) maps a qubit to its local bit or
// -1 (outside the tile).  Returns the gate count.
template <class P, int K, int R>
__device__ uint32_t hea_build(TileGate *sg, uint8_t *stage_layout, uint16_t *stage_end, uint32_t &nstages,
                              const double *ang, uint32_t n, uint32_t qmin, uint32_t qmax, bool with_cz,
                              const int8_t *local) {
    uint32_t cnt = 0;
    for (int pass = 0; pass < 2; pass++) {  // layout A bits first, then layout B bits
        const uint32_t start = cnt;
        for (uint32_t q = qmin; q < qmax; q++) {
            const int lb = local[q];
            const bool in_a = lb < kLaneBits + R;
            if ((pass == 0) != in_a) continue;
            const double th = ang[q], ph = ang[n + q];
            TileGate &ry = sg[cnt++];
            memset(&ry, 0, sizeof ry);
            ry.cls = TG_RY;
            ry.tb = (uint8_t)lb;
            double sn, cs;
            hea_sincos<P>(0.5 * th, &sn, &cs);
            HeaConst<P>::set(ry, cs, sn, 0.0, 0.0);
            TileGate &rz = sg[cnt++];
            memset(&rz, 0, sizeof rz);
            rz.cls = TG_RZ;
            rz.tb = (uint8_t)lb;
            hea_sincos<P>(0.5 * ph, &sn, &cs);
            HeaConst<P>::set(rz, cs, -sn, cs, sn);
        }
        if (pass == 1 && with_cz && n >= 2) {  // (appended after the layout-B rotations)
            for (uint32_t i = 0; i < n; i++) {
                const uint32_t j = (i + 1) % n;
                if (n == 2 && i == 1) break;
                TileGate &cz = sg[cnt++];
                memset(&cz, 0, sizeof cz);
                cz.cls = TG_Z;
                const int lt = local[j], lc = local[i];
                if (lt >= 0) {
                    cz.tb = (uint8_t)lt;
                } else {
                    cz.tb = TG_OUTER;
                    cz.tout = (uint8_t)j;
                }
                if (lc >= 0)
                    cz.cl = 1u << lc;
                else
                    cz.co = 1ull << i;
            }
        }
        if (cnt == start) continue;
        // a stage of diagonal gates only (the CZ ring) runs in the previous layout
        bool only_diag = true;
        for (uint32_t i = start; i < cnt; i++) only_diag = only_diag && tg_diagonal(sg[i].cls);
        if (only_diag && nstages > 0) {
            stage_end[nstages - 1] = (uint16_t)cnt;
        } else {
            stage_layout[nstages] = (uint8_t)(pass == 0 ? LAYOUT_A : LAYOUT_B);
            stage_end[nstages] = (uint16_t)cnt;
            nstages++;
        }
        const int R0 = stage_layout[nstages - 1] == LAYOUT_A ? kLaneBits : K - R;
        for (uint32_t i = start; i < cnt; i++) tile_gate_dispatch(sg[i], R0, R);
    }
    return cnt;
}

template <class P, int K, int R>
struct HeaKernel {
    using Mem = typename P::Mem;
    static constexpr int kThreads = 32 << (K - kLaneBits - R);
    static constexpr size_t kTileBytes = sizeof(Mem) << K;
    static constexpr size_t kSmem = kTileBytes + 256 * sizeof(uint64_t) + kHeaMaxGates * sizeof(TileGate) + 64 +
                                    2 * kMaxStages * 4 + 64 * 8 + 64;
};

// Energy contributions of the tile held in registers (layout `layout`):
// ZZ for every amplitude (when `zz_here`) and X_q for the qubits whose local
// bit sits in this layout's lanes or registers and is flagged in xmask.
template <class P, int K, int R>
__device__ __forceinline__ void hea_energy_tile(HeaAcc<P> &acc, const typename P::Amp (&v)[1 << R], int R0,
                                                uint32_t F, uint32_t n, const uint64_t *chunk_off, uint32_t l,
                                                uint64_t base, double zz, double xc, bool zz_here,
                                                uint32_t xmask_local) {
    constexpr int NR = 1 << R;
    const uint64_t lowmask = (1ull << l) - 1;
    if (zz_here && n >= 2) {
        const uint64_t nm = (n >= 64) ? ~0ull : ((1ull << n) - 1);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t u = F | ((uint32_t)j << R0);
            const uint64_t s = base + chunk_off[u >> l] + (u & lowmask);
            const uint64_t rot = (s >> 1) | ((s & 1ull) << (n - 1));
            const int pairs = (n == 2) ? 1 : (int)n;
            const int odd = (n == 2) ? (int)((s ^ (s >> 1)) & 1ull) : __popcll((s ^ rot) & nm);
            const double d = zz * (double)(pairs - 2 * odd);
            acc.add(hea_scale(hea_norm2(v[j]), d));
        }
    }
    // X_q on lane bits: partner in lane ^ (1 << b); only the |0> side adds
    for (int b = 0; b < kLaneBits; b++) {
        if (!((xmask_local >> b) & 1u)) continue;
        const bool zero_side = ((F >> b) & 1u) == 0;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const typename P::Amp o = P::shfl(v[j], 1 << b);
            if (zero_side) acc.add(hea_scale(hea_re2(v[j], o), xc));
        }
    }
    // X_q on register bits
#pragma unroll
    for (int b = 0; b < R; b++) {
        if (!((xmask_local >> (R0 + b)) & 1u)) continue;
#pragma unroll
        for (int j = 0; j < NR; j++)
            if (!((j >> b) & 1)) acc.add(hea_scale(hea_re2(v[j], v[j | (1 << b)]), xc));
    }
}

// complex64: two CTAs per SM (64 registers; 32 warps), 35 % more circuits/s
// than one CTA with 106 registers
template <class P, int K, int R>
__global__ void __launch_bounds__(HeaKernel<P, K, R>::kThreads, (sizeof(typename P::Mem) == 8 ? 2 : 1)) k_hea_batch(const __grid_constant__ HeaArgs a) {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    using HK = HeaKernel<P, K, R>;
    constexpr int NR = 1 << R;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Amp *tile = reinterpret_cast<Amp *>(smem_raw);
    Mem *tile_mem = reinterpret_cast<Mem *>(smem_raw);
    unsigned char *q = smem_raw + HK::kTileBytes;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(q);
    q += 256 * sizeof(uint64_t);
    TileGate *sg = reinterpret_cast<TileGate *>(q);
    q += kHeaMaxGates * sizeof(TileGate);
    uint8_t *stage_layout = q;
    q += kMaxStages * 2;
    uint16_t *stage_end = reinterpret_cast<uint16_t *>(q);
    q += kMaxStages * 2 + 32;
    int8_t *local = reinterpret_cast<int8_t *>(q);
    q += 64;
    double *red = reinterpret_cast<double *>(q);  // [32] block reduction
    q += 32 * 8;
    uint32_t *meta = reinterpret_cast<uint32_t *>(q);  // job index, gate count, nstages
    q += 64;
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
        const HeaJob job = a.jobs[jix];
        const uint32_t n = job.n, L = job.L;
        const double *ang = a.params + job.poff;
        HeaAcc<P> acc;
        if (n <= (uint32_t)K) {
            // ---- whole state in registers: programs of as many layers as fit ----
            const uint32_t per_layer = 3 * n;
            const uint32_t group = std::max<uint32_t>(1, std::min<uint32_t>(kHeaMaxGates / per_layer, kMaxStages / 2));
            Amp v[NR];
            int layout = LAYOUT_A;
            int R0 = kLaneBits;
            uint32_t F = FA;
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const uint32_t u = F | ((uint32_t)j << R0);
                v[j] = P::from_mem(mem_basis<Mem>(u == 0));
            }
            for (uint32_t ly0 = 0; ly0 < L; ly0 += group) {
                const uint32_t ly1 = std::min(L, ly0 + group);
                __syncthreads();
                if (threadIdx.x == 0) {
                    for (uint32_t qq = 0; qq < 64; qq++) local[qq] = (qq < n) ? (int8_t)qq : (int8_t)-1;
                    uint32_t ns = 0, cnt = 0;
                    for (uint32_t ly = ly0; ly < ly1; ly++) {
                        uint32_t nst = 0;
                        const uint32_t c = hea_build<P, K, R>(sg + cnt, stage_layout + ns, stage_end + ns, nst,
                                                              ang + (size_t)ly * 2 * n, n, 0, n, true, local);
                        for (uint32_t t = 0; t < nst; t++) stage_end[ns + t] += (uint16_t)cnt;
                        cnt += c;
                        ns += nst;
                    }
                    meta[1] = cnt;
                    meta[2] = ns;
                    chunk_off[0] = 0;
                }
                __syncthreads();
                const uint32_t nst = meta[2];
                uint32_t g0 = 0;
                for (uint32_t s = 0; s < nst; s++) {
                    const int nl = stage_layout[s];
                    if (nl != layout) {
#pragma unroll
                        for (int j = 0; j < NR; j++) tile[F | ((uint32_t)j << R0)] = v[j];
                        __syncthreads();
                        layout = nl;
                        R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
                        F = (layout == LAYOUT_A) ? FA : FB;
#pragma unroll
                        for (int j = 0; j < NR; j++) v[j] = tile[F | ((uint32_t)j << R0)];
                        __syncthreads();
                    }
                    const uint32_t g1 = stage_end[s];
                    for (uint32_t gi = g0; gi < g1; gi++) tile_gate<P, K, R>(sg[gi], v, R0, F, 0);
                    g0 = g1;
                }
            }
            // <H>: ZZ + X on this layout's lane/register bits, then the other layout
            const uint32_t real = (n >= 32) ? ~0u : ((1u << n) - 1);
            const uint32_t here = (((1u << kLaneBits) - 1) | (((1u << R) - 1) << R0)) & real;
            hea_energy_tile<P, K, R>(acc, v, R0, F, n, chunk_off, K, 0, a.zz, a.xc, true, here);
            const uint32_t rest = real & ~here;
            if (rest) {
#pragma unroll
                for (int j = 0; j < NR; j++) tile[F | ((uint32_t)j << R0)] = v[j];
                __syncthreads();
                layout ^= 1;
                R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
                F = (layout == LAYOUT_A) ? FA : FB;
#pragma unroll
                for (int j = 0; j < NR; j++) v[j] = tile[F | ((uint32_t)j << R0)];
                hea_energy_tile<P, K, R>(acc, v, R0, F, n, chunk_off, K, 0, a.zz, a.xc, false, rest);
            }
        } else {
            // ---- tiled passes over the CTA's global slot ----
            const uint32_t h = n - K;           // high qubits
            const uint32_t lB = K - h;          // contiguous low qubits of pass B
            const uint64_t tiles = 1ull << h;
            const uint32_t npass = 2 * L + 1;  // A_0 B_0 ... A_{L-1} B_{L-1} + final A (read-only)
            for (uint32_t ps = 0; ps < npass; ps++) {
                const bool passB = (ps & 1u) != 0;
                const bool last_read = ps == npass - 1;
                const uint32_t ly = ps / 2;
                const uint32_t l = passB ? lB : (uint32_t)K;
                const uint32_t m = passB ? h : 0;
                __syncthreads();
                if (threadIdx.x == 0) {
                    for (uint32_t qq = 0; qq < 64; qq++) local[qq] = -1;
                    for (uint32_t qq = 0; qq < l; qq++) local[qq] = (int8_t)qq;
                    for (uint32_t j = 0; j < m; j++) local[K + j] = (int8_t)(l + j);
                    uint32_t nst = 0, cnt = 0;
                    if (!last_read) {
                        const double *al = ang + (size_t)ly * 2 * n;
                        cnt = passB ? hea_build<P, K, R>(sg, stage_layout, stage_end, nst, al, n, K, n, true, local)
                                    : hea_build<P, K, R>(sg, stage_layout, stage_end, nst, al, n, 0, K, false, local);
                    } else {
                        stage_layout[0] = LAYOUT_A;
                        stage_end[0] = 0;
                        nst = 1;
                    }
                    meta[1] = cnt;
                    meta[2] = nst;
                }
                for (uint32_t c = threadIdx.x; c < (1u << m); c += blockDim.x) {
                    uint64_t off = 0;
                    for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << (K + j);
                    chunk_off[c] = off;
                }
                // the previous pass's global stores before this pass's TMA reads
                asm volatile("fence.proxy.async;" ::: "memory");
                __syncthreads();
                const uint32_t nst = meta[2];
                const uint32_t chunk = 1u << l, nchunks = 1u << m;
                const uint64_t lowmask = chunk - 1;
                for (uint64_t tau = 0; tau < tiles; tau++) {
                    uint64_t base = tau << l;
                    for (uint32_t j = 0; j < m; j++) {
                        const uint32_t pos = K + j;
                        const uint64_t low = (1ull << pos) - 1;
                        base = ((base & ~low) << 1) | (base & low);
                    }
                    Amp v[NR];
                    int layout = stage_layout[0];
                    int R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
                    uint32_t F = (layout == LAYOUT_A) ? FA : FB;
                    if (ps == 0) {
#pragma unroll
                        for (int j = 0; j < NR; j++) {
                            const uint32_t u = F | ((uint32_t)j << R0);
                            v[j] = P::from_mem(mem_basis<Mem>(base == 0 && u == 0));
                        }
                    } else {
                        if (warp == 0) {
                            if (lane == 0) mbar_expect_tx(bar, (uint32_t)HK::kTileBytes);
                            __syncwarp();
                            for (uint32_t c = lane; c < nchunks; c += 32)
                                tma_load(tile_mem + (size_t)c * chunk, slot + base + chunk_off[c],
                                         chunk * (uint32_t)sizeof(Mem), bar);
                        }
                        if (!tile_wait(bar, phase & 1u, a.err)) return;
                        phase++;
#pragma unroll
                        for (int j = 0; j < NR; j++) v[j] = P::from_mem(tile_mem[F | ((uint32_t)j << R0)]);
                    }
                    uint32_t g0 = 0;
                    for (uint32_t s = 0; s < nst; s++) {
                        const int nl = stage_layout[s];
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
                        const uint32_t g1 = stage_end[s];
                        for (uint32_t gi = g0; gi < g1; gi++) tile_gate<P, K, R>(sg[gi], v, R0, F, base);
                        g0 = g1;
                    }
                    if (ps == npass - 2) {
                        // last B pass: ZZ everywhere + X on the pass-B qubits
                        uint32_t xB = 0;
                        for (uint32_t qq = 0; qq < lB; qq++) xB |= 1u << qq;
                        for (uint32_t j = 0; j < h; j++) xB |= 1u << (lB + j);
                        const uint32_t here = (((1u << kLaneBits) - 1) | (((1u << R) - 1) << R0)) & xB;
                        hea_energy_tile<P, K, R>(acc, v, R0, F, n, chunk_off, l, base, a.zz, a.xc, true, here);
                        if (xB & ~here) {
#pragma unroll
                            for (int j = 0; j < NR; j++) tile[F | ((uint32_t)j << R0)] = v[j];
                            __syncthreads();
                            const int ol = layout ^ 1;
                            const int oR0 = (ol == LAYOUT_A) ? kLaneBits : (K - R);
                            const uint32_t oF = (ol == LAYOUT_A) ? FA : FB;
                            Amp w[NR];
#pragma unroll
                            for (int j = 0; j < NR; j++) w[j] = tile[oF | ((uint32_t)j << oR0)];
                            hea_energy_tile<P, K, R>(acc, w, oR0, oF, n, chunk_off, l, base, a.zz, a.xc, false,
                                                     xB & ~here);
                            __syncthreads();
                        }
                    }
                    if (last_read) {
                        // qubits lB..K-1 (local bits of pass A) not covered by pass B
                        uint32_t xA = 0;
                        for (uint32_t qq = lB; qq < (uint32_t)K; qq++) xA |= 1u << qq;
                        const uint32_t here = (((1u << kLaneBits) - 1) | (((1u << R) - 1) << R0)) & xA;
                        hea_energy_tile<P, K, R>(acc, v, R0, F, n, chunk_off, l, base, a.zz, a.xc, false, here);
                        if (xA & ~here) {
#pragma unroll
                            for (int j = 0; j < NR; j++) tile[F | ((uint32_t)j << R0)] = v[j];
                            __syncthreads();
                            const int ol = layout ^ 1;
                            const int oR0 = (ol == LAYOUT_A) ? kLaneBits : (K - R);
                            const uint32_t oF = (ol == LAYOUT_A) ? FA : FB;
                            Amp w[NR];
#pragma unroll
                            for (int j = 0; j < NR; j++) w[j] = tile[oF | ((uint32_t)j << oR0)];
                            hea_energy_tile<P, K, R>(acc, w, oR0, oF, n, chunk_off, l, base, a.zz, a.xc, false,
                                                     xA & ~here);
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < NR; j++) {
                            const uint32_t u = F | ((uint32_t)j << R0);
                            slot[base + chunk_off[u >> l] + (u & lowmask)] = P::to_mem(v[j]);
                        }
                    }
                    fence_proxy_async();
                    __syncthreads();
                }
            }
        }
        // block reduction of <H>
        double e = acc.value();
        for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
        __syncthreads();
        if (lane == 0) red[warp] = e;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int w2 = 0; w2 < (int)(blockDim.x >> 5); w2++) t += red[w2];
            a.energies[job.id] = t;
        }
    }
}

template <class P, int K, int R>
static int32_t hea_run(const std::vector<HeaJob> &jobs, const std::vector<double> &params, double zz, double xc,
                       uint32_t nmax, double *energies_host) {
    using HK = HeaKernel<P, K, R>;
    using Mem = typename P::Mem;
    auto fail = [](cudaError_t e, const char *what) {
        cudaGetLastError();
        set_error(e == cudaErrorMemoryAllocation ? KBWG_ENOMEM : KBWG_ECUDA,
                  std::string("batch: ") + what + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? (int32_t)KBWG_ENOMEM : (int32_t)KBWG_ECUDA;
    };
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_hea_batch<P, K, R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)HK::kSmem);
    if (e != cudaSuccess) return fail(e, "setup");
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_hea_batch<P, K, R>, HK::kThreads, HK::kSmem);
    if (e != cudaSuccess) return fail(e, "occupancy");
    const uint32_t grid = (uint32_t)std::min<size_t>(jobs.size(), (size_t)sms * std::max(occ, 1));
    const uint64_t slot_elems = nmax > (uint32_t)K ? (1ull << nmax) : 0;
    cudaStream_t st = nullptr;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(e, "stream");
    char *dbuf = nullptr;
    const size_t jb = jobs.size() * sizeof(HeaJob), pb = std::max<size_t>(params.size(), 1) * sizeof(double),
                 eb = jobs.size() * sizeof(double), sb = (size_t)grid * slot_elems * sizeof(Mem);
    const size_t off_p = (jb + 255) & ~(size_t)255, off_e = (off_p + pb + 255) & ~(size_t)255,
                 off_c = (off_e + eb + 255) & ~(size_t)255, off_err = off_c + 256, off_s = off_err + 256;
    e = cudaMalloc(&dbuf, off_s + sb);
    if (e != cudaSuccess) {
        cudaStreamDestroy(st);
        return fail(e, "buffers");
    }
    HeaArgs a;
    memset(&a, 0, sizeof a);
    a.jobs = (const HeaJob *)dbuf;
    a.njobs = (uint32_t)jobs.size();
    a.next = (unsigned *)(dbuf + off_c);
    a.params = (const double *)(dbuf + off_p);
    a.zz = zz;
    a.xc = xc;
    a.energies = (double *)(dbuf + off_e);
    a.slots = dbuf + off_s;
    a.slot_elems = slot_elems;
    a.err = (int *)(dbuf + off_err);
    int err_flag = 0;
    e = copy_async(dbuf, jobs.data(), jb, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = copy_async(dbuf + off_p, params.data(), params.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dbuf + off_c, 0, 512, st);
    if (e == cudaSuccess) {
        k_hea_batch<P, K, R><<<grid, HK::kThreads, HK::kSmem, st>>>(a);
        count_launch();
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = copy_async(energies_host, a.energies, eb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = copy_async(&err_flag, a.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dbuf);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) return fail(e, "run");
    if (err_flag) {
        set_error(KBWG_ETIMEOUT, "batch: a bounded device-side wait ran out");
        return KBWG_ETIMEOUT;
    }
    return KBWG_OK;
}

int32_t hea_batch(int precision, bool fast_c128, size_t ncirc, const uint32_t *num_qubits, const uint32_t *layers,
                  const uint64_t *param_offset, const double *params, size_t nparams, double zz, double xc,
                  double *energies) {
    std::vector<HeaJob> jobs(ncirc);
    uint32_t nmax = 0;
    for (size_t c = 0; c < ncirc; c++) {
        const uint32_t n = num_qubits[c], L = layers[c];
        if (n < 2 || n > 21 || L > 64) {
            set_error(KBWG_EINVAL, "batch: every circuit needs 2 <= n <= 21 qubits and at most 64 layers");
            return KBWG_EINVAL;
        }
        if (param_offset[c] + 2ull * n * L > nparams) {
            set_error(KBWG_EINVAL, "batch: a circuit's angles run past the parameter array");
            return KBWG_EINVAL;
        }
        jobs[c] = HeaJob{n, L, (uint32_t)c, 0, param_offset[c]};
        nmax = std::max(nmax, n);
    }
    // largest first: the persistent CTAs then finish together
    std::stable_sort(jobs.begin(), jobs.end(), [](const HeaJob &x, const HeaJob &y) {
        return (double)(1ull << x.n) * (x.L + 1) > (double)(1ull << y.n) * (y.L + 1);
    });
    std::vector<double> p(params, params + nparams);
    if (precision == 0) return hea_run<Fast<float>, 13, 4>(jobs, p, zz, xc, nmax, energies);
    if (fast_c128) return hea_run<FFPol, 12, 4>(jobs, p, zz, xc, nmax, energies);
    return hea_run<Fast<double>, 12, 4>(jobs, p, zz, xc, nmax, energies);
}

}  // namespace kbwg
