// Device building blocks of the adjoint-gradient sweep, shared by the
// compiled two-state kernel (adjoint.cu) and its run-time specialised form
// (jit.cpp writes one kernel per reverse sweep; NVRTC compiles it): the
// gradient terms per arithmetic policy, the kernel parameters and geometry.
#pragma once

#include "jit_dev.cuh"
#include "sweep_dev.cuh"

namespace kbwg {

template <bool B, class A, class C> struct pick { using type = A; };
template <class A, class C> struct pick<false, A, C> { using type = C; };

// ---- gradient terms --------------------------------------------------------------------
// Contribution of one amplitude (lam, phi) whose pair partner is phip, on
// the |one> side of the target bit:
//   X: Im(conj(lam) phip)          Y: (one ? +1 : -1) Re(conj(lam) phip)
//   Z: (one ? -1 : +1) Im(conj(lam) phi)     P1: one ? -2 Im(conj(lam) phi) : 0
template <class P> struct Grad;

template <class T>
struct Grad<Fast<T>> {
    using Amp = cx<T>;
    using Acc = T;
    static __device__ __forceinline__ Acc zero() { return (T)0; }
    // (each product and sum rounded on its own: a contracted form would depend
    // on how the compiler fuses the surrounding code)
    static __device__ __forceinline__ T im_conj(Amp l, Amp b) { return xsub(xmul(l.re, b.im), xmul(l.im, b.re)); }
    static __device__ __forceinline__ T re_conj(Amp l, Amp b) { return xadd(xmul(l.re, b.re), xmul(l.im, b.im)); }
    static __device__ __forceinline__ Acc term(int gt, bool one, Amp l, Amp p, Amp pp) {
        switch (gt) {
        case GT_X: return im_conj(l, pp);
        case GT_Y: {
            const T r = re_conj(l, pp);
            return one ? r : -r;
        }
        case GT_Z: {
            const T r = im_conj(l, p);
            return one ? -r : r;
        }
        default: return one ? (T)-2 * im_conj(l, p) : (T)0;
        }
    }
    static __device__ __forceinline__ Acc add(Acc a, Acc b) { return a + b; }
    static __device__ __forceinline__ Acc warp_sum(Acc a) {
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        return a;
    }
    // per-warp accumulator across tiles: float-float for complex64 (no FP64
    // instruction in the sweep), binary64 for complex128
    using Wacc = typename pick<sizeof(T) == 4, ff::f2, double>::type;
    static __device__ __forceinline__ Wacc wadd(Wacc w, Acc a) {
        if constexpr (sizeof(T) == 4) return ff::add(w, ff::f2{a, 0.f});
        else return w + a;
    }
    static __device__ __forceinline__ double wvalue(Wacc w) {
        if constexpr (sizeof(T) == 4) return (double)w.h + (double)w.l;
        else return w;
    }
};

template <>
struct Grad<FFPol> {
    using Amp = FFPol::Amp;
    using Acc = ff::f2;
    static __device__ __forceinline__ Acc zero() { return ff::f2{0.f, 0.f}; }
    static __device__ __forceinline__ ff::f2 im_conj(const Amp &l, const Amp &b) {  // Im(conj(l) b)
        return ff::dot2(l.re, b.im, ff::neg(l.im), b.re);
    }
    static __device__ __forceinline__ ff::f2 re_conj(const Amp &l, const Amp &b) {  // Re(conj(l) b)
        return ff::dot2(l.re, b.re, l.im, b.im);
    }
    static __device__ __forceinline__ Acc term(int gt, bool one, const Amp &l, const Amp &p, const Amp &pp) {
        switch (gt) {
        case GT_X: return im_conj(l, pp);
        case GT_Y: {
            const ff::f2 r = re_conj(l, pp);
            return one ? r : ff::neg(r);
        }
        case GT_Z: {
            const ff::f2 r = im_conj(l, p);
            return one ? ff::neg(r) : r;
        }
        default: {
            if (!one) return zero();
            const ff::f2 r = im_conj(l, p);
            return ff::f2{-2.f * r.h, -2.f * r.l};
        }
        }
    }
    static __device__ __forceinline__ Acc add(Acc a, Acc b) { return ff::add(a, b); }
    static __device__ __forceinline__ Acc warp_sum(Acc a) {
        for (int o = 16; o > 0; o >>= 1) {
            Acc b{__shfl_xor_sync(0xffffffffu, a.h, o), __shfl_xor_sync(0xffffffffu, a.l, o)};
            a = ff::add(a, b);
        }
        return a;
    }
    using Wacc = ff::f2;
    static __device__ __forceinline__ Wacc wadd(Wacc w, Acc a) { return ff::add(w, a); }
    static __device__ __forceinline__ double wvalue(Wacc w) { return (double)w.h + (double)w.l; }
};

// Packed complex64 amplitudes (float2 re, im): the terms of Fast<float>.
template <>
struct Grad<FastP> {
    using Amp = FastP::Amp;
    using G1 = Grad<Fast<float>>;
    using Acc = G1::Acc;
    static __device__ __forceinline__ cx<float> unpack(Amp a) { return cx<float>{a.x, a.y}; }
    static __device__ __forceinline__ Acc zero() { return G1::zero(); }
    static __device__ __forceinline__ Acc term(int gt, bool one, Amp l, Amp p, Amp pp) {
        return G1::term(gt, one, unpack(l), unpack(p), unpack(pp));
    }
    static __device__ __forceinline__ Acc add(Acc a, Acc b) { return G1::add(a, b); }
    static __device__ __forceinline__ Acc warp_sum(Acc a) { return G1::warp_sum(a); }
    using Wacc = G1::Wacc;
    static __device__ __forceinline__ Wacc wadd(Wacc w, Acc a) { return G1::wadd(w, a); }
    static __device__ __forceinline__ double wvalue(Wacc w) { return G1::wvalue(w); }
};

// Packed float-float amplitudes: the terms of FFPol on the unpacked pairs.
template <>
struct Grad<FF2B> {
    using Amp = FF2B::Amp;
    using G1 = Grad<FFPol>;
    using Acc = G1::Acc;
    static __device__ __forceinline__ FFPol::Amp unpack(const Amp &a) {
        return FFPol::Amp{ff::f2{a.h.x, a.l.x}, ff::f2{a.h.y, a.l.y}};
    }
    static __device__ __forceinline__ Acc zero() { return G1::zero(); }
    static __device__ __forceinline__ Acc term(int gt, bool one, const Amp &l, const Amp &p, const Amp &pp) {
        return G1::term(gt, one, unpack(l), unpack(p), unpack(pp));
    }
    static __device__ __forceinline__ Acc add(Acc a, Acc b) { return G1::add(a, b); }
    static __device__ __forceinline__ Acc warp_sum(Acc a) { return G1::warp_sum(a); }
    using Wacc = G1::Wacc;
    static __device__ __forceinline__ Wacc wadd(Wacc w, Acc a) { return G1::wadd(w, a); }
    static __device__ __forceinline__ double wvalue(Wacc w) { return G1::wvalue(w); }
};

// Float-float resident states (the forward sweeps' form): the same terms.
template <>
struct Grad<FF2> : Grad<FF2B> {};

template <class P, int R, int B>
__device__ __forceinline__ typename Grad<P>::Acc grad_pairs(int gt, const typename P::Amp (&ph)[1 << R],
                                                           const typename P::Amp (&la)[1 << R], uint32_t creg) {
    using G = Grad<P>;
    typename G::Acc acc = G::zero();
#pragma unroll
    for (int jj = 0; jj < (1 << (R - 1)); jj++) {
        const int j0 = ((jj >> B) << (B + 1)) | (jj & ((1 << B) - 1));
        const int j1 = j0 | (1 << B);
        if (creg == 0u || ((uint32_t)j0 & creg) == creg) {
            acc = G::add(acc, G::term(gt, false, la[j0], ph[j0], ph[j1]));
            acc = G::add(acc, G::term(gt, true, la[j1], ph[j1], ph[j0]));
        }
    }
    return acc;
}

// This thread's part of the gradient inner product of one step.  Every lane
// must call it (lane-bit targets shuffle).
template <class P, int K, int R>
__device__ __forceinline__ typename Grad<P>::Acc grad_partial(const TileGate &g, int gt,
                                                             const typename P::Amp (&ph)[1 << R],
                                                             const typename P::Amp (&la)[1 << R], int R0,
                                                             uint32_t F, uint64_t base) {
    using G = Grad<P>;
    constexpr int NR = 1 << R;
    typename G::Acc acc = G::zero();
    const uint32_t regmask = (uint32_t)(NR - 1) << R0;
    const uint32_t fixed_need = g.cl & ~regmask;
    const bool fok = (F & fixed_need) == fixed_need;
    const uint32_t creg = (g.cl & regmask) >> R0;
    const uint32_t tb = g.tb;
    if (gt == GT_Z || gt == GT_P1) {
        if (!fok) return acc;
        const int rb = (int)tb - R0;
        if (tb != TG_OUTER && rb >= 0 && rb < R) {
#pragma unroll
            for (int j = 0; j < NR; j++)
                if (creg == 0u || ((uint32_t)j & creg) == creg)
                    acc = G::add(acc, G::term(gt, ((j >> rb) & 1) != 0, la[j], ph[j], ph[j]));
        } else {
            const bool one = (tb == TG_OUTER) ? (((base >> g.tout) & 1ull) != 0) : (((F >> tb) & 1u) != 0);
#pragma unroll
            for (int j = 0; j < NR; j++)
                if (creg == 0u || ((uint32_t)j & creg) == creg) acc = G::add(acc, G::term(gt, one, la[j], ph[j], ph[j]));
        }
        return acc;
    }
    if (tb < (uint32_t)kLaneBits) {
        const bool one = ((F >> tb) & 1u) != 0;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const typename P::Amp pp = P::shfl(ph[j], 1 << tb);
            if (fok && (creg == 0u || ((uint32_t)j & creg) == creg)) acc = G::add(acc, G::term(gt, one, la[j], ph[j], pp));
        }
        return acc;
    }
    if (!fok) return acc;
    switch ((int)tb - R0) {
    case 0: return grad_pairs<P, R, 0>(gt, ph, la, creg);
    case 1: return grad_pairs<P, R, 1>(gt, ph, la, creg);
    case 2: return grad_pairs<P, R, 2>(gt, ph, la, creg);
    default:
        if constexpr (R > 3) return grad_pairs<P, R, (R > 3 ? 3 : 0)>(gt, ph, la, creg);
        return acc;
    }
}

// ---- two-state adjoint sweep -------------------------------------------------------------
template <class T> struct AdjCfg;
template <> struct AdjCfg<float> {
    static constexpr int K = 12, R = 4;
};
template <> struct AdjCfg<double> {
    static constexpr int K = 11, R = 3;
};

struct AdjParams {
    SweepParams sw;
    const uint32_t *ginfo;  // per program gate: gradient type | (slot << 4)
    double *partials;       // [gridDim.x][nslots]
    uint32_t nslots;
};

template <class P, int K, int R>
struct AdjKernel {
    using Mem = typename P::Mem;
    static constexpr int kThreads = 32 << (K - kLaneBits - R);
    static constexpr int kWarps = kThreads / 32;
    static constexpr size_t kTileBytes = sizeof(Mem) << K;
    static constexpr size_t kSmem = 2 * kTileBytes + 256 * sizeof(uint64_t) + kMaxSweepGates * sizeof(TileGate) +
                                    kMaxSweepGates * sizeof(uint32_t) + (size_t)kWarps * kMaxSweepGates * sizeof(double) +
                                    16;
};

// ---- run-time specialised reverse sweep ---------------------------------------------
namespace jit {

// Gradient part of a diagonal-generator step (RZ: GT_Z, P: GT_P1) whose
// target is register bit RB; CREG: controls on register bits.
template <class P, int R, int GT, int RB, uint32_t CREG>
__device__ __forceinline__ typename Grad<P>::Acc grad_dreg(const typename P::Amp (&ph)[1 << R],
                                                          const typename P::Amp (&la)[1 << R]) {
    using G = Grad<P>;
    typename G::Acc acc = G::zero();
#pragma unroll
    for (int j = 0; j < (1 << R); j++)
        if (((uint32_t)j & CREG) == CREG) acc = G::add(acc, G::term(GT, ((j >> RB) & 1) != 0, la[j], ph[j], ph[j]));
    return acc;
}

// The same with the target side fixed for the thread (lane/warp bit, or a
// qubit outside the tile).
template <class P, int R, int GT, uint32_t CREG>
__device__ __forceinline__ typename Grad<P>::Acc grad_dfix(const typename P::Amp (&ph)[1 << R],
                                                          const typename P::Amp (&la)[1 << R], bool one) {
    using G = Grad<P>;
    typename G::Acc acc = G::zero();
#pragma unroll
    for (int j = 0; j < (1 << R); j++)
        if (((uint32_t)j & CREG) == CREG) acc = G::add(acc, G::term(GT, one, la[j], ph[j], ph[j]));
    return acc;
}

// RX/RY step whose target is lane bit TB: the partner comes by shuffle, so
// every lane calls it; fok (controls on lane/warp bits) selects after.
template <class P, int R, int GT, int TB, uint32_t CREG>
__device__ __forceinline__ typename Grad<P>::Acc grad_lane(const typename P::Amp (&ph)[1 << R],
                                                          const typename P::Amp (&la)[1 << R], bool fok, uint32_t F) {
    using G = Grad<P>;
    typename G::Acc acc = G::zero();
    const bool one = ((F >> TB) & 1u) != 0u;
#pragma unroll
    for (int j = 0; j < (1 << R); j++) {
        if (((uint32_t)j & CREG) != CREG) continue;
        const typename P::Amp pp = P::shfl(ph[j], 1 << TB);
        if (fok) acc = G::add(acc, G::term(GT, one, la[j], ph[j], pp));
    }
    return acc;
}

// RX/RY step whose target is register bit B.
template <class P, int R, int GT, int B, uint32_t CREG>
__device__ __forceinline__ typename Grad<P>::Acc grad_reg(const typename P::Amp (&ph)[1 << R],
                                                         const typename P::Amp (&la)[1 << R]) {
    return grad_pairs<P, R, B>(GT, ph, la, CREG);
}

// Layout change of both states through their shared-memory tiles (one barrier).
template <class P, int K, int R, int FROM, int TO>
__device__ __forceinline__ void relayout2(typename P::Amp (&vp)[1 << R], typename P::Amp (&vl)[1 << R],
                                          typename P::Amp *tp, typename P::Amp *tl, uint32_t FA, uint32_t FB) {
    constexpr int R0f = (FROM == LAYOUT_A) ? kLaneBits : (K - R);
    constexpr int R0t = (TO == LAYOUT_A) ? kLaneBits : (K - R);
    const uint32_t Ff = (FROM == LAYOUT_A) ? FA : FB;
    const uint32_t Ft = (TO == LAYOUT_A) ? FA : FB;
#pragma unroll
    for (int j = 0; j < (1 << R); j++) {
        tp[Ff | ((uint32_t)j << R0f)] = vp[j];
        tl[Ff | ((uint32_t)j << R0f)] = vl[j];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < (1 << R); j++) {
        vp[j] = tp[Ft | ((uint32_t)j << R0t)];
        vl[j] = tl[Ft | ((uint32_t)j << R0t)];
    }
}

// Add a warp's part w of gradient slot SL to the warp's accumulator.
template <class P, int SL>
__device__ __forceinline__ void grad_store(typename Grad<P>::Wacc *acc, typename Grad<P>::Acc part) {
    using G = Grad<P>;
    const typename G::Acc w = G::warp_sum(part);
    if ((threadIdx.x & 31) == 0) {
        typename G::Wacc &slot = acc[(threadIdx.x >> 5) * kMaxSweepGates + SL];
        slot = G::wadd(slot, w);
    }
}

// The reverse sweep: k_adjoint's persistent two-state tile loop with the
// gate program (gradient parts, then the inverse gate on both states)
// replaced by Body::run.
template <class P, int K, int R, class Body>
__device__ __forceinline__ void adjoint_sweep(typename P::Mem *__restrict__ phi, typename P::Mem *__restrict__ lam,
                                              const AdjParams &a) {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    using AK = AdjKernel<P, K, R>;
    using G = Grad<P>;
    using Wacc = typename G::Wacc;
    constexpr int NR = 1 << R;
    const SweepParams &p = a.sw;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Mem *tphi_m = reinterpret_cast<Mem *>(smem_raw);
    Mem *tlam_m = reinterpret_cast<Mem *>(smem_raw + AK::kTileBytes);
    Amp *tphi = reinterpret_cast<Amp *>(smem_raw);
    Amp *tlam = reinterpret_cast<Amp *>(smem_raw + AK::kTileBytes);
    unsigned char *q = smem_raw + 2 * AK::kTileBytes;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(q);
    q += 256 * sizeof(uint64_t);
    TileGate *sg = reinterpret_cast<TileGate *>(q);
    q += kMaxSweepGates * sizeof(TileGate);
    q += kMaxSweepGates * sizeof(uint32_t);  // (gradient info: compiled in)
    Wacc *acc = reinterpret_cast<Wacc *>(q);  // [kWarps][kMaxSweepGates]
    q += (size_t)AK::kWarps * kMaxSweepGates * sizeof(Wacc);
    uint64_t *bar = reinterpret_cast<uint64_t *>(q);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t l = p.l, m = p.m;
    const uint32_t chunk = 1u << l, nchunks = 1u << m;
    const uint32_t chunk_bytes = chunk * (uint32_t)sizeof(Mem);
    const uint64_t lowmask = chunk - 1;

    for (uint32_t i = threadIdx.x; i < p.gate_count; i += blockDim.x) sg[i] = p.prog[i];
    for (uint32_t i = threadIdx.x; i < (uint32_t)AK::kWarps * kMaxSweepGates; i += blockDim.x) acc[i] = Wacc{};
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
            if (lane == 0) mbar_expect_tx(bar, (uint32_t)(2 * AK::kTileBytes));
            __syncwarp();
            for (uint32_t c = lane; c < nchunks; c += 32) {
                tma_load(tphi_m + (size_t)c * chunk, phi + b + chunk_off[c], chunk_bytes, bar);
                tma_load(tlam_m + (size_t)c * chunk, lam + b + chunk_off[c], chunk_bytes, bar);
            }
        }
    };

    uint64_t tau = blockIdx.x;
    if (tau < p.tiles) issue_load(tau);
    const uint32_t FA = (uint32_t)lane | ((uint32_t)warp << (kLaneBits + R));
    const uint32_t FB = (uint32_t)lane | ((uint32_t)warp << kLaneBits);
    constexpr int R0first = (Body::kFirst == LAYOUT_A) ? kLaneBits : (K - R);
    constexpr int R0last = (Body::kLast == LAYOUT_A) ? kLaneBits : (K - R);
    const uint32_t Ffirst = (Body::kFirst == LAYOUT_A) ? FA : FB;
    const uint32_t Flast = (Body::kLast == LAYOUT_A) ? FA : FB;
    for (uint32_t it = 0; tau < p.tiles; tau += gridDim.x, it++) {
        const uint64_t base = tile_base(tau);
        if (!tile_wait(bar, it & 1u, p.err)) return;
        Amp vp[NR], vl[NR];
#pragma unroll
        for (int j = 0; j < NR; j++) {
            vp[j] = P::from_mem(tphi_m[Ffirst | ((uint32_t)j << R0first)]);
            vl[j] = P::from_mem(tlam_m[Ffirst | ((uint32_t)j << R0first)]);
        }
        Body::template run<P, K, R>(vp, vl, tphi, tlam, FA, FB, base, sg, acc);
        fence_proxy_async();
        __syncthreads();
        const uint64_t next = tau + gridDim.x;
        if (next < p.tiles) issue_load(next);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t u = Flast | ((uint32_t)j << R0last);
            const uint64_t idx = base + chunk_off[u >> l] + (u & lowmask);
            phi[idx] = P::to_mem(vp[j]);
            lam[idx] = P::to_mem(vl[j]);
        }
    }
    __syncthreads();
    for (uint32_t sl = threadIdx.x; sl < a.nslots; sl += blockDim.x) {
        double t = 0.0;
        for (int w = 0; w < AK::kWarps; w++) t += G::wvalue(acc[w * kMaxSweepGates + sl]);
        a.partials[(size_t)blockIdx.x * a.nslots + sl] = t;
    }
}

}  // namespace jit
}  // namespace kbwg
