// Device building blocks of the tile sweeps, shared by the forward sweep
// (sweep.cu) and the adjoint-gradient sweep (adjoint.cu): TMA/mbarrier
// wrappers, the two arithmetic policies (exact reference order, float-float)
// and the per-gate register/shuffle code.
#pragma once

#include <string.h>

#include "ff.cuh"
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
// Orders this thread's generic-proxy shared-memory accesses before later
// async-proxy (TMA) accesses to the same memory.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ uint64_t insert_zero_at(uint64_t i, uint32_t m) {
    const uint64_t low = (1ull << m) - 1;
    return ((i & ~low) << 1) | (i & low);
}

// ---- exact arithmetic policy (reference operation order) ----------------------
template <class T>
struct Exact {
    using Amp = cx<T>;
    using Mem = cx<T>;  // amplitude format in HBM
    static __device__ __forceinline__ Amp from_mem(Mem a) { return a; }
    static __device__ __forceinline__ Mem to_mem(Amp a) { return a; }
    // Constants are stored in T on the host (exact: they are T values widened
    // to double), so no thread converts precision at run time (a float<->double
    // conversion issues at the FP64 rate on this chip).
    static void pack_host(TileGate &g) {
        T v[4];
        for (int i = 0; i < 4; i++) v[i] = (T)g.c[i];
        memset(g.c, 0, sizeof g.c);
        memcpy(g.c, v, sizeof v);
    }
    struct K4 {
        T c0, c1, c2, c3;
    };
    static __device__ __forceinline__ K4 load(const TileGate &g) {
        const T *v = reinterpret_cast<const T *>(g.c);
        return K4{v[0], v[1], v[2], v[3]};
    }
    static __device__ __forceinline__ Amp shfl(Amp v, int m) {
        Amp r;
        r.re = __shfl_xor_sync(0xffffffffu, v.re, m);
        r.im = __shfl_xor_sync(0xffffffffu, v.im, m);
        return r;
    }
    // X: swap.  Y: a0' = a1*(-i) = (a1.im, -a1.re), a1' = a0*i = (-a0.im, a0.re).
    static __device__ __forceinline__ void perm_pair(int sub, Amp &a0, Amp &a1) {
        if (sub == 0) {
            const Amp t = a0;
            a0 = a1;
            a1 = t;
        } else {
            const Amp n0{a1.im, xneg(a1.re)}, n1{xneg(a0.im), a0.re};
            a0 = n0;
            a1 = n1;
        }
    }
    static __device__ __forceinline__ Amp perm_half(int sub, Amp o, bool one) {
        if (sub == 0) return o;
        return one ? Amp{xneg(o.im), o.re} : Amp{o.im, xneg(o.re)};
    }
    // H: a0' = (a0 + a1) * h, a1' = (a0 - a1) * h
    static __device__ __forceinline__ void h_pair(int, const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0{xmul(xadd(a0.re, a1.re), k.c0), xmul(xadd(a0.im, a1.im), k.c0)};
        const Amp n1{xmul(xsub(a0.re, a1.re), k.c0), xmul(xsub(a0.im, a1.im), k.c0)};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp h_half(int, const K4 &k, Amp self, Amp o, bool one) {
        return one ? Amp{xmul(xsub(o.re, self.re), k.c0), xmul(xsub(o.im, self.im), k.c0)}
                   : Amp{xmul(xadd(self.re, o.re), k.c0), xmul(xadd(self.im, o.im), k.c0)};
    }
    // RY/RX: x' = c*x + s*t, t = -partner (RY, |0> side), +partner (RY, |1>
    // side), or (partner.im, -partner.re) (RX, either side); the same roundings
    // as the reference's c*x -/+ s*y forms.
    static __device__ __forceinline__ Amp rot_t(int sub, Amp o, bool one) {
        if (sub == 1) return Amp{o.im, xneg(o.re)};
        return one ? o : Amp{xneg(o.re), xneg(o.im)};
    }
    static __device__ __forceinline__ Amp rot_mix(const K4 &k, Amp x, Amp t) {
        return Amp{xadd(xmul(k.c0, x.re), xmul(k.c1, t.re)), xadd(xmul(k.c0, x.im), xmul(k.c1, t.im))};
    }
    static __device__ __forceinline__ void rot_pair(int sub, const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0 = rot_mix(k, a0, rot_t(sub, a1, false));
        const Amp n1 = rot_mix(k, a1, rot_t(sub, a0, true));
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp rot_half(int sub, const K4 &k, Amp self, Amp o, bool one) {
        return rot_mix(k, self, rot_t(sub, o, one));
    }
    // Z: negate the |1> amplitude; P: |1> * (c0 + i c1); RZ: |0> * (c0 + i c1), |1> * (c2 + i c3).
    static __device__ __forceinline__ Amp diag(int sub, const K4 &k, Amp a, bool one) {
        if (sub == 0) return one ? Amp{xneg(a.re), xneg(a.im)} : a;
        if (sub == 1) return one ? cmul_exact(a, k.c0, k.c1) : a;
        return one ? cmul_exact(a, k.c2, k.c3) : cmul_exact(a, k.c0, k.c1);
    }
};

// ---- float-float policy (complex128 fast path) ---------------------------------
// HBM keeps IEEE binary64; amplitudes become hi+lo float pairs on the way in
// and are rounded back on the way out.  Constants arrive pre-split by
// pack_host.  Extra classes used only here: H sub 1 (no 1/sqrt(2): the host
// folds it into a final scale gate), DIAG sub 3 (|1> times i^q, free) and
// DIAG sub 5 (every amplitude times c0 + i c1, the folded global factor).
struct FFPol {
    struct Amp {
        ff::f2 re, im;
    };
    using Mem = cx<double>;
    struct K4 {
        ff::f2 c0, c1, c2, c3;
    };
    static __device__ __forceinline__ Amp from_mem(Mem a) {
        return Amp{ff::from_double(a.re), ff::from_double(a.im)};
    }
    static __device__ __forceinline__ Mem to_mem(Amp a) { return Mem{ff::to_double(a.re), ff::to_double(a.im)}; }
    static void pack_host(TileGate &g) {
        float f[8];
        for (int i = 0; i < 4; i++) {
            const ff::f2 v = ff::split_constant(g.c[i]);
            f[2 * i] = v.h;
            f[2 * i + 1] = v.l;
        }
        memcpy(g.c, f, sizeof f);
    }
    static __device__ __forceinline__ K4 load(const TileGate &g) {
        const float *f = reinterpret_cast<const float *>(g.c);
        return K4{{f[0], f[1]}, {f[2], f[3]}, {f[4], f[5]}, {f[6], f[7]}};
    }
    static __device__ __forceinline__ Amp shfl(Amp v, int m) {
        Amp r;
        r.re.h = __shfl_xor_sync(0xffffffffu, v.re.h, m);
        r.re.l = __shfl_xor_sync(0xffffffffu, v.re.l, m);
        r.im.h = __shfl_xor_sync(0xffffffffu, v.im.h, m);
        r.im.l = __shfl_xor_sync(0xffffffffu, v.im.l, m);
        return r;
    }
    static __device__ __forceinline__ void perm_pair(int sub, Amp &a0, Amp &a1) {
        if (sub == 0) {
            const Amp t = a0;
            a0 = a1;
            a1 = t;
        } else {
            const Amp n0{a1.im, ff::neg(a1.re)}, n1{ff::neg(a0.im), a0.re};
            a0 = n0;
            a1 = n1;
        }
    }
    static __device__ __forceinline__ Amp perm_half(int sub, Amp o, bool one) {
        if (sub == 0) return o;
        return one ? Amp{ff::neg(o.im), o.re} : Amp{o.im, ff::neg(o.re)};
    }
    static __device__ __forceinline__ void h_pair(int sub, const K4 &k, Amp &a0, Amp &a1) {
        Amp n0{ff::add(a0.re, a1.re), ff::add(a0.im, a1.im)};
        Amp n1{ff::sub(a0.re, a1.re), ff::sub(a0.im, a1.im)};
        if (sub == 0) {
            n0 = Amp{ff::mul(n0.re, k.c0), ff::mul(n0.im, k.c0)};
            n1 = Amp{ff::mul(n1.re, k.c0), ff::mul(n1.im, k.c0)};
        }
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp h_half(int sub, const K4 &k, Amp self, Amp o, bool one) {
        Amp r = one ? Amp{ff::sub(o.re, self.re), ff::sub(o.im, self.im)}
                    : Amp{ff::add(self.re, o.re), ff::add(self.im, o.im)};
        if (sub == 0) r = Amp{ff::mul(r.re, k.c0), ff::mul(r.im, k.c0)};
        return r;
    }
    static __device__ __forceinline__ Amp rot_t(int sub, Amp o, bool one) {
        if (sub == 1) return Amp{o.im, ff::neg(o.re)};
        return one ? o : Amp{ff::neg(o.re), ff::neg(o.im)};
    }
    static __device__ __forceinline__ Amp rot_mix(const K4 &k, Amp x, Amp t) {
        return Amp{ff::dot2(k.c0, x.re, k.c1, t.re), ff::dot2(k.c0, x.im, k.c1, t.im)};
    }
    static __device__ __forceinline__ void rot_pair(int sub, const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0 = rot_mix(k, a0, rot_t(sub, a1, false));
        const Amp n1 = rot_mix(k, a1, rot_t(sub, a0, true));
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp rot_half(int sub, const K4 &k, Amp self, Amp o, bool one) {
        return rot_mix(k, self, rot_t(sub, o, one));
    }
    static __device__ __forceinline__ Amp cmul(Amp a, ff::f2 c, ff::f2 s) {
        return Amp{ff::dot2(c, a.re, ff::neg(s), a.im), ff::dot2(c, a.im, s, a.re)};
    }
    static __device__ __forceinline__ Amp diag(int sub, const K4 &k, Amp a, bool one) {
        switch (sub) {
        case 0: return one ? Amp{ff::neg(a.re), ff::neg(a.im)} : a;
        case 1: return one ? cmul(a, k.c0, k.c1) : a;
        case 2: return one ? cmul(a, k.c2, k.c3) : cmul(a, k.c0, k.c1);
        case 3: {
            if (!one) return a;
            const int q = (int)k.c0.h;
            if (q == 1) return Amp{ff::neg(a.im), a.re};
            if (q == 2) return Amp{ff::neg(a.re), ff::neg(a.im)};
            return Amp{a.im, ff::neg(a.re)};
        }
        default: return cmul(a, k.c0, k.c1);
        }
    }
};

template <class P, int R, int B, int CLS>
__device__ __forceinline__ void reg_pairs(typename P::Amp (&v)[1 << R], const TileGate &g,
                                          const typename P::K4 &k, uint32_t creg) {
    // creg == 0 (no control on a register bit) is the common case: no
    // per-pair test at all
#pragma unroll
    for (int jj = 0; jj < (1 << (R - 1)); jj++) {
        const int j0 = ((jj >> B) << (B + 1)) | (jj & ((1 << B) - 1));
        const int j1 = j0 | (1 << B);
        if (creg == 0u || ((uint32_t)j0 & creg) == creg) {
            if (CLS == TG_PERM) P::perm_pair(g.sub, v[j0], v[j1]);
            if (CLS == TG_H) P::h_pair(g.sub, k, v[j0], v[j1]);
            if (CLS == TG_ROT) P::rot_pair(g.sub, k, v[j0], v[j1]);
        }
    }
}

template <class P, int R, int CLS>
__device__ __forceinline__ void reg_gate(typename P::Amp (&v)[1 << R], const TileGate &g, const typename P::K4 &k,
                                         int b, uint32_t creg) {
    switch (b) {
    case 0: reg_pairs<P, R, 0, CLS>(v, g, k, creg); break;
    case 1: reg_pairs<P, R, 1, CLS>(v, g, k, creg); break;
    case 2: reg_pairs<P, R, 2, CLS>(v, g, k, creg); break;
    case 3: reg_pairs<P, R, 3, CLS>(v, g, k, creg); break;
    default: reg_pairs<P, R, R - 1, CLS>(v, g, k, creg); break;
    }
}

// Apply one gate to the thread's registers.  F = the thread's fixed local
// bits (lane and warp), R0 = first local bit held in registers.
template <class P, int K, int R>
__device__ __forceinline__ void tile_gate(const TileGate &g, typename P::Amp (&v)[1 << R], int R0, uint32_t F,
                                          uint64_t base) {
    static_assert(R == 4 || R == 5, "reg_gate covers register bits 0..4");
    constexpr int NR = 1 << R;
    if ((base & g.co) != g.co) return;  // a control outside the tile is 0 for the whole tile
    const uint32_t regmask = (uint32_t)(NR - 1) << R0;
    const uint32_t fixed_need = g.cl & ~regmask;
    const bool fok = (F & fixed_need) == fixed_need;  // controls on this thread's lane/warp bits
    const uint32_t tb = g.tb;
    const bool lane_target = g.cls != TG_DIAG && tb < (uint32_t)kLaneBits;
    // Threads whose lane/warp controls are 0 leave, except for lane-bit
    // targets: there every lane must take part in the warp shuffle.
    if (!fok && !lane_target) return;
    const typename P::K4 k = P::load(g);
    const uint32_t creg = (g.cl & regmask) >> R0;
    if (g.cls == TG_DIAG) {
        const int rb = (int)tb - R0;
        if (tb != TG_OUTER && rb >= 0 && rb < R) {  // target bit is a register bit
#pragma unroll
            for (int j = 0; j < NR; j++)
                if (creg == 0u || ((uint32_t)j & creg) == creg) v[j] = P::diag(g.sub, k, v[j], ((j >> rb) & 1) != 0);
        } else {  // target fixed for this thread (lane/warp bit) or for the whole tile
            const bool one = (tb == TG_OUTER) ? (((base >> g.tout) & 1ull) != 0) : (((F >> tb) & 1u) != 0);
#pragma unroll
            for (int j = 0; j < NR; j++)
                if (creg == 0u || ((uint32_t)j & creg) == creg) v[j] = P::diag(g.sub, k, v[j], one);
        }
        return;
    }
    if (lane_target) {
        // partner lives in lane F ^ (1 << tb); a control on a lane bit has the
        // same value on both halves of a pair (it is never the target bit)
        const bool one = ((F >> tb) & 1u) != 0;
        const int m = 1 << tb;
        if (g.cls == TG_PERM) {
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const typename P::Amp o = P::shfl(v[j], m);
                if (fok && (creg == 0u || ((uint32_t)j & creg) == creg)) v[j] = P::perm_half(g.sub, o, one);
            }
        } else if (g.cls == TG_H) {
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const typename P::Amp o = P::shfl(v[j], m);
                if (fok && (creg == 0u || ((uint32_t)j & creg) == creg)) v[j] = P::h_half(g.sub, k, v[j], o, one);
            }
        } else {
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const typename P::Amp o = P::shfl(v[j], m);
                if (fok && (creg == 0u || ((uint32_t)j & creg) == creg)) v[j] = P::rot_half(g.sub, k, v[j], o, one);
            }
        }
        return;
    }
    const int b = (int)tb - R0;
    if (g.cls == TG_PERM)
        reg_gate<P, R, TG_PERM>(v, g, k, b, creg);
    else if (g.cls == TG_H)
        reg_gate<P, R, TG_H>(v, g, k, b, creg);
    else
        reg_gate<P, R, TG_ROT>(v, g, k, b, creg);
}


}  // namespace kbwg
