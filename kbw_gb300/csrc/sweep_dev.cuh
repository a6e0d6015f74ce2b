// Device building blocks of the tile sweeps, shared by the forward sweep
// (sweep.cu) and the adjoint-gradient sweep (adjoint.cu): TMA/mbarrier
// wrappers, the two arithmetic policies (exact reference order, float-float)
// and the per-gate register/shuffle code.
#pragma once

#if !defined(__CUDACC_RTC__)
#include <string.h>
#endif

#include "ff.cuh"
#include "ff2.cuh"
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
// Every thread of the CTA waits for phase `parity` of a TMA mbarrier with a
// bounded number of polls (the only wait the tile kernels have).  If any
// thread's polls run out, thread 0 sets *err (the host turns it into
// KBWG_ETIMEOUT), the threads that gave up poll once more, again bounded, so
// that the copies they waited for can land before the CTA releases its
// shared memory, and every thread gets false: the caller returns.
__device__ __forceinline__ bool tile_wait(uint64_t *bar, uint32_t parity, int *err, uint32_t spins = 1u << 22) {
    bool ok = false;
    for (uint32_t spin = 0; spin < spins; spin++)
        if (mbar_try_wait(bar, parity)) {
            ok = true;
            break;
        }
    if (!__syncthreads_or(!ok)) return true;
    if (threadIdx.x == 0) atomicExch(err, 1);
    for (uint32_t spin = 0; !ok && spin < spins; spin++) ok = mbar_try_wait(bar, parity);
    return false;
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

// ---- arithmetic policies ----------------------------------------------------------
// A policy supplies the amplitude type in registers (Amp) and in HBM (Mem),
// the per-gate constants (K4), and one function per gate class.  *_pair
// updates both amplitudes of a pair held by one thread; *_half returns the new
// value of one side (`self`) given the other side (`o`) from another lane.

// Exact: the reference's per-amplitude operations, each product and sum
// rounded separately (no FMA contraction): bit-identical to Dense<F>.
template <class T>
struct Exact {
    using Amp = cx<T>;
    using Mem = cx<T>;
    using Scalar = T;
    static __device__ __forceinline__ Amp from_mem(Mem a) { return a; }
    static __device__ __forceinline__ Mem to_mem(Amp a) { return a; }
    // Constants are stored in T on the host (exact: they are T values widened
    // to double), so no thread converts precision at run time (a
    // float<->double conversion issues at the FP64 rate on this chip).
#if !defined(__CUDACC_RTC__)
    static void pack_host(TileGate &g) {
        T v[4];
        for (int i = 0; i < 4; i++) v[i] = (T)g.c[i];
        memset(g.c, 0, sizeof g.c);
        memcpy(g.c, v, sizeof v);
    }
#endif
    struct K4 {
        T c0, c1, c2, c3;
    };
    static __device__ __forceinline__ K4 load(const TileGate &g) {
        const T *v = reinterpret_cast<const T *>(g.c);
        return K4{v[0], v[1], v[2], v[3]};
    }
    static __device__ __forceinline__ Amp shfl(Amp v, int m) {
        return Amp{__shfl_xor_sync(0xffffffffu, v.re, m), __shfl_xor_sync(0xffffffffu, v.im, m)};
    }
    static __device__ __forceinline__ Amp neg(Amp a) { return Amp{-a.re, -a.im}; }
    // Y: a0' = a1*(-i) = (a1.im, -a1.re), a1' = a0*i = (-a0.im, a0.re)
    static __device__ __forceinline__ void y_pair(Amp &a0, Amp &a1) {
        const Amp n0{a1.im, -a1.re}, n1{-a0.im, a0.re};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp y_half(Amp o, bool one) {
        return one ? Amp{-o.im, o.re} : Amp{o.im, -o.re};
    }
    // H: a0' = (a0 + a1) h, a1' = (a0 - a1) h
    static __device__ __forceinline__ void h_pair(int, const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0{xmul(xadd(a0.re, a1.re), k.c0), xmul(xadd(a0.im, a1.im), k.c0)};
        const Amp n1{xmul(xsub(a0.re, a1.re), k.c0), xmul(xsub(a0.im, a1.im), k.c0)};
        a0 = n0;
        a1 = n1;
    }
    // sgn = +1 on the |0> side, -1 on the |1> side: (o + sgn*self) rounds
    // exactly like self + o resp. o - self, and sgn*self is exact, so one FMA
    // gives the reference's sum.
    static __device__ __forceinline__ Amp h_half(int, const K4 &k, Amp self, Amp o, T sgn) {
        return Amp{xmul(fma(sgn, self.re, o.re), k.c0), xmul(fma(sgn, self.im, o.im), k.c0)};
    }
    // RX: a0' = (c a0.re + s a1.im, c a0.im - s a1.re), a1' symmetric
    static __device__ __forceinline__ void rx_pair(const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0{xadd(xmul(k.c0, a0.re), xmul(k.c1, a1.im)), xsub(xmul(k.c0, a0.im), xmul(k.c1, a1.re))};
        const Amp n1{xadd(xmul(k.c0, a1.re), xmul(k.c1, a0.im)), xsub(xmul(k.c0, a1.im), xmul(k.c1, a0.re))};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp rx_half(const K4 &k, Amp self, Amp o) {
        return Amp{xadd(xmul(k.c0, self.re), xmul(k.c1, o.im)), xsub(xmul(k.c0, self.im), xmul(k.c1, o.re))};
    }
    // RY: a0' = c a0 - s a1, a1' = c a1 + s a0
    static __device__ __forceinline__ void ry_pair(const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0{xsub(xmul(k.c0, a0.re), xmul(k.c1, a1.re)), xsub(xmul(k.c0, a0.im), xmul(k.c1, a1.im))};
        const Amp n1{xadd(xmul(k.c0, a1.re), xmul(k.c1, a0.re)), xadd(xmul(k.c0, a1.im), xmul(k.c1, a0.im))};
        a0 = n0;
        a1 = n1;
    }
    // ss = +s on the |1> side, -s on the |0> side: c x + (-s) o == c x - s o
    static __device__ __forceinline__ T signed_s(const K4 &k, bool one) { return one ? k.c1 : -k.c1; }
    static __device__ __forceinline__ T sign(bool one) { return one ? (T)-1 : (T)1; }
    static __device__ __forceinline__ Amp ry_half(const K4 &k, Amp self, Amp o, T ss) {
        return Amp{xadd(xmul(k.c0, self.re), xmul(ss, o.re)), xadd(xmul(k.c0, self.im), xmul(ss, o.im))};
    }
    static __device__ __forceinline__ Amp cmul(Amp a, T c, T s) { return cmul_exact(a, c, s); }
    static __device__ __forceinline__ Amp pi_mul(Amp a, int) { return a; }  // float-float path only
};

// Fast: the same gates with fused multiply-adds (RX/RY 8 FP operations per
// pair instead of 12, a complex product 4 instead of 6) and one rounding
// fewer per step.  Used whenever bit-identity with the reference is not
// requested (the default planner also reorders commuting gates).
template <class T>
struct Fast : Exact<T> {
    using Amp = cx<T>;
    using K4 = typename Exact<T>::K4;
    // (the products are explicitly rounded: a plain product could be fused
    // with the next gate's sum once gates run as straight-line code)
    static __device__ __forceinline__ void h_pair(int, const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0{xmul(a0.re + a1.re, k.c0), xmul(a0.im + a1.im, k.c0)};
        const Amp n1{xmul(a0.re - a1.re, k.c0), xmul(a0.im - a1.im, k.c0)};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp h_half(int, const K4 &k, Amp self, Amp o, T sgn) {
        return Amp{xmul(fma(sgn, self.re, o.re), k.c0), xmul(fma(sgn, self.im, o.im), k.c0)};
    }
    static __device__ __forceinline__ void rx_pair(const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0{fma(k.c0, a0.re, k.c1 * a1.im), fma(k.c0, a0.im, -k.c1 * a1.re)};
        const Amp n1{fma(k.c0, a1.re, k.c1 * a0.im), fma(k.c0, a1.im, -k.c1 * a0.re)};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp rx_half(const K4 &k, Amp self, Amp o) {
        return Amp{fma(k.c0, self.re, k.c1 * o.im), fma(k.c0, self.im, -k.c1 * o.re)};
    }
    static __device__ __forceinline__ void ry_pair(const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0{fma(k.c0, a0.re, -k.c1 * a1.re), fma(k.c0, a0.im, -k.c1 * a1.im)};
        const Amp n1{fma(k.c0, a1.re, k.c1 * a0.re), fma(k.c0, a1.im, k.c1 * a0.im)};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp ry_half(const K4 &k, Amp self, Amp o, T ss) {
        return Amp{fma(k.c0, self.re, ss * o.re), fma(k.c0, self.im, ss * o.im)};
    }
    static __device__ __forceinline__ Amp cmul(Amp a, T c, T s) {
        return Amp{fma(a.re, c, -a.im * s), fma(a.re, s, a.im * c)};
    }
};

// Fast for complex64 on packed f32x2 instructions: an amplitude is one
// float2 (re, im) and every step advances both parts with one
// FADD2/FMUL2/FFMA2 (the real-coefficient rotations lane by lane as Fast;
// the complex product pairs (re, im) * c with (im, re) * (-s, s)).
struct FastP {
    using Amp = float2;
    using Mem = cx<float>;
    using Scalar = float;
    using K4 = Exact<float>::K4;
    static __device__ __forceinline__ Amp from_mem(Mem a) { return make_float2(a.re, a.im); }
    static __device__ __forceinline__ Mem to_mem(Amp a) { return Mem{a.x, a.y}; }
#if !defined(__CUDACC_RTC__)
    static void pack_host(TileGate &g) { Exact<float>::pack_host(g); }
#endif
    static __device__ __forceinline__ K4 load(const TileGate &g) { return Exact<float>::load(g); }
    static __device__ __forceinline__ Amp shfl(Amp v, int m) {
        return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
    }
    static __device__ __forceinline__ float2 bc(float x) { return make_float2(x, x); }
    static __device__ __forceinline__ float2 swp(float2 a) { return make_float2(a.y, a.x); }
    static __device__ __forceinline__ Amp neg(Amp a) { return ff2::neg(a); }
    static __device__ __forceinline__ void y_pair(Amp &a0, Amp &a1) {
        const Amp n0 = make_float2(a1.y, -a1.x), n1 = make_float2(-a0.y, a0.x);
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp y_half(Amp o, bool one) {
        return one ? make_float2(-o.y, o.x) : make_float2(o.y, -o.x);
    }
    // H is the one gate whose results are bare products.  A packed product
    // can be fused into the next gate's packed sum once gates run as
    // straight-line code (one rounding fewer), so it is rounded lane by lane
    // with the scalar multiply, which is never fused.
    static __device__ __forceinline__ float2 mul_rn(float2 a, float c) {
        return make_float2(__fmul_rn(a.x, c), __fmul_rn(a.y, c));
    }
    static __device__ __forceinline__ void h_pair(int, const K4 &k, Amp &a0, Amp &a1) {
        const Amp n0 = mul_rn(__fadd2_rn(a0, a1), k.c0);
        const Amp n1 = mul_rn(ff2::sub(a0, a1), k.c0);
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp h_half(int, const K4 &k, Amp self, Amp o, float sgn) {
        return mul_rn(__ffma2_rn(bc(sgn), self, o), k.c0);
    }
    static __device__ __forceinline__ void rx_pair(const K4 &k, Amp &a0, Amp &a1) {
        const float2 c = bc(k.c0), s = make_float2(k.c1, -k.c1);
        const Amp n0 = __ffma2_rn(c, a0, __fmul2_rn(s, swp(a1)));
        const Amp n1 = __ffma2_rn(c, a1, __fmul2_rn(s, swp(a0)));
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp rx_half(const K4 &k, Amp self, Amp o) {
        return __ffma2_rn(bc(k.c0), self, __fmul2_rn(make_float2(k.c1, -k.c1), swp(o)));
    }
    static __device__ __forceinline__ void ry_pair(const K4 &k, Amp &a0, Amp &a1) {
        const float2 c = bc(k.c0), s = bc(k.c1), ns = bc(-k.c1);
        const Amp n0 = __ffma2_rn(c, a0, __fmul2_rn(ns, a1));
        const Amp n1 = __ffma2_rn(c, a1, __fmul2_rn(s, a0));
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ float signed_s(const K4 &k, bool one) { return one ? k.c1 : -k.c1; }
    static __device__ __forceinline__ float sign(bool one) { return one ? -1.f : 1.f; }
    static __device__ __forceinline__ Amp ry_half(const K4 &k, Amp self, Amp o, float ss) {
        return __ffma2_rn(bc(k.c0), self, __fmul2_rn(bc(ss), o));
    }
    static __device__ __forceinline__ Amp cmul(Amp a, float c, float s) {
        return __ffma2_rn(a, bc(c), __fmul2_rn(swp(a), make_float2(-s, s)));
    }
    static __device__ __forceinline__ Amp pi_mul(Amp a, int) { return a; }  // float-float path only
};

// ---- float-float policy (complex128 fast path) ---------------------------------
// HBM keeps IEEE binary64; amplitudes become hi+lo float pairs on the way in
// and are rounded back on the way out.  Constants arrive pre-split by
// pack_host.  Classes used only here: H sub 1 (no 1/sqrt(2): the host folds
// it into a final scale gate), PI (|1> times i^q, free) and SCALE (every
// amplitude times one complex factor, the folded global factor).
struct FFPol {
    struct Amp {
        ff::f2 re, im;
    };
    using Mem = cx<double>;
    using Scalar = ff::f2;
    struct K4 {
        ff::f2 c0, c1, c2, c3;
    };
    static __device__ __forceinline__ Amp from_mem(Mem a) {
        return Amp{ff::from_double(a.re), ff::from_double(a.im)};
    }
    static __device__ __forceinline__ Mem to_mem(Amp a) { return Mem{ff::to_double(a.re), ff::to_double(a.im)}; }
#if !defined(__CUDACC_RTC__)
    static void pack_host(TileGate &g) {
        double c[4] = {g.c[0], g.c[1], g.c[2], g.c[3]};
        float f[8];
        for (int i = 0; i < 4; i++) {
            const ff::f2 v = ff::split_constant(c[i]);
            f[2 * i] = v.h;
            f[2 * i + 1] = v.l;
        }
        memcpy(g.c, f, sizeof f);
    }
#endif
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
    static __device__ __forceinline__ Amp neg(Amp a) { return Amp{ff::neg(a.re), ff::neg(a.im)}; }
    static __device__ __forceinline__ void y_pair(Amp &a0, Amp &a1) {
        const Amp n0{a1.im, ff::neg(a1.re)}, n1{ff::neg(a0.im), a0.re};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp y_half(Amp o, bool one) {
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
    // sgn = (+1, 0) or (-1, 0): o + sgn*self
    static __device__ __forceinline__ Amp h_half(int sub, const K4 &k, Amp self, Amp o, ff::f2 sgn) {
        const bool one = sgn.h < 0.f;
        Amp r = one ? Amp{ff::sub(o.re, self.re), ff::sub(o.im, self.im)}
                    : Amp{ff::add(self.re, o.re), ff::add(self.im, o.im)};
        if (sub == 0) r = Amp{ff::mul(r.re, k.c0), ff::mul(r.im, k.c0)};
        return r;
    }
    static __device__ __forceinline__ void rx_pair(const K4 &k, Amp &a0, Amp &a1) {
        const ff::f2 ns = ff::neg(k.c1);
        const Amp n0{ff::dot2(k.c0, a0.re, k.c1, a1.im), ff::dot2(k.c0, a0.im, ns, a1.re)};
        const Amp n1{ff::dot2(k.c0, a1.re, k.c1, a0.im), ff::dot2(k.c0, a1.im, ns, a0.re)};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp rx_half(const K4 &k, Amp self, Amp o) {
        return Amp{ff::dot2(k.c0, self.re, k.c1, o.im), ff::dot2(k.c0, self.im, ff::neg(k.c1), o.re)};
    }
    static __device__ __forceinline__ void ry_pair(const K4 &k, Amp &a0, Amp &a1) {
        const ff::f2 ns = ff::neg(k.c1);
        const Amp n0{ff::dot2(k.c0, a0.re, ns, a1.re), ff::dot2(k.c0, a0.im, ns, a1.im)};
        const Amp n1{ff::dot2(k.c0, a1.re, k.c1, a0.re), ff::dot2(k.c0, a1.im, k.c1, a0.im)};
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ ff::f2 signed_s(const K4 &k, bool one) { return one ? k.c1 : ff::neg(k.c1); }
    static __device__ __forceinline__ ff::f2 sign(bool one) { return one ? ff::f2{-1.f, 0.f} : ff::f2{1.f, 0.f}; }
    static __device__ __forceinline__ Amp ry_half(const K4 &k, Amp self, Amp o, ff::f2 ss) {
        return Amp{ff::dot2(k.c0, self.re, ss, o.re), ff::dot2(k.c0, self.im, ss, o.im)};
    }
    static __device__ __forceinline__ Amp cmul(Amp a, ff::f2 c, ff::f2 s) {
        return Amp{ff::dot2(c, a.re, ff::neg(s), a.im), ff::dot2(c, a.im, s, a.re)};
    }
    static __device__ __forceinline__ Amp pi_mul(Amp a, int q) {
        if (q == 1) return Amp{ff::neg(a.im), a.re};
        if (q == 2) return Amp{ff::neg(a.re), ff::neg(a.im)};
        return Amp{a.im, ff::neg(a.re)};
    }
};

// Packed float-float policy, state resident in float-float form in HBM:
// per amplitude h = (re.hi, im.hi), l = (re.lo, im.lo) (16 bytes, like
// binary64), loaded and stored unconverted.  The arithmetic is FFPol's, lane
// by lane, on f32x2 instructions: each FADD2/FMUL2/FFMA2 advances the real
// and the imaginary part together, halving the instruction count of the
// gate bodies (and their code size) at the same FP32 pipe time.
struct FF2 {
    using Amp = ff2::v2;
    using Mem = ff2::v2;
    using Scalar = ff::f2;
    using K4 = FFPol::K4;
    static __device__ __forceinline__ Amp from_mem(Mem a) { return a; }
    static __device__ __forceinline__ Mem to_mem(Amp a) { return a; }
#if !defined(__CUDACC_RTC__)
    static void pack_host(TileGate &g) { FFPol::pack_host(g); }
#endif
    static __device__ __forceinline__ K4 load(const TileGate &g) { return FFPol::load(g); }
    static __device__ __forceinline__ Amp shfl(Amp v, int m) {
        Amp r;
        r.h.x = __shfl_xor_sync(0xffffffffu, v.h.x, m);
        r.h.y = __shfl_xor_sync(0xffffffffu, v.h.y, m);
        r.l.x = __shfl_xor_sync(0xffffffffu, v.l.x, m);
        r.l.y = __shfl_xor_sync(0xffffffffu, v.l.y, m);
        return r;
    }
    static __device__ __forceinline__ Amp neg(Amp a) { return ff2::neg(a); }
    static __device__ __forceinline__ void y_pair(Amp &a0, Amp &a1) {
        const Amp n0 = ff2::mul_minus_i(a1), n1 = ff2::mul_i(a0);
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp y_half(Amp o, bool one) { return one ? ff2::mul_i(o) : ff2::mul_minus_i(o); }
    static __device__ __forceinline__ void h_pair(int sub, const K4 &k, Amp &a0, Amp &a1) {
        Amp n0 = ff2::add(a0, a1), n1 = ff2::sub(a0, a1);
        if (sub == 0) {
            const ff2::k2 c = ff2::konst(k.c0);
            n0 = ff2::mul(n0, c);
            n1 = ff2::mul(n1, c);
        }
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp h_half(int sub, const K4 &k, Amp self, Amp o, ff::f2 sgn) {
        const bool one = sgn.h < 0.f;
        Amp r = one ? ff2::sub(o, self) : ff2::add(self, o);
        if (sub == 0) r = ff2::mul(r, ff2::konst(k.c0));
        return r;
    }
    // RX: out0 = c a0 + s (a1.im, -a1.re), out1 = c a1 + s (a0.im, -a0.re)
    static __device__ __forceinline__ void rx_pair(const K4 &k, Amp &a0, Amp &a1) {
        const ff2::k2 c = ff2::konst(k.c0), s = ff2::konst(k.c1, ff::neg(k.c1));
        const Amp n0 = ff2::dot2(c, a0, s, ff2::swap(a1)), n1 = ff2::dot2(c, a1, s, ff2::swap(a0));
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ Amp rx_half(const K4 &k, Amp self, Amp o) {
        return ff2::dot2(ff2::konst(k.c0), self, ff2::konst(k.c1, ff::neg(k.c1)), ff2::swap(o));
    }
    // RY: out0 = c a0 - s a1, out1 = c a1 + s a0
    static __device__ __forceinline__ void ry_pair(const K4 &k, Amp &a0, Amp &a1) {
        const ff2::k2 c = ff2::konst(k.c0), s = ff2::konst(k.c1), ns = ff2::konst(ff::neg(k.c1));
        const Amp n0 = ff2::dot2(c, a0, ns, a1), n1 = ff2::dot2(c, a1, s, a0);
        a0 = n0;
        a1 = n1;
    }
    static __device__ __forceinline__ ff::f2 signed_s(const K4 &k, bool one) { return one ? k.c1 : ff::neg(k.c1); }
    static __device__ __forceinline__ ff::f2 sign(bool one) { return one ? ff::f2{-1.f, 0.f} : ff::f2{1.f, 0.f}; }
    static __device__ __forceinline__ Amp ry_half(const K4 &k, Amp self, Amp o, ff::f2 ss) {
        return ff2::dot2(ff2::konst(k.c0), self, ff2::konst(ss), o);
    }
    // a * (c + i s): (c re - s im, c im + s re) = c (re, im) + (-s, s) (im, re)
    static __device__ __forceinline__ Amp cmul(Amp a, ff::f2 c, ff::f2 s) {
        return ff2::dot2(ff2::konst(c), a, ff2::konst(ff::neg(s), s), ff2::swap(a));
    }
    static __device__ __forceinline__ Amp pi_mul(Amp a, int q) {
        if (q == 1) return ff2::mul_i(a);
        if (q == 2) return ff2::neg(a);
        return ff2::mul_minus_i(a);
    }
};

// FF2's packed arithmetic on binary64 storage (the adjoint keeps its two
// states and its checkpoints in binary64): amplitudes are split into
// float-float pairs on the way in and rounded back on the way out, as FFPol
// does, while the gate bodies run packed.
struct FF2B : FF2 {
    using Mem = cx<double>;
    static __device__ __forceinline__ Amp from_mem(Mem a) {
        const ff::f2 re = ff::from_double(a.re), im = ff::from_double(a.im);
        return Amp{make_float2(re.h, im.h), make_float2(re.l, im.l)};
    }
    static __device__ __forceinline__ Mem to_mem(Amp a) {
        return Mem{ff::to_double(ff::f2{a.h.x, a.l.x}), ff::to_double(ff::f2{a.h.y, a.l.y})};
    }
};

// ---- per-gate register code -------------------------------------------------------
// jm bit j: register j passes the gate's controls on register bits (from the
// planner), so a controlled gate costs one predicate per register.
#define KBWG_JM(j) (((jm >> (j)) & 1u) != 0u)

// Gate on register bit B: 2^(R-1) in-thread pairs (a control is never the
// target, so both halves of a pair share their control bits).
template <class P, int R, int B, int CLS>
__device__ __forceinline__ void reg_pairs(typename P::Amp (&v)[1 << R], const TileGate &g, uint32_t jm) {
    if constexpr (B < R) {
        const typename P::K4 k = P::load(g);
        const int sub = g.sub;
#pragma unroll
        for (int jj = 0; jj < (1 << (R - 1)); jj++) {
            const int j0 = ((jj >> B) << (B + 1)) | (jj & ((1 << B) - 1));
            const int j1 = j0 | (1 << B);
            if (KBWG_JM(j0)) {
                if constexpr (CLS == TG_X) {
                    const typename P::Amp t = v[j0];
                    v[j0] = v[j1];
                    v[j1] = t;
                }
                if constexpr (CLS == TG_Y) P::y_pair(v[j0], v[j1]);
                if constexpr (CLS == TG_H) P::h_pair(sub, k, v[j0], v[j1]);
                if constexpr (CLS == TG_RX) P::rx_pair(k, v[j0], v[j1]);
                if constexpr (CLS == TG_RY) P::ry_pair(k, v[j0], v[j1]);
            }
        }
    }
}

// Gate on lane bit tb: the partner is in lane ^ (1 << tb).  Every lane takes
// part in the shuffle; register j is updated when fok and (j & creg) == creg.
// (The predicate is formed at its use: the register mask jm, held as
// predicates across the shuffles, exhausts the predicate registers.)
template <class P, int R, int CLS>
__device__ __forceinline__ void lane_gate(typename P::Amp (&v)[1 << R], const TileGate &g, bool fok, uint32_t F) {
    constexpr int NR = 1 << R;
    const uint32_t creg = g.creg;
#define KBWG_LANE_ON(j) (fok && ((uint32_t)(j) & creg) == creg)
    const uint32_t tb = g.tb;
    const bool one = ((F >> tb) & 1u) != 0;
    const int m = 1 << tb;
    const typename P::K4 k = P::load(g);
    if constexpr (CLS == TG_X) {
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const typename P::Amp o = P::shfl(v[j], m);
            if (KBWG_LANE_ON(j)) v[j] = o;
        }
    } else if constexpr (CLS == TG_Y) {
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const typename P::Amp o = P::shfl(v[j], m);
            if (KBWG_LANE_ON(j)) v[j] = P::y_half(o, one);
        }
    } else if constexpr (CLS == TG_H) {
        const auto sg = P::sign(one);
        const int sub = g.sub;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const typename P::Amp o = P::shfl(v[j], m);
            if (KBWG_LANE_ON(j)) v[j] = P::h_half(sub, k, v[j], o, sg);
        }
    } else if constexpr (CLS == TG_RX) {
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const typename P::Amp o = P::shfl(v[j], m);
            if (KBWG_LANE_ON(j)) v[j] = P::rx_half(k, v[j], o);
        }
    } else {
        const auto ss = P::signed_s(k, one);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const typename P::Amp o = P::shfl(v[j], m);
            if (KBWG_LANE_ON(j)) v[j] = P::ry_half(k, v[j], o, ss);
        }
    }
#undef KBWG_LANE_ON
}

// Diagonal gate on register bit B: the side of every register is known at
// compile time.
template <class P, int R, int B, int CLS>
__device__ __forceinline__ void diag_reg(typename P::Amp (&v)[1 << R], const TileGate &g, uint32_t jm) {
    if constexpr (B < R) {
        constexpr int NR = 1 << R;
        const typename P::K4 k = P::load(g);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            if (!KBWG_JM(j)) continue;
            const bool hi = ((j >> B) & 1) != 0;
            if constexpr (CLS == TG_Z) {
                if (hi) v[j] = P::neg(v[j]);
            } else if constexpr (CLS == TG_P) {
                if (hi) v[j] = P::cmul(v[j], k.c0, k.c1);
            } else if constexpr (CLS == TG_RZ) {
                v[j] = hi ? P::cmul(v[j], k.c2, k.c3) : P::cmul(v[j], k.c0, k.c1);
            } else {  // TG_PI
                if (hi) v[j] = P::pi_mul(v[j], (int)reinterpret_cast<const float &>(k.c0));
            }
        }
    }
}

// Diagonal gate whose target bit is the same for all of this thread's
// registers (a lane/warp bit, or a qubit outside the tile): `one` is uniform.
template <class P, int R, int CLS>
__device__ __forceinline__ void diag_fixed(typename P::Amp (&v)[1 << R], const TileGate &g, uint32_t jm, bool one) {
    constexpr int NR = 1 << R;
    if constexpr (CLS != TG_SCALE && CLS != TG_RZ)
        if (!one) return;
    const typename P::K4 k = P::load(g);
    if constexpr (CLS == TG_Z) {
#pragma unroll
        for (int j = 0; j < NR; j++)
            if (KBWG_JM(j)) v[j] = P::neg(v[j]);
    } else if constexpr (CLS == TG_PI) {
        const int q = (int)reinterpret_cast<const float &>(k.c0);
#pragma unroll
        for (int j = 0; j < NR; j++)
            if (KBWG_JM(j)) v[j] = P::pi_mul(v[j], q);
    } else {
        // P: |1> * (c0, c1); SCALE: all * (c0, c1); RZ: (c0, c1) or (c2, c3)
        const auto c = (CLS == TG_RZ && one) ? k.c2 : k.c0;
        const auto s = (CLS == TG_RZ && one) ? k.c3 : k.c1;
#pragma unroll
        for (int j = 0; j < NR; j++)
            if (KBWG_JM(j)) v[j] = P::cmul(v[j], c, s);
    }
}

// Apply one gate to the thread's registers.  F = the thread's fixed local
// bits (lane and warp) in this stage's layout; base = the tile's global
// index of local 0.  A few header loads and one jump table per gate.
template <class T> struct ident { using type = T; };
template <bool W, class A, class C> struct pick_t { using type = A; };
template <class A, class C> struct pick_t<false, A, C> { using type = C; };

// B: type of the state index (32 bits up to 32 qubits, 64 bits above; not
// deduced from the argument, so a caller names 64 bits explicitly).
template <class P, int K, int R, class B = uint32_t>
__device__ __forceinline__ void tile_gate(const TileGate &g, typename P::Amp (&v)[1 << R], int /*R0*/, uint32_t F,
                                          typename ident<B>::type base) {
    static_assert(R >= 3 && R <= 4, "dispatch covers register bits 0..3");
    const uint32_t op = g.op;
    const uint32_t fneed = g.fneed;
    const uint32_t jm = g.jm;
    const B co = (B)g.co;
    if ((base & co) != co) return;  // a control outside the tile is 0 for the whole tile
    const bool fok = (F & fneed) == fneed;
    if (op < OP_REG) {  // lane targets: every lane shuffles, outside the jump table
        if (op == OP_LANE + TG_X) lane_gate<P, R, TG_X>(v, g, fok, F);
        else if (op == OP_LANE + TG_Y) lane_gate<P, R, TG_Y>(v, g, fok, F);
        else if (op == OP_LANE + TG_H) lane_gate<P, R, TG_H>(v, g, fok, F);
        else if (op == OP_LANE + TG_RX) lane_gate<P, R, TG_RX>(v, g, fok, F);
        else lane_gate<P, R, TG_RY>(v, g, fok, F);
        return;
    }
    if (!fok) return;
    switch (op) {
#define KBWG_REG(C)                                                    \
    case OP_REG + C * 4 + 0: reg_pairs<P, R, 0, C>(v, g, jm); break; \
    case OP_REG + C * 4 + 1: reg_pairs<P, R, 1, C>(v, g, jm); break; \
    case OP_REG + C * 4 + 2: reg_pairs<P, R, 2, C>(v, g, jm); break; \
    case OP_REG + C * 4 + 3: reg_pairs<P, R, 3, C>(v, g, jm); break;
#define KBWG_DREG(C)                                                               \
    case OP_DREG + (C - TG_Z) * 4 + 0: diag_reg<P, R, 0, C>(v, g, jm); break; \
    case OP_DREG + (C - TG_Z) * 4 + 1: diag_reg<P, R, 1, C>(v, g, jm); break; \
    case OP_DREG + (C - TG_Z) * 4 + 2: diag_reg<P, R, 2, C>(v, g, jm); break; \
    case OP_DREG + (C - TG_Z) * 4 + 3: diag_reg<P, R, 3, C>(v, g, jm); break;
#define KBWG_DFIX(C)                                                                                          \
    case OP_DFIX + (C - TG_Z): {                                                                           \
        const uint32_t tb = g.tb, tout = g.tout;                                    \
        const bool one = (C == TG_SCALE) || (tb == TG_OUTER ? ((base >> tout) & 1u) != 0 : ((F >> tb) & 1u) != 0); \
        diag_fixed<P, R, C>(v, g, jm, one);                                                                 \
        break;                                                                                              \
    }
        KBWG_REG(TG_X) KBWG_REG(TG_Y) KBWG_REG(TG_H) KBWG_REG(TG_RX) KBWG_REG(TG_RY)
        KBWG_DREG(TG_Z) KBWG_DREG(TG_P) KBWG_DREG(TG_RZ) KBWG_DREG(TG_PI)
        KBWG_DFIX(TG_Z) KBWG_DFIX(TG_P) KBWG_DFIX(TG_RZ) KBWG_DFIX(TG_PI) KBWG_DFIX(TG_SCALE)
#undef KBWG_REG
#undef KBWG_DREG
#undef KBWG_DFIX
    default: break;
    }
}

#undef KBWG_JM

}  // namespace kbwg
