// Packed float-float arithmetic: two float-float numbers per f32x2 register
// pair, one FADD2/FMUL2/FFMA2 instruction per step for both.  A complex
// amplitude is {h = (re.hi, im.hi), l = (re.lo, im.lo)}; the operation
// sequences are those of ff.cuh lane by lane (bit-identical results), with
// negations folded into the algebra: a product is formed negated, p' = -c*x,
// so that its exact error is fma(c, x, p') without a separate negation.
#pragma once

#include "ff.cuh"

namespace kbwg {
namespace ff2 {

struct __align__(16) v2 {
    float2 h, l;
};

// a per-lane float-float constant with its negated high part
struct k2 {
    float2 h, l, nh;
};

__device__ __forceinline__ float2 pk(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b in one packed instruction (the runtime headers offer no packed
// subtract; PTX sub.rn.f32x2 folds the negation into the FADD2)
union f2bits {
    float2 f;
    unsigned long long u;
};
__device__ __forceinline__ float2 sub(float2 a, float2 b) {
    f2bits x, y, d;
    x.f = a;
    y.f = b;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d.u) : "l"(x.u), "l"(y.u));
    return d.f;
}
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ __forceinline__ k2 konst(ff::f2 x, ff::f2 y) {  // lane 0 = x, lane 1 = y
    return k2{pk(x.h, y.h), pk(x.l, y.l), pk(-x.h, -y.h)};
}
__device__ __forceinline__ k2 konst(ff::f2 x) { return konst(x, x); }

// Knuth TwoSum / Dekker FastTwoSum, lane by lane
__device__ __forceinline__ v2 two_sum(float2 a, float2 b) {
    const float2 s = add(a, b);
    const float2 bb = sub(s, a);
    return v2{s, add(sub(a, sub(s, bb)), sub(b, bb))};
}
__device__ __forceinline__ v2 fast_two_sum(float2 a, float2 b) {
    const float2 s = add(a, b);
    return v2{s, sub(b, sub(s, a))};
}

__device__ __forceinline__ v2 add(v2 a, v2 b) {
    const v2 s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, add(s.l, add(a.l, b.l)));
}
// TwoSum(a, -b) without forming -b
__device__ __forceinline__ v2 two_diff(float2 a, float2 b) {
    const float2 s = sub(a, b);
    const float2 bb = sub(s, a);
    return v2{s, sub(sub(a, sub(s, bb)), add(b, bb))};
}
__device__ __forceinline__ v2 sub(v2 a, v2 b) {
    const v2 s = two_diff(a.h, b.h);
    return fast_two_sum(s.h, add(s.l, sub(a.l, b.l)));
}

// a * k (lo * lo dropped), as ff::mul per lane
__device__ __forceinline__ v2 mul(v2 a, const k2 &k) {
    const float2 np = mul(a.h, k.nh);  // -p
    float2 e = fma(a.h, k.h, np);      // exact error of p
    e = fma(a.h, k.l, e);
    e = fma(a.l, k.h, e);
    // fast_two_sum(p, e) with p = -np
    const float2 s = sub(e, np);
    return v2{s, sub(e, add(s, np))};
}

// c*x + s*y per lane, as ff::dot2 per lane
__device__ __forceinline__ v2 dot2(const k2 &c, v2 x, const k2 &s, v2 y) {
    const float2 np1 = mul(x.h, c.nh);
    float2 e1 = fma(x.h, c.h, np1);
    e1 = fma(x.l, c.h, e1);
    e1 = fma(x.h, c.l, e1);
    const float2 np2 = mul(y.h, s.nh);
    float2 e2 = fma(y.h, s.h, np2);
    e2 = fma(y.l, s.h, e2);
    e2 = fma(y.h, s.l, e2);
    // TwoSum of the negated products: t = -(p1 + p2) rounded, te its error
    const float2 t = add(np1, np2);
    const float2 bb = sub(t, np1);
    const float2 te = add(sub(np1, sub(t, bb)), sub(np2, bb));
    const float2 lo = sub(add(e1, e2), te);
    // FastTwoSum(-t, lo)
    const float2 r = sub(lo, t);
    return v2{r, sub(lo, add(r, t))};
}

// lane swap (re <-> im)
__device__ __forceinline__ v2 swap(v2 a) { return v2{pk(a.h.y, a.h.x), pk(a.l.y, a.l.x)}; }
// exact negation on the FMA pipe (keeps the sign of zero, like -x)
__device__ __forceinline__ float2 neg(float2 a) { return mul(a, make_float2(-1.f, -1.f)); }
__device__ __forceinline__ v2 neg(v2 a) { return v2{neg(a.h), neg(a.l)}; }
// (re, im) -> (im, -re) = -i * a   and   (-im, re) = i * a
__device__ __forceinline__ v2 mul_minus_i(v2 a) { return v2{pk(a.h.y, -a.h.x), pk(a.l.y, -a.l.x)}; }
__device__ __forceinline__ v2 mul_i(v2 a) { return v2{pk(-a.h.y, a.h.x), pk(-a.l.y, a.l.x)}; }

}  // namespace ff2
}  // namespace kbwg
