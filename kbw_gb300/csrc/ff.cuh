// Float-float ("double-float") arithmetic for the complex128 fast path.
//
// GB300 issues FP32 at ~62x its FP64 rate (1.2 vs 74 TFLOP/s measured), so
// binary64 gate arithmetic is FP64-bound by an order of magnitude.  In the
// fast path every real number is an unevaluated sum hi + lo of two floats
// (|lo| <= ulp(hi)/2, a 48-bit significand, relative rounding ~2^-47 per
// operation), built only from FP32 adds, multiplies and FMAs with the
// classic error-free transformations:
//   TwoSum (Knuth):   s = a + b,  e = (a - (s - bb)) + (b - bb),  bb = s - a
//   FastTwoSum (Dekker, |a| >= |b|): s = a + b, e = b - (s - a)
//   TwoProd (FMA):    p = a * b,  e = fma(a, b, -p)
// Conversions between binary64 and float-float use integer bit operations
// plus one I2F / F2I, never an FP64 instruction.
//
// Functions are __host__ __device__ so the arithmetic can be checked on the
// CPU against long double; on the device the *_rn intrinsics keep the
// compiler from contracting or reassociating any step.
#pragma once

#include <stdint.h>
#if !defined(__CUDACC_RTC__)
#include <string.h>
#endif

#if defined(__CUDACC__)
#define FFI __host__ __device__ __forceinline__
#else
#define FFI inline
#include <math.h>
#endif

namespace kbwg {
namespace ff {

struct f2 {
    float h, l;
};

#if defined(__CUDA_ARCH__)
FFI float add(float a, float b) { return __fadd_rn(a, b); }
FFI float sub(float a, float b) { return __fsub_rn(a, b); }
FFI float mul(float a, float b) { return __fmul_rn(a, b); }
FFI float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
FFI uint32_t fbits(float x) { return (uint32_t)__float_as_uint(x); }
FFI float bitsf(uint32_t u) { return __uint_as_float(u); }
FFI uint64_t dbits(double x) { return (uint64_t)__double_as_longlong(x); }
FFI double bitsd(uint64_t u) { return __longlong_as_double((long long)u); }
FFI float u2f(uint32_t r) { return __uint2float_rn(r); }
FFI int f2i(float q) { return __float2int_rn(q); }
#else
FFI float add(float a, float b) { return a + b; }
FFI float sub(float a, float b) { return a - b; }
FFI float mul(float a, float b) { return a * b; }
FFI float fma_(float a, float b, float c) { return fmaf(a, b, c); }
FFI uint32_t fbits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
}
FFI float bitsf(uint32_t u) {
    float x;
    memcpy(&x, &u, 4);
    return x;
}
FFI uint64_t dbits(double x) {
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
}
FFI double bitsd(uint64_t u) {
    double x;
    memcpy(&x, &u, 8);
    return x;
}
FFI float u2f(uint32_t r) { return (float)r; }
FFI int f2i(float q) { return (int)lrintf(q); }
#endif

// Exact; as an operand it folds into the consuming instruction's negate modifier.
FFI float neg(float a) { return -a; }
FFI f2 neg(f2 a) { return f2{neg(a.h), neg(a.l)}; }

FFI f2 two_sum(float a, float b) {
    const float s = add(a, b);
    const float bb = sub(s, a);
    const float e = add(sub(a, sub(s, bb)), sub(b, bb));
    return f2{s, e};
}
FFI f2 fast_two_sum(float a, float b) {
    const float s = add(a, b);
    return f2{s, sub(b, sub(s, a))};
}

FFI f2 add(f2 a, f2 b) {
    const f2 s = two_sum(a.h, b.h);
    return fast_two_sum(s.h, add(s.l, add(a.l, b.l)));
}
FFI f2 sub(f2 a, f2 b) { return add(a, neg(b)); }

// a * k for a constant k (both float-float); the lo*lo term (~2^-48) is dropped.
FFI f2 mul(f2 a, f2 k) {
    const float p = mul(a.h, k.h);
    float e = fma_(a.h, k.h, neg(p));
    e = fma_(a.h, k.l, e);
    e = fma_(a.l, k.h, e);
    return fast_two_sum(p, e);
}

// c*x + s*y in one rounding chain.
FFI f2 dot2(f2 c, f2 x, f2 s, f2 y) {
    const float p1 = mul(c.h, x.h);
    float e1 = fma_(c.h, x.h, neg(p1));
    e1 = fma_(c.h, x.l, e1);
    e1 = fma_(c.l, x.h, e1);
    const float p2 = mul(s.h, y.h);
    float e2 = fma_(s.h, y.h, neg(p2));
    e2 = fma_(s.h, y.l, e2);
    e2 = fma_(s.l, y.h, e2);
    const f2 t = two_sum(p1, p2);
    return fast_two_sum(t.h, add(t.l, add(e1, e2)));
}

// Split a binary64 value: hi = its top 24 significand bits (truncated), lo =
// the remaining 29 bits rounded to 24.  Values below 2^-126 become 0, and lo
// is dropped below 2^-74 (both far under the 1e-12 relative bar for a unit
// state vector).
FFI f2 from_double(double d) {
    const uint64_t b = dbits(d);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t e = (uint32_t)(b >> 52) & 0x7FFu;
    const uint64_t man = b & 0xFFFFFFFFFFFFFull;
    if (e < 897u || e > 1150u) return f2{0.f, 0.f};
    const float hi = bitsf(sign | ((e - 896u) << 23) | (uint32_t)(man >> 29));
    const uint32_t r = (uint32_t)(man & 0x1FFFFFFFull);
    float lo = 0.f;
    if (r != 0u && e >= 949u) {
        lo = mul(u2f(r), bitsf((e - 948u) << 23));  // r * 2^(e-1075), exact scaling
        lo = bitsf(fbits(lo) | sign);
    }
    return f2{hi, lo};
}

// hi + lo rounded to binary64 (|lo| <= ulp(hi)/2 expected).  The low part is
// scaled to units of the double's last place, rounded to an integer and added
// to hi's bit pattern (monotonic within a binade).  The one case that leaves
// the binade (hi a power of two, lo of the other sign) falls back to FP64.
FFI double to_double(f2 v) {
    const uint32_t hb = fbits(v.h);
    const uint32_t ef = (hb >> 23) & 0xFFu;
    if (ef == 0u) return 0.0;
    uint64_t db = ((uint64_t)(hb & 0x80000000u) << 32) | ((uint64_t)(ef + 896u) << 52) |
                  ((uint64_t)(hb & 0x7FFFFFu) << 29);
    if (v.l == 0.f || ef < 52u) return bitsd(db);
    const float q = mul(v.l, bitsf((306u - ef) << 23));  // lo / ulp64(hi), exact scaling
    const int qi = f2i(q);
    const bool same = ((hb ^ fbits(v.l)) & 0x80000000u) == 0u;
    if (!same && (hb & 0x7FFFFFu) == 0u) return (double)v.h + (double)v.l;
    const int64_t mag = same ? (int64_t)(qi < 0 ? -qi : qi) : -(int64_t)(qi < 0 ? -qi : qi);
    db = (uint64_t)((int64_t)db + mag);
    return bitsd(db);
}

// Split a binary64 constant on the host (round-to-nearest hi).
FFI f2 split_constant(double c) {
    const float h = (float)c;
    return f2{h, (float)(c - (double)h)};
}

}  // namespace ff
}  // namespace kbwg
