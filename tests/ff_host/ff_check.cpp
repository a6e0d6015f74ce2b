// Host check of the float-float arithmetic of the complex128 fast path
// (kbw_gb300/csrc/ff.cuh, compiled here as plain C++ with contraction off),
// against long double on seeded random operands.  Prints the worst relative
// errors as "name value" lines; tests/test_ff_host.py holds the bounds.
//
//   from_double  hi + lo against the binary64 input (lo keeps 24 of the
//                remaining 29 significand bits: ~2^-48)
//   to_double    hi + lo rounded to binary64, compared with the exact sum
//                (mismatches are counted; the sum of a normalised pair fits
//                a double, so there should be none)
//   mul          a * k, relative to |a k|
//   dot2         c x + s y, relative to |c x| + |s y|
//   add          a + b, relative to |a| + |b|
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <random>

#include "../../kbw_gb300/csrc/ff.cuh"

using namespace kbwg::ff;

static long double val(f2 v) { return (long double)v.h + (long double)v.l; }

int main(int argc, char **argv) {
    const long count = argc > 1 ? atol(argv[1]) : 400000;
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    auto amp = [&]() {  // amplitudes of a unit state: magnitudes down to 2^-40
        return U(rng) * ldexp(1.0, -(int)(rng() % 40));
    };
    double e_from = 0, e_mul = 0, e_dot = 0, e_add = 0;
    long td_fail = 0;
    for (long i = 0; i < count; i++) {
        const double d = amp(), y = amp();
        const f2 vd = from_double(d), vy = from_double(y);
        e_from = fmax(e_from, (double)(fabsl(val(vd) - d) / fabs(d)));
        if (to_double(vd) != (double)val(vd)) td_fail++;
        const double c = U(rng), s = U(rng);
        const f2 kc = split_constant(c), ks = split_constant(s);
        // the constants as the engine holds them (hi + lo of the binary64 value)
        const long double lc = val(kc), ls = val(ks);
        const f2 m = mul(vd, kc);
        const long double xm = val(vd) * lc;
        if (xm != 0) e_mul = fmax(e_mul, (double)(fabsl(val(m) - xm) / fabsl(xm)));
        const f2 r = dot2(kc, vd, ks, vy);
        const long double xd = lc * val(vd) + ls * val(vy);
        const long double sc = fabsl(lc * val(vd)) + fabsl(ls * val(vy));
        if (sc != 0) e_dot = fmax(e_dot, (double)(fabsl(val(r) - xd) / sc));
        const f2 a = add(vd, vy);
        const long double xa = val(vd) + val(vy);
        const long double sa = fabsl(val(vd)) + fabsl(val(vy));
        if (sa != 0) e_add = fmax(e_add, (double)(fabsl(val(a) - xa) / sa));
    }
    printf("from_double %.6g\nto_double_mismatches %ld\nmul %.6g\ndot2 %.6g\nadd %.6g\n", e_from, td_fail, e_mul,
           e_dot, e_add);
    return 0;
}
