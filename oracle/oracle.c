/*
 * CPU oracle for the dense state-vector path -- TEST INFRASTRUCTURE ONLY.
 * See oracle.h for scope and parity status.  Build with floating-point
 * contraction off (-ffp-contract=off) so every product and sum rounds the
 * way the reference's Rust code does.
 */
#include "oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define F float
#define SUF(x) x##_f32
#define FCOS cosf
#define FSIN sinf
#define FHYPOT hypotf
#define FRAC_1_SQRT_2_F 0.70710678118654752440f
#define EPS_F 1e-6
#include "oracle_body.inc"
#undef F
#undef SUF
#undef FCOS
#undef FSIN
#undef FHYPOT
#undef FRAC_1_SQRT_2_F
#undef EPS_F

#define F double
#define SUF(x) x##_f64
#define FCOS cos
#define FSIN sin
#define FHYPOT hypot
#define FRAC_1_SQRT_2_F 0.70710678118654752440
#define EPS_F 1e-15
#include "oracle_body.inc"
#undef F
#undef SUF
#undef FCOS
#undef FSIN
#undef FHYPOT
#undef FRAC_1_SQRT_2_F
#undef EPS_F

/* Dense<F> fields (src/dense.rs:42-48): two buffers and a flag naming the
 * current one. */
struct od_state {
    int prec; /* 0: f32, 1: f64 */
    size_t n;
    size_t ns;
    void *s0, *s1;
    int state; /* 1 -> current is s0 (the reference's `state: true`) */
};

int od_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void od_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

static size_t elem_size(int prec) { return prec ? 2 * sizeof(double) : 2 * sizeof(float); }

static void *cur_buf(od_state *s) { return s->state ? s->s0 : s->s1; }

/* Dense::get_states (src/dense.rs:51-58): flip, then (current, next). */
static void flip_buffers(od_state *s, void **cur, void **nxt) {
    s->state = !s->state;
    if (s->state) {
        *cur = s->s1;
        *nxt = s->s0;
    } else {
        *cur = s->s0;
        *nxt = s->s1;
    }
}

od_state *od_new(size_t num_qubits, int prec) {
    if (num_qubits > 32) return NULL;
    od_state *s = (od_state *)calloc(1, sizeof(od_state));
    if (!s) return NULL;
    s->prec = prec ? 1 : 0;
    s->n = num_qubits;
    s->ns = (size_t)1 << num_qubits;
    s->s0 = malloc(s->ns * elem_size(s->prec));
    s->s1 = malloc(s->ns * elem_size(s->prec));
    if (!s->s0 || !s->s1) {
        od_free(s);
        return NULL;
    }
    od_clear(s);
    return s;
}

void od_free(od_state *s) {
    if (!s) return;
    free(s->s0);
    free(s->s1);
    free(s);
}

/* Dense::clear (src/dense.rs:399-406). */
void od_clear(od_state *s) {
    if (s->prec)
        clear_f64(s->s0, s->s1, s->ns);
    else
        clear_f32(s->s0, s->s1, s->ns);
    s->state = 1;
}

size_t od_num_qubits(const od_state *s) { return s->n; }

static size_t ctrl_mask(const size_t *control, size_t n_control) {
    size_t m = 0;
    for (size_t i = 0; i < n_control; i++) m |= (size_t)1 << control[i];
    return m;
}

int od_gate(od_state *s, int kind, double angle, size_t target, const size_t *control,
            size_t n_control) {
    if (target >= s->n) return -1;
    for (size_t i = 0; i < n_control; i++)
        if (control[i] >= s->n) return -1;
    const size_t mask = ctrl_mask(control, n_control);
    void *cur, *nxt;
    const int d = s->prec;
    switch (kind) {
    case OD_X:
        flip_buffers(s, &cur, &nxt);
        d ? pauli_x_f64(cur, nxt, s->ns, target, mask) : pauli_x_f32(cur, nxt, s->ns, target, mask);
        break;
    case OD_Y:
        flip_buffers(s, &cur, &nxt);
        d ? pauli_y_f64(cur, nxt, s->ns, target, mask) : pauli_y_f32(cur, nxt, s->ns, target, mask);
        break;
    case OD_Z:
        d ? pauli_z_f64(cur_buf(s), s->ns, target, mask)
          : pauli_z_f32(cur_buf(s), s->ns, target, mask);
        break;
    case OD_H:
        flip_buffers(s, &cur, &nxt);
        d ? hadamard_f64(cur, nxt, s->ns, target, mask)
          : hadamard_f32(cur, nxt, s->ns, target, mask);
        break;
    case OD_P:
        d ? phase_f64(cur_buf(s), s->ns, angle, target, mask)
          : phase_f32(cur_buf(s), s->ns, angle, target, mask);
        break;
    case OD_RX:
        flip_buffers(s, &cur, &nxt);
        d ? rx_f64(cur, nxt, s->ns, angle, target, mask)
          : rx_f32(cur, nxt, s->ns, angle, target, mask);
        break;
    case OD_RY:
        flip_buffers(s, &cur, &nxt);
        d ? ry_f64(cur, nxt, s->ns, angle, target, mask)
          : ry_f32(cur, nxt, s->ns, angle, target, mask);
        break;
    case OD_RZ:
        d ? rz_f64(cur_buf(s), s->ns, angle, target, mask)
          : rz_f32(cur_buf(s), s->ns, angle, target, mask);
        break;
    default:
        return -1;
    }
    return 0;
}

int od_apply_gates(od_state *s, const int *kinds, const size_t *targets, const uint64_t *masks,
                   const double *angles, size_t n_gates) {
    size_t ctrl[64];
    for (size_t i = 0; i < n_gates; i++) {
        size_t nc = 0;
        for (size_t q = 0; q < 64; q++)
            if ((masks[i] >> q) & 1u) ctrl[nc++] = q;
        if (od_gate(s, kinds[i], angles[i], targets[i], ctrl, nc) != 0) return -1;
    }
    return 0;
}

double od_measure_p1(od_state *s, size_t target) {
    return s->prec ? measure_p1_f64(cur_buf(s), s->ns, target)
                   : measure_p1_f32(cur_buf(s), s->ns, target);
}

void od_measure_collapse(od_state *s, size_t target, int result, double p) {
    void *cur, *nxt;
    flip_buffers(s, &cur, &nxt);
    if (s->prec)
        measure_collapse_f64(cur, nxt, s->ns, target, result, p);
    else
        measure_collapse_f32(cur, nxt, s->ns, target, result, p);
}

size_t od_dump(od_state *s, const size_t *qubits, size_t n_qubits, uint64_t *states, double *re,
               double *im) {
    return s->prec ? dump_f64(cur_buf(s), s->ns, qubits, n_qubits, states, re, im)
                   : dump_f32(cur_buf(s), s->ns, qubits, n_qubits, states, re, im);
}

void od_get_state(const od_state *s, double *out) {
    od_state *m = (od_state *)s;
    if (s->prec)
        get_state_f64(cur_buf(m), s->ns, out);
    else
        get_state_f32(cur_buf(m), s->ns, out);
}

void od_set_state(od_state *s, const double *in) {
    if (s->prec)
        set_state_f64(cur_buf(s), s->ns, in);
    else
        set_state_f32(cur_buf(s), s->ns, in);
}

void od_swap_qubits(od_state *s, size_t a, size_t b) {
    void *cur, *nxt;
    flip_buffers(s, &cur, &nxt);
    if (s->prec)
        swap_qubits_f64(cur, nxt, s->ns, a, b);
    else
        swap_qubits_f32(cur, nxt, s->ns, a, b);
}

/* ---- rand's WeightedIndex / UniformFloat, restated ------------------------
 * UniformFloat::new(low=0, high=total): scale = total, then while
 * scale * max_rand + low >= high, step scale down by one ulp, where
 * max_rand = 1 - 2^-52 is the largest value of the 52-bit [0,1) draw.
 * A sample is u * scale + low.  WeightedIndex keeps the running sums
 * w0, w0+w1, ... (all but the total) and picks the first one above the
 * sample (the partition point of "cum <= chosen"). */
double od_uniform_scale(double total) {
    const double max_rand = 1.0 - DBL_EPSILON;
    double scale = total;
    while (scale * max_rand + 0.0 >= total) {
        uint64_t bits;
        memcpy(&bits, &scale, sizeof bits);
        bits -= 1;
        memcpy(&scale, &bits, sizeof bits);
    }
    return scale;
}

size_t od_weighted_pick(const double *cumulative, size_t n_cumulative, double chosen) {
    size_t lo = 0, hi = n_cumulative;
    while (lo < hi) {
        const size_t mid = lo + (hi - lo) / 2;
        if (cumulative[mid] <= chosen)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* QubitManager::do_measure (src/quantum_execution.rs:272-292). */
uint64_t od_measure(od_state *s, const size_t *qubits, size_t n_qubits, const double *draws) {
    uint64_t out = 0;
    for (size_t index = 0; index < n_qubits; index++) {
        const size_t q = qubits[n_qubits - 1 - index];
        const double p1 = od_measure_p1(s, q);
        double p0 = 1.0 - p1;
        if (!(p0 > 0.0)) p0 = 0.0; /* f64::max(1-p1, 0) */
        const double total = p0 + p1;
        const double chosen = draws[index] * od_uniform_scale(total) + 0.0;
        const int result = (p0 <= chosen) ? 1 : 0;
        double prob = result ? p1 : p0;
        if (!(prob > DBL_MIN)) prob = DBL_MIN; /* prob.max(f64::MIN_POSITIVE) */
        const double p = 1.0 / sqrt(prob);
        od_measure_collapse(s, q, result, p);
        out |= (uint64_t)result << index;
    }
    return out;
}

static int cmp_u64(const void *a, const void *b) {
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* Default sample() (src/quantum_execution.rs:99-102) with
 * from_dump_to_prob / from_prob_to_shots (src/convert.rs:30-73). */
long od_sample(od_state *s, const size_t *qubits, size_t n_qubits, size_t shots,
               const double *draws, uint64_t *states, uint64_t *counts) {
    const size_t m = od_dump(s, qubits, n_qubits, NULL, NULL, NULL);
    if (m == 0) return -1;
    uint64_t *bs = (uint64_t *)malloc(m * sizeof(uint64_t));
    double *re = (double *)malloc(m * sizeof(double));
    double *im = (double *)malloc(m * sizeof(double));
    double *cum = (double *)malloc(m * sizeof(double));
    uint64_t *picked = (uint64_t *)malloc((shots ? shots : 1) * sizeof(uint64_t));
    if (!bs || !re || !im || !cum || !picked) {
        free(bs), free(re), free(im), free(cum), free(picked);
        return -1;
    }
    od_dump(s, qubits, n_qubits, bs, re, im);
    /* |a|^2 via Complex64::abs (= hypot) squared; running sums left to right. */
    double total = 0.0;
    for (size_t i = 0; i < m; i++) {
        const double a = hypot(re[i], im[i]);
        const double w = a * a;
        if (i == 0) {
            total = w;
        } else {
            cum[i - 1] = total;
            total += w;
        }
    }
    long result = -1;
    if (total > 0.0) {
        const double scale = od_uniform_scale(total);
        for (size_t k = 0; k < shots; k++) {
            const double chosen = draws[k] * scale + 0.0;
            picked[k] = bs[od_weighted_pick(cum, m - 1, chosen)];
        }
        qsort(picked, shots, sizeof(uint64_t), cmp_u64);
        long nout = 0;
        for (size_t k = 0; k < shots; k++) {
            if (nout > 0 && states[nout - 1] == picked[k]) {
                counts[nout - 1]++;
            } else {
                states[nout] = picked[k];
                counts[nout] = 1;
                nout++;
            }
        }
        result = nout;
    }
    free(bs), free(re), free(im), free(cum), free(picked);
    return result;
}

/* Default exp_value() (src/quantum_execution.rs:109-158). */
double od_exp_value(od_state *s, const int *paulis, const size_t *qubits, const size_t *offsets,
                    const double *coefficients, size_t n_strings) {
    const double half_pi = 1.57079632679489661923; /* FRAC_PI_2 */
    double total = 0.0;
    for (size_t k = 0; k < n_strings; k++) {
        const size_t b = offsets[k], e = offsets[k + 1];
        for (size_t i = b; i < e; i++) {
            if (paulis[i] == OD_PAULI_X) {
                od_gate(s, OD_H, 0.0, qubits[i], NULL, 0);
            } else if (paulis[i] == OD_PAULI_Y) {
                od_gate(s, OD_P, -half_pi, qubits[i], NULL, 0);
                od_gate(s, OD_H, 0.0, qubits[i], NULL, 0);
            }
        }
        const size_t m = od_dump(s, qubits + b, e - b, NULL, NULL, NULL);
        uint64_t *bs = (uint64_t *)malloc((m ? m : 1) * sizeof(uint64_t));
        double *re = (double *)malloc((m ? m : 1) * sizeof(double));
        double *im = (double *)malloc((m ? m : 1) * sizeof(double));
        od_dump(s, qubits + b, e - b, bs, re, im);
        double result = 0.0;
        for (size_t i = 0; i < m; i++) {
            const double a = hypot(re[i], im[i]);
            const double prob = a * a;
            const double parity = (__builtin_popcountll(bs[i]) % 2 == 0) ? 1.0 : -1.0;
            result += prob * parity;
        }
        free(bs), free(re), free(im);
        for (size_t i = b; i < e; i++) {
            if (paulis[i] == OD_PAULI_X) {
                od_gate(s, OD_H, 0.0, qubits[i], NULL, 0);
            } else if (paulis[i] == OD_PAULI_Y) {
                od_gate(s, OD_H, 0.0, qubits[i], NULL, 0);
                od_gate(s, OD_P, half_pi, qubits[i], NULL, 0);
            }
        }
        total += result * coefficients[k];
    }
    return total;
}

/* <H> = sum_k c_k <P_k> computed directly from the amplitudes (test
 * infrastructure for parity checks that need many energies): for
 * P = i^{ny} X^x Z^z, (P a)_s = i^{ny} (-1)^{|(s^x) & z|} a_{s^x}.  It
 * differs from od_exp_value (the reference's dump-based default) only by
 * keeping amplitudes the dump's epsilon filter drops. */
double od_pauli_expect(const od_state *s, const int *paulis, const size_t *qubits, const size_t *offsets,
                       const double *coefficients, size_t n_strings) {
    const size_t ns = s->ns;
    const void *cur = s->state ? s->s0 : s->s1;
    double total = 0.0;
    for (size_t k = 0; k < n_strings; k++) {
        uint64_t x = 0, z = 0;
        int ny = 0;
        for (size_t i = offsets[k]; i < offsets[k + 1]; i++) {
            const uint64_t b = 1ull << qubits[i];
            if (paulis[i] == OD_PAULI_X) x |= b;
            else if (paulis[i] == OD_PAULI_Y) x |= b, z |= b, ny++;
            else if (paulis[i] == OD_PAULI_Z) z |= b;
        }
        double sr = 0.0, si = 0.0;
#pragma omp parallel for reduction(+ : sr, si) schedule(static)
        for (size_t t = 0; t < ns; t++) {
            const size_t u = t ^ (size_t)x;
            double ar, ai, br, bi;
            if (s->prec) {
                const double *d = (const double *)cur;
                ar = d[2 * t], ai = d[2 * t + 1], br = d[2 * u], bi = d[2 * u + 1];
            } else {
                const float *f = (const float *)cur;
                ar = f[2 * t], ai = f[2 * t + 1], br = f[2 * u], bi = f[2 * u + 1];
            }
            const double sg = (__builtin_popcountll((uint64_t)u & z) & 1) ? -1.0 : 1.0;
            /* conj(a_t) * a_u */
            sr += sg * (ar * br + ai * bi);
            si += sg * (ar * bi - ai * br);
        }
        /* times i^ny */
        double re = sr, im = si;
        for (int q = 0; q < (ny & 3); q++) {
            const double t = re;
            re = -im;
            im = t;
        }
        total += coefficients[k] * re;
    }
    return total;
}

/* <Z_q> for every qubit q in one pass (out[q], n entries). */
void od_z_all(const od_state *s, double *out) {
    const size_t n = s->n, ns = s->ns;
    const void *cur = s->state ? s->s0 : s->s1;
    for (size_t q = 0; q < n; q++) out[q] = 0.0;
#pragma omp parallel
    {
        double acc[64] = {0};
#pragma omp for schedule(static)
        for (size_t t = 0; t < ns; t++) {
            double p;
            if (s->prec) {
                const double *d = (const double *)cur;
                p = d[2 * t] * d[2 * t] + d[2 * t + 1] * d[2 * t + 1];
            } else {
                const float *f = (const float *)cur;
                p = (double)f[2 * t] * f[2 * t] + (double)f[2 * t + 1] * f[2 * t + 1];
            }
            for (size_t q = 0; q < n; q++) acc[q] += ((t >> q) & 1) ? -p : p;
        }
#pragma omp critical
        for (size_t q = 0; q < n; q++) out[q] += acc[q];
    }
}
