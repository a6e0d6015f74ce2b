/*
 * CPU oracle for the dense state-vector path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference simulator `Dense<F>` (kbw
 * src/dense.rs:42-406) for F = f32 and F = f64, together with the trait
 * defaults the reference builds on top of it (src/quantum_execution.rs:99-158,
 * 272-292) and the dump/shot conversions (src/convert.rs:30-73).
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark may
 * load this library; the product path never calls it.
 *
 * Parity status: UNPINNED against the reference itself.  The reference ships
 * no tests, no golden vectors and cannot be built here (Rust toolchain and
 * crates absent).  The oracle is instead pinned against an independent numpy
 * matrix-product model (tests/golden/make_golden.py) and against closed-form
 * known answers (Grover, GHZ, rotation expectations).
 *
 * Random draws: the reference draws from rand's StdRng through
 * WeightedIndex.  That stream is not reproducible here, so every stochastic
 * entry point takes the uniform draws u in [0,1) explicitly and applies
 * WeightedIndex's documented selection rule to them (see od_weighted_pick).
 */
#ifndef KBW_ORACLE_H
#define KBW_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct od_state od_state;

/* Gate kinds, in the order of the QuantumExecution trait methods
 * (src/quantum_execution.rs:58-79). */
enum { OD_X = 0, OD_Y = 1, OD_Z = 2, OD_H = 3, OD_P = 4, OD_RX = 5, OD_RY = 6, OD_RZ = 7 };
/* Pauli codes for exp_value strings. */
enum { OD_PAULI_X = 1, OD_PAULI_Y = 2, OD_PAULI_Z = 3 };

/* prec: 0 -> Dense<f32>, 1 -> Dense<f64>.  NULL when n > 32
 * (src/dense.rs:71-73) or on allocation failure. */
od_state *od_new(size_t num_qubits, int prec);
void od_free(od_state *s);
void od_clear(od_state *s);
int od_num_threads(void);
void od_set_num_threads(int n);

/* One trait gate call; returns 0, or -1 for a bad qubit index. */
int od_gate(od_state *s, int kind, double angle, size_t target, const size_t *control,
            size_t n_control);

/* A gate list in one call (the loop of LiveExecution::compute_gate,
 * src/quantum_execution.rs:310-314): record i = kinds[i], targets[i],
 * control mask masks[i], angles[i].  Returns 0, or -1 at the first bad
 * qubit index (the gates before it stay applied). */
int od_apply_gates(od_state *s, const int *kinds, const size_t *targets, const uint64_t *masks,
                   const double *angles, size_t n_gates);

double od_measure_p1(od_state *s, size_t target);
void od_measure_collapse(od_state *s, size_t target, int result, double p);

/* dump: returns the support size; when states != NULL also fills
 * states/re/im (capacity must be >= the support size). */
size_t od_dump(od_state *s, const size_t *qubits, size_t n_qubits, uint64_t *states, double *re,
               double *im);

/* QubitManager::do_measure with one injected draw per qubit, consumed in
 * measurement order (last qubit of the list first). */
uint64_t od_measure(od_state *s, const size_t *qubits, size_t n_qubits, const double *draws);

/* Default sample(): dump -> |a|^2 -> WeightedIndex -> histogram.  Writes the
 * histogram sorted by basis state; returns its length, or -1 when every
 * weight is zero (the reference panics there, src/convert.rs:60). */
long od_sample(od_state *s, const size_t *qubits, size_t n_qubits, size_t shots,
               const double *draws, uint64_t *states, uint64_t *counts);

/* Default exp_value(): per string basis rotation, dump, parity sum, undo.
 * paulis/qubits are flattened; string k spans [offsets[k], offsets[k+1]). */
double od_exp_value(od_state *s, const int *paulis, const size_t *qubits, const size_t *offsets,
                    const double *coefficients, size_t n_strings);

/* <H> from the amplitudes directly (no basis rotations, no dump): for
 * parity checks that need many energies.  Same arguments as od_exp_value. */
double od_pauli_expect(const od_state *s, const int *paulis, const size_t *qubits, const size_t *offsets,
                       const double *coefficients, size_t n_strings);

/* <Z_q> of every qubit in one pass over the state (out: num_qubits entries). */
void od_z_all(const od_state *s, double *out);

/* Raw state access (interleaved re,im as double). */
void od_get_state(const od_state *s, double *out);
void od_set_state(od_state *s, const double *in);
size_t od_num_qubits(const od_state *s);

/* Block-swap restatement (DenseV2 BlockSimulator::swap, src/dense_v2.rs:360-396)
 * expressed on the flat index: exchanges physical qubits a and b. */
void od_swap_qubits(od_state *s, size_t a, size_t b);

/* WeightedIndex selection helpers (rand's UniformFloat::new scale rule and
 * the partition-point pick), exposed for tests. */
double od_uniform_scale(double total);
size_t od_weighted_pick(const double *cumulative, size_t n_cumulative, double chosen);

#ifdef __cplusplus
}
#endif
#endif
