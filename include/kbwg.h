/*
 * kbwg.h -- C ABI of the GB300 dense state-vector engine ("densegb300").
 *
 * The engine is a drop-in backend for the Ket Bitwise Simulator's dense path.
 * Each entry point below replaces one method of the reference's backend trait
 * `QuantumExecution` (kbw src/quantum_execution.rs:48-162) or one piece of the
 * `QubitManager` adapter built on it (src/quantum_execution.rs:171-427); the
 * citation is given per entry.  A Rust `QuantumExecution` impl binds these
 * symbols one to one, exactly as the reference's
 * `kbw_make_configuration` (kbw.h:48-54, src/c_api.rs:60-129) binds its own
 * backends.
 *
 * Conventions
 *  - Every function returns an int32 status: KBWG_OK (0) or a KBWG_E* code.
 *    No C++ exception or CUDA error crosses this boundary; the text of the
 *    last error on the calling thread is available from kbwg_last_error().
 *  - Qubit indices and counts are uintptr_t (the reference's usize).  Bit q
 *    of a basis-state index is qubit q, as in the reference (src/bitwise.rs).
 *  - Angles and probabilities are double, as in the trait.
 *  - A handle owns one state vector on one GPU (the device current when it
 *    was created) and one CUDA stream.  Use a handle from one host thread at
 *    a time (the trait's `&mut self`).  Gate calls are queued on the host and
 *    executed by fused kernels at the next call that reads the state.
 *  - Host buffers are plain pointers; nothing here takes torch types.
 */
#ifndef KBWG_H_INCLUDED
#define KBWG_H_INCLUDED

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct kbwg_sim kbwg_sim;

/* status codes (KetError analogues; 0 = Success) */
enum {
    KBWG_OK = 0,
    KBWG_EINVAL = 1,    /* bad argument: qubit index, null pointer, size */
    KBWG_EQUBITS = 2,   /* num_qubits out of range (above 40): KetError::ExecutionFailed as in src/dense.rs:71-73 */
    KBWG_ENOMEM = 3,    /* device or pinned-host allocation failed */
    KBWG_ECUDA = 4,     /* a CUDA runtime call failed */
    KBWG_EWEIGHT = 5,   /* all sampling weights are zero (src/convert.rs:60 panics) */
    KBWG_ECAPACITY = 6, /* caller buffer too small; *size holds the size needed */
    KBWG_ETIMEOUT = 7,  /* a bounded device-side wait ran out */
    KBWG_EUNSUPPORTED = 8
};

/* amplitude precision: complex64 (Dense<f32>, the reference default alias,
 * src/lib.rs:130) or complex128 (Dense<f64>) */
enum { KBWG_C64 = 0, KBWG_C128 = 1 };

/* gate kinds, in trait order (src/quantum_execution.rs:58-79) */
enum {
    KBWG_X = 0, KBWG_Y = 1, KBWG_Z = 2, KBWG_H = 3,
    KBWG_P = 4, KBWG_RX = 5, KBWG_RY = 6, KBWG_RZ = 7
};

/* Pauli codes of ket Hamiltonian terms (ket::ir::hamiltonian::Pauli) */
enum { KBWG_PAULI_X = 1, KBWG_PAULI_Y = 2, KBWG_PAULI_Z = 3 };

/* creation flags */
enum {
    KBWG_FLAG_NO_FUSION = 1u << 0, /* run one kernel per gate (debug / A-B timing) */
    KBWG_FLAG_FAST_C128 = 1u << 1, /* complex128 gates in float-float arithmetic (pairs of floats,
                                      ~48-bit significand, < 1e-12 relative to binary64) */
    KBWG_FLAG_EXACT_ORDER = 1u << 2, /* fuse without reordering commuting gates: amplitudes then
                                        equal the reference's bit for bit */
    KBWG_FLAG_NO_GRAPHS = 1u << 3,   /* do not replay repeated gate structures from CUDA graphs */
    KBWG_FLAG_NO_FOLD = 1u << 4      /* do not fold runs of diagonal one-qubit gates on a qubit into one
                                        (per-gate cost measurements) */
};

/* QuantumExecution::new (src/quantum_execution.rs:53; src/dense.rs:70-89).
 * Allocates 2^num_qubits amplitudes in |0...0>.  Dense::new stops at 32
 * qubits; DenseGPU and the Block backends have no cap (src/c_api.rs:93-109),
 * and neither has this engine below 40 (KBWG_EQUBITS above): the device's
 * memory decides (KBWG_ENOMEM), one GB300 holding 34 qubits in complex128 or
 * 35 in complex64 (256 GiB).  Above 32 qubits gates run in the default tile geometry
 * with 64-bit state indices; the adjoint gradient too, as far as memory holds
 * its state, lambda and checkpoints (33 qubits in complex64 on one GB300). */
int32_t kbwg_new(uintptr_t num_qubits, int32_t precision, uint32_t flags, kbwg_sim **out);

/* Drop of the backend (ket frees its QPUConfig, src/c_api.rs:124). */
int32_t kbwg_free(kbwg_sim *sim);

/* QuantumExecution::pauli_x/pauli_y/pauli_z/hadamard
 * (src/quantum_execution.rs:58-67; src/dense.rs:91-209). */
int32_t kbwg_pauli_x(kbwg_sim *sim, uintptr_t target, const uintptr_t *control, uintptr_t n_control);
int32_t kbwg_pauli_y(kbwg_sim *sim, uintptr_t target, const uintptr_t *control, uintptr_t n_control);
int32_t kbwg_pauli_z(kbwg_sim *sim, uintptr_t target, const uintptr_t *control, uintptr_t n_control);
int32_t kbwg_hadamard(kbwg_sim *sim, uintptr_t target, const uintptr_t *control, uintptr_t n_control);

/* QuantumExecution::phase/rx/ry/rz (src/quantum_execution.rs:70-79;
 * src/dense.rs:211-334). */
int32_t kbwg_phase(kbwg_sim *sim, double lambda, uintptr_t target, const uintptr_t *control,
                   uintptr_t n_control);
int32_t kbwg_rx(kbwg_sim *sim, double theta, uintptr_t target, const uintptr_t *control,
                uintptr_t n_control);
int32_t kbwg_ry(kbwg_sim *sim, double theta, uintptr_t target, const uintptr_t *control,
                uintptr_t n_control);
int32_t kbwg_rz(kbwg_sim *sim, double theta, uintptr_t target, const uintptr_t *control,
                uintptr_t n_control);

/* One gate record for kbwg_apply_gates: controls as a bit mask. */
typedef struct kbwg_gate {
    uint32_t kind;   /* KBWG_X .. KBWG_RZ */
    uint32_t target; /* qubit index */
    uint64_t control_mask;
    double angle;    /* ignored for X, Y, Z, H */
} kbwg_gate;

/* A gate list in one call: LiveExecution::compute_gate per element
 * (src/quantum_execution.rs:310-314, 251-270). */
int32_t kbwg_apply_gates(kbwg_sim *sim, const kbwg_gate *gates, uintptr_t n_gates);

/* QuantumExecution::measure_p1 (src/quantum_execution.rs:84; src/dense.rs:336-352).
 * FP64 on-device reduction; does not collapse. */
int32_t kbwg_measure_p1(kbwg_sim *sim, uintptr_t target, double *p1);

/* QuantumExecution::measure_collapse (src/quantum_execution.rs:90;
 * src/dense.rs:354-367): keep amplitudes whose bit `target` equals `result`,
 * scaled by p (= 1/sqrt(P(result))), zero the rest. */
int32_t kbwg_measure_collapse(kbwg_sim *sim, uintptr_t target, bool result, double p);

/* QubitManager::do_measure (src/quantum_execution.rs:272-292): measure the
 * listed qubits one at a time, last listed first, with one uniform draw in
 * [0,1) per qubit taken from `draws` in that order (the reference draws
 * these from its StdRng: pass the UniformFloat<f64> value WeightedIndex
 * takes from one next_u64, (x >> 12 | 0x3FF0000000000000) as a double
 * minus 1, not rand's 53-bit StandardUniform).  draws == NULL uses the
 * handle's own generator (kbwg_draws)
 * (seeded from KBW_SEED).  *result packs qubits[0] as the most significant
 * bit. */
int32_t kbwg_measure(kbwg_sim *sim, const uintptr_t *qubits, uintptr_t n_qubits,
                     const double *draws, uint64_t *result);

/* QuantumExecution::dump (src/quantum_execution.rs:93; src/dense.rs:369-397):
 * basis states with |a| > eps (1e-6 for c64, 1e-15 for c128), in index
 * order, re-packed with qubits[0] as the most significant bit.  Two-call
 * protocol: with capacity smaller than the support, fills nothing, sets
 * *size and returns KBWG_ECAPACITY (pass capacity 0 to query). */
int32_t kbwg_dump(kbwg_sim *sim, const uintptr_t *qubits, uintptr_t n_qubits,
                  uint64_t *basis_states, double *re, double *im, uintptr_t capacity,
                  uintptr_t *size);

/* QuantumExecution::sample default (src/quantum_execution.rs:99-102) with
 * src/convert.rs:30-73: `shots` draws u_k in [0,1) (NULL: the handle's
 * generator) pick basis states by WeightedIndex over the support.  Writes
 * the histogram sorted by packed basis state; *n_out = number of distinct
 * states.  capacity must be >= min(shots, 2^n_qubits). */
int32_t kbwg_sample(kbwg_sim *sim, const uintptr_t *qubits, uintptr_t n_qubits, uintptr_t shots,
                    const double *draws, uint64_t *states, uint64_t *counts, uintptr_t capacity,
                    uintptr_t *n_out);

/* QuantumExecution::exp_value (src/quantum_execution.rs:104-158): sum over
 * Pauli strings of coefficient * <psi|P|psi>, computed directly on the GPU
 * (no basis rotations, FP64 accumulation).  String k has terms
 * [offsets[k], offsets[k+1]) of paulis[] / qubits[]. */
int32_t kbwg_exp_value(kbwg_sim *sim, const uint8_t *paulis, const uintptr_t *qubits,
                       const uintptr_t *offsets, const double *coefficients, uintptr_t n_strings,
                       double *out);

/* Gradient of E = <psi|H|psi>, psi = gates|0...0>, by the reverse-mode
 * adjoint method: forward, lambda = H psi, then one backward walk that
 * uncomputes both states with inverse gates and accumulates
 * dE/dtheta = Im<lambda|Pi_C P|phi> per RX/RY/RZ (P = X/Y/Z of the target,
 * Pi_C the control projector) and -2 Im<lambda|Pi_C Pi_1|phi> per phase gate.
 * Replaces the parameter-shift rule libket runs when the backend reports no
 * native gradient (BatchExecution::gradient, src/quantum_execution.rs:420-426;
 * GradientStrategy::ParameterShiftRule, :237-241).
 * param_index[i] in [0, n_params) marks gate i (P/RX/RY/RZ only) as depending
 * on parameter param_index[i] (shared parameters add up); -1 = constant.  The
 * Hamiltonian is given as in kbwg_exp_value.  Up to max_checkpoints copies of
 * the forward state (as memory allows) bound the uncompute drift.  Writes E
 * and gradient[n_params]; the handle is left in |0...0>.  Needs >= 12 qubits
 * (complex64) or >= 11 (complex128).  The call's scratch (lambda and the
 * checkpoints) stays with the handle for the next call while it takes at most
 * a sixteenth of the device's memory, and is freed by kbwg_free. */
int32_t kbwg_adjoint_gradient(kbwg_sim *sim, const kbwg_gate *gates, uintptr_t n_gates,
                              const int32_t *param_index, uintptr_t n_params, const uint8_t *paulis,
                              const uintptr_t *qubits, const uintptr_t *offsets, const double *coefficients,
                              uintptr_t n_strings, uint32_t max_checkpoints, double *energy, double *gradient);

/* The same gradient by the parameter-shift rule on the GPU, the strategy
 * libket applies to KBW (GradientStrategy::ParameterShiftRule,
 * src/quantum_execution.rs:237-241): two fresh circuit evaluations
 * (BatchExecution::exp_value, :392-405) per parameterised gate, at
 * theta +- pi/2.  The handle is left in the last evaluated state. */
int32_t kbwg_param_shift_gradient(kbwg_sim *sim, const kbwg_gate *gates, uintptr_t n_gates,
                                  const int32_t *param_index, uintptr_t n_params, const uint8_t *paulis,
                                  const uintptr_t *qubits, const uintptr_t *offsets, const double *coefficients,
                                  uintptr_t n_strings, double *energy, double *gradient);

/* Many small variational circuits in one persistent launch.  Replaces the
 * reference's one-fresh-simulator-per-request batch path
 * (BatchExecution::exp_value, src/quantum_execution.rs:392-418) for the
 * hardware-efficient ansatz: circuit c has num_qubits[c] (2..21) qubits and
 * layers[c] layers of RY(theta) then RZ(phi) on every qubit followed by CZ on
 * the ring (i, i+1 mod n); its 2 n L angles start at params[param_offset[c]]
 * (per layer: the n RY angles, then the n RZ angles).  Writes
 * <H> = zz sum <Z_i Z_i+1> + x sum <X_i> (ring) into energies[c].
 * precision: KBWG_C64 or KBWG_C128 (flags: KBWG_FLAG_FAST_C128).  Runs on the
 * current device, allocates its buffers per call. */
int32_t kbwg_batch_hea_tfim(uintptr_t n_circuits, const uint32_t *num_qubits, const uint32_t *layers,
                            const uint64_t *param_offset, const double *params, uintptr_t n_params, double zz,
                            double x, int32_t precision, uint32_t flags, double *energies);

/* ---- whole-circuit batch entries --------------------------------------- */
/* BatchExecution (src/quantum_execution.rs:367-427) hands the backend a whole
 * circuit per call and gets a fresh simulator each time.  These entries do
 * the same without a handle: a register of num_qubits qubits in |0...0>
 * (precision and flags as for kbwg_new), the whole gate list (gates, as for
 * kbwg_apply_gates) planned and run as one flush, then the read-out.  The
 * register comes from a per-process pool (up to 4 registers, keyed by
 * device, size, precision and flags) and is reset for every call, its draw
 * generator re-seeded from KBW_SEED as QubitManager::new seeds a fresh one
 * (:183-191); so repeated calls skip the state allocation and replay
 * repeated circuit structures from CUDA graphs.  Pooled registers keep
 * their device memory until kbwg_batch_release.  Safe to call from several
 * host threads: a register serves one call at a time. */

/* BatchExecution::exp_value / exp_value_native (:392-418): one <H_k> per
 * Hamiltonian; Hamiltonian k is the strings [ham_offsets[k],
 * ham_offsets[k+1]) of the string arrays, which are laid out as for
 * kbwg_exp_value (offsets[] indexes paulis[] / qubits[] absolutely). */
int32_t kbwg_batch_exp_value(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                             uintptr_t n_gates, const uint8_t *paulis, const uintptr_t *qubits,
                             const uintptr_t *offsets, const double *coefficients, const uintptr_t *ham_offsets,
                             uintptr_t n_hamiltonians, double *out);

/* BatchExecution::sample / sample_native (:367-390): `shots` samples of the
 * listed qubits (at least one, as do_sample asserts), arguments and output as
 * for kbwg_sample. */
int32_t kbwg_batch_sample(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                          uintptr_t n_gates, const uintptr_t *qubits, uintptr_t n_qubits, uintptr_t shots,
                          const double *draws, uint64_t *states, uint64_t *counts, uintptr_t capacity,
                          uintptr_t *n_out);

/* BatchExecution::gradient (:420-426): the reference answers
 * NativeGateUnsupported and libket falls back to the parameter-shift rule;
 * this computes E and dE/dparams natively with the adjoint method
 * (arguments as for kbwg_adjoint_gradient). */
int32_t kbwg_batch_gradient(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                            uintptr_t n_gates, const int32_t *param_index, uintptr_t n_params,
                            const uint8_t *paulis, const uintptr_t *qubits, const uintptr_t *offsets,
                            const double *coefficients, uintptr_t n_strings, uint32_t max_checkpoints,
                            double *energy, double *gradient);

/* Free the pooled registers no call is using. */
int32_t kbwg_batch_release(void);

/* Many BatchExecution::exp_value requests (src/quantum_execution.rs:392-405,
 * each of which the reference runs on a fresh simulator) in one persistent
 * launch: circuit c has num_qubits[c] qubits (1..24), the gates
 * gates[gate_offsets[c] .. gate_offsets[c+1]) (as for kbwg_apply_gates) and
 * the Hamiltonian made of the strings [ham_offsets[c], ham_offsets[c+1]) of
 * the flattened string arrays (string k: paulis/qubits
 * [term_offsets[k], term_offsets[k+1]) with coefficient coefficients[k], as
 * for kbwg_exp_value); energies[c] = <H_c> after the circuit from |0...0>.
 * gate_offsets and ham_offsets have n_circuits + 1 entries.  precision:
 * KBWG_C64, or KBWG_C128 (flags: KBWG_FLAG_FAST_C128 for float-float gate
 * arithmetic).  Every circuit is planned into tile sweeps on the host;
 * persistent CTAs take the circuits largest first, a register of at most 12
 * (complex64) / 11 (complex128) qubits held on the SM, larger ones in a
 * per-CTA global slot.  <H> accumulates FP64-grade. */
int32_t kbwg_batch_circuits_exp_value(uintptr_t n_circuits, int32_t precision, uint32_t flags,
                                      const uint32_t *num_qubits, const kbwg_gate *gates,
                                      const uintptr_t *gate_offsets, const uint8_t *paulis, const uintptr_t *qubits,
                                      const uintptr_t *term_offsets, const double *coefficients,
                                      const uintptr_t *ham_offsets, double *energies);

/* QuantumExecution::clear (src/quantum_execution.rs:161; src/dense.rs:399-406). */
int32_t kbwg_clear(kbwg_sim *sim);

/* Execute queued gates now and wait for the device. */
int32_t kbwg_flush(kbwg_sim *sim);

/* Raw amplitude access (interleaved re,im in the handle's precision). */
int32_t kbwg_get_state(kbwg_sim *sim, void *host_dst, uintptr_t bytes);
int32_t kbwg_set_state(kbwg_sim *sim, const void *host_src, uintptr_t bytes);
int32_t kbwg_state_info(kbwg_sim *sim, uintptr_t *num_qubits, int32_t *precision,
                        void **device_ptr, uintptr_t *bytes);

/* BlockSimulator::swap (src/block.rs:41-53; src/dense_v2.rs:360-396;
 * GPU in_place_swap src/dense_gpu/kernel.rs:437-466), flat-index form:
 * exchange physical qubits a and b with one in-place permutation pass. */
int32_t kbwg_swap_qubits(kbwg_sim *sim, uintptr_t a, uintptr_t b);

/* kbw_build_info (kbw.h:64; src/c_api.rs:149-163). */
int32_t kbwg_build_info(const uint8_t **msg, uintptr_t *size);

/* ---- diagnostics (no counterpart in the reference) ---------------------- */

/* Run the fusion planner on the host for a gate list (no GPU needed) and
 * report how the engine would execute it: order[] receives the gate indices
 * in execution order, sweep_end[k] the end (exclusive) in order[] of sweep k,
 * tile_mask[k] the qubits of sweep k's tile.  The arrays need n_gates
 * entries.  With precision KBWG_C64 tiles have 13 qubits, with KBWG_C128 12
 * (11 with KBWG_FLAG_FAST_C128); num_qubits must be at least that.  flags:
 * KBWG_FLAG_EXACT_ORDER, KBWG_FLAG_FAST_C128 or 0. */
int32_t kbwg_plan(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                  uintptr_t n_gates, uint32_t *order, uint32_t *sweep_end, uint64_t *tile_mask,
                  uintptr_t *n_sweeps);

/* kbwg_plan for a given tile size (0: the default of a handle with these
 * arguments; else one of the compiled sizes, KBWG_EINVAL otherwise) and
 * fusion depth (0: 256): how a handle tuned to them would execute the gates. */
int32_t kbwg_plan_tuned(uintptr_t num_qubits, int32_t precision, uint32_t flags, uint32_t tile_qubits,
                        uint32_t fusion_depth, const kbwg_gate *gates, uintptr_t n_gates, uint32_t *order,
                        uint32_t *sweep_end, uint64_t *tile_mask, uintptr_t *n_sweeps);

/* The draws a register takes when the caller passes none: rand's StdRng
 * (ChaCha12) seeded with StdRng::seed_from_u64(seed), as the reference's
 * QubitManager seeds it from KBW_SEED (src/quantum_execution.rs:181-191);
 * each draw is the UniformFloat<f64> sample WeightedIndex consumes, the 52
 * high bits of one next_u64 as a double in [1, 2) minus 1
 * (src/convert.rs:60-64).  Writes the first `count` draws of a fresh
 * generator.  (The crates are not available here: the stream is restated
 * from their published algorithms, its ChaCha core checked against
 * RFC 7539.) */
int32_t kbwg_draws(uint64_t seed, uintptr_t count, double *out);

/* One ChaCha block (diagnostic of the generator above): 8 key words, 64-bit
 * block counter (state words 12-13), 64-bit stream (words 14-15), an even
 * number of rounds (12 for StdRng, 20 for RFC 7539); 16 output words. */
int32_t kbwg_chacha_block(const uint32_t *key, uint64_t counter, uint64_t stream, uint32_t rounds, uint32_t *out);

/* Make `device` current for this library on the calling thread; kbwg_new
 * places new handles on the current device (0 unless selected). */
int32_t kbwg_select_device(int32_t device);

/* The CUDA stream (cudaStream_t) every kernel of this handle runs on. */
int32_t kbwg_stream(kbwg_sim *sim, void **stream);

/* Per-launch timing of the gate kernels (fused sweeps and single-gate
 * passes) with CUDA events on the handle's stream.  enable != 0 starts a new
 * measurement; kbwg_profile_read waits for the stream and returns the launch
 * count, the summed device time and the summed algorithmic bytes
 * (2 x amplitude bytes x 2^n per full pass). */
int32_t kbwg_profile(kbwg_sim *sim, int32_t enable);
int32_t kbwg_profile_read(kbwg_sim *sim, uint64_t *launches, double *total_ms, double *bytes);

/* Bytes this library copied host->device and device->host (all handles). */
int32_t kbwg_transfer_bytes(uint64_t *h2d, uint64_t *d2h);

/* ||a - b|| / ||b|| over two handles of equal size and precision (FP64
 * reduction on a's device; both handles must live on the same device). */
int32_t kbwg_state_distance(kbwg_sim *a, kbwg_sim *b, double *relative);

/* State fidelity |<a|b>|^2 / (<a|a> <b|b>) of two handles of equal size on
 * the same device, of either precision (FP64 on-device reduction): the error
 * statement of a complex64 run against a complex128 run of the same circuit
 * (infidelity = 1 - fidelity). */
int32_t kbwg_state_fidelity(kbwg_sim *a, kbwg_sim *b, double *fidelity);

/* Passes (kernel sweeps or single-gate kernels) used by the last flush. */
int32_t kbwg_last_flush_stats(kbwg_sim *sim, uint64_t *gates, uint64_t *passes);

/* Failure-path check without a GPU fault: queued gates are flushed, then one
 * CTA runs the bounded wait every tile kernel uses for its TMA copies, on a
 * barrier that nothing completes, for `spins` polls (1..2^22).  The polls run
 * out, the kernel sets the handle's error flag and returns, and the call
 * reports it as any tile kernel's timeout is reported: KBWG_ETIMEOUT.  The
 * state is untouched and the handle stays usable. */
int32_t kbwg_wait_probe(kbwg_sim *sim, uint32_t spins);

/* ---- sweep tuning (no counterpart in the reference) ---------------------- */

/* Gate calls run as fused sweeps (one pass over the state applies many
 * gates).  Two settings shape them: the tile size (2^tile_qubits amplitudes
 * staged per tile; each arithmetic has a few compiled sizes) and the fusion
 * depth (the most gates one sweep applies, 1..256).  The environment
 * variables KBWG_TILE_QUBITS and KBWG_FUSION_DEPTH set them for every handle
 * kbwg_new creates (kbwg_new fails with KBWG_EINVAL on a value no kernel
 * exists for); a tile size larger than a handle's qubit count falls back to
 * the default on that handle.  The default tile is the arithmetic's
 * (complex64 13, complex128 12, float-float 11 qubits), or for a smaller
 * register the largest compiled size that fits it.  They apply wherever gates are applied to a
 * handle's state (gate calls, the forward pass of kbwg_adjoint_gradient, the
 * circuit runs of kbwg_param_shift_gradient), not to the adjoint's reverse
 * sweeps or to the batch and reduction kernels. */
enum {
    KBWG_TUNE_DEFAULT = 0, /* built-in defaults */
    KBWG_TUNE_SET = 1,     /* kbwg_set_tuning */
    KBWG_TUNE_ENV = 2,     /* KBWG_TILE_QUBITS / KBWG_FUSION_DEPTH */
    KBWG_TUNE_TIMED = 3,   /* kbwg_autotune timed the candidates */
    KBWG_TUNE_CACHED = 4   /* kbwg_autotune reused this process's earlier result */
};
typedef struct kbwg_tuning {
    uint32_t tile_qubits;      /* tile size the next flush uses; 0 = one kernel per gate */
    uint32_t fusion_depth;     /* most gates one sweep applies */
    uint32_t source;           /* KBWG_TUNE_* */
    uint32_t candidates;       /* (tile size, depth) pairs the last kbwg_autotune timed */
    double ms_per_run;         /* device time of one run of the tuned circuit, chosen settings */
    double default_ms_per_run; /* the same with the default settings */
} kbwg_tuning;

/* Tile sizes with a compiled sweep kernel for this handle's arithmetic and
 * qubit count, the default first (none when the handle runs one kernel per
 * gate).  capacity >= 4 always suffices. */
int32_t kbwg_tile_options(kbwg_sim *sim, uint32_t *tile_qubits, uintptr_t capacity, uintptr_t *n);

/* Set the tile size (0 = default, else one of kbwg_tile_options) and the
 * fusion depth (0 = default 256, else 1..256); KBWG_EINVAL otherwise.
 * Applies from the next flush; queued gates stay queued. */
int32_t kbwg_set_tuning(kbwg_sim *sim, uint32_t tile_qubits, uint32_t fusion_depth);
int32_t kbwg_get_tuning(kbwg_sim *sim, kbwg_tuning *out);

/* Autotuner: runs the circuit (gates, as for kbwg_apply_gates) under every
 * compiled tile size x fusion depths {256, 64, 16}, each 2 + reps times
 * (reps 0 = 1), times the last reps with CUDA events on the handle's
 * stream, and sets the fastest pair on the handle.  Queued gates are flushed
 * first; the state is copied aside and put back afterwards, so the handle's
 * state is unchanged (this needs device memory for one more state:
 * KBWG_ENOMEM otherwise, settings unchanged).  Results are cached for the
 * process by device, qubit count, arithmetic and circuit structure (kinds,
 * targets, controls; not angles): a later call with the same structure
 * times nothing.  With KBWG_TILE_QUBITS or KBWG_FUSION_DEPTH in the
 * environment the override stands and nothing is timed.  out may be NULL. */
int32_t kbwg_autotune(kbwg_sim *sim, const kbwg_gate *gates, uintptr_t n_gates, uint32_t reps,
                      kbwg_tuning *out);

/* ---- run-time specialised sweeps (no counterpart in the reference) ------- */

/* A fused sweep normally runs one compiled kernel that interprets the
 * sweep's gate program per tile.  A specialised kernel instead has the
 * sweep's gates as straight-line code, every structural property (gate
 * class, target, controls) fixed at compile time and only the angles read at
 * run time; it is written from the plan and compiled for sm_103a with NVRTC
 * (opened at run time) the first time a structure needs it, and cached for
 * the process.  Modes:
 *   KBWG_JIT_OFF    interpreted kernels only;
 *   KBWG_JIT_AUTO   (default) a gate structure flushed before on a handle
 *                   gets specialised kernels, compiled in the background,
 *                   when the state has at least KBWG_JIT_MIN_QUBITS (default
 *                   20) qubits;
 *   KBWG_JIT_ALWAYS every fused flush, any size, compiling synchronously.
 * The environment variable KBWG_JIT (0, 1, 2) sets the mode of new handles.
 * Where NVRTC is missing or a compilation fails, the sweep runs the
 * interpreted kernel and kbwg_jit_info reports the failure. */
enum { KBWG_JIT_OFF = 0, KBWG_JIT_AUTO = 1, KBWG_JIT_ALWAYS = 2 };
int32_t kbwg_set_jit(kbwg_sim *sim, int32_t mode);

/* In auto mode the specialised kernels of a structure are compiled in the
 * background from its second flush on, while flushes keep running the
 * interpreted kernels (the same amplitudes); the first flush after the
 * compilation has finished takes them in.  kbwg_jit_wait blocks until the
 * handle's pending compilations have finished, so that the next flush of
 * each of those structures runs specialised (e.g. before a timed region). */
int32_t kbwg_jit_wait(kbwg_sim *sim);

/* Stop background compilation for the rest of the process and wait for the
 * compilations in progress (each finishes; none starts).  Call it before the
 * process exits if flushes may have started compilations: a compilation
 * still running while the process tears down its libraries can crash the
 * exit.  (The Python binding registers it to run at interpreter exit.)
 * Later flushes run the kernels already compiled and the interpreted ones. */
int32_t kbwg_jit_shutdown(void);

typedef struct kbwg_jit_stats {
    int32_t mode;                /* the handle's KBWG_JIT_* mode */
    int32_t available;           /* 1 if NVRTC could be opened */
    uint64_t last_specialised;   /* sweeps of the handle's last flush that ran a specialised kernel */
    uint64_t compiled;           /* kernels compiled in this process */
    uint64_t reused;             /* requests served from the process's cache */
    uint64_t failed;             /* failed compilations or loads */
    double compile_seconds;      /* wall time spent compiling */
} kbwg_jit_stats;
/* sim may be NULL (then mode and last_specialised are 0).  The text of the
 * last compilation failure is in kbwg_jit_last_error(). */
int32_t kbwg_jit_info(kbwg_sim *sim, kbwg_jit_stats *out);
const char *kbwg_jit_last_error(void);

/* Host-only check (no GPU needed): plan `gates` as a flush on a handle with
 * these arguments and settings would (tile_qubits / fusion_depth as for
 * kbwg_plan_tuned) and compile the specialised kernel of every sweep with
 * NVRTC, without loading it.  *n_sweeps: the sweeps; *n_failed: the failed
 * compilations (text in kbwg_jit_last_error).  KBWG_EUNSUPPORTED when NVRTC
 * is missing. */
int32_t kbwg_jit_check(uintptr_t num_qubits, int32_t precision, uint32_t flags, uint32_t tile_qubits,
                       uint32_t fusion_depth, const kbwg_gate *gates, uintptr_t n_gates, uintptr_t *n_sweeps,
                       uintptr_t *n_failed);

/* The same for the specialised reverse sweeps of kbwg_adjoint_gradient on
 * `gates` (one segment, every P/RX/RY/RZ gate differentiated). */
int32_t kbwg_jit_check_adjoint(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                               uintptr_t n_gates, uintptr_t *n_sweeps, uintptr_t *n_failed);

/* ---- allocation-free entry (no counterpart in the reference) ------------- */

/* For callers that cannot allocate device memory: code recorded into a CUDA
 * graph (cudaMalloc cannot be captured), plugins whose host runtime owns all
 * device allocations, real-time loops that cannot absorb an allocation's
 * implicit synchronisation.  Writes to *out (device memory, one double) the
 * sum of |a_s|^2 over the basis states s with (s & mask) == value -- with
 * mask = value = 1 << t that is kbwg_measure_p1(t) -- for the caller's state
 * (device pointer, 2^num_qubits interleaved amplitudes in `precision`),
 * launched on `stream` (NULL: the legacy default stream) without waiting.
 * It calls no cudaMalloc/cudaFree and no allocating library routine: its
 * scratch is a fixed 8 KiB device array in this library (608 partial sums
 * and a ticket), held by every GPU that loads the library until exit.
 * Limits: num_qubits <= 32 (KBWG_EQUBITS otherwise); value must lie inside
 * mask, and state and out must be device (or managed) memory of the current
 * device (KBWG_EINVAL otherwise).  The first call in a CUDA context (per
 * device, and again after a cudaDeviceReset) looks up the array's device
 * address with that device current (kbwg_select_device), so make it before
 * any stream capture.  All calls share the array: calls that overlap on the
 * GPU (other streams, other threads) race; serialise them. */
int32_t kbwg_masked_norm_noalloc(const void *state, uintptr_t num_qubits, int32_t precision,
                                 uint64_t mask, uint64_t value, double *out, void *stream);

/* Text of the last error on this thread ("" if none). */
const char *kbwg_last_error(void);

/* Number of kernels this library has launched in this process (all handles). */
uint64_t kbwg_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
