// Launchers of the engine's CUDA kernels (host-callable, template on the
// amplitude real type T = float for complex64, double for complex128).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace kbwg {

// Device scratch layout used by reductions (allocated once per handle).
struct ReduceScratch {
    double *partials;   // [kMaxBlocks * kMaxTerms]
    unsigned *ticket;   // last-block counter (returns to 0 after each use)
    double *result;     // [kMaxTerms]
};
constexpr int kReduceBlocks = 152 * 4;  // fixed grid: deterministic partition
constexpr int kReduceThreads = 256;
constexpr int kMaxTerms = 32;

// Sequential-measurement control block, updated on the device by the last
// block of each reduction step (kbw src/quantum_execution.rs:272-292).
struct MeasureCtl {
    uint64_t M, V;        // measured-qubit mask and outcome bits so far
    uint64_t result;      // packed result (bit k = k-th measured qubit)
    double scale2;        // product of F(p_k)^2 over collapses so far
    double p[64];         // collapse factors p_k = 1/sqrt(max(prob, MIN_POSITIVE))
    double draws[64];     // uniform draws, one per qubit, in measurement order
    uint32_t qubit[64];   // qubit measured at step k
    uint32_t steps;
    uint32_t pad;
};

template <class T> cudaError_t launch_gate1(void *st, uint32_t n, const GateDesc &g, cudaStream_t s);
template <class T> cudaError_t launch_init(void *st, uint32_t n, cudaStream_t s);
// complex128 storage: binary64 -> float-float pairs (to_ff) or back, in place.
cudaError_t launch_ff_convert(void *st, uint32_t n, bool to_ff, cudaStream_t s);
// |0...0> in the float-float resident form.
cudaError_t launch_init_ff(void *st, uint32_t n, cudaStream_t s);
// One CTA runs the tile kernels' bounded wait on a barrier nothing completes.
cudaError_t launch_wait_probe(int *err, uint32_t spins, cudaStream_t s);
template <class T> cudaError_t launch_swap(void *st, uint32_t n, uint32_t a, uint32_t b, cudaStream_t s);

// Sum of |a_s|^2 over s with (s & M) == V, FP64 result in scratch.result[0].
template <class T>
cudaError_t launch_masked_norm(const void *st, uint32_t n, uint64_t M, uint64_t V, const ReduceScratch &rs,
                               cudaStream_t s);

// sum |a - b|^2 into scratch.result[0] and sum |b|^2 into result[1].
template <class T>
cudaError_t launch_distance(const void *a, const void *b, uint32_t n, const ReduceScratch &rs, cudaStream_t s);
// Re<a|b>, Im<a|b>, <a|a>, <b|b> into rs.result[0..3]; prec_*: 0 complex64, 1 complex128.
cudaError_t launch_overlap(const void *a, int prec_a, const void *b, int prec_b, uint32_t n, const ReduceScratch &rs,
                           cudaStream_t s);

// One step of the sequential measurement: conditional p1 of ctl->qubit[step]
// given the outcomes so far, then the WeightedIndex decision, all on device.
template <class T>
cudaError_t launch_measure_step(const void *st, uint32_t n, MeasureCtl *ctl, uint32_t step,
                                const ReduceScratch &rs, cudaStream_t s);

// Keep amplitudes with (s & M) == V multiplied by F(p[0])*F(p[1])*... in
// sequence, zero the others.  M, V, p come from ctl when ctl != nullptr,
// otherwise from the explicit arguments.
template <class T>
cudaError_t launch_collapse(void *st, uint32_t n, const MeasureCtl *ctl, uint64_t M, uint64_t V, double p,
                            cudaStream_t s);

// Pauli-string group with common flip mask x: per term k, <psi|P_k|psi>
// (without coefficient) into scratch.result[k].
struct PauliGroup {
    uint64_t x;                 // flip mask (X or Y positions)
    uint32_t nterms;
    uint32_t pad;
    uint64_t z[kMaxTerms];      // phase mask (Z or Y positions)
    double factor[kMaxTerms];   // +-1 (x == 0) or +-2 (pair form)
    uint32_t use_im[kMaxTerms]; // pair form: Im(conj(a_s) a_{s^x}) instead of Re
};
// ff_resident: the state is in the float-float resident form (complex128,
// diagonal groups only).
// Float-float resident complex128 state (sweeps leave it so): the masked
// norm, one measurement step and the collapse read and write that form.
cudaError_t launch_masked_norm_ff(const void *st, uint32_t n, uint64_t M, uint64_t V, const ReduceScratch &rs,
                                  cudaStream_t s);
cudaError_t launch_measure_step_ff(const void *st, uint32_t n, MeasureCtl *ctl, uint32_t step,
                                   const ReduceScratch &rs, cudaStream_t s);
cudaError_t launch_collapse_ff(void *st, uint32_t n, const MeasureCtl *ctl, uint64_t M, uint64_t V, double p,
                               cudaStream_t s);
template <class T>
cudaError_t launch_pauli_group(const void *st, uint32_t n, const PauliGroup &g, const ReduceScratch &rs,
                               cudaStream_t s, bool ff_resident = false);

// Pair-form Pauli strings with different flip masks in one pass: a tile of
// 2^K amplitudes (local bits 0..l-1 = qubits 0..l-1, l..K-1 = qubits hq[])
// holds both members of every pair of every string whose flip mask lies in
// the tile.  Per term: <psi|P_k|psi> without coefficient into result[k].
struct PauliTileTerm {
    uint32_t xl;    // flip mask on local bits
    uint32_t zl;    // phase mask on local bits
    uint64_t zo;    // phase mask on qubits outside the tile
    uint32_t hb;    // highest local bit of xl: each pair is visited with it clear
    uint32_t im;    // Im(conj(a_s) a_{s^x}) instead of Re
    double factor;  // +-2 (i^{nY} and (-1)^{|x & z|} folded in)
};
struct PauliTilePass {
    uint32_t K, l, m, nterms;
    uint8_t hq[16];
    PauliTileTerm t[kMaxTerms];
};
// Tile size of the pass kernel (32 KiB of shared memory: several CTAs per SM
// overlap one tile's loads with another's arithmetic).
template <class T> constexpr int pauli_tile_bits() { return sizeof(T) == 4 ? 12 : 11; }
template <class T>
cudaError_t launch_pauli_tile(const void *st, uint32_t n, bool ff_resident, const PauliTilePass &p,
                              const ReduceScratch &rs, cudaStream_t s);

// dump: support counts per block, then compaction.
struct DumpSpec {
    uint32_t nq;
    uint8_t qubits[64];
};
int dump_blocks(uint32_t n);
template <class T>
cudaError_t launch_dump_count(const void *st, uint32_t n, uint64_t *counts, cudaStream_t s);
template <class T>
cudaError_t launch_dump_write(const void *st, uint32_t n, const uint64_t *offsets, const DumpSpec &spec,
                              uint64_t *states, double *re, double *im, cudaStream_t s);

// sampling: per-block weight sums, then per-block picks for sorted draws.
int sample_blocks(uint32_t n);
template <class T>
cudaError_t launch_weight_blocksum(const void *st, uint32_t n, double *blocksum, cudaStream_t s);
// For every block b with shots: shots [shot_begin[b], shot_begin[b+1]) of the
// sorted chosen[] array; prefix[b] = weight before the block.  Writes the
// picked amplitude index per shot into pick[].
template <class T>
cudaError_t launch_sample_pick(const void *st, uint32_t n, const uint32_t *blocks, uint32_t nblocks_with_shots,
                               const uint64_t *shot_begin, const double *prefix, const double *chosen,
                               uint64_t *pick, cudaStream_t s);

}  // namespace kbwg
