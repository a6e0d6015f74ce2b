// Host side of the engine: one handle = one state vector on one GPU.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/kbwg.h"
#include "common.cuh"
#include "kernels.h"
#include "stdrng.h"

namespace kbwg {

// Grow-only device buffer owned by a handle.
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes);
    void release();
};

// CUDA-event timing of gate-kernel launches on the handle's stream.
struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    double bytes = 0.0;
    cudaError_t mark(cudaStream_t s) {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) return r;
            pool.push_back(e);
        }
        return cudaEventRecord(pool[used++], s);
    }
    void release() {
        for (cudaEvent_t e : pool) cudaEventDestroy(e);
        pool.clear();
        used = 0;
    }
};

// Largest register: Dense/DenseV2 stop at 32 qubits (src/dense.rs:71-73),
// DenseGPU and the Block backends have no cap (src/c_api.rs:93-109); here the
// tile kernels index tiles with 32 bits (2^(n - K) tiles) and the device's
// memory decides below that (one GB300: 34 qubits complex128 or 35 complex64).
constexpr uintptr_t kMaxQubits = 40;

struct Sim {
    uint32_t n = 0;
    int prec = 0;  // 0: complex64, 1: complex128
    uint32_t flags = 0;
    int device = 0;
    uint64_t ns = 0;
    size_t elem = 0;
    void *state = nullptr;
    cudaStream_t stream = nullptr;
    // complex128 fast path: the buffer holds float-float pairs (hi, lo of the
    // real part, then of the imaginary part) instead of binary64 while true
    bool ff_resident = false;

    std::vector<GateDesc> queue;  // gates waiting for the next flush

    void *scratch = nullptr;  // reductions + measurement control
    ReduceScratch rs{};
    MeasureCtl *d_ctl = nullptr;
    int *d_err = nullptr;         // set by a kernel whose bounded wait ran out
    MeasureCtl *h_ctl = nullptr;  // pinned mirror
    double *h_result = nullptr;   // pinned, kMaxTerms entries
    DevBuf tmp0, tmp1, tmp2, tmp3, tmp4, tmp5;

    StdRng rng;  // the handle's own draw generator (rand's StdRng, seeded from KBW_SEED)

    Profiler prof;
    void *graphs = nullptr;  // replay cache of planned sweeps (sweep.cu)
    void *adj = nullptr;     // adjoint gradient scratch kept between calls (adjoint.cu)

    // execution settings of the fused sweeps (0 = built-in default): tile
    // geometry 2^tile_k amplitudes, at most fusion_depth gates per sweep
    uint32_t tile_k = 0;
    uint32_t fusion_depth = 0;
    // where they came from (KBWG_TUNE_*) and the last tuner's measurements
    uint32_t tune_source = 0, tune_candidates = 0;
    double tune_ms = 0.0, tune_default_ms = 0.0;

    // run-time specialised sweep kernels: KBWG_JIT_OFF / _AUTO / _ALWAYS
    int jit_mode = 1;

    // statistics of the last flush
    uint64_t last_passes = 0;
    uint64_t last_specialised = 0;  // sweeps of it that ran a specialised kernel
    uint64_t last_gates = 0;
};

// True when the handle's gates run in float-float arithmetic with the
// state kept in float-float form between sweeps.
bool ff_capable(const Sim &s);
// Turn a float-float resident state back into binary64 (no-op otherwise).
cudaError_t ensure_binary64(Sim &s);
// |0...0> in the handle's resident format.
cudaError_t init_state(Sim &s);
// Free the replay cache of planned sweeps.
void release_graphs(Sim &s);
// Free the adjoint gradient's scratch.
void release_adjoint(Sim &s);

// Build the descriptor of one trait gate: constants computed in the state
// precision exactly as kbw Dense<F> does (src/dense.rs:211-334).
GateDesc make_gate_desc(int prec, uint32_t kind, uint32_t target, uint64_t ctrl, double angle);

// Run every queued gate (fused sweeps unless KBWG_FLAG_NO_FUSION).
cudaError_t flush_queue(Sim &s);

// Fusion planner entry used by flush_queue (sweep.cu).
cudaError_t run_fused(Sim &s, const GateDesc *gates, size_t count);

// Specialised kernels (entry point `entry`) for complete sources, following
// the handle's JIT mode: always: compiled now; auto: from the second request
// of the same sources on, compiled in the background, loaded once done (null
// entries until then); off: none.  *final (if given): the answer will not
// change for these sources (compiled, loaded or failed).
std::vector<const void *> specialised_kernels(Sim &s, const std::vector<std::string> &srcs, const char *entry,
                                              bool *final = nullptr);

// Wait for the handle's background compilations of specialised kernels;
// true if any was still to be used (a later flush of its structure loads it).
bool wait_specialised(Sim &s);

// Write and compile (NVRTC, without loading: no GPU needed) the specialised
// kernel of every sweep a flush of `gates` would run on `s`; returns the
// number of failed compilations and sets `sweeps`.
size_t jit_check(const Sim &s, const GateDesc *gates, size_t count, size_t &sweeps);

// The same for the reverse sweeps of an adjoint gradient of `fwd` (gtype:
// GT_* per gate), one segment.
size_t jit_check_adjoint(const Sim &s, const std::vector<GateDesc> &fwd, const std::vector<int> &gtype,
                         size_t &sweeps);

// Tile sizes K (2^K amplitudes per tile) with a compiled sweep kernel for
// the handle's arithmetic and qubit count, the default first; empty when the
// handle runs one kernel per gate.  Fusion depths the tuner tries.
std::vector<uint32_t> tile_options(const Sim &s);
// The same without the qubit-count filter.
std::vector<uint32_t> compiled_tiles(const Sim &s);
// Register bits R of the compiled geometry with 2^k-amplitude tiles (0: none).
uint32_t tile_register_bits(const Sim &s, uint32_t k);
uint32_t default_tile_k(const Sim &s);
// Tile size the next flush uses (0: one kernel per gate).
uint32_t effective_tile_k(const Sim &s);
constexpr uint32_t kFusionDepths[] = {256, 64, 16};

double next_draw(Sim &s);

// A parsed Pauli string: P = i^{ny} X^x Z^z (per qubit), with its coefficient.
struct PauliString {
    uint64_t x = 0, z = 0;
    int ny = 0;
    double coef = 0.0;
};


// Batched hardware-efficient-ansatz circuits with ring-TFIM energies (hea.cu).
int32_t hea_batch(int precision, bool fast_c128, size_t ncirc, const uint32_t *num_qubits, const uint32_t *layers,
                  const uint64_t *param_offset, const double *params, size_t nparams, double zz, double xc,
                  double *energies);

// Many circuits with their own gates and Pauli Hamiltonians in one launch (batch.cu).
int32_t batch_circuits(int precision, uint32_t flags, size_t ncirc, const uint32_t *num_qubits,
                       const kbwg_gate *gates, const uintptr_t *gate_offsets, const uint8_t *paulis,
                       const uintptr_t *qubits, const uintptr_t *term_offsets, const double *coefficients,
                       const uintptr_t *ham_offsets, double *energies);

// Adjoint gradient (adjoint.cu).  fwd: the circuit; angles: each gate's
// angle; gtype: GT_* per gate (GT_NONE if not differentiated).  Writes E and
// dE/dtheta per gate; the handle ends in |0...0>.  Returns 0 or a KBWG_* code.
int32_t adjoint_gradient(Sim &s, const std::vector<GateDesc> &fwd, const std::vector<double> &angles,
                         const std::vector<int> &gtype, const std::vector<PauliString> &H, double *energy,
                         std::vector<double> &grad_per_gate, uint32_t max_ckpt);
double host_uniform_scale(double total);

}  // namespace kbwg
