// Fused tile sweeps: types shared by the planner (host) and the kernel.
#pragma once

#include <stdint.h>

#if !defined(__CUDACC_RTC__)
#include <vector>
#endif

#include "common.cuh"

namespace kbwg {

constexpr int kLaneBits = 5;        // local bits 0..4 live across the 32 lanes of a warp
constexpr int kMaxStages = 48;      // register-layout stages per sweep
constexpr int kMaxSweepGates = 256; // gates per sweep (the program is staged in shared memory)

// Tile geometry per precision: 2^K amplitudes per tile (64 KiB), 2^R per
// thread, 32 * 2^(K-5-R) threads per CTA.
template <class T> struct TileCfg;
template <> struct TileCfg<float> {
    static constexpr int K = 13, R = 4;
};
template <> struct TileCfg<double> {
    static constexpr int K = 12, R = 4;
};
// Complex128 float-float sweeps: 2^11 amplitudes (32 KiB) per tile, 8 per
// thread (32 data registers of the 80 a thread gets), three 256-thread CTAs
// per SM: 24 warps hide the latency of the float-float chains better than 16
// warps with 16 amplitudes each (30q brickwork 14 % faster).
struct TileCfgFF {
    static constexpr int K = 11, R = 3;
};

// Arithmetic classes of the gates, one per code path of the tile kernels.
enum {
    TG_X = 0,      // swap
    TG_Y = 1,      // a0' = -i a1, a1' = i a0
    TG_H = 2,      // (a0 +- a1) * c0 (sub 0); sub 1: without the factor (float-float path)
    TG_RX = 3,     // c a - i s partner
    TG_RY = 4,     // c a -+ s partner
    TG_Z = 5,      // |1> negated (first diagonal class)
    TG_P = 6,      // |1> * (c0 + i c1)
    TG_RZ = 7,     // |0> * (c0 + i c1), |1> * (c2 + i c3)
    TG_PI = 8,     // |1> * i^q, q = c0 (float-float path)
    TG_SCALE = 9   // every amplitude * (c0 + i c1) (float-float path)
};
__host__ __device__ inline bool tg_diagonal(uint32_t cls) { return cls >= TG_Z; }
constexpr uint8_t TG_OUTER = 0xFF;  // tb value: diagonal gate whose target lies outside the tile

// Dispatch codes: what a thread does for a gate in its stage's layout.
enum {
    OP_LANE = 0,   // + class (X..RY): target on a lane bit, partner by warp shuffle
    OP_REG = 8,    // + class * 4 + register bit: target on a register bit, in-thread pairs
    OP_DREG = 32,  // + (class - TG_Z) * 4 + register bit: diagonal, target on a register bit
    OP_DFIX = 48   // + (class - TG_Z): diagonal, side fixed per thread (lane/warp bit) or per tile
};

// One gate as a tile sees it (64 bytes; staged in shared memory).  The
// first 16 bytes are the dispatch header a thread reads with one load; op,
// jm and fneed are precomputed by the planner for the layout of the stage
// the gate runs in.
struct alignas(16) TileGate {
    uint8_t op;      // OP_* dispatch code
    uint8_t sub;
    uint8_t tb;      // local target bit, or TG_OUTER
    uint8_t tout;    // global target qubit when tb == TG_OUTER
    uint16_t jm;     // bit j: register j passes the controls on register bits
    uint8_t cls;
    uint8_t rb;      // register bit of the target (when it is one)
    uint32_t fneed;  // controls on this stage's lane/warp bits
    uint32_t cl;     // control mask on local bits
    uint64_t co;     // control mask on bits outside the tile (global positions)
    uint32_t creg;   // controls on this stage's register bits (register-index mask)
    uint32_t pad;
    double c[4];
};
static_assert(sizeof(TileGate) == 64, "TileGate layout");

// Fill op/rb/jm/fneed/creg of a gate for a stage whose register bits start
// at local bit R0 (R register bits, R <= 4).
__host__ __device__ inline void tile_gate_dispatch(TileGate &g, int R0, int R) {
    const uint32_t regmask = ((1u << R) - 1u) << R0;
    g.fneed = g.cl & ~regmask;
    g.creg = (g.cl & regmask) >> R0;
    uint32_t jm = 0;
    for (uint32_t j = 0; j < (1u << R); j++)
        if ((j & g.creg) == g.creg) jm |= 1u << j;
    g.jm = (uint16_t)jm;
    const int rb = (int)g.tb - R0;
    const bool reg_target = g.tb != TG_OUTER && rb >= 0 && rb < R;
    g.rb = reg_target ? (uint8_t)rb : 0;
    if (!tg_diagonal(g.cls)) g.op = (g.tb < kLaneBits) ? OP_LANE + g.cls : OP_REG + g.cls * 4 + rb;
    else if (g.cls != TG_SCALE && reg_target) g.op = OP_DREG + (g.cls - TG_Z) * 4 + rb;
    else g.op = OP_DFIX + (g.cls - TG_Z);
}

// Gradient types of the adjoint sweep: the generator of a differentiated
// gate (RX: X, RY: Y, RZ: Z, P: the |1> projector).
enum { GT_NONE = 0, GT_X = 1, GT_Y = 2, GT_Z = 3, GT_P1 = 4 };

// Layout A holds local bits [5, 5+R) in registers, layout B [K-R, K).
enum { LAYOUT_A = 0, LAYOUT_B = 1 };

struct SweepParams {
    uint64_t hmask;     // global positions of the tile's high qubits
    uint32_t l;         // the tile's contiguous low qubits 0..l-1
    uint32_t m;         // number of high qubits (K - l)
    uint8_t hq[16];     // high qubit positions, ascending
    uint32_t nstages;
    uint32_t gate_count;
    uint8_t stage_layout[kMaxStages];
    uint16_t stage_end[kMaxStages];  // exclusive gate index at which each stage ends
    const TileGate *prog;           // gate_count gates of this sweep
    int *err;                        // set to 1 if a bounded wait ran out
    uint64_t tiles;                  // 2^(n-K)
};

#if !defined(__CUDACC_RTC__)
struct PlannedSweep {
    uint32_t l = 0, m = 0;
    uint8_t hq[16] = {0};
    uint64_t hmask = 0;
    std::vector<TileGate> gates;
    std::vector<uint8_t> stage_layout;
    std::vector<uint16_t> stage_end;
    std::vector<uint32_t> src;  // index in the input list of each gate, in execution order
};

// Greedy commutation-aware planner: groups the gate list into sweeps over
// tiles of K qubits (targets of non-diagonal gates must lie in the tile;
// diagonal gates and controls may lie anywhere) and orders each sweep's gates
// into register-layout stages.
// keep_order: never move a gate past another one (bit-exact mode).
// max_gates: fusion depth, the most gates one sweep may apply.
std::vector<PlannedSweep> plan_sweeps(uint32_t n, int K, int R, const GateDesc *g, size_t count,
                                      bool keep_order = false, size_t max_gates = kMaxSweepGates);

bool is_diagonal(uint32_t kind);

// Fold each uncontrolled diagonal one-qubit gate (Z, P, RZ) into an earlier
// one on the same qubit when no gate in between acts non-diagonally on that
// qubit (those gates touch it only as a control or diagonally, so they
// commute with it).  A merged gate is a phase gate, or a general diagonal in
// the RZ slots (|0> phase c0 + i c1, |1> phase c2 + i c3).  Changes rounding
// only; not used when the program order must be kept.
std::vector<GateDesc> fold_diagonals(const GateDesc *g, size_t count);

// Passes over tiles of 2^K amplitudes for Pauli strings: a pass holds the
// strings whose flip mask fits one tile (local bits 0..l-1 = qubits 0..l-1,
// l..l+m-1 = qubits hq[]), at most max_terms of them.  Strings with flip
// masks too wide for any tile are returned in `wide`.
struct PauliPass {
    uint32_t l = 0, m = 0;
    uint8_t hq[16] = {0};
    uint64_t tile_mask = 0;           // global qubits held by the tile
    std::vector<size_t> members;      // indices into the input masks
    uint32_t local(uint64_t mask) const;  // qubit mask -> local bit mask (qubits in the tile)
};
std::vector<PauliPass> plan_pauli_passes(uint32_t n, int K, const std::vector<uint64_t> &xmasks, size_t max_terms,
                                         std::vector<size_t> &wide);
#endif  // !__CUDACC_RTC__

}  // namespace kbwg
