// Fused tile sweeps: types shared by the planner (host) and the kernel.
#pragma once

#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace kbwg {

constexpr int kLaneBits = 5;        // local bits 0..4 live across the 32 lanes of a warp
constexpr int kMaxStages = 48;      // register-layout stages per sweep
constexpr int kMaxSweepGates = 256; // gates per sweep (the program is staged in shared memory)

// Tile geometry per precision: 2^K amplitudes per tile (64 KiB), 2^R per
// thread, 32 * 2^(K-5-R) threads per CTA.
template <class T> struct TileCfg;
template <> struct TileCfg<float> {
    static constexpr int K = 13, R = 5;
};
template <> struct TileCfg<double> {
    static constexpr int K = 12, R = 4;
};

// Arithmetic classes of the trait gates.
enum {
    TG_PERM = 0,  // X (sub 0), Y (sub 1): permutation with sign/i factors
    TG_H = 1,     // Hadamard: (a0 +- a1) * c0
    TG_ROT = 2,   // RY (sub 0), RX (sub 1): c*a + s*T(partner)
    TG_DIAG = 3   // Z (sub 0), P (sub 1: a1 * (c0,c1)), RZ (sub 2: a0 * (c0,c1), a1 * (c2,c3))
};
constexpr uint8_t TG_OUTER = 0xFF;  // tb value: diagonal gate whose target lies outside the tile

// One gate as a tile sees it (48 bytes; staged in shared memory).
struct TileGate {
    uint8_t cls;
    uint8_t sub;
    uint8_t tb;    // local target bit, or TG_OUTER
    uint8_t tout;  // global target qubit when tb == TG_OUTER
    uint32_t cl;   // control mask on local bits
    uint64_t co;   // control mask on bits outside the tile (global positions)
    double c[4];
};
static_assert(sizeof(TileGate) == 48, "TileGate layout");

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
std::vector<PlannedSweep> plan_sweeps(uint32_t n, int K, int R, const GateDesc *g, size_t count,
                                      bool keep_order = false);

bool is_diagonal(uint32_t kind);

}  // namespace kbwg
