// Fused tile sweeps: types shared by the planner (host) and the kernel.
#pragma once

#include <stdint.h>

#include <vector>

#include "common.cuh"

namespace kbwg {

constexpr int kLaneBits = 5;    // local bits 0..4 live across the 32 lanes of a warp
constexpr int kMaxStages = 48;  // register-layout stages per sweep

// Tile geometry per precision: 2^K amplitudes per tile (64 KiB), 2^R per thread.
template <class T> struct TileCfg;
template <> struct TileCfg<float> {
    static constexpr int K = 13, R = 5;
};
template <> struct TileCfg<double> {
    static constexpr int K = 12, R = 4;
};

// One gate as a tile sees it.
struct TileGate {
    uint32_t kind;
    uint32_t tb;     // local target bit (valid unless TG_OUTER_TARGET)
    uint32_t cl;     // control mask on local bits
    uint32_t flags;  // TG_*
    uint64_t co;     // control mask on bits outside the tile (global positions)
    uint64_t tout;   // global target bit when the target lies outside the tile
    double c[4];
};
enum { TG_OUTER_TARGET = 1 };

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
