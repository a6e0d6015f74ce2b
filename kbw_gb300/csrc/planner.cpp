// Host fusion planner for the tile sweeps (pure C++, no CUDA calls).
#include <string.h>

#include <algorithm>

#include "sweep.h"

namespace kbwg {

bool is_diagonal(uint32_t kind) { return is_diag_kind(kind); }

static inline uint64_t qubits_of(const GateDesc &g) { return g.ctrl | (1ull << g.target); }

// Gates left behind (deferred), summarised for commutation: `any` = every
// qubit they touch, `ndt` = the targets of their non-diagonal gates.  Two
// gates commute when every qubit they share is acted on diagonally by both
// (a control, or a diagonal gate's qubit), so a later gate may pass the
// deferred ones iff it touches no deferred non-diagonal target and, if it is
// non-diagonal, its own target is untouched by them.
struct Deferred {
    uint64_t any = 0, ndt = 0;
    bool all = false;  // order-preserving mode: nothing passes
    bool passes(const GateDesc &x) const {
        if (all) return false;
        if (qubits_of(x) & ndt) return false;
        return is_diagonal(x.kind) || !((any >> x.target) & 1);
    }
    void add(const GateDesc &x, bool keep_order) {
        any |= qubits_of(x);
        if (!is_diagonal(x.kind)) ndt |= 1ull << x.target;
        if (keep_order) all = true;
    }
};

// Choose the tile's contiguous low block l (as large as possible) and its
// high qubits: every needed high target, padded up to K qubits.
static void choose_tile(uint32_t n, int K, uint64_t needed, PlannedSweep &sw) {
    int l = K;
    for (; l >= kLaneBits; l--) {
        const uint64_t above = (l >= 64) ? 0 : (needed & ~((1ull << l) - 1));
        if (l + __builtin_popcountll(above) <= K) break;
    }
    uint64_t h = needed & ~((1ull << l) - 1);
    for (uint32_t q = l; q < n && l + __builtin_popcountll(h) < K; q++) h |= 1ull << q;
    sw.l = (uint32_t)l;
    sw.hmask = h;
    sw.m = 0;
    for (uint32_t q = 0; q < 64; q++)
        if (h >> q & 1) sw.hq[sw.m++] = (uint8_t)q;
}

static inline int local_bit(const PlannedSweep &sw, uint32_t q) {
    if (q < sw.l) return (int)q;
    for (uint32_t j = 0; j < sw.m; j++)
        if (sw.hq[j] == q) return (int)(sw.l + j);
    return -1;
}

static inline bool runs_in(int lb, int layout, int K, int R) {
    if (lb < kLaneBits) return true;
    if (layout == LAYOUT_A) return lb < kLaneBits + R;
    return lb >= K - R;
}

std::vector<PlannedSweep> plan_sweeps(uint32_t n, int K, int R, const GateDesc *g, size_t count,
                                      bool keep_order, size_t max_gates) {
    max_gates = std::min(std::max<size_t>(max_gates, 1), (size_t)kMaxSweepGates);
    std::vector<PlannedSweep> out;
    // rem[start..] are the gates not placed yet, in program order; a sweep
    // rewrites only the part of it its selection examined
    std::vector<size_t> rem(count);
    for (size_t i = 0; i < count; i++) rem[i] = i;
    size_t start = 0;
    const size_t window = 8192;  // gates examined per sweep
    const int max_high = K - kLaneBits;
    // Greedy selection of a sweep's gates.  grow: the admissible high targets
    // (bits >= 5) are collected first come, first served up to max_high;
    // otherwise they are the fixed set `needed`.
    const uint64_t all_qubits = (n >= 64) ? ~0ull : ((1ull << n) - 1);
    // rest receives the examined gates not taken; *stop is where the
    // examination ended (rem[*stop..] were not looked at)
    auto select = [&](uint64_t needed, bool grow, std::vector<size_t> *take, std::vector<size_t> *rest,
                      size_t *stop) {
        Deferred blocked;
        size_t taken = 0;
        const size_t scan = std::min(rem.size(), start + window);
        size_t ii = start;
        for (; ii < scan; ii++) {
            // every qubit is a deferred non-diagonal target: no later gate can
            // pass; or the sweep is full
            if ((blocked.ndt & all_qubits) == all_qubits || blocked.all || taken >= max_gates) break;
            const size_t i = rem[ii];
            const GateDesc &x = g[i];
            bool ok = blocked.passes(x) && taken < max_gates;
            if (ok && !is_diagonal(x.kind) && x.target >= (uint32_t)kLaneBits) {
                const uint64_t b = 1ull << x.target;
                if (!(needed & b)) {
                    if (grow && __builtin_popcountll(needed) < max_high)
                        needed |= b;
                    else
                        ok = false;
                }
            }
            if (ok) {
                taken++;
                if (take) take->push_back(i);
            } else {
                if (rest) rest->push_back(i);
                blocked.add(x, keep_order);
            }
        }
        if (stop) *stop = ii;
        return std::make_pair(taken, needed);
    };
    while (start < rem.size()) {
        // 1. choose the sweep's gates: first-come high targets, or the window
        // of max_high consecutive qubits that admits the most gates
        auto best = select(0, true, nullptr, nullptr, nullptr);
        bool best_grow = true;
        if (!keep_order && n > (uint32_t)K) {
            for (uint32_t a = kLaneBits; a + max_high <= n; a++) {
                const uint64_t w = ((1ull << max_high) - 1) << a;
                const auto c = select(w, false, nullptr, nullptr, nullptr);
                if (c.first > best.first) {
                    best = c;
                    best_grow = false;
                }
            }
        }
        std::vector<size_t> take, rest;
        size_t stop = start;
        const uint64_t needed = select(best_grow ? 0 : best.second, best_grow, &take, &rest, &stop).second;

        PlannedSweep sw;
        choose_tile(n, K, needed, sw);
        const uint64_t tile_mask = ((1ull << sw.l) - 1) | sw.hmask;

        // 2. order the taken gates into register-layout stages
        std::vector<size_t> pending = take, leftover;
        int layout = LAYOUT_A;
        // start in the layout the first register-bound gate wants
        for (size_t i : pending) {
            const GateDesc &x = g[i];
            if (is_diagonal(x.kind)) continue;
            const int lb = local_bit(sw, x.target);
            if (lb >= kLaneBits) {
                layout = runs_in(lb, LAYOUT_A, K, R) ? LAYOUT_A : LAYOUT_B;
                break;
            }
        }
        int idle_switches = 0;
        while (!pending.empty()) {
            if ((int)sw.stage_layout.size() == kMaxStages) {
                leftover = pending;
                break;
            }
            std::vector<size_t> now, later;
            Deferred blk;
            for (size_t i : pending) {
                const GateDesc &x = g[i];
                bool ok = blk.passes(x);
                if (ok && !is_diagonal(x.kind)) ok = runs_in(local_bit(sw, x.target), layout, K, R);
                if (ok) {
                    now.push_back(i);
                } else {
                    later.push_back(i);
                    blk.add(x, keep_order);
                }
            }
            if (now.empty()) {
                if (++idle_switches > 2) {  // cannot happen for a valid tile; guard anyway
                    leftover = pending;
                    break;
                }
                layout ^= 1;
                continue;
            }
            idle_switches = 0;
            for (size_t i : now) {
                const GateDesc &x = g[i];
                TileGate t;
                memset(&t, 0, sizeof t);
                switch (x.kind) {
                case G_X: t.cls = TG_X; break;
                case G_Y: t.cls = TG_Y; break;
                case G_H: t.cls = TG_H; break;
                case G_HN: t.cls = TG_H; t.sub = 1; break;
                case G_RX: t.cls = TG_RX; break;
                case G_RY: t.cls = TG_RY; break;
                case G_Z: t.cls = TG_Z; break;
                case G_P: t.cls = TG_P; break;
                case G_RZ: t.cls = TG_RZ; break;
                case G_PI: t.cls = TG_PI; break;
                default: t.cls = TG_SCALE; break;
                }
                memcpy(t.c, x.c, sizeof t.c);
                const int lb = local_bit(sw, x.target);
                if (lb < 0) {  // diagonal gate on a qubit outside the tile
                    t.tb = TG_OUTER;
                    t.tout = (uint8_t)x.target;
                } else {
                    t.tb = (uint8_t)lb;
                }
                uint64_t cm = x.ctrl;
                while (cm) {
                    const uint32_t q = __builtin_ctzll(cm);
                    cm &= cm - 1;
                    const int cb = (tile_mask >> q & 1) ? local_bit(sw, q) : -1;
                    if (cb >= 0)
                        t.cl |= 1u << cb;
                    else
                        t.co |= 1ull << q;
                }
                tile_gate_dispatch(t, layout == LAYOUT_A ? kLaneBits : K - R, R);
                sw.gates.push_back(t);
                sw.src.push_back((uint32_t)i);
            }
            sw.stage_layout.push_back((uint8_t)layout);
            sw.stage_end.push_back((uint16_t)sw.gates.size());
            pending.swap(later);
            layout ^= 1;
        }
        // gates that did not fit go back in front, in program order, ahead of
        // the ones the selection did not examine (all later in the program)
        std::sort(leftover.begin(), leftover.end());
        std::vector<size_t> merged;
        merged.reserve(leftover.size() + rest.size());
        std::merge(leftover.begin(), leftover.end(), rest.begin(), rest.end(), std::back_inserter(merged));
        start = stop - merged.size();  // every examined gate was taken or left in rest
        std::copy(merged.begin(), merged.end(), rem.begin() + (std::ptrdiff_t)start);
        if (sw.gates.empty()) break;  // no gate placeable (invalid tile geometry): the caller sees the shortfall
        out.push_back(std::move(sw));
    }
    return out;
}

// ---- diagonal folding -------------------------------------------------------------
static void diag_sides(const GateDesc &x, double s[4]) {  // |0> and |1> phases (re, im)
    s[0] = 1.0, s[1] = 0.0, s[2] = 1.0, s[3] = 0.0;
    if (x.kind == G_Z) s[2] = -1.0;
    else if (x.kind == G_P) s[2] = x.c[0], s[3] = x.c[1];
    else s[0] = x.c[0], s[1] = x.c[1], s[2] = x.c[2], s[3] = x.c[3];  // G_RZ slot convention
}

std::vector<GateDesc> fold_diagonals(const GateDesc *g, size_t count) {
    std::vector<GateDesc> out;
    out.reserve(count);
    int64_t pend[64];
    for (int q = 0; q < 64; q++) pend[q] = -1;
    for (size_t i = 0; i < count; i++) {
        const GateDesc &x = g[i];
        const bool fold = x.ctrl == 0 && (x.kind == G_Z || x.kind == G_P || x.kind == G_RZ);
        if (fold && pend[x.target] >= 0) {
            GateDesc &y = out[(size_t)pend[x.target]];
            double a[4], b[4];
            diag_sides(y, a);
            diag_sides(x, b);
            const double s0r = a[0] * b[0] - a[1] * b[1], s0i = a[0] * b[1] + a[1] * b[0];
            const double s1r = a[2] * b[2] - a[3] * b[3], s1i = a[2] * b[3] + a[3] * b[2];
            if (s0r == 1.0 && s0i == 0.0) {  // |0> untouched: a phase gate
                y.kind = G_P;
                y.c[0] = s1r, y.c[1] = s1i, y.c[2] = y.c[3] = 0.0;
            } else {
                y.kind = G_RZ;
                y.c[0] = s0r, y.c[1] = s0i, y.c[2] = s1r, y.c[3] = s1i;
            }
            continue;
        }
        if (!is_diag_kind(x.kind)) pend[x.target] = -1;  // a non-diagonal action on its target
        out.push_back(x);
        if (fold) pend[x.target] = (int64_t)out.size() - 1;
    }
    return out;
}

uint32_t PauliPass::local(uint64_t mask) const {
    uint32_t r = (uint32_t)(mask & ((1ull << l) - 1));
    for (uint32_t j = 0; j < m; j++)
        if (mask >> hq[j] & 1) r |= 1u << (l + j);
    return r;
}

// Largest contiguous low block l >= 5 such that l plus the bits of `need`
// above it fit K; -1 if none.
static int pauli_low_bits(uint64_t need, int K) {
    for (int l = K; l >= kLaneBits; l--) {
        const uint64_t above = need & ~((1ull << l) - 1);
        if (l + __builtin_popcountll(above) <= K) return l;
    }
    return -1;
}

std::vector<PauliPass> plan_pauli_passes(uint32_t n, int K, const std::vector<uint64_t> &xmasks, size_t max_terms,
                                         std::vector<size_t> &wide) {
    std::vector<PauliPass> out;
    std::vector<size_t> pend;
    wide.clear();
    for (size_t k = 0; k < xmasks.size(); k++) {
        if (pauli_low_bits(xmasks[k], K) >= 0)
            pend.push_back(k);
        else
            wide.push_back(k);
    }
    while (!pend.empty()) {
        uint64_t needed = 0;
        std::vector<size_t> take, rest;
        for (size_t k : pend) {
            const uint64_t nn = needed | xmasks[k];
            if (take.size() < max_terms && pauli_low_bits(nn, K) >= 0) {
                needed = nn;
                take.push_back(k);
            } else {
                rest.push_back(k);
            }
        }
        PauliPass p;
        p.l = (uint32_t)pauli_low_bits(needed, K);
        uint64_t h = needed & ~((1ull << p.l) - 1);
        for (uint32_t q = p.l; q < n && p.l + __builtin_popcountll(h) < (uint32_t)K; q++) h |= 1ull << q;
        for (uint32_t q = 0; q < 64; q++)
            if (h >> q & 1) p.hq[p.m++] = (uint8_t)q;
        p.tile_mask = ((1ull << p.l) - 1) | h;
        p.members = std::move(take);
        out.push_back(std::move(p));
        pend.swap(rest);
    }
    return out;
}

}  // namespace kbwg
