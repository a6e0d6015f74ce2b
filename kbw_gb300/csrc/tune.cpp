// Autotuner of the fused gate sweeps (host code, CUDA runtime only).
//
// Two settings shape a flush: the tile size K (2^K amplitudes staged per
// tile; each arithmetic has a few compiled geometries, see tile_options) and
// the fusion depth (the most gates one sweep applies).  Which pair is fastest
// depends on the circuit: deep fusion on small tiles trades memory passes for
// instruction issue, larger tiles admit more gates per sweep but hold fewer
// warps per SM.  The tuner runs the caller's circuit under every pair on the
// handle's own state, times each with CUDA events on the handle's stream,
// keeps the fastest, and puts the state back as it was.  Results are cached
// per process, keyed by device, qubit count, arithmetic and the circuit's
// structure (gate kinds, targets and controls), so a second handle with the
// same circuit reuses them without timing.
#include <string.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "../../include/kbwg.h"
#include "sim.h"
#include "tune.h"

namespace kbwg {

namespace {

using Key = std::tuple<int, uint32_t, int, uint32_t, uint64_t>;
std::mutex g_tune_mu;
std::map<Key, TuneResult> g_tune_cache;

uint64_t structure_hash(const std::vector<GateDesc> &g) {
    uint64_t h = 1469598103934665603ull;  // FNV-1a
    auto mix = [&](uint64_t w) {
        h ^= w;
        h *= 1099511628211ull;
    };
    for (const GateDesc &x : g) {
        mix((uint64_t)x.kind | ((uint64_t)x.target << 8));
        mix(x.ctrl);
    }
    return h;
}

Key key_of(const Sim &s, const std::vector<GateDesc> &g) {
    const uint32_t arith =
        s.flags & (KBWG_FLAG_FAST_C128 | KBWG_FLAG_EXACT_ORDER | KBWG_FLAG_NO_FUSION | KBWG_FLAG_NO_FOLD);
    return Key(s.device, s.n, s.prec, arith, structure_hash(g));
}

// Device time of `reps` applications of the circuit with the handle's
// current settings, after two untimed ones (the first plans and launches
// directly, the second records the CUDA graph that later ones replay and
// starts compiling the specialised kernels, and a third takes them in).
int32_t time_runs(Sim &s, const std::vector<GateDesc> &g, uint32_t reps, cudaEvent_t e0, cudaEvent_t e1, double &ms,
                  std::string &err) {
    auto cuda_fail = [&](cudaError_t e, const char *what) {
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return (int32_t)KBWG_ECUDA;
    };
    cudaError_t e;
    for (int w = 0; w < 2; w++)
        if ((e = run_fused(s, g.data(), g.size())) != cudaSuccess) return cuda_fail(e, "tuning run");
    // the second run started compiling the specialised kernels of these
    // settings (auto mode): wait, and run once more to take them into the graph
    if (wait_specialised(s) && (e = run_fused(s, g.data(), g.size())) != cudaSuccess)
        return cuda_fail(e, "tuning run");
    if ((e = cudaEventRecord(e0, s.stream)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    for (uint32_t r = 0; r < reps; r++)
        if ((e = run_fused(s, g.data(), g.size())) != cudaSuccess) return cuda_fail(e, "tuning run");
    if ((e = cudaEventRecord(e1, s.stream)) != cudaSuccess) return cuda_fail(e, "cudaEventRecord");
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) return cuda_fail(e, "cudaEventSynchronize");
    int flag = 0;
    if ((e = cudaMemcpyAsync(&flag, s.d_err, sizeof flag, cudaMemcpyDeviceToHost, s.stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s.stream)) != cudaSuccess)
        return cuda_fail(e, "error flag read");
    if (flag) {
        cudaMemsetAsync(s.d_err, 0, sizeof flag, s.stream);
        err = "a device-side bounded wait ran out while tuning";
        return KBWG_ETIMEOUT;
    }
    float t = 0.f;
    if ((e = cudaEventElapsedTime(&t, e0, e1)) != cudaSuccess) return cuda_fail(e, "cudaEventElapsedTime");
    ms = (double)t / (double)reps;
    return KBWG_OK;
}

}  // namespace

int32_t autotune(Sim &s, const std::vector<GateDesc> &gates, uint32_t reps, TuneResult &out, std::string &err) {
    out = TuneResult();
    const std::vector<uint32_t> tiles = tile_options(s);
    if (tiles.empty() || gates.empty()) {  // one kernel per gate, or nothing to time
        out.tile_k = effective_tile_k(s);
        out.depth = s.fusion_depth ? s.fusion_depth : kFusionDepths[0];
        return KBWG_OK;
    }
    const Key key = key_of(s, gates);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            out = it->second;
            out.cached = true;
            out.candidates = 0;
            s.tile_k = out.tile_k;
            s.fusion_depth = out.depth;
            return KBWG_OK;
        }
    }
    reps = reps ? reps : 1;

    // keep the state (and its resident format) to put back afterwards
    cudaError_t e = flush_queue(s);
    if (e != cudaSuccess) {
        err = std::string("flush before tuning: ") + cudaGetErrorString(e);
        return KBWG_ECUDA;
    }
    const size_t bytes = (size_t)s.ns * s.elem;
    void *saved = nullptr;
    if (cudaMalloc(&saved, bytes) != cudaSuccess) {
        cudaGetLastError();
        err = "not enough device memory for a copy of the state while tuning";
        return KBWG_ENOMEM;
    }
    const bool saved_ff = s.ff_resident;
    const uint32_t old_k = s.tile_k, old_depth = s.fusion_depth;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int32_t rc = KBWG_OK;
    if ((e = cudaMemcpyAsync(saved, s.state, bytes, cudaMemcpyDeviceToDevice, s.stream)) != cudaSuccess ||
        (e = cudaEventCreate(&e0)) != cudaSuccess || (e = cudaEventCreate(&e1)) != cudaSuccess) {
        err = std::string("tuning set-up: ") + cudaGetErrorString(e);
        rc = KBWG_ECUDA;
    }
    double best = 0.0;
    for (size_t ti = 0; rc == KBWG_OK && ti < tiles.size(); ti++) {
        for (uint32_t d : kFusionDepths) {
            s.tile_k = tiles[ti];
            s.fusion_depth = d;
            double ms = 0.0;
            rc = time_runs(s, gates, reps, e0, e1, ms, err);
            if (rc != KBWG_OK) break;
            out.candidates++;
            if (tiles[ti] == default_tile_k(s) && d == kFusionDepths[0]) out.default_ms = ms;
            if (out.candidates == 1 || ms < best) {
                best = ms;
                out.tile_k = tiles[ti];
                out.depth = d;
            }
        }
    }
    out.ms = best;
    // put the state back whatever happened
    e = cudaMemcpyAsync(s.state, saved, bytes, cudaMemcpyDeviceToDevice, s.stream);
    const cudaError_t es = cudaStreamSynchronize(s.stream);
    s.ff_resident = saved_ff;
    cudaFree(saved);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (rc == KBWG_OK && (e != cudaSuccess || es != cudaSuccess)) {
        err = std::string("restoring the state after tuning: ") + cudaGetErrorString(e != cudaSuccess ? e : es);
        rc = KBWG_ECUDA;
    }
    if (rc != KBWG_OK) {
        s.tile_k = old_k;
        s.fusion_depth = old_depth;
        return rc;
    }
    s.tile_k = out.tile_k;
    s.fusion_depth = out.depth;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[key] = out;
    return KBWG_OK;
}

}  // namespace kbwg
