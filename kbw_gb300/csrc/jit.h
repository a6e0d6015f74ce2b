// Run-time specialised sweep kernels: one straight-line kernel per planned
// sweep, written from the plan and compiled with NVRTC for sm_103a.
#pragma once

#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "sweep.h"

namespace kbwg {

// What a specialised kernel is compiled for: the arithmetic policy (its C++
// name in sweep_dev.cuh), the tile geometry and the launch shape.
struct JitGeometry {
    const char *policy;
    int K, R, threads, ctas_per_sm;
    bool wide = false;  // 64-bit state indices (registers above 32 qubits)
};

// Source of the kernel that applies `sw`'s gates (entry point kbwg_jit_sweep,
// launched like k_sweep with (Mem *state, SweepParams)).
std::string jit_sweep_source(const JitGeometry &geo, const PlannedSweep &sw);

// Source of the specialised reverse (adjoint) sweep of `sw` (entry point
// kbwg_jit_adjoint, launched like k_adjoint with (phi, lambda, AdjParams));
// ginfo per gate of the sweep: gradient type | slot << 4.
std::string jit_adjoint_source(const JitGeometry &geo, const PlannedSweep &sw, const std::vector<uint32_t> &ginfo);

// Compiled kernels for the sweeps of a plan, one entry per sweep (nullptr
// where none could be built).  Sources already compiled in this process are
// reused; the others are compiled in parallel.  Returns false if NVRTC is
// unavailable or a compilation failed (the reason goes to jit_last_error()).
bool jit_sweep_kernels(const JitGeometry &geo, const std::vector<PlannedSweep> &plan, std::vector<const void *> &out);

// Kernel for one complete source with entry point `entry` (compiled once per
// process and source).
const void *jit_kernel(const std::string &src, const char *entry);

// Compile sources (entry kbwg_jit_sweep) to cubins without loading them (no
// GPU needed), in parallel; returns how many failed.
size_t jit_compile_only(const std::vector<std::string> &srcs);

// Background compilation of sources (to cubins, not loaded): started by
// jit_prefetch on a worker thread; jit_kernel and jit_sweep_kernels then load
// its results without compiling.  NVRTC only; no CUDA call off the caller's
// thread.
struct JitJob;
std::shared_ptr<JitJob> jit_prefetch(std::vector<std::string> srcs);
bool jit_job_done(const JitJob &job);
// Stop background compilation for good (between compilations) and wait for
// the jobs; later jobs complete at once without compiling.
void jit_shutdown();
void jit_job_wait(JitJob &job);

bool jit_available();
std::string jit_last_error();

struct JitStats {
    uint64_t compiled = 0;   // sources compiled by NVRTC in this process
    uint64_t reused = 0;     // requests served from the cache
    uint64_t failed = 0;     // failed compilations or loads
    double compile_s = 0.0;  // wall time spent compiling
};
JitStats jit_stats();

// Modes of a handle (KBWG_JIT_* in kbwg.h): off; auto (a gate structure
// flushed before, states of at least jit_min_qubits() qubits); always.
int jit_default_mode();
uint32_t jit_min_qubits();

}  // namespace kbwg
