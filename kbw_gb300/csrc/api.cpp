// extern "C" boundary of the engine (declared in include/kbwg.h).  Every
// entry validates its arguments, turns CUDA failures into status codes and
// never lets an exception cross the ABI.
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/kbwg.h"
#include "jit.h"
#include "sim.h"
#include "sweep.h"
#include "tune.h"

namespace kbwg {

std::atomic<uint64_t> g_launches{0};
std::atomic<uint64_t> g_h2d_bytes{0}, g_d2h_bytes{0};
static thread_local std::string g_last_error;

void set_error(int32_t code, const std::string &msg) {
    (void)code;
    g_last_error = msg;
}

cudaError_t DevBuf::ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    size_t want = std::max(bytes, (size_t)4096);
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) cap = want;
    return e;
}

void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
}

GateDesc make_gate_desc(int prec, uint32_t kind, uint32_t target, uint64_t ctrl, double angle) {
    GateDesc g;
    memset(&g, 0, sizeof g);
    g.kind = kind;
    g.target = target;
    g.ctrl = ctrl;
    if (prec) {  // Dense<f64>
        switch (kind) {
        case G_H: g.c[0] = 0.70710678118654752440; break;
        case G_P: g.c[0] = cos(angle); g.c[1] = sin(angle); break;
        case G_RX:
        case G_RY: g.c[0] = cos(angle / 2.0); g.c[1] = sin(angle / 2.0); break;
        case G_RZ:
            g.c[0] = cos(-angle / 2.0); g.c[1] = sin(-angle / 2.0);
            g.c[2] = cos(angle / 2.0); g.c[3] = sin(angle / 2.0);
            break;
        default: break;
        }
    } else {  // Dense<f32>: F::from(x) rounds the f64 argument to f32 first
        switch (kind) {
        case G_H: g.c[0] = (double)0.70710678118654752440f; break;
        case G_P: g.c[0] = cosf((float)angle); g.c[1] = sinf((float)angle); break;
        case G_RX:
        case G_RY: g.c[0] = cosf((float)(angle / 2.0)); g.c[1] = sinf((float)(angle / 2.0)); break;
        case G_RZ:
            g.c[0] = cosf((float)(-angle / 2.0)); g.c[1] = sinf((float)(-angle / 2.0));
            g.c[2] = cosf((float)(angle / 2.0)); g.c[3] = sinf((float)(angle / 2.0));
            break;
        default: break;
        }
    }
    return g;
}

double host_uniform_scale(double total) {
    const double max_rand = 1.0 - DBL_EPSILON;
    double scale = total;
    while (scale * max_rand >= total) {
        uint64_t u;
        memcpy(&u, &scale, 8);
        u -= 1;
        memcpy(&scale, &u, 8);
    }
    return scale;
}

// One draw of the handle's generator, used when the caller passes no draws:
// the UniformFloat<f64> sample WeightedIndex takes from rand's StdRng
// (src/quantum_execution.rs:279-282, src/convert.rs:60-64).
double next_draw(Sim &s) { return s.rng.uniform01(); }

template <class T>
static cudaError_t flush_t(Sim &s) {
    if (s.queue.empty()) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    s.last_gates = s.queue.size();
    s.last_specialised = 0;
    if (s.flags & KBWG_FLAG_NO_FUSION) {
        for (const GateDesc &g : s.queue) {
            if (s.prof.on) s.prof.mark(s.stream);
            e = launch_gate1<T>(s.state, s.n, g, s.stream);
            if (s.prof.on) {
                s.prof.mark(s.stream);
                s.prof.bytes += 2.0 * (double)s.elem * (double)s.ns;
            }
            if (e != cudaSuccess) break;
        }
        s.last_passes = s.queue.size();
    } else {
        e = run_fused(s, s.queue.data(), s.queue.size());
    }
    s.queue.clear();
    return e;
}

cudaError_t flush_queue(Sim &s) { return s.prec ? flush_t<double>(s) : flush_t<float>(s); }

// Flush, then bring a float-float resident state back to binary64: every
// operation other than gate application and qubit swaps reads binary64.
static cudaError_t settle(Sim &s) {
    cudaError_t e = flush_queue(s);
    if (e != cudaSuccess) return e;
    return ensure_binary64(s);
}

}  // namespace kbwg

using namespace kbwg;

struct kbwg_sim : public Sim {};

#define CUDA_TRY(expr)                                                                            \
    do {                                                                                          \
        cudaError_t _e = (expr);                                                                  \
        if (_e != cudaSuccess) {                                                                  \
            set_error(KBWG_ECUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));            \
            return KBWG_ECUDA;                                                                    \
        }                                                                                         \
    } while (0)

#define GUARD_BEGIN try {
#define GUARD_END                                                   \
    }                                                               \
    catch (const std::bad_alloc &) {                                \
        set_error(KBWG_ENOMEM, "host allocation failed");           \
        return KBWG_ENOMEM;                                         \
    }                                                               \
    catch (...) {                                                   \
        set_error(KBWG_EINVAL, "unexpected exception");             \
        return KBWG_EINVAL;                                         \
    }

static int32_t fail(int32_t code, const char *msg) {
    set_error(code, msg);
    return code;
}

static int32_t select_device(kbwg_sim *s) {
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cur != s->device) CUDA_TRY(cudaSetDevice(s->device));
    return KBWG_OK;
}

#define ENTER(sim)                                            \
    if (!(sim)) return fail(KBWG_EINVAL, "null handle");      \
    {                                                         \
        int32_t _r = select_device(sim);                      \
        if (_r) return _r;                                    \
    }

// KBWG_TILE_QUBITS / KBWG_FUSION_DEPTH: sweep settings for every new handle.
static bool env_u32(const char *name, uint32_t &v, bool &present) {
    const char *t = getenv(name);
    present = t && *t;
    if (!present) return true;
    char *end = nullptr;
    const unsigned long x = strtoul(t, &end, 10);
    if (!end || *end || x > 0xFFFFFFFFul) return false;
    v = (uint32_t)x;
    return true;
}

static bool env_tuning_set() {
    const char *a = getenv("KBWG_TILE_QUBITS"), *b = getenv("KBWG_FUSION_DEPTH");
    return (a && *a) || (b && *b);
}

static int32_t apply_env_tuning(Sim &s, std::string &msg) {
    uint32_t k = 0, d = 0;
    bool hk = false, hd = false;
    if (!env_u32("KBWG_TILE_QUBITS", k, hk)) return msg = "KBWG_TILE_QUBITS is not a number", KBWG_EINVAL;
    if (!env_u32("KBWG_FUSION_DEPTH", d, hd)) return msg = "KBWG_FUSION_DEPTH is not a number", KBWG_EINVAL;
    if (hk) {
        const std::vector<uint32_t> ks = compiled_tiles(s);
        if (k && std::find(ks.begin(), ks.end(), k) == ks.end())
            return msg = "KBWG_TILE_QUBITS=" + std::to_string(k) + ": no sweep kernel of that tile size for this arithmetic",
                   KBWG_EINVAL;
        s.tile_k = k;
    }
    if (hd) {
        if (d > (uint32_t)kMaxSweepGates) return msg = "KBWG_FUSION_DEPTH must be 0..256", KBWG_EINVAL;
        s.fusion_depth = d;
    }
    if (hk || hd) s.tune_source = KBWG_TUNE_ENV;
    return KBWG_OK;
}

template <class F>
static auto dispatch(kbwg_sim *s, F &&f) -> decltype(f((float *)nullptr)) {
    return s->prec ? f((double *)nullptr) : f((float *)nullptr);
}

extern "C" {

int32_t kbwg_new(uintptr_t num_qubits, int32_t precision, uint32_t flags, kbwg_sim **out) {
    GUARD_BEGIN
    if (!out) return fail(KBWG_EINVAL, "null out pointer");
    *out = nullptr;
    if (num_qubits > kMaxQubits) return fail(KBWG_EQUBITS, "num_qubits > 40");
    if (precision != KBWG_C64 && precision != KBWG_C128) return fail(KBWG_EINVAL, "bad precision");
    kbwg_sim *s = new kbwg_sim();
    s->n = (uint32_t)num_qubits;
    s->prec = precision;
    s->flags = flags;
    s->ns = 1ull << num_qubits;
    s->elem = precision ? 16 : 8;
    CUDA_TRY(cudaGetDevice(&s->device));
    auto cleanup = [&](int32_t code, const std::string &m) {
        kbwg_free(s);
        set_error(code, m);
        return code;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cleanup(KBWG_ECUDA, cudaGetErrorString(e));
    e = cudaMalloc(&s->state, s->ns * s->elem);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cleanup(KBWG_ENOMEM, std::string("state allocation: ") + cudaGetErrorString(e));
    }
    const size_t part = (size_t)kReduceBlocks * kMaxTerms * sizeof(double);
    const size_t scratch_bytes = part + 256 + 256 + sizeof(MeasureCtl) + 256;
    e = cudaMalloc(&s->scratch, scratch_bytes);
    if (e != cudaSuccess) return cleanup(KBWG_ENOMEM, "scratch allocation");
    char *p = (char *)s->scratch;
    s->rs.partials = (double *)p;
    s->rs.ticket = (unsigned *)(p + part);
    s->rs.result = (double *)(p + part + 256);
    s->d_ctl = (MeasureCtl *)(p + part + 512);
    s->d_err = (int *)(p + part + 128);
    e = cudaMemsetAsync(s->scratch, 0, scratch_bytes, s->stream);
    if (e != cudaSuccess) return cleanup(KBWG_ECUDA, cudaGetErrorString(e));
    e = cudaMallocHost(&s->h_ctl, sizeof(MeasureCtl) + kMaxTerms * sizeof(double));
    if (e != cudaSuccess) return cleanup(KBWG_ENOMEM, "pinned allocation");
    s->h_result = (double *)(s->h_ctl + 1);
    // StdRng::seed_from_u64(KBW_SEED) as QubitManager::new (src/quantum_execution.rs:181-191)
    s->rng = StdRng::seed_from_u64(kbw_seed_from_env());
    s->jit_mode = jit_default_mode();
    std::string tmsg;
    const int32_t trc = apply_env_tuning(*s, tmsg);
    if (trc != KBWG_OK) return cleanup(trc, tmsg);
    e = init_state(*s);
    if (e != cudaSuccess) return cleanup(KBWG_ECUDA, cudaGetErrorString(e));
    e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return cleanup(KBWG_ECUDA, cudaGetErrorString(e));
    *out = s;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_free(kbwg_sim *s) {
    GUARD_BEGIN
    if (!s) return KBWG_OK;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->state) cudaFree(s->state);
    if (s->scratch) cudaFree(s->scratch);
    if (s->h_ctl) cudaFreeHost(s->h_ctl);
    s->tmp0.release();
    s->tmp1.release();
    s->tmp2.release();
    s->tmp3.release();
    s->tmp4.release();
    s->tmp5.release();
    s->prof.release();
    release_graphs(*s);
    release_adjoint(*s);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return KBWG_OK;
    GUARD_END
}

static int32_t push_gate(kbwg_sim *s, uint32_t kind, double angle, uintptr_t target, const uintptr_t *control,
                         uintptr_t n_control) {
    GUARD_BEGIN
    if (!s) return fail(KBWG_EINVAL, "null handle");
    if (target >= s->n) return fail(KBWG_EINVAL, "target qubit out of range");
    if (n_control && !control) return fail(KBWG_EINVAL, "null control list");
    uint64_t mask = 0;
    for (uintptr_t i = 0; i < n_control; i++) {
        if (control[i] >= s->n) return fail(KBWG_EINVAL, "control qubit out of range");
        if (control[i] == target) return fail(KBWG_EINVAL, "control equals target");
        mask |= 1ull << control[i];
    }
    s->queue.push_back(make_gate_desc(s->prec, kind, (uint32_t)target, mask, angle));
    if (s->queue.size() >= 65536) {
        ENTER(s);
        CUDA_TRY(flush_queue(*s));
    }
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_pauli_x(kbwg_sim *s, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_X, 0.0, t, c, nc); }
int32_t kbwg_pauli_y(kbwg_sim *s, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_Y, 0.0, t, c, nc); }
int32_t kbwg_pauli_z(kbwg_sim *s, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_Z, 0.0, t, c, nc); }
int32_t kbwg_hadamard(kbwg_sim *s, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_H, 0.0, t, c, nc); }
int32_t kbwg_phase(kbwg_sim *s, double a, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_P, a, t, c, nc); }
int32_t kbwg_rx(kbwg_sim *s, double a, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_RX, a, t, c, nc); }
int32_t kbwg_ry(kbwg_sim *s, double a, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_RY, a, t, c, nc); }
int32_t kbwg_rz(kbwg_sim *s, double a, uintptr_t t, const uintptr_t *c, uintptr_t nc) { return push_gate(s, G_RZ, a, t, c, nc); }

int32_t kbwg_apply_gates(kbwg_sim *s, const kbwg_gate *gates, uintptr_t n_gates) {
    GUARD_BEGIN
    if (!s) return fail(KBWG_EINVAL, "null handle");
    if (n_gates && !gates) return fail(KBWG_EINVAL, "null gate list");
    const uint64_t all = (s->n >= 64) ? ~0ull : ((1ull << s->n) - 1);
    for (uintptr_t i = 0; i < n_gates; i++) {
        const kbwg_gate &g = gates[i];
        if (g.kind > KBWG_RZ) return fail(KBWG_EINVAL, "bad gate kind");
        if (g.target >= s->n) return fail(KBWG_EINVAL, "target qubit out of range");
        if (g.control_mask & ~all) return fail(KBWG_EINVAL, "control qubit out of range");
        if (g.control_mask & (1ull << g.target)) return fail(KBWG_EINVAL, "control equals target");
    }
    s->queue.reserve(s->queue.size() + n_gates);
    for (uintptr_t i = 0; i < n_gates; i++) {
        const kbwg_gate &g = gates[i];
        s->queue.push_back(make_gate_desc(s->prec, g.kind, g.target, g.control_mask, g.angle));
    }
    if (s->queue.size() >= 65536) {
        ENTER(s);
        CUDA_TRY(flush_queue(*s));
    }
    return KBWG_OK;
    GUARD_END
}

static int32_t check_device_error(kbwg_sim *s) {
    int flag = 0;
    CUDA_TRY(copy_async(&flag, s->d_err, sizeof flag, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (flag) {
        CUDA_TRY(cudaMemsetAsync(s->d_err, 0, sizeof flag, s->stream));
        return fail(KBWG_ETIMEOUT, "a device-side bounded wait ran out; the state is not valid");
    }
    return KBWG_OK;
}

int32_t kbwg_flush(kbwg_sim *s) {
    GUARD_BEGIN
    ENTER(s);
    CUDA_TRY(flush_queue(*s));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return check_device_error(s);
    GUARD_END
}

int32_t kbwg_measure_p1(kbwg_sim *s, uintptr_t target, double *p1) {
    GUARD_BEGIN
    ENTER(s);
    if (!p1) return fail(KBWG_EINVAL, "null output");
    if (target >= s->n) return fail(KBWG_EINVAL, "target qubit out of range");
    CUDA_TRY(flush_queue(*s));  // (a float-float resident state is read as is)
    const uint64_t bit = 1ull << target;
    if (s->ff_resident) {
        CUDA_TRY(launch_masked_norm_ff(s->state, s->n, bit, bit, s->rs, s->stream));
    } else {
        CUDA_TRY(dispatch(s, [&](auto *tp) {
            using T = std::remove_pointer_t<decltype(tp)>;
            return launch_masked_norm<T>(s->state, s->n, bit, bit, s->rs, s->stream);
        }));
    }
    CUDA_TRY(copy_async(s->h_result, s->rs.result, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    *p1 = s->h_result[0];
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_measure_collapse(kbwg_sim *s, uintptr_t target, bool result, double p) {
    GUARD_BEGIN
    ENTER(s);
    if (target >= s->n) return fail(KBWG_EINVAL, "target qubit out of range");
    CUDA_TRY(flush_queue(*s));  // (a float-float resident state is collapsed as is)
    const uint64_t bit = 1ull << target;
    if (s->ff_resident) {
        CUDA_TRY(launch_collapse_ff(s->state, s->n, nullptr, bit, result ? bit : 0ull, p, s->stream));
    } else {
        CUDA_TRY(dispatch(s, [&](auto *tp) {
            using T = std::remove_pointer_t<decltype(tp)>;
            return launch_collapse<T>(s->state, s->n, nullptr, bit, result ? bit : 0ull, p, s->stream);
        }));
    }
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_measure(kbwg_sim *s, const uintptr_t *qubits, uintptr_t n_qubits, const double *draws,
                     uint64_t *result) {
    GUARD_BEGIN
    ENTER(s);
    if (!result || (n_qubits && !qubits)) return fail(KBWG_EINVAL, "null argument");
    if (n_qubits > 64) return fail(KBWG_EINVAL, "more than 64 qubits in one measurement");
    uint64_t seen = 0;
    for (uintptr_t i = 0; i < n_qubits; i++) {
        if (qubits[i] >= s->n) return fail(KBWG_EINVAL, "qubit out of range");
        if (seen & (1ull << qubits[i])) return fail(KBWG_EINVAL, "qubit listed twice");
        seen |= 1ull << qubits[i];
    }
    *result = 0;
    if (n_qubits == 0) return KBWG_OK;
    CUDA_TRY(flush_queue(*s));  // (a float-float resident state is measured as is)
    MeasureCtl &c = *s->h_ctl;
    memset(&c, 0, sizeof c);
    c.scale2 = 1.0;
    for (uintptr_t k = 0; k < n_qubits; k++) {
        c.qubit[k] = (uint32_t)qubits[n_qubits - 1 - k];  // last listed first
        c.draws[k] = draws ? draws[k] : next_draw(*s);
    }
    CUDA_TRY(copy_async(s->d_ctl, &c, sizeof c, cudaMemcpyHostToDevice, s->stream));
    if (s->ff_resident) {
        for (uint32_t k = 0; k < n_qubits; k++)
            CUDA_TRY(launch_measure_step_ff(s->state, s->n, s->d_ctl, k, s->rs, s->stream));
        CUDA_TRY(launch_collapse_ff(s->state, s->n, s->d_ctl, 0, 0, 0.0, s->stream));
    } else {
        CUDA_TRY(dispatch(s, [&](auto *tp) {
            using T = std::remove_pointer_t<decltype(tp)>;
            for (uint32_t k = 0; k < n_qubits; k++) {
                cudaError_t e = launch_measure_step<T>(s->state, s->n, s->d_ctl, k, s->rs, s->stream);
                if (e != cudaSuccess) return e;
            }
            return launch_collapse<T>(s->state, s->n, s->d_ctl, 0, 0, 0.0, s->stream);
        }));
    }
    CUDA_TRY(copy_async(&c, s->d_ctl, sizeof c, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    *result = c.result;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_dump(kbwg_sim *s, const uintptr_t *qubits, uintptr_t n_qubits, uint64_t *basis_states, double *re,
                  double *im, uintptr_t capacity, uintptr_t *size) {
    GUARD_BEGIN
    ENTER(s);
    if (!size || (n_qubits && !qubits)) return fail(KBWG_EINVAL, "null argument");
    if (n_qubits > 64) return fail(KBWG_EINVAL, "more than 64 qubits");
    for (uintptr_t i = 0; i < n_qubits; i++)
        if (qubits[i] >= s->n) return fail(KBWG_EINVAL, "qubit out of range");
    CUDA_TRY(settle(*s));
    const int B = dump_blocks(s->n);
    CUDA_TRY(s->tmp0.ensure((size_t)B * 8));
    uint64_t *d_counts = (uint64_t *)s->tmp0.ptr;
    CUDA_TRY(dispatch(s, [&](auto *tp) {
        using T = std::remove_pointer_t<decltype(tp)>;
        return launch_dump_count<T>(s->state, s->n, d_counts, s->stream);
    }));
    std::vector<uint64_t> counts(B), offs(B + 1);
    CUDA_TRY(copy_async(counts.data(), d_counts, (size_t)B * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    offs[0] = 0;
    for (int b = 0; b < B; b++) offs[b + 1] = offs[b] + counts[b];
    const uint64_t total = offs[B];
    *size = (uintptr_t)total;
    if (capacity < total) {
        if (capacity == 0 && !basis_states) return KBWG_OK;  // size query
        set_error(KBWG_ECAPACITY, "dump capacity too small");
        return KBWG_ECAPACITY;
    }
    if (!basis_states || !re || !im) return fail(KBWG_EINVAL, "null output buffer");
    if (total == 0) return KBWG_OK;
    DumpSpec spec;
    memset(&spec, 0, sizeof spec);
    spec.nq = (uint32_t)n_qubits;
    for (uintptr_t i = 0; i < n_qubits; i++) spec.qubits[i] = (uint8_t)qubits[i];
    CUDA_TRY(s->tmp1.ensure((size_t)(B + 1) * 8));
    CUDA_TRY(s->tmp2.ensure((size_t)total * 24));
    uint64_t *d_off = (uint64_t *)s->tmp1.ptr;
    uint64_t *d_states = (uint64_t *)s->tmp2.ptr;
    double *d_re = (double *)(d_states + total);
    double *d_im = d_re + total;
    CUDA_TRY(copy_async(d_off, offs.data(), (size_t)(B + 1) * 8, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(dispatch(s, [&](auto *tp) {
        using T = std::remove_pointer_t<decltype(tp)>;
        return launch_dump_write<T>(s->state, s->n, d_off, spec, d_states, d_re, d_im, s->stream);
    }));
    CUDA_TRY(copy_async(basis_states, d_states, total * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(copy_async(re, d_re, total * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(copy_async(im, d_im, total * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_sample(kbwg_sim *s, const uintptr_t *qubits, uintptr_t n_qubits, uintptr_t shots, const double *draws,
                    uint64_t *states, uint64_t *counts, uintptr_t capacity, uintptr_t *n_out) {
    GUARD_BEGIN
    ENTER(s);
    if (!n_out || (n_qubits && !qubits) || (shots && (!states || !counts)))
        return fail(KBWG_EINVAL, "null argument");
    if (n_qubits > 64) return fail(KBWG_EINVAL, "more than 64 qubits");
    for (uintptr_t i = 0; i < n_qubits; i++)
        if (qubits[i] >= s->n) return fail(KBWG_EINVAL, "qubit out of range");
    *n_out = 0;
    const uint64_t need = std::min<uint64_t>(shots, n_qubits >= 64 ? ~0ull : (1ull << n_qubits));
    if (capacity < need) {
        set_error(KBWG_ECAPACITY, "sample capacity too small");
        return KBWG_ECAPACITY;
    }
    CUDA_TRY(settle(*s));
    const int B = sample_blocks(s->n);
    CUDA_TRY(s->tmp0.ensure((size_t)B * 8));
    double *d_bs = (double *)s->tmp0.ptr;
    CUDA_TRY(dispatch(s, [&](auto *tp) {
        using T = std::remove_pointer_t<decltype(tp)>;
        return launch_weight_blocksum<T>(s->state, s->n, d_bs, s->stream);
    }));
    std::vector<double> bs(B), pre(B + 1);
    CUDA_TRY(copy_async(bs.data(), d_bs, (size_t)B * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    pre[0] = 0.0;
    for (int b = 0; b < B; b++) pre[b + 1] = pre[b] + bs[b];
    const double total = pre[B];
    if (!(total > 0.0)) return fail(KBWG_EWEIGHT, "all sampling weights are zero");
    if (shots == 0) return KBWG_OK;
    const double scale = host_uniform_scale(total);
    std::vector<double> chosen(shots);
    for (uintptr_t k = 0; k < shots; k++) chosen[k] = (draws ? draws[k] : next_draw(*s)) * scale;
    std::sort(chosen.begin(), chosen.end());
    // block of each shot: first b whose end prefix exceeds the chosen weight
    std::vector<uint32_t> blocks;
    std::vector<uint64_t> begin;
    std::vector<double> bprefix;
    int b = 0;
    for (uintptr_t k = 0; k < shots; k++) {
        while (b < B - 1 && !(pre[b + 1] > chosen[k])) b++;
        if (blocks.empty() || blocks.back() != (uint32_t)b) {
            blocks.push_back((uint32_t)b);
            begin.push_back(k);
            bprefix.push_back(pre[b]);
        }
    }
    begin.push_back(shots);
    const size_t nb = blocks.size();
    const size_t bytes = nb * 4 + (nb + 1) * 8 + nb * 8 + shots * 8 + shots * 8 + 64;
    CUDA_TRY(s->tmp1.ensure(bytes));
    char *base = (char *)s->tmp1.ptr;
    uint64_t *d_pick = (uint64_t *)base;
    double *d_chosen = (double *)(d_pick + shots);
    uint64_t *d_begin = (uint64_t *)(d_chosen + shots);
    double *d_pre = (double *)(d_begin + nb + 1);
    uint32_t *d_blocks = (uint32_t *)(d_pre + nb);
    CUDA_TRY(copy_async(d_chosen, chosen.data(), shots * 8, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(copy_async(d_begin, begin.data(), (nb + 1) * 8, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(copy_async(d_pre, bprefix.data(), nb * 8, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(copy_async(d_blocks, blocks.data(), nb * 4, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(dispatch(s, [&](auto *tp) {
        using T = std::remove_pointer_t<decltype(tp)>;
        return launch_sample_pick<T>(s->state, s->n, d_blocks, (uint32_t)nb, d_begin, d_pre, d_chosen, d_pick,
                                     s->stream);
    }));
    std::vector<uint64_t> pick(shots);
    CUDA_TRY(copy_async(pick.data(), d_pick, shots * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (uintptr_t k = 0; k < shots; k++) {
        uint64_t packed = 0;
        for (uintptr_t j = 0; j < n_qubits; j++) packed |= ((pick[k] >> qubits[n_qubits - 1 - j]) & 1ull) << j;
        pick[k] = packed;
    }
    std::sort(pick.begin(), pick.end());
    uintptr_t m = 0;
    for (uintptr_t k = 0; k < shots; k++) {
        if (m > 0 && states[m - 1] == pick[k]) {
            counts[m - 1]++;
        } else {
            states[m] = pick[k];
            counts[m] = 1;
            m++;
        }
    }
    *n_out = m;
    return KBWG_OK;
    GUARD_END
}

}  // extern "C"

// Parse the flattened Pauli strings of the ABI.  Returns 0 or KBWG_EINVAL.
static int32_t parse_hamiltonian(uint32_t n, const uint8_t *paulis, const uintptr_t *qubits,
                                 const uintptr_t *offsets, const double *coefficients, uintptr_t n_strings,
                                 std::vector<PauliString> &out) {
    if (n_strings && (!offsets || !coefficients)) return fail(KBWG_EINVAL, "null Hamiltonian arrays");
    out.assign(n_strings, PauliString());
    for (uintptr_t k = 0; k < n_strings; k++) {
        PauliString t;
        t.coef = coefficients[k];
        if (offsets[k + 1] < offsets[k]) return fail(KBWG_EINVAL, "offsets not ascending");
        for (uintptr_t i = offsets[k]; i < offsets[k + 1]; i++) {
            if (!paulis || !qubits) return fail(KBWG_EINVAL, "null term arrays");
            const uintptr_t q = qubits[i];
            if (q >= n) return fail(KBWG_EINVAL, "qubit out of range");
            const uint64_t bit = 1ull << q;
            if ((t.x | t.z) & bit) return fail(KBWG_EINVAL, "qubit repeated in one Pauli string");
            switch (paulis[i]) {
            case KBWG_PAULI_X: t.x |= bit; break;
            case KBWG_PAULI_Y: t.x |= bit; t.z |= bit; t.ny++; break;
            case KBWG_PAULI_Z: t.z |= bit; break;
            default: return fail(KBWG_EINVAL, "bad Pauli code");
            }
        }
        out[k] = t;
    }
    return KBWG_OK;
}

// <psi|H|psi> on the handle's current state (queue flushed by the caller).
// True when every string of H is summed by a kernel that reads the
// float-float resident form as is: the diagonal groups (x = 0) and the tiled
// pair passes (no string too wide for a tile).
static bool exp_reads_ff(const Sim &s, const std::vector<PauliString> &strs) {
    const int K = pauli_tile_bits<double>();
    if (s.n < (uint32_t)K) return false;
    std::vector<uint64_t> xm;
    for (const PauliString &t : strs)
        if (t.x != 0) xm.push_back(t.x);
    std::vector<size_t> wide;
    plan_pauli_passes(s.n, K, xm, kMaxTerms, wide);
    return wide.empty();
}

// Flush for exp_value: a float-float resident state stays in that form when
// exp_value_core can read it (no conversion pass), else it goes to binary64.
static cudaError_t settle_for_exp(Sim &s, const std::vector<PauliString> &strs) {
    cudaError_t e = flush_queue(s);
    if (e != cudaSuccess) return e;
    if (s.ff_resident && !exp_reads_ff(s, strs)) return ensure_binary64(s);
    return cudaSuccess;
}

static int32_t exp_value_core(kbwg_sim *s, const std::vector<PauliString> &strs, double *out) {
    const bool ff = s->ff_resident;  // (settle_for_exp left it so only when every kernel below reads that form)
    const size_t n_strings = strs.size();
    std::vector<size_t> order(n_strings);
    for (size_t k = 0; k < n_strings; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return strs[a].x < strs[b].x; });
    CUDA_TRY(s->tmp3.ensure((n_strings + 1) * 8));
    double *d_vals = (double *)s->tmp3.ptr;
    size_t i = 0;
    std::vector<size_t> slot_of;  // group order -> string index
    slot_of.reserve(n_strings);
    auto pair_term = [](const PauliString &t, double &factor, uint32_t &use_im) {
        const int m = t.ny & 3;
        use_im = (m & 1) ? 1 : 0;
        factor = (m == 0 || m == 1) ? 2.0 : -2.0;
    };
    // strings with a flip mask: tiled passes, each covering every string whose
    // flip mask fits one tile (ring TFIM, 30 qubits: 4 passes instead of 30)
    const int K = s->prec ? pauli_tile_bits<double>() : pauli_tile_bits<float>();
    const bool tiled = s->n >= (uint32_t)K;
    std::vector<char> by_tile(n_strings, 0);
    if (tiled) {
        std::vector<size_t> pair_idx;
        std::vector<uint64_t> xm;
        for (size_t k = 0; k < n_strings; k++)
            if (strs[order[k]].x != 0) {
                pair_idx.push_back(order[k]);
                xm.push_back(strs[order[k]].x);
            }
        std::vector<size_t> wide;
        for (const PauliPass &pp : plan_pauli_passes(s->n, K, xm, kMaxTerms, wide)) {
            PauliTilePass pass;
            memset(&pass, 0, sizeof pass);
            pass.K = (uint32_t)K;
            pass.l = pp.l;
            pass.m = pp.m;
            memcpy(pass.hq, pp.hq, sizeof pass.hq);
            std::vector<size_t> take;
            for (size_t j = 0; j < pp.members.size(); j++) {
                const size_t k = pair_idx[pp.members[j]];
                const PauliString &t = strs[k];
                PauliTileTerm &tt = pass.t[j];
                tt.xl = pp.local(t.x);
                tt.hb = 31 - __builtin_clz(tt.xl);
                tt.zl = pp.local(t.z & pp.tile_mask);
                tt.zo = t.z & ~pp.tile_mask;
                pair_term(t, tt.factor, tt.im);
                take.push_back(k);
                by_tile[k] = 1;
            }
            pass.nterms = (uint32_t)take.size();
            CUDA_TRY(dispatch(s, [&](auto *tp) {
                using T = std::remove_pointer_t<decltype(tp)>;
                return launch_pauli_tile<T>(s->state, s->n, ff, pass, s->rs, s->stream);
            }));
            CUDA_TRY(cudaMemcpyAsync(d_vals + slot_of.size(), s->rs.result, take.size() * 8,
                                     cudaMemcpyDeviceToDevice, s->stream));
            slot_of.insert(slot_of.end(), take.begin(), take.end());
        }
    }
    while (i < n_strings) {
        if (by_tile[order[i]]) {  // done by the tiled passes
            i++;
            continue;
        }
        PauliGroup g;
        memset(&g, 0, sizeof g);
        g.x = strs[order[i]].x;
        std::vector<size_t> idx;
        while (i < n_strings && strs[order[i]].x == g.x && idx.size() < (size_t)kMaxTerms) {
            const PauliString &t = strs[order[i]];
            const int k = (int)idx.size();
            g.z[k] = t.z;
            if (g.x == 0) {
                g.factor[k] = 1.0;
                g.use_im[k] = 0;
            } else {
                pair_term(t, g.factor[k], g.use_im[k]);
            }
            idx.push_back(order[i]);
            i++;
        }
        g.nterms = (uint32_t)idx.size();
        CUDA_TRY(dispatch(s, [&](auto *tp) {
            using T = std::remove_pointer_t<decltype(tp)>;
            return launch_pauli_group<T>(s->state, s->n, g, s->rs, s->stream, ff);
        }));
        CUDA_TRY(cudaMemcpyAsync(d_vals + slot_of.size(), s->rs.result, idx.size() * 8, cudaMemcpyDeviceToDevice,
                                 s->stream));
        slot_of.insert(slot_of.end(), idx.begin(), idx.end());
    }
    std::vector<double> grouped(n_strings + 1), vals(n_strings + 1);
    if (n_strings) CUDA_TRY(copy_async(grouped.data(), d_vals, n_strings * 8, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (size_t j = 0; j < n_strings; j++) vals[slot_of[j]] = grouped[j];
    double total = 0.0;  // sum in string order, as the reference's zip/map/sum
    for (size_t k = 0; k < n_strings; k++) total += vals[k] * strs[k].coef;
    *out = total;
    return KBWG_OK;
}

// Validate a gradient circuit; fills the engine gates, angles and gradient types.
static int32_t parse_grad_circuit(kbwg_sim *s, const kbwg_gate *gates, uintptr_t n_gates, const int32_t *param_index,
                                  uintptr_t n_params, std::vector<GateDesc> &fwd, std::vector<double> &angles,
                                  std::vector<int> &gtype) {
    if (n_gates && (!gates || !param_index)) return fail(KBWG_EINVAL, "null gate list");
    const uint64_t all = (s->n >= 64) ? ~0ull : ((1ull << s->n) - 1);
    fwd.resize(n_gates);
    angles.resize(n_gates);
    gtype.assign(n_gates, GT_NONE);
    for (uintptr_t i = 0; i < n_gates; i++) {
        const kbwg_gate &g = gates[i];
        if (g.kind > KBWG_RZ || g.target >= s->n || (g.control_mask & ~all) || (g.control_mask & (1ull << g.target)))
            return fail(KBWG_EINVAL, "bad gate");
        fwd[i] = make_gate_desc(s->prec, g.kind, g.target, g.control_mask, g.angle);
        angles[i] = g.angle;
        const int32_t pi = param_index[i];
        if (pi >= 0) {
            if ((uintptr_t)pi >= n_params) return fail(KBWG_EINVAL, "param_index out of range");
            switch (g.kind) {
            case KBWG_RX: gtype[i] = GT_X; break;
            case KBWG_RY: gtype[i] = GT_Y; break;
            case KBWG_RZ: gtype[i] = GT_Z; break;
            case KBWG_P: gtype[i] = GT_P1; break;
            default: return fail(KBWG_EINVAL, "only P, RX, RY, RZ gates take a parameter");
            }
        } else if (pi != -1) {
            return fail(KBWG_EINVAL, "param_index must be -1 or a parameter index");
        }
    }
    return KBWG_OK;
}

extern "C" {

int32_t kbwg_exp_value(kbwg_sim *s, const uint8_t *paulis, const uintptr_t *qubits, const uintptr_t *offsets,
                       const double *coefficients, uintptr_t n_strings, double *out) {
    GUARD_BEGIN
    ENTER(s);
    if (!out) return fail(KBWG_EINVAL, "null output");
    std::vector<PauliString> strs;
    int32_t r = parse_hamiltonian(s->n, paulis, qubits, offsets, coefficients, n_strings, strs);
    if (r) return r;
    CUDA_TRY(settle_for_exp(*s, strs));
    return exp_value_core(s, strs, out);
    GUARD_END
}

int32_t kbwg_adjoint_gradient(kbwg_sim *s, const kbwg_gate *gates, uintptr_t n_gates, const int32_t *param_index,
                              uintptr_t n_params, const uint8_t *paulis, const uintptr_t *qubits,
                              const uintptr_t *offsets, const double *coefficients, uintptr_t n_strings,
                              uint32_t max_checkpoints, double *energy, double *gradient) {
    GUARD_BEGIN
    ENTER(s);
    if (!energy || (n_params && !gradient)) return fail(KBWG_EINVAL, "null output");
    std::vector<PauliString> strs;
    int32_t r = parse_hamiltonian(s->n, paulis, qubits, offsets, coefficients, n_strings, strs);
    if (r) return r;
    std::vector<GateDesc> fwd;
    std::vector<double> angles;
    std::vector<int> gtype;
    r = parse_grad_circuit(s, gates, n_gates, param_index, n_params, fwd, angles, gtype);
    if (r) return r;
    CUDA_TRY(settle(*s));
    std::vector<double> per_gate;
    r = adjoint_gradient(*s, fwd, angles, gtype, strs, energy, per_gate, max_checkpoints);
    if (r) return r;
    for (uintptr_t p = 0; p < n_params; p++) gradient[p] = 0.0;
    for (uintptr_t i = 0; i < n_gates; i++)
        if (param_index[i] >= 0) gradient[param_index[i]] += per_gate[i];
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_param_shift_gradient(kbwg_sim *s, const kbwg_gate *gates, uintptr_t n_gates,
                                  const int32_t *param_index, uintptr_t n_params, const uint8_t *paulis,
                                  const uintptr_t *qubits, const uintptr_t *offsets, const double *coefficients,
                                  uintptr_t n_strings, double *energy, double *gradient) {
    GUARD_BEGIN
    ENTER(s);
    if (!energy || (n_params && !gradient)) return fail(KBWG_EINVAL, "null output");
    std::vector<PauliString> strs;
    int32_t r = parse_hamiltonian(s->n, paulis, qubits, offsets, coefficients, n_strings, strs);
    if (r) return r;
    std::vector<GateDesc> fwd;
    std::vector<double> angles;
    std::vector<int> gtype;
    r = parse_grad_circuit(s, gates, n_gates, param_index, n_params, fwd, angles, gtype);
    if (r) return r;
    for (uintptr_t i = 0; i < n_gates; i++)
        if (gtype[i] != GT_NONE && gates[i].control_mask)
            return fail(KBWG_EINVAL, "the +-pi/2 shift rule needs uncontrolled parameterised gates");
    // one fresh evaluation per circuit, as BatchExecution::exp_value does
    // (src/quantum_execution.rs:392-405)
    auto evaluate = [&](const std::vector<GateDesc> &circ, double *e) -> int32_t {
        s->queue.clear();
        CUDA_TRY(init_state(*s));
        s->queue = circ;
        CUDA_TRY(settle_for_exp(*s, strs));
        return exp_value_core(s, strs, e);
    };
    r = evaluate(fwd, energy);
    if (r) return r;
    for (uintptr_t p = 0; p < n_params; p++) gradient[p] = 0.0;
    const double shift = 1.57079632679489661923;  // pi/2
    std::vector<GateDesc> circ = fwd;
    for (uintptr_t i = 0; i < n_gates; i++) {
        if (gtype[i] == GT_NONE) continue;
        double ep = 0.0, em = 0.0;
        circ[i] = make_gate_desc(s->prec, gates[i].kind, gates[i].target, gates[i].control_mask, angles[i] + shift);
        r = evaluate(circ, &ep);
        if (r) return r;
        circ[i] = make_gate_desc(s->prec, gates[i].kind, gates[i].target, gates[i].control_mask, angles[i] - shift);
        r = evaluate(circ, &em);
        if (r) return r;
        circ[i] = fwd[i];
        gradient[param_index[i]] += 0.5 * (ep - em);
    }
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_batch_hea_tfim(uintptr_t n_circuits, const uint32_t *num_qubits, const uint32_t *layers,
                            const uint64_t *param_offset, const double *params, uintptr_t n_params, double zz,
                            double x, int32_t precision, uint32_t flags, double *energies) {
    GUARD_BEGIN
    if (n_circuits == 0) return KBWG_OK;
    if (!num_qubits || !layers || !param_offset || !energies || (n_params && !params))
        return fail(KBWG_EINVAL, "null argument");
    if (precision != KBWG_C64 && precision != KBWG_C128) return fail(KBWG_EINVAL, "bad precision");
    return hea_batch(precision, (flags & KBWG_FLAG_FAST_C128) != 0, n_circuits, num_qubits, layers, param_offset,
                     params, n_params, zz, x, energies);
    GUARD_END
}

int32_t kbwg_clear(kbwg_sim *s) {
    GUARD_BEGIN
    ENTER(s);
    s->queue.clear();
    CUDA_TRY(init_state(*s));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_get_state(kbwg_sim *s, void *host_dst, uintptr_t bytes) {
    GUARD_BEGIN
    ENTER(s);
    if (!host_dst || bytes != s->ns * s->elem) return fail(KBWG_EINVAL, "buffer size must equal 2^n * element size");
    CUDA_TRY(settle(*s));
    CUDA_TRY(copy_async(host_dst, s->state, bytes, cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return check_device_error(s);
    GUARD_END
}

int32_t kbwg_set_state(kbwg_sim *s, const void *host_src, uintptr_t bytes) {
    GUARD_BEGIN
    ENTER(s);
    if (!host_src || bytes != s->ns * s->elem) return fail(KBWG_EINVAL, "buffer size must equal 2^n * element size");
    s->queue.clear();
    s->ff_resident = false;
    CUDA_TRY(copy_async(s->state, host_src, bytes, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_state_info(kbwg_sim *s, uintptr_t *num_qubits, int32_t *precision, void **device_ptr,
                        uintptr_t *bytes) {
    GUARD_BEGIN
    ENTER(s);
    CUDA_TRY(settle(*s));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (num_qubits) *num_qubits = s->n;
    if (precision) *precision = s->prec;
    if (device_ptr) *device_ptr = s->state;
    if (bytes) *bytes = s->ns * s->elem;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_swap_qubits(kbwg_sim *s, uintptr_t a, uintptr_t b) {
    GUARD_BEGIN
    ENTER(s);
    if (a >= s->n || b >= s->n) return fail(KBWG_EINVAL, "qubit out of range");
    CUDA_TRY(flush_queue(*s));
    CUDA_TRY(dispatch(s, [&](auto *tp) {
        using T = std::remove_pointer_t<decltype(tp)>;
        return launch_swap<T>(s->state, s->n, (uint32_t)a, (uint32_t)b, s->stream);
    }));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_build_info(const uint8_t **msg, uintptr_t *size) {
    static const char info[] = "kbw-gb300 densegb300 v0.1 [nvcc sm_103a]";
    if (!msg || !size) return KBWG_EINVAL;
    *msg = (const uint8_t *)info;
    *size = sizeof(info) - 1;
    return KBWG_OK;
}

int32_t kbwg_plan(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                  uintptr_t n_gates, uint32_t *order, uint32_t *sweep_end, uint64_t *tile_mask,
                  uintptr_t *n_sweeps) {
    const bool ff = precision && (flags & KBWG_FLAG_FAST_C128);
    const uint32_t K = ff ? TileCfgFF::K : precision ? TileCfg<double>::K : TileCfg<float>::K;
    return kbwg_plan_tuned(num_qubits, precision, flags, K, 0, gates, n_gates, order, sweep_end, tile_mask, n_sweeps);
}

int32_t kbwg_plan_tuned(uintptr_t num_qubits, int32_t precision, uint32_t flags, uint32_t tile_qubits,
                        uint32_t fusion_depth, const kbwg_gate *gates, uintptr_t n_gates, uint32_t *order,
                        uint32_t *sweep_end, uint64_t *tile_mask, uintptr_t *n_sweeps) {
    GUARD_BEGIN
    if (!n_sweeps || (n_gates && (!gates || !order || !sweep_end || !tile_mask)))
        return fail(KBWG_EINVAL, "null argument");
    if (precision != KBWG_C64 && precision != KBWG_C128) return fail(KBWG_EINVAL, "bad precision");
    if (num_qubits > kMaxQubits) return fail(KBWG_EQUBITS, "num_qubits > 40");
    Sim tmp;  // the geometry rules of a handle of this size, precision and flags (no device state)
    tmp.n = (uint32_t)num_qubits;
    tmp.prec = precision;
    tmp.flags = flags;
    const uint32_t K = tile_qubits ? tile_qubits : default_tile_k(tmp);
    const int R = (int)tile_register_bits(tmp, K);
    if (R == 0) return fail(KBWG_EINVAL, "no sweep kernel of that tile size for this arithmetic");
    if (fusion_depth > (uint32_t)kMaxSweepGates) return fail(KBWG_EINVAL, "fusion depth must be 0..256");
    if (num_qubits < (uintptr_t)K) return fail(KBWG_EQUBITS, "num_qubits below the tile size");
    std::vector<GateDesc> gd(n_gates);
    for (uintptr_t i = 0; i < n_gates; i++) {
        const kbwg_gate &g = gates[i];
        if (g.kind > KBWG_RZ || g.target >= num_qubits || (g.control_mask >> num_qubits) ||
            (g.control_mask & (1ull << g.target)))
            return fail(KBWG_EINVAL, "bad gate");
        gd[i] = make_gate_desc(precision, g.kind, g.target, g.control_mask, g.angle);
    }
    std::vector<PlannedSweep> plan =
        plan_sweeps((uint32_t)num_qubits, (int)K, R, gd.data(), gd.size(), (flags & KBWG_FLAG_EXACT_ORDER) != 0,
                    fusion_depth ? fusion_depth : (size_t)kMaxSweepGates);
    uintptr_t pos = 0;
    for (size_t k = 0; k < plan.size(); k++) {
        for (uint32_t i : plan[k].src) order[pos++] = i;
        sweep_end[k] = (uint32_t)pos;
        tile_mask[k] = ((1ull << plan[k].l) - 1) | plan[k].hmask;
    }
    *n_sweeps = plan.size();
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_jit_check(uintptr_t num_qubits, int32_t precision, uint32_t flags, uint32_t tile_qubits,
                       uint32_t fusion_depth, const kbwg_gate *gates, uintptr_t n_gates, uintptr_t *n_sweeps,
                       uintptr_t *n_failed) {
    GUARD_BEGIN
    if (!n_sweeps || !n_failed || (n_gates && !gates)) return fail(KBWG_EINVAL, "null argument");
    if (precision != KBWG_C64 && precision != KBWG_C128) return fail(KBWG_EINVAL, "bad precision");
    if (num_qubits > kMaxQubits) return fail(KBWG_EQUBITS, "num_qubits > 40");
    if (!jit_available()) return fail(KBWG_EUNSUPPORTED, "NVRTC (libnvrtc.so.13) not found");
    Sim tmp;  // the rules of a handle of this size, precision and flags (no device state)
    tmp.n = (uint32_t)num_qubits;
    tmp.prec = precision;
    tmp.flags = flags;
    if (tile_qubits) {
        const std::vector<uint32_t> ks = tile_options(tmp);
        if (std::find(ks.begin(), ks.end(), tile_qubits) == ks.end())
            return fail(KBWG_EINVAL, "no sweep kernel of that tile size for this arithmetic");
    }
    if (fusion_depth > (uint32_t)kMaxSweepGates) return fail(KBWG_EINVAL, "fusion depth must be 0..256");
    tmp.tile_k = tile_qubits;
    tmp.fusion_depth = fusion_depth;
    std::vector<GateDesc> gd(n_gates);
    for (uintptr_t i = 0; i < n_gates; i++) {
        const kbwg_gate &g = gates[i];
        if (g.kind > KBWG_RZ || g.target >= num_qubits || (g.control_mask >> num_qubits) ||
            (g.control_mask & (1ull << g.target)))
            return fail(KBWG_EINVAL, "bad gate");
        gd[i] = make_gate_desc(precision, g.kind, g.target, g.control_mask, g.angle);
    }
    size_t sweeps = 0;
    *n_failed = jit_check(tmp, gd.data(), gd.size(), sweeps);
    *n_sweeps = sweeps;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_jit_check_adjoint(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                               uintptr_t n_gates, uintptr_t *n_sweeps, uintptr_t *n_failed) {
    GUARD_BEGIN
    if (!n_sweeps || !n_failed || (n_gates && !gates)) return fail(KBWG_EINVAL, "null argument");
    if (precision != KBWG_C64 && precision != KBWG_C128) return fail(KBWG_EINVAL, "bad precision");
    if (num_qubits > kMaxQubits) return fail(KBWG_EQUBITS, "num_qubits > 40");
    if (!jit_available()) return fail(KBWG_EUNSUPPORTED, "NVRTC (libnvrtc.so.13) not found");
    Sim tmp;
    tmp.n = (uint32_t)num_qubits;
    tmp.prec = precision;
    tmp.flags = flags;
    std::vector<GateDesc> gd(n_gates);
    std::vector<int> gtype(n_gates, GT_NONE);
    for (uintptr_t i = 0; i < n_gates; i++) {
        const kbwg_gate &g = gates[i];
        if (g.kind > KBWG_RZ || g.target >= num_qubits || (g.control_mask >> num_qubits) ||
            (g.control_mask & (1ull << g.target)))
            return fail(KBWG_EINVAL, "bad gate");
        gd[i] = make_gate_desc(precision, g.kind, g.target, g.control_mask, g.angle);
        switch (g.kind) {
        case KBWG_RX: gtype[i] = GT_X; break;
        case KBWG_RY: gtype[i] = GT_Y; break;
        case KBWG_RZ: gtype[i] = GT_Z; break;
        case KBWG_P: gtype[i] = GT_P1; break;
        default: break;
        }
    }
    size_t sweeps = 0;
    *n_failed = jit_check_adjoint(tmp, gd, gtype, sweeps);
    *n_sweeps = sweeps;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_chacha_block(const uint32_t *key, uint64_t counter, uint64_t stream, uint32_t rounds, uint32_t *out) {
    if (!key || !out || rounds == 0 || (rounds & 1)) return fail(KBWG_EINVAL, "bad ChaCha arguments");
    chacha_block(key, counter, stream, (int)rounds, out);
    return KBWG_OK;
}

int32_t kbwg_draws(uint64_t seed, uintptr_t count, double *out) {
    if (count && !out) return fail(KBWG_EINVAL, "null output");
    StdRng r = StdRng::seed_from_u64(seed);
    for (uintptr_t i = 0; i < count; i++) out[i] = r.uniform01();
    return KBWG_OK;
}

int32_t kbwg_select_device(int32_t device) {
    CUDA_TRY(cudaSetDevice(device));
    return KBWG_OK;
}

int32_t kbwg_stream(kbwg_sim *s, void **stream) {
    if (!s || !stream) return fail(KBWG_EINVAL, "null argument");
    *stream = (void *)s->stream;
    return KBWG_OK;
}

int32_t kbwg_profile(kbwg_sim *s, int32_t enable) {
    GUARD_BEGIN
    ENTER(s);
    CUDA_TRY(flush_queue(*s));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->prof.on = enable != 0;
    s->prof.used = 0;
    s->prof.bytes = 0.0;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_profile_read(kbwg_sim *s, uint64_t *launches, double *total_ms, double *bytes) {
    GUARD_BEGIN
    ENTER(s);
    CUDA_TRY(flush_queue(*s));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    double t = 0.0;
    for (size_t i = 0; i + 1 < s->prof.used; i += 2) {
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, s->prof.pool[i], s->prof.pool[i + 1]));
        t += ms;
    }
    if (launches) *launches = s->prof.used / 2;
    if (total_ms) *total_ms = t;
    if (bytes) *bytes = s->prof.bytes;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_state_distance(kbwg_sim *a, kbwg_sim *b, double *relative) {
    GUARD_BEGIN
    if (!a || !b || !relative) return fail(KBWG_EINVAL, "null argument");
    if (a->n != b->n || a->prec != b->prec || a->device != b->device)
        return fail(KBWG_EINVAL, "handles differ in size, precision or device");
    ENTER(a);
    CUDA_TRY(settle(*a));
    CUDA_TRY(settle(*b));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(dispatch(a, [&](auto *tp) {
        using T = std::remove_pointer_t<decltype(tp)>;
        return launch_distance<T>(a->state, b->state, a->n, a->rs, a->stream);
    }));
    CUDA_TRY(copy_async(a->h_result, a->rs.result, 2 * sizeof(double), cudaMemcpyDeviceToHost, a->stream));
    CUDA_TRY(cudaStreamSynchronize(a->stream));
    *relative = a->h_result[1] > 0 ? sqrt(a->h_result[0] / a->h_result[1]) : sqrt(a->h_result[0]);
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_state_fidelity(kbwg_sim *a, kbwg_sim *b, double *fidelity) {
    GUARD_BEGIN
    if (!a || !b || !fidelity) return fail(KBWG_EINVAL, "null argument");
    if (a->n != b->n || a->device != b->device) return fail(KBWG_EINVAL, "handles differ in size or device");
    ENTER(a);
    CUDA_TRY(settle(*a));
    CUDA_TRY(settle(*b));
    CUDA_TRY(cudaStreamSynchronize(b->stream));
    CUDA_TRY(launch_overlap(a->state, a->prec, b->state, b->prec, a->n, a->rs, a->stream));
    CUDA_TRY(copy_async(a->h_result, a->rs.result, 4 * sizeof(double), cudaMemcpyDeviceToHost, a->stream));
    CUDA_TRY(cudaStreamSynchronize(a->stream));
    const double *r = a->h_result;
    const double den = r[2] * r[3];
    *fidelity = den > 0.0 ? (r[0] * r[0] + r[1] * r[1]) / den : 0.0;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_transfer_bytes(uint64_t *h2d, uint64_t *d2h) {
    if (h2d) *h2d = g_h2d_bytes.load();
    if (d2h) *d2h = g_d2h_bytes.load();
    return KBWG_OK;
}

int32_t kbwg_wait_probe(kbwg_sim *s, uint32_t spins) {
    GUARD_BEGIN
    ENTER(s);
    if (spins == 0 || spins > (1u << 22)) return fail(KBWG_EINVAL, "spins must be 1..2^22");
    CUDA_TRY(flush_queue(*s));
    CUDA_TRY(launch_wait_probe(s->d_err, spins, s->stream));
    return check_device_error(s);
    GUARD_END
}

int32_t kbwg_last_flush_stats(kbwg_sim *s, uint64_t *gates, uint64_t *passes) {
    if (!s) return fail(KBWG_EINVAL, "null handle");
    if (gates) *gates = s->last_gates;
    if (passes) *passes = s->last_passes;
    return KBWG_OK;
}

// ---- whole-circuit batch entries ------------------------------------------------
// BatchExecution gives every call a fresh simulator (src/quantum_execution.rs:
// 367-418).  Here a call checks a register of the right size out of a small
// per-process pool, resets it to |0...0> (and its draw generator to KBW_SEED,
// as a fresh QubitManager would seed it), runs the whole gate list as one
// flush and returns the register to the pool.  Repeated calls then skip the
// state allocation, and circuits of a repeated structure (variational loops)
// replay their planned sweeps from the register's CUDA-graph cache.
namespace {
struct PoolEntry {
    int device = 0;
    uintptr_t n = 0;
    int32_t prec = 0;
    uint32_t flags = 0;
    kbwg_sim *sim = nullptr;
    bool busy = false;
    uint64_t last = 0;
};
std::mutex g_pool_mu;
std::vector<PoolEntry> g_pool;
uint64_t g_pool_clock = 0;
constexpr size_t kPoolEntries = 4;

// A fresh QubitManager's generator: StdRng::seed_from_u64(KBW_SEED), or a
// random seed when KBW_SEED is not a u64 (src/quantum_execution.rs:181-191).
void reseed_from_env(Sim &s) { s.rng = StdRng::seed_from_u64(kbw_seed_from_env()); }
}  // namespace

// A reset register for (current device, n, precision, flags); *pooled says
// whether pool_put must hand it back (false: the pool was full of busy ones).
static int32_t pool_get(uintptr_t n, int32_t prec, uint32_t flags, kbwg_sim **out, bool *pooled) {
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    kbwg_sim *s = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        for (PoolEntry &p : g_pool)
            if (!p.busy && p.device == dev && p.n == n && p.prec == prec && p.flags == flags) {
                p.busy = true;
                p.last = ++g_pool_clock;
                s = p.sim;
                break;
            }
    }
    *pooled = s != nullptr;
    if (s) {
        *out = s;  // handed back by the caller's lease even if the reset fails
        const int32_t rc = kbwg_clear(s);
        if (rc != KBWG_OK) return rc;
    } else {
        kbwg_sim *victim = nullptr;
        const int32_t rc = kbwg_new(n, prec, flags, &s);
        if (rc != KBWG_OK) return rc;
        {
            std::lock_guard<std::mutex> lk(g_pool_mu);
            if (g_pool.size() >= kPoolEntries) {  // evict the least recently used idle register
                size_t lru = g_pool.size();
                for (size_t i = 0; i < g_pool.size(); i++)
                    if (!g_pool[i].busy && (lru == g_pool.size() || g_pool[i].last < g_pool[lru].last)) lru = i;
                if (lru < g_pool.size()) {
                    victim = g_pool[lru].sim;
                    g_pool.erase(g_pool.begin() + (long)lru);
                }
            }
            if (g_pool.size() < kPoolEntries) {
                PoolEntry p;
                p.device = dev;
                p.n = n;
                p.prec = prec;
                p.flags = flags;
                p.sim = s;
                p.busy = true;
                p.last = ++g_pool_clock;
                g_pool.push_back(p);
                *pooled = true;
            }
        }
        if (victim) kbwg_free(victim);
        *out = s;
    }
    reseed_from_env(*s);
    return KBWG_OK;
}

static void pool_put(kbwg_sim *s, bool pooled) {
    if (!pooled) {
        kbwg_free(s);
        return;
    }
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (PoolEntry &p : g_pool)
        if (p.sim == s) p.busy = false;
}

struct PoolLease {
    kbwg_sim *sim = nullptr;
    bool pooled = false;
    ~PoolLease() {
        if (sim) pool_put(sim, pooled);
    }
};

int32_t kbwg_batch_exp_value(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                             uintptr_t n_gates, const uint8_t *paulis, const uintptr_t *qubits,
                             const uintptr_t *offsets, const double *coefficients, const uintptr_t *ham_offsets,
                             uintptr_t n_hamiltonians, double *out) {
    GUARD_BEGIN
    if (n_hamiltonians && (!ham_offsets || !out)) return fail(KBWG_EINVAL, "null argument");
    for (uintptr_t k = 0; k < n_hamiltonians; k++)
        if (ham_offsets[k + 1] < ham_offsets[k]) return fail(KBWG_EINVAL, "ham_offsets must not decrease");
    PoolLease L;
    int32_t rc = pool_get(num_qubits, precision, flags, &L.sim, &L.pooled);
    if (rc != KBWG_OK) return rc;
    rc = kbwg_apply_gates(L.sim, gates, n_gates);
    for (uintptr_t k = 0; rc == KBWG_OK && k < n_hamiltonians; k++) {
        const uintptr_t a = ham_offsets[k];
        rc = kbwg_exp_value(L.sim, paulis, qubits, offsets ? offsets + a : nullptr,
                            coefficients ? coefficients + a : nullptr, ham_offsets[k + 1] - a, &out[k]);
    }
    if (rc == KBWG_OK && !n_hamiltonians) rc = kbwg_flush(L.sim);
    return rc;
    GUARD_END
}

int32_t kbwg_batch_sample(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                          uintptr_t n_gates, const uintptr_t *qubits, uintptr_t n_qubits, uintptr_t shots,
                          const double *draws, uint64_t *states, uint64_t *counts, uintptr_t capacity,
                          uintptr_t *n_out) {
    GUARD_BEGIN
    if (n_qubits == 0) return fail(KBWG_EINVAL, "no qubits to sample (do_sample asserts a non-empty list)");
    PoolLease L;
    int32_t rc = pool_get(num_qubits, precision, flags, &L.sim, &L.pooled);
    if (rc != KBWG_OK) return rc;
    rc = kbwg_apply_gates(L.sim, gates, n_gates);
    if (rc == KBWG_OK) rc = kbwg_sample(L.sim, qubits, n_qubits, shots, draws, states, counts, capacity, n_out);
    return rc;
    GUARD_END
}

int32_t kbwg_batch_gradient(uintptr_t num_qubits, int32_t precision, uint32_t flags, const kbwg_gate *gates,
                            uintptr_t n_gates, const int32_t *param_index, uintptr_t n_params,
                            const uint8_t *paulis, const uintptr_t *qubits, const uintptr_t *offsets,
                            const double *coefficients, uintptr_t n_strings, uint32_t max_checkpoints,
                            double *energy, double *gradient) {
    GUARD_BEGIN
    PoolLease L;
    int32_t rc = pool_get(num_qubits, precision, flags, &L.sim, &L.pooled);
    if (rc != KBWG_OK) return rc;
    return kbwg_adjoint_gradient(L.sim, gates, n_gates, param_index, n_params, paulis, qubits, offsets,
                                 coefficients, n_strings, max_checkpoints, energy, gradient);
    GUARD_END
}

int32_t kbwg_batch_circuits_exp_value(uintptr_t n_circuits, int32_t precision, uint32_t flags,
                                      const uint32_t *num_qubits, const kbwg_gate *gates,
                                      const uintptr_t *gate_offsets, const uint8_t *paulis, const uintptr_t *qubits,
                                      const uintptr_t *term_offsets, const double *coefficients,
                                      const uintptr_t *ham_offsets, double *energies) {
    GUARD_BEGIN
    if (n_circuits == 0) return KBWG_OK;
    if (!num_qubits || !gate_offsets || !ham_offsets || !energies) return fail(KBWG_EINVAL, "null argument");
    if (precision != KBWG_C64 && precision != KBWG_C128) return fail(KBWG_EINVAL, "bad precision");
    if (gate_offsets[n_circuits] > gate_offsets[0] && !gates) return fail(KBWG_EINVAL, "null gate list");
    const uintptr_t nstr = ham_offsets[n_circuits];
    if (nstr > ham_offsets[0] && (!term_offsets || !coefficients)) return fail(KBWG_EINVAL, "null Hamiltonian arrays");
    if (nstr > ham_offsets[0] && term_offsets[nstr] > term_offsets[0] && (!paulis || !qubits))
        return fail(KBWG_EINVAL, "null Pauli arrays");
    return batch_circuits(precision, flags, n_circuits, num_qubits, gates, gate_offsets, paulis, qubits,
                          term_offsets, coefficients, ham_offsets, energies);
    GUARD_END
}

int32_t kbwg_batch_release(void) {
    GUARD_BEGIN
    std::vector<kbwg_sim *> idle;
    {
        std::lock_guard<std::mutex> lk(g_pool_mu);
        for (size_t i = g_pool.size(); i-- > 0;)
            if (!g_pool[i].busy) {
                idle.push_back(g_pool[i].sim);
                g_pool.erase(g_pool.begin() + (long)i);
            }
    }
    for (kbwg_sim *s : idle) kbwg_free(s);
    return KBWG_OK;
    GUARD_END
}

static void fill_tuning(const Sim &s, kbwg_tuning *out) {
    out->tile_qubits = effective_tile_k(s);
    out->fusion_depth = s.fusion_depth ? s.fusion_depth : (uint32_t)kMaxSweepGates;
    out->source = s.tune_source;
    out->candidates = s.tune_candidates;
    out->ms_per_run = s.tune_ms;
    out->default_ms_per_run = s.tune_default_ms;
}

int32_t kbwg_tile_options(kbwg_sim *s, uint32_t *tile_qubits, uintptr_t capacity, uintptr_t *n) {
    GUARD_BEGIN
    if (!s || !n) return fail(KBWG_EINVAL, "null argument");
    const std::vector<uint32_t> ks = tile_options(*s);
    *n = ks.size();
    if (capacity < ks.size()) return fail(KBWG_ECAPACITY, "tile option buffer too small");
    if (!ks.empty() && !tile_qubits) return fail(KBWG_EINVAL, "null argument");
    for (size_t i = 0; i < ks.size(); i++) tile_qubits[i] = ks[i];
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_set_tuning(kbwg_sim *s, uint32_t tile_qubits, uint32_t fusion_depth) {
    GUARD_BEGIN
    if (!s) return fail(KBWG_EINVAL, "null handle");
    if (tile_qubits) {
        const std::vector<uint32_t> ks = tile_options(*s);
        if (std::find(ks.begin(), ks.end(), tile_qubits) == ks.end())
            return fail(KBWG_EINVAL, "no sweep kernel of that tile size for this handle");
    }
    if (fusion_depth > (uint32_t)kMaxSweepGates) return fail(KBWG_EINVAL, "fusion depth must be 0..256");
    s->tile_k = tile_qubits;
    s->fusion_depth = fusion_depth;
    s->tune_source = (tile_qubits || fusion_depth) ? KBWG_TUNE_SET : KBWG_TUNE_DEFAULT;
    s->tune_candidates = 0;
    s->tune_ms = s->tune_default_ms = 0.0;
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_get_tuning(kbwg_sim *s, kbwg_tuning *out) {
    if (!s || !out) return fail(KBWG_EINVAL, "null argument");
    fill_tuning(*s, out);
    return KBWG_OK;
}

int32_t kbwg_autotune(kbwg_sim *s, const kbwg_gate *gates, uintptr_t n_gates, uint32_t reps, kbwg_tuning *out) {
    GUARD_BEGIN
    ENTER(s);
    if (n_gates && !gates) return fail(KBWG_EINVAL, "null gate list");
    const uint64_t all = (s->n >= 64) ? ~0ull : ((1ull << s->n) - 1);
    std::vector<GateDesc> gd(n_gates);
    for (uintptr_t i = 0; i < n_gates; i++) {
        const kbwg_gate &g = gates[i];
        if (g.kind > KBWG_RZ || g.target >= s->n || (g.control_mask & ~all) || (g.control_mask & (1ull << g.target)))
            return fail(KBWG_EINVAL, "bad gate");
        gd[i] = make_gate_desc(s->prec, g.kind, g.target, g.control_mask, g.angle);
    }
    if (!env_tuning_set()) {
        TuneResult r;
        std::string msg;
        const int32_t rc = autotune(*s, gd, reps, r, msg);
        if (rc != KBWG_OK) return fail(rc, msg.c_str());
        if (r.candidates || r.cached) {
            s->tune_source = r.cached ? KBWG_TUNE_CACHED : KBWG_TUNE_TIMED;
            s->tune_candidates = r.candidates;
            s->tune_ms = r.ms;
            s->tune_default_ms = r.default_ms;
        }
    }
    if (out) fill_tuning(*s, out);
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_set_jit(kbwg_sim *s, int32_t mode) {
    if (!s) return fail(KBWG_EINVAL, "null handle");
    if (mode < KBWG_JIT_OFF || mode > KBWG_JIT_ALWAYS) return fail(KBWG_EINVAL, "bad JIT mode");
    s->jit_mode = mode;
    return KBWG_OK;
}

int32_t kbwg_jit_wait(kbwg_sim *s) {
    GUARD_BEGIN
    if (!s) return fail(KBWG_EINVAL, "null handle");
    wait_specialised(*s);
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_jit_shutdown(void) {
    GUARD_BEGIN
    jit_shutdown();
    return KBWG_OK;
    GUARD_END
}

int32_t kbwg_jit_info(kbwg_sim *s, kbwg_jit_stats *out) {
    GUARD_BEGIN
    if (!out) return fail(KBWG_EINVAL, "null argument");
    const JitStats st = jit_stats();
    out->mode = s ? s->jit_mode : 0;
    out->available = jit_available() ? 1 : 0;
    out->last_specialised = s ? s->last_specialised : 0;
    out->compiled = st.compiled;
    out->reused = st.reused;
    out->failed = st.failed;
    out->compile_seconds = st.compile_s;
    return KBWG_OK;
    GUARD_END
}

const char *kbwg_jit_last_error(void) {
    static thread_local std::string msg;
    msg = jit_last_error();
    return msg.c_str();
}

const char *kbwg_last_error(void) { return g_last_error.c_str(); }

uint64_t kbwg_launch_count(void) { return g_launches.load(); }

}  // extern "C"
