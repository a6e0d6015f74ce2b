// Shared device/host definitions of the GB300 dense state-vector engine.
#pragma once

#include <stdint.h>

// Host-only parts are left out when NVRTC compiles the run-time-generated
// sweep kernels (jit.cpp), which see only the device definitions.
#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <string>
#include <utility>
#include <vector>
#endif

namespace kbwg {

// Interleaved complex amplitude (AoS re,im), 8 B for c64 and 16 B for c128,
// aligned so one amplitude is one vector load.
template <class T>
struct alignas(2 * sizeof(T)) cx {
    T re, im;
};

#if !defined(__CUDACC_RTC__)
// Kernel launch counter (all handles, this process).
extern std::atomic<uint64_t> g_launches;
inline void count_launch(uint64_t n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Host<->device copy accounting (all handles, this process).
extern std::atomic<uint64_t> g_h2d_bytes, g_d2h_bytes;
inline cudaError_t copy_async(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
    if (kind == cudaMemcpyHostToDevice) g_h2d_bytes.fetch_add(bytes, std::memory_order_relaxed);
    if (kind == cudaMemcpyDeviceToHost) g_d2h_bytes.fetch_add(bytes, std::memory_order_relaxed);
    return cudaMemcpyAsync(dst, src, bytes, kind, s);
}

// Raise a kernel's dynamic shared-memory limit once per device (the setting
// belongs to the device's context), safely from any host thread.
inline cudaError_t ensure_smem_limit(const void *func, size_t bytes) {
    static std::mutex mu;
    static std::vector<std::pair<int, const void *>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(mu);
    for (const auto &d : done)
        if (d.first == dev && d.second == func) return cudaSuccess;
    e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) done.emplace_back(dev, func);
    return e;
}

// Number of SMs of the current device.
inline cudaError_t current_sm_count(int &sms) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return e;
}

#endif  // !__CUDACC_RTC__

// One gate as the kernels see it.  Constants are pre-computed on the host in
// the state precision F exactly as the reference does (cos/sin of F(theta/2),
// Complex::exp of F(angle)) and stored widened to double, which is exact.
struct GateDesc {
    uint32_t kind;   // KBWG_X .. KBWG_RZ
    uint32_t target; // qubit (global index) or, inside a tile, a local slot
    uint64_t ctrl;   // control mask on the global basis index
    double c[4];     // see make_gate_desc
};

enum { G_X = 0, G_Y = 1, G_Z = 2, G_H = 3, G_P = 4, G_RX = 5, G_RY = 6, G_RZ = 7 };
// Internal kinds of the complex128 float-float path (never seen at the ABI):
// H without its 1/sqrt(2), |1> times i^q (c[0] = q), multiply every amplitude by c[0] + i c[1].
enum { G_HN = 8, G_PI = 9, G_SCALE = 10 };

#if defined(__CUDACC__)
// ---- rounding-exact arithmetic -------------------------------------------
// The reference evaluates every product and sum separately in F.  These
// wrappers stop the compiler from contracting a*b+c into one FMA so that the
// device results equal the reference's bit for bit.
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }

// Sign flip on the integer pipe (no FP64 instruction for c128).
__device__ __forceinline__ float xneg(float a) { return __int_as_float(__float_as_int(a) ^ 0x80000000); }
__device__ __forceinline__ double xneg(double a) {
    return __longlong_as_double(__double_as_longlong(a) ^ 0x8000000000000000ull);
}

template <class T>
__device__ __forceinline__ cx<T> cmul_exact(cx<T> a, T br, T bi) {
    // num-complex Mul: (a.re*b.re - a.im*b.im, a.re*b.im + a.im*b.re)
    cx<T> r;
    r.re = xsub(xmul(a.re, br), xmul(a.im, bi));
    r.im = xadd(xmul(a.re, bi), xmul(a.im, br));
    return r;
}

// Gate constants in T.
template <class T>
struct GateK {
    T c0, c1, c2, c3;
};

template <class T>
__device__ __forceinline__ GateK<T> load_k(const GateDesc &g) {
    GateK<T> k;
    k.c0 = (T)g.c[0];
    k.c1 = (T)g.c[1];
    k.c2 = (T)g.c[2];
    k.c3 = (T)g.c[3];
    return k;
}

// Apply one gate to the amplitude pair (a0: target bit 0, a1: target bit 1),
// reproducing kbw Dense<F> per-amplitude formulas (src/dense.rs:91-334):
//   Y : a0' = a1*(-i), a1' = a0*i
//   H : a0' = (a0 + a1)*h, a1' = (a0 - a1)*h        (c0 = h = FRAC_1_SQRT_2)
//   P : a1' = a1*(c0 + i c1)                          (c0,c1 = cos, sin of F(l))
//   RX: a0' = (c a0.re + s a1.im, c a0.im - s a1.re), a1' symmetric (c0=c, c1=s)
//   RY: a0' = c a0 - s a1, a1' = c a1 + s a0
//   RZ: a0' = a0*(c0 + i c1), a1' = a1*(c2 + i c3)
template <class T>
__device__ __forceinline__ void apply_pair(uint32_t kind, const GateK<T> &k, cx<T> &a0, cx<T> &a1) {
    switch (kind) {
    case G_X: {
        cx<T> t = a0;
        a0 = a1;
        a1 = t;
        break;
    }
    case G_Y: {
        cx<T> n0, n1;
        n0.re = a1.im;
        n0.im = xneg(a1.re);
        n1.re = xneg(a0.im);
        n1.im = a0.re;
        a0 = n0;
        a1 = n1;
        break;
    }
    case G_Z:
        a1.re = xneg(a1.re);
        a1.im = xneg(a1.im);
        break;
    case G_H: {
        cx<T> n0, n1;
        n0.re = xmul(xadd(a0.re, a1.re), k.c0);
        n0.im = xmul(xadd(a0.im, a1.im), k.c0);
        n1.re = xmul(xsub(a0.re, a1.re), k.c0);
        n1.im = xmul(xsub(a0.im, a1.im), k.c0);
        a0 = n0;
        a1 = n1;
        break;
    }
    case G_P:
        a1 = cmul_exact(a1, k.c0, k.c1);
        break;
    case G_RX: {
        cx<T> n0, n1;
        n0.re = xadd(xmul(k.c0, a0.re), xmul(k.c1, a1.im));
        n0.im = xsub(xmul(k.c0, a0.im), xmul(k.c1, a1.re));
        n1.re = xadd(xmul(k.c0, a1.re), xmul(k.c1, a0.im));
        n1.im = xsub(xmul(k.c0, a1.im), xmul(k.c1, a0.re));
        a0 = n0;
        a1 = n1;
        break;
    }
    case G_RY: {
        cx<T> n0, n1;
        n0.re = xsub(xmul(k.c0, a0.re), xmul(k.c1, a1.re));
        n0.im = xsub(xmul(k.c0, a0.im), xmul(k.c1, a1.im));
        n1.re = xadd(xmul(k.c0, a1.re), xmul(k.c1, a0.re));
        n1.im = xadd(xmul(k.c0, a1.im), xmul(k.c1, a0.im));
        a0 = n0;
        a1 = n1;
        break;
    }
    case G_RZ:
        a0 = cmul_exact(a0, k.c0, k.c1);
        a1 = cmul_exact(a1, k.c2, k.c3);
        break;
    default:
        break;
    }
}

#endif  // __CUDACC__

// Diagonal gates: each amplitude only picks up a phase.
__host__ __device__ __forceinline__ bool is_diag_kind(uint32_t kind) {
    return kind == G_Z || kind == G_P || kind == G_RZ || kind == G_PI || kind == G_SCALE;
}

// Gates that only change the |1> amplitude of the pair.
__host__ __device__ __forceinline__ bool touches_only_one(uint32_t kind) {
    return kind == G_Z || kind == G_P;
}

#if !defined(__CUDACC_RTC__)
// ---- host-side error plumbing ----------------------------------------------
struct Status {
    int32_t code = 0;
    std::string msg;
};

void set_error(int32_t code, const std::string &msg);
#endif  // !__CUDACC_RTC__

}  // namespace kbwg
