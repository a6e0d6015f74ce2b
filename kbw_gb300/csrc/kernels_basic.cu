// Unfused kernels: one gate per pass, state initialisation and the
// qubit-exchange permutation.  The fused tile sweeps live in sweep.cu.
#include "common.cuh"
#include "ff.cuh"
#include "kernels.h"

namespace kbwg {

// One gate over all 2^(n-1) amplitude pairs (the reference's one-trait-call
// per-sweep semantics, src/dense.rs:91-334).  Pairs whose controls are not
// all set are skipped without being read or written.  Z and P read and write
// only the |1> amplitude of each pair.
template <class T>
__global__ void __launch_bounds__(256) k_gate1(cx<T> *__restrict__ st, uint64_t npairs, GateDesc g) {
    const uint32_t t = g.target;
    const uint64_t bit = 1ull << t, low = bit - 1;
    const GateK<T> k = load_k<T>(g);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < npairs; p += stride) {
        const uint64_t s0 = ((p & ~low) << 1) | (p & low);
        if ((s0 & g.ctrl) != g.ctrl) continue;
        const uint64_t s1 = s0 | bit;
        if (touches_only_one(g.kind)) {
            cx<T> a0{}, a1 = st[s1];
            apply_pair<T>(g.kind, k, a0, a1);
            st[s1] = a1;
        } else {
            cx<T> a0 = st[s0], a1 = st[s1];
            apply_pair<T>(g.kind, k, a0, a1);
            st[s0] = a0;
            st[s1] = a1;
        }
    }
}

template <class T>
__global__ void __launch_bounds__(256) k_init_zero_state(cx<T> *__restrict__ st, uint64_t ns) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        cx<T> v;
        v.re = (s == 0) ? (T)1 : (T)0;
        v.im = (T)0;
        st[s] = v;
    }
}

// |0...0> in float-float form: amplitude 0 is (re.hi 1, 0, 0, 0); zero
// amplitudes have the same all-zero bytes in both formats.
__global__ void __launch_bounds__(256) k_init_zero_state_ff(float4 *__restrict__ st, uint64_t ns) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride)
        st[s] = make_float4(s == 0 ? 1.f : 0.f, 0.f, 0.f, 0.f);
}

// binary64 <-> float-float, in place (each thread rewrites its own 16 bytes).
// Float-float layout per amplitude: re.hi, im.hi, re.lo, im.lo.
__global__ void __launch_bounds__(256) k_ff_convert(cx<double> *__restrict__ st, uint64_t ns, int to_ff) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        if (to_ff) {
            const cx<double> a = st[s];
            const ff::f2 re = ff::from_double(a.re), im = ff::from_double(a.im);
            reinterpret_cast<float4 *>(st)[s] = make_float4(re.h, im.h, re.l, im.l);
        } else {
            const float4 f = reinterpret_cast<const float4 *>(st)[s];
            st[s] = cx<double>{ff::to_double(ff::f2{f.x, f.z}), ff::to_double(ff::f2{f.y, f.w})};
        }
    }
}

// In-place exchange of physical qubits a < b: amplitudes with (bit a, bit b)
// = (1, 0) and (0, 1) trade places; the others stay.  One thread per swapped
// pair; 2^(n-2) pairs.
template <class T>
__global__ void __launch_bounds__(256) k_swap_qubits(cx<T> *__restrict__ st, uint64_t nquads, uint32_t a,
                                                     uint32_t b) {
    const uint64_t ba = 1ull << a, bb = 1ull << b;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nquads; i += stride) {
        // insert zero bits at a then b (a < b)
        uint64_t s = ((i & ~(ba - 1)) << 1) | (i & (ba - 1));
        s = ((s & ~(bb - 1)) << 1) | (s & (bb - 1));
        const uint64_t s10 = s | ba, s01 = s | bb;
        const cx<T> x = st[s10], y = st[s01];
        st[s10] = y;
        st[s01] = x;
    }
}

static unsigned grid_for(uint64_t work, unsigned block, unsigned max_blocks) {
    uint64_t g = (work + block - 1) / block;
    if (g > max_blocks) g = max_blocks;
    if (g == 0) g = 1;
    return (unsigned)g;
}

template <class T>
cudaError_t launch_gate1(void *st, uint32_t n, const GateDesc &g, cudaStream_t s) {
    const uint64_t npairs = n ? (1ull << (n - 1)) : 0;
    if (npairs == 0) return cudaSuccess;
    k_gate1<T><<<grid_for(npairs, 256, 152 * 16), 256, 0, s>>>((cx<T> *)st, npairs, g);
    count_launch();
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_init(void *st, uint32_t n, cudaStream_t s) {
    const uint64_t ns = 1ull << n;
    k_init_zero_state<T><<<grid_for(ns, 256, 152 * 16), 256, 0, s>>>((cx<T> *)st, ns);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_init_ff(void *st, uint32_t n, cudaStream_t s) {
    const uint64_t ns = 1ull << n;
    k_init_zero_state_ff<<<grid_for(ns, 256, 152 * 16), 256, 0, s>>>((float4 *)st, ns);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_ff_convert(void *st, uint32_t n, bool to_ff, cudaStream_t s) {
    const uint64_t ns = 1ull << n;
    k_ff_convert<<<grid_for(ns, 256, 152 * 16), 256, 0, s>>>((cx<double> *)st, ns, to_ff ? 1 : 0);
    count_launch();
    return cudaGetLastError();
}


template <class T>
cudaError_t launch_swap(void *st, uint32_t n, uint32_t a, uint32_t b, cudaStream_t s) {
    if (a == b || n < 2) return cudaSuccess;
    if (a > b) {
        uint32_t t = a;
        a = b;
        b = t;
    }
    const uint64_t nq = 1ull << (n - 2);
    k_swap_qubits<T><<<grid_for(nq, 256, 152 * 16), 256, 0, s>>>((cx<T> *)st, nq, a, b);
    count_launch();
    return cudaGetLastError();
}

template cudaError_t launch_gate1<float>(void *, uint32_t, const GateDesc &, cudaStream_t);
template cudaError_t launch_gate1<double>(void *, uint32_t, const GateDesc &, cudaStream_t);
template cudaError_t launch_init<float>(void *, uint32_t, cudaStream_t);
template cudaError_t launch_init<double>(void *, uint32_t, cudaStream_t);
template cudaError_t launch_swap<float>(void *, uint32_t, uint32_t, uint32_t, cudaStream_t);
template cudaError_t launch_swap<double>(void *, uint32_t, uint32_t, uint32_t, cudaStream_t);

}  // namespace kbwg
