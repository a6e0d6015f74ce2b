// Reductions over the state: probabilities, sequential measurement,
// collapse, Pauli-string expectation values, dump compaction and sampling.
//
// Every reduction runs on a fixed grid and finishes in the last block to
// arrive (ticket counter, no spin-wait), so results are deterministic run to
// run.  Accumulation is FP64-grade: native double for complex128 data and
// float-float (error-free products and sums) for complex64 data, widened to
// double per thread before the block tree.
#include <float.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/kbwg.h"
#include "ff.cuh"
#include "kernels.h"

namespace kbwg {

// ---- accumulators ---------------------------------------------------------
struct AccF {  // float-float running sum of products
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add2(float p, float e) {
        const float s = __fadd_rn(hi, p);
        const float bb = __fsub_rn(s, hi);
        float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        err = __fadd_rn(err, __fadd_rn(lo, e));
        hi = __fadd_rn(s, err);
        lo = __fsub_rn(err, __fsub_rn(hi, s));
    }
    __device__ __forceinline__ void add_prod(float a, float b) {
        const float p = __fmul_rn(a, b);
        add2(p, __fmaf_rn(a, b, -p));
    }
    __device__ __forceinline__ void add_prod_neg(float a, float b) {
        const float p = __fmul_rn(a, b);
        add2(-p, -__fmaf_rn(a, b, -p));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
struct AccD {
    double v = 0.0;
    __device__ __forceinline__ void add_prod(double a, double b) { v = __fma_rn(a, b, v); }
    __device__ __forceinline__ void add_prod_neg(double a, double b) { v = __fma_rn(-a, b, v); }
    __device__ __forceinline__ double value() const { return v; }
};
template <class T> struct AccOf;
template <> struct AccOf<float> { using type = AccF; };
template <> struct AccOf<double> { using type = AccD; };

// float-float value (products kept exactly)
struct FF {
    float hi, lo;
};

// ---- block helpers ----------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block; the result is valid in thread 0.
__device__ double block_sum(double v) {
    __shared__ double sh[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (w == 0) {
        r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

// Inclusive scan over the block in a fixed order; also returns the total.
__device__ double block_inclusive_scan(double v, double *total) {
    __shared__ double wsum[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    __syncthreads();
    if (lane == 31) wsum[w] = v;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        double x = (lane < nw) ? wsum[lane] : 0.0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane < nw) wsum[lane] = x;  // inclusive warp prefix
    }
    __syncthreads();
    if (w > 0) v += wsum[w - 1];
    *total = wsum[(blockDim.x >> 5) - 1];
    return v;
}

// True in the last block to finish; partials written before are visible.
__device__ bool last_block(unsigned *ticket) {
    __shared__ bool is_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) is_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
    __syncthreads();
    return is_last;
}

// Deterministic sum of partials[b * stride + k] over b by the whole block.
__device__ double sum_partials(const double *partials, int nblocks, int stride, int k) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v += partials[(size_t)b * stride + k];
    return block_sum(v);
}

__device__ __forceinline__ uint64_t insert_zero(uint64_t i, uint32_t m) {
    const uint64_t low = (1ull << m) - 1;
    return ((i & ~low) << 1) | (i & low);
}

// Insert zero bits at every set position of M (ascending).
__device__ __forceinline__ uint64_t insert_zeros(uint64_t i, uint64_t M) {
    while (M) {
        const uint32_t m = __ffsll((long long)M) - 1;
        M &= M - 1;
        i = insert_zero(i, m);
    }
    return i;
}

// rand's UniformFloat::new(0, total) scale rule (largest draw 1 - 2^-52).
__host__ __device__ inline double uniform_scale(double total) {
    const double max_rand = 1.0 - DBL_EPSILON;
    double scale = total;
#ifdef __CUDA_ARCH__
    while (__dmul_rn(scale, max_rand) >= total) scale = __longlong_as_double(__double_as_longlong(scale) - 1);
#else
    while (scale * max_rand >= total) {
        union {
            double d;
            uint64_t u;
        } x;
        x.d = scale;
        x.u -= 1;
        scale = x.d;
    }
#endif
    return scale;
}

// ---- masked norm / p1 -------------------------------------------------------
template <class T>
__device__ __forceinline__ double masked_norm_body(const cx<T> *__restrict__ st, uint64_t count, uint64_t M,
                                                   uint64_t V) {
    typename AccOf<T>::type acc;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < count; i += 4 * stride) {
        cx<T> a[4];
#pragma unroll
        for (int u = 0; u < 4; u++) a[u] = st[insert_zeros(i + u * stride, M) | V];
#pragma unroll
        for (int u = 0; u < 4; u++) {
            acc.add_prod(a[u].re, a[u].re);
            acc.add_prod(a[u].im, a[u].im);
        }
    }
    for (; i < count; i += stride) {
        const cx<T> a = st[insert_zeros(i, M) | V];
        acc.add_prod(a.re, a.re);
        acc.add_prod(a.im, a.im);
    }
    return block_sum(acc.value());
}

template <class T>
__global__ void __launch_bounds__(kReduceThreads)
    k_masked_norm(const cx<T> *__restrict__ st, uint64_t count, uint64_t M, uint64_t V, ReduceScratch rs) {
    const double v = masked_norm_body<T>(st, count, M, V);
    if (threadIdx.x == 0) rs.partials[blockIdx.x] = v;
    if (last_block(rs.ticket)) {
        const double t = sum_partials(rs.partials, gridDim.x, 1, 0);
        if (threadIdx.x == 0) {
            rs.result[0] = t;
            *rs.ticket = 0;
        }
    }
}

template <class T>
cudaError_t launch_masked_norm(const void *st, uint32_t n, uint64_t M, uint64_t V, const ReduceScratch &rs,
                               cudaStream_t s) {
    const uint64_t count = 1ull << (n - __builtin_popcountll(M));
    k_masked_norm<T><<<kReduceBlocks, kReduceThreads, 0, s>>>((const cx<T> *)st, count, M, V, rs);
    count_launch();
    return cudaGetLastError();
}

// The same over the float-float resident form of a complex128 state
// (re.hi, im.hi, re.lo, im.lo per amplitude): |a|^2 as a float-float dot
// product, summed per thread in float-float (FP32-pipe work), then in binary64.
__device__ __forceinline__ double masked_norm_body_ff(const float4 *__restrict__ st, uint64_t count, uint64_t M,
                                                      uint64_t V) {
    ff::f2 acc{0.f, 0.f};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const float4 f = st[insert_zeros(i, M) | V];
        const ff::f2 re{f.x, f.z}, im{f.y, f.w};
        acc = ff::add(acc, ff::dot2(re, re, im, im));
    }
    return block_sum((double)acc.h + (double)acc.l);
}

__global__ void __launch_bounds__(kReduceThreads)
    k_masked_norm_ff(const float4 *__restrict__ st, uint64_t count, uint64_t M, uint64_t V, ReduceScratch rs) {
    const double v = masked_norm_body_ff(st, count, M, V);
    if (threadIdx.x == 0) rs.partials[blockIdx.x] = v;
    if (last_block(rs.ticket)) {
        const double t = sum_partials(rs.partials, gridDim.x, 1, 0);
        if (threadIdx.x == 0) {
            rs.result[0] = t;
            *rs.ticket = 0;
        }
    }
}

cudaError_t launch_masked_norm_ff(const void *st, uint32_t n, uint64_t M, uint64_t V, const ReduceScratch &rs,
                                  cudaStream_t s) {
    const uint64_t count = 1ull << (n - __builtin_popcountll(M));
    k_masked_norm_ff<<<kReduceBlocks, kReduceThreads, 0, s>>>((const float4 *)st, count, M, V, rs);
    count_launch();
    return cudaGetLastError();
}

// ---- distance between two states ----------------------------------------------
// partials: sum |a - b|^2 and sum |b|^2 (two values per block).
template <class T>
__global__ void __launch_bounds__(kReduceThreads)
    k_distance(const cx<T> *__restrict__ a, const cx<T> *__restrict__ b, uint64_t count, ReduceScratch rs) {
    typename AccOf<T>::type d, nb;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const cx<T> x = a[i], y = b[i];
        const T dr = x.re - y.re, di = x.im - y.im;
        d.add_prod(dr, dr);
        d.add_prod(di, di);
        nb.add_prod(y.re, y.re);
        nb.add_prod(y.im, y.im);
    }
    const double vd = block_sum(d.value());
    const double vn = block_sum(nb.value());
    if (threadIdx.x == 0) {
        rs.partials[2 * blockIdx.x] = vd;
        rs.partials[2 * blockIdx.x + 1] = vn;
    }
    if (last_block(rs.ticket)) {
        const double td = sum_partials(rs.partials, gridDim.x, 2, 0);
        const double tn = sum_partials(rs.partials, gridDim.x, 2, 1);
        if (threadIdx.x == 0) {
            rs.result[0] = td;
            rs.result[1] = tn;
            *rs.ticket = 0;
        }
    }
}

template <class T>
cudaError_t launch_distance(const void *a, const void *b, uint32_t n, const ReduceScratch &rs, cudaStream_t s) {
    k_distance<T><<<kReduceBlocks, kReduceThreads, 0, s>>>((const cx<T> *)a, (const cx<T> *)b, 1ull << n, rs);
    count_launch();
    return cudaGetLastError();
}
template cudaError_t launch_distance<float>(const void *, const void *, uint32_t, const ReduceScratch &, cudaStream_t);
template cudaError_t launch_distance<double>(const void *, const void *, uint32_t, const ReduceScratch &, cudaStream_t);

// partials: Re<a|b>, Im<a|b>, <a|a>, <b|b> (four values per block), either
// precision on either side, accumulated in FP64.
template <class TA, class TB>
__global__ void __launch_bounds__(kReduceThreads)
    k_overlap(const cx<TA> *__restrict__ a, const cx<TB> *__restrict__ b, uint64_t count, ReduceScratch rs) {
    AccD re, im, na, nb;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
        const cx<TA> x = a[i];
        const cx<TB> y = b[i];
        const double ar = x.re, ai = x.im, br = y.re, bi = y.im;
        re.add_prod(ar, br);  // conj(a) b = (ar br + ai bi) + i (ar bi - ai br)
        re.add_prod(ai, bi);
        im.add_prod(ar, bi);
        im.add_prod_neg(ai, br);
        na.add_prod(ar, ar);
        na.add_prod(ai, ai);
        nb.add_prod(br, br);
        nb.add_prod(bi, bi);
    }
    const double v0 = block_sum(re.value());
    const double v1 = block_sum(im.value());
    const double v2 = block_sum(na.value());
    const double v3 = block_sum(nb.value());
    if (threadIdx.x == 0) {
        rs.partials[4 * blockIdx.x] = v0;
        rs.partials[4 * blockIdx.x + 1] = v1;
        rs.partials[4 * blockIdx.x + 2] = v2;
        rs.partials[4 * blockIdx.x + 3] = v3;
    }
    if (last_block(rs.ticket)) {
        double t[4];
        for (int k = 0; k < 4; k++) t[k] = sum_partials(rs.partials, gridDim.x, 4, k);
        if (threadIdx.x == 0) {
            for (int k = 0; k < 4; k++) rs.result[k] = t[k];
            *rs.ticket = 0;
        }
    }
}

cudaError_t launch_overlap(const void *a, int prec_a, const void *b, int prec_b, uint32_t n, const ReduceScratch &rs,
                           cudaStream_t s) {
    const uint64_t count = 1ull << n;
    if (prec_a && prec_b)
        k_overlap<double, double><<<kReduceBlocks, kReduceThreads, 0, s>>>((const cx<double> *)a,
                                                                           (const cx<double> *)b, count, rs);
    else if (prec_a)
        k_overlap<double, float><<<kReduceBlocks, kReduceThreads, 0, s>>>((const cx<double> *)a,
                                                                          (const cx<float> *)b, count, rs);
    else if (prec_b)
        k_overlap<float, double><<<kReduceBlocks, kReduceThreads, 0, s>>>((const cx<float> *)a,
                                                                          (const cx<double> *)b, count, rs);
    else
        k_overlap<float, float><<<kReduceBlocks, kReduceThreads, 0, s>>>((const cx<float> *)a, (const cx<float> *)b,
                                                                         count, rs);
    count_launch();
    return cudaGetLastError();
}

// ---- sequential measurement step ------------------------------------------
template <class T, bool kFF = false>
__global__ void __launch_bounds__(kReduceThreads)
    k_measure_step(const void *__restrict__ st, uint32_t n, MeasureCtl *ctl, uint32_t step, ReduceScratch rs) {
    const uint64_t bit = 1ull << ctl->qubit[step];
    const uint64_t M = ctl->M | bit, V = ctl->V | bit;
    const uint64_t count = 1ull << (n - __popcll(M));
    double v;
    if constexpr (kFF)
        v = masked_norm_body_ff((const float4 *)st, count, M, V);
    else
        v = masked_norm_body<T>((const cx<T> *)st, count, M, V);
    if (threadIdx.x == 0) rs.partials[blockIdx.x] = v;
    if (last_block(rs.ticket)) {
        const double s1 = sum_partials(rs.partials, gridDim.x, 1, 0);
        if (threadIdx.x == 0) {
            // QubitManager::do_measure decision (src/quantum_execution.rs:278-287)
            const double p1 = __dmul_rn(s1, ctl->scale2);
            double p0 = __dsub_rn(1.0, p1);
            if (!(p0 > 0.0)) p0 = 0.0;
            const double total = __dadd_rn(p0, p1);
            const double chosen = __dmul_rn(ctl->draws[step], uniform_scale(total));
            const int r = (p0 <= chosen) ? 1 : 0;
            double prob = r ? p1 : p0;
            if (!(prob > DBL_MIN)) prob = DBL_MIN;
            const double p = 1.0 / sqrt(prob);
            const double pf = (double)(T)p;
            ctl->p[step] = p;
            ctl->scale2 = __dmul_rn(__dmul_rn(ctl->scale2, pf), pf);
            ctl->M = ctl->M | bit;
            ctl->V = ctl->V | (r ? bit : 0ull);
            ctl->result |= (uint64_t)r << step;
            ctl->steps = step + 1;
            *rs.ticket = 0;
        }
    }
}

template <class T>
cudaError_t launch_measure_step(const void *st, uint32_t n, MeasureCtl *ctl, uint32_t step,
                                const ReduceScratch &rs, cudaStream_t s) {
    k_measure_step<T><<<kReduceBlocks, kReduceThreads, 0, s>>>(st, n, ctl, step, rs);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_measure_step_ff(const void *st, uint32_t n, MeasureCtl *ctl, uint32_t step,
                                   const ReduceScratch &rs, cudaStream_t s) {
    k_measure_step<double, true><<<kReduceBlocks, kReduceThreads, 0, s>>>(st, n, ctl, step, rs);
    count_launch();
    return cudaGetLastError();
}

// ---- collapse -----------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256)
    k_collapse(cx<T> *__restrict__ st, uint64_t ns, const MeasureCtl *ctl, uint64_t M, uint64_t V, double p) {
    __shared__ T pf[64];
    __shared__ uint64_t sM, sV;
    __shared__ uint32_t nf;
    if (threadIdx.x == 0) {
        if (ctl) {
            sM = ctl->M;
            sV = ctl->V;
            nf = ctl->steps;
        } else {
            sM = M;
            sV = V;
            nf = 1;
        }
    }
    if (threadIdx.x < 64) pf[threadIdx.x] = ctl ? (T)ctl->p[threadIdx.x] : (T)p;
    __syncthreads();
    const uint64_t m = sM, v = sV;
    const uint32_t k = nf;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        cx<T> a;
        if ((s & m) == v) {
            a = st[s];
            for (uint32_t j = 0; j < k; j++) {  // one multiply per collapse, in order
                a.re = xmul(a.re, pf[j]);
                a.im = xmul(a.im, pf[j]);
            }
        } else {
            a.re = (T)0;
            a.im = (T)0;
        }
        st[s] = a;
    }
}

// The collapse of a float-float resident state: each kept amplitude's parts
// times the binary64 factors 1/sqrt(P) in float-float, one per collapse, in
// order.
__global__ void __launch_bounds__(256)
    k_collapse_ff(float4 *__restrict__ st, uint64_t ns, const MeasureCtl *ctl, uint64_t M, uint64_t V, double p) {
    __shared__ float ph[64], pl[64];
    __shared__ uint64_t sM, sV;
    __shared__ uint32_t nf;
    if (threadIdx.x == 0) {
        if (ctl) {
            sM = ctl->M;
            sV = ctl->V;
            nf = ctl->steps;
        } else {
            sM = M;
            sV = V;
            nf = 1;
        }
    }
    if (threadIdx.x < 64) {
        const ff::f2 f = ff::split_constant(ctl ? ctl->p[threadIdx.x] : p);
        ph[threadIdx.x] = f.h;
        pl[threadIdx.x] = f.l;
    }
    __syncthreads();
    const uint64_t m = sM, v = sV;
    const uint32_t k = nf;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
        if ((s & m) == v) {
            a = st[s];
            ff::f2 re{a.x, a.z}, im{a.y, a.w};
            for (uint32_t j = 0; j < k; j++) {
                const ff::f2 f{ph[j], pl[j]};
                re = ff::mul(re, f);
                im = ff::mul(im, f);
            }
            a = make_float4(re.h, im.h, re.l, im.l);
        }
        st[s] = a;
    }
}

cudaError_t launch_collapse_ff(void *st, uint32_t n, const MeasureCtl *ctl, uint64_t M, uint64_t V, double p,
                               cudaStream_t s) {
    const uint64_t ns = 1ull << n;
    uint64_t g = (ns + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    k_collapse_ff<<<(unsigned)g, 256, 0, s>>>((float4 *)st, ns, ctl, M, V, p);
    count_launch();
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_collapse(void *st, uint32_t n, const MeasureCtl *ctl, uint64_t M, uint64_t V, double p,
                            cudaStream_t s) {
    const uint64_t ns = 1ull << n;
    uint64_t g = (ns + 255) / 256;
    if (g > 152 * 16) g = 152 * 16;
    k_collapse<T><<<(unsigned)g, 256, 0, s>>>((cx<T> *)st, ns, ctl, M, V, p);
    count_launch();
    return cudaGetLastError();
}

// ---- Pauli strings ------------------------------------------------------------
// <psi|P|psi> with P = i^{nY} X^x Z^z (per qubit).  For x == 0 the sum is
// sum_s (-1)^{|s & z|} |a_s|^2.  For x != 0 each pair (s, s^x) with bit h
// (the highest of x) clear contributes +-2 (-1)^{|s & z|} Re or Im of
// conj(a_s) a_{s^x}; the host folds i^{nY} and (-1)^{|x & z|} into `factor`
// and `use_im`.
template <class T>
__global__ void __launch_bounds__(kReduceThreads)
    k_pauli_group(const cx<T> *__restrict__ st, uint32_t n, PauliGroup g, ReduceScratch rs) {
    typename AccOf<T>::type acc[kMaxTerms];
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint32_t nt = g.nterms;
    if (g.x == 0) {
        const uint64_t count = 1ull << n;
        for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < count; s += stride) {
            const cx<T> a = st[s];
#pragma unroll
            for (int k = 0; k < kMaxTerms; k++) {
                if (k < (int)nt) {
                    if ((__popcll(s & g.z[k]) & 1) ^ (g.factor[k] < 0)) {
                        acc[k].add_prod_neg(a.re, a.re);
                        acc[k].add_prod_neg(a.im, a.im);
                    } else {
                        acc[k].add_prod(a.re, a.re);
                        acc[k].add_prod(a.im, a.im);
                    }
                }
            }
        }
    } else {
        const uint32_t h = 63 - __clzll((long long)g.x);
        const uint64_t count = 1ull << (n - 1);
        for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += stride) {
            const uint64_t s = insert_zero(i, h);
            const cx<T> a = st[s], b = st[s ^ g.x];
#pragma unroll
            for (int k = 0; k < kMaxTerms; k++) {
                if (k < (int)nt) {
                    const bool neg = (__popcll(s & g.z[k]) & 1) ^ (g.factor[k] < 0);
                    // Re(conj(a) b) = a.re b.re + a.im b.im ; Im = a.re b.im - a.im b.re
                    if (!g.use_im[k]) {
                        if (neg) {
                            acc[k].add_prod_neg(a.re, b.re);
                            acc[k].add_prod_neg(a.im, b.im);
                        } else {
                            acc[k].add_prod(a.re, b.re);
                            acc[k].add_prod(a.im, b.im);
                        }
                    } else {
                        if (neg) {
                            acc[k].add_prod_neg(a.re, b.im);
                            acc[k].add_prod(a.im, b.re);
                        } else {
                            acc[k].add_prod(a.re, b.im);
                            acc[k].add_prod_neg(a.im, b.re);
                        }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int k = 0; k < kMaxTerms; k++) {
        if (k < (int)nt) {
            const double f = fabs(g.factor[k]);
            const double v = block_sum(acc[k].value() * f);
            if (threadIdx.x == 0) rs.partials[(size_t)blockIdx.x * kMaxTerms + k] = v;
        }
    }
    if (last_block(rs.ticket)) {
        for (int k = 0; k < (int)nt; k++) {
            const double t = sum_partials(rs.partials, gridDim.x, kMaxTerms, k);
            if (threadIdx.x == 0) rs.result[k] = t;
        }
        if (threadIdx.x == 0) *rs.ticket = 0;
    }
}

// Diagonal groups (x == 0) with a Walsh transform.  A warp reads 512
// consecutive amplitudes s = b + lane + 32u (u = 0..15, coalesced), so
// (-1)^{|s & z|} = (-1)^{|(b | lane) & z|} * (-1)^{|u & zu|}, zu = (z >> 5) & 15.
// Each thread forms the 16-point Walsh-Hadamard transform W of its
// probabilities p_u (64 adds) and every term adds +-W[zu]: about 4 + nt/16
// additions per amplitude instead of nt.  Probabilities and sums are
// float-float: error-free products of the complex64 parts, and for complex128
// a float-float dot product of the amplitude split into float-float (binary64
// storage) or read as is (the float-float resident form) -- FP32-pipe work
// instead of GB300's slow FP64 pipe, ~2^-48 relative per operation.
template <class T> struct DiagArith;
template <> struct DiagArith<double> {
    using V = ff::f2;
    static __device__ __forceinline__ V zero() { return V{0.f, 0.f}; }
    static __device__ __forceinline__ V prob(cx<double> a) {
        const ff::f2 re = ff::from_double(a.re), im = ff::from_double(a.im);
        return ff::dot2(re, re, im, im);
    }
    static __device__ __forceinline__ V prob(float4 f) {  // re.hi, im.hi, re.lo, im.lo
        const ff::f2 re{f.x, f.z}, im{f.y, f.w};
        return ff::dot2(re, re, im, im);
    }
    static __device__ __forceinline__ V add(V a, V b) { return ff::add(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return ff::sub(a, b); }
    static __device__ __forceinline__ double to_d(V a) { return (double)a.h + (double)a.l; }
};
template <> struct DiagArith<float> {
    using V = ff::f2;
    static __device__ __forceinline__ V zero() { return V{0.f, 0.f}; }
    static __device__ __forceinline__ V prob(cx<float> a) {
        const float pr = __fmul_rn(a.re, a.re), pi = __fmul_rn(a.im, a.im);
        const ff::f2 s = ff::two_sum(pr, pi);
        const float e = __fadd_rn(__fmaf_rn(a.re, a.re, -pr), __fmaf_rn(a.im, a.im, -pi));
        return ff::fast_two_sum(s.h, __fadd_rn(s.l, e));
    }
    static __device__ __forceinline__ V add(V a, V b) { return ff::add(a, b); }
    static __device__ __forceinline__ V sub(V a, V b) { return ff::sub(a, b); }
    static __device__ __forceinline__ double to_d(V a) { return (double)a.h + (double)a.l; }
};

constexpr int kDiagRun = 16;                   // amplitudes per thread per run
constexpr int kDiagWarpSpan = 32 * kDiagRun;  // 512 consecutive amplitudes per warp

template <class T, bool kFF>
__global__ void __launch_bounds__(kReduceThreads, 2)
    k_pauli_diag(const void *__restrict__ st, uint32_t n, PauliGroup g, ReduceScratch rs) {
    using A = DiagArith<T>;
    using V = typename A::V;
    __shared__ V wsh[kReduceThreads / 32][kDiagRun][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t nt = g.nterms;
    V acc[kMaxTerms];
    uint32_t lanepar = 0;  // bit k: parity of (lane & z_k) xor the term's sign
#pragma unroll
    for (int k = 0; k < kMaxTerms; k++) {
        acc[k] = A::zero();
        if (k < (int)nt) lanepar |= (uint32_t)((__popc((uint32_t)lane & (uint32_t)g.z[k]) & 1) ^ (g.factor[k] < 0))
                                    << k;
    }
    const uint64_t runs = (1ull << n) / kDiagWarpSpan;
    const uint64_t wstride = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t r = (uint64_t)blockIdx.x * (blockDim.x >> 5) + w; r < runs; r += wstride) {
        const uint64_t b = r * kDiagWarpSpan;
        V p[kDiagRun];
#pragma unroll
        for (int u = 0; u < kDiagRun; u++) {
            if constexpr (kFF)
                p[u] = A::prob(reinterpret_cast<const float4 *>(st)[b + lane + 32 * u]);
            else
                p[u] = A::prob(reinterpret_cast<const cx<T> *>(st)[b + lane + 32 * u]);
        }
#pragma unroll
        for (int h = 1; h < kDiagRun; h <<= 1) {
#pragma unroll
            for (int u = 0; u < kDiagRun; u++) {
                if (u & h) continue;
                const V x = p[u], y = p[u | h];
                p[u] = A::add(x, y);
                p[u | h] = A::sub(x, y);
            }
        }
#pragma unroll
        for (int u = 0; u < kDiagRun; u++) wsh[w][u][lane] = p[u];
        __syncwarp();
#pragma unroll
        for (int k = 0; k < kMaxTerms; k++) {
            if (k < (int)nt) {
                const V v = wsh[w][(g.z[k] >> 5) & 15][lane];
                const bool neg = ((__popcll(b & g.z[k]) & 1) ^ (lanepar >> k)) & 1;
                acc[k] = neg ? A::sub(acc[k], v) : A::add(acc[k], v);
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int k = 0; k < kMaxTerms; k++) {
        if (k < (int)nt) {
            const double v = block_sum(A::to_d(acc[k]));
            if (threadIdx.x == 0) rs.partials[(size_t)blockIdx.x * kMaxTerms + k] = v;
        }
    }
    if (last_block(rs.ticket)) {
        for (int k = 0; k < (int)nt; k++) {
            const double t = sum_partials(rs.partials, gridDim.x, kMaxTerms, k);
            if (threadIdx.x == 0) rs.result[k] = t;
        }
        if (threadIdx.x == 0) *rs.ticket = 0;
    }
}

template <class T>
cudaError_t launch_pauli_group(const void *st, uint32_t n, const PauliGroup &g, const ReduceScratch &rs,
                               cudaStream_t s, bool ff_resident) {
    if (ff_resident && !(sizeof(T) == 8 && g.x == 0 && (1ull << n) >= (uint64_t)kDiagWarpSpan))
        return cudaErrorInvalidValue;  // (only the diagonal form reads the float-float resident state)
    if (g.x == 0 && (1ull << n) >= (uint64_t)kDiagWarpSpan) {
        if constexpr (sizeof(T) == 8) {
            if (ff_resident)
                k_pauli_diag<T, true><<<kReduceBlocks, kReduceThreads, 0, s>>>(st, n, g, rs);
            else
                k_pauli_diag<T, false><<<kReduceBlocks, kReduceThreads, 0, s>>>(st, n, g, rs);
        } else {
            k_pauli_diag<T, false><<<kReduceBlocks, kReduceThreads, 0, s>>>(st, n, g, rs);
        }
    } else {
        k_pauli_group<T><<<kReduceBlocks, kReduceThreads, 0, s>>>((const cx<T> *)st, n, g, rs);
    }
    count_launch();
    return cudaGetLastError();
}

// ---- tiled pass over many pair-form strings ---------------------------------------
// One tile of 2^K amplitudes per CTA iteration, staged in shared memory with
// coalesced loads (chunks of 2^l contiguous amplitudes); every term then
// visits its 2^(K-1) pairs inside the tile.  complex64: exact float products
// summed in float-float (AccF) per thread.  complex128: the tile is held in
// float-float form (binary64 split on load, or the float-float resident
// form as is), each pair product is a float-float dot product, summed per
// tile in float-float and added to a binary64 accumulator once per tile.
template <class T> struct TileVal;
template <> struct TileVal<float> {
    using V = cx<float>;
};
template <> struct TileVal<double> {
    struct V {
        ff::f2 re, im;
    };
};

__device__ __forceinline__ uint64_t tile_base_of(uint64_t tau, uint32_t l, uint32_t m, const uint8_t *hq) {
    uint64_t b = tau << l;
    for (uint32_t j = 0; j < m; j++) b = insert_zero(b, hq[j]);
    return b;
}

template <class T, bool kFF>
__global__ void __launch_bounds__(256) k_pauli_tile(const void *__restrict__ st, uint32_t n,
                                                    const __grid_constant__ PauliTilePass p, ReduceScratch rs) {
    using V = typename TileVal<T>::V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    V *tile = reinterpret_cast<V *>(smem_raw);
    const uint32_t K = p.K, l = p.l, m = p.m, nt = p.nterms;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(smem_raw + (sizeof(V) << K));
    for (uint32_t c = threadIdx.x; c < (1u << m); c += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
        chunk_off[c] = off;
    }
    const uint64_t tiles = 1ull << (n - K);
    const uint32_t lowmask = (1u << l) - 1u;
    const uint32_t npairs = 1u << (K - 1);
    typename AccOf<T>::type acc[kMaxTerms];
    __syncthreads();
    for (uint64_t tau = blockIdx.x; tau < tiles; tau += gridDim.x) {
        const uint64_t base = tile_base_of(tau, l, m, p.hq);
        for (uint32_t u = threadIdx.x; u < (1u << K); u += blockDim.x) {
            const uint64_t gidx = base + chunk_off[u >> l] + (u & lowmask);
            if constexpr (sizeof(T) == 4) {
                tile[u] = reinterpret_cast<const cx<float> *>(st)[gidx];
            } else if constexpr (kFF) {
                const float4 f = reinterpret_cast<const float4 *>(st)[gidx];  // re.hi, im.hi, re.lo, im.lo
                tile[u] = V{ff::f2{f.x, f.z}, ff::f2{f.y, f.w}};
            } else {
                const cx<double> a = reinterpret_cast<const cx<double> *>(st)[gidx];
                tile[u] = V{ff::from_double(a.re), ff::from_double(a.im)};
            }
        }
        __syncthreads();
        // (not unrolled: one copy of the pair loop; acc[] lives in local
        // memory, touched once per term and tile)
#pragma unroll 1
        for (int k = 0; k < (int)nt; k++) {
            const PauliTileTerm &t = p.t[k];
            const uint32_t tile_par = (uint32_t)__popcll(base & t.zo) & 1u;
            // four independent partial sums per thread (the pair products are
            // independent; one running sum would serialise its rounding chain)
            constexpr int U = 4;
            if constexpr (sizeof(T) == 4) {
                AccF part[U];
                for (uint32_t q0 = threadIdx.x; q0 < npairs; q0 += U * blockDim.x) {
#pragma unroll
                    for (int j = 0; j < U; j++) {
                        const uint32_t q = q0 + j * blockDim.x;
                        if (q >= npairs) break;
                        const uint32_t u = (uint32_t)insert_zero(q, t.hb);
                        const cx<float> a = tile[u], b = tile[u ^ t.xl];
                        const bool neg = ((__popc(u & t.zl) & 1u) ^ tile_par) != 0;
                        if (!t.im) {  // Re(conj(a) b) = a.re b.re + a.im b.im
                            if (neg) {
                                part[j].add_prod_neg(a.re, b.re);
                                part[j].add_prod_neg(a.im, b.im);
                            } else {
                                part[j].add_prod(a.re, b.re);
                                part[j].add_prod(a.im, b.im);
                            }
                        } else {  // Im(conj(a) b) = a.re b.im - a.im b.re
                            if (neg) {
                                part[j].add_prod_neg(a.re, b.im);
                                part[j].add_prod(a.im, b.re);
                            } else {
                                part[j].add_prod(a.re, b.im);
                                part[j].add_prod_neg(a.im, b.re);
                            }
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < U; j++) acc[k].add2(part[j].hi, part[j].lo);
            } else {
                ff::f2 part[U];
#pragma unroll
                for (int j = 0; j < U; j++) part[j] = ff::f2{0.f, 0.f};
                for (uint32_t q0 = threadIdx.x; q0 < npairs; q0 += U * blockDim.x) {
#pragma unroll
                    for (int j = 0; j < U; j++) {
                        const uint32_t q = q0 + j * blockDim.x;
                        if (q >= npairs) break;
                        const uint32_t u = (uint32_t)insert_zero(q, t.hb);
                        const V a = tile[u], b = tile[u ^ t.xl];
                        const ff::f2 v =
                            t.im ? ff::dot2(a.re, b.im, ff::neg(a.im), b.re) : ff::dot2(a.re, b.re, a.im, b.im);
                        const bool neg = ((__popc(u & t.zl) & 1u) ^ tile_par) != 0;
                        part[j] = neg ? ff::sub(part[j], v) : ff::add(part[j], v);
                    }
                }
                const ff::f2 sum = ff::add(ff::add(part[0], part[1]), ff::add(part[2], part[3]));
                acc[k].v += (double)sum.h + (double)sum.l;
            }
        }
        __syncthreads();
    }
    for (int k = 0; k < (int)nt; k++) {
        {
            const double v = block_sum(acc[k].value() * p.t[k].factor);
            if (threadIdx.x == 0) rs.partials[(size_t)blockIdx.x * kMaxTerms + k] = v;
        }
    }
    if (last_block(rs.ticket)) {
        for (int k = 0; k < (int)nt; k++) {
            const double tsum = sum_partials(rs.partials, gridDim.x, kMaxTerms, k);
            if (threadIdx.x == 0) rs.result[k] = tsum;
        }
        if (threadIdx.x == 0) *rs.ticket = 0;
    }
}

template <class T>
cudaError_t launch_pauli_tile(const void *st, uint32_t n, bool ff_resident, const PauliTilePass &p,
                              const ReduceScratch &rs, cudaStream_t s) {
    using V = typename TileVal<T>::V;
    const size_t smem = (sizeof(V) << p.K) + (sizeof(uint64_t) << p.m);
    auto kern = (sizeof(T) == 8 && ff_resident) ? k_pauli_tile<T, true> : k_pauli_tile<T, false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const uint64_t tiles = 1ull << (n - p.K);
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, (uint64_t)kReduceBlocks);
    kern<<<grid, 256, smem, s>>>(st, n, p, rs);
    count_launch();
    return cudaGetLastError();
}

// ---- support test for dump / sample ---------------------------------------
// Reference: hypot(re, im) > F(eps) in F (src/dense.rs:374).  With hypot
// correctly rounded this is re^2 + im^2 > m^2, m the midpoint between F(eps)
// and the next F value; decided in double with a guard band, and with an
// exact double evaluation inside the band.
__device__ __forceinline__ bool above_eps(cx<float> a) {
    const float q = __fmaf_rn(a.re, a.re, __fmul_rn(a.im, a.im));
    const float lo = 9.99998e-13f, hi = 1.000002e-12f;  // band around (1e-6)^2
    if (q > hi) return true;
    if (q < lo) return false;
    const double e = (double)1e-6f, e_next = (double)__int_as_float(__float_as_int(1e-6f) + 1);
    const double mid = 0.5 * (e + e_next);
    const double x = (double)a.re * (double)a.re + (double)a.im * (double)a.im;
    return x > mid * mid;
}
__device__ __forceinline__ bool above_eps(cx<double> a) {
    const double q = a.re * a.re + a.im * a.im;
    return q > 1e-30;
}

template <class T>
__device__ __forceinline__ double weight(cx<T> a) {
    if (!above_eps(a)) return 0.0;
    const double r = (double)a.re, i = (double)a.im;
    return __fma_rn(r, r, __dmul_rn(i, i));
}

int dump_blocks(uint32_t n) {
    const uint64_t ns = 1ull << n;
    uint64_t R = ns / 4096;
    if (R < 256) R = 256;
    if (R > ns) R = ns;
    return (int)(ns / R);
}
int sample_blocks(uint32_t n) { return dump_blocks(n); }

template <class T>
__global__ void __launch_bounds__(256) k_dump_count(const cx<T> *__restrict__ st, uint64_t R, uint64_t *counts) {
    const uint64_t base = (uint64_t)blockIdx.x * R;
    unsigned c = 0;
    for (uint64_t i = threadIdx.x; i < R; i += blockDim.x) c += above_eps(st[base + i]) ? 1u : 0u;
    const double t = block_sum((double)c);
    if (threadIdx.x == 0) counts[blockIdx.x] = (uint64_t)t;
}

template <class T>
__global__ void __launch_bounds__(256)
    k_dump_write(const cx<T> *__restrict__ st, uint64_t R, const uint64_t *offsets, DumpSpec spec, uint64_t *states,
                 double *re, double *im) {
    __shared__ unsigned wcount[8];
    __shared__ uint8_t q[64];
    if (threadIdx.x < 64) q[threadIdx.x] = spec.qubits[threadIdx.x];
    const uint64_t base = (uint64_t)blockIdx.x * R;
    uint64_t running = offsets[blockIdx.x];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    for (uint64_t c0 = 0; c0 < R; c0 += blockDim.x) {
        const uint64_t i = c0 + threadIdx.x;
        bool keep = false;
        cx<T> a{};
        if (i < R) {
            a = st[base + i];
            keep = above_eps(a);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) wcount[w] = __popc(bal);
        __syncthreads();
        unsigned before = 0, total = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) {
            if (k < w) before += wcount[k];
            total += wcount[k];
        }
        if (keep) {
            const uint64_t pos = running + before + __popc(bal & ((1u << lane) - 1));
            const uint64_t s = base + i;
            uint64_t packed = 0;
            for (uint32_t j = 0; j < spec.nq; j++) packed |= ((s >> q[spec.nq - 1 - j]) & 1ull) << j;
            states[pos] = packed;
            re[pos] = (double)a.re;
            im[pos] = (double)a.im;
        }
        running += total;
        __syncthreads();
    }
}

template <class T>
cudaError_t launch_dump_count(const void *st, uint32_t n, uint64_t *counts, cudaStream_t s) {
    const int B = dump_blocks(n);
    const uint64_t R = (1ull << n) / B;
    k_dump_count<T><<<B, 256, 0, s>>>((const cx<T> *)st, R, counts);
    count_launch();
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_dump_write(const void *st, uint32_t n, const uint64_t *offsets, const DumpSpec &spec,
                              uint64_t *states, double *re, double *im, cudaStream_t s) {
    const int B = dump_blocks(n);
    const uint64_t R = (1ull << n) / B;
    k_dump_write<T><<<B, 256, 0, s>>>((const cx<T> *)st, R, offsets, spec, states, re, im);
    count_launch();
    return cudaGetLastError();
}

// ---- sampling -------------------------------------------------------------------
// Both kernels walk a block's range in chunks of blockDim with the same scan,
// so the in-block running sums of the pick kernel end exactly at the block
// sums the host prefixes.
template <class T>
__global__ void __launch_bounds__(256) k_weight_blocksum(const cx<T> *__restrict__ st, uint64_t R, double *blocksum) {
    const uint64_t base = (uint64_t)blockIdx.x * R;
    double running = 0.0;
    for (uint64_t c0 = 0; c0 < R; c0 += blockDim.x) {
        const uint64_t i = c0 + threadIdx.x;
        const double w = (i < R) ? weight(st[base + i]) : 0.0;
        double total;
        block_inclusive_scan(w, &total);
        running = running + total;
        __syncthreads();
    }
    if (threadIdx.x == 0) blocksum[blockIdx.x] = running;
}

template <class T>
__global__ void __launch_bounds__(256)
    k_sample_pick(const cx<T> *__restrict__ st, uint64_t R, const uint32_t *blocks, const uint64_t *shot_begin,
                  const double *prefix, const double *chosen, uint64_t *pick) {
    __shared__ double pre[256];
    __shared__ uint64_t last_nz;
    const uint32_t b = blocks[blockIdx.x];
    const uint64_t base = (uint64_t)b * R;
    const double P = prefix[blockIdx.x];
    uint64_t sh = shot_begin[blockIdx.x];
    const uint64_t sh_end = shot_begin[blockIdx.x + 1];
    double running = 0.0;
    if (threadIdx.x == 0) last_nz = base;
    __syncthreads();
    for (uint64_t c0 = 0; c0 < R && sh < sh_end; c0 += blockDim.x) {
        const uint64_t i = c0 + threadIdx.x;
        const double w = (i < R) ? weight(st[base + i]) : 0.0;
        double total;
        const double incl = block_inclusive_scan(w, &total);
        pre[threadIdx.x] = P + (running + incl);
        if (w > 0.0) atomicMax((unsigned long long *)&last_nz, (unsigned long long)(base + i));
        __syncthreads();
        const double chunk_end = pre[blockDim.x - 1];
        // shots whose first prefix above `chosen` lies in this chunk
        while (sh < sh_end && chosen[sh] < chunk_end) {
            const uint64_t j = sh + threadIdx.x;
            if (j < sh_end && chosen[j] < chunk_end) {
                const double c = chosen[j];
                int lo = 0, hi = blockDim.x - 1;  // first pre[] > c
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (pre[mid] > c)
                        hi = mid;
                    else
                        lo = mid + 1;
                }
                pick[j] = base + c0 + lo;
            }
            // advance past every shot resolved in this chunk
            uint64_t adv = 0;
            while (sh + adv < sh_end && adv < blockDim.x && chosen[sh + adv] < chunk_end) adv++;
            sh += adv;
            __syncthreads();
        }
        running = running + total;
        __syncthreads();
    }
    // rounding leftovers: the block's last element with weight
    for (uint64_t j = sh + threadIdx.x; j < sh_end; j += blockDim.x) pick[j] = last_nz;
}

template <class T>
cudaError_t launch_weight_blocksum(const void *st, uint32_t n, double *blocksum, cudaStream_t s) {
    const int B = sample_blocks(n);
    const uint64_t R = (1ull << n) / B;
    k_weight_blocksum<T><<<B, 256, 0, s>>>((const cx<T> *)st, R, blocksum);
    count_launch();
    return cudaGetLastError();
}

template <class T>
cudaError_t launch_sample_pick(const void *st, uint32_t n, const uint32_t *blocks, uint32_t nblocks_with_shots,
                               const uint64_t *shot_begin, const double *prefix, const double *chosen,
                               uint64_t *pick, cudaStream_t s) {
    const int B = sample_blocks(n);
    const uint64_t R = (1ull << n) / B;
    if (nblocks_with_shots == 0) return cudaSuccess;
    k_sample_pick<T><<<nblocks_with_shots, 256, 0, s>>>((const cx<T> *)st, R, blocks, shot_begin, prefix, chosen,
                                                          pick);
    count_launch();
    return cudaGetLastError();
}

// ---- allocation-free masked norm ----------------------------------------------
// Some callers of this library cannot allocate device memory: code that runs
// while a CUDA graph is being captured (cudaMalloc is not capturable), plugins
// hosted by a runtime that owns every device allocation through its own pool,
// and real-time loops that cannot take the implicit synchronisation of an
// allocation.  kbwg_masked_norm_noalloc serves them: it runs the same
// reduction as kbwg_measure_p1 but keeps its scratch (608 per-block partial
// sums and the last-block ticket) in the fixed device array below instead of
// a per-handle cudaMalloc.  Every GPU that loads this library holds the array
// (8 KiB) until the process exits.
constexpr size_t kNoAllocScratchBytes = 8192;
constexpr size_t kNoAllocTicketOffset = 4864;  // after kReduceBlocks doubles, 256-aligned
static_assert(kReduceBlocks * sizeof(double) <= kNoAllocTicketOffset, "partials overflow the fixed scratch");
static_assert(kNoAllocTicketOffset + 256 <= kNoAllocScratchBytes, "ticket overflows the fixed scratch");
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Host code may not use g_noalloc_scratch as an address (it names a host-side
// stand-in); the device address is looked up with the device current, once
// per CUDA context.  The cache is keyed on the context's id, not on the
// device ordinal: after cudaDeviceReset the device gets a new context in
// which the array may have another address.
namespace {
typedef int (*CtxGetCurrentFn)(void **);
typedef int (*CtxGetIdFn)(void *, unsigned long long *);
std::mutex g_noalloc_mu;
std::vector<std::pair<unsigned long long, void *>> g_noalloc_addr;  // context id -> array address

// Id of the calling thread's current CUDA context (driver entry points
// obtained through the runtime); false if none is current or unknown.
bool current_context_id(unsigned long long &id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool resolved = false;
    if (!resolved) {
        resolved = true;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", (void **)&get_current, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess || q != cudaDriverEntryPointSuccess)
            get_current = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", (void **)&get_id, 12000, cudaEnableDefault, &q) !=
                cudaSuccess || q != cudaDriverEntryPointSuccess)
            get_id = nullptr;
    }
    void *ctx = nullptr;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, &id) == 0;
}
}  // namespace

static cudaError_t noalloc_scratch(void **out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long id = 0;
    if (current_context_id(id))
        for (const auto &a : g_noalloc_addr)
            if (a.first == id) {
                *out = a.second;
                return cudaSuccess;
            }
    // set-up on this context (the lookup makes the current device's context current if none is)
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    if (current_context_id(id)) g_noalloc_addr.emplace_back(id, p);
    *out = p;
    return cudaSuccess;
}

// A device or managed allocation on the current device (a host pointer, or
// memory of another device, would make the kernel fault).
static bool on_current_device(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) return false;
    int dev = -1;
    return cudaGetDevice(&dev) == cudaSuccess && a.device == dev;
}

}  // namespace kbwg

extern "C" int32_t kbwg_masked_norm_noalloc(const void *state, uintptr_t num_qubits, int32_t precision,
                                            uint64_t mask, uint64_t value, double *out, void *stream) {
    using namespace kbwg;
    if (!state || !out) {
        set_error(KBWG_EINVAL, "kbwg_masked_norm_noalloc: null state or output pointer");
        return KBWG_EINVAL;
    }
    if (num_qubits > 32) {
        set_error(KBWG_EQUBITS, "kbwg_masked_norm_noalloc: at most 32 qubits (its fixed scratch serves "
                                "a 608-block grid over up to 2^32 amplitudes)");
        return KBWG_EQUBITS;
    }
    if (precision != KBWG_C64 && precision != KBWG_C128) {
        set_error(KBWG_EINVAL, "kbwg_masked_norm_noalloc: bad precision");
        return KBWG_EINVAL;
    }
    const uint64_t all = (1ull << num_qubits) - 1;  // num_qubits <= 32 here
    if ((mask & ~all) || (value & ~mask)) {
        set_error(KBWG_EINVAL, "kbwg_masked_norm_noalloc: mask/value outside the register or value outside mask");
        return KBWG_EINVAL;
    }
    if (!on_current_device(state) || !on_current_device(out)) {
        set_error(KBWG_EINVAL, "kbwg_masked_norm_noalloc: state and out must be device (or managed) memory of the "
                               "current device");
        return KBWG_EINVAL;
    }
    void *base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    if (e != cudaSuccess) {
        set_error(KBWG_ECUDA, std::string("kbwg_masked_norm_noalloc: scratch lookup: ") + cudaGetErrorString(e));
        return KBWG_ECUDA;
    }
    ReduceScratch rs;
    rs.partials = (double *)base;
    rs.ticket = (unsigned *)((char *)base + kNoAllocTicketOffset);
    rs.result = out;
    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemsetAsync(rs.ticket, 0, sizeof(unsigned), s);  // the array keeps the last call's contents
    if (e == cudaSuccess)
        e = precision ? launch_masked_norm<double>(state, (uint32_t)num_qubits, mask, value, rs, s)
                      : launch_masked_norm<float>(state, (uint32_t)num_qubits, mask, value, rs, s);
    if (e != cudaSuccess) {
        set_error(KBWG_ECUDA, std::string("kbwg_masked_norm_noalloc: ") + cudaGetErrorString(e));
        return KBWG_ECUDA;
    }
    return KBWG_OK;
}

namespace kbwg {

#define INST(T)                                                                                               \
    template cudaError_t launch_masked_norm<T>(const void *, uint32_t, uint64_t, uint64_t, const ReduceScratch &, \
                                               cudaStream_t);                                                 \
    template cudaError_t launch_measure_step<T>(const void *, uint32_t, MeasureCtl *, uint32_t,                \
                                                const ReduceScratch &, cudaStream_t);                         \
    template cudaError_t launch_collapse<T>(void *, uint32_t, const MeasureCtl *, uint64_t, uint64_t, double,   \
                                            cudaStream_t);                                                    \
    template cudaError_t launch_pauli_group<T>(const void *, uint32_t, const PauliGroup &, const ReduceScratch &, \
                                               cudaStream_t, bool);                                           \
    template cudaError_t launch_pauli_tile<T>(const void *, uint32_t, bool, const PauliTilePass &,               \
                                              const ReduceScratch &, cudaStream_t);                           \
    template cudaError_t launch_dump_count<T>(const void *, uint32_t, uint64_t *, cudaStream_t);               \
    template cudaError_t launch_dump_write<T>(const void *, uint32_t, const uint64_t *, const DumpSpec &,        \
                                              uint64_t *, double *, double *, cudaStream_t);                  \
    template cudaError_t launch_weight_blocksum<T>(const void *, uint32_t, double *, cudaStream_t);            \
    template cudaError_t launch_sample_pick<T>(const void *, uint32_t, const uint32_t *, uint32_t,             \
                                               const uint64_t *, const double *, const double *, uint64_t *,  \
                                               cudaStream_t);
INST(float)
INST(double)

}  // namespace kbwg
