// Reverse-mode adjoint gradient of E(theta) = <psi|H|psi>, psi = U_M...U_1|0>.
//
// The reference has no native gradient: BatchExecution::gradient returns
// NativeGateUnsupported (kbw src/quantum_execution.rs:420-426) and libket
// falls back to the parameter-shift rule, two full circuit evaluations per
// parameter (src/quantum_execution.rs:237-241, 392-405).  Here:
//   1. forward: phi = psi with the fused sweeps, copying phi at segment
//      boundaries ("checkpoints") while memory allows;
//   2. lambda = H phi (one pass per group of Pauli strings sharing X/Y
//      positions), E = Re<phi|lambda>;
//   3. reverse: walk the gates backwards; for gate j (phi = phi_j,
//      lambda = lambda_j) accumulate
//        RX/RY/RZ(t) = exp(-i t P/2):  dE/dt = Im <lambda| Pi_C P |phi>
//        P(t) = diag(1, e^{it}):       dE/dt = -2 Im <lambda| Pi_C Pi_1 |phi>
//      (Pi_C = projector on the gate's controls), then uncompute
//      phi <- U_j^dag phi and lambda <- U_j^dag lambda.  Both states move
//      through one fused two-state tile sweep; at a checkpoint boundary phi
//      is reloaded from its copy so rounding does not accumulate across
//      segments.
// Inner products accumulate FP64-grade (float partials per warp widened to
// double for complex64, double or float-float for complex128).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/kbwg.h"
#include "kernels.h"
#include "sim.h"
#include "adjoint_dev.cuh"
#include "jit.h"
#include "sweep_dev.cuh"

namespace kbwg {

// C++ names of the adjoint's arithmetic policies, for its specialised kernels.
template <class P> struct AdjPolicyName;
template <> struct AdjPolicyName<FastP> { static constexpr const char *s = "kbwg::FastP"; };
template <> struct AdjPolicyName<FF2B> { static constexpr const char *s = "kbwg::FF2B"; };
template <> struct AdjPolicyName<FF2> { static constexpr const char *s = "kbwg::FF2"; };
template <> struct AdjPolicyName<Fast<double>> { static constexpr const char *s = "kbwg::Fast<double>"; };

// ---- lambda = H phi ------------------------------------------------------------------
// One group of strings with common flip mask x:
//   lambda_s (+)= sum_k c_k i^{ny_k} (-1)^{|(s^x) & z_k|} phi_{s^x}
struct ApplyGroup {
    uint64_t x;
    uint32_t nterms;
    uint32_t init;  // 1: write lambda instead of accumulating
    uint64_t z[kMaxTerms];
    double cre[kMaxTerms];  // c_k * Re(i^{ny_k})
    double cim[kMaxTerms];  // c_k * Im(i^{ny_k})
};

template <class T>
__global__ void __launch_bounds__(256) k_apply_group(const cx<T> *__restrict__ phi, cx<T> *__restrict__ lam,
                                                     uint64_t ns, ApplyGroup g) {
    __shared__ T sre[kMaxTerms], sim_[kMaxTerms];
    if (threadIdx.x < kMaxTerms) {
        sre[threadIdx.x] = (T)g.cre[threadIdx.x];
        sim_[threadIdx.x] = (T)g.cim[threadIdx.x];
    }
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        const uint64_t src = s ^ g.x;
        const cx<T> a = phi[src];
        T wr = 0, wi = 0;
        for (uint32_t k = 0; k < g.nterms; k++) {
            const bool neg = (__popcll(src & g.z[k]) & 1) != 0;
            wr += neg ? -sre[k] : sre[k];
            wi += neg ? -sim_[k] : sim_[k];
        }
        cx<T> r;
        r.re = wr * a.re - wi * a.im;
        r.im = wr * a.im + wi * a.re;
        if (!g.init) {
            const cx<T> o = lam[s];
            r.re += o.re;
            r.im += o.im;
        }
        lam[s] = r;
    }
}

// lambda (+)= H phi for every string of one tiled pass (the strings' flip
// masks lie in the tile): the phi tile is staged in shared memory with
// coalesced loads, then each thread sums, for the amplitudes it owns, the
// terms c_k i^{ny_k} (-1)^{|src & z_k|} phi_src, src = s ^ x_k.
struct ApplyTileTerm {
    uint32_t xl, zl;  // flip and phase masks on local bits
    uint64_t zo;      // phase mask on qubits outside the tile
    double cre, cim;  // c_k * i^{ny_k}
};
struct ApplyTilePass {
    uint32_t K, l, m, nterms, init;
    uint8_t hq[16];
    ApplyTileTerm t[kMaxTerms];
};
constexpr int kApplyTileBits = 11;  // 2^11 amplitudes (16/32 KiB) per tile

template <class T>
__global__ void __launch_bounds__(256) k_apply_tile(const cx<T> *__restrict__ phi, cx<T> *__restrict__ lam, uint32_t n,
                                                    const __grid_constant__ ApplyTilePass p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T cre[kMaxTerms], cim[kMaxTerms];  // coefficients converted once (no per-term F2F)
    cx<T> *tile = reinterpret_cast<cx<T> *>(smem_raw);
    const uint32_t K = p.K, l = p.l, m = p.m;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(smem_raw + (sizeof(cx<T>) << K));
    if (threadIdx.x < kMaxTerms) {
        cre[threadIdx.x] = (T)p.t[threadIdx.x].cre;
        cim[threadIdx.x] = (T)p.t[threadIdx.x].cim;
    }
    for (uint32_t c = threadIdx.x; c < (1u << m); c += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
        chunk_off[c] = off;
    }
    const uint64_t tiles = 1ull << (n - K);
    const uint32_t lowmask = (1u << l) - 1u;
    __syncthreads();
    for (uint64_t tau = blockIdx.x; tau < tiles; tau += gridDim.x) {
        uint64_t base = tau << l;
        for (uint32_t j = 0; j < m; j++) {
            const uint64_t low = (1ull << p.hq[j]) - 1;
            base = ((base & ~low) << 1) | (base & low);
        }
        for (uint32_t u = threadIdx.x; u < (1u << K); u += blockDim.x)
            tile[u] = phi[base + chunk_off[u >> l] + (u & lowmask)];
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < (1u << K); u += blockDim.x) {
            // strings without flips and with a real factor (Z-type) only add
            // their signed coefficient to d, applied once to the amplitude;
            // real-factor strings with flips take two FMAs, the rest four
            // (the branches are uniform: they depend on the term only)
            T ar = 0, ai = 0, d = 0;
            for (uint32_t k = 0; k < p.nterms; k++) {
                const ApplyTileTerm &t = p.t[k];
                const uint32_t src = u ^ t.xl;
                const bool neg = ((__popc(src & t.zl) + __popcll(base & t.zo)) & 1) != 0;
                const T wr = neg ? -cre[k] : cre[k];
                if (cim[k] == (T)0) {
                    if (t.xl == 0) {
                        d += wr;
                        continue;
                    }
                    const cx<T> a = tile[src];
                    ar += wr * a.re;
                    ai += wr * a.im;
                    continue;
                }
                const T wi = neg ? -cim[k] : cim[k];
                const cx<T> a = tile[src];
                ar += wr * a.re - wi * a.im;
                ai += wr * a.im + wi * a.re;
            }
            {
                const cx<T> a = tile[u];
                ar += d * a.re;
                ai += d * a.im;
            }
            const uint64_t gidx = base + chunk_off[u >> l] + (u & lowmask);
            if (!p.init) {
                const cx<T> o = lam[gidx];
                ar += o.re;
                ai += o.im;
            }
            lam[gidx] = cx<T>{ar, ai};
        }
        __syncthreads();
    }
}

// ---- the same on float-float resident states (complex128 fast path) ----------
// Amplitudes are ff2::v2 {h = (re.hi, im.hi), l = (re.lo, im.lo)}.  A pass's
// strings come in runs of one coefficient: Z-type strings with a real
// factor (no flip) count their signs in an integer and scale the amplitude
// once per run; real-factor strings with flips add the signed partner
// amplitudes and scale the sum once per run; complex factors multiply each.
struct ApplyTileTermFF {
    uint32_t xl, zl;  // flip and phase masks on local bits
    uint64_t zo;      // phase mask on qubits outside the tile
    float rh, rl, ih, il;  // c_k * i^{ny_k} as float-float (re, im)
    uint32_t cat;     // 0: real, no flip; 1: real with flips; 2: complex
    uint32_t last;    // 1: the last string of its run
};
struct ApplyTilePassFF {
    uint32_t K, l, m, nterms, init;
    uint8_t hq[16];
    ApplyTileTermFF t[kMaxTerms];
};

__global__ void __launch_bounds__(256) k_apply_tile_ff(const ff2::v2 *__restrict__ phi, ff2::v2 *__restrict__ lam,
                                                       uint32_t n, const __grid_constant__ ApplyTilePassFF p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ff2::v2 *tile = reinterpret_cast<ff2::v2 *>(smem_raw);
    const uint32_t K = p.K, l = p.l, m = p.m;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(smem_raw + (sizeof(ff2::v2) << K));
    for (uint32_t c = threadIdx.x; c < (1u << m); c += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
        chunk_off[c] = off;
    }
    const uint64_t tiles = 1ull << (n - K);
    const uint32_t lowmask = (1u << l) - 1u;
    const ff2::v2 zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    __syncthreads();
    for (uint64_t tau = blockIdx.x; tau < tiles; tau += gridDim.x) {
        uint64_t base = tau << l;
        for (uint32_t j = 0; j < m; j++) {
            const uint64_t low = (1ull << p.hq[j]) - 1;
            base = ((base & ~low) << 1) | (base & low);
        }
        for (uint32_t u = threadIdx.x; u < (1u << K); u += blockDim.x)
            tile[u] = phi[base + chunk_off[u >> l] + (u & lowmask)];
        __syncthreads();
        for (uint32_t u = threadIdx.x; u < (1u << K); u += blockDim.x) {
            const ff2::v2 self = tile[u];
            ff2::v2 acc = zero, run = zero;
            int cnt = 0;
            for (uint32_t k = 0; k < p.nterms; k++) {  // (branches depend on the term only: uniform)
                const ApplyTileTermFF &t = p.t[k];
                const uint32_t src = u ^ t.xl;
                const bool neg = ((__popc(src & t.zl) + __popcll(base & t.zo)) & 1) != 0;
                if (t.cat == 0u) {
                    cnt += neg ? -1 : 1;
                    if (t.last) {
                        const ff::f2 w = ff::mul(ff::f2{t.rh, t.rl}, ff::f2{(float)cnt, 0.f});
                        acc = ff2::add(acc, ff2::mul(self, ff2::konst(w)));
                        cnt = 0;
                    }
                } else if (t.cat == 1u) {
                    const ff2::v2 a = tile[src];
                    run = neg ? ff2::sub(run, a) : ff2::add(run, a);
                    if (t.last) {
                        acc = ff2::add(acc, ff2::mul(run, ff2::konst(ff::f2{t.rh, t.rl})));
                        run = zero;
                    }
                } else {
                    const ff2::v2 a = tile[src];
                    const ff::f2 cr{t.rh, t.rl}, ci{t.ih, t.il};
                    // (cr re - ci im, cr im + ci re)
                    const ff2::v2 prod = ff2::dot2(ff2::konst(cr), a, ff2::konst(ff::neg(ci), ci), ff2::swap(a));
                    acc = neg ? ff2::sub(acc, prod) : ff2::add(acc, prod);
                }
            }
            const uint64_t gidx = base + chunk_off[u >> l] + (u & lowmask);
            if (!p.init) acc = ff2::add(acc, lam[gidx]);
            lam[gidx] = acc;
        }
        __syncthreads();
    }
}

// One group of strings with a common flip mask (strings too wide for a
// tile), float-float: lambda_s (+)= sum_k c_k i^{ny_k} (-1)^{|(s^x) & z_k|} phi_{s^x}.
__global__ void __launch_bounds__(256) k_apply_group_ff(const ff2::v2 *__restrict__ phi, ff2::v2 *__restrict__ lam,
                                                        uint64_t ns, ApplyGroup g) {
    __shared__ float rh[kMaxTerms], rl[kMaxTerms], ih[kMaxTerms], il[kMaxTerms];
    if (threadIdx.x < kMaxTerms) {
        const ff::f2 r = ff::split_constant(g.cre[threadIdx.x]), i = ff::split_constant(g.cim[threadIdx.x]);
        rh[threadIdx.x] = r.h;
        rl[threadIdx.x] = r.l;
        ih[threadIdx.x] = i.h;
        il[threadIdx.x] = i.l;
    }
    __syncthreads();
    const ff2::v2 zero{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        const uint64_t src = s ^ g.x;
        const ff2::v2 a = phi[src];
        ff2::v2 acc = zero;
        for (uint32_t k = 0; k < g.nterms; k++) {
            const bool neg = (__popcll(src & g.z[k]) & 1) != 0;
            const ff::f2 cr{rh[k], rl[k]}, ci{ih[k], il[k]};
            const ff2::v2 prod = ff2::dot2(ff2::konst(cr), a, ff2::konst(ff::neg(ci), ci), ff2::swap(a));
            acc = neg ? ff2::sub(acc, prod) : ff2::add(acc, prod);
        }
        if (!g.init) acc = ff2::add(acc, lam[s]);
        lam[s] = acc;
    }
}

// The same runs for complex64 states (float arithmetic; the coefficients are
// the high parts rh/ih): each thread keeps its 2^K/256 amplitudes u = tid +
// 256 i in registers, the strings run in the outer loop (their fields read
// once per tile), signs are counted per amplitude and partners summed per run.
__global__ void __launch_bounds__(256) k_apply_tile_f32(const cx<float> *__restrict__ phi, cx<float> *__restrict__ lam,
                                                        uint32_t n, const __grid_constant__ ApplyTilePassFF p) {
    constexpr int K = kApplyTileBits, NA = (1 << K) / 256;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<float> *tile = reinterpret_cast<cx<float> *>(smem_raw);
    const uint32_t l = p.l, m = p.m;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(smem_raw + (sizeof(cx<float>) << K));
    for (uint32_t c = threadIdx.x; c < (1u << m); c += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
        chunk_off[c] = off;
    }
    const uint64_t tiles = 1ull << (n - K);
    const uint32_t lowmask = (1u << l) - 1u;
    __syncthreads();
    for (uint64_t tau = blockIdx.x; tau < tiles; tau += gridDim.x) {
        uint64_t base = tau << l;
        for (uint32_t j = 0; j < m; j++) {
            const uint64_t low = (1ull << p.hq[j]) - 1;
            base = ((base & ~low) << 1) | (base & low);
        }
        cx<float> self[NA];
#pragma unroll
        for (int i = 0; i < NA; i++) {
            const uint32_t u = threadIdx.x + 256u * (uint32_t)i;
            self[i] = phi[base + chunk_off[u >> l] + (u & lowmask)];
            tile[u] = self[i];
        }
        __syncthreads();
        float ar[NA], ai[NA], rr[NA], ri[NA];
        int cnt[NA];
#pragma unroll
        for (int i = 0; i < NA; i++) ar[i] = ai[i] = rr[i] = ri[i] = 0.f, cnt[i] = 0;
        for (uint32_t k = 0; k < p.nterms; k++) {  // (branches depend on the string only: uniform)
            const ApplyTileTermFF t = p.t[k];
            const uint32_t op = (uint32_t)__popcll(base & t.zo) & 1u;
#pragma unroll
            for (int i = 0; i < NA; i++) {
                const uint32_t u = threadIdx.x + 256u * (uint32_t)i, src = u ^ t.xl;
                const bool neg = (((uint32_t)__popc(src & t.zl) + op) & 1u) != 0u;
                if (t.cat == 0u) {
                    cnt[i] += neg ? -1 : 1;
                    if (t.last) {
                        const float w = (float)cnt[i] * t.rh;
                        ar[i] += w * self[i].re;
                        ai[i] += w * self[i].im;
                        cnt[i] = 0;
                    }
                } else if (t.cat == 1u) {
                    const cx<float> a = tile[src];
                    rr[i] += neg ? -a.re : a.re;
                    ri[i] += neg ? -a.im : a.im;
                    if (t.last) {
                        ar[i] += t.rh * rr[i];
                        ai[i] += t.rh * ri[i];
                        rr[i] = ri[i] = 0.f;
                    }
                } else {
                    const cx<float> a = tile[src];
                    const float pr = t.rh * a.re - t.ih * a.im, pi = t.rh * a.im + t.ih * a.re;
                    ar[i] += neg ? -pr : pr;
                    ai[i] += neg ? -pi : pi;
                }
            }
        }
#pragma unroll
        for (int i = 0; i < NA; i++) {
            const uint32_t u = threadIdx.x + 256u * (uint32_t)i;
            const uint64_t gidx = base + chunk_off[u >> l] + (u & lowmask);
            if (!p.init) {
                const cx<float> o = lam[gidx];
                ar[i] += o.re;
                ai[i] += o.im;
            }
            lam[gidx] = cx<float>{ar[i], ai[i]};
        }
        __syncthreads();
    }
}

// Re<a|b> of float-float states: per-thread float-float sums, then FP64.
__global__ void __launch_bounds__(256) k_inner_re_ff(const ff2::v2 *__restrict__ a, const ff2::v2 *__restrict__ b,
                                                     uint64_t ns, double *partials, unsigned *ticket, double *result) {
    ff::f2 t{0.f, 0.f};
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        const ff2::v2 x = a[s], y = b[s];
        t = ff::add(t, ff::dot2(ff::f2{x.h.x, x.l.x}, ff::f2{y.h.x, y.l.x}, ff::f2{x.h.y, x.l.y}, ff::f2{y.h.y, y.l.y}));
    }
    double acc = (double)t.h + (double)t.l;
    __shared__ double sh[8];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += sh[w];
        partials[blockIdx.x] = tot;
        __threadfence();
        if (atomicAdd(ticket, 1u) == gridDim.x - 1) {
            double all = 0.0;
            for (unsigned b2 = 0; b2 < gridDim.x; b2++) all += partials[b2];
            result[0] = all;
            *ticket = 0;
        }
    }
}

// Re<a|b> (FP64-grade) into result[0].
template <class T>
__global__ void __launch_bounds__(256) k_inner_re(const cx<T> *__restrict__ a, const cx<T> *__restrict__ b,
                                                  uint64_t ns, double *partials, unsigned *ticket, double *result) {
    double acc = 0.0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += stride) {
        const cx<T> x = a[s], y = b[s];
        acc = fma((double)x.re, (double)y.re, acc);
        acc = fma((double)x.im, (double)y.im, acc);
    }
    __shared__ double sh[8];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
        partials[blockIdx.x] = t;
        __threadfence();
        if (atomicAdd(ticket, 1u) == gridDim.x - 1) {
            double tot = 0.0;
            for (unsigned b2 = 0; b2 < gridDim.x; b2++) tot += partials[b2];
            result[0] = tot;
            *ticket = 0;
        }
    }
}

// W: registers above 32 qubits (the gates read bits of the 64-bit tile base).
template <class P, int K, int R, bool W = false>
__global__ void __launch_bounds__(AdjKernel<P, K, R>::kThreads, 2)
    k_adjoint(typename P::Mem *__restrict__ phi, typename P::Mem *__restrict__ lam, const __grid_constant__ AdjParams a) {
    using Amp = typename P::Amp;
    using Mem = typename P::Mem;
    using AK = AdjKernel<P, K, R>;
    using G = Grad<P>;
    constexpr int NR = 1 << R;
    const SweepParams &p = a.sw;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Mem *tphi_m = reinterpret_cast<Mem *>(smem_raw);
    Mem *tlam_m = reinterpret_cast<Mem *>(smem_raw + AK::kTileBytes);
    Amp *tphi = reinterpret_cast<Amp *>(smem_raw);
    Amp *tlam = reinterpret_cast<Amp *>(smem_raw + AK::kTileBytes);
    unsigned char *q = smem_raw + 2 * AK::kTileBytes;
    uint64_t *chunk_off = reinterpret_cast<uint64_t *>(q);
    q += 256 * sizeof(uint64_t);
    TileGate *sg = reinterpret_cast<TileGate *>(q);
    q += kMaxSweepGates * sizeof(TileGate);
    uint32_t *sinfo = reinterpret_cast<uint32_t *>(q);
    q += kMaxSweepGates * sizeof(uint32_t);
    using Wacc = typename G::Wacc;
    static_assert(sizeof(Wacc) == sizeof(double), "per-warp accumulator slot");
    Wacc *acc = reinterpret_cast<Wacc *>(q);  // [kWarps][kMaxSweepGates]
    q += (size_t)AK::kWarps * kMaxSweepGates * sizeof(Wacc);
    uint64_t *bar = reinterpret_cast<uint64_t *>(q);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t l = p.l, m = p.m;
    const uint32_t chunk = 1u << l, nchunks = 1u << m;
    const uint32_t chunk_bytes = chunk * (uint32_t)sizeof(Mem);
    const uint64_t lowmask = chunk - 1;

    for (uint32_t i = threadIdx.x; i < p.gate_count; i += blockDim.x) {
        sg[i] = p.prog[i];
        sinfo[i] = a.ginfo[i];
    }
    for (uint32_t i = threadIdx.x; i < (uint32_t)AK::kWarps * kMaxSweepGates; i += blockDim.x) acc[i] = Wacc{};
    for (uint32_t c = threadIdx.x; c < nchunks; c += blockDim.x) {
        uint64_t off = 0;
        for (uint32_t j = 0; j < m; j++) off |= (uint64_t)((c >> j) & 1u) << p.hq[j];
        chunk_off[c] = off;
    }
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    __syncthreads();

    auto tile_base = [&](uint64_t tau) {
        uint64_t b = tau << l;
        for (uint32_t j = 0; j < m; j++) b = insert_zero_at(b, p.hq[j]);
        return b;
    };
    auto issue_load = [&](uint64_t tau) {
        if (warp == 0) {
            const uint64_t b = tile_base(tau);
            if (lane == 0) mbar_expect_tx(bar, (uint32_t)(2 * AK::kTileBytes));
            __syncwarp();
            for (uint32_t c = lane; c < nchunks; c += 32) {
                tma_load(tphi_m + (size_t)c * chunk, phi + b + chunk_off[c], chunk_bytes, bar);
                tma_load(tlam_m + (size_t)c * chunk, lam + b + chunk_off[c], chunk_bytes, bar);
            }
        }
    };

    uint64_t tau = blockIdx.x;
    if (tau < p.tiles) issue_load(tau);
    const uint32_t FA = (uint32_t)lane | ((uint32_t)warp << (kLaneBits + R));
    const uint32_t FB = (uint32_t)lane | ((uint32_t)warp << kLaneBits);
    for (uint32_t it = 0; tau < p.tiles; tau += gridDim.x, it++) {
        const uint64_t base = tile_base(tau);
        if (!tile_wait(bar, it & 1u, p.err)) return;
        Amp vp[NR], vl[NR];
        int layout = p.stage_layout[0];
        int R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
        uint32_t F = (layout == LAYOUT_A) ? FA : FB;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            vp[j] = P::from_mem(tphi_m[F | ((uint32_t)j << R0)]);
            vl[j] = P::from_mem(tlam_m[F | ((uint32_t)j << R0)]);
        }
        uint32_t g0 = 0;
        for (uint32_t s = 0; s < p.nstages; s++) {
            const int nl = p.stage_layout[s];
            if (nl != layout) {
#pragma unroll
                for (int j = 0; j < NR; j++) {
                    tphi[F | ((uint32_t)j << R0)] = vp[j];
                    tlam[F | ((uint32_t)j << R0)] = vl[j];
                }
                __syncthreads();
                layout = nl;
                R0 = (layout == LAYOUT_A) ? kLaneBits : (K - R);
                F = (layout == LAYOUT_A) ? FA : FB;
#pragma unroll
                for (int j = 0; j < NR; j++) {
                    vp[j] = tphi[F | ((uint32_t)j << R0)];
                    vl[j] = tlam[F | ((uint32_t)j << R0)];
                }
            }
            const uint32_t g1 = p.stage_end[s];
            for (uint32_t gi = g0; gi < g1; gi++) {
                const TileGate &g = sg[gi];
                if ((base & g.co) != g.co) continue;  // uniform over the tile
                const uint32_t info = sinfo[gi];
                const int gt = (int)(info & 15u);
                if (gt != GT_NONE) {
                    const typename G::Acc w = G::warp_sum(grad_partial<P, K, R>(g, gt, vp, vl, R0, F, base));
                    if (lane == 0) {
                        Wacc &slot = acc[warp * kMaxSweepGates + (info >> 4)];
                        slot = G::wadd(slot, w);
                    }
                }
                using B = typename pick_t<W, uint64_t, uint32_t>::type;
                tile_gate<P, K, R, B>(g, vp, R0, F, (B)base);
                tile_gate<P, K, R, B>(g, vl, R0, F, (B)base);
            }
            g0 = g1;
        }
        fence_proxy_async();
        __syncthreads();
        const uint64_t next = tau + gridDim.x;
        if (next < p.tiles) issue_load(next);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t u = F | ((uint32_t)j << R0);
            const uint64_t idx = base + chunk_off[u >> l] + (u & lowmask);
            phi[idx] = P::to_mem(vp[j]);
            lam[idx] = P::to_mem(vl[j]);
        }
    }
    __syncthreads();
    for (uint32_t sl = threadIdx.x; sl < a.nslots; sl += blockDim.x) {
        double t = 0.0;
        for (int w = 0; w < AK::kWarps; w++) t += G::wvalue(acc[w * kMaxSweepGates + sl]);
        a.partials[(size_t)blockIdx.x * a.nslots + sl] = t;
    }
}

// grads[gate_of_slot[s]] = sum over blocks of partials[b][s]: one warp per
// slot, lane l sums blocks l, l+32, ..., then a fixed butterfly (the order is
// the same in every run).
__global__ void k_sum_slots(const double *partials, uint32_t nblocks, uint32_t nslots, const uint32_t *gate_of_slot,
                            double *grads) {
    const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (s >= nslots) return;  // the whole warp leaves together
    double t = 0.0;
    for (uint32_t b = lane; b < nblocks; b += 32) t += partials[(size_t)b * nslots + s];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) grads[gate_of_slot[s]] = t;
}

// ---- host orchestration ----------------------------------------------------------------
// Scratch of the adjoint gradient, kept with the handle between calls:
// lambda, the checkpoints (both only while they are small against the
// device, see adjoint_run), the per-block partials, the gradient, the
// programs and gradient info of every reverse sweep (device, and a pinned
// staging copy uploaded once per call), and the specialised reverse-sweep
// kernels of each segment structure seen.
struct AdjScratch {
    size_t sb = 0;  // state bytes lam/ckpt were made for
    void *lam = nullptr;
    std::vector<void *> ckpt;
    double *partials = nullptr;
    size_t partials_cap = 0;
    double *grads = nullptr;
    size_t grads_cap = 0;
    unsigned char *dprog = nullptr;
    size_t dprog_cap = 0;
    unsigned char *hprog = nullptr;  // pinned
    size_t hprog_cap = 0;
    struct Kernels {
        uint64_t key;
        std::vector<const void *> f;
    };
    std::vector<Kernels> kernels;  // final entries only (compiled, loaded or failed)
    void release_states() {
        if (lam) cudaFree(lam);
        lam = nullptr;
        for (void *c : ckpt) cudaFree(c);
        ckpt.clear();
        sb = 0;
    }
    void release() {
        release_states();
        if (partials) cudaFree(partials);
        if (grads) cudaFree(grads);
        if (dprog) cudaFree(dprog);
        if (hprog) cudaFreeHost(hprog);
        partials = grads = nullptr;
        dprog = hprog = nullptr;
        partials_cap = grads_cap = dprog_cap = hprog_cap = 0;
        kernels.clear();
    }
};
constexpr size_t kAdjKernelEntries = 256;

void release_adjoint(Sim &s) {
    AdjScratch *a = (AdjScratch *)s.adj;
    if (!a) return;
    a->release();
    delete a;
    s.adj = nullptr;
}

template <class B>
static cudaError_t adj_grow(B *&p, size_t &cap, size_t want) {
    if (want <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    const cudaError_t e = cudaMalloc((void **)&p, want);
    if (e == cudaSuccess) cap = want;
    return e;
}

static GateDesc inverse_desc(int prec, const GateDesc &g, double angle) {
    // X, Y, Z, H are their own inverses; P/RX/RY/RZ invert by negating the angle
    switch (g.kind) {
    case G_P:
    case G_RX:
    case G_RY:
    case G_RZ: return make_gate_desc(prec, g.kind, g.target, g.ctrl, -angle);
    default: return g;
    }
}

// One reverse sweep, planned: its parameters (program and gradient info
// pointers filled once the upload buffer exists), the byte offsets of its
// program and info in that buffer, and its specialised kernel (or null).
struct RevSweep {
    AdjParams a;
    size_t prog_off = 0, info_off = 0;
    const void *spec = nullptr;
};

static uint64_t fnv(uint64_t h, const void *p, size_t n) {
    const unsigned char *c = (const unsigned char *)p;
    for (size_t i = 0; i < n; i++) {
        h ^= c[i];
        h *= 1099511628211ull;
    }
    return h;
}

// Plan the reverse sweeps of gates [lo, hi) (inverse gates, last first),
// append their programs and gradient info to the staging bytes, and find
// their specialised kernels (from the handle's cache, else following the
// JIT mode).
template <class P, int K, int R>
static cudaError_t plan_segment(Sim &s, AdjScratch &sc, const std::vector<GateDesc> &fwd,
                                const std::vector<double> &angles, const std::vector<int> &gtype, size_t lo, size_t hi,
                                std::vector<unsigned char> &progs, std::vector<unsigned char> &infos,
                                std::vector<RevSweep> &out) {
    using AK = AdjKernel<P, K, R>;
    std::vector<GateDesc> rev;
    std::vector<size_t> rev_src;
    for (size_t j = hi; j-- > lo;) {
        rev.push_back(inverse_desc(s.prec, fwd[j], angles[j]));
        rev_src.push_back(j);
    }
    const std::vector<PlannedSweep> plan = plan_sweeps(s.n, K, R, rev.data(), rev.size(), false);
    // gradient info per sweep: type | slot << 4 per gate, then the gate of each slot
    std::vector<std::vector<uint32_t>> metas(plan.size());
    uint64_t key = fnv(1469598103934665603ull, AdjPolicyName<P>::s, strlen(AdjPolicyName<P>::s));
    const size_t first = out.size();
    for (size_t k = 0; k < plan.size(); k++) {
        const PlannedSweep &sw = plan[k];
        std::vector<uint32_t> &meta = metas[k];
        meta.assign(sw.gates.size(), 0);
        std::vector<uint32_t> gate_of_slot;
        for (size_t i = 0; i < sw.gates.size(); i++) {
            const size_t j = rev_src[sw.src[i]];
            if (gtype[j] != GT_NONE) {
                meta[i] = (uint32_t)gtype[j] | ((uint32_t)gate_of_slot.size() << 4);
                gate_of_slot.push_back((uint32_t)j);
            }
        }
        RevSweep r;
        memset(&r.a, 0, sizeof r.a);
        r.a.sw.hmask = sw.hmask;
        r.a.sw.l = sw.l;
        r.a.sw.m = sw.m;
        memcpy(r.a.sw.hq, sw.hq, sizeof r.a.sw.hq);
        r.a.sw.nstages = (uint32_t)sw.stage_layout.size();
        r.a.sw.gate_count = (uint32_t)sw.gates.size();
        for (uint32_t i = 0; i < r.a.sw.nstages; i++) {
            r.a.sw.stage_layout[i] = sw.stage_layout[i];
            r.a.sw.stage_end[i] = sw.stage_end[i];
        }
        r.a.sw.err = s.d_err;
        r.a.sw.tiles = 1ull << (s.n - K);
        r.a.nslots = (uint32_t)gate_of_slot.size();
        // structure key: everything the specialised source is written from
        key = fnv(key, &r.a.sw.l, sizeof r.a.sw.l);
        key = fnv(key, &r.a.sw.m, sizeof r.a.sw.m);
        key = fnv(key, sw.hq, sizeof sw.hq);
        key = fnv(key, sw.stage_layout.data(), sw.stage_layout.size());
        key = fnv(key, sw.stage_end.data(), sw.stage_end.size() * sizeof(uint16_t));
        key = fnv(key, meta.data(), meta.size() * sizeof(uint32_t));
        for (const TileGate &t : sw.gates) {
            key = fnv(key, &t, offsetof(TileGate, c));
            if (t.cls == TG_PI) key = fnv(key, &t.c[0], sizeof(double));
        }
        key = fnv(key, "|", 1);
        // program (policy-packed constants) and gradient info into the staging bytes
        r.prog_off = progs.size();
        progs.resize(progs.size() + sw.gates.size() * sizeof(TileGate));
        for (size_t i = 0; i < sw.gates.size(); i++) {
            TileGate t = sw.gates[i];
            P::pack_host(t);
            memcpy(progs.data() + r.prog_off + i * sizeof(TileGate), &t, sizeof t);
        }
        r.info_off = infos.size();
        const size_t nb = (meta.size() + gate_of_slot.size()) * sizeof(uint32_t);
        infos.resize(infos.size() + ((nb + 15) & ~(size_t)15));
        if (!meta.empty()) memcpy(infos.data() + r.info_off, meta.data(), meta.size() * sizeof(uint32_t));
        if (!gate_of_slot.empty())
            memcpy(infos.data() + r.info_off + meta.size() * sizeof(uint32_t), gate_of_slot.data(),
                   gate_of_slot.size() * sizeof(uint32_t));
        out.push_back(r);
    }
    // specialised reverse sweeps (the handle's JIT mode, as for the forward
    // sweeps); a sweep without one runs the compiled k_adjoint
    if (s.jit_mode == KBWG_JIT_OFF) return cudaSuccess;
    key = fnv(key, &s.jit_mode, sizeof s.jit_mode);
    for (const AdjScratch::Kernels &kc : sc.kernels)
        if (kc.key == key && kc.f.size() == plan.size()) {
            for (size_t k = 0; k < plan.size(); k++) out[first + k].spec = kc.f[k];
            return cudaSuccess;
        }
    const JitGeometry geo{AdjPolicyName<P>::s, K, R, AK::kThreads, 2};
    std::vector<std::string> srcs;
    for (size_t k = 0; k < plan.size(); k++) srcs.push_back(jit_adjoint_source(geo, plan[k], metas[k]));
    bool final = false;
    const std::vector<const void *> jk = specialised_kernels(s, srcs, "kbwg_jit_adjoint", &final);
    for (size_t k = 0; k < plan.size(); k++) {
        const void *f = jk.empty() ? nullptr : jk[k];
        if (!f) continue;
        cudaError_t e = ensure_smem_limit(f, AK::kSmem);
        if (e != cudaSuccess) return e;
        out[first + k].spec = f;
    }
    if (final) {
        if (sc.kernels.size() >= kAdjKernelEntries) sc.kernels.erase(sc.kernels.begin());
        sc.kernels.push_back({key, jk});
    }
    return cudaSuccess;
}

// Launch the planned reverse sweeps of one segment (programs already uploaded).
template <class P, int K, int R>
static cudaError_t run_segment(Sim &s, AdjScratch &sc, std::vector<RevSweep> &sweeps,
                               const std::vector<uint64_t> &grids, size_t from, size_t to) {
    using AK = AdjKernel<P, K, R>;
    using Mem = typename P::Mem;
    for (size_t k = from; k < to; k++) {
        RevSweep &r = sweeps[k];
        const uint64_t grid = grids[k];
        if (s.prof.on) s.prof.mark(s.stream);
        cudaError_t e;
        if (r.spec) {
            Mem *ph = (Mem *)s.state, *la = (Mem *)sc.lam;
            void *args[] = {(void *)&ph, (void *)&la, (void *)&r.a};
            e = cudaLaunchKernel(r.spec, dim3((unsigned)grid), dim3(AK::kThreads), args, AK::kSmem, s.stream);
        } else {
            if (s.n > 32)
                k_adjoint<P, K, R, true><<<(unsigned)grid, AK::kThreads, AK::kSmem, s.stream>>>(
                    (Mem *)s.state, (Mem *)sc.lam, r.a);
            else
                k_adjoint<P, K, R><<<(unsigned)grid, AK::kThreads, AK::kSmem, s.stream>>>((Mem *)s.state, (Mem *)sc.lam,
                                                                                    r.a);
            e = cudaGetLastError();
        }
        count_launch();
        if (s.prof.on) {
            s.prof.mark(s.stream);
            s.prof.bytes += 4.0 * (double)s.elem * (double)s.ns;
        }
        if (e != cudaSuccess) return e;
        if (r.a.nslots) {
            k_sum_slots<<<(r.a.nslots + 3) / 4, 128, 0, s.stream>>>(sc.partials, (uint32_t)grid, r.a.nslots,
                                                                    r.a.ginfo + r.a.sw.gate_count, sc.grads);
            count_launch();
            e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

// lambda = H phi in tiled passes (ring TFIM at 24 qubits: 3 passes instead
// of one per flip mask); strings too wide for a tile fall back to one pass
// per flip mask.
template <class T>
static cudaError_t apply_hamiltonian_tiled(Sim &s, void *lam, const std::vector<PauliString> &H, bool &done) {
    done = false;
    const int K = kApplyTileBits;
    if (s.n < (uint32_t)K + 1 || H.empty()) return cudaSuccess;
    std::vector<uint64_t> xm;
    for (const PauliString &t : H) xm.push_back(t.x);
    std::vector<size_t> wide;
    const std::vector<PauliPass> passes = plan_pauli_passes(s.n, K, xm, kMaxTerms, wide);
    if (!wide.empty()) return cudaSuccess;
    const size_t smem = (sizeof(cx<T>) << K) + (sizeof(uint64_t) << (K - kLaneBits));
    {
        const cudaError_t e = ensure_smem_limit((const void *)k_apply_tile<T>, smem);
        if (e != cudaSuccess) return e;
    }
    const uint64_t tiles = 1ull << (s.n - K);
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, 152ull * 8);
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const PauliPass &pp = passes[pi];
        ApplyTilePass a;
        memset(&a, 0, sizeof a);
        a.K = (uint32_t)K;
        a.l = pp.l;
        a.m = pp.m;
        a.init = pi == 0 ? 1u : 0u;
        memcpy(a.hq, pp.hq, sizeof a.hq);
        for (size_t j = 0; j < pp.members.size(); j++) {
            const PauliString &t = H[pp.members[j]];
            ApplyTileTerm &tt = a.t[j];
            tt.xl = pp.local(t.x);
            tt.zl = pp.local(t.z & pp.tile_mask);
            tt.zo = t.z & ~pp.tile_mask;
            const int q = t.ny & 3;  // i^ny
            tt.cre = (q == 0) ? t.coef : (q == 2 ? -t.coef : 0.0);
            tt.cim = (q == 1) ? t.coef : (q == 3 ? -t.coef : 0.0);
        }
        a.nterms = (uint32_t)pp.members.size();
        k_apply_tile<T><<<grid, 256, smem, s.stream>>>((const cx<T> *)s.state, (cx<T> *)lam, s.n, a);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    done = true;
    return cudaSuccess;
}

template <class T>
static cudaError_t apply_hamiltonian(Sim &s, void *lam, const std::vector<ApplyGroup> &groups) {
    const uint64_t ns = s.ns;
    uint64_t g = (ns + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    for (const ApplyGroup &ag : groups) {
        k_apply_group<T><<<(unsigned)g, 256, 0, s.stream>>>((const cx<T> *)s.state, (cx<T> *)lam, ns, ag);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The same passes on float-float resident states: each pass's strings are
// ordered into runs of one coefficient (Z-type real, real with flips,
// complex), the form k_apply_tile_ff sums.
static cudaError_t apply_hamiltonian_tiled_ff(Sim &s, void *lam, const std::vector<PauliString> &H, bool &done,
                                              bool c64 = false) {
    done = false;
    const int K = kApplyTileBits;
    if (s.n < (uint32_t)K + 1 || H.empty()) return cudaSuccess;
    std::vector<uint64_t> xm;
    for (const PauliString &t : H) xm.push_back(t.x);
    std::vector<size_t> wide;
    const std::vector<PauliPass> passes = plan_pauli_passes(s.n, K, xm, kMaxTerms, wide);
    if (!wide.empty()) return cudaSuccess;
    const size_t smem = ((c64 ? sizeof(cx<float>) : sizeof(ff2::v2)) << K) + (sizeof(uint64_t) << (K - kLaneBits));
    {
        const cudaError_t e =
            ensure_smem_limit(c64 ? (const void *)k_apply_tile_f32 : (const void *)k_apply_tile_ff, smem);
        if (e != cudaSuccess) return e;
    }
    const uint64_t tiles = 1ull << (s.n - K);
    const unsigned grid = (unsigned)std::min<uint64_t>(tiles, 152ull * 8);
    for (size_t pi = 0; pi < passes.size(); pi++) {
        const PauliPass &pp = passes[pi];
        ApplyTilePassFF a;
        memset(&a, 0, sizeof a);
        a.K = (uint32_t)K;
        a.l = pp.l;
        a.m = pp.m;
        a.init = pi == 0 ? 1u : 0u;
        memcpy(a.hq, pp.hq, sizeof a.hq);
        struct Item {
            ApplyTileTermFF t;
            double cre, cim;
        };
        std::vector<Item> items;
        for (size_t j = 0; j < pp.members.size(); j++) {
            const PauliString &ps = H[pp.members[j]];
            Item it;
            memset(&it, 0, sizeof it);
            it.t.xl = pp.local(ps.x);
            it.t.zl = pp.local(ps.z & pp.tile_mask);
            it.t.zo = ps.z & ~pp.tile_mask;
            const int q = ps.ny & 3;  // i^ny
            it.cre = (q == 0) ? ps.coef : (q == 2 ? -ps.coef : 0.0);
            it.cim = (q == 1) ? ps.coef : (q == 3 ? -ps.coef : 0.0);
            it.t.cat = it.cim != 0.0 ? 2u : (it.t.xl == 0u ? 0u : 1u);
            const ff::f2 r = ff::split_constant(it.cre), i = ff::split_constant(it.cim);
            it.t.rh = r.h;
            it.t.rl = r.l;
            it.t.ih = i.h;
            it.t.il = i.l;
            items.push_back(it);
        }
        std::stable_sort(items.begin(), items.end(), [](const Item &x, const Item &y) {
            if (x.t.cat != y.t.cat) return x.t.cat < y.t.cat;
            if (x.cre != y.cre) return x.cre < y.cre;
            return x.cim < y.cim;
        });
        for (size_t j = 0; j < items.size(); j++) {
            const bool end = j + 1 == items.size() || items[j + 1].t.cat != items[j].t.cat ||
                             items[j + 1].cre != items[j].cre || items[j + 1].cim != items[j].cim;
            items[j].t.last = end ? 1u : 0u;
            a.t[j] = items[j].t;
        }
        a.nterms = (uint32_t)items.size();
        if (c64)
            k_apply_tile_f32<<<grid, 256, smem, s.stream>>>((const cx<float> *)s.state, (cx<float> *)lam, s.n, a);
        else
            k_apply_tile_ff<<<grid, 256, smem, s.stream>>>((const ff2::v2 *)s.state, (ff2::v2 *)lam, s.n, a);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    done = true;
    return cudaSuccess;
}

static cudaError_t apply_hamiltonian_ff(Sim &s, void *lam, const std::vector<ApplyGroup> &groups) {
    uint64_t g = (s.ns + 255) / 256;
    if (g > 152 * 8) g = 152 * 8;
    for (const ApplyGroup &ag : groups) {
        k_apply_group_ff<<<(unsigned)g, 256, 0, s.stream>>>((const ff2::v2 *)s.state, (ff2::v2 *)lam, s.ns, ag);
        count_launch();
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

static cudaError_t inner_re_ff_async(Sim &s, const void *a, const void *b) {
    k_inner_re_ff<<<kReduceBlocks, 256, 0, s.stream>>>((const ff2::v2 *)a, (const ff2::v2 *)b, s.ns, s.rs.partials,
                                                        s.rs.ticket, s.rs.result);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return copy_async(s.h_result, s.rs.result, sizeof(double), cudaMemcpyDeviceToHost, s.stream);
}

// Re<a|b> into the handle's pinned result slot; readable after the stream's
// next synchronisation.
template <class T>
static cudaError_t inner_re_async(Sim &s, const void *a, const void *b) {
    k_inner_re<T><<<kReduceBlocks, 256, 0, s.stream>>>((const cx<T> *)a, (const cx<T> *)b, s.ns, s.rs.partials,
                                                        s.rs.ticket, s.rs.result);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return copy_async(s.h_result, s.rs.result, sizeof(double), cudaMemcpyDeviceToHost, s.stream);
}

static std::vector<ApplyGroup> make_groups(const std::vector<PauliString> &H) {
    std::vector<size_t> order(H.size());
    for (size_t k = 0; k < H.size(); k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return H[a].x < H[b].x; });
    std::vector<ApplyGroup> groups;
    size_t i = 0;
    while (i < order.size()) {
        ApplyGroup g;
        memset(&g, 0, sizeof g);
        g.x = H[order[i]].x;
        while (i < order.size() && H[order[i]].x == g.x && g.nterms < (uint32_t)kMaxTerms) {
            const PauliString &t = H[order[i]];
            const int k = (int)g.nterms++;
            g.z[k] = t.z;
            const int m = t.ny & 3;  // i^ny
            g.cre[k] = (m == 0) ? t.coef : (m == 2 ? -t.coef : 0.0);
            g.cim[k] = (m == 1) ? t.coef : (m == 3 ? -t.coef : 0.0);
            i++;
        }
        g.init = groups.empty() ? 1u : 0u;
        groups.push_back(g);
    }
    if (groups.empty()) {  // H = 0
        ApplyGroup g;
        memset(&g, 0, sizeof g);
        g.init = 1;
        groups.push_back(g);
    }
    return groups;
}

template <class P, class T, int K, int R>
static int32_t adjoint_run(Sim &s, const std::vector<GateDesc> &fwd, const std::vector<double> &angles,
                           const std::vector<int> &gtype, const std::vector<PauliString> &H, double *energy,
                           std::vector<double> &grad_per_gate, uint32_t max_ckpt) {
    using AK = AdjKernel<P, K, R>;
    // float-float resident: the forward state, the checkpoints, lambda and
    // the reverse sweeps all keep the forward sweeps' float-float form
    constexpr bool kFF = std::is_same<P, FF2>::value;
    if (!s.adj) s.adj = new AdjScratch();
    AdjScratch &sc = *(AdjScratch *)s.adj;
    auto fail_cuda = [&](cudaError_t e, const char *what) {
        cudaGetLastError();
        cudaStreamSynchronize(s.stream);
        sc.release();  // (nothing of it is in flight any more)
        cudaGetLastError();
        set_error(e == cudaErrorMemoryAllocation ? KBWG_ENOMEM : KBWG_ECUDA,
                  std::string("adjoint: ") + what + ": " + cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? (int32_t)KBWG_ENOMEM : (int32_t)KBWG_ECUDA;
    };
    const size_t M = fwd.size();
    const size_t sb = (size_t)s.ns * s.elem;
    int dev = 0, num_sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev);
    const void *kadj = s.n > 32 ? (const void *)k_adjoint<P, K, R, true> : (const void *)k_adjoint<P, K, R>;
    if (e == cudaSuccess) e = ensure_smem_limit(kadj, AK::kSmem);
    if (e != cudaSuccess) return fail_cuda(e, "device query");
    // scratch (kept from an earlier call when it is there)
    if (sc.sb != sb) sc.release_states();
    if (!sc.lam) {
        e = cudaMalloc(&sc.lam, sb);
        if (e != cudaSuccess) return fail_cuda(e, "lambda buffer");
        sc.sb = sb;
    }
    e = adj_grow(sc.partials, sc.partials_cap, (size_t)num_sms * 8 * kMaxSweepGates * sizeof(double));
    if (e == cudaSuccess) e = adj_grow(sc.grads, sc.grads_cap, std::max<size_t>(M, 1) * sizeof(double));
    if (e != cudaSuccess) return fail_cuda(e, "scratch");
    // checkpoints: at most max_ckpt, new ones only while they fit in 80% of
    // the free memory
    const size_t want = std::min<size_t>(max_ckpt, M > 1 ? M - 1 : 0);
    size_t free_b = 0, total_b = 0;
    e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return fail_cuda(e, "memory query");
    while (sc.ckpt.size() < want && sb <= (size_t)(0.8 * (double)free_b)) {
        void *c = nullptr;
        if (cudaMalloc(&c, sb) != cudaSuccess) {
            cudaGetLastError();
            break;
        }
        sc.ckpt.push_back(c);
        free_b -= std::min(free_b, sb);
    }
    const size_t S = std::min(want, sc.ckpt.size()) + 1;
    std::vector<size_t> b(S + 1);
    for (size_t i = 0; i <= S; i++) b[i] = i * M / S;

    // 1. forward from |0>
    s.queue.clear();
    e = init_state(s);
    if (e != cudaSuccess) return fail_cuda(e, "init");
    for (size_t seg = 0; seg < S; seg++) {
        s.queue.assign(fwd.begin() + b[seg], fwd.begin() + b[seg + 1]);
        e = flush_queue(s);
        if (e != cudaSuccess) return fail_cuda(e, "forward");
        if (seg + 1 < S) {
            // checkpoints are copies in the reverse sweeps' form (float-float
            // for FF2, binary64 otherwise)
            if (kFF && !s.ff_resident) {
                e = launch_ff_convert(s.state, s.n, true, s.stream);
                if (e != cudaSuccess) return fail_cuda(e, "checkpoint");
                s.ff_resident = true;
            }
            if (!kFF) e = ensure_binary64(s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(sc.ckpt[seg], s.state, sb, cudaMemcpyDeviceToDevice, s.stream);
            if (e != cudaSuccess) return fail_cuda(e, "checkpoint");
        }
    }
    // plan every reverse sweep while the GPU runs the forward pass; their
    // programs and gradient info go up in one copy from pinned memory
    std::vector<unsigned char> progs, infos;
    std::vector<RevSweep> sweeps;
    std::vector<size_t> seg_first(S + 1, 0);
    for (size_t seg = S; seg-- > 0;) {
        seg_first[seg + 1] = sweeps.size();  // (segments run last first)
        e = plan_segment<P, K, R>(s, sc, fwd, angles, gtype, b[seg], b[seg + 1], progs, infos, sweeps);
        if (e != cudaSuccess) return fail_cuda(e, "reverse plan");
    }
    const size_t up = progs.size() + infos.size();
    if (up > sc.hprog_cap) {
        if (sc.hprog) cudaFreeHost(sc.hprog);
        sc.hprog = nullptr;
        sc.hprog_cap = 0;
        e = cudaHostAlloc((void **)&sc.hprog, up, cudaHostAllocDefault);
        if (e != cudaSuccess) return fail_cuda(e, "staging buffer");
        sc.hprog_cap = up;
    }
    e = adj_grow(sc.dprog, sc.dprog_cap, std::max<size_t>(up, 16));
    if (e != cudaSuccess) return fail_cuda(e, "program buffer");
    if (up) {
        memcpy(sc.hprog, progs.data(), progs.size());
        if (!infos.empty()) memcpy(sc.hprog + progs.size(), infos.data(), infos.size());
        e = copy_async(sc.dprog, sc.hprog, up, cudaMemcpyHostToDevice, s.stream);
        if (e != cudaSuccess) return fail_cuda(e, "program upload");
    }
    // one grid per kernel: as many CTAs as fit (the partials buffer holds 8 per SM)
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kadj, AK::kThreads, AK::kSmem);
    if (e != cudaSuccess) return fail_cuda(e, "occupancy");
    const uint64_t tiles = 1ull << (s.n - K);
    std::vector<std::pair<const void *, uint64_t>> grids;
    auto grid_of = [&](const void *f) -> uint64_t {
        for (const auto &g : grids)
            if (g.first == f) return g.second;
        int o = occ;
        if (f && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, f, AK::kThreads, AK::kSmem) != cudaSuccess) {
            cudaGetLastError();
            o = occ;
        }
        const uint64_t g = std::min<uint64_t>(tiles, (uint64_t)num_sms * std::min(std::max(o, 1), 8));
        grids.emplace_back(f, g);
        return g;
    };
    std::vector<uint64_t> grid(sweeps.size());
    for (size_t k = 0; k < sweeps.size(); k++) {
        RevSweep &r = sweeps[k];
        r.a.sw.prog = (const TileGate *)(sc.dprog + r.prog_off);
        r.a.ginfo = (const uint32_t *)(sc.dprog + progs.size() + r.info_off);
        r.a.partials = sc.partials;
        grid[k] = grid_of(r.spec);
    }
    if (kFF) {
        if (!s.ff_resident) {
            e = launch_ff_convert(s.state, s.n, true, s.stream);
            s.ff_resident = true;
        }
    } else {
        e = ensure_binary64(s);  // lambda and the reverse sweeps use binary64
    }
    if (e != cudaSuccess) return fail_cuda(e, "forward");
    // 2. lambda = H phi, E = Re<phi|lambda>
    bool tiled = false;
    if (kFF) {
        e = apply_hamiltonian_tiled_ff(s, sc.lam, H, tiled);
        if (e == cudaSuccess && !tiled) e = apply_hamiltonian_ff(s, sc.lam, make_groups(H));
    } else {
        if constexpr (sizeof(T) == 4)  // complex64: the run form of the float-float pass, in float
            e = apply_hamiltonian_tiled_ff(s, sc.lam, H, tiled, true);
        else
            e = apply_hamiltonian_tiled<T>(s, sc.lam, H, tiled);
        if (e == cudaSuccess && !tiled) e = apply_hamiltonian<T>(s, sc.lam, make_groups(H));
    }
    if (e != cudaSuccess) return fail_cuda(e, "H|phi>");
    e = kFF ? inner_re_ff_async(s, s.state, sc.lam) : inner_re_async<T>(s, s.state, sc.lam);
    if (e != cudaSuccess) return fail_cuda(e, "energy");
    // 3. reverse, segment by segment
    e = cudaMemsetAsync(sc.grads, 0, std::max<size_t>(M, 1) * sizeof(double), s.stream);
    if (e != cudaSuccess) return fail_cuda(e, "gradient buffer");
    for (size_t seg = S; seg-- > 0;) {
        const size_t from = seg_first[seg + 1], to = seg > 0 ? seg_first[seg] : sweeps.size();
        e = run_segment<P, K, R>(s, sc, sweeps, grid, from, to);
        if (e != cudaSuccess) return fail_cuda(e, "reverse sweep");
        if (seg > 0) {
            e = cudaMemcpyAsync(s.state, sc.ckpt[seg - 1], sb, cudaMemcpyDeviceToDevice, s.stream);
            if (e != cudaSuccess) return fail_cuda(e, "checkpoint reload");
        }
    }
    grad_per_gate.assign(M, 0.0);
    if (M) {
        e = copy_async(grad_per_gate.data(), sc.grads, M * sizeof(double), cudaMemcpyDeviceToHost, s.stream);
        if (e != cudaSuccess) return fail_cuda(e, "gradient read-back");
    }
    // leave the handle in |0...0>
    e = init_state(s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
    if (e != cudaSuccess) return fail_cuda(e, "finish");
    *energy = s.h_result[0];
    // lambda and the checkpoints stay for the next call while they are small
    // against the device (a sixteenth of its memory); larger ones go now
    if (sb * (1 + sc.ckpt.size()) > total_b / 16) sc.release_states();
    return KBWG_OK;
}

// ---- compile-only check of the specialised reverse sweeps (no GPU) ----------------
template <class P, int K, int R>
static size_t check_adjoint_p(const Sim &s, const std::vector<GateDesc> &fwd, const std::vector<int> &gtype,
                              size_t &sweeps) {
    using AK = AdjKernel<P, K, R>;
    std::vector<GateDesc> rev;
    std::vector<size_t> rev_src;
    for (size_t j = fwd.size(); j-- > 0;) {
        rev.push_back(fwd[j]);  // (the structure of the inverse gate is the gate's)
        rev_src.push_back(j);
    }
    const std::vector<PlannedSweep> plan = plan_sweeps(s.n, K, R, rev.data(), rev.size(), false);
    const JitGeometry geo{AdjPolicyName<P>::s, K, R, AK::kThreads, 2};
    std::vector<std::string> srcs;
    for (const PlannedSweep &sw : plan) {
        std::vector<uint32_t> meta(sw.gates.size(), 0);
        uint32_t nslots = 0;
        for (size_t i = 0; i < sw.gates.size(); i++) {
            const size_t j = rev_src[sw.src[i]];
            if (gtype[j] != GT_NONE) meta[i] = (uint32_t)gtype[j] | (nslots++ << 4);
        }
        srcs.push_back(jit_adjoint_source(geo, sw, meta));
    }
    sweeps = plan.size();
    return jit_compile_only(srcs);
}

size_t jit_check_adjoint(const Sim &s, const std::vector<GateDesc> &fwd, const std::vector<int> &gtype,
                         size_t &sweeps) {
    sweeps = 0;
    if (s.prec == 0) {
        if (s.n < (uint32_t)AdjCfg<float>::K) return 0;
        return check_adjoint_p<FastP, AdjCfg<float>::K, AdjCfg<float>::R>(s, fwd, gtype, sweeps);
    }
    if (s.n < (uint32_t)AdjCfg<double>::K) return 0;
    if (ff_capable(s))
        return check_adjoint_p<FF2, AdjCfg<double>::K, AdjCfg<double>::R>(s, fwd, gtype, sweeps);
    if (s.flags & KBWG_FLAG_FAST_C128)
        return check_adjoint_p<FF2B, AdjCfg<double>::K, AdjCfg<double>::R>(s, fwd, gtype, sweeps);
    return check_adjoint_p<Fast<double>, AdjCfg<double>::K, AdjCfg<double>::R>(s, fwd, gtype, sweeps);
}

int32_t adjoint_gradient(Sim &s, const std::vector<GateDesc> &fwd, const std::vector<double> &angles,
                         const std::vector<int> &gtype, const std::vector<PauliString> &H, double *energy,
                         std::vector<double> &grad_per_gate, uint32_t max_ckpt) {
    // (above 32 qubits the reverse sweeps read gate bits of a 64-bit tile
    // base; memory decides how far: the state, lambda and the checkpoints)
    if (s.n < (uint32_t)AdjCfg<float>::K || (s.prec && s.n < (uint32_t)AdjCfg<double>::K)) {
        set_error(KBWG_EUNSUPPORTED, "adjoint: needs at least 12 qubits (complex64) or 11 (complex128)");
        return KBWG_EUNSUPPORTED;
    }
    if (s.prec == 0)
        return adjoint_run<FastP, float, AdjCfg<float>::K, AdjCfg<float>::R>(s, fwd, angles, gtype, H, energy,
                                                                                 grad_per_gate, max_ckpt);
    if (ff_capable(s))  // the forward state stays float-float
        return adjoint_run<FF2, double, AdjCfg<double>::K, AdjCfg<double>::R>(s, fwd, angles, gtype, H, energy,
                                                                            grad_per_gate, max_ckpt);
    if (s.flags & KBWG_FLAG_FAST_C128)
        return adjoint_run<FF2B, double, AdjCfg<double>::K, AdjCfg<double>::R>(s, fwd, angles, gtype, H, energy,
                                                                             grad_per_gate, max_ckpt);
    return adjoint_run<Fast<double>, double, AdjCfg<double>::K, AdjCfg<double>::R>(s, fwd, angles, gtype, H, energy,
                                                                                grad_per_gate, max_ckpt);
}

}  // namespace kbwg
