// FP64 reduction kernels (Pauli expectations, norms), shared by the engine
// and the allocation-free entry point.
#pragma once
#include "device.cuh"
#include "kernels.h"

namespace qsv {

// ---------------------------------------------------------------------------
// FP64 reductions
// ---------------------------------------------------------------------------
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NT / 32; ++i) s += red[i];
    }
    return s;  // valid in thread 0
}

// Z-only Pauli terms: sum_j |a_j|^2 (-1)^popcount(j & z_t)  (statevector.hpp:1281-1290)
template <class P>
__global__ void __launch_bounds__(256) k_expect_z(const typename P::G* __restrict__ state, uint64_t N,
                                                  const uint64_t* __restrict__ zm, int nterms,
                                                  double* __restrict__ partial) {
    __shared__ double red[8];
    double acc[EXPECT_BATCH];
#pragma unroll
    for (int t = 0; t < EXPECT_BATCH; ++t) acc[t] = 0.0;
    uint64_t zl[EXPECT_BATCH];
#pragma unroll
    for (int t = 0; t < EXPECT_BATCH; ++t) zl[t] = t < nterms ? zm[t] : 0;
    for (uint64_t j = blockIdx.x * 256ULL + threadIdx.x; j < N; j += gridDim.x * 256ULL) {
        const typename P::G g = state[j];
        const double re = P::gre(g), im = P::gim(g);
        const double p = __fma_rn(re, re, __dmul_rn(im, im));
#pragma unroll
        for (int t = 0; t < EXPECT_BATCH; ++t)
            if (t < nterms) acc[t] += (__popcll(j & zl[t]) & 1) ? -p : p;
    }
    for (int t = 0; t < nterms; ++t) {
        const double s = block_sum<256>(acc[t], red);
        if (threadIdx.x == 0) partial[static_cast<size_t>(blockIdx.x) * EXPECT_BATCH + t] = s;
    }
}

// Terms sharing one flip mask x: sum over pairs (i0, i0^x) of
// 2 Re(a_i0 conj(a_i1) phase) (statevector.hpp:1291-1304)
template <class P>
__global__ void __launch_bounds__(256) k_expect_x(const typename P::G* __restrict__ state, uint64_t N, uint64_t xmask,
                                                  int flip_q, const uint64_t* __restrict__ zm,
                                                  const int32_t* __restrict__ ny, int nterms,
                                                  double* __restrict__ partial) {
    __shared__ double red[8];
    double acc[EXPECT_BATCH];
    uint64_t zl[EXPECT_BATCH];
    int yl[EXPECT_BATCH];
#pragma unroll
    for (int t = 0; t < EXPECT_BATCH; ++t) {
        acc[t] = 0.0;
        zl[t] = t < nterms ? zm[t] : 0;
        yl[t] = t < nterms ? ny[t] : 0;
    }
    const uint64_t half = N >> 1;
    for (uint64_t j = blockIdx.x * 256ULL + threadIdx.x; j < half; j += gridDim.x * 256ULL) {
        const uint64_t i0 = insert0(j, flip_q), i1 = i0 ^ xmask;
        const typename P::G a = state[i0], b = state[i1];
        const double ar = P::gre(a), ai = P::gim(a), br = P::gre(b), bi = P::gim(b);
        // v = a * conj(b)
        const double vr = __fma_rn(ar, br, __dmul_rn(ai, bi));
        const double vi = __fma_rn(ai, br, -__dmul_rn(ar, bi));
#pragma unroll
        for (int t = 0; t < EXPECT_BATCH; ++t) {
            if (t < nterms) {
                const int ph = ((__popcll(i0 & zl[t]) & 1) * 2 + yl[t]) & 3;
                const double c = (ph == 0) ? vr : (ph == 1) ? -vi : (ph == 2) ? -vr : vi;
                acc[t] += 2.0 * c;
            }
        }
    }
    for (int t = 0; t < nterms; ++t) {
        const double s = block_sum<256>(acc[t], red);
        if (threadIdx.x == 0) partial[static_cast<size_t>(blockIdx.x) * EXPECT_BATCH + t] = s;
    }
}

static __global__ void k_reduce_partials(const double* __restrict__ partial, int nblocks, int nterms,
                                  double* __restrict__ out) {
    __shared__ double red[8];
    for (int t = 0; t < nterms; ++t) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nblocks; b += 256) s += partial[static_cast<size_t>(b) * EXPECT_BATCH + t];
        s = block_sum<256>(s, red);
        if (threadIdx.x == 0) out[t] = s;
    }
}

}  // namespace qsv
