// Exact shot sampling in parallel.
//
// The reference draws a shot by scanning the state in index order with an
// FP64 running sum, p = fl(p + q_i), q_i = fl(fl(re^2) + fl(im^2)), and
// returning the first i with r < p (N when there is none;
// statevector.hpp:1380-1412).  That sum is sequential, but its rounding has
// structure: while p stays inside one binade [2^e, 2^(e+1)), p is a multiple
// of G = 2^(e-52) and fl(p + q) = p + G * round(q / G), the rounding of q
// alone onto the grid G (independent of p), except for exact ties, whose
// round-half-even direction depends on p's last bit.  So:
//
//   1. k_binade_counts (all SMs): for every block of SAMPLE_BS elements and
//      every candidate binade e of the top BINADES binades below the total,
//      the saturating sum of round(q_i / 2^(e-52)) and whether a tie occurs.
//   2. k_binade_scan (one warp): walks the blocks in order keeping the exact
//      running sum; a block that stays inside the current binade and has no
//      tie advances it by one integer addition (32 blocks per step with a warp
//      scan); a block that crosses a binade, holds a tie, or starts below the
//      candidate range is summed element by element with the reference's own
//      FP64 additions.  Output: the exact running sum at every block start.
//   3. k_sample_blocks (a warp per shot): binary search of the block whose
//      exact end exceeds r, then the reference's sequential additions inside
//      that block from its exact start.
//
// Every value is the reference's own FP64 running sum, so every sampled index
// equals the sequential scan's, with no uncertain case left.  All loops are
// bounded by the state length.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.h"
#include "policy.cuh"

namespace qsv {

namespace {

constexpr uint64_t KCAP = 1ULL << 60;  // saturation of grid counts (any binade has < 2^53 steps)
constexpr uint64_t MTOP = 1ULL << 53;  // a binade's grid has 2^52 .. 2^53 - 1 steps from 0

template <class P>
__device__ __forceinline__ double qprob(const typename P::G g) {
    const double re = P::gre(g), im = P::gim(g);
    return __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
}

__device__ __forceinline__ uint64_t sat_add(uint64_t a, uint64_t b) {
    const uint64_t s = a + b;  // a, b <= KCAP: no wrap
    return s > KCAP ? KCAP : s;
}

// round(q / 2^(e-52)) for q >= 0 (nearest; *tie when q sits exactly half-way)
__device__ __forceinline__ uint64_t grid_count(double q, int e, bool* tie) {
    const uint64_t bits = static_cast<uint64_t>(__double_as_longlong(q));
    const int ex = static_cast<int>((bits >> 52) & 0x7FF);
    uint64_t mant = bits & ((1ULL << 52) - 1);
    int eb = 1;
    if (ex != 0) {
        mant |= 1ULL << 52;
        eb = ex;
    }
    *tie = false;
    if (mant == 0) return 0;
    const int sh = eb - 1023 - e;  // q / G = mant * 2^sh
    if (sh >= 0) return sh >= 7 ? KCAP : (mant << sh);
    const int d = -sh;
    if (d > 54) return 0;  // q < G / 4
    const uint64_t qi = d >= 64 ? 0 : (mant >> d);
    const uint64_t rem = mant & ((1ULL << d) - 1);
    const uint64_t half = 1ULL << (d - 1);
    *tie = rem == half;
    return qi + (rem > half ? 1 : 0);
}

__device__ __forceinline__ int binade_of(double p) {  // p > 0 normal
    return static_cast<int>((static_cast<uint64_t>(__double_as_longlong(p)) >> 52) & 0x7FF) - 1023;
}

template <class P>
__global__ void __launch_bounds__(256) k_binade_counts(const typename P::G* __restrict__ state, uint64_t N,
                                                       int e_top, uint64_t* __restrict__ cnt,
                                                       uint8_t* __restrict__ ties, uint64_t nb) {
    __shared__ uint64_t red[8][SAMPLE_BINADES];
    __shared__ uint32_t tred[8];
    for (uint64_t b = blockIdx.x; b < nb; b += gridDim.x) {
        uint64_t acc[SAMPLE_BINADES];
        uint32_t tie_bits = 0;
#pragma unroll
        for (int c = 0; c < SAMPLE_BINADES; ++c) acc[c] = 0;
        const uint64_t i0 = b * SAMPLE_BS, i1 = (i0 + SAMPLE_BS < N) ? i0 + SAMPLE_BS : N;
        for (uint64_t i = i0 + threadIdx.x; i < i1; i += 256) {
            const double q = qprob<P>(state[i]);
#pragma unroll
            for (int c = 0; c < SAMPLE_BINADES; ++c) {
                bool t;
                acc[c] = sat_add(acc[c], grid_count(q, e_top - c, &t));
                tie_bits |= t ? (1u << c) : 0u;
            }
        }
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
        for (int c = 0; c < SAMPLE_BINADES; ++c) {
            uint64_t v = acc[c];
            for (int o = 16; o; o >>= 1) v = sat_add(v, __shfl_xor_sync(0xffffffffu, v, o));
            if (lane == 0) red[w][c] = v;
        }
        for (int o = 16; o; o >>= 1) tie_bits |= __shfl_xor_sync(0xffffffffu, tie_bits, o);
        if (lane == 0) tred[w] = tie_bits;
        __syncthreads();
        if (threadIdx.x < SAMPLE_BINADES) {
            uint64_t v = 0;
            for (int k = 0; k < 8; ++k) v = sat_add(v, red[k][threadIdx.x]);
            cnt[static_cast<uint64_t>(threadIdx.x) * nb + b] = v;
        }
        if (threadIdx.x == 0) {
            uint32_t t = 0;
            for (int k = 0; k < 8; ++k) t |= tred[k];
            for (int c = 0; c < SAMPLE_BINADES; ++c) ties[static_cast<uint64_t>(c) * nb + b] = (t >> c) & 1u;
        }
        __syncthreads();
    }
}

// One warp: the exact running sum at every block start (start[b], b = 0..nb;
// start[nb] is the sum over the whole state).  *seq counts the blocks summed
// element by element.
template <class P>
__global__ void __launch_bounds__(32) k_binade_scan(const typename P::G* __restrict__ state, uint64_t N, int e_top,
                                                    const uint64_t* __restrict__ cnt, const uint8_t* __restrict__ ties,
                                                    uint64_t nb, double* __restrict__ start, int64_t* __restrict__ seq) {
    const int lane = threadIdx.x;
    double p = 0.0;
    int64_t nseq = 0;
    uint64_t b = 0;
    while (b < nb) {
        int c = -1;
        if (p > 0.0) {
            const int e = binade_of(p);
            if (e <= e_top && e > e_top - SAMPLE_BINADES) c = e_top - e;
        }
        if (c >= 0) {
            // up to 32 whole blocks inside the current binade at once
            const int e = e_top - c;
            const uint64_t m = static_cast<uint64_t>(ldexp(p, 52 - e));  // exact: p is on the grid 2^(e-52)
            const uint64_t bj = b + lane;
            const bool have = bj < nb;
            const uint64_t k = have ? cnt[static_cast<uint64_t>(c) * nb + bj] : 0;
            const bool tie = have ? ties[static_cast<uint64_t>(c) * nb + bj] != 0 : true;
            uint64_t incl = k;
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl = sat_add(incl, y);
            }
            const uint64_t excl = incl - k;
            const bool ok = have && !tie && m + incl < MTOP;  // the block ends inside the binade
            const unsigned bad = __ballot_sync(0xffffffffu, !ok);
            const int nok = bad ? __ffs(bad) - 1 : 32;
            if (lane < nok) start[bj] = ldexp(static_cast<double>(m + excl), e - 52);
            if (nok > 0) {
                const uint64_t tot = __shfl_sync(0xffffffffu, incl, nok - 1);
                p = ldexp(static_cast<double>(m + tot), e - 52);
                b += nok;
                continue;
            }
        }
        // block b element by element: lanes fetch 32 probabilities, lane 0 adds them in order
        if (lane == 0) start[b] = p;
        ++nseq;
        const uint64_t i0 = b * SAMPLE_BS, i1 = (i0 + SAMPLE_BS < N) ? i0 + SAMPLE_BS : N;
        for (uint64_t i = i0; i < i1; i += 32) {
            const double q = (i + lane < i1) ? qprob<P>(state[i + lane]) : 0.0;
            for (int j = 0; j < 32 && i + j < i1; ++j) {
                const double qj = __shfl_sync(0xffffffffu, q, j);
                p = __dadd_rn(p, qj);
            }
        }
        ++b;
    }
    if (lane == 0) {
        start[nb] = p;
        *seq = nseq;
    }
}

// A warp per shot: the first index whose running sum exceeds r.
template <class P>
__global__ void __launch_bounds__(256) k_sample_blocks(const typename P::G* __restrict__ state, uint64_t N,
                                                       uint64_t nb, const double* __restrict__ start,
                                                       const double* __restrict__ uni, int64_t shots,
                                                       uint64_t* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    const int64_t s = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (s >= shots) return;
    const double r = uni[s];
    if (!(r < start[nb])) {
        if (lane == 0) out[s] = N;
        return;
    }
    // first block b with r < start[b + 1]
    uint64_t lo = 0, hi = nb - 1;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (r < start[mid + 1]) hi = mid;
        else lo = mid + 1;
    }
    double p = start[lo];
    const uint64_t i0 = lo * SAMPLE_BS, i1 = (i0 + SAMPLE_BS < N) ? i0 + SAMPLE_BS : N;
    uint64_t found = i1 - 1;  // start[lo + 1] > r: the block's last index at the latest
    bool done = false;
    for (uint64_t i = i0; i < i1 && !done; i += 32) {
        const double q = (i + lane < i1) ? qprob<P>(state[i + lane]) : 0.0;
        for (int j = 0; j < 32 && i + j < i1; ++j) {
            p = __dadd_rn(p, __shfl_sync(0xffffffffu, q, j));
            if (r < p) {
                found = i + j;
                done = true;
                break;
            }
        }
    }
    if (lane == 0) out[s] = found;
}

template <class P>
cudaError_t launch_binade(const void* state, uint64_t N, int e_top, uint64_t* cnt, uint8_t* ties, double* start,
                          int64_t* seq, const double* uni, int64_t shots, uint64_t* out, cudaStream_t st) {
    using G = typename P::G;
    const G* s = static_cast<const G*>(state);
    const uint64_t nb = (N + SAMPLE_BS - 1) / SAMPLE_BS;
    const unsigned g1 = static_cast<unsigned>(nb < 152 * 16 ? nb : 152 * 16);
    k_binade_counts<P><<<g1, 256, 0, st>>>(s, N, e_top, cnt, ties, nb);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_binade_scan<P><<<1, 32, 0, st>>>(s, N, e_top, cnt, ties, nb, start, seq);
    e = cudaGetLastError();
    if (e != cudaSuccess || shots <= 0) return e;
    const unsigned g3 = static_cast<unsigned>((static_cast<uint64_t>(shots) * 32 + 255) / 256);
    k_sample_blocks<P><<<g3, 256, 0, st>>>(s, N, nb, start, uni, shots, out);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_sample_binade(int precision, const void* state, uint64_t N, int e_top, uint64_t* cnt,
                                 uint8_t* ties, double* start, int64_t* seq, const double* uni, int64_t shots,
                                 uint64_t* out, cudaStream_t st) {
    if (precision == QFVM_C64)
        return launch_binade<P32>(state, N, e_top, cnt, ties, start, seq, uni, shots, out, st);
    return launch_binade<P64>(state, N, e_top, cnt, ties, start, seq, uni, shots, out, st);
}

}  // namespace qsv
