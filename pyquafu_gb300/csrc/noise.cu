// Noise-channel trajectories (NoiseSVSimulator, quafu/simulators/simulator.py:
// 148-225) on batch items: every shot is an item; a channel on one qubit is
// resolved per item from the item's uniform, then applied as that item's own
// 2x2 matrix.  Unitary channels pick operator i with probability p_i
// (np.random.choice over the gate list, noise.py:86-91); Kraus channels follow
// the reference's rule (simulator.py:61-76): operators are tried in order,
// s += ||K_i psi|| / ||psi||, the first i with u < s is applied as
// K_i psi / ||K_i psi||, and the state is left unchanged when none is picked.
// The final sample of every shot is one index drawn from the item's
// probabilities in index order (measure_samples, statevector.hpp:1380-1412).
#include "kernels.h"
#include "reduce.cuh"

namespace qsv {

// Bits of the nonzero entries of a row-major 2x2 complex matrix k[8]
// (bit j <-> k[j]), from the bit patterns (integer work only).  Products
// with exact zeros are skipped below: they add exact zeros, so the skipped
// forms compute the same sums.
__device__ __forceinline__ uint32_t nonzero_mask(const double* k) {
    uint32_t nz = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (static_cast<uint64_t>(__double_as_longlong(k[j])) << 1) nz |= 1u << j;
    return nz;
}

// One output row of K (a, c)^T: (k0 + i k1) a + (k2 + i k3) c, zero terms
// skipped (nz: the row's 4 mask bits).
__device__ __forceinline__ double2 row_apply(const double* k, uint32_t nz, double2 a, double2 c) {
    double re = 0.0, im = 0.0;
    if (nz & 1) {
        re = __fma_rn(k[0], a.x, re);
        im = __fma_rn(k[0], a.y, im);
    }
    if (nz & 2) {
        re = __fma_rn(-k[1], a.y, re);
        im = __fma_rn(k[1], a.x, im);
    }
    if (nz & 4) {
        re = __fma_rn(k[2], c.x, re);
        im = __fma_rn(k[2], c.y, im);
    }
    if (nz & 8) {
        re = __fma_rn(-k[3], c.y, re);
        im = __fma_rn(k[3], c.x, im);
    }
    return make_double2(re, im);
}

// Kraus norms through the Gram matrices M_i = K_i^dagger K_i: summed over
// the pairs (a, c) of qubit q,
//   sum ||K_i (a, c)||^2 = m00 sum|a|^2 + m11 sum|c|^2 + 2 Re(m01 sum conj(a) c),
// so the state is reduced once to four sums, whatever the number of
// operators.  part[(item * bpi + b) * 4 + {0,1,2,3}] = block b's
// sum |a|^2, sum |c|^2, Re and Im of sum conj(a) c (CROSS: the last two are
// needed only when some m01 is nonzero).
constexpr int NORM_PAIRS = 8;
template <bool CROSS>
__global__ void __launch_bounds__(256) k_channel_norms(const double2* __restrict__ state, int n, int q, int bpi,
                                                       double* __restrict__ part) {
    __shared__ double red[8];
    const int item = blockIdx.x / bpi, b = blockIdx.x - item * bpi;
    const double2* st = state + (static_cast<uint64_t>(item) << n);
    const uint64_t ng = 1ULL << (n - 1);
    const uint64_t g0 = static_cast<uint64_t>(b) * 256 * NORM_PAIRS + threadIdx.x;
    double sa = 0.0, sc = 0.0, xr = 0.0, xi = 0.0;
#pragma unroll
    for (int r = 0; r < NORM_PAIRS; ++r) {
        const uint64_t g = g0 + static_cast<uint64_t>(r) * 256;
        if (g < ng) {
            const uint64_t i0 = insert0(g, q), i1 = i0 | (1ULL << q);
            const double2 a = st[i0], c = st[i1];
            sa = __fma_rn(a.x, a.x, __fma_rn(a.y, a.y, sa));
            sc = __fma_rn(c.x, c.x, __fma_rn(c.y, c.y, sc));
            if (CROSS) {
                xr = __fma_rn(a.x, c.x, __fma_rn(a.y, c.y, xr));
                xi = __fma_rn(a.x, c.y, __fma_rn(-a.y, c.x, xi));
            }
        }
    }
    double* out = part + static_cast<size_t>(blockIdx.x) * 4;
    double v = block_sum<256>(sa, red);
    if (threadIdx.x == 0) out[0] = v;
    v = block_sum<256>(sc, red);
    if (threadIdx.x == 0) out[1] = v;
    if (CROSS) {
        v = block_sum<256>(xr, red);
        if (threadIdx.x == 0) out[2] = v;
        v = block_sum<256>(xi, red);
        if (threadIdx.x == 0) out[3] = v;
    } else if (threadIdx.x == 0) {
        out[2] = 0.0;
        out[3] = 0.0;
    }
}

// One thread per item: the channel's operator for this item, written as the
// item's 2x2 matrix (identity when a Kraus channel picks nothing).
__global__ void k_channel_choose(const double* __restrict__ part, int bpi, int m, int kraus,
                                 const double* __restrict__ mats, const double* __restrict__ probs, int items,
                                 const double* __restrict__ uni, int draw, int ndraws, double* __restrict__ imat) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= items) return;
    const double u = uni[static_cast<size_t>(item) * ndraws + draw];
    double* out = imat + 8 * static_cast<size_t>(item);
    int pick = -1;
    double scale = 1.0;
    if (!kraus) {
        // np.random.choice: cdf = cumsum(p) / cdf[-1], first i with cdf[i] > u
        double tot = 0.0;
        for (int i = 0; i < m; ++i) tot += probs[i];
        double cum = 0.0;
        for (int i = 0; i < m; ++i) {
            cum += probs[i];
            if (cum / tot > u) {
                pick = i;
                break;
            }
        }
        if (pick < 0) pick = m - 1;
    } else {
        double sum[4] = {0.0, 0.0, 0.0, 0.0};
        for (int b = 0; b < bpi; ++b)
            for (int j = 0; j < 4; ++j) sum[j] += part[(static_cast<size_t>(item) * bpi + b) * 4 + j];
        const double norm0 = sqrt(sum[0] + sum[1]);
        double s = 0.0;
        for (int i = 0; i < m; ++i) {
            // M = K^dagger K: m00 = |k00|^2 + |k10|^2, m11 = |k01|^2 + |k11|^2,
            // m01 = conj(k00) k01 + conj(k10) k11
            const double* k = mats + 8 * i;
            const double m00 = k[0] * k[0] + k[1] * k[1] + k[4] * k[4] + k[5] * k[5];
            const double m11 = k[2] * k[2] + k[3] * k[3] + k[6] * k[6] + k[7] * k[7];
            const double m01r = k[0] * k[2] + k[1] * k[3] + k[4] * k[6] + k[5] * k[7];
            const double m01i = k[0] * k[3] - k[1] * k[2] + k[4] * k[7] - k[5] * k[6];
            double nrm = m00 * sum[0] + m11 * sum[1] + 2.0 * (m01r * sum[2] - m01i * sum[3]);
            if (nrm < 0.0) nrm = 0.0;  // rounding of a vanishing norm
            const double norm1 = sqrt(nrm);
            s += norm1 / norm0;
            if (u < s) {
                pick = i;
                scale = 1.0 / norm1;
                break;
            }
        }
    }
    if (pick < 0) {
        const double id[8] = {1, 0, 0, 0, 0, 0, 1, 0};
        for (int k = 0; k < 8; ++k) out[k] = id[k];
    } else {
        for (int k = 0; k < 8; ++k) out[k] = mats[8 * pick + k] * scale;
    }
}

// Every item's own 2x2 matrix on qubit q: a run of CTAs per item, each
// thread a few pairs.  An item whose matrix is exactly the identity (the
// usual pick of a unitary channel) is not touched; zero entries are skipped.
constexpr int GATE1_PAIRS = 8;  // pairs per thread
__global__ void __launch_bounds__(256) k_item_gate1(double2* __restrict__ state, int n, int q, int bpi,
                                                    const double* __restrict__ imat) {
    const int item = blockIdx.x / bpi, b = blockIdx.x - item * bpi;
    const double* k = imat + 8 * static_cast<size_t>(item);
    const uint32_t nz = nonzero_mask(k);
    if (nz == 0x41u && __double_as_longlong(k[0]) == 0x3FF0000000000000LL &&
        __double_as_longlong(k[6]) == 0x3FF0000000000000LL)
        return;
    double2* st = state + (static_cast<uint64_t>(item) << n);
    const uint64_t ng = 1ULL << (n - 1);
    const uint64_t g0 = static_cast<uint64_t>(b) * 256 * GATE1_PAIRS + threadIdx.x;
#pragma unroll
    for (int r = 0; r < GATE1_PAIRS; ++r) {
        const uint64_t g = g0 + static_cast<uint64_t>(r) * 256;
        if (g >= ng) break;
        const uint64_t i0 = insert0(g, q), i1 = i0 | (1ULL << q);
        const double2 a = st[i0], c = st[i1];
        st[i0] = row_apply(k, nz & 0x0f, a, c);
        st[i1] = row_apply(k + 4, nz >> 4, a, c);
    }
}

// One CTA per item: one index drawn from the item's probabilities with the
// scan of measure_samples (statevector.hpp:1387-1401): the first index whose
// running sum of |a|^2 exceeds u, or 2^n when none does.  Thread t owns a
// contiguous slice of indices; the slice sums are scanned in order, then the
// owning slice element by element.
__global__ void __launch_bounds__(256) k_item_sample(const double2* __restrict__ state, int n, int items,
                                                     const double* __restrict__ uni, int draw, int ndraws,
                                                     uint64_t* __restrict__ out) {
    __shared__ double sums[256];
    __shared__ int owner;
    __shared__ double base;
    const int item = blockIdx.x;
    const double2* st = state + (static_cast<uint64_t>(item) << n);
    const uint64_t N = 1ULL << n;
    const uint64_t per = (N + 255) / 256;
    const uint64_t lo = threadIdx.x * per < N ? threadIdx.x * per : N;
    const uint64_t hi = lo + per < N ? lo + per : N;
    const double r = uni[static_cast<size_t>(item) * ndraws + draw];
    double s = 0.0;
    for (uint64_t i = lo; i < hi; ++i) {
        const double2 a = st[i];
        s = __dadd_rn(s, __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)));
    }
    sums[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double cum = 0.0;
        int own = -1;
        for (int t = 0; t < 256; ++t) {
            const double next = __dadd_rn(cum, sums[t]);
            if (r < next) {
                own = t;
                base = cum;
                break;
            }
            cum = next;
        }
        owner = own;
        if (own < 0) out[item] = N;
    }
    __syncthreads();
    if (threadIdx.x == owner) {
        double cum = base;
        uint64_t pick = N;
        for (uint64_t i = lo; i < hi; ++i) {
            const double2 a = st[i];
            cum = __dadd_rn(cum, __dadd_rn(__dmul_rn(a.x, a.x), __dmul_rn(a.y, a.y)));
            if (r < cum) {
                pick = i;
                break;
            }
        }
        // rounding can leave r between the slice total and its element-wise sum
        out[item] = pick < N ? pick : (hi > lo ? hi - 1 : N);
    }
}

int channel_blocks_per_item(int n) {
    const uint64_t per = 256ULL * NORM_PAIRS;
    return static_cast<int>(((1ULL << (n - 1)) + per - 1) / per);
}

cudaError_t launch_channel(void* state, int n, int q, int m, int kraus, int cross, const double* dmats,
                           const double* dprobs, int items, const double* duni, int draw, int ndraws, double* dpart,
                           double* dimat, cudaStream_t st) {
    if (m < 1 || m > MAX_CHANNEL_OPS) return cudaErrorInvalidValue;
    const int bpi = channel_blocks_per_item(n);
    if (kraus) {
        const unsigned grid = static_cast<unsigned>(bpi) * items;
        if (cross)
            k_channel_norms<true><<<grid, 256, 0, st>>>(static_cast<const double2*>(state), n, q, bpi, dpart);
        else
            k_channel_norms<false><<<grid, 256, 0, st>>>(static_cast<const double2*>(state), n, q, bpi, dpart);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_channel_choose<<<(items + 127) / 128, 128, 0, st>>>(dpart, bpi, m, kraus, dmats, dprobs, items, duni, draw,
                                                          ndraws, dimat);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const uint64_t per_block = 256ULL * GATE1_PAIRS;
    const int gbpi = static_cast<int>(((1ULL << (n - 1)) + per_block - 1) / per_block);
    k_item_gate1<<<static_cast<unsigned>(gbpi) * items, 256, 0, st>>>(static_cast<double2*>(state), n, q, gbpi,
                                                                     dimat);
    return cudaGetLastError();
}

cudaError_t launch_item_sample(const void* state, int n, int items, const double* duni, int draw, int ndraws,
                               uint64_t* dout, cudaStream_t st) {
    k_item_sample<<<items, 256, 0, st>>>(static_cast<const double2*>(state), n, items, duni, draw, ndraws, dout);
    return cudaGetLastError();
}

}  // namespace qsv
