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
// (bit j <-> k[j]).  Products with exact zeros are skipped below: they add
// exact zeros, so the skipped forms compute the same sums.
__device__ __forceinline__ uint32_t nonzero_mask(const double* k) {
    uint32_t nz = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (k[j] != 0.0) nz |= 1u << j;
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

// part[(item * bpi + b) * (m + 1) + i] = block b's sum of ||K_i (a_g0, a_g1)||^2
// for i < m, and of |a_g0|^2 + |a_g1|^2 at i = m; groups g = the pairs on qubit q
__global__ void __launch_bounds__(256) k_channel_norms(const double2* __restrict__ state, int n, int q, int m,
                                                       const double* __restrict__ mats, uint64_t groups_per_block,
                                                       int bpi, double* __restrict__ part) {
    __shared__ double red[8];
    const int item = blockIdx.x / bpi, b = blockIdx.x - item * bpi;
    const double2* st = state + (static_cast<uint64_t>(item) << n);
    const uint64_t ng = 1ULL << (n - 1);
    const uint64_t g0 = b * groups_per_block;
    const uint64_t g1 = g0 + groups_per_block < ng ? g0 + groups_per_block : ng;
    double acc[MAX_CHANNEL_OPS + 1];
    uint32_t nz[MAX_CHANNEL_OPS];
#pragma unroll
    for (int i = 0; i <= MAX_CHANNEL_OPS; ++i) acc[i] = 0.0;
#pragma unroll
    for (int i = 0; i < MAX_CHANNEL_OPS; ++i) nz[i] = i < m ? nonzero_mask(mats + 8 * i) : 0u;
    for (uint64_t g = g0 + threadIdx.x; g < g1; g += 256) {
        const uint64_t i0 = insert0(g, q), i1 = i0 | (1ULL << q);
        const double2 a = st[i0], c = st[i1];
        acc[MAX_CHANNEL_OPS] += a.x * a.x + a.y * a.y + c.x * c.x + c.y * c.y;
#pragma unroll
        for (int i = 0; i < MAX_CHANNEL_OPS; ++i) {
            if (i >= m) break;
            const double* k = mats + 8 * i;  // row-major 2x2, (re, im) pairs
            double s = 0.0;
            if (nz[i] & 0x0f) {
                const double2 v = row_apply(k, nz[i] & 0x0f, a, c);
                s = __fma_rn(v.x, v.x, __dmul_rn(v.y, v.y));
            }
            if (nz[i] & 0xf0) {
                const double2 v = row_apply(k + 4, nz[i] >> 4, a, c);
                s = __fma_rn(v.x, v.x, __fma_rn(v.y, v.y, s));
            }
            acc[i] += s;
        }
    }
    for (int i = 0; i <= m; ++i) {
        const double s = block_sum<256>(acc[i == m ? MAX_CHANNEL_OPS : i], red);
        if (threadIdx.x == 0) part[(static_cast<size_t>(blockIdx.x)) * (m + 1) + i] = s;
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
        double nrm[MAX_CHANNEL_OPS + 1];
        for (int i = 0; i <= m; ++i) {
            double s = 0.0;
            for (int b = 0; b < bpi; ++b) s += part[(static_cast<size_t>(item) * bpi + b) * (m + 1) + i];
            nrm[i] = s;
        }
        const double norm0 = sqrt(nrm[m]);
        double s = 0.0;
        for (int i = 0; i < m; ++i) {
            const double norm1 = sqrt(nrm[i]);
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

// Every item's own 2x2 matrix on qubit q: one thread per (item, pair).  An
// item whose matrix is exactly the identity (the common pick of a unitary
// channel) is not touched; zero entries are skipped.
__global__ void __launch_bounds__(256) k_item_gate1(double2* __restrict__ state, int n, int q, int items,
                                                    const double* __restrict__ imat) {
    const uint64_t ng = 1ULL << (n - 1);
    const uint64_t total = ng * static_cast<uint64_t>(items);
    uint64_t cur = ~0ULL;
    uint32_t nz = 0;
    bool ident = false;
    const double* k = imat;
    for (uint64_t t = blockIdx.x * 256ULL + threadIdx.x; t < total; t += gridDim.x * 256ULL) {
        const uint64_t item = t / ng, g = t - item * ng;
        if (item != cur) {
            cur = item;
            k = imat + 8 * item;
            nz = nonzero_mask(k);
            ident = nz == 0x41u && k[0] == 1.0 && k[6] == 1.0;
        }
        if (ident) continue;
        double2* st = state + (item << n);
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

static unsigned grid_for_items(uint64_t work) {
    const uint64_t b = (work + 255) / 256;
    return static_cast<unsigned>(b < 1 ? 1 : (b < 152 * 16 ? b : 152 * 16));
}

cudaError_t launch_channel(void* state, int n, int q, int m, int kraus, const double* dmats, const double* dprobs,
                           int items, const double* duni, int draw, int ndraws, double* dpart, double* dimat,
                           cudaStream_t st) {
    if (m < 1 || m > MAX_CHANNEL_OPS) return cudaErrorInvalidValue;
    const int bpi = outcome_blocks_per_item(n, 1);
    if (kraus) {
        k_channel_norms<<<static_cast<unsigned>(bpi) * items, 256, 0, st>>>(static_cast<const double2*>(state), n, q,
                                                                          m, dmats, 256ULL * 16, bpi, dpart);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    k_channel_choose<<<(items + 127) / 128, 128, 0, st>>>(dpart, bpi, m, kraus, dmats, dprobs, items, duni, draw,
                                                          ndraws, dimat);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_item_gate1<<<grid_for_items((1ULL << (n - 1)) * items), 256, 0, st>>>(static_cast<double2*>(state), n, q,
                                                                           items, dimat);
    return cudaGetLastError();
}

cudaError_t launch_item_sample(const void* state, int n, int items, const double* duni, int draw, int ndraws,
                               uint64_t* dout, cudaStream_t st) {
    k_item_sample<<<items, 256, 0, st>>>(static_cast<const double2*>(state), n, items, duni, draw, ndraws, dout);
    return cudaGetLastError();
}

}  // namespace qsv
