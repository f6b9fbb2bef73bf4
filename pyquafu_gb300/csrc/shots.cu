// Per-shot trajectories of circuits with mid-circuit measurement, reset and
// classically controlled blocks (the per-shot branch of qfvm.cpp:104-133).
// Shots run side by side as batch items (item i's state at i << n); every
// measure/reset is three kernels: FP64 outcome probabilities per item, the
// outcome drawn from the item's uniform, and the collapse (projection,
// 1/sqrt(p) scaling, and for reset the move of the outcome block to 0).
#include "kernels.h"
#include "reduce.cuh"

namespace qsv {

// index of group g (the 2^(n-k) assignments of the unmeasured qubits) with
// measured bits set to outcome m (bit j of m <-> qubit q[j]); srt = q sorted
__device__ __forceinline__ uint64_t group_index(uint64_t g, const uint8_t* srt, int k) {
    for (int j = 0; j < k; ++j) g = insert0(g, srt[j]);
    return g;
}
__device__ __forceinline__ uint64_t deposit(uint32_t m, const uint8_t* q, int k) {
    uint64_t d = 0;
    for (int j = 0; j < k; ++j)
        if ((m >> j) & 1) d |= 1ULL << q[j];
    return d;
}

// part[(item * bpi + b) * 2^k + m] = sum over block b's groups of |a(g, m)|^2
template <class P>
__global__ void __launch_bounds__(256) k_outcome_probs(const typename P::G* __restrict__ state, int n, MeasureSpec ms,
                                                       uint64_t groups_per_block, int bpi, double* __restrict__ part) {
    __shared__ double red[8];
    const int item = blockIdx.x / bpi, b = blockIdx.x - item * bpi;
    const typename P::G* st = state + (static_cast<uint64_t>(item) << n);
    const uint64_t ng = 1ULL << (n - ms.k);
    const uint64_t g0 = b * groups_per_block;
    const uint64_t g1 = g0 + groups_per_block < ng ? g0 + groups_per_block : ng;
    const uint32_t K = 1u << ms.k;
    for (uint32_t m = 0; m < K; ++m) {
        const uint64_t dm = deposit(m, ms.q, ms.k);
        double acc = 0.0;
        for (uint64_t g = g0 + threadIdx.x; g < g1; g += 256) {
            const typename P::G a = st[group_index(g, ms.srt, ms.k) | dm];
            const double re = P::gre(a), im = P::gim(a);
            acc = __dadd_rn(acc, __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im)));
        }
        const double s = block_sum<256>(acc, red);
        if (threadIdx.x == 0) part[(static_cast<size_t>(blockIdx.x)) * K + m] = s;
    }
}

// One thread per item: outcome probabilities (blocks summed in order), the
// first outcome m with u * total < cum[m], classical bits, scale 1/sqrt(p).
__global__ void k_outcome_choose(const double* __restrict__ part, int bpi, MeasureSpec ms, int items,
                                 const double* __restrict__ uni, int draw, int ndraws, uint8_t* __restrict__ creg,
                                 int ncb, int32_t* __restrict__ outcome, double* __restrict__ scale) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= items) return;
    const uint32_t K = 1u << ms.k;
    double total = 0.0;
    for (uint32_t m = 0; m < K; ++m) {
        double p = 0.0;
        for (int b = 0; b < bpi; ++b) p = __dadd_rn(p, part[(static_cast<size_t>(item) * bpi + b) * K + m]);
        total = __dadd_rn(total, p);
    }
    const double r = __dmul_rn(uni[static_cast<size_t>(item) * ndraws + draw], total);
    double cum = 0.0, pm = 0.0, plast = 0.0;
    uint32_t pick = K, last = 0;
    for (uint32_t m = 0; m < K; ++m) {
        double p = 0.0;
        for (int b = 0; b < bpi; ++b) p = __dadd_rn(p, part[(static_cast<size_t>(item) * bpi + b) * K + m]);
        cum = __dadd_rn(cum, p);
        if (p > 0.0) {
            last = m;
            plast = p;
        }
        if (pick == K && r < cum) {
            pick = m;
            pm = p;
        }
    }
    if (pick == K) {
        pick = last;
        pm = plast;
    }
    outcome[item] = static_cast<int32_t>(pick);
    scale[item] = pm > 0.0 ? 1.0 / sqrt(pm) : 0.0;
    if (!ms.reset)
        for (int j = 0; j < ms.k; ++j) creg[static_cast<size_t>(item) * ncb + ms.cb[j]] = (pick >> j) & 1;
}

// One thread per (item, group): keep the chosen outcome's amplitude, scaled,
// at the final block (the outcome for measure, 0 for reset); zero the rest.
template <class P>
__global__ void __launch_bounds__(256) k_collapse(typename P::G* __restrict__ state, int n, MeasureSpec ms, int items,
                                                  const int32_t* __restrict__ outcome,
                                                  const double* __restrict__ scale) {
    const uint64_t ng = 1ULL << (n - ms.k);
    const uint64_t total = ng * static_cast<uint64_t>(items);
    const uint32_t K = 1u << ms.k;
    for (uint64_t t = blockIdx.x * 256ULL + threadIdx.x; t < total; t += gridDim.x * 256ULL) {
        const uint64_t item = t / ng, g = t - item * ng;
        typename P::G* st = state + (item << n);
        const uint64_t base = group_index(g, ms.srt, ms.k);
        const uint32_t oc = static_cast<uint32_t>(outcome[item]);
        const uint32_t fin = ms.reset ? 0u : oc;
        const double sc = scale[item];
        const typename P::G a = st[base | deposit(oc, ms.q, ms.k)];
        for (uint32_t m = 0; m < K; ++m) {
            const uint64_t ix = base | deposit(m, ms.q, ms.k);
            st[ix] = m == fin ? P::make_g(sc * P::gre(a), sc * P::gim(a)) : P::make_g(0.0, 0.0);
        }
    }
}

// active[item] = (classical bits cb[0..nc) read as a binary number, first
// most significant) == condition   (check_cif, statevector.hpp:186-193)
__global__ void k_cif_mask(const uint8_t* __restrict__ creg, int ncb, int items, CifSpec cs,
                           uint8_t* __restrict__ active) {
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= items) return;
    uint64_t v = 0;
    for (int j = 0; j < cs.nc; ++j) v = v * 2 + creg[static_cast<size_t>(item) * ncb + cs.cb[j]];
    active[item] = v == cs.condition ? 1 : 0;
}

// every item <- psi0 (2^n amplitudes, complex128 on the device)
__global__ void k_items_copy(double2* __restrict__ state, int n, int items, const double2* __restrict__ psi0) {
    const uint64_t N = 1ULL << n, total = N * static_cast<uint64_t>(items);
    for (uint64_t i = blockIdx.x * 256ULL + threadIdx.x; i < total; i += gridDim.x * 256ULL)
        state[i] = psi0[i & (N - 1)];
}

static unsigned grid_of(uint64_t work, unsigned cap = 152 * 16) {
    const uint64_t b = (work + 255) / 256;
    return static_cast<unsigned>(b < 1 ? 1 : (b < cap ? b : cap));
}

int outcome_blocks_per_item(int n, int k) {
    const uint64_t ng = 1ULL << (n - k);
    const uint64_t per = 256ULL * 16;  // groups per block
    return static_cast<int>((ng + per - 1) / per);
}

cudaError_t launch_measure(void* state, int n, const MeasureSpec& ms, int items, const double* duni, int draw,
                           int ndraws, uint8_t* dcreg, int ncb, double* dpart, int32_t* doutcome, double* dscale,
                           cudaStream_t st) {
    const int bpi = outcome_blocks_per_item(n, ms.k);
    const uint64_t gpb = 256ULL * 16;
    k_outcome_probs<P64><<<static_cast<unsigned>(bpi) * items, 256, 0, st>>>(static_cast<const double2*>(state), n, ms,
                                                                             gpb, bpi, dpart);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_outcome_choose<<<(items + 127) / 128, 128, 0, st>>>(dpart, bpi, ms, items, duni, draw, ndraws, dcreg, ncb,
                                                          doutcome, dscale);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_collapse<P64><<<grid_of((1ULL << (n - ms.k)) * items), 256, 0, st>>>(static_cast<double2*>(state), n, ms, items,
                                                                          doutcome, dscale);
    return cudaGetLastError();
}

cudaError_t launch_cif_mask(const uint8_t* dcreg, int ncb, int items, const CifSpec& cs, uint8_t* dactive,
                            cudaStream_t st) {
    k_cif_mask<<<(items + 127) / 128, 128, 0, st>>>(dcreg, ncb, items, cs, dactive);
    return cudaGetLastError();
}

cudaError_t launch_items_copy(void* state, int n, int items, const void* psi0, cudaStream_t st) {
    k_items_copy<<<grid_of((1ULL << n) * items), 256, 0, st>>>(static_cast<double2*>(state), n, items,
                                                              static_cast<const double2*>(psi0));
    return cudaGetLastError();
}

}  // namespace qsv
