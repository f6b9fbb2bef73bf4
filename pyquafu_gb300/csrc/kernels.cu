// GB300 statevector kernels: whole-state passes, the generic k-target gate,
// FP64 reductions (Pauli expectation, norms) and the sampling pipeline (block
// sums, block prefix, per-shot locate, exact fallback).  The fused tile-pass
// kernel is instantiated per precision in pass_c128.cu / pass_c64.cu.
#include <atomic>

#include "device.cuh"
#include "kernels.h"
#include "reduce.cuh"

namespace qsv {

template <class P>
__global__ void __launch_bounds__(512) k_small(typename P::G* __restrict__ state, uint64_t stride, int n,
                                               const KOp* __restrict__ ops, int nops,
                                               const typename P::C* __restrict__ coef0, uint64_t cstride,
                                               const uint8_t* __restrict__ active) {
    if (active && !active[blockIdx.x]) return;  // the whole block: item blockIdx.x keeps its state
    constexpr int GB = P::GBITS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typename P::S* sm = reinterpret_cast<typename P::S*>(smem_raw);
    typename P::G* st = state + stride * blockIdx.x;
    const typename P::C* coef = coef0 + cstride * blockIdx.x;  // item blockIdx.x's coefficient pool
    const uint32_t N = 1u << n;
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) sm[swz<GB>(i)] = P::g2s(st[i]);
    __syncthreads();
    for (int oi = 0; oi < nops; ++oi) {
        const KOp o = ops[oi];
        small_apply<P>(sm, n, o, coef);
        __syncthreads();
    }
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) st[i] = P::s2g(sm[swz<GB>(i)]);
}

// ---------------------------------------------------------------------------
// Dense gate on k targets straight on global memory (large states; rare).
// ---------------------------------------------------------------------------
template <class P>
__global__ void __launch_bounds__(256) k_globalop(typename P::G* __restrict__ state, int n, int items,
                                                  const KOp* __restrict__ opp, const typename P::C* __restrict__ coef0,
                                                  uint64_t cstride, const uint8_t* __restrict__ active) {
    using A = typename P::A;
    using C = typename P::C;
    const KOp op = *opp;
    const int k = op.k;
    const uint32_t dim = 1u << k;
    uint8_t srt[MAXK];
    for (int j = 0; j < k; ++j) srt[j] = op.tk[j];
    for (int x = 1; x < k; ++x)
        for (int y = x; y > 0 && srt[y - 1] > srt[y]; --y) {
            uint8_t t = srt[y];
            srt[y] = srt[y - 1];
            srt[y - 1] = t;
        }
    // batched states: the item index sits above the n gate qubits
    const uint64_t groups = static_cast<uint64_t>(items) << (n - k);
    for (uint64_t g = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; g < groups;
         g += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        uint64_t i = g;
        for (int j = 0; j < k; ++j) i = insert0(i, srt[j]);
        if ((i & op.cthr) != op.cthr) continue;
        if (active && !active[i >> n]) continue;
        const typename P::C* coef = coef0 + (i >> n) * cstride;
        A in[1 << MAXK];
        for (uint32_t m = 0; m < dim; ++m) {
            uint64_t idx = i;
            for (int j = 0; j < k; ++j)
                if ((m >> j) & 1) idx |= 1ULL << op.tk[j];
            in[m] = P::s2a(P::g2s(state[idx]));
        }
        for (uint32_t r = 0; r < dim; ++r) {
            typename P::R xr = P::mul(P::coef(coef, op.coef + 2 * (r * dim)), in[0].x);
            typename P::R xi = P::mul(P::coef(coef, op.coef + 2 * (r * dim)), in[0].y);
            xr = P::madd(P::cneg(P::coef(coef, op.coef + 2 * (r * dim) + 1)), in[0].y, xr);
            xi = P::madd(P::coef(coef, op.coef + 2 * (r * dim) + 1), in[0].x, xi);
            for (uint32_t c = 1; c < dim; ++c) {
                const C mr = P::coef(coef, op.coef + 2 * (r * dim + c));
                const C mi = P::coef(coef, op.coef + 2 * (r * dim + c) + 1);
                xr = P::madd(mr, in[c].x, xr);
                xr = P::madd(P::cneg(mi), in[c].y, xr);
                xi = P::madd(mr, in[c].y, xi);
                xi = P::madd(mi, in[c].x, xi);
            }
            uint64_t idx = i;
            for (int j = 0; j < k; ++j)
                if ((r >> j) & 1) idx |= 1ULL << op.tk[j];
            A o;
            o.x = xr;
            o.y = xi;
            state[idx] = P::s2g(P::a2s(o));
        }
    }
}

// ---------------------------------------------------------------------------
// Dense gate on MAXK+1 .. MAX_DENSE_TARGETS targets (statevector.hpp:945-995
// applies any target count): one CTA per group of 2^k amplitudes, the group
// staged in shared memory, each thread computing output rows.  The targets
// are ascending (op.pthr is their mask; the host relabelled the matrix), so
// group member m sits at base | deposit(m, mask).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t deposit_bits(uint32_t m, uint64_t mask) {
    uint64_t r = 0;
    for (int j = 0; mask; ++j) {
        const uint64_t low = mask & (~mask + 1);
        if ((m >> j) & 1u) r |= low;
        mask &= mask - 1;
    }
    return r;
}

template <class P>
__global__ void __launch_bounds__(256) k_globalop_wide(typename P::G* __restrict__ state, int n, int items,
                                                       const KOp* __restrict__ opp,
                                                       const typename P::C* __restrict__ coef0, uint64_t cstride,
                                                       const uint8_t* __restrict__ active) {
    using A = typename P::A;
    using C = typename P::C;
    extern __shared__ __align__(16) unsigned char wide_smem[];
    A* in = reinterpret_cast<A*>(wide_smem);
    const KOp op = *opp;
    const int k = op.k;
    const uint32_t dim = 1u << k;
    const uint64_t tmask = op.pthr;
    const uint64_t groups = static_cast<uint64_t>(items) << (n - k);
    for (uint64_t g = blockIdx.x; g < groups; g += gridDim.x) {
        uint64_t i = g;
        for (uint64_t mm = tmask; mm; mm &= mm - 1) i = insert0(i, __ffsll(static_cast<long long>(mm)) - 1);
        if ((i & op.cthr) != op.cthr) continue;  // the same for the whole CTA
        if (active && !active[i >> n]) continue;
        const C* coef = coef0 + (i >> n) * cstride;
        for (uint32_t m = threadIdx.x; m < dim; m += blockDim.x) in[m] = P::s2a(P::g2s(state[i | deposit_bits(m, tmask)]));
        __syncthreads();
        for (uint32_t r = threadIdx.x; r < dim; r += blockDim.x) {
            const uint32_t row = op.coef + 2 * (r * dim);
            typename P::R xr = P::mul(P::coef(coef, row), in[0].x);
            typename P::R xi = P::mul(P::coef(coef, row), in[0].y);
            xr = P::madd(P::cneg(P::coef(coef, row + 1)), in[0].y, xr);
            xi = P::madd(P::coef(coef, row + 1), in[0].x, xi);
            for (uint32_t c = 1; c < dim; ++c) {
                const C mr = P::coef(coef, row + 2 * c);
                const C mi = P::coef(coef, row + 2 * c + 1);
                xr = P::madd(mr, in[c].x, xr);
                xr = P::madd(P::cneg(mi), in[c].y, xr);
                xi = P::madd(mr, in[c].y, xi);
                xi = P::madd(mi, in[c].x, xi);
            }
            A o;
            o.x = xr;
            o.y = xi;
            state[i | deposit_bits(r, tmask)] = P::s2g(P::a2s(o));
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Utility kernels
// ---------------------------------------------------------------------------
template <class P>
__global__ void k_set_basis(typename P::G* state, uint64_t N, uint64_t index) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < N;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        state[i] = P::make_g(i == index ? 1.0 : 0.0, 0.0);
}

__global__ void k_c128_to_c64(const double2* __restrict__ in, float2* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const double2 v = in[i];
        out[i] = make_float2(static_cast<float>(v.x), static_cast<float>(v.y));
    }
}

__global__ void k_c64_to_c128(const float2* __restrict__ in, double2* __restrict__ out, uint64_t n) {
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
        const float2 v = in[i];
        out[i] = make_double2(static_cast<double>(v.x), static_cast<double>(v.y));
    }
}

// ---------------------------------------------------------------------------
// Sampling.  q_i = fl(fl(re^2) + fl(im^2)) exactly as the sequential scan of
// measure_samples (statevector.hpp:1392-1396) forms it.
// ---------------------------------------------------------------------------
template <class P>
__device__ __forceinline__ double prob_of(const typename P::G g) {
    const double re = P::gre(g), im = P::gim(g);
    return __dadd_rn(__dmul_rn(re, re), __dmul_rn(im, im));
}

template <class P>
__global__ void __launch_bounds__(256) k_block_sums(const typename P::G* __restrict__ state, uint64_t bs,
                                                    double* __restrict__ bsum) {
    __shared__ double red[8];
    const uint64_t b0 = static_cast<uint64_t>(blockIdx.x) * bs;
    double s = 0.0;
    for (uint64_t i = threadIdx.x; i < bs; i += 256) s += prob_of<P>(state[b0 + i]);
    s = block_sum<256>(s, red);
    if (threadIdx.x == 0) bsum[blockIdx.x] = s;
}

// Exclusive prefix over nb block sums (one CTA of 1024 threads); pre[nb] = total.
__global__ void __launch_bounds__(1024) k_scan_blocks(const double* __restrict__ bsum, uint64_t nb,
                                                      double* __restrict__ pre) {
    __shared__ double wsum[32];
    __shared__ double carry_s;
    if (threadIdx.x == 0) carry_s = 0.0;
    __syncthreads();
    const int l = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (uint64_t base = 0; base < nb; base += 1024) {
        const uint64_t i = base + threadIdx.x;
        const double v = i < nb ? bsum[i] : 0.0;
        double x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const double y = __shfl_up_sync(0xffffffffu, x, o);
            if (l >= o) x += y;
        }
        if (l == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            double z = wsum[l];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const double y = __shfl_up_sync(0xffffffffu, z, o);
                if (l >= o) z += y;
            }
            wsum[l] = z;
        }
        __syncthreads();
        const double carry = carry_s;
        const double incl = x + (w > 0 ? wsum[w - 1] : 0.0) + carry;
        if (i < nb) pre[i] = incl - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry_s = incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) pre[nb] = carry_s;
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
// Shapes picked by the autotuner per (arithmetic, pass kind, qubit count),
// packed as T | R << 8; 0 means the built-in default.
static std::atomic<int32_t> g_tuned[3][2][QFVM_MAX_QUBITS + 1];

void resolve_shape(int arith, int kind, int n, int* T, int* R) {
    const int a = (arith == QFVM_C64) ? 1 : (arith == QFVM_C128_DS ? 2 : 0);
    const int32_t v = (n >= 0 && n <= QFVM_MAX_QUBITS && (kind == 0 || kind == 1))
                          ? g_tuned[a][kind][n].load(std::memory_order_relaxed)
                          : 0;
    if (v) {
        *T = v & 0xff;
        *R = (v >> 8) & 0xff;
        return;
    }
    if (kind == 1) adjoint_shape(arith, T, R);
    else default_shape(n, arith, T, R);
}

bool set_tuned_shape(int arith, int kind, int n, int T, int R) {
    if (n < 0 || n > QFVM_MAX_QUBITS || (kind != 0 && kind != 1)) return false;
    const int a = (arith == QFVM_C64) ? 1 : (arith == QFVM_C128_DS ? 2 : 0);
    if (T == 0) {
        g_tuned[a][kind][n].store(0);
        return true;
    }
    const bool ok = kind == 0 ? pass_shape_supported(arith, T, R) : pass2_shape_supported(arith, T, R);
    if (!ok) return false;
    g_tuned[a][kind][n].store(T | (R << 8));
    return true;
}

bool pass_shape_supported(int precision, int T, int R) {
    if (precision == QFVM_C64) return pass_shape_c64(T, R);
    if (precision == QFVM_C128_DS) return pass_shape_ds(T, R);
    return pass_shape_c128(T, R);
}

cudaError_t launch_tile_pass(int precision, int T, int R, void* state, const PassDesc* dpass,
                             const StepDesc* dsteps, const KOp* dops, const void* dcoef, int n, int H,
                             int items, uint64_t cstride, const uint8_t* active, cudaStream_t st) {
    if (precision == QFVM_C64) return launch_pass_c64(T, R, state, dpass, dsteps, dops, dcoef, n, H, items, cstride, active, st);
    if (precision == QFVM_C128_DS) return launch_pass_ds(T, R, state, dpass, dsteps, dops, dcoef, n, H, items, cstride, active, st);
    return launch_pass_c128(T, R, state, dpass, dsteps, dops, dcoef, n, H, items, cstride, active, st);
}

template <class P>
static cudaError_t launch_small_p(void* state, uint64_t stride, int batch, int n, const KOp* dops, int nops,
                                  const void* dcoef, uint64_t cstride, const uint8_t* active, cudaStream_t st) {
    const int threads = n >= 10 ? 512 : 256;
    const size_t smem = sizeof(typename P::S) << n;
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(k_small<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    k_small<P><<<batch, threads, smem, st>>>(static_cast<typename P::G*>(state), stride, n, dops, nops,
                                            static_cast<const typename P::C*>(dcoef), cstride, active);
    return cudaGetLastError();
}

cudaError_t launch_small(int precision, void* state, uint64_t stride, int batch, int n, const KOp* dops, int nops,
                         const void* dcoef, uint64_t cstride, const uint8_t* active, cudaStream_t st) {
    if (precision == QFVM_C64) return launch_small_p<P32>(state, stride, batch, n, dops, nops, dcoef, cstride, active, st);
    if (precision == QFVM_C128_DS) return launch_small_p<PDS>(state, stride, batch, n, dops, nops, dcoef, cstride, active, st);
    return launch_small_p<P64>(state, stride, batch, n, dops, nops, dcoef, cstride, active, st);
}

template <class P>
static cudaError_t launch_wide(void* state, int n, int k, const KOp* dop, const void* dcoef, int items,
                               uint64_t cstride, const uint8_t* active, cudaStream_t st) {
    const size_t smem = sizeof(typename P::A) << k;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_globalop_wide<P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    const uint64_t groups = static_cast<uint64_t>(items) << (n - k);
    const unsigned blocks = static_cast<unsigned>(groups < 152 * 8 ? groups : 152 * 8);
    k_globalop_wide<P><<<blocks, 256, smem, st>>>(static_cast<typename P::G*>(state), n, items, dop,
                                                  static_cast<const typename P::C*>(dcoef), cstride, active);
    return cudaGetLastError();
}

cudaError_t launch_globalop(int precision, void* state, int n, int k, const KOp* dop, const void* dcoef, int items,
                            uint64_t cstride, const uint8_t* active, cudaStream_t st) {
    if (k > MAXK) {
        if (k > MAX_DENSE_TARGETS || k > n) return cudaErrorInvalidValue;
        if (precision == QFVM_C64) return launch_wide<P32>(state, n, k, dop, dcoef, items, cstride, active, st);
        if (precision == QFVM_C128_DS) return launch_wide<PDS>(state, n, k, dop, dcoef, items, cstride, active, st);
        return launch_wide<P64>(state, n, k, dop, dcoef, items, cstride, active, st);
    }
    const uint64_t groups = static_cast<uint64_t>(items) << (n - 1);
    const unsigned blocks = static_cast<unsigned>(groups / 256 < 152 * 16 ? (groups + 255) / 256 : 152 * 16);
    if (precision == QFVM_C64)
        k_globalop<P32><<<blocks, 256, 0, st>>>(static_cast<float2*>(state), n, items, dop,
                                               static_cast<const float*>(dcoef), cstride, active);
    else if (precision == QFVM_C128_DS)
        k_globalop<PDS><<<blocks, 256, 0, st>>>(static_cast<double2*>(state), n, items, dop,
                                               static_cast<const ds*>(dcoef), cstride, active);
    else
        k_globalop<P64><<<blocks, 256, 0, st>>>(static_cast<double2*>(state), n, items, dop,
                                               static_cast<const double*>(dcoef), cstride, active);
    return cudaGetLastError();
}

static unsigned grid_for(uint64_t work, unsigned per_block, unsigned cap) {
    uint64_t b = (work + per_block - 1) / per_block;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return static_cast<unsigned>(b);
}

cudaError_t launch_set_basis(int precision, void* state, uint64_t N, uint64_t index, cudaStream_t st) {
    const unsigned g = grid_for(N, 256, 152 * 32);
    if (precision == QFVM_C64) k_set_basis<P32><<<g, 256, 0, st>>>(static_cast<float2*>(state), N, index);
    else k_set_basis<P64><<<g, 256, 0, st>>>(static_cast<double2*>(state), N, index);
    return cudaGetLastError();
}

cudaError_t launch_convert(bool to64, const void* in, void* out, uint64_t n, cudaStream_t st) {
    const unsigned g = grid_for(n, 256, 152 * 32);
    if (to64) k_c128_to_c64<<<g, 256, 0, st>>>(static_cast<const double2*>(in), static_cast<float2*>(out), n);
    else k_c64_to_c128<<<g, 256, 0, st>>>(static_cast<const float2*>(in), static_cast<double2*>(out), n);
    return cudaGetLastError();
}

cudaError_t launch_expect_z(int precision, const void* state, uint64_t N, const uint64_t* dzm, int nterms,
                            double* dpartial, int nblocks, cudaStream_t st) {
    if (precision == QFVM_C64)
        k_expect_z<P32><<<nblocks, 256, 0, st>>>(static_cast<const float2*>(state), N, dzm, nterms, dpartial);
    else
        k_expect_z<P64><<<nblocks, 256, 0, st>>>(static_cast<const double2*>(state), N, dzm, nterms, dpartial);
    return cudaGetLastError();
}

cudaError_t launch_expect_x(int precision, const void* state, uint64_t N, uint64_t xmask, int flip_q,
                            const uint64_t* dzm, const int32_t* dny, int nterms, double* dpartial, int nblocks,
                            cudaStream_t st) {
    if (precision == QFVM_C64)
        k_expect_x<P32><<<nblocks, 256, 0, st>>>(static_cast<const float2*>(state), N, xmask, flip_q, dzm, dny,
                                                 nterms, dpartial);
    else
        k_expect_x<P64><<<nblocks, 256, 0, st>>>(static_cast<const double2*>(state), N, xmask, flip_q, dzm, dny,
                                                 nterms, dpartial);
    return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const double* dpartial, int nblocks, int nterms, double* dout, cudaStream_t st) {
    k_reduce_partials<<<1, 256, 0, st>>>(dpartial, nblocks, nterms, dout);
    return cudaGetLastError();
}

cudaError_t launch_block_prefix(int precision, const void* state, uint64_t N, uint64_t bs, double* dbsum,
                                double* dpre, cudaStream_t st) {
    const uint64_t nb = N / bs;
    if (precision == QFVM_C64)
        k_block_sums<P32><<<static_cast<unsigned>(nb), 256, 0, st>>>(static_cast<const float2*>(state), bs, dbsum);
    else
        k_block_sums<P64><<<static_cast<unsigned>(nb), 256, 0, st>>>(static_cast<const double2*>(state), bs, dbsum);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_scan_blocks<<<1, 1024, 0, st>>>(dbsum, nb, dpre);
    return cudaGetLastError();
}


}  // namespace qsv
