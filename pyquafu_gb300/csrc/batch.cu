// Batched-run kernels.  A batch holds `items` states of n qubits back to back
// (item i at offset i << n) that share one plan; what differs per item is the
// coefficient pool (rewritten here from each item's slot values) and the
// results.  Every sum is FP64 and adds in a fixed order, so a batch run is
// deterministic and item i's result does not depend on the other items.
#include "kernels.h"
#include "reduce.cuh"

namespace qsv {

// Coefficients of a bindable gate at angle th, in the layout classify() uses
// for that gate (see bind_coef in plan.cpp).
__device__ __forceinline__ int bind_eval(int kind, double th, double* c) {
    double s, co;
    switch (kind) {
        case QFVM_OP_RX:
            sincos(0.5 * th, &s, &co);
            c[0] = co;
            c[1] = s;
            return 2;
        case QFVM_OP_RY:
            sincos(0.5 * th, &s, &co);
            c[0] = co;
            c[1] = -s;
            c[2] = s;
            c[3] = co;
            return 4;
        case QFVM_OP_RZ:
        case QFVM_OP_RZZ:
            sincos(0.5 * th, &s, &co);
            c[0] = co;
            c[1] = -s;
            c[2] = co;
            c[3] = s;
            return 4;
        case QFVM_OP_P:
        case QFVM_OP_CP:
            sincos(th, &s, &co);
            c[0] = 1.0;
            c[1] = 0.0;
            c[2] = co;
            c[3] = s;
            return 4;
        default: return 0;
    }
}

__device__ __forceinline__ void put_coef(double* d, double v) { *d = v; }
__device__ __forceinline__ void put_coef(float* d, double v) { *d = static_cast<float>(v); }
__device__ __forceinline__ void put_coef(ds* d, double v) {
    const float h = static_cast<float>(v);
    d->h = h;
    d->l = static_cast<float>(v - static_cast<double>(h));
}

// pool[item * cstride + bind.off ..] = coefficients at sign * vals[item * nslots + bind.slot]
template <class C>
__global__ void __launch_bounds__(256) k_bind(C* __restrict__ pool, uint64_t cstride, const Bind* __restrict__ binds,
                                              int nb, const double* __restrict__ vals, int nslots, int items) {
    const uint64_t total = static_cast<uint64_t>(items) * nb;
    for (uint64_t i = blockIdx.x * 256ULL + threadIdx.x; i < total; i += gridDim.x * 256ULL) {
        const uint64_t item = i / nb;
        const Bind bd = binds[i - item * nb];
        const double th = static_cast<double>(bd.sign) * vals[item * nslots + bd.slot];
        double c[4];
        const int m = bind_eval(bd.kind, th, c);
        C* dst = pool + item * cstride + bd.off;
        for (int k = 0; k < m; ++k) put_coef(dst + k, c[k]);
    }
}

// pool[item * cstride + j] = pool[j] for items 1.. (the template is item 0)
template <class C>
__global__ void __launch_bounds__(256) k_replicate(C* __restrict__ pool, uint64_t cstride, uint64_t len, int items) {
    const uint64_t total = static_cast<uint64_t>(items - 1) * len;
    for (uint64_t i = blockIdx.x * 256ULL + threadIdx.x; i < total; i += gridDim.x * 256ULL) {
        const uint64_t item = 1 + i / len, j = i % len;
        pool[item * cstride + j] = pool[j];
    }
}

// amplitude 0 of every item = 1 (the rest was cleared by a memset)
template <class G>
__global__ void k_first_amp(G* __restrict__ state, int n, int items) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < items) {
        G one;
        one.x = 1;
        one.y = 0;
        state[static_cast<uint64_t>(i) << n] = one;
    }
}

// (O psi)[i] for the terms [t0, t1) of a Pauli sum, FP64:
// (P psi)[i] = i^ny (-1)^popcount((i ^ x) & z) psi[i ^ x]  (statevector.hpp:1281-1305)
template <class P>
__device__ __forceinline__ void pauli_sum_at(const typename P::G* __restrict__ psi, uint64_t i,
                                             const uint64_t* __restrict__ xs, const uint64_t* __restrict__ zs,
                                             const int32_t* __restrict__ ny, const double* __restrict__ cs, int t0,
                                             int t1, const double* w, const int32_t* tobs, double& ar, double& ai) {
    uint64_t lastx = ~0ULL;
    double wr = 0.0, wi = 0.0;
    for (int t = t0; t < t1; ++t) {
        const uint64_t x = xs[t];
        if (x != lastx) {
            const typename P::G v = psi[i ^ x];
            wr = P::gre(v);
            wi = P::gim(v);
            lastx = x;
        }
        double c = cs[t];
        if (w) c *= w[tobs[t]];
        if (__popcll((i ^ x) & zs[t]) & 1) c = -c;
        switch (ny[t] & 3) {
            case 0: ar = __fma_rn(c, wr, ar); ai = __fma_rn(c, wi, ai); break;
            case 1: ar = __fma_rn(-c, wi, ar); ai = __fma_rn(c, wr, ai); break;
            case 2: ar = __fma_rn(-c, wr, ar); ai = __fma_rn(-c, wi, ai); break;
            default: ar = __fma_rn(c, wi, ar); ai = __fma_rn(-c, wr, ai); break;
        }
    }
}

// Chunk sums of <psi|O_o|psi> for every observable o (terms optr[o]..optr[o+1]),
// FP64.  CTA c covers amplitudes [c * chunk, (c + 1) * chunk); chunk divides
// 2^n, so a chunk never spans items.  epart[c * nobs + o].
template <class P>
__global__ void __launch_bounds__(256) k_expect_seg(const typename P::G* __restrict__ psi, uint64_t chunk,
                                                    const uint64_t* __restrict__ xs, const uint64_t* __restrict__ zs,
                                                    const int32_t* __restrict__ ny, const double* __restrict__ cs,
                                                    const int32_t* __restrict__ optr, int nobs,
                                                    double* __restrict__ epart) {
    __shared__ double red[8];
    const uint64_t lo = blockIdx.x * chunk;
    for (int o = 0; o < nobs; ++o) {
        double acc = 0.0;
        for (uint64_t i = lo + threadIdx.x; i < lo + chunk; i += 256) {
            double ar = 0.0, ai = 0.0;
            pauli_sum_at<P>(psi, i, xs, zs, ny, cs, optr[o], optr[o + 1], nullptr, nullptr, ar, ai);
            const typename P::G p = psi[i];
            acc = __fma_rn(P::gre(p), ar, acc);
            acc = __fma_rn(P::gim(p), ai, acc);
        }
        const double s = block_sum<256>(acc, red);
        if (threadIdx.x == 0) epart[static_cast<uint64_t>(blockIdx.x) * nobs + o] = s;
    }
}

// lam = sum_o w[item, o] O_o psi for every item (w == nullptr: all weights 1)
template <class P>
__global__ void __launch_bounds__(256) k_lambda_seg(const typename P::G* __restrict__ psi,
                                                    typename P::G* __restrict__ lam, uint64_t total, int n,
                                                    const uint64_t* __restrict__ xs, const uint64_t* __restrict__ zs,
                                                    const int32_t* __restrict__ ny, const double* __restrict__ cs,
                                                    const int32_t* __restrict__ tobs, int nterms, int nobs,
                                                    const double* __restrict__ w) {
    for (uint64_t i = blockIdx.x * 256ULL + threadIdx.x; i < total; i += gridDim.x * 256ULL) {
        double ar = 0.0, ai = 0.0;
        const double* wi = w ? w + (i >> n) * nobs : nullptr;
        pauli_sum_at<P>(psi, i, xs, zs, ny, cs, 0, nterms, wi, tobs, ar, ai);
        lam[i] = P::make_g(ar, ai);
    }
}

// out[i * nobs + o] = sum_{k < per} in[(i * per + k) * nobs + o]
__global__ void k_seg_sum(const double* __restrict__ in, int per, int segs, int nobs, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < segs * nobs) {
        const int seg = i / nobs, o = i - seg * nobs;
        double s = 0.0;
        for (int k = 0; k < per; ++k) s += in[(static_cast<size_t>(seg) * per + k) * nobs + o];
        out[i] = s;
    }
}

// Per-item probe sums of a batched two-state pass: the item's tiles are
// consecutive, partial holds one row of ntiles values per probe.
__global__ void k_probe_reduce_seg(const double* __restrict__ partial, uint64_t ntiles, int tpi, int items, int np,
                                   double* __restrict__ out, int ostride, int ooff) {
    const uint64_t total = static_cast<uint64_t>(items) * np;
    for (uint64_t i = blockIdx.x * 256ULL + threadIdx.x; i < total; i += gridDim.x * 256ULL) {
        const uint64_t item = i / np;
        const int p = static_cast<int>(i - item * np);
        const double* src = partial + static_cast<uint64_t>(p) * ntiles + item * tpi;
        double s = 0.0;
        for (int t = 0; t < tpi; ++t) s += src[t];
        out[item * ostride + ooff + p] = s;
    }
}

// grads[item * nslots + s] = sum over the probes of slot s (ascending probe id)
__global__ void k_slot_gather(const double* __restrict__ vals, int nprobe, int items,
                              const int32_t* __restrict__ sptr, const int32_t* __restrict__ sidx, int nslots,
                              double* __restrict__ grads) {
    const uint64_t total = static_cast<uint64_t>(items) * nslots;
    for (uint64_t i = blockIdx.x * 256ULL + threadIdx.x; i < total; i += gridDim.x * 256ULL) {
        const uint64_t item = i / nslots;
        const int s = static_cast<int>(i - item * nslots);
        double g = 0.0;
        for (int k = sptr[s]; k < sptr[s + 1]; ++k) g += vals[item * nprobe + sidx[k]];
        grads[i] = g;
    }
}

static unsigned blocks_for(uint64_t work, unsigned cap = 152 * 8) {
    const uint64_t b = (work + 255) / 256;
    return static_cast<unsigned>(b < 1 ? 1 : (b < cap ? b : cap));
}

cudaError_t launch_bind(int arith, void* pool, uint64_t cstride, const Bind* dbinds, int nb, const double* dvals,
                        int nslots, int items, cudaStream_t st) {
    if (nb <= 0 || items <= 0) return cudaSuccess;
    const unsigned g = blocks_for(static_cast<uint64_t>(items) * nb);
    if (arith == QFVM_C64)
        k_bind<float><<<g, 256, 0, st>>>(static_cast<float*>(pool), cstride, dbinds, nb, dvals, nslots, items);
    else if (arith == QFVM_C128_DS)
        k_bind<ds><<<g, 256, 0, st>>>(static_cast<ds*>(pool), cstride, dbinds, nb, dvals, nslots, items);
    else
        k_bind<double><<<g, 256, 0, st>>>(static_cast<double*>(pool), cstride, dbinds, nb, dvals, nslots, items);
    return cudaGetLastError();
}

cudaError_t launch_replicate(int arith, void* pool, uint64_t cstride, uint64_t len, int items, cudaStream_t st) {
    if (items <= 1 || len == 0) return cudaSuccess;
    const unsigned g = blocks_for(static_cast<uint64_t>(items - 1) * len);
    if (arith == QFVM_C64)
        k_replicate<float><<<g, 256, 0, st>>>(static_cast<float*>(pool), cstride, len, items);
    else if (arith == QFVM_C128_DS)
        k_replicate<ds><<<g, 256, 0, st>>>(static_cast<ds*>(pool), cstride, len, items);
    else
        k_replicate<double><<<g, 256, 0, st>>>(static_cast<double*>(pool), cstride, len, items);
    return cudaGetLastError();
}

cudaError_t launch_zero_items(int storage, void* state, int n, int items, cudaStream_t st) {
    const size_t bytes = (static_cast<size_t>(items) << n) * (storage == QFVM_C64 ? 8 : 16);
    cudaError_t e = cudaMemsetAsync(state, 0, bytes, st);
    if (e != cudaSuccess) return e;
    const unsigned g = static_cast<unsigned>((items + 255) / 256);
    if (storage == QFVM_C64) k_first_amp<float2><<<g, 256, 0, st>>>(static_cast<float2*>(state), n, items);
    else k_first_amp<double2><<<g, 256, 0, st>>>(static_cast<double2*>(state), n, items);
    return cudaGetLastError();
}

uint64_t hamiltonian_chunk(int n) { return n >= 11 ? 2048ULL : (1ULL << n); }

cudaError_t launch_expect_seg(int storage, const void* psi, int n, int items, const uint64_t* dx, const uint64_t* dz,
                              const int32_t* dny, const double* dc, const int32_t* doptr, int nobs, double* epart,
                              double* out, cudaStream_t st) {
    const uint64_t chunk = hamiltonian_chunk(n);
    const uint64_t per = (1ULL << n) / chunk;
    const uint64_t ctas = per * static_cast<uint64_t>(items);
    if (ctas > 0x7fffffffULL) return cudaErrorInvalidValue;
    if (storage == QFVM_C64)
        k_expect_seg<P32><<<static_cast<unsigned>(ctas), 256, 0, st>>>(static_cast<const float2*>(psi), chunk, dx, dz,
                                                                       dny, dc, doptr, nobs, epart);
    else
        k_expect_seg<P64><<<static_cast<unsigned>(ctas), 256, 0, st>>>(static_cast<const double2*>(psi), chunk, dx,
                                                                       dz, dny, dc, doptr, nobs, epart);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const int outs = items * nobs;
    k_seg_sum<<<(outs + 127) / 128, 128, 0, st>>>(epart, static_cast<int>(per), items, nobs, out);
    return cudaGetLastError();
}

cudaError_t launch_lambda_seg(int storage, const void* psi, void* lam, int n, int items, const uint64_t* dx,
                              const uint64_t* dz, const int32_t* dny, const double* dc, const int32_t* dtobs,
                              int nterms, int nobs, const double* dw, cudaStream_t st) {
    const uint64_t total = static_cast<uint64_t>(items) << n;
    if (storage == QFVM_C64)
        k_lambda_seg<P32><<<blocks_for(total, 152 * 16), 256, 0, st>>>(static_cast<const float2*>(psi),
                                                                       static_cast<float2*>(lam), total, n, dx, dz,
                                                                       dny, dc, dtobs, nterms, nobs, dw);
    else
        k_lambda_seg<P64><<<blocks_for(total, 152 * 16), 256, 0, st>>>(static_cast<const double2*>(psi),
                                                                       static_cast<double2*>(lam), total, n, dx, dz,
                                                                       dny, dc, dtobs, nterms, nobs, dw);
    return cudaGetLastError();
}

cudaError_t launch_probe_reduce_seg(const double* partial, uint64_t ntiles, int tpi, int items, int np, double* out,
                                    int ostride, int ooff, cudaStream_t st) {
    if (np <= 0) return cudaSuccess;
    k_probe_reduce_seg<<<blocks_for(static_cast<uint64_t>(items) * np), 256, 0, st>>>(partial, ntiles, tpi, items, np,
                                                                                     out, ostride, ooff);
    return cudaGetLastError();
}

cudaError_t launch_slot_gather(const double* vals, int nprobe, int items, const int32_t* sptr, const int32_t* sidx,
                               int nslots, double* grads, cudaStream_t st) {
    if (nslots <= 0) return cudaSuccess;
    k_slot_gather<<<blocks_for(static_cast<uint64_t>(items) * nslots), 256, 0, st>>>(vals, nprobe, items, sptr, sidx,
                                                                                    nslots, grads);
    return cudaGetLastError();
}

}  // namespace qsv
