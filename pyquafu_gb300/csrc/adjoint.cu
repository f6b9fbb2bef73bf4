// Adjoint-method kernels and launchers (whole-state two-state passes for small
// states, lam = H psi, probe reductions, and the dispatch of the tiled
// two-state passes, which adjoint_c128.cu, adjoint_ds.cu and adjoint_c64.cu
// instantiate).  The reverse sweep itself is planned by build_adjoint_sweep.
#include "adjoint.cuh"
#include "kernels.h"

namespace qsv {

// Whole-state two-state pass for small states: psi and lam both live in the
// shared memory of one CTA; a probe is reduced over the CTA in a fixed order
// and written straight to probe_out[probe].  CTA b handles item b of a batch:
// states at offset b << n, coefficients at coef0 + b * cstride, probe values
// at probe_out + b * pstride.
template <class P>
__global__ void __launch_bounds__(512) k_small2(typename P::G* __restrict__ psi0, typename P::G* __restrict__ lam0,
                                                int n, const KOp* __restrict__ ops, int nops,
                                                const typename P::C* __restrict__ coef0, uint64_t cstride,
                                                double* __restrict__ probe0, uint64_t pstride) {
    typename P::G* psi_g = psi0 + (static_cast<uint64_t>(blockIdx.x) << n);
    typename P::G* lam_g = lam0 + (static_cast<uint64_t>(blockIdx.x) << n);
    const typename P::C* coef = coef0 + blockIdx.x * cstride;
    double* probe_out = probe0 + blockIdx.x * pstride;
    constexpr int GB = P::GBITS;
    using T = typename ProbeMath<P>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typename P::S* sp = reinterpret_cast<typename P::S*>(smem_raw);
    const uint32_t N = 1u << n;
    typename P::S* sl = sp + N;
    __shared__ double red[32];
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
        sp[swz<GB>(i)] = P::g2s(psi_g[i]);
        sl[swz<GB>(i)] = P::g2s(lam_g[i]);
    }
    __syncthreads();
    for (int oi = 0; oi < nops; ++oi) {
        const KOp o = ops[oi];
        if (o.kind == K_PROBE) {
            double acc = 0.0;
            const uint32_t cm = static_cast<uint32_t>(o.cthr), zm = static_cast<uint32_t>(o.pthr), xm = o.xreg;
            for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
                if ((i & cm) != cm) continue;
                const uint32_t ix = i ^ xm;
                T zr, zi;
                ProbeMath<P>::zc(P::s2a(sl[swz<GB>(i)]), P::s2a(sp[swz<GB>(ix)]), zr, zi);
                const T v = im_rot<T>(zr, zi, o.special);
                acc += static_cast<double>((__popc(ix & zm) & 1) ? -v : v);
            }
            acc = warp_sum(acc);
            const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
            if ((threadIdx.x & 31) == 0) red[w] = acc;
            __syncthreads();
            if (threadIdx.x == 0) {
                double s = 0.0;
                for (int k = 0; k < nw; ++k) s += red[k];
                probe_out[o.probe] = s * P::coef_d(coef, o.coef);
            }
        } else {
            small_apply<P>(sp, n, o, coef);
            small_apply<P>(sl, n, o, coef);
        }
        __syncthreads();
    }
    for (uint32_t i = threadIdx.x; i < N; i += blockDim.x) {
        psi_g[i] = P::s2g(sp[swz<GB>(i)]);
        lam_g[i] = P::s2g(sl[swz<GB>(i)]);
    }
}

// lam = sum_t c_t P_t psi with (P psi)[i] = i^ny (-1)^popcount((i^x) & z) psi[i^x]
// (FP64 accumulation; terms arrive sorted by flip mask).
template <class P>
__global__ void __launch_bounds__(256) k_hamiltonian(const typename P::G* __restrict__ psi,
                                                     typename P::G* __restrict__ lam, uint64_t N,
                                                     const uint64_t* __restrict__ xs, const uint64_t* __restrict__ zs,
                                                     const int32_t* __restrict__ ny, const double* __restrict__ cs,
                                                     int nterms) {
    for (uint64_t i = blockIdx.x * 256ULL + threadIdx.x; i < N; i += gridDim.x * 256ULL) {
        double ar = 0.0, ai = 0.0;
        uint64_t lastx = ~0ULL;
        double wr = 0.0, wi = 0.0;
        for (int t = 0; t < nterms; ++t) {
            const uint64_t x = xs[t];
            if (x != lastx) {
                const typename P::G w = psi[i ^ x];
                wr = P::gre(w);
                wi = P::gim(w);
                lastx = x;
            }
            double c = cs[t];
            if (__popcll((i ^ x) & zs[t]) & 1) c = -c;
            switch (ny[t] & 3) {
                case 0: ar = __fma_rn(c, wr, ar); ai = __fma_rn(c, wi, ai); break;
                case 1: ar = __fma_rn(-c, wi, ar); ai = __fma_rn(c, wr, ai); break;
                case 2: ar = __fma_rn(-c, wr, ar); ai = __fma_rn(-c, wi, ai); break;
                default: ar = __fma_rn(c, wi, ar); ai = __fma_rn(-c, wr, ai); break;
            }
        }
        lam[i] = P::make_g(ar, ai);
    }
}

// values[p] = sum over CTAs of partial[p * grid + b], in CTA order
__global__ void k_probe_reduce(const double* __restrict__ partial, int grid, int np, double* __restrict__ out) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < grid; ++b) s += partial[static_cast<size_t>(p) * grid + b];
        out[p] = s;
    }
}

namespace {

template <class P>
cudaError_t launch_small2_p(void* psi, void* lam, int n, const KOp* dops, int nops, const void* dcoef, int items,
                            uint64_t cstride, double* probe_out, uint64_t pstride, cudaStream_t st) {
    const size_t smem = 2 * (sizeof(typename P::S) << n);
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(k_small2<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    k_small2<P><<<items, n >= 10 ? 512 : 256, smem, st>>>(static_cast<typename P::G*>(psi),
                                                          static_cast<typename P::G*>(lam), n, dops, nops,
                                                          static_cast<const typename P::C*>(dcoef), cstride,
                                                          probe_out, pstride);
    return cudaGetLastError();
}

}  // namespace

void adjoint_shape(int arith, int* T, int* R) {
    if (arith == QFVM_C64) {
        *T = 12;
        *R = 4;
    } else if (arith == QFVM_C128_DS) {
        // three register qubits: the specialised float-pair sweep of two
        // states at R = 4 outgrew the instruction cache (ncu: no_instruction
        // the top stall); 24-qubit gradient 132.9 ms against 191.5 ms
        *T = 11;
        *R = 3;
    } else {
        *T = 11;
        *R = 4;
    }
}

bool pass2_shape_supported(int arith, int T, int R) {
    if (arith == QFVM_C64) return pass2_shape_c64(T, R);
    if (arith == QFVM_C128_DS) return pass2_shape_ds(T, R);
    return pass2_shape_c128(T, R);
}

int adjoint_small_max(int arith) { return arith == QFVM_C64 ? 11 : 10; }

cudaError_t launch_pass2(int arith, int T, int R, void* psi, void* lam, const PassDesc* dpass, const StepDesc* dsteps,
                         const KOp* dops, const void* dcoef, int n, int H, int items, uint64_t cstride, int per_tile,
                         double* partial, int* grid_out, cudaStream_t st) {
    if (arith == QFVM_C64)
        return launch_pass2_c64(T, R, psi, lam, dpass, dsteps, dops, dcoef, n, H, items, cstride, per_tile, partial,
                                grid_out, st);
    if (arith == QFVM_C128_DS)
        return launch_pass2_ds(T, R, psi, lam, dpass, dsteps, dops, dcoef, n, H, items, cstride, per_tile, partial,
                               grid_out, st);
    return launch_pass2_c128(T, R, psi, lam, dpass, dsteps, dops, dcoef, n, H, items, cstride, per_tile, partial,
                             grid_out, st);
}

int pass2_grid_cap() { return 152 * 4; }

cudaError_t launch_small2(int arith, void* psi, void* lam, int n, const KOp* dops, int nops, const void* dcoef,
                          int items, uint64_t cstride, double* probe_out, uint64_t pstride, cudaStream_t st) {
    if (arith == QFVM_C64)
        return launch_small2_p<P32>(psi, lam, n, dops, nops, dcoef, items, cstride, probe_out, pstride, st);
    if (arith == QFVM_C128_DS)
        return launch_small2_p<PDS>(psi, lam, n, dops, nops, dcoef, items, cstride, probe_out, pstride, st);
    return launch_small2_p<P64>(psi, lam, n, dops, nops, dcoef, items, cstride, probe_out, pstride, st);
}

cudaError_t launch_hamiltonian(int storage, const void* psi, void* lam, uint64_t N, const uint64_t* dx,
                               const uint64_t* dz, const int32_t* dny, const double* dc, int nterms, cudaStream_t st) {
    uint64_t blocks = (N + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (storage == QFVM_C64)
        k_hamiltonian<P32><<<static_cast<unsigned>(blocks), 256, 0, st>>>(static_cast<const float2*>(psi),
                                                                          static_cast<float2*>(lam), N, dx, dz, dny,
                                                                          dc, nterms);
    else
        k_hamiltonian<P64><<<static_cast<unsigned>(blocks), 256, 0, st>>>(static_cast<const double2*>(psi),
                                                                          static_cast<double2*>(lam), N, dx, dz, dny,
                                                                          dc, nterms);
    return cudaGetLastError();
}

cudaError_t launch_probe_reduce(const double* partial, int grid, int np, double* out, cudaStream_t st) {
    if (np <= 0) return cudaSuccess;
    k_probe_reduce<<<(np + 63) / 64, 64, 0, st>>>(partial, grid, np, out);
    return cudaGetLastError();
}

}  // namespace qsv
