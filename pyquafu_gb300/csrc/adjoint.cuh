// Adjoint-method kernels: two states (psi, lam) swept backwards through the
// inverse gates, with "probes" that accumulate Im<lam| Q |psi> for the
// generator Q of every parameterised gate (quafu/algorithms/gradients/
// gradiant.py:144-173 computes the same quantity one gate at a time).
#pragma once
#include "device.cuh"

namespace qsv {

// Probe accumulator type: FP64 for complex128 storage, FP32 per thread (then
// FP64 across the warp, CTA and grid) for complex64.
template <class P>
struct ProbeMath;

template <>
struct ProbeMath<P64> {
    using T = double;
    __device__ static __forceinline__ void zc(const double2& l, const double2& w, T& zr, T& zi) {
        zr = __fma_rn(l.x, w.x, __dmul_rn(l.y, w.y));   // Re conj(l) w
        zi = __fma_rn(l.x, w.y, -__dmul_rn(l.y, w.x));  // Im conj(l) w
    }
};
template <>
struct ProbeMath<P32> {
    using T = float;
    __device__ static __forceinline__ void zc(const float2& l, const float2& w, T& zr, T& zi) {
        zr = __fmaf_rn(l.x, w.x, __fmul_rn(l.y, w.y));
        zi = __fmaf_rn(l.x, w.y, -__fmul_rn(l.y, w.x));
    }
};
template <>
struct ProbeMath<PDS> {
    using T = double;
    __device__ static __forceinline__ void zc(const ds2& l, const ds2& w, T& zr, T& zi) {
        const double lr = ds_to_double(l.x), li = ds_to_double(l.y);
        const double wr = ds_to_double(w.x), wi = ds_to_double(w.y);
        zr = __fma_rn(lr, wr, __dmul_rn(li, wi));
        zi = __fma_rn(lr, wi, -__dmul_rn(li, wr));
    }
};

// Im(conj(l) * i^ny * w) from z = conj(l) w
template <class T>
__device__ __forceinline__ T im_rot(T zr, T zi, int ny) {
    switch (ny & 3) {
        case 0: return zi;
        case 1: return zr;
        case 2: return -zi;
        default: return -zr;
    }
}

// One thread's share of a probe in a register round:
//   sum_j (-1)^parity((j ^ XM) & Z) conj(lam_j) psi_(j ^ XM)   (j over the registers)
// accumulated as a complex pair, so the i^ny rotation and the thread's own
// parity bit are applied once per probe, not per amplitude.  XM (flip bits)
// is compile-time; ZM >= 0 is the compile-time Z mask, ZM < 0 reads `zrt`.
template <class P, int R, int XM, int ZM>
__device__ __forceinline__ void probe_sum(const typename P::A (&psi)[1 << R], const typename P::A (&lam)[1 << R],
                                          uint32_t creg, uint32_t zrt, typename ProbeMath<P>::T& ar,
                                          typename ProbeMath<P>::T& ai) {
    using T = typename ProbeMath<P>::T;
#pragma unroll
    for (int j = 0; j < (1 << R); ++j) {
        if ((static_cast<uint32_t>(j) & creg) != creg) continue;  // warp-uniform
        const int jx = j ^ XM;
        const bool neg = ZM >= 0 ? ((__popc(static_cast<uint32_t>(jx & (ZM < 0 ? 0 : ZM))) & 1) != 0)
                                 : ((__popc(static_cast<uint32_t>(jx) & zrt) & 1) != 0);
        T zr, zi;
        ProbeMath<P>::zc(lam[j], psi[jx], zr, zi);
        if (neg) {
            ar -= zr;
            ai -= zi;
        } else {
            ar += zr;
            ai += zi;
        }
    }
}

template <class P, int R>
__device__ __forceinline__ typename ProbeMath<P>::T reg_probe(const typename P::A (&psi)[1 << R],
                                                              const typename P::A (&lam)[1 << R], const KOp& op,
                                                              uint64_t gthr) {
    using T = typename ProbeMath<P>::T;
    if ((op.flags & F_TCTRL) && (gthr & op.cthr) != op.cthr) return T(0);
    const int pt = (op.flags & F_TPAR) ? (__popcll(gthr & op.pthr) & 1) : 0;
    T ar = T(0), ai = T(0);
    const uint32_t x = op.xreg, z = op.preg, c = op.creg;
    if (x == 0) {
        if (z == 0) {
            probe_sum<P, R, 0, 0>(psi, lam, c, z, ar, ai);
        } else if ((z & (z - 1)) == 0) {
            with_bit<R>(__ffs(z) - 1, [&](auto b) {
                constexpr int B = decltype(b)::value;
                probe_sum<P, R, 0, (1 << B)>(psi, lam, c, z, ar, ai);
            });
        } else {
            probe_sum<P, R, 0, -1>(psi, lam, c, z, ar, ai);
        }
    } else if ((x & (x - 1)) == 0) {
        with_bit<R>(__ffs(x) - 1, [&](auto b) {
            constexpr int B = decltype(b)::value;
            if (z == 0) probe_sum<P, R, (1 << B), 0>(psi, lam, c, z, ar, ai);
            else if (z == x) probe_sum<P, R, (1 << B), (1 << B)>(psi, lam, c, z, ar, ai);
            else probe_sum<P, R, (1 << B), -1>(psi, lam, c, z, ar, ai);
        });
    } else {
        const int b0 = __ffs(x) - 1;
        const int b1 = __ffs(x & (x - 1)) - 1;
        with_bit<R>(b0, [&](auto c0) {
            constexpr int B0 = decltype(c0)::value;
            with_bit<R>(b1, [&](auto c1) {
                constexpr int B1 = decltype(c1)::value;
                if constexpr (B0 != B1) probe_sum<P, R, (1 << B0) | (1 << B1), -1>(psi, lam, c, z, ar, ai);
            });
        });
    }
    const T v = im_rot<T>(ar, ai, op.special);
    return pt ? -v : v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// Two-state fused tile pass (persistent, double-buffered, like k_pass).
// Gates apply to both states; probes add their warp sums into pacc[warp][p]
// in a fixed order.  Single state (per_tile == 0): at the end every CTA writes
// its per-probe total to partial[p * gridDim.x + blockIdx.x].  Batched states
// (per_tile == 1): tile b belongs to item b >> ishift, reads that item's
// coefficients at coef0 + item * cstride, and writes its own per-probe sums to
// partial[p * ntiles + b], so sums never mix items.
// ---------------------------------------------------------------------------
template <class P, int T, int R, int NB, int MINB>
__global__ void __launch_bounds__(1 << (T - R), MINB)
    k_pass2(typename P::G* __restrict__ psi_g, typename P::G* __restrict__ lam_g, uint64_t ntiles,
            const PassDesc* __restrict__ pdp, const StepDesc* __restrict__ steps, const KOp* __restrict__ ops,
            const typename P::C* __restrict__ coef0, uint64_t cstride, int ishift, int per_tile,
            double* __restrict__ partial) {
    constexpr int NT = 1 << (T - R);
    constexpr int NW = NT / 32;
    constexpr int NA = 1 << R;
    constexpr int PER = (1 << T) / NT;
    constexpr uint32_t TE = tile_elems(T, sizeof(typename P::S));  // elements per tile buffer
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typename P::S* base_s = reinterpret_cast<typename P::S*>(smem_raw);
    // buffers: [slot][state], NB slots
    uint64_t* choff = reinterpret_cast<uint64_t*>(smem_raw + 2 * NB * sizeof(typename P::S) * TE);
    double* pacc = reinterpret_cast<double*>(choff + (1 << pdp->H));

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t stid = sm_off<P, true>(static_cast<uint32_t>(tid));
    const int L = pdp->L, H = pdp->H;
    const uint8_t* tq = pdp->tq;
    const int np = pdp->nprobe;
    for (int c = tid; c < (1 << H); c += NT) {
        uint64_t off = 0;
        for (int k = 0; k < H; ++k)
            if ((c >> k) & 1) off |= 1ULL << tq[L + k];
        choff[c] = off;
    }
    for (int i = tid; i < NW * MAX_PASS_PROBES; i += NT) pacc[i] = 0.0;
    __syncthreads();
    const uint32_t lmask = (1u << L) - 1;
    const int nsteps = pdp->step_count;
    auto buf = [&](int slot, int st) { return base_s + (2 * (slot & (NB - 1)) + st) * TE; };

    uint64_t b = blockIdx.x;
    if (NB == 2 && b < ntiles) {
        const uint64_t bb = tile_base(b, L, H, tq);
        tile_prefetch<P, T, NT>(buf(0, 0), psi_g, bb, choff, L);
        tile_prefetch<P, T, NT>(buf(0, 1), lam_g, bb, choff, L);
    }
    for (int it = 0; b < ntiles; ++it, b += gridDim.x) {
        typename P::S* sm[2] = {buf(it, 0), buf(it, 1)};
        const uint64_t base = tile_base(b, L, H, tq);
        const typename P::C* coef = coef0 + (b >> ishift) * cstride;
        if constexpr (NB == 1) {
            tile_prefetch<P, T, NT>(sm[0], psi_g, base, choff, L);
            tile_prefetch<P, T, NT>(sm[1], lam_g, base, choff, L);
            cp_async_wait<0>();
        } else {
            const uint64_t bn = b + gridDim.x;
            if (bn < ntiles) {
                const uint64_t nb = tile_base(bn, L, H, tq);
                tile_prefetch<P, T, NT>(buf(it + 1, 0), psi_g, nb, choff, L);
                tile_prefetch<P, T, NT>(buf(it + 1, 1), lam_g, nb, choff, L);
                cp_async_wait<2>();
            } else {
                cp_async_wait<0>();
            }
        }
        __syncthreads();
        if constexpr (P::RAW_STAGING) {
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const uint32_t ad = sm_off<P, true>(static_cast<uint32_t>(k * NT)) + stid;
                sm[0][ad] = P::g2s(P::raw_to_g(sm[0][ad]));
                sm[1][ad] = P::g2s(P::raw_to_g(sm[1][ad]));
            }
            __syncthreads();
        }
        const StepDesc* sd = steps + pdp->step_begin;
        for (int si = 0; si < nsteps; ++si, ++sd) {
            if (sd->type == STEP_SMEM) {
                for (int oi = 0; oi < sd->op_count; ++oi) {
                    tile_smem_op<P>(sm[0], T, base, ops[sd->op_begin + oi], coef);
                    tile_smem_op<P>(sm[1], T, base, ops[sd->op_begin + oi], coef);
                    __syncthreads();
                }
                continue;
            }
            // the thread's base offset in the tile layout and its global
            // index: both are sums over its index bits
            uint32_t psb = 0;
            uint64_t gthr = base;
#pragma unroll
            for (int k = 0; k < T - R; ++k) {
                if ((tid >> k) & 1) {
                    psb += sd->tsw[k];
                    gthr |= 1ULL << sd->tglob[k];
                }
            }
            uint32_t rsw[R];
#pragma unroll
            for (int k = 0; k < R; ++k) rsw[k] = sd->rsw[k];
            typename P::A a[2][NA];
#pragma unroll
            for (int j = 0; j < NA; ++j) {
                uint32_t ad = psb;
#pragma unroll
                for (int k = 0; k < R; ++k)
                    if ((j >> k) & 1) ad += rsw[k];
                a[0][j] = P::s2a(sm[0][ad]);
                a[1][j] = P::s2a(sm[1][ad]);
            }
            RoundPhase<P> ph;
            ph.reset();
            const KOp* op = ops + sd->op_begin;
            for (int oi = 0; oi < sd->op_count; ++oi) {
                const KOp o = op[oi];
                if (o.kind == K_PROBE) {
                    // pending uniform phases act on both states alike, so the
                    // probe (a product of conj(lam) and psi) is unaffected by
                    // them; the warp sum runs in the probe type (FP32 for
                    // complex64), FP64 from the warp total on
                    const auto ws = warp_sum(reg_probe<P, R>(a[0], a[1], o, gthr));
                    if constexpr (std::is_same<P, P32>::value) {
                        // the generator scale (1 or -2) is exact in FP32: one
                        // conversion and one FP64 add per probe and warp
                        const float vf = ws * P::coef(coef, o.coef);
                        if (lane == 0) pacc[warp * MAX_PASS_PROBES + o.probe] += static_cast<double>(vf);
                    } else {
                        const double v = static_cast<double>(ws);
                        if (lane == 0) pacc[warp * MAX_PASS_PROBES + o.probe] += v * P::coef_d(coef, o.coef);
                    }
                } else {
                    reg_apply<P, R, 2>(a, o, gthr, coef, ph);
                }
            }
            reg_finish_phase<P, R, 2>(a, ph);
            uint32_t psb2 = psb;
            asm volatile("" : "+r"(psb2));
#pragma unroll
            for (int j = 0; j < NA; ++j) {
                uint32_t ad = psb2;
#pragma unroll
                for (int k = 0; k < R; ++k)
                    if ((j >> k) & 1) ad += rsw[k];
                sm[0][ad] = P::a2s(a[0][j]);
                sm[1][ad] = P::a2s(a[1][j]);
            }
            __syncthreads();
        }
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const uint32_t s = static_cast<uint32_t>(k * NT) | tid;
            const uint64_t g = base | choff[s >> L] | (s & lmask);
            const uint32_t ad = sm_off<P, true>(static_cast<uint32_t>(k * NT)) + stid;
            __stcs(psi_g + g, P::s2g(sm[0][ad]));
            __stcs(lam_g + g, P::s2g(sm[1][ad]));
        }
        __syncthreads();
        if (per_tile) {
            for (int p = tid; p < np; p += NT) {
                double s = 0.0;
                for (int w = 0; w < NW; ++w) {
                    s += pacc[w * MAX_PASS_PROBES + p];
                    pacc[w * MAX_PASS_PROBES + p] = 0.0;
                }
                partial[static_cast<size_t>(p) * ntiles + b] = s;
            }
            __syncthreads();
        }
    }
    if (per_tile) return;
    __syncthreads();
    for (int p = tid; p < np; p += NT) {
        double s = 0.0;
        for (int w = 0; w < NW; ++w) s += pacc[w * MAX_PASS_PROBES + p];
        partial[static_cast<size_t>(p) * gridDim.x + blockIdx.x] = s;
    }
}

}  // namespace qsv
