// Device-side building blocks of the statevector kernels (templates shared by
// the per-precision translation units).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "engine.h"
#include "policy.cuh"

namespace qsv {

// ---------------------------------------------------------------------------
// shared-memory swizzle: XOR-fold the higher index bits onto the bits that
// select the 16-byte (or 8-byte) slot inside a 128-byte wavefront.  Bit p of
// the element index lands on slot bit (p mod GB), so any GB lane bits with
// distinct residues mod GB hit distinct bank groups.
// ---------------------------------------------------------------------------
template <int GB>
__device__ __forceinline__ uint32_t swz(uint32_t s) {
    constexpr uint32_t M = (1u << GB) - 1;
    uint32_t x = s;
#pragma unroll
    for (int k = 1; k * GB < 32; ++k) x ^= (s >> (k * GB)) & M;
    return x;
}

// Element offset of index i in shared memory: whole-state kernels use the
// XOR swizzle above, tile passes the padded tile layout (tile_off, engine.h).
template <class P, bool TILE>
__device__ __forceinline__ uint32_t sm_off(uint32_t i) {
    if constexpr (TILE) return tile_off(i, 16u / sizeof(typename P::S));
    else return swz<P::GBITS>(i);
}

__device__ __forceinline__ uint64_t insert0(uint64_t j, int p) {
    return ((j >> p) << (p + 1)) | (j & ((1ULL << p) - 1));
}

template <int N, class F>
__device__ __forceinline__ void with_bit(int b, F&& f) {
    switch (b) {
        case 0: f(std::integral_constant<int, 0>()); break;
        case 1: if constexpr (N > 1) f(std::integral_constant<int, 1>()); break;
        case 2: if constexpr (N > 2) f(std::integral_constant<int, 2>()); break;
        case 3: if constexpr (N > 3) f(std::integral_constant<int, 3>()); break;
        case 4: if constexpr (N > 4) f(std::integral_constant<int, 4>()); break;
        case 5: if constexpr (N > 5) f(std::integral_constant<int, 5>()); break;
        default: break;
    }
}

// ---------------------------------------------------------------------------
// Register-round operations: a thread holds 2^R amplitudes of each of NS
// states (the adjoint sweep carries psi and lam together); they differ in the
// R register bits, and target bits are compile-time after the with_bit
// dispatch.  One dispatch serves all NS states, whose arithmetic interleaves.
// ---------------------------------------------------------------------------
template <class P, int R, int NS>
using RegState = typename P::A[NS][1 << R];

template <class P, int R, int NS, int TB, bool CTRL, class F>
__device__ __forceinline__ void reg_pairs(RegState<P, R, NS>& a, uint32_t creg, F&& f) {
#pragma unroll
    for (int j = 0; j < (1 << R); ++j) {
        if (j & (1 << TB)) continue;
        // controls inside the registers: creg is warp-uniform, so this
        // branch never diverges
        if (CTRL && (static_cast<uint32_t>(j) & creg) != creg) continue;
#pragma unroll
        for (int s = 0; s < NS; ++s) f(a[s][j], a[s][j | (1 << TB)]);
    }
}

template <class P, int R, int NS, bool CTRL>
__device__ __forceinline__ void reg_op1(RegState<P, R, NS>& a, const KOp& op, const typename P::C* coef) {
    using C = typename P::C;
    using A = typename P::A;
    const uint32_t creg = op.creg;
    switch (op.kind) {
        case K_X:
            if (CTRL && (creg & (creg - 1)) == 0) {
                // one register control (cx): the swapped pairs are known at
                // compile time after dispatching the control bit as well
                with_bit<R>(__ffs(creg) - 1, [&](auto cb) {
                    constexpr int CB = decltype(cb)::value;
                    with_bit<R>(op.t0, [&](auto tb) {
                        constexpr int TB = decltype(tb)::value;
#pragma unroll
                        for (int j = 0; j < (1 << R); ++j) {
                            if ((j & (1 << TB)) || !(j & (1 << CB))) continue;
#pragma unroll
                            for (int s = 0; s < NS; ++s) {
                                A t = a[s][j];
                                a[s][j] = a[s][j | (1 << TB)];
                                a[s][j | (1 << TB)] = t;
                            }
                        }
                    });
                });
                break;
            }
            with_bit<R>(op.t0, [&](auto tb) {
                constexpr int TB = decltype(tb)::value;
                reg_pairs<P, R, NS, TB, CTRL>(a, creg, [](A& x, A& y) {
                    A t = x;
                    x = y;
                    y = t;
                });
            });
            break;
        case K_Y:
            with_bit<R>(op.t0, [&](auto tb) {
                constexpr int TB = decltype(tb)::value;
                reg_pairs<P, R, NS, TB, CTRL>(a, creg, [](A& x, A& y) { pair_y<P>(x, y); });
            });
            break;
        case K_HAD:
            with_bit<R>(op.t0, [&](auto tb) {
                constexpr int TB = decltype(tb)::value;
                reg_pairs<P, R, NS, TB, CTRL>(a, creg, [](A& x, A& y) { pair_had<P>(x, y); });
            });
            break;
        case K_REAL: {
            C mm[4];
            P::coef4(coef, op.coef, mm);
            const C m0 = mm[0], m1 = mm[1], m2 = mm[2], m3 = mm[3];
            with_bit<R>(op.t0, [&](auto tb) {
                constexpr int TB = decltype(tb)::value;
                reg_pairs<P, R, NS, TB, CTRL>(a, creg, [&](A& x, A& y) { pair_real<P>(x, y, m0, m1, m2, m3); });
            });
            break;
        }
        case K_RX: {
            const C c = P::coef(coef, op.coef), s = P::coef(coef, op.coef + 1);
            const C ns = P::cneg(s);
            with_bit<R>(op.t0, [&](auto tb) {
                constexpr int TB = decltype(tb)::value;
                reg_pairs<P, R, NS, TB, CTRL>(a, creg, [&](A& x, A& y) { pair_rx<P>(x, y, c, s, ns); });
            });
            break;
        }
        case K_DENSE: {
            C m[8], nmi[4], lo[4], hi[4];
            P::coef4(coef, op.coef, lo);
            P::coef4(coef, op.coef + 4, hi);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                m[i] = lo[i];
                m[4 + i] = hi[i];
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) nmi[i] = P::cneg(m[2 * i + 1]);
            with_bit<R>(op.t0, [&](auto tb) {
                constexpr int TB = decltype(tb)::value;
                reg_pairs<P, R, NS, TB, CTRL>(a, creg, [&](A& x, A& y) { pair_dense<P>(x, y, m, nmi); });
            });
            break;
        }
        default: break;
    }
}

template <class P, int R, int NS, bool CTRL>
__device__ __forceinline__ void reg_swap(RegState<P, R, NS>& a, const KOp& op) {
    const uint32_t creg = op.creg;
    with_bit<R>(op.t0, [&](auto b0) {
        constexpr int B0 = decltype(b0)::value;
        with_bit<R>(op.t1, [&](auto b1) {
            constexpr int B1 = decltype(b1)::value;
            // SWAP is symmetric in its two targets: order the register bits
            if constexpr (B0 != B1) {
                constexpr int LO = B0 < B1 ? B0 : B1;
                constexpr int HI = B0 < B1 ? B1 : B0;
#pragma unroll
                for (int j = 0; j < (1 << R); ++j) {
                    if (j & ((1 << LO) | (1 << HI))) continue;
                    if (CTRL && (static_cast<uint32_t>(j) & creg) != creg) continue;
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        typename P::A t = a[s][j | (1 << LO)];
                        a[s][j | (1 << LO)] = a[s][j | (1 << HI)];
                        a[s][j | (1 << HI)] = t;
                    }
                }
            }
        });
    });
}

// Accumulated thread-uniform phase of a register round (the same for every
// state of the round: all states see the same gates).
// Quarter turns (multiples of i) are counted apart from the general phase,
// so a round whose uniform phases are all quarter turns costs no
// multiplication: swaps and sign flips at the end.
template <class P>
struct RoundPhase {
    typename P::A f;
    bool on;
    int q4;  // accumulated i^q4
    __device__ __forceinline__ void reset() {
        f = P::one();
        on = false;
        q4 = 0;
    }
};

// quarter turns of a special phase: -1 = i^2, i = i^1, -i = i^3
__device__ __forceinline__ int special_quarters(int sp) { return sp == SP_NEG1 ? 2 : (sp == SP_I ? 1 : 3); }
// the special-phase code of i^q (q = 1, 2, 3)
__device__ __forceinline__ int quarters_special(int q) { return q == 2 ? SP_NEG1 : (q == 1 ? SP_I : SP_NEGI); }

template <class P>
__device__ __forceinline__ void phase_mul(typename P::A& f, typename P::C dr, typename P::C di) {
    amp_phase<P>(f, dr, di, P::cneg(di));
}

// Diagonal ops.  Three shapes, chosen by the planner:
//  F_UNIFORM  no parity or control bit in the registers: one factor per
//             thread, folded into the round's phase (it commutes with every
//             op of the round) and applied once when the round ends;
//  F_ONEBIT   exactly one parity bit in the registers (t0), no register
//             control: two factors per thread, bit position compile-time;
//  otherwise  per-amplitude parity and control, branch-free selects.
template <class P, int R, int NS>
__device__ __forceinline__ void reg_diag(RegState<P, R, NS>& a, const KOp& op, uint64_t gthr,
                                         const typename P::C* coef, RoundPhase<P>& ph) {
    using C = typename P::C;
    const int pt = (op.flags & F_TPAR) ? (__popcll(gthr & op.pthr) & 1) : 0;
    const bool d0one = (op.flags & F_D0_ONE) != 0;
    if (op.flags & F_UNIFORM) {
        if (pt == 0 && d0one) return;
        if (pt == 1 && (op.flags & F_D1_SPEC)) {  // d0 = 1, d1 a quarter turn
            ph.q4 += special_quarters(op.special);
            return;
        }
        const uint32_t o = op.coef + (pt ? 2u : 0u);
        phase_mul<P>(ph.f, P::coef(coef, o), P::coef(coef, o + 1));
        ph.on = true;
        return;
    }
    if (op.flags & F_ONEBIT) {
        C dd[4];
        P::coef4(coef, op.coef, dd);
        with_bit<R>(op.t0, [&](auto tb) {
            constexpr int TB = decltype(tb)::value;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int idx = pt ^ h;
                if (idx == 0 && d0one) continue;
                if (idx == 1 && (op.flags & F_D1_SPEC)) {  // quarter turn: swaps and sign flips only
#pragma unroll
                    for (int j = 0; j < (1 << R); ++j)
                        if (((j >> TB) & 1) == h) {
#pragma unroll
                            for (int s = 0; s < NS; ++s) amp_special<P>(a[s][j], op.special);
                        }
                    continue;
                }
                const C dr = idx ? dd[2] : dd[0], di = idx ? dd[3] : dd[1], ndi = P::cneg(di);
#pragma unroll
                for (int j = 0; j < (1 << R); ++j)
                    if (((j >> TB) & 1) == h) {
#pragma unroll
                        for (int s = 0; s < NS; ++s) amp_phase<P>(a[s][j], dr, di, ndi);
                    }
            }
        });
        return;
    }
    const uint32_t creg = op.creg, preg = op.preg;
    C dd[4];
    P::coef4(coef, op.coef, dd);
    const C d0r = dd[0], d0i = dd[1], d1r = dd[2], d1i = dd[3];
    const C nd0i = P::cneg(d0i), nd1i = P::cneg(d1i);
#pragma unroll
    for (int j = 0; j < (1 << R); ++j) {
        if ((static_cast<uint32_t>(j) & creg) != creg) continue;  // warp-uniform
        // the parity depends on the thread: selects, no divergent branch
        const bool par = (pt ^ (__popc(static_cast<uint32_t>(j) & preg) & 1)) != 0;
        const C dr = par ? d1r : d0r;
        const C di = par ? d1i : d0i;
        const C ndi = par ? nd1i : nd0i;
#pragma unroll
        for (int s = 0; s < NS; ++s) amp_phase<P>(a[s][j], dr, di, ndi);
    }
}

template <class P, int R, int NS>
__device__ __forceinline__ void reg_apply(RegState<P, R, NS>& a, const KOp& op, uint64_t gthr,
                                          const typename P::C* coef, RoundPhase<P>& ph) {
    if ((op.flags & F_TCTRL) && (gthr & op.cthr) != op.cthr) return;  // a control outside the registers is 0
    switch (op.kind) {
        case K_DIAG: reg_diag<P, R, NS>(a, op, gthr, coef, ph); break;
        case K_DIAGR:
#pragma unroll
            for (int j = 0; j < (1 << R); ++j) {
                const int code = diagr_code(op, j);
                if (code == DIAGR_ONE) continue;
                if (code != DIAGR_GENERAL) {
                    const int sp = code == DIAGR_NEG1 ? SP_NEG1 : (code == DIAGR_I ? SP_I : SP_NEGI);
#pragma unroll
                    for (int s = 0; s < NS; ++s) amp_special<P>(a[s][j], sp);
                    continue;
                }
                const typename P::C dr = P::coef(coef, op.coef + 2 * j), di = P::coef(coef, op.coef + 2 * j + 1);
                const typename P::C ndi = P::cneg(di);
#pragma unroll
                for (int s = 0; s < NS; ++s) amp_phase<P>(a[s][j], dr, di, ndi);
            }
            break;
        case K_SWAP:
            if (op.creg) reg_swap<P, R, NS, true>(a, op);
            else reg_swap<P, R, NS, false>(a, op);
            break;
        default:
            if (op.creg) reg_op1<P, R, NS, true>(a, op, coef);
            else reg_op1<P, R, NS, false>(a, op, coef);
            break;
    }
}

// Applies a round's accumulated phase to every state.
template <class P, int R, int NS>
__device__ __forceinline__ void reg_finish_phase(RegState<P, R, NS>& a, const RoundPhase<P>& ph) {
    const int q = ph.q4 & 3;
    if (!ph.on) {
        if (q == 0) return;
        const int sp = quarters_special(q);
#pragma unroll
        for (int s = 0; s < NS; ++s)
#pragma unroll
            for (int j = 0; j < (1 << R); ++j) amp_special<P>(a[s][j], sp);
        return;
    }
    typename P::A f = ph.f;
    if (q) amp_special<P>(f, quarters_special(q));  // fold i^q into the phase: once per thread
    const typename P::C nfi = P::cneg(f.y);
#pragma unroll
    for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int j = 0; j < (1 << R); ++j) amp_phase<P>(a[s][j], f.x, f.y, nfi);
}

// ---------------------------------------------------------------------------
// Whole-state pass: the state (<= 2^13 complex128 / 2^14 complex64) lives in
// shared memory of one CTA per state; every gate is one sweep over it.
// blockIdx.x selects a state of a batch (stride `stride` elements).
// ---------------------------------------------------------------------------
template <class P, bool TILE = false>
__device__ __forceinline__ void small_apply(typename P::S* sm, int n, const KOp& op, const typename P::C* coef) {
    using A = typename P::A;
    using C = typename P::C;
    const uint32_t N = 1u << n;
    const int tid = threadIdx.x, nt = blockDim.x;
    const uint32_t cm = static_cast<uint32_t>(op.cthr);
    switch (op.kind) {
        case K_DIAG: {
            const uint32_t pm = static_cast<uint32_t>(op.pthr);
            const C d0r = P::coef(coef, op.coef), d0i = P::coef(coef, op.coef + 1);
            const C d1r = P::coef(coef, op.coef + 2), d1i = P::coef(coef, op.coef + 3);
            for (uint32_t i = tid; i < N; i += nt) {
                if ((i & cm) != cm) continue;
                const int par = __popc(i & pm) & 1;
                if (!par && (op.flags & F_D0_ONE)) continue;
                const uint32_t ad = sm_off<P, TILE>(i);
                A v = P::s2a(sm[ad]);
                if (op.flags & F_D1_SPEC) amp_special<P>(v, op.special);
                else if (par) amp_phase<P>(v, d1r, d1i, P::cneg(d1i));
                else amp_phase<P>(v, d0r, d0i, P::cneg(d0i));
                sm[ad] = P::a2s(v);
            }
            break;
        }
        case K_SWAP:
        case K_DENSE2: {
            const int t0 = op.t0, t1 = op.t1;
            const int lo = t0 < t1 ? t0 : t1, hi = t0 < t1 ? t1 : t0;
            for (uint32_t qd = tid; qd < (N >> 2); qd += nt) {
                const uint32_t i = static_cast<uint32_t>(insert0(insert0(qd, lo), hi));
                if ((i & cm) != cm) continue;
                const uint32_t a0 = sm_off<P, TILE>(i), a1 = sm_off<P, TILE>(i | (1u << t0)), a2 = sm_off<P, TILE>(i | (1u << t1)),
                               a3 = sm_off<P, TILE>(i | (1u << t0) | (1u << t1));
                A v0 = P::s2a(sm[a0]), v1 = P::s2a(sm[a1]), v2 = P::s2a(sm[a2]), v3 = P::s2a(sm[a3]);
                if (op.kind == K_SWAP) {
                    A t = v1;
                    v1 = v2;
                    v2 = t;
                } else {
                    quad_dense<P>(v0, v1, v2, v3, coef, op.coef);
                }
                sm[a0] = P::a2s(v0);
                sm[a1] = P::a2s(v1);
                sm[a2] = P::a2s(v2);
                sm[a3] = P::a2s(v3);
            }
            break;
        }
        case K_DENSEK: {
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
            for (uint32_t g = tid; g < (N >> k); g += nt) {
                uint32_t i = g;
                for (int j = 0; j < k; ++j) i = static_cast<uint32_t>(insert0(i, srt[j]));
                if ((i & cm) != cm) continue;
                A in[1 << MAXK];
                for (uint32_t m = 0; m < dim; ++m) {
                    uint32_t idx = i;
                    for (int j = 0; j < k; ++j)
                        if ((m >> j) & 1) idx |= 1u << op.tk[j];
                    in[m] = P::s2a(sm[sm_off<P, TILE>(idx)]);
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
                    uint32_t idx = i;
                    for (int j = 0; j < k; ++j)
                        if ((r >> j) & 1) idx |= 1u << op.tk[j];
                    A o;
                    o.x = xr;
                    o.y = xi;
                    sm[sm_off<P, TILE>(idx)] = P::a2s(o);
                }
            }
            break;
        }
        default: {
            const int t = op.t0;
            C m[8], nmi[4];
            if (op.kind == K_REAL) {
                for (int x = 0; x < 4; ++x) m[x] = P::coef(coef, op.coef + x);
            } else if (op.kind == K_RX) {
                m[0] = P::coef(coef, op.coef);
                m[1] = P::coef(coef, op.coef + 1);
                m[2] = P::cneg(m[1]);
            } else if (op.kind == K_DENSE) {
                for (int x = 0; x < 8; ++x) m[x] = P::coef(coef, op.coef + x);
                for (int x = 0; x < 4; ++x) nmi[x] = P::cneg(m[2 * x + 1]);
            }
            for (uint32_t pr = tid; pr < (N >> 1); pr += nt) {
                const uint32_t i0 = static_cast<uint32_t>(insert0(pr, t));
                if ((i0 & cm) != cm) continue;
                const uint32_t a0 = sm_off<P, TILE>(i0), a1 = sm_off<P, TILE>(i0 | (1u << t));
                A x = P::s2a(sm[a0]), y = P::s2a(sm[a1]);
                switch (op.kind) {
                    case K_X: {
                        A tt = x;
                        x = y;
                        y = tt;
                        break;
                    }
                    case K_Y: pair_y<P>(x, y); break;
                    case K_HAD: pair_had<P>(x, y); break;
                    case K_REAL: pair_real<P>(x, y, m[0], m[1], m[2], m[3]); break;
                    case K_RX: pair_rx<P>(x, y, m[0], m[1], m[2]); break;
                    case K_DENSE: pair_dense<P>(x, y, m, nmi); break;
                    default: break;
                }
                sm[a0] = P::a2s(x);
                sm[a1] = P::a2s(y);
            }
            break;
        }
    }
}

// ---------------------------------------------------------------------------
// Fused tile pass (persistent, double-buffered).
//
// A tile is 2^T amplitudes: tile-local bit k is global qubit tq[k], and the
// low L qubits are the contiguous qubits 0..L-1, so every global access is a
// run of 2^L amplitudes.  Each CTA walks tiles blockIdx.x, +gridDim.x, ...:
// while it computes tile i in one shared-memory buffer, the asynchronous
// copies (cp.async, 8 or 16 bytes per element, written straight to the
// element's place in the tile layout, tile_off of engine.h) of tile i+1 land
// in the other.  (The circuit-specialised passes of jit_ptx.cpp move whole
// runs with bulk copies instead.)  A tile's gates run in
// register rounds: each thread loads 2^R amplitudes that differ in the
// round's R register qubits, applies every gate of the round in registers and
// writes them back.  Two-target dense gates run as shared-memory steps.
// ---------------------------------------------------------------------------

// Shared-memory step of a tile pass (kept out of line so its registers do not
// weigh on the register rounds).
template <class P>
__device__ __noinline__ void tile_smem_op(typename P::S* sm, int T, uint64_t base, KOp o,
                                          const typename P::C* coef) {
    if ((base & o.cthr) == o.cthr) {
        o.cthr = o.creg;  // tile-local control mask
        small_apply<P, true>(sm, T, o, coef);
    }
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem_dst, const void* gmem_src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    if constexpr (BYTES == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gmem_src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(gmem_src), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

__device__ __forceinline__ uint64_t tile_base(uint64_t b, int L, int H, const uint8_t* tq) {
    uint64_t base = b << L;
    for (int k = 0; k < H; ++k) base = insert0(base, tq[L + k]);
    return base;
}

// Raw global elements of a tile -> shared memory, asynchronously.
template <class P, int T, int NT>
__device__ __forceinline__ void tile_prefetch(typename P::S* buf, const typename P::G* state, uint64_t base,
                                              const uint64_t* choff, int L) {
    static_assert(sizeof(typename P::G) == sizeof(typename P::S), "raw staging needs equal element sizes");
    const uint32_t lmask = (1u << L) - 1;
    const uint32_t tid = threadIdx.x;
    const uint32_t stid = sm_off<P, true>(tid);
    // k * NT and tid share no bits and the layout is additive over disjoint
    // bits: the offset is a compile-time constant plus the thread's own part
#pragma unroll
    for (int k = 0; k < (1 << T) / NT; ++k) {
        const uint32_t s = static_cast<uint32_t>(k * NT) | tid;
        cp_async<sizeof(typename P::G)>(buf + (sm_off<P, true>(static_cast<uint32_t>(k * NT)) + stid),
                                        state + (base | choff[s >> L] | (s & lmask)));
    }
    cp_async_commit();
}

// NB = tile buffers: 2 overlaps the next tile's load with this tile's rounds
// (one resident CTA per SM); 1 leaves that overlap to the other CTAs resident
// on the SM, which MINB (the launch-bounds minimum) makes room for.
template <class P, int T, int R, int NB, int MINB>
__global__ void __launch_bounds__(1 << (T - R), MINB) k_pass(typename P::G* __restrict__ state, uint64_t ntiles,
                                                        const PassDesc* __restrict__ pdp,
                                                        const StepDesc* __restrict__ steps,
                                                        const KOp* __restrict__ ops,
                                                        const typename P::C* __restrict__ coef0,
                                                        uint64_t cstride, int ishift,
                                                        const uint8_t* __restrict__ active) {
    // active (optional): items whose tiles are written back; the others keep
    // their state (classically controlled blocks of per-shot trajectories)
    // batched runs: tile b belongs to item b >> ishift, whose coefficients
    // start at coef0 + item * cstride (cstride = 0 for a single state)
    constexpr int NT = 1 << (T - R);
    constexpr int NA = 1 << R;
    constexpr int PER = (1 << T) / NT;  // elements per thread
    constexpr uint32_t TE = tile_elems(T, sizeof(typename P::S));  // elements per tile buffer
    extern __shared__ __align__(16) unsigned char smem_raw[];
    typename P::S* bufs[2] = {reinterpret_cast<typename P::S*>(smem_raw),
                              reinterpret_cast<typename P::S*>(smem_raw) + (NB - 1) * TE};
    uint64_t* choff = reinterpret_cast<uint64_t*>(smem_raw + NB * sizeof(typename P::S) * TE);

    const int tid = threadIdx.x;
    const uint32_t stid = sm_off<P, true>(static_cast<uint32_t>(tid));
    const int L = pdp->L;
    const int H = pdp->H;
    const uint8_t* tq = pdp->tq;
    for (int c = tid; c < (1 << H); c += NT) {
        uint64_t off = 0;
        for (int k = 0; k < H; ++k)
            if ((c >> k) & 1) off |= 1ULL << tq[L + k];
        choff[c] = off;
    }
    __syncthreads();
    const uint32_t lmask = (1u << L) - 1;
    const int nsteps = pdp->step_count;

    uint64_t b = blockIdx.x;
    if (NB == 2 && b < ntiles) tile_prefetch<P, T, NT>(bufs[0], state, tile_base(b, L, H, tq), choff, L);
    for (int it = 0; b < ntiles; ++it, b += gridDim.x) {
        typename P::S* sm = bufs[it & 1];
        const uint64_t base = tile_base(b, L, H, tq);
        const typename P::C* coef = coef0 + (b >> ishift) * cstride;
        if constexpr (NB == 1) {
            tile_prefetch<P, T, NT>(sm, state, base, choff, L);
            cp_async_wait<0>();
        } else {
            const uint64_t bn = b + gridDim.x;
            if (bn < ntiles) {
                tile_prefetch<P, T, NT>(bufs[(it + 1) & 1], state, tile_base(bn, L, H, tq), choff, L);
                cp_async_wait<1>();  // this tile's group is complete; the next one may be in flight
            } else {
                cp_async_wait<0>();
            }
        }
        __syncthreads();
        if constexpr (P::RAW_STAGING) {  // convert the raw FP64 tile to the register format in place
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const uint32_t ad = sm_off<P, true>(static_cast<uint32_t>(k * NT)) + stid;
                sm[ad] = P::g2s(P::raw_to_g(sm[ad]));
            }
            __syncthreads();
        }

        const StepDesc* sd = steps + pdp->step_begin;
        for (int si = 0; si < nsteps; ++si, ++sd) {
            if (sd->type == STEP_SMEM) {
                // dense multi-target gate applied in shared memory over the tile
                for (int oi = 0; oi < sd->op_count; ++oi) {
                    tile_smem_op<P>(sm, T, base, ops[sd->op_begin + oi], coef);
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
            typename P::A a[1][NA];
#pragma unroll
            for (int j = 0; j < NA; ++j) {
                uint32_t ad = psb;
#pragma unroll
                for (int k = 0; k < R; ++k)
                    if ((j >> k) & 1) ad += rsw[k];
                a[0][j] = P::s2a(sm[ad]);
            }
            const KOp* op = ops + sd->op_begin;
            const int nop = sd->op_count;
            RoundPhase<P> ph;
            ph.reset();
            for (int oi = 0; oi < nop; ++oi) {
                const KOp o = op[oi];
                reg_apply<P, R, 1>(a, o, gthr, coef, ph);
            }
            reg_finish_phase<P, R, 1>(a, ph);
            uint32_t psb2 = psb;
            asm volatile("" : "+r"(psb2));  // recompute the addresses instead of keeping 2^R of them live
#pragma unroll
            for (int j = 0; j < NA; ++j) {
                uint32_t ad = psb2;
#pragma unroll
                for (int k = 0; k < R; ++k)
                    if ((j >> k) & 1) ad += rsw[k];
                sm[ad] = P::a2s(a[0][j]);
            }
            __syncthreads();
        }

        if (active == nullptr || active[b >> ishift]) {
#pragma unroll
            for (int k = 0; k < PER; ++k) {
                const uint32_t s = static_cast<uint32_t>(k * NT) | tid;
                __stcs(state + (base | choff[s >> L] | (s & lmask)),
                       P::s2g(sm[sm_off<P, true>(static_cast<uint32_t>(k * NT)) + stid]));
            }
        }
        __syncthreads();  // the buffer is re-filled by the prefetch two tiles later
    }
}

}  // namespace qsv
