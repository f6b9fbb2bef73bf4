// Arithmetic policies of the statevector kernels.
//
//   P64 : complex128 storage, IEEE FP64 arithmetic
//   P32 : complex64 storage, FP32 arithmetic
//
// A policy defines the global/shared/register element types and the handful
// of real-number primitives the gate math is written in (mul, madd, add, neg),
// so one kernel template serves every precision.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qsv {

struct P64 {
    using R = double;   // real scalar in registers
    using C = double;   // coefficient
    using A = double2;  // complex amplitude in registers
    using S = double2;  // shared-memory element
    using G = double2;  // global-memory element
    static constexpr int SBYTES = 16;
    static constexpr int GBITS = 3;  // log2(elements per 128-byte wavefront)
    static constexpr bool RAW_STAGING = false;  // shared memory holds the global format
    __device__ static __forceinline__ A s2a(S s) { return s; }
    __device__ static __forceinline__ S a2s(A a) { return a; }
    __device__ static __forceinline__ S g2s(G g) { return g; }
    __device__ static __forceinline__ G s2g(S s) { return s; }
    __device__ static __forceinline__ R mul(C c, R x) { return __dmul_rn(c, x); }
    __device__ static __forceinline__ R madd(C c, R x, R acc) { return __fma_rn(c, x, acc); }
    __device__ static __forceinline__ R add(R x, R y) { return __dadd_rn(x, y); }
    __device__ static __forceinline__ R neg(R x) {
        // sign flip on the high word: no FP64 instruction
        return __hiloint2double(__double2hiint(x) ^ 0x80000000, __double2loint(x));
    }
    __device__ static __forceinline__ C cneg(C c) { return -c; }
    __device__ static __forceinline__ C coef(const C* pool, uint32_t i) { return __ldg(pool + i); }
    __device__ static __forceinline__ A one() { return make_double2(1.0, 0.0); }
    __device__ static __forceinline__ double coef_d(const C* pool, uint32_t i) { return __ldg(pool + i); }
    // four consecutive coefficients of a 4-aligned block: two 16-byte loads
    __device__ static __forceinline__ void coef4(const C* pool, uint32_t i, C (&m)[4]) {
        const double2 a = __ldg(reinterpret_cast<const double2*>(pool + i));
        const double2 b = __ldg(reinterpret_cast<const double2*>(pool + i) + 1);
        m[0] = a.x;
        m[1] = a.y;
        m[2] = b.x;
        m[3] = b.y;
    }
    __device__ static __forceinline__ double to_d_re(A a) { return a.x; }
    __device__ static __forceinline__ double to_d_im(A a) { return a.y; }
    __device__ static __forceinline__ G make_g(double re, double im) { return make_double2(re, im); }
    __device__ static __forceinline__ double gre(G g) { return g.x; }
    __device__ static __forceinline__ double gim(G g) { return g.y; }
};

struct P32 {
    using R = float;
    using C = float;
    using A = float2;
    using S = float2;
    using G = float2;
    static constexpr int SBYTES = 8;
    static constexpr int GBITS = 4;
    static constexpr bool RAW_STAGING = false;
    __device__ static __forceinline__ A s2a(S s) { return s; }
    __device__ static __forceinline__ S a2s(A a) { return a; }
    __device__ static __forceinline__ S g2s(G g) { return g; }
    __device__ static __forceinline__ G s2g(S s) { return s; }
    __device__ static __forceinline__ R mul(C c, R x) { return __fmul_rn(c, x); }
    __device__ static __forceinline__ R madd(C c, R x, R acc) { return __fmaf_rn(c, x, acc); }
    __device__ static __forceinline__ R add(R x, R y) { return __fadd_rn(x, y); }
    __device__ static __forceinline__ R neg(R x) { return __int_as_float(__float_as_int(x) ^ 0x80000000); }
    __device__ static __forceinline__ C cneg(C c) { return -c; }
    // four consecutive coefficients of a 4-aligned block: one 16-byte load
    __device__ static __forceinline__ void coef4(const C* pool, uint32_t i, C (&m)[4]) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(pool + i));
        m[0] = v.x;
        m[1] = v.y;
        m[2] = v.z;
        m[3] = v.w;
    }
    __device__ static __forceinline__ C coef(const C* pool, uint32_t i) { return __ldg(pool + i); }
    __device__ static __forceinline__ A one() { return make_float2(1.f, 0.f); }
    __device__ static __forceinline__ double coef_d(const C* pool, uint32_t i) {
        return static_cast<double>(__ldg(pool + i));
    }
    __device__ static __forceinline__ G make_g(double re, double im) {
        return make_float2(static_cast<float>(re), static_cast<float>(im));
    }
    __device__ static __forceinline__ double gre(G g) { return static_cast<double>(g.x); }
    __device__ static __forceinline__ double gim(G g) { return static_cast<double>(g.y); }
};

// ------------------------------------------------------------------------
// PDS : complex128 storage, double-single arithmetic.  Each real is carried
// as an unevaluated sum h + l of two floats (about 48 significand bits) and
// combined with error-free transformations (TwoSum, FMA-based TwoProd)
// on the FP32 pipes, which on this GPU issue ~57x faster than FP64.
// Conversions to and from FP64 happen once per pass, at the shared-memory
// staging of a tile.
// ------------------------------------------------------------------------
struct ds {
    float h, l;
};
struct ds2 {
    ds x, y;
};

// FP64 -> float pair with integer and FP32 instructions only (the FP64 pipe
// of GB300 issues about 2 instructions per clock per SM).  The high float is
// v truncated to 24 significant bits (v's own exponent and top mantissa
// bits, re-biased), the low float the next 23 mantissa bits, exactly.
// |v| < 2^-103 becomes (0, 0); |v| must stay below 2^127.
__device__ __forceinline__ ds ds_from_double(double v) {
    const uint32_t hw = static_cast<uint32_t>(__double2hiint(v));
    const uint32_t lw = static_cast<uint32_t>(__double2loint(v));
    const uint32_t sg = hw & 0x80000000u;
    const bool tiny = (hw & 0x7FFFFFFFu) < 0x39800000u;  // exponent field < 920
    const uint32_t f = __funnelshift_l(lw, hw, 3);       // exponent low 8 bits | 23 mantissa bits
    const uint32_t hb = ((f ^ 0x40000000u) & 0x7FFFFFFFu) | sg;  // FP32 exponent = FP64 exponent - 896
    const uint32_t e = ((f & 0x7F800000u) + 0x34800000u) & 0x7F800000u;  // FP64 exponent - 919
    const float lo = __fsub_rn(__uint_as_float(e | ((lw >> 6) & 0x7FFFFFu)), __uint_as_float(e));
    const uint32_t lb = __float_as_uint(lo) | sg;
    return {__uint_as_float(tiny ? sg : hb), __uint_as_float(tiny ? sg : lb)};
}
// Float pair -> FP64, again without FP64 instructions: both significands
// are aligned in a 64-bit integer (h's at bits 62..39), added or subtracted,
// normalised with a leading-zero count and truncated to 53 bits.  Needs
// |l| <= |h| (every float pair the arithmetic below produces is normalised);
// h zero or below the FP32 normal range gives zero.
__device__ __forceinline__ double ds_to_double(ds a) {
    const uint32_t H = __float_as_uint(a.h), Lb = __float_as_uint(a.l);
    const uint32_t sh = H & 0x80000000u;
    const uint32_t eh = (H >> 23) & 0xFFu, el = (Lb >> 23) & 0xFFu;
    const uint64_t mh = static_cast<uint64_t>((H & 0x7FFFFFu) | 0x800000u) << 39;
    const uint64_t ml = static_cast<uint64_t>((Lb & 0x7FFFFFu) | 0x800000u) << 39;
    const uint32_t d = el == 0 ? 64u : eh - el;
    const uint64_t mls = d < 64u ? (ml >> d) : 0ull;
    const uint64_t m = (static_cast<int32_t>(H ^ Lb) < 0) ? mh - mls : mh + mls;
    const int z = __clzll(static_cast<long long>(m));
    const uint64_t mant = z < 64 ? ((m << z) >> 11) : 0ull;
    const uint32_t hw = (((eh - static_cast<uint32_t>(z) + 896u) << 20) + static_cast<uint32_t>(mant >> 32)) | sh;
    const bool zero = eh == 0 || z == 64;
    return __hiloint2double(static_cast<int>(zero ? sh : hw), static_cast<int>(zero ? 0u : static_cast<uint32_t>(mant)));
}
// a + b with TwoSum on the high parts
__device__ __forceinline__ ds ds_add(ds a, ds b) {
    const float s = __fadd_rn(a.h, b.h);
    const float v = __fsub_rn(s, a.h);
    float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(b.h, v));
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
// c * x, unnormalised (p + e) via FMA TwoProd plus the cross terms
__device__ __forceinline__ ds ds_mul_raw(ds c, ds x) {
    const float p = __fmul_rn(c.h, x.h);
    float e = __fmaf_rn(c.h, x.h, -p);
    e = __fmaf_rn(c.h, x.l, e);
    e = __fmaf_rn(c.l, x.h, e);
    return {p, e};
}

struct PDS {
    using R = ds;
    using C = ds;
    using A = ds2;
    using S = float4;   // (re.h, re.l, im.h, im.l)
    using G = double2;
    static constexpr int SBYTES = 16;
    static constexpr int GBITS = 3;
    // tiles arrive in shared memory as raw FP64 and are converted in place
    static constexpr bool RAW_STAGING = true;
    __device__ static __forceinline__ G raw_to_g(S s) {
        return make_double2(__hiloint2double(__float_as_int(s.y), __float_as_int(s.x)),
                            __hiloint2double(__float_as_int(s.w), __float_as_int(s.z)));
    }
    __device__ static __forceinline__ A s2a(S s) { return {{s.x, s.y}, {s.z, s.w}}; }
    __device__ static __forceinline__ S a2s(A a) { return make_float4(a.x.h, a.x.l, a.y.h, a.y.l); }
    __device__ static __forceinline__ S g2s(G g) {
        const ds r = ds_from_double(g.x), i = ds_from_double(g.y);
        return make_float4(r.h, r.l, i.h, i.l);
    }
    __device__ static __forceinline__ G s2g(S s) {
        return make_double2(ds_to_double({s.x, s.y}), ds_to_double({s.z, s.w}));
    }
    __device__ static __forceinline__ R mul(C c, R x) {
        const ds p = ds_mul_raw(c, x);
        const float h = __fadd_rn(p.h, p.l);
        return {h, __fsub_rn(p.l, __fsub_rn(h, p.h))};
    }
    __device__ static __forceinline__ R madd(C c, R x, R acc) { return ds_add(acc, ds_mul_raw(c, x)); }
    __device__ static __forceinline__ R add(R x, R y) { return ds_add(x, y); }
    __device__ static __forceinline__ R neg(R x) { return {-x.h, -x.l}; }
    __device__ static __forceinline__ C cneg(C c) { return {-c.h, -c.l}; }
    __device__ static __forceinline__ A one() { return {{1.f, 0.f}, {0.f, 0.f}}; }
    __device__ static __forceinline__ double coef_d(const C* pool, uint32_t i) { return ds_to_double(coef(pool, i)); }
    __device__ static __forceinline__ C coef(const C* pool, uint32_t i) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(pool) + i);
        return {v.x, v.y};
    }
    // four consecutive coefficients of a 4-aligned block: two 16-byte loads
    __device__ static __forceinline__ void coef4(const C* pool, uint32_t i, C (&m)[4]) {
        const float4 a = __ldg(reinterpret_cast<const float4*>(pool + i));
        const float4 b = __ldg(reinterpret_cast<const float4*>(pool + i) + 1);
        m[0] = {a.x, a.y};
        m[1] = {a.z, a.w};
        m[2] = {b.x, b.y};
        m[3] = {b.z, b.w};
    }
};

// ------------------------------------------------------------------------
// Gate math on amplitude pairs, written once over the policy primitives.
// ------------------------------------------------------------------------

// [[m0, m1], [m2, m3]] real
template <class P>
__device__ __forceinline__ void pair_real(typename P::A& a, typename P::A& b, typename P::C m0, typename P::C m1,
                                          typename P::C m2, typename P::C m3) {
    typename P::A na, nb;
    na.x = P::madd(m1, b.x, P::mul(m0, a.x));
    na.y = P::madd(m1, b.y, P::mul(m0, a.y));
    nb.x = P::madd(m3, b.x, P::mul(m2, a.x));
    nb.y = P::madd(m3, b.y, P::mul(m2, a.y));
    a = na;
    b = nb;
}

// [[c, -i s], [-i s, c]]; ns = -s
template <class P>
__device__ __forceinline__ void pair_rx(typename P::A& a, typename P::A& b, typename P::C c, typename P::C s,
                                        typename P::C ns) {
    typename P::A na, nb;
    na.x = P::madd(s, b.y, P::mul(c, a.x));
    na.y = P::madd(ns, b.x, P::mul(c, a.y));
    nb.x = P::madd(s, a.y, P::mul(c, b.x));
    nb.y = P::madd(ns, a.x, P::mul(c, b.y));
    a = na;
    b = nb;
}

// general 2x2 complex; m[8] = m00 re, im, m01 re, im, m10 re, im, m11 re, im;
// nm[k] = -m[k] for the imaginary parts
template <class P>
__device__ __forceinline__ void pair_dense(typename P::A& a, typename P::A& b, const typename P::C* m,
                                           const typename P::C* nmi) {
    typename P::A na, nb;
    na.x = P::madd(nmi[1], b.y, P::madd(m[2], b.x, P::madd(nmi[0], a.y, P::mul(m[0], a.x))));
    na.y = P::madd(m[3], b.x, P::madd(m[2], b.y, P::madd(m[1], a.x, P::mul(m[0], a.y))));
    nb.x = P::madd(nmi[3], b.y, P::madd(m[6], b.x, P::madd(nmi[2], a.y, P::mul(m[4], a.x))));
    nb.y = P::madd(m[7], b.x, P::madd(m[6], b.y, P::madd(m[5], a.x, P::mul(m[4], a.y))));
    a = na;
    b = nb;
}

// a *= (dr + i di); ndi = -di
template <class P>
__device__ __forceinline__ void amp_phase(typename P::A& a, typename P::C dr, typename P::C di, typename P::C ndi) {
    typename P::A na;
    na.x = P::madd(ndi, a.y, P::mul(dr, a.x));
    na.y = P::madd(di, a.x, P::mul(dr, a.y));
    a = na;
}

template <class P>
__device__ __forceinline__ void amp_special(typename P::A& a, int sp) {
    typename P::A na;
    if (sp == 1) {  // * -1
        na.x = P::neg(a.x);
        na.y = P::neg(a.y);
    } else if (sp == 2) {  // * i
        na.x = P::neg(a.y);
        na.y = a.x;
    } else {  // * -i
        na.x = a.y;
        na.y = P::neg(a.x);
    }
    a = na;
}

// sqrt(2) H = [[1, 1], [1, -1]]: additions only
template <class P>
__device__ __forceinline__ void pair_had(typename P::A& a, typename P::A& b) {
    typename P::A na, nb;
    na.x = P::add(a.x, b.x);
    na.y = P::add(a.y, b.y);
    nb.x = P::add(a.x, P::neg(b.x));
    nb.y = P::add(a.y, P::neg(b.y));
    a = na;
    b = nb;
}

// Y = [[0, -i], [i, 0]]
template <class P>
__device__ __forceinline__ void pair_y(typename P::A& a, typename P::A& b) {
    typename P::A na, nb;
    na.x = b.y;
    na.y = P::neg(b.x);
    nb.x = P::neg(a.y);
    nb.y = a.x;
    a = na;
    b = nb;
}

// 4x4 complex on (v0, v1, v2, v3) = amplitudes with (t1 t0) = 00, 01, 10, 11
template <class P>
__device__ __forceinline__ void quad_dense(typename P::A& v0, typename P::A& v1, typename P::A& v2,
                                           typename P::A& v3, const typename P::C* pool, uint32_t off) {
    typename P::A in[4] = {v0, v1, v2, v3};
    typename P::A out[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        typename P::R xr = P::mul(P::coef(pool, off + 8 * r), in[0].x);
        typename P::R xi = P::mul(P::coef(pool, off + 8 * r), in[0].y);
        xr = P::madd(P::cneg(P::coef(pool, off + 8 * r + 1)), in[0].y, xr);
        xi = P::madd(P::coef(pool, off + 8 * r + 1), in[0].x, xi);
#pragma unroll
        for (int c = 1; c < 4; ++c) {
            const typename P::C mr = P::coef(pool, off + 8 * r + 2 * c);
            const typename P::C mi = P::coef(pool, off + 8 * r + 2 * c + 1);
            xr = P::madd(mr, in[c].x, xr);
            xr = P::madd(P::cneg(mi), in[c].y, xr);
            xi = P::madd(mr, in[c].y, xi);
            xi = P::madd(mi, in[c].x, xi);
        }
        out[r].x = xr;
        out[r].y = xi;
    }
    v0 = out[0];
    v1 = out[1];
    v2 = out[2];
    v3 = out[3];
}

}  // namespace qsv
