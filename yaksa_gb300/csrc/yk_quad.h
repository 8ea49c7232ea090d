/*
 * yk_quad.h -- IEEE 754 binary128 arithmetic in integer registers: the long double
 * operators (SUM, PROD, MIN, MAX; complex SUM and PROD) of hosts whose long double is
 * binary128 (aarch64 Linux), where the reference's seq backend computes `*out = *out op
 * *in` with the host compiler's soft-float (src/backend/seq/genpup.py:119-211 emits the
 * loops; the operator table is src/backend/gencomm.py:14-27).
 *
 * The method is the textbook one for a correctly rounded add and multiply (Goldberg,
 * "What every computer scientist should know about floating-point arithmetic", 1991,
 * section 1.4; Muller et al., Handbook of Floating-Point Arithmetic, chapter 7): the
 * significands carry three extra low bits (guard, round, and a sticky bit that ORs
 * every bit shifted out below it), and one rounding to nearest-even happens at the
 * end, after a result below the normal range has been shifted to the subnormal
 * exponent.  Subnormal inputs and outputs, signed zeros, infinities and overflow to
 * infinity follow IEEE 754-2008.  A NaN operand gives that NaN made quiet (the first
 * one when both are NaN); an invalid operation (inf - inf, 0 * inf) gives the positive
 * quiet NaN with a zero payload.  NaN payloads are the one place the result may
 * differ from a host's soft-float, and only in payload and sign.
 *
 * Complex multiplication is ISO C11 Annex G.5.1: the naive (ac - bd) + i(ad + bc),
 * each product and sum rounded, and the infinity recovery when both parts are NaN.
 *
 * The header is C as well as CUDA: a host test compiles it with gcc and checks every
 * function against the compiler's own _Float128 arithmetic.
 */
#ifndef YK_QUAD_H
#define YK_QUAD_H

#include <stdint.h>

#if defined(__CUDACC__)
#define YK_QFN static __host__ __device__ __forceinline__
#else
#define YK_QFN static inline
#endif

typedef unsigned __int128 yk_u128;

#define YK_Q_IMPLICIT ((yk_u128) 1 << 112)
#define YK_Q_FRAC (YK_Q_IMPLICIT - 1)
#define YK_Q_SIGN ((yk_u128) 1 << 127)
#define YK_Q_ABS (YK_Q_SIGN - 1)
#define YK_Q_INF ((yk_u128) 0x7fff << 112)
#define YK_Q_ONE ((yk_u128) 0x3fff << 112)
#define YK_Q_DNAN ((yk_u128) 0xffff << 111)     /* exponent all ones, top fraction bit */
#define YK_Q_BIAS 16383

YK_QFN int yk_q_exp(yk_u128 a) { return (int) (a >> 112) & 0x7fff; }
YK_QFN int yk_q_isnan(yk_u128 a) { return (a & YK_Q_ABS) > YK_Q_INF; }
YK_QFN int yk_q_isinf(yk_u128 a) { return (a & YK_Q_ABS) == YK_Q_INF; }
YK_QFN yk_u128 yk_q_quiet(yk_u128 a) { return a | ((yk_u128) 1 << 111); }
YK_QFN yk_u128 yk_q_copysign(yk_u128 m, yk_u128 s) { return (m & YK_Q_ABS) | (s & YK_Q_SIGN); }

/* leading zeros of a nonzero value */
YK_QFN int yk_q_clz(yk_u128 a)
{
    const uint64_t hi = (uint64_t) (a >> 64), lo = (uint64_t) a;
#if defined(__CUDA_ARCH__)
    return hi ? __clzll((long long) hi) : 64 + __clzll((long long) lo);
#else
    return hi ? __builtin_clzll(hi) : 64 + __builtin_clzll(lo);
#endif
}

/* a >> n with every bit shifted out ORed into bit 0 */
YK_QFN yk_u128 yk_q_srs(yk_u128 a, int n)
{
    if (n <= 0)
        return a;
    if (n >= 128)
        return a != 0;
    return (a >> n) | (yk_u128) ((a << (128 - n)) != 0);
}

/* The value m * 2^(e - bias - 115), rounded to nearest-even.  m carries three extra low
 * bits; either m is in [2^115, 2^116), or e == 1 and m < 2^115 (a subnormal result),
 * or e <= 0 (below the normal range: shifted to e == 1 first, with sticky). */
YK_QFN yk_u128 yk_q_round_pack(int s, int e, yk_u128 m)
{
    const yk_u128 sign = (yk_u128) s << 127;
    if (e <= 0) {
        m = yk_q_srs(m, 1 - e);
        e = 1;
    }
    const unsigned low = (unsigned) m & 7u;
    m >>= 3;
    if (low > 4u || (low == 4u && (m & 1)))
        m++;
    if (m >> 113) {             /* rounding carried out of the significand */
        m >>= 1;
        e++;
    }
    if (e >= 0x7fff)
        return sign | YK_Q_INF;
    /* m >= 2^112 adds one to the exponent field: e for a normal result, 0 -> 1 for a
     * subnormal that rounded up to the smallest normal */
    return sign | ((((yk_u128) (e - 1)) << 112) + m);
}

YK_QFN yk_u128 yk_q_add(yk_u128 a, yk_u128 b)
{
    int ea = yk_q_exp(a), eb = yk_q_exp(b);
    if (ea == 0x7fff || eb == 0x7fff) {
        if (yk_q_isnan(a))
            return yk_q_quiet(a);
        if (yk_q_isnan(b))
            return yk_q_quiet(b);
        if (ea == 0x7fff && eb == 0x7fff && ((a ^ b) >> 127))
            return YK_Q_DNAN;   /* inf - inf */
        return ea == 0x7fff ? a : b;
    }
    yk_u128 ma = a & YK_Q_ABS, mb = b & YK_Q_ABS;
    if (ma < mb) {              /* |a| >= |b| from here */
        yk_u128 t = a;
        a = b;
        b = t;
        t = ma;
        ma = mb;
        mb = t;
        int u = ea;
        ea = eb;
        eb = u;
    }
    if (mb == 0)                /* b is a zero: -0 only for -0 + -0 */
        return ma == 0 ? (a & b & YK_Q_SIGN) : a;
    const int sa = (int) (a >> 127), sb = (int) (b >> 127);
    yk_u128 fa = (a & YK_Q_FRAC) | (ea ? YK_Q_IMPLICIT : 0);
    yk_u128 fb = (b & YK_Q_FRAC) | (eb ? YK_Q_IMPLICIT : 0);
    if (!ea)
        ea = 1;
    if (!eb)
        eb = 1;
    fa <<= 3;
    fb = yk_q_srs(fb << 3, ea - eb);
    yk_u128 m;
    if (sa == sb) {
        m = fa + fb;
        if (m >> 116) {
            m = yk_q_srs(m, 1);
            ea++;
        }
    } else {
        m = fa - fb;
        if (m == 0)
            return 0;           /* exact cancellation is +0 */
        /* normalise to bit 115, but not below the subnormal exponent */
        int sh = yk_q_clz(m) - 12;
        if (sh > ea - 1)
            sh = ea - 1;
        if (sh > 0) {
            m <<= sh;
            ea -= sh;
        }
    }
    return yk_q_round_pack(sa, ea, m);
}

YK_QFN yk_u128 yk_q_sub(yk_u128 a, yk_u128 b)
{
    return yk_q_add(a, b ^ YK_Q_SIGN);
}

YK_QFN yk_u128 yk_q_mul(yk_u128 a, yk_u128 b)
{
    int ea = yk_q_exp(a), eb = yk_q_exp(b);
    const int s = (int) ((a ^ b) >> 127);
    const yk_u128 sign = (yk_u128) s << 127;
    const int za = (a & YK_Q_ABS) == 0, zb = (b & YK_Q_ABS) == 0;
    if (ea == 0x7fff || eb == 0x7fff) {
        if (yk_q_isnan(a))
            return yk_q_quiet(a);
        if (yk_q_isnan(b))
            return yk_q_quiet(b);
        if (za || zb)
            return YK_Q_DNAN;   /* 0 * inf */
        return sign | YK_Q_INF;
    }
    if (za || zb)
        return sign;
    yk_u128 fa = a & YK_Q_FRAC, fb = b & YK_Q_FRAC;
    if (ea) {
        fa |= YK_Q_IMPLICIT;
    } else {                    /* subnormal: leading bit to 112, exponent below 1 */
        const int sh = yk_q_clz(fa) - 15;
        fa <<= sh;
        ea = 1 - sh;
    }
    if (eb) {
        fb |= YK_Q_IMPLICIT;
    } else {
        const int sh = yk_q_clz(fb) - 15;
        fb <<= sh;
        eb = 1 - sh;
    }
    /* the 226-bit product fa * fb from 64-bit limbs: phi * 2^128 + plo */
    const uint64_t al = (uint64_t) fa, ah = (uint64_t) (fa >> 64);
    const uint64_t bl = (uint64_t) fb, bh = (uint64_t) (fb >> 64);
    const yk_u128 lo = (yk_u128) al * bl;
    const yk_u128 mid = (yk_u128) al * bh + (yk_u128) ah * bl;
    const yk_u128 plo = lo + (mid << 64);
    const yk_u128 phi = (yk_u128) ah * bh + (mid >> 64) + (yk_u128) (plo < lo);
    /* leading bit at 224 or 225; keep it at 115 with the rest as sticky */
    int e = ea + eb - YK_Q_BIAS, sh = 109;
    if (phi >> 97) {
        sh = 110;
        e++;
    }
    const yk_u128 m = (phi << (128 - sh)) | (plo >> sh) | (yk_u128) ((plo << (128 - sh)) != 0);
    return yk_q_round_pack(s, e, m);
}

/* a < b; false when either is a NaN, and -0 < +0 is false */
YK_QFN int yk_q_lt(yk_u128 a, yk_u128 b)
{
    if (yk_q_isnan(a) || yk_q_isnan(b))
        return 0;
    const int sa = (int) (a >> 127), sb = (int) (b >> 127);
    const yk_u128 ma = a & YK_Q_ABS, mb = b & YK_Q_ABS;
    if (sa != sb)
        return sa && (ma | mb) != 0;
    return sa ? ma > mb : ma < mb;
}

/* (a + ib) * (c + id), ISO C11 Annex G.5.1 */
YK_QFN void yk_q_cmul(yk_u128 a, yk_u128 b, yk_u128 c, yk_u128 d, yk_u128 * x, yk_u128 * y)
{
    const yk_u128 ac = yk_q_mul(a, c), bd = yk_q_mul(b, d);
    const yk_u128 ad = yk_q_mul(a, d), bc = yk_q_mul(b, c);
    *x = yk_q_sub(ac, bd);
    *y = yk_q_add(ad, bc);
    if (!(yk_q_isnan(*x) && yk_q_isnan(*y)))
        return;
    int recalc = 0;
    if (yk_q_isinf(a) || yk_q_isinf(b)) {
        a = yk_q_copysign(yk_q_isinf(a) ? YK_Q_ONE : 0, a);
        b = yk_q_copysign(yk_q_isinf(b) ? YK_Q_ONE : 0, b);
        if (yk_q_isnan(c))
            c = yk_q_copysign(0, c);
        if (yk_q_isnan(d))
            d = yk_q_copysign(0, d);
        recalc = 1;
    }
    if (yk_q_isinf(c) || yk_q_isinf(d)) {
        c = yk_q_copysign(yk_q_isinf(c) ? YK_Q_ONE : 0, c);
        d = yk_q_copysign(yk_q_isinf(d) ? YK_Q_ONE : 0, d);
        if (yk_q_isnan(a))
            a = yk_q_copysign(0, a);
        if (yk_q_isnan(b))
            b = yk_q_copysign(0, b);
        recalc = 1;
    }
    if (!recalc && (yk_q_isinf(ac) || yk_q_isinf(bd) || yk_q_isinf(ad) || yk_q_isinf(bc))) {
        if (yk_q_isnan(a))
            a = yk_q_copysign(0, a);
        if (yk_q_isnan(b))
            b = yk_q_copysign(0, b);
        if (yk_q_isnan(c))
            c = yk_q_copysign(0, c);
        if (yk_q_isnan(d))
            d = yk_q_copysign(0, d);
        recalc = 1;
    }
    if (recalc) {
        *x = yk_q_mul(YK_Q_INF, yk_q_sub(yk_q_mul(a, c), yk_q_mul(b, d)));
        *y = yk_q_mul(YK_Q_INF, yk_q_add(yk_q_mul(a, d), yk_q_mul(b, c)));
    }
}

#endif
