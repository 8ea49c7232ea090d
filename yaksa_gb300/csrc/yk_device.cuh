/*
 * yk_device.cuh -- device code shared by the launch kernels (yk_kernels.cu) and the
 * persistent request server (yk_server.cu): unit types and loads, the regular-nest
 * tile, the elementwise operators, and the per-range bodies of the kernels whose
 * server items run the same code.
 */
#pragma once
#include <atomic>
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>
#include "yk_desc.h"
#include "yk_locate.h"
#include "yk_quad.h"

#define YK_THREADS 256
#define YK_UNROLL 4

extern "C" int yk_cuda_num_sms(void);
extern "C" void yk_tma_count_launch(void);

/* address decomposition shared with the host (yk_locate.h) */
/* ------------------------------------------------------------------------- */

__device__ __forceinline__ uint32_t yk_div(uint32_t n, const yk_level & l) { return yk_div32(n, &l); }
__device__ __forceinline__ uint64_t yk_div(uint64_t n, const yk_level & l) { return yk_div64(n, &l); }

template <typename IDX>
__device__ __forceinline__ int64_t yk_locate(const yk_desc & d, IDX p, int *bt, uint64_t * inseg);
template <>
__device__ __forceinline__ int64_t yk_locate<uint32_t>(const yk_desc & d, uint32_t p, int *bt,
                                                       uint64_t * inseg)
{
    return yk_locate32(&d, p, bt, inseg);
}
template <>
__device__ __forceinline__ int64_t yk_locate<uint64_t>(const yk_desc & d, uint64_t p, int *bt,
                                                       uint64_t * inseg)
{
    return yk_locate64(&d, p, bt, inseg);
}

/* ------------------------------------------------------------------------- */
/* REPLACE: byte movement in V-byte units                                    */
/* ------------------------------------------------------------------------- */

template <int V> struct yk_vec;
template <> struct yk_vec<1> { typedef uint8_t T; };
template <> struct yk_vec<2> { typedef uint16_t T; };
template <> struct yk_vec<4> { typedef uint32_t T; };
template <> struct yk_vec<8> { typedef uint2 T; };
template <> struct yk_vec<16> { typedef uint4 T; };

/* Loads cached in L2 only: the strided side is read once, so it does not displace L1.
 * (An isolated 8-byte run still costs a whole 128-byte line from L2 on GB300, whatever
 * the cache operator or prefetch-size qualifier; measured for every documented form.) */
__device__ __forceinline__ uint8_t yk_ldcg(const uint8_t * p)
{
    uint16_t v;
    asm volatile ("ld.global.cg.u8 %0, [%1];" : "=h"(v) : "l"(p));
    return (uint8_t) v;
}

__device__ __forceinline__ uint16_t yk_ldcg(const uint16_t * p)
{
    uint16_t v;
    asm volatile ("ld.global.cg.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t yk_ldcg(const uint32_t * p)
{
    uint32_t v;
    asm volatile ("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint2 yk_ldcg(const uint2 * p)
{
    uint2 v;
    asm volatile ("ld.global.cg.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ uint4 yk_ldcg(const uint4 * p)
{
    uint4 v;
    asm volatile ("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                  : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}

/* One tile: units t0 + k * YK_THREADS + threadIdx.x, k < U, of a request with
 * `nunits` V-byte units.  All U addresses are computed first and all U loads issued
 * before any store, so every thread keeps U independent memory requests in flight.
 * Loads use ld.global.cg (cache in L2 only): an L1-allocating load of an isolated
 * 8-byte run fills a 128-byte line, which is 16x the useful DRAM traffic for runs
 * at a large stride. */
template <typename IDX, int V, int DIR, int U>
__device__ __forceinline__ void yk_bytes_tile(const yk_launch & L, IDX t0, IDX nunits)
{
    typedef typename yk_vec<V>::T VT;
    const IDX p0 = (IDX) L.p0;
    VT *packed = (VT *) L.packed;
    char *typed = L.typed;
    int64_t off[U];
    VT v[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
        IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
        if (u < nunits)
            off[k] = yk_locate<IDX>(L.desc, p0 + u * (IDX) V, nullptr, nullptr);
    }
    if (DIR == 0) {
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                v[k] = yk_ldcg((const VT *) (typed + off[k]));
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                packed[u] = v[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                v[k] = yk_ldcg((const VT *) (packed + u));
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                *(VT *) (typed + off[k]) = v[k];
        }
    }
}

/* Regular nests (NL strided levels over one contiguous run, 32-bit positions): the
 * decomposition unrolls at compile time into NL multiply-high/shift/multiply-add steps
 * with no table loads, which keeps the kernel near 32 registers and lets eight
 * 256-thread CTAs share an SM (full occupancy, the most loads in flight). */
/* the few fields of a regular request a tile needs, held in registers */
struct yk_rt {
    char *typed;                /* typed pointer + descriptor base */
    char *packed;
    uint32_t p0;
    uint32_t m[YK_REGULAR_MAX];
    uint32_t cps[YK_REGULAR_MAX];
    uint32_t sh1[YK_REGULAR_MAX], sh2[YK_REGULAR_MAX];
    int64_t stride[YK_REGULAR_MAX];
};

template <int NL>
__device__ __forceinline__ void yk_rt_load(yk_rt & t, const yk_launch & L)
{
    t.typed = L.typed + L.desc.base;
    t.packed = L.packed;
    t.p0 = (uint32_t) L.p0;
#pragma unroll
    for (int i = 0; i < NL; i++) {
        t.m[i] = L.desc.lv[i].m32;
        t.cps[i] = (uint32_t) L.desc.lv[i].cps;
        t.sh1[i] = L.desc.lv[i].l ? 1u : 0u;
        t.sh2[i] = L.desc.lv[i].l ? (uint32_t) L.desc.lv[i].l - 1u : 0u;
        t.stride[i] = L.desc.lv[i].stride;
    }
}

template <int V, int DIR, int U, int NL>
__device__ __forceinline__ void yk_regular_tile(const yk_launch & L, uint32_t t0, uint32_t nunits)
{
    typedef typename yk_vec<V>::T VT;
    yk_rt rt;
    yk_rt_load<NL>(rt, L);
    VT *packed = (VT *) rt.packed;
    char *typed = rt.typed;
    int64_t off[U];
    VT v[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
        uint32_t u = t0 + (uint32_t) (k * YK_THREADS + threadIdx.x);
        uint32_t r = rt.p0 + u * (uint32_t) V;
        int64_t o = 0;
#pragma unroll
        for (int i = 0; i < NL; i++) {
            uint32_t t = __umulhi(rt.m[i], r);
            uint32_t q = (t + ((r - t) >> rt.sh1[i])) >> rt.sh2[i];
            r -= q * rt.cps[i];
            o += (int64_t) q * rt.stride[i];
        }
        off[k] = o + (int64_t) r;
    }
    if (DIR == 0) {
#pragma unroll
        for (int k = 0; k < U; k++)
            if (t0 + (uint32_t) (k * YK_THREADS + threadIdx.x) < nunits)
                v[k] = yk_ldcg((const VT *) (typed + off[k]));
#pragma unroll
        for (int k = 0; k < U; k++) {
            uint32_t u = t0 + (uint32_t) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                packed[u] = v[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < U; k++) {
            uint32_t u = t0 + (uint32_t) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                v[k] = yk_ldcg((const VT *) (packed + u));
        }
#pragma unroll
        for (int k = 0; k < U; k++)
            if (t0 + (uint32_t) (k * YK_THREADS + threadIdx.x) < nunits)
                *(VT *) (typed + off[k]) = v[k];
    }
}

template <int V, int DIR, int U>
__device__ __forceinline__ void yk_regular_dispatch(const yk_launch & L, uint32_t t0,
                                                    uint32_t nunits)
{
    switch (L.regular) {
        case 0: yk_regular_tile<V, DIR, U, 0>(L, t0, nunits); break;
        case 1: yk_regular_tile<V, DIR, U, 1>(L, t0, nunits); break;
        case 2: yk_regular_tile<V, DIR, U, 2>(L, t0, nunits); break;
        default: yk_regular_tile<V, DIR, U, 3>(L, t0, nunits); break;
    }
}

/* ------------------------------------------------------------------------- */
/* elementwise operators                                                     */
/* ------------------------------------------------------------------------- */

enum { OP_MAX = 0, OP_MIN = 1, OP_SUM = 2, OP_PROD = 3, OP_LAND = 4, OP_BAND = 5, OP_LOR = 6,
    OP_BOR = 7, OP_LXOR = 8, OP_BXOR = 9, OP_REPLACE = 10 };

template <typename T> __device__ __forceinline__ T yk_ld(const char *p)
{
    if (((uintptr_t) p & (sizeof(T) - 1)) == 0)
        return *(const T *) p;
    T v;
    char *q = (char *) &v;
#pragma unroll
    for (int i = 0; i < (int) sizeof(T); i++)
        q[i] = p[i];
    return v;
}

template <typename T> __device__ __forceinline__ void yk_st(char *p, T v)
{
    if (((uintptr_t) p & (sizeof(T) - 1)) == 0) {
        *(T *) p = v;
        return;
    }
    const char *q = (const char *) &v;
#pragma unroll
    for (int i = 0; i < (int) sizeof(T); i++)
        p[i] = q[i];
}

/* integer operators; returns false when op is outside the type's table */
template <typename S, typename U>
__device__ __forceinline__ bool yk_int_op(int op, S in, S & out)
{
    switch (op) {
        case OP_REPLACE:
            out = in;
            return true;
        case OP_MAX:
            out = (in < out) ? out : in;
            return true;
        case OP_MIN:
            out = (in < out) ? in : out;
            return true;
        case OP_SUM:
            out = (S) (U) ((U) out + (U) in);
            return true;
        case OP_PROD:
            out = (S) (U) ((U) out * (U) in);
            return true;
        case OP_LAND:
            out = (S) (out && in);
            return true;
        case OP_LOR:
            out = (S) (out || in);
            return true;
        case OP_LXOR:
            out = (S) (!out != !in);
            return true;
        case OP_BAND:
            out = (S) (out & in);
            return true;
        case OP_BOR:
            out = (S) (out | in);
            return true;
        case OP_BXOR:
            out = (S) (out ^ in);
            return true;
    }
    return false;
}

__device__ __forceinline__ float yk_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double yk_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float yk_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double yk_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float yk_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double yk_mul(double a, double b) { return __dmul_rn(a, b); }

template <typename F>
__device__ __forceinline__ bool yk_flt_op(int op, F in, F & out)
{
    switch (op) {
        case OP_REPLACE:
            out = in;
            return true;
        case OP_MAX:
            out = (in < out) ? out : in;
            return true;
        case OP_MIN:
            out = (in > out) ? out : in;
            return true;
        case OP_SUM:
            out = yk_add(out, in);
            return true;
        case OP_PROD:
            out = yk_mul(out, in);
            return true;
    }
    return false;
}

/* (a + ib) * (c + id) with the infinity recovery of ISO C11 Annex G.5.1 */
template <typename F>
__device__ __forceinline__ void yk_cmul(F a, F b, F c, F d, F & x, F & y)
{
    F ac = yk_mul(a, c), bd = yk_mul(b, d), ad = yk_mul(a, d), bc = yk_mul(b, c);
    x = yk_sub(ac, bd);
    y = yk_add(ad, bc);
    if (isnan(x) && isnan(y)) {
        bool recalc = false;
        const F one = (F) 1, zero = (F) 0;
        if (isinf(a) || isinf(b)) {
            a = copysign(isinf(a) ? one : zero, a);
            b = copysign(isinf(b) ? one : zero, b);
            if (isnan(c))
                c = copysign(zero, c);
            if (isnan(d))
                d = copysign(zero, d);
            recalc = true;
        }
        if (isinf(c) || isinf(d)) {
            c = copysign(isinf(c) ? one : zero, c);
            d = copysign(isinf(d) ? one : zero, d);
            if (isnan(a))
                a = copysign(zero, a);
            if (isnan(b))
                b = copysign(zero, b);
            recalc = true;
        }
        if (!recalc && (isinf(ac) || isinf(bd) || isinf(ad) || isinf(bc))) {
            if (isnan(a))
                a = copysign(zero, a);
            if (isnan(b))
                b = copysign(zero, b);
            if (isnan(c))
                c = copysign(zero, c);
            if (isnan(d))
                d = copysign(zero, d);
            recalc = true;
        }
        if (recalc) {
            const F inf = (F) INFINITY;
            x = yk_mul(inf, yk_sub(yk_mul(a, c), yk_mul(b, d)));
            y = yk_mul(inf, yk_add(yk_mul(a, d), yk_mul(b, c)));
        }
    }
}

template <typename F>
__device__ __forceinline__ bool yk_cplx_op(int op, const F in[2], F out[2])
{
    switch (op) {
        case OP_REPLACE:
            out[0] = in[0];
            out[1] = in[1];
            return true;
        case OP_SUM:
            out[0] = yk_add(out[0], in[0]);
            out[1] = yk_add(out[1], in[1]);
            return true;
        case OP_PROD:{
                F x, y;
                yk_cmul(out[0], out[1], in[0], in[1], x, y);
                out[0] = x;
                out[1] = y;
                return true;
            }
    }
    return false;
}

__device__ __forceinline__ yk_u128 yk_ldq(const char *p)
{
    return ((yk_u128) yk_ld<uint64_t>(p + 8) << 64) | (yk_u128) yk_ld<uint64_t>(p);
}

__device__ __forceinline__ void yk_stq(char *p, yk_u128 v)
{
    yk_st<uint64_t>(p, (uint64_t) v);
    yk_st<uint64_t>(p + 8, (uint64_t) (v >> 64));
}

/* long double and long double complex in binary128: `out = out op in` as the
 * reference's seq loops compute it (MAX and MIN are the selects of the float types) */
__device__ __forceinline__ void yk_q_apply(int bt, int op, char *dst, const char *src)
{
    if (bt == YK_BT_LDOUBLE) {
        const yk_u128 in = yk_ldq(src), out = yk_ldq(dst);
        yk_u128 r;
        switch (op) {
            case OP_REPLACE: r = in; break;
            case OP_MAX: r = yk_q_lt(in, out) ? out : in; break;
            case OP_MIN: r = yk_q_lt(out, in) ? out : in; break;
            case OP_SUM: r = yk_q_add(out, in); break;
            case OP_PROD: r = yk_q_mul(out, in); break;
            default: return;
        }
        yk_stq(dst, r);
        return;
    }
    const yk_u128 ir = yk_ldq(src), ii = yk_ldq(src + 16);
    yk_u128 orr = yk_ldq(dst), oi = yk_ldq(dst + 16);
    switch (op) {
        case OP_REPLACE:
            orr = ir;
            oi = ii;
            break;
        case OP_SUM:
            orr = yk_q_add(orr, ir);
            oi = yk_q_add(oi, ii);
            break;
        case OP_PROD:
            yk_q_cmul(orr, oi, ir, ii, &orr, &oi);
            break;
        default:
            return;
    }
    yk_stq(dst, orr);
    yk_stq(dst + 16, oi);
}

/* apply op to one element of base type bt; `dst` is updated in place from `src`.
 * LD: the instance for types that hold long double, with the binary128 operators;
 * the other instance moves long double bytes for REPLACE only (the host sends every
 * long double operator to the LD instances), which keeps the 128-bit arithmetic out
 * of the register budget of the common kernels. */
template <bool LD>
__device__ __forceinline__ void yk_apply(int bt, int op, char *dst, const char *src)
{
    switch (bt) {
        case YK_BT_BOOL:{
                if (op != OP_REPLACE && op != OP_LAND && op != OP_LOR && op != OP_LXOR)
                    return;
                uint8_t i = yk_ld<uint8_t>(src), o = yk_ld<uint8_t>(dst);
                uint8_t r = op == OP_REPLACE ? i : op == OP_LAND ? (uint8_t) (o && i) :
                    op == OP_LOR ? (uint8_t) (o || i) : (uint8_t) (!o != !i);
                yk_st<uint8_t>(dst, r);
                return;
            }
        case YK_BT_I8:{
                int8_t i = yk_ld<int8_t>(src), o = yk_ld<int8_t>(dst);
                if (yk_int_op<int8_t, uint8_t>(op, i, o))
                    yk_st<int8_t>(dst, o);
                return;
            }
        case YK_BT_I16:{
                int16_t i = yk_ld<int16_t>(src), o = yk_ld<int16_t>(dst);
                if (yk_int_op<int16_t, uint16_t>(op, i, o))
                    yk_st<int16_t>(dst, o);
                return;
            }
        case YK_BT_I32:{
                int32_t i = yk_ld<int32_t>(src), o = yk_ld<int32_t>(dst);
                if (yk_int_op<int32_t, uint32_t>(op, i, o))
                    yk_st<int32_t>(dst, o);
                return;
            }
        case YK_BT_I64:{
                int64_t i = yk_ld<int64_t>(src), o = yk_ld<int64_t>(dst);
                if (yk_int_op<int64_t, uint64_t>(op, i, o))
                    yk_st<int64_t>(dst, o);
                return;
            }
        case YK_BT_F32:{
                float i = yk_ld<float>(src), o = yk_ld<float>(dst);
                if (yk_flt_op<float>(op, i, o))
                    yk_st<float>(dst, o);
                return;
            }
        case YK_BT_F64:{
                double i = yk_ld<double>(src), o = yk_ld<double>(dst);
                if (yk_flt_op<double>(op, i, o))
                    yk_st<double>(dst, o);
                return;
            }
        case YK_BT_C32:{
                float i[2] = { yk_ld<float>(src), yk_ld<float>(src + 4) };
                float o[2] = { yk_ld<float>(dst), yk_ld<float>(dst + 4) };
                if (yk_cplx_op<float>(op, i, o)) {
                    yk_st<float>(dst, o[0]);
                    yk_st<float>(dst + 4, o[1]);
                }
                return;
            }
        case YK_BT_C64:{
                double i[2] = { yk_ld<double>(src), yk_ld<double>(src + 8) };
                double o[2] = { yk_ld<double>(dst), yk_ld<double>(dst + 8) };
                if (yk_cplx_op<double>(op, i, o)) {
                    yk_st<double>(dst, o[0]);
                    yk_st<double>(dst + 8, o[1]);
                }
                return;
            }
        case YK_BT_LDOUBLE: case YK_BT_CLDOUBLE:
            if (LD) {
                yk_q_apply(bt, op, dst, src);
            } else if (op == OP_REPLACE) {
                yk_stq(dst, yk_ldq(src));
                if (bt == YK_BT_CLDOUBLE)
                    yk_stq(dst + 16, yk_ldq(src + 16));
            }
            return;
        default:
            /* CHAR/WCHAR only have REPLACE, which never reaches the typed kernel */
            return;
    }
}

__host__ __device__ __forceinline__ int yk_bt_size(int bt)
{
    switch (bt) {
        case YK_BT_BOOL: case YK_BT_CHAR: case YK_BT_I8: return 1;
        case YK_BT_I16: return 2;
        case YK_BT_WCHAR: case YK_BT_I32: case YK_BT_F32: return 4;
        case YK_BT_I64: case YK_BT_F64: case YK_BT_C32: return 8;
        case YK_BT_C64: case YK_BT_LDOUBLE: return 16;
        case YK_BT_CLDOUBLE: return 32;
        default: return 1;
    }
}

/* element types in registers, for the typed kernels (ordered unpacks, L2 reductions) */
template <int BT> struct yk_elem;
template <> struct yk_elem<YK_BT_I8> {
    typedef int8_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int8_t, uint8_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_I16> {
    typedef int16_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int16_t, uint16_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_I32> {
    typedef int32_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int32_t, uint32_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_I64> {
    typedef int64_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int64_t, uint64_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_F32> {
    typedef float T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_flt_op<float>(o, in, out); }
};
template <> struct yk_elem<YK_BT_F64> {
    typedef double T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_flt_op<double>(o, in, out); }
};
template <> struct yk_elem<YK_BT_C32> {
    typedef float2 T;
    static __device__ __forceinline__ bool op(int o, T in, T & out)
    {
        float a[2] = { in.x, in.y }, b[2] = { out.x, out.y };
        bool r = yk_cplx_op<float>(o, a, b);
        out = make_float2(b[0], b[1]);
        return r;
    }
};
template <> struct yk_elem<YK_BT_C64> {
    typedef double2 T;
    static __device__ __forceinline__ bool op(int o, T in, T & out)
    {
        double a[2] = { in.x, in.y }, b[2] = { out.x, out.y };
        bool r = yk_cplx_op<double>(o, a, b);
        out = make_double2(b[0], b[1]);
        return r;
    }
};


/* Reductions at L2 for the integer operators whose result does not depend on the order
 * in which contributions arrive: SUM (addition modulo 2^n), MAX, MIN (signed, as the
 * reference's unsigned handles alias the signed types), BAND, BOR and BXOR, on 4- and
 * 8-byte integers.  The value is sent to the L2 with a reduction (red.global.*, the
 * form an atomic whose result is unused compiles to), which reads, combines and writes
 * the target element there. */
template <int OP, typename T> __device__ __forceinline__ void yk_red(T *p, T v);
template <int OP> __device__ __forceinline__ void yk_red(int32_t *p, int32_t v)
{
    unsigned int *q = (unsigned int *) p;
    if constexpr (OP == OP_SUM) atomicAdd(q, (unsigned int) v);
    else if constexpr (OP == OP_MAX) atomicMax((int *) p, (int) v);
    else if constexpr (OP == OP_MIN) atomicMin((int *) p, (int) v);
    else if constexpr (OP == OP_BAND) atomicAnd(q, (unsigned int) v);
    else if constexpr (OP == OP_BOR) atomicOr(q, (unsigned int) v);
    else atomicXor(q, (unsigned int) v);
}
template <int OP> __device__ __forceinline__ void yk_red(int64_t *p, int64_t v)
{
    unsigned long long *q = (unsigned long long *) p;
    if constexpr (OP == OP_SUM) atomicAdd(q, (unsigned long long) v);
    else if constexpr (OP == OP_MAX) atomicMax((long long *) p, (long long) v);
    else if constexpr (OP == OP_MIN) atomicMin((long long *) p, (long long) v);
    else if constexpr (OP == OP_BAND) atomicAnd(q, (unsigned long long) v);
    else if constexpr (OP == OP_BOR) atomicOr(q, (unsigned long long) v);
    else atomicXor(q, (unsigned long long) v);
}

/* The contiguous-block hindexed walk (yk_hidx_kernel) for ranges of up to YK_POS32_END
 * bytes: the groups of 32 blocks that meet the packed range [p0, p1) (a launch's whole
 * request, or one server item), warp `warp` of `nwarps` taking every nwarps-th group.
 * Positions are relative to each group's first byte: 32-bit search keys (one shuffle
 * per step instead of two) and per-lane state small enough for every warp slot of the SM
 * to stay resident.  Lane k keeps its block's start relative to the group (0 for a block that
 * starts before the range) and the typed offset of relative position 0 in that block,
 * so a unit's typed offset is one shuffle and one add.
 *
 * The walk is latency-bound (random block starts, a few KiB per group), so each warp
 * keeps as much in flight as its registers allow: the four index words of its next
 * group are loaded while the current group is walked, and U units per lane move per
 * step.  A pack finds the units' typed offsets first and then loads them; an unpack
 * loads its contiguous packed units first (no offsets needed) and locates each unit
 * only to store it, so no offsets are live across the load. */
template <int V, int DIR, int U, bool PF>
__device__ __forceinline__ void yk_hidx32_groups(const yk_launch & L, uint64_t p0, uint64_t p1,
                                                 uint64_t warp, uint64_t nwarps)
{
    typedef typename yk_vec<V>::T VT;
    const yk_level *lv = &L.desc.lv[0];
    const int lane = threadIdx.x & 31;
    char *typed = L.typed + L.desc.base;
    const uint64_t jb = yk_hidx_block(lv, p0), je = yk_hidx_block(lv, p1 - 1);
    const uint64_t ngroups = (je - jb + 32) / 32;
    /* the index words of the group a warp takes next: its first block's packed start,
     * the end of its last block, and this lane's block start and displacement */
    uint64_t f_first = 0, f_end = 0, f_bp = 0;
    int64_t f_disp = 0;
    auto fetch = [&](uint64_t gg) {
        const uint64_t j0 = jb + gg * 32, jl = j0 + (uint64_t) lane;
        const uint64_t jend = min(j0 + 32, je + 1);
        f_first = __ldg(lv->pfx + j0);
        f_end = __ldg(lv->pfx + jend);
        if (jl < jend) {
            f_bp = __ldg(lv->pfx + jl);
            f_disp = __ldg(lv->disp + jl);
        }
    };
    if (PF && warp < ngroups)
        fetch(warp);
    for (uint64_t g = warp; g < ngroups; g += nwarps) {
        const uint64_t j0 = jb + g * 32;
        const uint64_t jl = j0 + (uint64_t) lane;
        const uint64_t jend = min(j0 + 32, je + 1);
        if (!PF)
            fetch(g);
        const uint64_t gs = max(f_first, p0);
        const uint32_t n = (uint32_t) (min(f_end, p1) - gs);
        uint32_t my_rel = 0xffffffffu;
        int64_t my_adj = 0;
        if (jl < jend) {
            my_rel = f_bp <= gs ? 0u : (uint32_t) (f_bp - gs);
            my_adj = f_disp - ((int64_t) f_bp - (int64_t) gs);
        }
        if (PF && g + nwarps < ngroups)
            fetch(g + nwarps);
        VT *pk = (VT *) (L.packed + (gs - L.p0));
        for (uint32_t base = 0; base < n; base += 32u * V * U) {
            if (DIR == 0) {
                int64_t off[U];
#pragma unroll
                for (int k = 0; k < U; k++) {
                    const uint32_t r = base + (uint32_t) (k * 32 + lane) * V;
                    int idx = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const uint32_t c = __shfl_sync(0xffffffffu, my_rel, idx + step);
                        if (c <= r)
                            idx += step;
                    }
                    off[k] = __shfl_sync(0xffffffffu, my_adj, idx) + (int64_t) r;
                }
                VT v[U];
#pragma unroll
                for (int k = 0; k < U; k++)
                    if (base + (uint32_t) (k * 32 + lane) * V < n)
                        v[k] = yk_ldcg((const VT *) (typed + off[k]));
#pragma unroll
                for (int k = 0; k < U; k++)
                    if (base + (uint32_t) (k * 32 + lane) * V < n)
                        pk[base / V + (uint32_t) (k * 32 + lane)] = v[k];
            } else {
                VT v[U];
#pragma unroll
                for (int k = 0; k < U; k++)
                    if (base + (uint32_t) (k * 32 + lane) * V < n)
                        v[k] = yk_ldcg(pk + base / V + (uint32_t) (k * 32 + lane));
#pragma unroll
                for (int k = 0; k < U; k++) {
                    const uint32_t r = base + (uint32_t) (k * 32 + lane) * V;
                    int idx = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const uint32_t c = __shfl_sync(0xffffffffu, my_rel, idx + step);
                        if (c <= r)
                            idx += step;
                    }
                    const int64_t off = __shfl_sync(0xffffffffu, my_adj, idx) + (int64_t) r;
                    if (r < n)
                        *(VT *) (typed + off) = v[k];
                }
            }
        }
    }
}

/* yk_red_units' P2X form applies: an IDX level with its 32-bit table, every target
 * offset in 32 bits and blocks of a power-of-two length */
__host__ __device__ inline bool yk_red_p2x(const yk_level & lv)
{
    return lv.kind == YK_LV_IDX && (lv.has_d32 & YK_D32_TABLE) && (lv.has_d32 & YK_D32_OFFSETS) &&
        lv.cps && (lv.cps & (lv.cps - 1)) == 0;
}

/* Overlapping blocks of R bytes (one IDX level in any block order, or one VEC level
 * whose stride is under its block) under one of those operators:
 * every packed element in the range is folded into its target element by one L2
 * reduction.  The operators are commutative and associative on integers, so the
 * target ends equal to the reference's in-order application (src/backend/seq/
 * genpup.py:119-211 with the operators of :302-327) whatever order the L2 applies the
 * contributions in, and no lane reads the target or resolves which block comes first.
 * Elements u0, u0 + nthr, ... below nunits (counted from packed byte p0), U per step
 * with their loads issued together; consecutive threads take consecutive
 * elements, so the lanes of one block reduce into consecutive target elements (one L2
 * sector request per 32 bytes).  Both sides are aligned to the element size (checked
 * on the host).  K: the level's kind (IDX or VEC); D32: the IDX level's 32-bit copy of
 * its displacements. */
template <int BT, int OP, int K, bool D32, int U = 4, bool P2X = false>
__device__ __forceinline__ void yk_red_units(const yk_launch & L, uint32_t u0, uint32_t nunits,
                                             uint32_t nthr)
{
    typedef typename yk_elem<BT>::T T;
    constexpr uint32_t es = (uint32_t) sizeof(T);
    /* P2X (an IDX level read through its 32-bit table): blocks of a power-of-two length
     * and every target offset in 32 bits (YK_D32_OFFSETS), so a lane keeps a shift
     * instead of the division and 32-bit offsets.  Fewer live values matter where the
     * record is not a kernel parameter (the server's items keep every invariant in
     * thread registers). */
    typedef typename std::conditional<P2X, int32_t, int64_t>::type OFF;
    const yk_level & lv = L.desc.lv[0];
    const uint32_t p0 = (uint32_t) L.p0;
    const T *packed = (const T *) L.packed;     /* element 0 is packed byte p0 */
    char *typed = L.typed + L.desc.base;
    for (; u0 < nunits; u0 += U * nthr) {
        OFF x[U];
        T in[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            const uint32_t u = u0 + k * nthr;
            if (u < nunits) {
                const uint32_t p = p0 + u * es;
                if constexpr (P2X) {
                    const uint32_t b = p >> lv.l;
                    x[k] = __ldg((const int32_t *) (lv.disp + lv.count) + b) +
                        (int32_t) (p & ((uint32_t) lv.cps - 1u));
                } else {
                    const uint32_t b = yk_div(p, lv);
                    int64_t at;
                    if constexpr (K != YK_LV_IDX)
                        at = (int64_t) b * lv.stride;
                    else if constexpr (D32)
                        at = __ldg((const int32_t *) (lv.disp + lv.count) + b);
                    else
                        at = __ldg(lv.disp + b);
                    x[k] = at + (int64_t) (p - b * (uint32_t) lv.cps);
                }
                in[k] = __ldg(packed + u);
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++)
            if (u0 + k * nthr < nunits)
                yk_red<OP>((T *) (typed + (int64_t) x[k]), in[k]);
    }
}

/* Sorted blocks of a power-of-two byte length R, one packed element per lane (32-bit
 * positions), operator fixed at compile time.  The ownership rule of yk_owner_kernel
 * (yk_kernels.cu): element x = disp[b] + j of block b belongs to b unless block b-1 covers x from
 * a position inside the range; no earlier block can cover x when b-1 does not, because
 * the displacements ascend.  The owner folds in the blocks b+1, b+2, ... that start at
 * or before x, in block order.  Lanes of one block read the same displacement words
 * (one broadcast per warp), packed elements are read contiguously across the warp and
 * each block's target run is read and written by consecutive lanes.  This thread's
 * elements are u0, u0 + nthr, ... below nunits, counted from packed byte p0; ownership
 * is decided against the whole request's range [p0, p0 + nbytes). */
template <int BT, int OP, bool D32, int UO = 0>
__device__ __forceinline__ void yk_owner_lane_units(const yk_launch & L, int rshift, uint32_t u0,
                                                    uint32_t nunits, uint32_t nthr)
{
    typedef typename yk_elem<BT>::T T;
    /* D32: offsets in 32 bits on the level's 32-bit copy of the displacements, where the
     * host found that every target offset fits (as in yk_owner_chunk_kernel) */
    typedef typename std::conditional<D32, int32_t, int64_t>::type OFF;
    constexpr OFF OFF_MAX = D32 ? (OFF) INT32_MAX : (OFF) INT64_MAX;
    constexpr uint32_t es = (uint32_t) sizeof(T);
    /* elements per lane, loads issued together: UO when the caller sets it, else two
     * (complex pairs keep one, within the register budget of full occupancy) */
    constexpr int U = UO ? UO : (BT == YK_BT_C32 || BT == YK_BT_C64) ? 1 : 2;
    const uint32_t R = 1u << rshift;
    const yk_level & lv = L.desc.lv[0];
    const uint32_t p0 = (uint32_t) L.p0, p1 = (uint32_t) (L.p0 + L.nbytes);
    const uint32_t nblk = (uint32_t) lv.count;
    const T *packed = (const T *) L.packed;     /* element 0 is packed byte p0 */
    char *typed = L.typed + L.desc.base;
    auto disp = [&](uint32_t i) -> OFF {
        if constexpr (D32)
            return __ldg((const int32_t *) (lv.disp + lv.count) + i);   /* the 32-bit copy */
        else
            return __ldg(lv.disp + i);
    };
    for (; u0 < nunits; u0 += U * nthr) {
        /* every load that does not depend on another first: the block's displacement,
         * its predecessor's and successor's, and the packed element */
        OFF x[U], dn[U];
        uint32_t b[U];
        bool own[U];
        T in[U], out[U], in1[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            const uint32_t u = u0 + k * nthr;
            own[k] = u < nunits;
            if (!own[k])
                continue;
            const uint32_t p = p0 + u * es;
            b[k] = p >> rshift;
            const OFF d = disp(b[k]);
            const OFF dp = b[k] > 0 ? disp(b[k] - 1) : 0;
            dn[k] = b[k] + 1 < nblk ? disp(b[k] + 1) : OFF_MAX;
            in[k] = __ldg(packed + u);
            x[k] = d + (OFF) (p & (R - 1));
            /* an earlier in-range block owns this element */
            if (b[k] > 0 && x[k] < dp + (OFF) R && (b[k] - 1) * R + (uint32_t) (x[k] - dp) >= p0)
                own[k] = false;
        }
        /* then the target element and the next block's contribution, if any */
#pragma unroll
        for (int k = 0; k < U; k++) {
            if (!own[k])
                continue;
            out[k] = *(const T *) (typed + x[k]);
            if (dn[k] <= x[k]) {
                const uint64_t pp = ((uint64_t) (b[k] + 1) << rshift) + (uint64_t) (x[k] - dn[k]);
                if (pp < p1)
                    in1[k] = __ldg(packed + ((uint32_t) pp - p0) / es);
                else
                    dn[k] = OFF_MAX;
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            if (!own[k])
                continue;
            yk_elem<BT>::op(OP, in[k], out[k]);
            if (dn[k] <= x[k]) {
                yk_elem<BT>::op(OP, in1[k], out[k]);
                /* rarer: the blocks after that, in block order */
                for (uint32_t bb = b[k] + 2; bb < nblk; bb++) {
                    const OFF d2 = disp(bb);
                    if (d2 > x[k])
                        break;
                    const uint64_t pp = ((uint64_t) bb << rshift) + (uint64_t) (x[k] - d2);
                    if (pp >= p1)
                        break;  /* later blocks place x later still */
                    yk_elem<BT>::op(OP, __ldg(packed + ((uint32_t) pp - p0) / es), out[k]);
                }
            }
            *(T *) (typed + x[k]) = out[k];
        }
    }
}


/* The same with one CW-byte packed chunk per lane (CW 8 or 16; elements of 1, 2 or 4
 * bytes, or 8-byte elements other than double): the chunk's elements share one block
 * (blocks are a multiple of CW bytes long and the range and the packed pointer sit on
 * CW bytes, checked on the host), so its displacement words and the packed load serve
 * CW/es elements.
 *
 * With at most four elements per chunk the fold has no loop for the common cases: the
 * displacements of the next two blocks are loaded with the chunk's own, their
 * contributions are loaded by predicated loads, and each is folded in by a select.  A
 * warp then executes one instruction stream with all its lanes, instead of a branch
 * per owner and a loop of dependent loads run by a few lanes (which left 12.8 of 32
 * lanes active per instruction).  Only a third later block, rare at these shapes,
 * takes the loop.  double keeps yk_owner_lane_kernel: there every fold is a DADD on
 * GB300's narrow FP64 pipe, which the selects would spend on every lane.
 *
 * D32: offsets and ownership tests in 32 bits on the level's 32-bit copy of the
 * displacements, where the host found that every target offset fits.  This
 * thread's chunks are u, u + nthr, ... below nchunks, counted from packed byte p0. */
template <int BT, int OP, int CW, bool D32>
__device__ __forceinline__ void yk_owner_chunk_units(const yk_launch & L, int rshift, uint32_t u,
                                                     uint32_t nchunks, uint32_t nthr)
{
    typedef typename yk_elem<BT>::T T;
    typedef typename yk_vec<CW>::T CT;
    /* target offsets in 32 bits when the host found that every one fits (the level's
     * 32-bit copy of the displacements is read), else in 64 bits */
    typedef typename std::conditional<D32, int32_t, int64_t>::type OFF;
    constexpr OFF OFF_MAX = D32 ? (OFF) INT32_MAX : (OFF) INT64_MAX;
    constexpr uint32_t es = (uint32_t) sizeof(T);
    constexpr int E = CW / (int) es;
    const uint32_t R = 1u << rshift;
    const yk_level & lv = L.desc.lv[0];
    const uint32_t p0 = (uint32_t) L.p0, p1 = (uint32_t) (L.p0 + L.nbytes);
    const uint32_t nblk = (uint32_t) lv.count;
    const CT *packedc = (const CT *) L.packed;  /* chunk 0 is byte p0 */
    const T *packed = (const T *) L.packed;
    char *typed = L.typed + L.desc.base;
    auto disp = [&](uint32_t i) -> OFF {
        if constexpr (D32)
            return __ldg((const int32_t *) (lv.disp + lv.count) + i);   /* the 32-bit copy */
        else
            return __ldg(lv.disp + i);
    };
    for (; u < nchunks; u += nthr) {
        const uint32_t p = p0 + u * CW;
        const uint32_t b = p >> rshift;
        const OFF d = disp(b);
        const OFF dp = b > 0 ? disp(b - 1) : 0;
        const OFF dn = b + 1 < nblk ? disp(b + 1) : OFF_MAX;
        union {
            CT w;
            T e[E];
        } in;
        in.w = __ldg(packedc + u);
        const OFF x0 = d + (OFF) (p & (R - 1));
        bool own[E];
        T out[E];
        if constexpr (E <= 4) {
            const OFF dn2 = b + 2 < nblk ? disp(b + 2) : OFF_MAX;
            bool h1[E], h2[E];
            T c1[E], c2[E];
#pragma unroll
            for (int k = 0; k < E; k++) {
                const OFF x = x0 + (OFF) (k * (int) es);
                /* an earlier in-range block owns this element */
                own[k] = !(b > 0 && x < dp + (OFF) R && (b - 1) * R + (uint32_t) (x - dp) >= p0);
                if (own[k])
                    out[k] = *(const T *) (typed + x);
                /* the next two blocks' elements at x, when they exist and are in range (a
                 * later block places x later in the packed stream still) */
                h1[k] = false;
                h2[k] = false;
                c1[k] = c2[k] = T();
                if (own[k] && dn <= x) {
                    const uint64_t q1 = ((uint64_t) (b + 1) << rshift) + (uint64_t) (x - dn);
                    if (q1 < p1) {
                        h1[k] = true;
                        c1[k] = __ldg(packed + ((uint32_t) q1 - p0) / es);
                        if (dn2 <= x) {
                            const uint64_t q2 = ((uint64_t) (b + 2) << rshift) + (uint64_t) (x - dn2);
                            if (q2 < p1) {
                                h2[k] = true;
                                c2[k] = __ldg(packed + ((uint32_t) q2 - p0) / es);
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < E; k++) {
                const OFF x = x0 + (OFF) (k * (int) es);
                T v = out[k];
                yk_elem<BT>::op(OP, in.e[k], v);
                T t = v;
                yk_elem<BT>::op(OP, c1[k], t);
                v = h1[k] ? t : v;
                t = v;
                yk_elem<BT>::op(OP, c2[k], t);
                v = h2[k] ? t : v;
                if (h2[k]) {
                    /* rare: the blocks after those, in block order */
                    for (uint32_t bb = b + 3; bb < nblk; bb++) {
                        const OFF d3 = disp(bb);
                        if (d3 > x)
                            break;
                        const uint64_t pp = ((uint64_t) bb << rshift) + (uint64_t) (x - d3);
                        if (pp >= p1)
                            break;
                        yk_elem<BT>::op(OP, __ldg(packed + ((uint32_t) pp - p0) / es), v);
                    }
                }
                if (own[k])
                    *(T *) (typed + x) = v;
            }
        } else {
#pragma unroll
            for (int k = 0; k < E; k++) {
                const OFF x = x0 + (OFF) (k * (int) es);
                /* an earlier in-range block owns this element */
                own[k] = !(b > 0 && x < dp + (OFF) R && (b - 1) * R + (uint32_t) (x - dp) >= p0);
                if (own[k])
                    out[k] = *(const T *) (typed + x);
            }
#pragma unroll
            for (int k = 0; k < E; k++) {
                if (!own[k])
                    continue;
                const OFF x = x0 + (OFF) (k * (int) es);
                yk_elem<BT>::op(OP, in.e[k], out[k]);
                /* the blocks after this one that start at or before x, in block order */
                OFF dd = dn;
                for (uint32_t bb = b + 1; bb < nblk && dd <= x;) {
                    const uint64_t pp = ((uint64_t) bb << rshift) + (uint64_t) (x - dd);
                    if (pp >= p1)
                        break;
                    yk_elem<BT>::op(OP, __ldg(packed + ((uint32_t) pp - p0) / es), out[k]);
                    bb++;
                    dd = bb < nblk ? disp(bb) : OFF_MAX;
                }
                *(T *) (typed + x) = out[k];
            }
        }
    }
}

/* The struct-like pack (yk_runs_pack_kernel) with the packed side staged per warp: each
 * lane still reads its run with 16-byte loads and puts its R bytes at lane * R in the
 * warp's shared-memory tile; after __syncwarp the warp writes the tile's 32 * R packed
 * bytes as 16-byte chunks at consecutive addresses.  The per-lane form writes R/4
 * pieces of 4 bytes at an R-byte stride, so each of its store instructions touches
 * about R sectors for 128 bytes; here a store instruction fills whole sectors.  Only a
 * warp, not the CTA, waits on the tile.  Needs the packed pointer on 16 bytes (checked
 * by the launcher) and R a multiple of 4; a group of fewer than 32 elements writes its
 * last bytes as 4-byte words.  The calling warp packs the 32-element groups that start
 * at elements i0, i0 + step, ... below nel (counted from the element at packed byte
 * p0), staging each in `st`, its own 32 * 48 bytes of shared memory. */
template <int NV>
__device__ __forceinline__ void yk_runs_pack_groups(const yk_launch & L, uint32_t R, unsigned char *st,
                                                    uint32_t i0, uint32_t nel, uint32_t step)
{
    const int lane = threadIdx.x & 31;
    const int64_t E = L.desc.lv[0].stride;
    const uint32_t e0 = (uint32_t) (L.p0 / R);
    const char *tb = L.typed + L.desc.base;
    const uint32_t nw4 = R / 4;      /* R <= 16 * NV */
    for (; i0 < nel; i0 += step) {
        const uint32_t i = i0 + (uint32_t) lane;
        const uint32_t n = min(32u, nel - i0);
        if (i < nel) {
            const char *src = tb + (int64_t) (e0 + i) * E;
            union {
                uint4 w[NV];
                uint32_t u[4 * NV];
            } v;
#pragma unroll
            for (int k = 0; k < NV; k++)
                v.w[k] = yk_ldcg((const uint4 *) (src + 16 * k));
            uint32_t *sw = (uint32_t *) (st + (uint32_t) lane * R);
#pragma unroll
            for (int j = 0; j < 4 * NV; j++)
                if ((uint32_t) j < nw4)
                    sw[j] = v.u[j];
        }
        __syncwarp();
        char *dst = L.packed + (uint64_t) i0 * R;
        const uint32_t nbytes = n * R, nch = nbytes / 16;
        for (uint32_t c = (uint32_t) lane; c < nch; c += 32)
            *(uint4 *) (dst + 16 * c) = *(const uint4 *) (st + 16 * c);
        for (uint32_t q = nch * 16 + (uint32_t) lane * 4; q < nbytes; q += 128)
            *(uint32_t *) (dst + q) = *(const uint32_t *) (st + q);
        __syncwarp();
    }
}

