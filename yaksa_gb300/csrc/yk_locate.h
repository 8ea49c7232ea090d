/*
 * yk_locate.h -- packed position -> typed-buffer byte offset (see yk_desc.h).
 *
 * One definition compiled twice: into the sm_103a kernels, and into the host library
 * where yaksa_gb300_debug_locate() runs it on the CPU so tests can compare every
 * address the kernels will use against the oracle's typemap before any GPU run.
 */
#ifndef YK_LOCATE_H_INCLUDED
#define YK_LOCATE_H_INCLUDED

#include <stdint.h>
#include "yk_desc.h"

#if defined(__CUDACC__)
#define YK_HD __host__ __device__ __forceinline__
#else
#define YK_HD static inline
#endif

#if defined(__CUDA_ARCH__)
#define YK_LD(p) __ldg(p)
#define YK_MULHI32(a, b) __umulhi((a), (b))
#define YK_MULHI64(a, b) __umul64hi((a), (b))
#else
#define YK_LD(p) (*(p))
#define YK_MULHI32(a, b) ((uint32_t) (((uint64_t) (a) * (uint64_t) (b)) >> 32))
#define YK_MULHI64(a, b) ((uint64_t) (((unsigned __int128) (a) * (unsigned __int128) (b)) >> 64))
#endif

/* n / cps by the Granlund-Montgomery round-up method (constants from yk_level_set_magic) */
YK_HD uint32_t yk_div32(uint32_t n, const yk_level * l)
{
    uint32_t t = YK_MULHI32(l->m32, n);
    uint32_t sh1 = l->l ? 1u : 0u;
    uint32_t sh2 = l->l ? (uint32_t) l->l - 1u : 0u;
    return (t + ((n - t) >> sh1)) >> sh2;
}

YK_HD uint64_t yk_div64(uint64_t n, const yk_level * l)
{
    uint64_t t = YK_MULHI64(l->m64, n);
    uint32_t sh1 = l->l ? 1u : 0u;
    uint32_t sh2 = l->l ? (uint32_t) l->l - 1u : 0u;
    return (t + ((n - t) >> sh1)) >> sh2;
}

/* largest j in [lo, hi) with pfx[j] <= r, given pfx[lo] <= r < pfx[hi] */
YK_HD uint64_t yk_search_range(const uint64_t * pfx, uint64_t lo, uint64_t hi, uint64_t r)
{
    while (hi - lo > 1) {
        uint64_t mid = (lo + hi) >> 1;
        if (YK_LD(pfx + mid) <= r)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

/* HIDX block of packed position r: the tile table narrows the search to the blocks
 * overlapping r's 2^tshift-byte tile (tfb[t] is the block holding tile t's first byte) */
YK_HD uint64_t yk_hidx_block(const yk_level * l, uint64_t r)
{
    if (l->tfb) {
        uint64_t t = r >> l->tshift;
        uint64_t lo = YK_LD(l->tfb + t);
        uint64_t hi = (uint64_t) YK_LD(l->tfb + t + 1) + 1;
        if (hi > l->count)
            hi = l->count;
        return yk_search_range(l->pfx, lo, hi, r);
    }
    return yk_search_range(l->pfx, 0, l->count, r);
}

/* largest j in [0, n) with pfx[j] <= r, given pfx[0] <= r < pfx[n] */
YK_HD uint64_t yk_search(const uint64_t * pfx, uint64_t n, uint64_t r)
{
    uint64_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint64_t mid = (lo + hi) >> 1;
        if (YK_LD(pfx + mid) <= r)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

/* typed-side byte offset of packed position p; *bt and *inseg (optional) receive the
 * base type of the piece and the position within its segment */
#define YK_DEFINE_LOCATE(NAME, IDX, DIV)                                               \
YK_HD int64_t NAME(const yk_desc * d, IDX p, int *bt, uint64_t * inseg)               \
{                                                                                      \
    int64_t off = d->base;                                                             \
    IDX r = p;                                                                         \
    for (int i = 0; i < d->nlev; i++) {                                                \
        const yk_level *l = &d->lv[i];                                                 \
        if (l->kind == YK_LV_HIDX) {                                                   \
            uint64_t j = yk_hidx_block(l, (uint64_t) r);                               \
            r -= (IDX) YK_LD(l->pfx + j);                                              \
            off += YK_LD(l->disp + j);                                                 \
            IDX q = DIV(r, l);                                                         \
            r -= q * (IDX) l->cps;                                                     \
            off += (int64_t) q * l->stride;                                            \
        } else {                                                                       \
            IDX q = DIV(r, l);                                                         \
            r -= q * (IDX) l->cps;                                                     \
            if (l->kind == YK_LV_VEC)                                                  \
                off += (int64_t) q * l->stride;                                        \
            else                                                                       \
                off += YK_LD(l->disp + q);                                             \
        }                                                                              \
    }                                                                                  \
    if (d->leaf == YK_LEAF_SEG) {                                                      \
        uint64_t s = yk_search(d->seg_pfx, d->nseg, (uint64_t) r);                     \
        uint64_t rr = (uint64_t) r - YK_LD(d->seg_pfx + s);                            \
        off += YK_LD(d->seg_off + s) + (int64_t) rr;                                   \
        if (bt)                                                                        \
            *bt = d->seg_type[s];                                                      \
        if (inseg)                                                                     \
            *inseg = rr;                                                               \
    } else {                                                                           \
        off += (int64_t) r;                                                            \
        if (bt)                                                                        \
            *bt = d->leaf_type;                                                        \
        if (inseg)                                                                     \
            *inseg = (uint64_t) r;                                                     \
    }                                                                                  \
    return off;                                                                        \
}

YK_DEFINE_LOCATE(yk_locate32, uint32_t, yk_div32)
YK_DEFINE_LOCATE(yk_locate64, uint64_t, yk_div64)

#endif /* YK_LOCATE_H_INCLUDED */
