/*
 * yk_iov.c -- segment lists: yaksa_iov_len, yaksa_iov, yaksa_iov_len_max.
 *
 * A segment list names the contiguous pieces of `count` elements of a type in typemap
 * order, as (address, length) pairs for readv/writev-style and RDMA gather callers.  The
 * pieces are those of the type tree, not of the flattened device descriptor: callers
 * index them with iov_offset and size their arrays with yaksa_iov_len, so the list must
 * have exactly count * num_contig entries with the reference's boundaries
 * (src/frontend/iov/yaksa_iov.c:48-359):
 *   - a contiguous type is one piece covering all `count` elements, whatever the offset;
 *   - a pair builtin whose second field follows the first directly is one piece per
 *     element, otherwise two (the reference's BUILTIN_PAIRTYPE_IOV, :12-46);
 *   - every other kind lists its blocks in order, recursing into the child for each
 *     block and skipping zero-length blocks of hindexed and struct types.
 * The walk is host code: it writes the caller's host array and does no data movement.
 * yaksa_gb300_iov_stream writes the same list into device memory with a kernel, from a
 * one-element template the walk builds once per type.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "yk_internal.h"
#include "yaksa_gb300.h"

int yaksa_iov_len(uintptr_t count, yaksa_type_t type, uintptr_t * iov_len)
{
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    *iov_len = t->is_contig ? 1 : count * t->num_contig;
    return YAKSA_SUCCESS;
}

static uintptr_t pieces(uintptr_t count, const yk_type * t)
{
    return t->is_contig ? 1 : count * t->num_contig;
}

/* segment list state: entries still allowed, entries to skip, output cursor */
typedef struct {
    struct iovec *out;
    uintptr_t room;
    uintptr_t skip;
    uintptr_t n;
    uint8_t *first;             /* optional: marks the first piece of a two-piece pair */
} iov_cur;

static int iov_walk(const char *buf, uintptr_t count, const yk_type * t, iov_cur * c);

/* one block of `n` children at `p`: skipped whole while the offset covers it */
static int iov_block(const char *p, uintptr_t n, const yk_type * child, iov_cur * c)
{
    uintptr_t k = pieces(n, child);
    if (c->skip >= k) {
        c->skip -= k;
        return YAKSA_SUCCESS;
    }
    return iov_walk(p, n, child, c);
}

static int iov_walk(const char *buf, uintptr_t count, const yk_type * t, iov_cur * c)
{
    if (c->room == 0)
        return YAKSA_SUCCESS;
    if (t->is_contig) {
        /* one piece for the whole run; the offset does not apply inside it */
        c->out[c->n].iov_base = (char *) buf + t->true_lb;
        c->out[c->n].iov_len = count * t->size;
        c->n++;
        c->room--;
        c->skip = 0;
        return YAKSA_SUCCESS;
    }
    if (c->skip >= count * t->num_contig) {
        c->skip -= count * t->num_contig;
        return YAKSA_SUCCESS;
    }
    switch (t->kind) {
        case YK_K_BUILTIN:{
                size_t off[2], sz[2];
                int bt[2];
                if (!yk_pair_fields(t->builtin, off, sz, bt))
                    return YAKSA_ERR__INTERNAL;
                const uintptr_t ext = (uintptr_t) t->extent;
                if (off[1] == sz[0]) {
                    /* fields back to back: one piece per element */
                    const char *z = buf + c->skip * ext;
                    uintptr_t m = YK_MIN(c->room, count - c->skip);
                    for (uintptr_t x = 0; x < m; x++, z += ext) {
                        c->out[c->n].iov_base = (char *) z;
                        c->out[c->n].iov_len = sz[0] + sz[1];
                        c->n++;
                    }
                    c->room -= m;
                } else {
                    /* two pieces per element, never split: the offset must be even and
                     * only whole pairs that fit are listed */
                    if (c->skip % 2)
                        return YAKSA_ERR__INTERNAL;
                    const char *z = buf + (c->skip / 2) * ext;
                    uintptr_t m = YK_MIN(c->room - 1, count * 2 - c->skip);
                    for (uintptr_t x = 0; x < m; x += 2, z += ext) {
                        if (c->first)
                            c->first[c->n] = 1;
                        c->out[c->n].iov_base = (char *) z;
                        c->out[c->n].iov_len = sz[0];
                        c->out[c->n + 1].iov_base = (char *) z + off[1];
                        c->out[c->n + 1].iov_len = sz[1];
                        c->n += 2;
                        c->room -= 2;
                    }
                }
                c->skip = 0;
                return YAKSA_SUCCESS;
            }
        case YK_K_CONTIG:
            return iov_walk(buf, count * (uintptr_t) t->count, t->child, c);
        case YK_K_RESIZED:
            for (uintptr_t i = 0; i < count && c->room; i++) {
                int rc = iov_block(buf + (intptr_t) i * t->extent, 1, t->child, c);
                if (rc)
                    return rc;
            }
            return YAKSA_SUCCESS;
        case YK_K_SUBARRAY:{
                const char *p = buf + t->true_lb - t->primary->true_lb;
                for (uintptr_t i = 0; i < count && c->room; i++, p += t->extent) {
                    int rc = iov_block(p, 1, t->primary, c);
                    if (rc)
                        return rc;
                }
                return YAKSA_SUCCESS;
            }
        case YK_K_HVECTOR:
        case YK_K_BLKHINDX:
        case YK_K_HINDEXED:
        case YK_K_STRUCT:
            for (uintptr_t i = 0; i < count && c->room; i++) {
                const char *el = buf + (intptr_t) i * t->extent;
                for (intptr_t j = 0; j < t->count && c->room; j++) {
                    const yk_type *ch = t->kind == YK_K_STRUCT ? t->types[j] : t->child;
                    uintptr_t n;
                    const char *p;
                    if (t->kind == YK_K_HVECTOR) {
                        n = (uintptr_t) t->blocklength;
                        p = el + j * t->stride;
                    } else if (t->kind == YK_K_BLKHINDX) {
                        n = (uintptr_t) t->blocklength;
                        p = el + t->displs[j];
                    } else {
                        n = (uintptr_t) t->blens[j];
                        p = el + t->displs[j];
                        if (n == 0)
                            continue;
                    }
                    int rc = iov_block(p, n, ch, c);
                    if (rc)
                        return rc;
                }
            }
            return YAKSA_SUCCESS;
    }
    return YAKSA_ERR__INTERNAL;
}

int yaksa_iov(const char *buf, uintptr_t count, yaksa_type_t type, uintptr_t iov_offset,
              struct iovec *iov, uintptr_t max_iov_len, uintptr_t * actual_iov_len)
{
    *actual_iov_len = 0;
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    if (max_iov_len == 0)
        return YAKSA_SUCCESS;
    iov_cur c = { iov, max_iov_len, iov_offset, 0, NULL };
    int rc = iov_walk(buf, count, t, &c);
    *actual_iov_len = c.n;
    return rc;
}

/* ------------------------------------------------------------------------- */
/* segment lists written by the GPU (no counterpart in the reference)          */
/* ------------------------------------------------------------------------- */

void yk_iov_release(yk_type * t)
{
    free(t->iov_tpl);
    free(t->iov_first);
    if (t->iov_dev)
        cudaFree(t->iov_dev);
    t->iov_tpl = NULL;
    t->iov_first = NULL;
    t->iov_dev = NULL;
    t->iov_built = 0;
}

/* one element's pieces, relative to the element's address, on the host and the device;
 * caller holds t->desc_mutex */
static int iov_template(yk_type * t)
{
    const uintptr_t n = t->num_contig;
    struct iovec *tmp = malloc(sizeof(struct iovec) * (n ? n : 1));
    t->iov_tpl = malloc(sizeof(int64_t) * 2 * (n ? n : 1));
    t->iov_first = calloc(n ? n : 1, 1);
    if (!tmp || !t->iov_tpl || !t->iov_first) {
        free(tmp);
        return YAKSA_ERR__OUT_OF_MEM;
    }
    iov_cur c = { tmp, n, 0, 0, t->iov_first };
    int rc = iov_walk((const char *) 0, 1, t, &c);
    if (!rc && c.n != n)
        rc = YAKSA_ERR__INTERNAL;
    for (uintptr_t j = 0; !rc && j < n; j++) {
        t->iov_tpl[2 * j] = (int64_t) (intptr_t) tmp[j].iov_base;
        t->iov_tpl[2 * j + 1] = (int64_t) tmp[j].iov_len;
    }
    free(tmp);
    if (rc)
        return rc;
    const size_t bytes = sizeof(int64_t) * 2 * n;
    if (yk_fail_injected() || cudaMalloc(&t->iov_dev, bytes) != cudaSuccess) {
        t->iov_dev = NULL;
        return YAKSA_ERR__OUT_OF_MEM;
    }
    /* on a private stream, waited for: a kernel already resident must not see it early */
    cudaStream_t us;
    cudaError_t e = cudaStreamCreateWithFlags(&us, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        e = cudaMemcpyAsync(t->iov_dev, t->iov_tpl, bytes, cudaMemcpyHostToDevice, us);
        cudaError_t e2 = cudaStreamSynchronize(us);
        if (e == cudaSuccess)
            e = e2;
        cudaStreamDestroy(us);
    }
    return e == cudaSuccess ? YAKSA_SUCCESS : YAKSA_ERR__INTERNAL;
}

int yaksa_gb300_iov_stream(const char *buf, uintptr_t count, yaksa_type_t type,
                           uintptr_t iov_offset, struct iovec *iov, uintptr_t max_iov_len,
                           uintptr_t * actual_iov_len, void *stream)
{
    *actual_iov_len = 0;
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    if (max_iov_len == 0 || count == 0)
        return YAKSA_SUCCESS;
    cudaStream_t s = stream ? *(cudaStream_t *) stream : (cudaStream_t) 0;
    if (t->is_contig) {
        /* one piece for all `count` elements; as in yaksa_iov, the offset does not apply
         * inside a contiguous run */
        int e = yk_cuda_iov_expand(buf, 0, NULL, 1, 0, 1, (int64_t) t->true_lb,
                                   (uint64_t) (count * t->size), iov, s);
        if (e) {
            fprintf(stderr, "yaksa-gb300: segment list launch failed: %s\n",
                    cudaGetErrorString((cudaError_t) e));
            return YAKSA_ERR__INTERNAL;
        }
        *actual_iov_len = 1;
        return YAKSA_SUCCESS;
    }
    pthread_mutex_lock(&t->desc_mutex);
    if (!t->iov_built) {
        t->iov_status = iov_template(t);
        if (t->iov_status == YAKSA_ERR__OUT_OF_MEM)
            yk_iov_release(t);          /* allocation failures are retried next time */
        else
            t->iov_built = 1;
    }
    int rc = t->iov_status;
    pthread_mutex_unlock(&t->desc_mutex);
    if (rc)
        return rc;
    const uintptr_t n = t->num_contig, total = count * n;
    if (iov_offset >= total)
        return YAKSA_SUCCESS;
    /* a two-piece pair is listed whole: never start on its second piece, never end on
     * its first (the reference's rule, src/frontend/iov/yaksa_iov.c:12-46) */
    if (iov_offset % n && t->iov_first[iov_offset % n - 1])
        return YAKSA_ERR__INTERNAL;
    uintptr_t m = YK_MIN(max_iov_len, total - iov_offset);
    if (t->iov_first[(iov_offset + m - 1) % n])
        m--;
    int e = yk_cuda_iov_expand(buf, (int64_t) t->extent, (const int64_t *) t->iov_dev, n, iov_offset, m,
                               0, 0, iov, s);
    if (e) {
        fprintf(stderr, "yaksa-gb300: segment list launch failed: %s\n",
                cudaGetErrorString((cudaError_t) e));
        return YAKSA_ERR__INTERNAL;
    }
    *actual_iov_len = m;
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* yaksa_iov_len_max: the longest leading part of the segment list whose bytes  */
/* fit in max_iov_bytes, never splitting one builtin element.  The reference's  */
/* recursion (src/frontend/iov/yaksa_iov_len_max.c:20-170) computes this for    */
/* well-formed inputs, but reads the child's block length where it means the    */
/* type's own (:59-69); this walk follows the segment list itself instead.      */
/* ------------------------------------------------------------------------- */

typedef struct {
    uintptr_t room;             /* bytes left */
    uintptr_t n, bytes;
    int full;                   /* a piece did not fit: stop */
} len_cur;

static void len_walk(uintptr_t count, const yk_type * t, len_cur * c)
{
    if (c->full)
        return;
    if (t->is_contig) {
        uintptr_t b = count * t->size;
        if (b > c->room) {
            c->full = 1;
            return;
        }
        c->room -= b;
        c->bytes += b;
        c->n++;
        return;
    }
    /* whole elements first: each adds num_contig pieces */
    uintptr_t whole = t->size ? YK_MIN(count, c->room / t->size) : count;
    c->room -= whole * t->size;
    c->bytes += whole * t->size;
    c->n += whole * t->num_contig;
    if (whole == count)
        return;
    /* the first element that does not fit, piece by piece */
    switch (t->kind) {
        case YK_K_BUILTIN:     /* a pair element is listed whole or not at all */
            c->full = 1;
            return;
        case YK_K_CONTIG:
            len_walk((uintptr_t) t->count, t->child, c);
            break;
        case YK_K_RESIZED:
            len_walk(1, t->child, c);
            break;
        case YK_K_SUBARRAY:
            len_walk(1, t->primary, c);
            break;
        case YK_K_HVECTOR:
        case YK_K_BLKHINDX:
        case YK_K_HINDEXED:
        case YK_K_STRUCT:
            for (intptr_t j = 0; j < t->count && !c->full; j++) {
                uintptr_t n = (t->kind == YK_K_HVECTOR || t->kind == YK_K_BLKHINDX) ?
                    (uintptr_t) t->blocklength : (uintptr_t) t->blens[j];
                if (n == 0 && (t->kind == YK_K_HINDEXED || t->kind == YK_K_STRUCT))
                    continue;
                len_walk(n, t->kind == YK_K_STRUCT ? t->types[j] : t->child, c);
            }
            break;
    }
    c->full = 1;
}

int yaksa_iov_len_max(uintptr_t count, yaksa_type_t type, uintptr_t max_iov_bytes,
                      uintptr_t * iov_len, uintptr_t * actual_iov_bytes)
{
    *iov_len = 0;
    *actual_iov_bytes = 0;
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    len_cur c = { max_iov_bytes, 0, 0, 0 };
    len_walk(count, t, &c);
    *iov_len = c.n;
    *actual_iov_bytes = c.bytes;
    return YAKSA_SUCCESS;
}
