/*
 * yk_iov.c -- segment-list and serialisation entry points.
 *
 * yaksa_iov_len follows src/frontend/iov/yaksa_iov_len.c:11-19 (1 for a contiguous
 * type, count * num_contig otherwise).  The segment list itself (yaksa_iov,
 * yaksa_iov_len_max) and type serialisation (yaksa_flatten*) sit next to the
 * pack/unpack path rather than on it; until they are built they report
 * YAKSA_ERR__NOT_SUPPORTED, which the reference also uses for operations a backend
 * does not provide.
 */
#include "yk_internal.h"

int yaksa_iov_len(uintptr_t count, yaksa_type_t type, uintptr_t * iov_len)
{
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    *iov_len = t->is_contig ? 1 : count * t->num_contig;
    return YAKSA_SUCCESS;
}

int yaksa_iov_len_max(uintptr_t count, yaksa_type_t type, uintptr_t max_iov_bytes,
                      uintptr_t * iov_len, uintptr_t * actual_iov_bytes)
{
    (void) count;
    (void) type;
    (void) max_iov_bytes;
    *iov_len = 0;
    *actual_iov_bytes = 0;
    return YAKSA_ERR__NOT_SUPPORTED;
}

int yaksa_iov(const char *buf, uintptr_t count, yaksa_type_t type, uintptr_t iov_offset,
              struct iovec *iov, uintptr_t max_iov_len, uintptr_t * actual_iov_len)
{
    (void) buf;
    (void) count;
    (void) type;
    (void) iov_offset;
    (void) iov;
    (void) max_iov_len;
    *actual_iov_len = 0;
    return YAKSA_ERR__NOT_SUPPORTED;
}

int yaksa_flatten_size(yaksa_type_t type, uintptr_t * flattened_type_size)
{
    (void) type;
    *flattened_type_size = 0;
    return YAKSA_ERR__NOT_SUPPORTED;
}

int yaksa_flatten(yaksa_type_t type, void *flattened_type)
{
    (void) type;
    (void) flattened_type;
    return YAKSA_ERR__NOT_SUPPORTED;
}

int yaksa_unflatten(yaksa_type_t * type, const void *flattened_type)
{
    (void) flattened_type;
    *type = YAKSA_TYPE__NULL;
    return YAKSA_ERR__NOT_SUPPORTED;
}
