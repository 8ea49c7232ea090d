/*
 * yaksa.h -- public C interface of the GB300 pack/unpack engine.
 *
 * This header is ABI-identical to the reference library's public header
 * (src/frontend/include/yaksa.h.in): every constant below has the same value and
 * every function has the same signature, so code built against the reference
 * header links against libyaksa.so from this project unchanged.  The values are an
 * interface contract, which is why they match; the text is this project's own.
 */

#ifndef YAKSA_H_INCLUDED
#define YAKSA_H_INCLUDED

#include <stdio.h>
#include <stdint.h>
#include <sys/types.h>
#include <sys/uio.h>

#if defined(__cplusplus)
extern "C" {
#endif

/* ---------------------------------------------------------------------------
 * Reduction operators applied elementwise by pack/unpack
 * (reference: yaksa.h.in:35-48).  The operator combines the incoming value `in`
 * with the value already at the destination `out`: out = op(in, out).
 * ------------------------------------------------------------------------- */
typedef uint64_t yaksa_op_t;

#define YAKSA_OP__MAX       ((yaksa_op_t) 0)
#define YAKSA_OP__MIN       ((yaksa_op_t) 1)
#define YAKSA_OP__SUM       ((yaksa_op_t) 2)
#define YAKSA_OP__PROD      ((yaksa_op_t) 3)
#define YAKSA_OP__LAND      ((yaksa_op_t) 4)
#define YAKSA_OP__BAND      ((yaksa_op_t) 5)
#define YAKSA_OP__LOR       ((yaksa_op_t) 6)
#define YAKSA_OP__BOR       ((yaksa_op_t) 7)
#define YAKSA_OP__LXOR      ((yaksa_op_t) 8)
#define YAKSA_OP__BXOR      ((yaksa_op_t) 9)
#define YAKSA_OP__REPLACE   ((yaksa_op_t) 10)
#define YAKSA_OP__LAST      ((yaksa_op_t) 11)

/* ---------------------------------------------------------------------------
 * Type handles (reference: yaksa.h.in:62-139).  A builtin handle's value is its
 * object id; the library creates the builtin objects in exactly this order.
 * ------------------------------------------------------------------------- */
typedef uint64_t yaksa_type_t;

#define YAKSA_TYPE__NULL                  ((yaksa_type_t) 0)
#define YAKSA_TYPE___BOOL                 ((yaksa_type_t) 1)
#define YAKSA_TYPE__CHAR                  ((yaksa_type_t) 2)
#define YAKSA_TYPE__SIGNED_CHAR           ((yaksa_type_t) 3)
#define YAKSA_TYPE__UNSIGNED_CHAR         ((yaksa_type_t) 4)
#define YAKSA_TYPE__WCHAR_T               ((yaksa_type_t) 5)
#define YAKSA_TYPE__INT8_T                ((yaksa_type_t) 6)
#define YAKSA_TYPE__INT16_T               ((yaksa_type_t) 7)
#define YAKSA_TYPE__INT32_T               ((yaksa_type_t) 8)
#define YAKSA_TYPE__INT64_T               ((yaksa_type_t) 9)
#define YAKSA_TYPE__UINT8_T               ((yaksa_type_t) 10)
#define YAKSA_TYPE__UINT16_T              ((yaksa_type_t) 11)
#define YAKSA_TYPE__UINT32_T              ((yaksa_type_t) 12)
#define YAKSA_TYPE__UINT64_T              ((yaksa_type_t) 13)
#define YAKSA_TYPE__INT                   ((yaksa_type_t) 14)
#define YAKSA_TYPE__UNSIGNED              ((yaksa_type_t) 15)
#define YAKSA_TYPE__SHORT                 ((yaksa_type_t) 16)
#define YAKSA_TYPE__UNSIGNED_SHORT        ((yaksa_type_t) 17)
#define YAKSA_TYPE__LONG                  ((yaksa_type_t) 18)
#define YAKSA_TYPE__UNSIGNED_LONG         ((yaksa_type_t) 19)
#define YAKSA_TYPE__LONG_LONG             ((yaksa_type_t) 20)
#define YAKSA_TYPE__UNSIGNED_LONG_LONG    ((yaksa_type_t) 21)
#define YAKSA_TYPE__INT_FAST8_T           ((yaksa_type_t) 22)
#define YAKSA_TYPE__INT_FAST16_T          ((yaksa_type_t) 23)
#define YAKSA_TYPE__INT_FAST32_T          ((yaksa_type_t) 24)
#define YAKSA_TYPE__INT_FAST64_T          ((yaksa_type_t) 25)
#define YAKSA_TYPE__UINT_FAST8_T          ((yaksa_type_t) 26)
#define YAKSA_TYPE__UINT_FAST16_T         ((yaksa_type_t) 27)
#define YAKSA_TYPE__UINT_FAST32_T         ((yaksa_type_t) 28)
#define YAKSA_TYPE__UINT_FAST64_T         ((yaksa_type_t) 29)
#define YAKSA_TYPE__INT_LEAST8_T          ((yaksa_type_t) 30)
#define YAKSA_TYPE__INT_LEAST16_T         ((yaksa_type_t) 31)
#define YAKSA_TYPE__INT_LEAST32_T         ((yaksa_type_t) 32)
#define YAKSA_TYPE__INT_LEAST64_T         ((yaksa_type_t) 33)
#define YAKSA_TYPE__UINT_LEAST8_T         ((yaksa_type_t) 34)
#define YAKSA_TYPE__UINT_LEAST16_T        ((yaksa_type_t) 35)
#define YAKSA_TYPE__UINT_LEAST32_T        ((yaksa_type_t) 36)
#define YAKSA_TYPE__UINT_LEAST64_T        ((yaksa_type_t) 37)
#define YAKSA_TYPE__BYTE                  ((yaksa_type_t) 38)
#define YAKSA_TYPE__INTMAX_T              ((yaksa_type_t) 39)
#define YAKSA_TYPE__UINTMAX_T             ((yaksa_type_t) 40)
#define YAKSA_TYPE__SIZE_T                ((yaksa_type_t) 41)
#define YAKSA_TYPE__INTPTR_T              ((yaksa_type_t) 42)
#define YAKSA_TYPE__UINTPTR_T             ((yaksa_type_t) 43)
#define YAKSA_TYPE__PTRDIFF_T             ((yaksa_type_t) 44)
#define YAKSA_TYPE__FLOAT                 ((yaksa_type_t) 45)
#define YAKSA_TYPE__DOUBLE                ((yaksa_type_t) 46)
#define YAKSA_TYPE__LONG_DOUBLE           ((yaksa_type_t) 47)
#define YAKSA_TYPE__C_COMPLEX             ((yaksa_type_t) 48)
#define YAKSA_TYPE__C_DOUBLE_COMPLEX      ((yaksa_type_t) 49)
#define YAKSA_TYPE__C_LONG_DOUBLE_COMPLEX ((yaksa_type_t) 50)
#define YAKSA_TYPE__FLOAT_INT             ((yaksa_type_t) 51)
#define YAKSA_TYPE__DOUBLE_INT            ((yaksa_type_t) 52)
#define YAKSA_TYPE__LONG_INT              ((yaksa_type_t) 53)
#define YAKSA_TYPE__2INT                  ((yaksa_type_t) 54)
#define YAKSA_TYPE__SHORT_INT             ((yaksa_type_t) 55)
#define YAKSA_TYPE__LONG_DOUBLE_INT       ((yaksa_type_t) 56)

/* Request handles (reference: yaksa.h.in:148-153). */
typedef uint64_t yaksa_request_t;
#define YAKSA_REQUEST__NULL ((yaksa_request_t) 0)

/* Return codes (reference: yaksa.h.in:160-172). */
#define YAKSA_SUCCESS             (0)
#define YAKSA_ERR__OUT_OF_MEM     (1)
#define YAKSA_ERR__INTERNAL       (2)
#define YAKSA_ERR__NOT_SUPPORTED  (3)

/* Subarray storage order (reference: yaksa.h.in:182-190). */
typedef enum {
    YAKSA_SUBARRAY_ORDER__C,
    YAKSA_SUBARRAY_ORDER__FORTRAN
} yaksa_subarray_order_e;

/* Info objects carry key/value hints (reference: yaksa.h.in:196-204). */
typedef void *yaksa_info_t;
#define YAKSA_INFO_MAX_KEYLEN (256)

/* ---------------------------------------------------------------------------
 * Functions (reference prototypes: yaksa.h.in:221-634).
 * ------------------------------------------------------------------------- */

/* Info objects (yaksa.h.in:221-239).  Recognised keys: "yaksa_gpu_driver"
 * ("cuda" | "nogpu" ...), "yaksa_mapped_device" (int), "yaksa_has_wait_kernel",
 * "yaksa_{seq,cuda}_iov_{pack,unpack}_threshold" (uintptr_t). */
int yaksa_info_create(yaksa_info_t * info);
int yaksa_info_free(yaksa_info_t info);
int yaksa_info_keyval_append(yaksa_info_t info, const char *key, const void *val,
                             unsigned int vallen);

/* Reference-counted library initialisation (yaksa.h.in:246-251). */
int yaksa_init(yaksa_info_t info);
int yaksa_finalize(void);

/* Type constructors (yaksa.h.in:264-402).  A constructor whose result holds no
 * data returns YAKSA_TYPE__NULL. */
int yaksa_type_create_vector(intptr_t count, intptr_t blocklength, intptr_t stride,
                             yaksa_type_t oldtype, yaksa_info_t info, yaksa_type_t * newtype);
int yaksa_type_create_hvector(intptr_t count, intptr_t blocklength, intptr_t stride,
                              yaksa_type_t oldtype, yaksa_info_t info, yaksa_type_t * newtype);
int yaksa_type_create_contig(intptr_t count, yaksa_type_t oldtype, yaksa_info_t info,
                             yaksa_type_t * newtype);
int yaksa_type_create_dup(yaksa_type_t oldtype, yaksa_info_t info, yaksa_type_t * newtype);
int yaksa_type_create_indexed_block(intptr_t count, intptr_t blocklength,
                                    const intptr_t * array_of_displacements, yaksa_type_t oldtype,
                                    yaksa_info_t info, yaksa_type_t * newtype);
int yaksa_type_create_hindexed_block(intptr_t count, intptr_t blocklength,
                                     const intptr_t * array_of_displacements,
                                     yaksa_type_t oldtype, yaksa_info_t info,
                                     yaksa_type_t * newtype);
int yaksa_type_create_indexed(intptr_t count, const intptr_t * array_of_blocklengths,
                              const intptr_t * array_of_displacements, yaksa_type_t oldtype,
                              yaksa_info_t info, yaksa_type_t * newtype);
int yaksa_type_create_hindexed(intptr_t count, const intptr_t * array_of_blocklengths,
                               const intptr_t * array_of_displacements, yaksa_type_t oldtype,
                               yaksa_info_t info, yaksa_type_t * newtype);
int yaksa_type_create_resized(yaksa_type_t oldtype, intptr_t lb, intptr_t extent,
                              yaksa_info_t info, yaksa_type_t * newtype);
int yaksa_type_create_struct(intptr_t count, const intptr_t * array_of_blocklengths,
                             const intptr_t * array_of_displacements,
                             const yaksa_type_t * array_of_types, yaksa_info_t info,
                             yaksa_type_t * newtype);
int yaksa_type_create_subarray(int ndims, const intptr_t * array_of_sizes,
                               const intptr_t * array_of_subsizes,
                               const intptr_t * array_of_starts, yaksa_subarray_order_e order,
                               yaksa_type_t oldtype, yaksa_info_t info, yaksa_type_t * newtype);

/* Bounds queries (yaksa.h.in:413-445) and release (yaksa.h.in:452). */
int yaksa_type_get_size(yaksa_type_t type, uintptr_t * size);
int yaksa_type_get_true_extent(yaksa_type_t type, intptr_t * lb, intptr_t * extent);
int yaksa_type_get_extent(yaksa_type_t type, intptr_t * lb, intptr_t * extent);
int yaksa_type_free(yaksa_type_t type);

/* Requests (yaksa.h.in:460-467).  test/wait release the request once it completes. */
int yaksa_request_test(yaksa_request_t request, int *completed);
int yaksa_request_wait(yaksa_request_t request);

/* Pack: copy bytes [inoffset, inoffset + *actual_pack_bytes) of the packed form of
 * (inbuf, incount, type) into outbuf, combining with op (out = op(in, out)).  Only
 * whole builtin elements are moved, so *actual_pack_bytes may be less than
 * max_pack_bytes (yaksa.h.in:484-503). */
int yaksa_ipack(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
                void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
                yaksa_info_t info, yaksa_op_t op, yaksa_request_t * request);
int yaksa_pack(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
               void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
               yaksa_info_t info, yaksa_op_t op);

/* Unpack: the mirror of pack; insize bytes of packed data land at packed offset
 * outoffset of (outbuf, outcount, type) (yaksa.h.in:520-539). */
int yaksa_iunpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                  yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                  yaksa_info_t info, yaksa_op_t op, yaksa_request_t * request);
int yaksa_unpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                 yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                 yaksa_info_t info, yaksa_op_t op);

/* Stream-ordered variants: `stream` points to a cudaStream_t (yaksa.h.in:555-575). */
int yaksa_pack_stream(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
                      void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
                      yaksa_info_t info, yaksa_op_t op, void *stream);
int yaksa_unpack_stream(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                        yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                        yaksa_info_t info, yaksa_op_t op, void *stream);

/* Contiguous-segment lists (yaksa.h.in:584-609): the pieces of `count` elements in
 * typemap order, with the reference's piece boundaries.  yaksa_iov_len_max reports the
 * leading pieces whose bytes fit in max_iov_bytes, never splitting one builtin. */
int yaksa_iov_len(uintptr_t count, yaksa_type_t type, uintptr_t * iov_len);
int yaksa_iov_len_max(uintptr_t count, yaksa_type_t type, uintptr_t max_iov_bytes,
                      uintptr_t * iov_len, uintptr_t * actual_iov_bytes);
int yaksa_iov(const char *buf, uintptr_t count, yaksa_type_t type, uintptr_t iov_offset,
              struct iovec *iov, uintptr_t max_iov_len, uintptr_t * actual_iov_len);

/* Type serialisation (yaksa.h.in:618-634).  The flattened bytes hold no pointers, so
 * they can be sent to another process running this library; yaksa_unflatten creates a
 * new handle with the same bounds, typemap and segment list. */
int yaksa_flatten_size(yaksa_type_t type, uintptr_t * flattened_type_size);
int yaksa_flatten(yaksa_type_t type, void *flattened_type);
int yaksa_unflatten(yaksa_type_t * type, const void *flattened_type);

/* Version information (reference: yaksa.h.in:640-660). */
#define YAKSA_VERSION "0.4-gb300"
#define YAKSA_RELEASE_TYPE_ALPHA  0
#define YAKSA_RELEASE_TYPE_BETA   1
#define YAKSA_RELEASE_TYPE_RC     2
#define YAKSA_RELEASE_TYPE_PATCH  3
#define YAKSA_CALC_VERSION(MAJOR, MINOR, REVISION, TYPE, PATCH) \
    (((MAJOR) * 10000000) + ((MINOR) * 100000) + ((REVISION) * 1000) + ((TYPE) * 100) + (PATCH))
#define YAKSA_NUMVERSION YAKSA_CALC_VERSION(0, 4, 0, YAKSA_RELEASE_TYPE_PATCH, 0)

#if defined(__cplusplus)
}
#endif

#endif /* YAKSA_H_INCLUDED */
