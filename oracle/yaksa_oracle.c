/*
 * yaksa_oracle.c -- CPU oracle for the pack/unpack path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the test oracle, never the product: only tests/, the smoke check and the
 * bench's CPU-baseline leg load the library built from it (liboracle_yaksa.so).  It
 * exports the same C ABI as libyaksa.so (include/yaksa.h) so that the reference's own
 * test programs (test/pack/pack.c with dtpools, the programs in test/simple) compile unchanged
 * against it; those runs pin this oracle to the reference's known-answer checks.
 *
 * Semantics restated from the reference (each function cites what it follows):
 *   - type objects, bounds and constructor normalisations:
 *       src/frontend/types/yaksa_{vector,contig,dup,resized,indexed,blkindx,struct,
 *       subarray}.c; builtin objects and pair types: src/frontend/init/yaksa_init.c
 *   - pack/unpack order: the nested loops of the seq backend
 *       (src/backend/seq/genpup.py:119-211) and the frontend recursion
 *       (src/frontend/pup/yaksi_ipack_backend.c:42-220), i.e. elements in order,
 *       blocks in order, builtins in order ("typemap order");
 *   - partial packs at builtin granularity: src/frontend/pup/yaksi_ipack.c:12-107,
 *       yaksi_iunpack.c:11-116, yaksi_ipack_element.c:436-506;
 *   - elementwise operators and the per-type operator table:
 *       src/backend/seq/genpup.py:302-327, src/backend/gencomm.py:14-27.  An operator
 *       that is not in a type's table leaves the destination untouched (the generated
 *       switch has no case for it).
 *
 * The algorithm here is deliberately different from the GPU engine's: a recursive
 * walk over the type tree that keeps a running packed position and clips to the
 * requested byte range [b0, b1), instead of a flattened descriptor decomposed by
 * mixed-radix arithmetic.
 *
 * Build with -std=c11 (no FP contraction), the flags the reference itself uses
 * (configure.ac:97-112), so that float/complex arithmetic rounds like the reference.
 */

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <stdbool.h>
#include <assert.h>
#include <pthread.h>
#include <wchar.h>
#include <complex.h>
#include "yaksa.h"

/* ------------------------------------------------------------------------- */
/* type objects                                                              */
/* ------------------------------------------------------------------------- */

enum okind { OK_BUILTIN, OK_CONTIG, OK_RESIZED, OK_HVECTOR, OK_BLKHINDX, OK_HINDEXED,
    OK_STRUCT, OK_SUBARRAY };

typedef struct otype otype;
struct otype {
    int refcount;
    int kind;
    int tree_depth;
    int alignment;
    uintptr_t size;
    intptr_t extent, lb, ub, true_lb, true_ub;
    bool is_contig;
    uintptr_t num_contig;
    /* builtin: canonical handle (the object id it was created under) */
    yaksa_type_t builtin;
    /* derived parameters */
    intptr_t count, blocklength, stride;
    intptr_t *blens, *displs;
    otype *child;
    otype **types;
    int ndims;
    otype *primary;
};

static pthread_mutex_t o_mutex = PTHREAD_MUTEX_INITIALIZER;
static pthread_mutex_t o_init_mutex = PTHREAD_MUTEX_INITIALIZER;
static int o_init_count = 0;
static otype **o_handles = NULL;
static size_t o_nhandles = 0, o_cap = 0;

#define OMIN(a, b) ((a) < (b) ? (a) : (b))
#define OMAX(a, b) ((a) > (b) ? (a) : (b))

static void o_ref(otype * t)
{
    __atomic_add_fetch(&t->refcount, 1, __ATOMIC_SEQ_CST);
}

static void o_unref(otype * t)
{
    if (__atomic_sub_fetch(&t->refcount, 1, __ATOMIC_SEQ_CST) != 0)
        return;
    switch (t->kind) {
        case OK_CONTIG:
        case OK_RESIZED:
        case OK_HVECTOR:
            o_unref(t->child);
            break;
        case OK_BLKHINDX:
            free(t->displs);
            o_unref(t->child);
            break;
        case OK_HINDEXED:
            free(t->displs);
            free(t->blens);
            o_unref(t->child);
            break;
        case OK_STRUCT:
            for (intptr_t i = 0; i < t->count; i++)
                o_unref(t->types[i]);
            free(t->types);
            free(t->displs);
            free(t->blens);
            break;
        case OK_SUBARRAY:
            o_unref(t->primary);
            break;
        default:
            break;
    }
    free(t);
}

static yaksa_type_t o_handle_alloc(otype * t)
{
    pthread_mutex_lock(&o_mutex);
    size_t id = o_nhandles;
    for (size_t i = YAKSA_TYPE__LONG_DOUBLE_INT + 1; i < o_nhandles; i++)
        if (o_handles[i] == NULL) {
            id = i;
            break;
        }
    if (id == o_nhandles) {
        if (o_nhandles == o_cap) {
            o_cap = o_cap ? 2 * o_cap : 256;
            o_handles = realloc(o_handles, o_cap * sizeof(otype *));
        }
        o_nhandles++;
    }
    o_handles[id] = t;
    pthread_mutex_unlock(&o_mutex);
    return (yaksa_type_t) id;
}

static otype *o_get(yaksa_type_t h)
{
    uint64_t id = h & 0xffffffffull;
    pthread_mutex_lock(&o_mutex);
    otype *t = (id < o_nhandles) ? o_handles[id] : NULL;
    pthread_mutex_unlock(&o_mutex);
    return t;
}

static otype *o_new(int kind)
{
    otype *t = calloc(1, sizeof(otype));
    t->refcount = 1;
    t->kind = kind;
    return t;
}

/* builtin object (reference: yaksa_init.c:52-81) */
static otype *o_builtin(yaksa_type_t h, uintptr_t size, int align)
{
    otype *t = o_new(OK_BUILTIN);
    t->builtin = h;
    t->size = size;
    t->alignment = align;
    t->extent = (intptr_t) size;
    t->ub = (intptr_t) size;
    t->true_ub = (intptr_t) size;
    t->is_contig = true;
    t->num_contig = 1;
    return t;
}

/* pair object: size = sum of field sizes, extent = sizeof(struct)
 * (reference: yaksa_init.c:83-122) */
static otype *o_pair(yaksa_type_t h, size_t s1, size_t a1, size_t s2, size_t a2, size_t off2,
                     size_t structsize)
{
    otype *t = o_new(OK_BUILTIN);
    bool elem_contig = (off2 == s1);
    t->builtin = h;
    t->size = s1 + s2;
    t->alignment = (int) OMAX(a1, a2);
    t->extent = (intptr_t) structsize;
    t->ub = (intptr_t) structsize;
    t->true_ub = elem_contig ? (intptr_t) t->size : (intptr_t) structsize;
    t->is_contig = (t->size == (uintptr_t) t->extent);
    t->num_contig = 1 + !elem_contig;
    return t;
}

#define PAIR(H, T1, T2) do {                                                   \
        struct ps_ { T1 x; T2 y; };                                            \
        otype *p_ = o_pair(H, sizeof(T1), _Alignof(T1), sizeof(T2), _Alignof(T2), \
                           offsetof(struct ps_, y), sizeof(struct ps_));        \
        yaksa_type_t id_ = o_handle_alloc(p_);                                 \
        assert(id_ == H); (void) id_;                                          \
    } while (0)

#include <stddef.h>

static void o_alias(yaksa_type_t target, yaksa_type_t h)
{
    otype *t = o_get(target);
    o_ref(t);
    yaksa_type_t id = o_handle_alloc(t);
    assert(id == h);
    (void) id;
}

static void o_int_alias(size_t sz, yaksa_type_t h)
{
    yaksa_type_t tgt = sz == 1 ? YAKSA_TYPE__INT8_T : sz == 2 ? YAKSA_TYPE__INT16_T :
        sz == 4 ? YAKSA_TYPE__INT32_T : YAKSA_TYPE__INT64_T;
    o_alias(tgt, h);
}

#define BUILTIN(H, T) do {                                                     \
        yaksa_type_t id_ = o_handle_alloc(o_builtin(H, sizeof(T), _Alignof(T))); \
        assert(id_ == H); (void) id_;                                          \
    } while (0)

int yaksa_init(yaksa_info_t info)
{
    (void) info;
    /* init is reference counted and serialised (yaksa_init.c:148-160) */
    pthread_mutex_lock(&o_init_mutex);
    if (o_init_count++ > 0) {
        pthread_mutex_unlock(&o_init_mutex);
        return YAKSA_SUCCESS;
    }

    /* handle order == enum order (reference: yaksa_init.c:163-258) */
    otype *null_t = o_builtin(YAKSA_TYPE__NULL, 0, 1);
    null_t->num_contig = 0;
    o_handle_alloc(null_t);
    BUILTIN(YAKSA_TYPE___BOOL, _Bool);
    BUILTIN(YAKSA_TYPE__CHAR, char);
    o_alias(YAKSA_TYPE__CHAR, YAKSA_TYPE__SIGNED_CHAR);
    o_alias(YAKSA_TYPE__CHAR, YAKSA_TYPE__UNSIGNED_CHAR);
    BUILTIN(YAKSA_TYPE__WCHAR_T, wchar_t);
    BUILTIN(YAKSA_TYPE__INT8_T, int8_t);
    BUILTIN(YAKSA_TYPE__INT16_T, int16_t);
    BUILTIN(YAKSA_TYPE__INT32_T, int32_t);
    BUILTIN(YAKSA_TYPE__INT64_T, int64_t);
    o_alias(YAKSA_TYPE__INT8_T, YAKSA_TYPE__UINT8_T);
    o_alias(YAKSA_TYPE__INT16_T, YAKSA_TYPE__UINT16_T);
    o_alias(YAKSA_TYPE__INT32_T, YAKSA_TYPE__UINT32_T);
    o_alias(YAKSA_TYPE__INT64_T, YAKSA_TYPE__UINT64_T);
    o_int_alias(sizeof(int), YAKSA_TYPE__INT);
    o_int_alias(sizeof(unsigned), YAKSA_TYPE__UNSIGNED);
    o_int_alias(sizeof(short), YAKSA_TYPE__SHORT);
    o_int_alias(sizeof(unsigned short), YAKSA_TYPE__UNSIGNED_SHORT);
    o_int_alias(sizeof(long), YAKSA_TYPE__LONG);
    o_int_alias(sizeof(unsigned long), YAKSA_TYPE__UNSIGNED_LONG);
    o_int_alias(sizeof(long long), YAKSA_TYPE__LONG_LONG);
    o_int_alias(sizeof(unsigned long long), YAKSA_TYPE__UNSIGNED_LONG_LONG);
    o_int_alias(sizeof(int_fast8_t), YAKSA_TYPE__INT_FAST8_T);
    o_int_alias(sizeof(int_fast16_t), YAKSA_TYPE__INT_FAST16_T);
    o_int_alias(sizeof(int_fast32_t), YAKSA_TYPE__INT_FAST32_T);
    o_int_alias(sizeof(int_fast64_t), YAKSA_TYPE__INT_FAST64_T);
    o_int_alias(sizeof(uint_fast8_t), YAKSA_TYPE__UINT_FAST8_T);
    o_int_alias(sizeof(uint_fast16_t), YAKSA_TYPE__UINT_FAST16_T);
    o_int_alias(sizeof(uint_fast32_t), YAKSA_TYPE__UINT_FAST32_T);
    o_int_alias(sizeof(uint_fast64_t), YAKSA_TYPE__UINT_FAST64_T);
    o_int_alias(sizeof(int_least8_t), YAKSA_TYPE__INT_LEAST8_T);
    o_int_alias(sizeof(int_least16_t), YAKSA_TYPE__INT_LEAST16_T);
    o_int_alias(sizeof(int_least32_t), YAKSA_TYPE__INT_LEAST32_T);
    o_int_alias(sizeof(int_least64_t), YAKSA_TYPE__INT_LEAST64_T);
    o_int_alias(sizeof(uint_least8_t), YAKSA_TYPE__UINT_LEAST8_T);
    o_int_alias(sizeof(uint_least16_t), YAKSA_TYPE__UINT_LEAST16_T);
    o_int_alias(sizeof(uint_least32_t), YAKSA_TYPE__UINT_LEAST32_T);
    o_int_alias(sizeof(uint_least64_t), YAKSA_TYPE__UINT_LEAST64_T);
    o_alias(YAKSA_TYPE__UINT8_T, YAKSA_TYPE__BYTE);
    o_int_alias(sizeof(intmax_t), YAKSA_TYPE__INTMAX_T);
    o_int_alias(sizeof(uintmax_t), YAKSA_TYPE__UINTMAX_T);
    o_int_alias(sizeof(size_t), YAKSA_TYPE__SIZE_T);
    o_int_alias(sizeof(intptr_t), YAKSA_TYPE__INTPTR_T);
    o_int_alias(sizeof(uintptr_t), YAKSA_TYPE__UINTPTR_T);
    o_int_alias(sizeof(ptrdiff_t), YAKSA_TYPE__PTRDIFF_T);
    BUILTIN(YAKSA_TYPE__FLOAT, float);
    BUILTIN(YAKSA_TYPE__DOUBLE, double);
    BUILTIN(YAKSA_TYPE__LONG_DOUBLE, long double);
    PAIR(YAKSA_TYPE__C_COMPLEX, float, float);
    PAIR(YAKSA_TYPE__C_DOUBLE_COMPLEX, double, double);
    PAIR(YAKSA_TYPE__C_LONG_DOUBLE_COMPLEX, long double, long double);
    PAIR(YAKSA_TYPE__FLOAT_INT, float, int);
    PAIR(YAKSA_TYPE__DOUBLE_INT, double, int);
    PAIR(YAKSA_TYPE__LONG_INT, long, int);
    PAIR(YAKSA_TYPE__2INT, int, int);
    PAIR(YAKSA_TYPE__SHORT_INT, short, int);
    PAIR(YAKSA_TYPE__LONG_DOUBLE_INT, long double, int);
    pthread_mutex_unlock(&o_init_mutex);
    return YAKSA_SUCCESS;
}

int yaksa_finalize(void)
{
    pthread_mutex_lock(&o_init_mutex);
    if (--o_init_count > 0) {
        pthread_mutex_unlock(&o_init_mutex);
        return YAKSA_SUCCESS;
    }
    for (size_t i = 0; i <= YAKSA_TYPE__LONG_DOUBLE_INT && i < o_nhandles; i++) {
        otype *t = o_handles[i];
        o_handles[i] = NULL;
        if (t)
            o_unref(t);
    }
    /* the handle table is rebuilt from scratch by the next init */
    pthread_mutex_lock(&o_mutex);
    o_nhandles = 0;
    pthread_mutex_unlock(&o_mutex);
    pthread_mutex_unlock(&o_init_mutex);
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* info objects: the oracle accepts and ignores every hint                   */
/* ------------------------------------------------------------------------- */

int yaksa_info_create(yaksa_info_t * info)
{
    *info = malloc(16);
    return *info ? YAKSA_SUCCESS : YAKSA_ERR__OUT_OF_MEM;
}

int yaksa_info_free(yaksa_info_t info)
{
    free(info);
    return YAKSA_SUCCESS;
}

int yaksa_info_keyval_append(yaksa_info_t info, const char *key, const void *val,
                             unsigned int vallen)
{
    (void) info;
    (void) key;
    (void) val;
    (void) vallen;
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* constructors (bounds follow the reference's constructor files)            */
/* ------------------------------------------------------------------------- */

static otype *mk_contig(intptr_t count, otype * in);

static otype *mk_dup(otype * in)
{
    o_ref(in);
    return in;
}

/* yaksa_vector.c:11-84 */
static otype *mk_hvector(intptr_t count, intptr_t bl, intptr_t stride, otype * in)
{
    if (count == 1)
        return mk_contig(bl, in);
    otype *t = o_new(OK_HVECTOR);
    o_ref(in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size * bl * count;
    t->alignment = in->alignment;
    t->lb = in->lb + (stride < 0 ? stride * (count - 1) : 0) +
        (in->extent < 0 ? in->extent * (bl - 1) : 0);
    t->ub = in->ub + (stride > 0 ? stride * (count - 1) : 0) +
        (in->extent > 0 ? in->extent * (bl - 1) : 0);
    t->true_lb = t->lb + in->true_lb - in->lb;
    t->true_ub = t->ub - in->ub + in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = in->is_contig && (t->ub - t->lb) == (intptr_t) t->size && stride > 0;
    if (t->is_contig)
        t->num_contig = 1;
    else if (in->is_contig)
        t->num_contig = count * in->num_contig;
    else
        t->num_contig = count * bl * in->num_contig;
    t->count = count;
    t->blocklength = bl;
    t->stride = stride;
    t->child = in;
    return t;
}

/* yaksa_contig.c:11-57 */
static otype *mk_contig(intptr_t count, otype * in)
{
    if (count == 1)
        return mk_dup(in);
    otype *t = o_new(OK_CONTIG);
    o_ref(in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size * count;
    t->alignment = in->alignment;
    if (in->extent > 0) {
        t->lb = in->lb;
        t->ub = in->ub + (count - 1) * in->extent;
    } else {
        t->lb = in->lb + (count - 1) * in->extent;
        t->ub = in->ub;
    }
    t->true_lb = t->lb + in->true_lb - in->lb;
    t->true_ub = t->ub - in->ub + in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = in->is_contig;
    t->num_contig = t->is_contig ? 1 : count * in->num_contig;
    t->count = count;
    t->child = in;
    return t;
}

/* yaksa_resized.c:11-50 */
static otype *mk_resized(otype * in, intptr_t lb, intptr_t extent)
{
    if (lb == in->lb && extent == in->extent)
        return mk_dup(in);
    otype *t = o_new(OK_RESIZED);
    o_ref(in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size;
    t->alignment = in->alignment;
    t->lb = lb;
    t->ub = lb + extent;
    t->true_lb = in->true_lb;
    t->true_ub = in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = in->is_contig && (t->ub - t->lb) == (intptr_t) t->size;
    t->num_contig = in->num_contig;
    t->child = in;
    return t;
}

/* yaksa_blkindx.c:11-110 */
static otype *mk_blkhindx(intptr_t count, intptr_t bl, const intptr_t * displs, otype * in)
{
    bool as_hvector = (displs[0] == 0);
    for (intptr_t i = 2; i < count; i++)
        if (displs[i] - displs[i - 1] != displs[1] - displs[0])
            as_hvector = false;
    if (as_hvector)
        return mk_hvector(count, bl, count > 1 ? displs[1] - displs[0] : 0, in);

    otype *t = o_new(OK_BLKHINDX);
    o_ref(in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size * bl * count;
    t->alignment = in->alignment;
    intptr_t dmin = displs[0], dmax = displs[0];
    for (intptr_t i = 1; i < count; i++) {
        dmin = OMIN(dmin, displs[i]);
        dmax = OMAX(dmax, displs[i]);
    }
    if (in->extent > 0) {
        t->lb = dmin + in->lb;
        t->ub = dmax + in->ub + in->extent * (bl - 1);
    } else {
        t->lb = dmin + in->lb + in->extent * (bl - 1);
        t->ub = dmax + in->ub;
    }
    t->true_lb = t->lb + in->true_lb - in->lb;
    t->true_ub = t->ub - in->ub + in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = false;
    if (in->is_contig && (t->ub - t->lb) == (intptr_t) t->size) {
        t->is_contig = true;
        for (intptr_t i = 1; i < count; i++)
            if (displs[i] != displs[i - 1] + in->extent * bl) {
                t->is_contig = false;
                break;
            }
    }
    if (t->is_contig)
        t->num_contig = 1;
    else if (in->is_contig)
        t->num_contig = in->num_contig * count;
    else
        t->num_contig = in->num_contig * count * bl;
    t->count = count;
    t->blocklength = bl;
    t->displs = malloc(count * sizeof(intptr_t));
    memcpy(t->displs, displs, count * sizeof(intptr_t));
    t->child = in;
    return t;
}

/* yaksa_indexed.c:11-125 */
static otype *mk_hindexed(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                          otype * in)
{
    bool same = true;
    for (intptr_t i = 1; i < count; i++)
        if (blens[i] != blens[i - 1])
            same = false;
    if (same)
        return mk_blkhindx(count, blens[0], displs, in);

    otype *t = o_new(OK_HINDEXED);
    o_ref(in);
    t->tree_depth = in->tree_depth + 1;
    t->size = 0;
    for (intptr_t i = 0; i < count; i++)
        t->size += in->size * blens[i];
    t->alignment = in->alignment;
    bool set = false, noncontig = false;
    intptr_t last_ub = 0;
    for (intptr_t i = 0; i < count; i++) {
        if (blens[i] == 0)
            continue;
        intptr_t lb, ub;
        if (in->extent > 0) {
            lb = displs[i] + in->lb;
            ub = displs[i] + in->ub + in->extent * (blens[i] - 1);
        } else {
            lb = displs[i] + in->lb + in->extent * (blens[i] - 1);
            ub = displs[i] + in->ub;
        }
        if (i > 0 && lb != last_ub)
            noncontig = true;
        last_ub = ub;
        intptr_t tlb = lb - in->lb + in->true_lb;
        intptr_t tub = ub - in->ub + in->true_ub;
        if (set) {
            t->lb = OMIN(lb, t->lb);
            t->true_lb = OMIN(tlb, t->true_lb);
            t->ub = OMAX(ub, t->ub);
            t->true_ub = OMAX(tub, t->true_ub);
        } else {
            t->lb = lb;
            t->true_lb = tlb;
            t->ub = ub;
            t->true_ub = tub;
        }
        set = true;
    }
    t->extent = t->ub - t->lb;
    t->count = count;
    t->blens = malloc(count * sizeof(intptr_t));
    t->displs = malloc(count * sizeof(intptr_t));
    memcpy(t->blens, blens, count * sizeof(intptr_t));
    memcpy(t->displs, displs, count * sizeof(intptr_t));
    t->child = in;
    t->is_contig = !noncontig && in->is_contig && (t->ub - t->lb) == (intptr_t) t->size;
    if (t->is_contig) {
        t->num_contig = 1;
    } else if (in->is_contig) {
        uintptr_t nz = 0;
        for (intptr_t i = 0; i < count; i++)
            nz += (blens[i] != 0);
        t->num_contig = in->num_contig * nz;
    } else {
        uintptr_t tot = 0;
        for (intptr_t i = 0; i < count; i++)
            tot += blens[i];
        t->num_contig = in->num_contig * tot;
    }
    return t;
}

/* yaksa_struct.c:11-140 */
static otype *mk_struct(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                        otype ** types)
{
    bool same = true;
    for (intptr_t i = 1; i < count; i++)
        if (types[i] != types[i - 1])
            same = false;
    if (same)
        return mk_hindexed(count, blens, displs, types[0]);

    otype *t = o_new(OK_STRUCT);
    t->size = 0;
    for (intptr_t i = 0; i < count; i++) {
        t->size += types[i]->size * blens[i];
        o_ref(types[i]);
    }
    bool set = false, noncontig = false;
    intptr_t last_ub = 0;
    t->alignment = 0;
    for (intptr_t i = 0; i < count; i++) {
        if (blens[i] == 0)
            continue;
        otype *c = types[i];
        intptr_t lb, ub;
        if (c->extent > 0) {
            lb = displs[i] + c->lb;
            ub = displs[i] + c->ub + c->extent * (blens[i] - 1);
        } else {
            lb = displs[i] + c->lb + c->extent * (blens[i] - 1);
            ub = displs[i] + c->ub;
        }
        intptr_t tlb = lb - c->lb + c->true_lb;
        intptr_t tub = ub - c->ub + c->true_ub;
        if (i > 0 && tlb != last_ub)
            noncontig = true;
        last_ub = tub;
        if (t->alignment < c->alignment)
            t->alignment = c->alignment;
        if (set) {
            t->lb = OMIN(lb, t->lb);
            t->true_lb = OMIN(tlb, t->true_lb);
            t->ub = OMAX(ub, t->ub);
            t->true_ub = OMAX(tub, t->true_ub);
            t->tree_depth = OMAX(c->tree_depth, t->tree_depth);
        } else {
            t->lb = lb;
            t->true_lb = tlb;
            t->ub = ub;
            t->true_ub = tub;
            t->tree_depth = c->tree_depth;
        }
        set = true;
    }
    assert(t->alignment);
    uintptr_t rem = (uintptr_t) (t->ub - t->lb) % (uintptr_t) t->alignment;
    if (rem)
        t->ub += t->alignment - rem;
    t->tree_depth++;
    t->extent = t->ub - t->lb;
    t->is_contig = false;
    if (!noncontig && (t->ub - t->lb) == (intptr_t) t->size) {
        t->is_contig = true;
        for (intptr_t i = 0; i < count; i++)
            if (!types[i]->is_contig) {
                t->is_contig = false;
                break;
            }
    }
    if (t->is_contig && t->ub == t->extent) {
        t->num_contig = 1;
    } else {
        t->num_contig = 0;
        for (intptr_t i = 0; i < count; i++) {
            if (types[i]->is_contig && blens[i])
                t->num_contig++;
            else
                t->num_contig += types[i]->num_contig * blens[i];
        }
    }
    t->count = count;
    t->blens = malloc(count * sizeof(intptr_t));
    t->displs = malloc(count * sizeof(intptr_t));
    t->types = malloc(count * sizeof(otype *));
    memcpy(t->blens, blens, count * sizeof(intptr_t));
    memcpy(t->displs, displs, count * sizeof(intptr_t));
    memcpy(t->types, types, count * sizeof(otype *));
    return t;
}

/* yaksa_subarray.c:11-119 */
static otype *mk_subarray(int ndims, const intptr_t * sizes, const intptr_t * subsizes,
                          const intptr_t * starts, yaksa_subarray_order_e order, otype * in)
{
    otype *t = o_new(OK_SUBARRAY);
    t->tree_depth = in->tree_depth + 1;
    t->alignment = in->alignment;
    t->ndims = ndims;
    intptr_t stride = in->extent;
    otype *cur, *next;
    if (order == YAKSA_SUBARRAY_ORDER__C) {
        cur = mk_contig(subsizes[ndims - 1], in);
        for (int i = ndims - 2; i >= 0; i--) {
            stride *= sizes[i + 1];
            next = mk_hvector(subsizes[i], 1, stride, cur);
            o_unref(cur);
            cur = next;
        }
    } else {
        cur = mk_contig(subsizes[0], in);
        for (int i = 1; i < ndims; i++) {
            stride *= sizes[i - 1];
            next = mk_hvector(subsizes[i], 1, stride, cur);
            o_unref(cur);
            cur = next;
        }
    }
    intptr_t extent = in->extent;
    for (int i = 0; i < ndims; i++)
        extent *= sizes[i];
    next = mk_resized(cur, 0, extent);
    o_unref(cur);
    t->primary = next;
    t->lb = 0;
    t->ub = extent;
    t->extent = extent;
    t->size = in->size;
    t->true_lb = in->true_lb;
    t->true_ub = in->true_ub;
    for (int i = 0; i < ndims; i++) {
        t->size *= subsizes[i];
        intptr_t tlb = starts[i] * in->extent;
        intptr_t tub = (starts[i] + subsizes[i] - 1) * in->extent;
        if (order == YAKSA_SUBARRAY_ORDER__C) {
            for (int j = i + 1; j < ndims; j++) {
                tlb *= sizes[j];
                tub *= sizes[j];
            }
        } else {
            for (int j = 0; j < i; j++) {
                tlb *= sizes[j];
                tub *= sizes[j];
            }
        }
        t->true_lb += tlb;
        t->true_ub += tub;
    }
    t->is_contig = in->is_contig && (t->ub - t->lb) == (intptr_t) t->size;
    t->num_contig = t->primary->num_contig;
    return t;
}

#define GET_OR_FAIL(h, t) otype *t = o_get(h); if (!t) return YAKSA_ERR__INTERNAL

static int o_finish(otype * t, yaksa_type_t * newtype)
{
    *newtype = o_handle_alloc(t);
    return YAKSA_SUCCESS;
}

int yaksa_type_create_hvector(intptr_t count, intptr_t bl, intptr_t stride, yaksa_type_t old,
                              yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    if (count * (intptr_t) in->size == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    return o_finish(mk_hvector(count, bl, stride, in), newtype);
}

int yaksa_type_create_vector(intptr_t count, intptr_t bl, intptr_t stride, yaksa_type_t old,
                             yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    if (count * (intptr_t) in->size == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    return o_finish(mk_hvector(count, bl, stride * in->extent, in), newtype);
}

int yaksa_type_create_contig(intptr_t count, yaksa_type_t old, yaksa_info_t info,
                             yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    if (count * (intptr_t) in->size == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    return o_finish(mk_contig(count, in), newtype);
}

int yaksa_type_create_dup(yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    return o_finish(mk_dup(in), newtype);
}

int yaksa_type_create_hindexed_block(intptr_t count, intptr_t bl, const intptr_t * displs,
                                     yaksa_type_t old, yaksa_info_t info,
                                     yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    if (count * (intptr_t) in->size == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    return o_finish(mk_blkhindx(count, bl, displs, in), newtype);
}

int yaksa_type_create_indexed_block(intptr_t count, intptr_t bl, const intptr_t * displs,
                                    yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    if (count * (intptr_t) in->size == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    intptr_t *d = malloc(count * sizeof(intptr_t));
    for (intptr_t i = 0; i < count; i++)
        d[i] = displs[i] * in->extent;
    int rc = o_finish(mk_blkhindx(count, bl, d, in), newtype);
    free(d);
    return rc;
}

int yaksa_type_create_hindexed(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                               yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    uintptr_t total = 0;
    for (intptr_t i = 0; i < count; i++)
        total += in->size * blens[i];
    if (total == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    return o_finish(mk_hindexed(count, blens, displs, in), newtype);
}

int yaksa_type_create_indexed(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                              yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    uintptr_t total = 0;
    for (intptr_t i = 0; i < count; i++)
        total += in->size * blens[i];
    if (total == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    intptr_t *d = malloc(count * sizeof(intptr_t));
    for (intptr_t i = 0; i < count; i++)
        d[i] = displs[i] * in->extent;
    int rc = o_finish(mk_hindexed(count, blens, d, in), newtype);
    free(d);
    return rc;
}

int yaksa_type_create_resized(yaksa_type_t old, intptr_t lb, intptr_t extent,
                              yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    return o_finish(mk_resized(in, lb, extent), newtype);
}

int yaksa_type_create_struct(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                             const yaksa_type_t * types, yaksa_info_t info,
                             yaksa_type_t * newtype)
{
    (void) info;
    uintptr_t total = 0;
    for (intptr_t i = 0; i < count; i++) {
        GET_OR_FAIL(types[i], c);
        total += c->size * blens[i];
    }
    if (total == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    otype **in = malloc(count * sizeof(otype *));
    for (intptr_t i = 0; i < count; i++)
        in[i] = o_get(types[i]);
    int rc = o_finish(mk_struct(count, blens, displs, in), newtype);
    free(in);
    return rc;
}

int yaksa_type_create_subarray(int ndims, const intptr_t * sizes, const intptr_t * subsizes,
                               const intptr_t * starts, yaksa_subarray_order_e order,
                               yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    GET_OR_FAIL(old, in);
    if (ndims * (intptr_t) in->size == 0) {
        *newtype = YAKSA_TYPE__NULL;
        return YAKSA_SUCCESS;
    }
    return o_finish(mk_subarray(ndims, sizes, subsizes, starts, order, in), newtype);
}

int yaksa_type_get_size(yaksa_type_t type, uintptr_t * size)
{
    GET_OR_FAIL(type, t);
    *size = t->size;
    return YAKSA_SUCCESS;
}

int yaksa_type_get_extent(yaksa_type_t type, intptr_t * lb, intptr_t * extent)
{
    GET_OR_FAIL(type, t);
    *lb = t->lb;
    *extent = t->extent;
    return YAKSA_SUCCESS;
}

int yaksa_type_get_true_extent(yaksa_type_t type, intptr_t * lb, intptr_t * extent)
{
    GET_OR_FAIL(type, t);
    *lb = t->true_lb;
    *extent = t->true_ub - t->true_lb;
    return YAKSA_SUCCESS;
}

int yaksa_type_free(yaksa_type_t type)
{
    uint64_t id = type & 0xffffffffull;
    if (id <= YAKSA_TYPE__LONG_DOUBLE_INT)
        return YAKSA_SUCCESS;   /* builtins live until finalize */
    pthread_mutex_lock(&o_mutex);
    otype *t = (id < o_nhandles) ? o_handles[id] : NULL;
    if (t)
        o_handles[id] = NULL;
    pthread_mutex_unlock(&o_mutex);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    o_unref(t);
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* elementwise operators (seq/genpup.py:302-327; per-type table gencomm.py:14-27) */
/* ------------------------------------------------------------------------- */

#define OPS_INT(T)                                                             \
static void op_##T(yaksa_op_t op, T *out, const T *in)                         \
{                                                                              \
    switch (op) {                                                              \
    case YAKSA_OP__REPLACE: *out = *in; break;                                 \
    case YAKSA_OP__MAX: *out = (*in < *out) ? *out : *in; break;              \
    case YAKSA_OP__MIN: *out = (*in < *out) ? *in : *out; break;              \
    case YAKSA_OP__SUM: *out = (T) ((uint64_t) *out + (uint64_t) *in); break;  \
    case YAKSA_OP__PROD: *out = (T) ((uint64_t) *out * (uint64_t) *in); break; \
    case YAKSA_OP__LAND: *out = (*out && *in); break;                          \
    case YAKSA_OP__LOR: *out = (*out || *in); break;                           \
    case YAKSA_OP__LXOR: *out = (!*out != !*in); break;                        \
    case YAKSA_OP__BAND: *out &= *in; break;                                   \
    case YAKSA_OP__BOR: *out |= *in; break;                                    \
    case YAKSA_OP__BXOR: *out ^= *in; break;                                   \
    default: break;                                                            \
    }                                                                          \
}
OPS_INT(int8_t)
OPS_INT(int16_t)
OPS_INT(int32_t)
OPS_INT(int64_t)

/* float MAX/MIN are selects, not fmax/fmin: x_[in < out] and x_[in > out] */
#define OPS_FLT(T, N)                                                          \
static void op_##N(yaksa_op_t op, T *out, const T *in)                         \
{                                                                              \
    T a = *in, b = *out;                                                       \
    switch (op) {                                                              \
    case YAKSA_OP__REPLACE: *out = a; break;                                   \
    case YAKSA_OP__MAX: *out = (a < b) ? b : a; break;                         \
    case YAKSA_OP__MIN: *out = (a > b) ? b : a; break;                         \
    case YAKSA_OP__SUM: *out = b + a; break;                                   \
    case YAKSA_OP__PROD: *out = b * a; break;                                  \
    default: break;                                                            \
    }                                                                          \
}
OPS_FLT(float, float)
OPS_FLT(double, double)
OPS_FLT(long double, ldouble)

#define OPS_CPLX(T, N)                                                         \
static void op_##N(yaksa_op_t op, T *out, const T *in)                         \
{                                                                              \
    switch (op) {                                                              \
    case YAKSA_OP__REPLACE: *out = *in; break;                                 \
    case YAKSA_OP__SUM: *out += *in; break;                                    \
    case YAKSA_OP__PROD: *out *= *in; break;                                   \
    default: break;                                                            \
    }                                                                          \
}
OPS_CPLX(float _Complex, cfloat)
OPS_CPLX(double _Complex, cdouble)
OPS_CPLX(long double _Complex, cldouble)

static void op_bool(yaksa_op_t op, _Bool * out, const _Bool * in)
{
    switch (op) {
        case YAKSA_OP__REPLACE:
            *out = *in;
            break;
        case YAKSA_OP__LAND:
            *out = (*out && *in);
            break;
        case YAKSA_OP__LOR:
            *out = (*out || *in);
            break;
        case YAKSA_OP__LXOR:
            *out = (!*out != !*in);
            break;
        default:
            break;
    }
}

/* Apply op to n consecutive builtins of canonical handle h.  `tb` walks the typed
 * (strided) side with stride `tstride`; `pk` walks the packed side contiguously.
 * dir 0 = pack (out = packed), 1 = unpack (out = typed side). */
static void apply_builtin(yaksa_type_t h, yaksa_op_t op, int dir, char *tb, intptr_t tstride,
                          char *pk, uintptr_t n);

#define LOOP(T, FN) do {                                                       \
        for (uintptr_t i_ = 0; i_ < n; i_++) {                                 \
            T a_, b_;                                                          \
            memcpy(&a_, tb + (intptr_t) i_ * tstride, sizeof(T));             \
            memcpy(&b_, pk + i_ * sizeof(T), sizeof(T));                       \
            if (dir == 0) { FN(op, &b_, &a_); memcpy(pk + i_ * sizeof(T), &b_, sizeof(T)); } \
            else { FN(op, &a_, &b_); memcpy(tb + (intptr_t) i_ * tstride, &a_, sizeof(T)); } \
        }                                                                      \
    } while (0)

#define PAIRLOOP(T1, T2, H1, H2) do {                                          \
        struct ps_ { T1 x; T2 y; };                                            \
        for (uintptr_t i_ = 0; i_ < n; i_++) {                                 \
            apply_builtin(H1, op, dir, tb + (intptr_t) i_ * tstride, 0,        \
                          pk + i_ * (sizeof(T1) + sizeof(T2)), 1);             \
            apply_builtin(H2, op, dir, tb + (intptr_t) i_ * tstride + offsetof(struct ps_, y), 0, \
                          pk + i_ * (sizeof(T1) + sizeof(T2)) + sizeof(T1), 1); \
        }                                                                      \
    } while (0)

static void apply_builtin(yaksa_type_t h, yaksa_op_t op, int dir, char *tb, intptr_t tstride,
                          char *pk, uintptr_t n)
{
    switch (h) {
        case YAKSA_TYPE___BOOL:
            LOOP(_Bool, op_bool);
            break;
        case YAKSA_TYPE__CHAR:
        case YAKSA_TYPE__WCHAR_T:
            if (op == YAKSA_OP__REPLACE) {
                size_t s = (h == YAKSA_TYPE__CHAR) ? 1 : sizeof(wchar_t);
                for (uintptr_t i = 0; i < n; i++) {
                    if (dir == 0)
                        memcpy(pk + i * s, tb + (intptr_t) i * tstride, s);
                    else
                        memcpy(tb + (intptr_t) i * tstride, pk + i * s, s);
                }
            }
            break;
        case YAKSA_TYPE__INT8_T:
            LOOP(int8_t, op_int8_t);
            break;
        case YAKSA_TYPE__INT16_T:
            LOOP(int16_t, op_int16_t);
            break;
        case YAKSA_TYPE__INT32_T:
            LOOP(int32_t, op_int32_t);
            break;
        case YAKSA_TYPE__INT64_T:
            LOOP(int64_t, op_int64_t);
            break;
        case YAKSA_TYPE__FLOAT:
            LOOP(float, op_float);
            break;
        case YAKSA_TYPE__DOUBLE:
            LOOP(double, op_double);
            break;
        case YAKSA_TYPE__LONG_DOUBLE:
            LOOP(long double, op_ldouble);
            break;
        case YAKSA_TYPE__C_COMPLEX:
            LOOP(float _Complex, op_cfloat);
            break;
        case YAKSA_TYPE__C_DOUBLE_COMPLEX:
            LOOP(double _Complex, op_cdouble);
            break;
        case YAKSA_TYPE__C_LONG_DOUBLE_COMPLEX:
            LOOP(long double _Complex, op_cldouble);
            break;
            /* pair types move field by field (yaksi_ipack_backend.c:13-40) */
        case YAKSA_TYPE__FLOAT_INT:
            PAIRLOOP(float, int, YAKSA_TYPE__FLOAT, YAKSA_TYPE__INT32_T);
            break;
        case YAKSA_TYPE__DOUBLE_INT:
            PAIRLOOP(double, int, YAKSA_TYPE__DOUBLE, YAKSA_TYPE__INT32_T);
            break;
        case YAKSA_TYPE__LONG_INT:
            PAIRLOOP(long, int, YAKSA_TYPE__INT64_T, YAKSA_TYPE__INT32_T);
            break;
        case YAKSA_TYPE__2INT:
            PAIRLOOP(int, int, YAKSA_TYPE__INT32_T, YAKSA_TYPE__INT32_T);
            break;
        case YAKSA_TYPE__SHORT_INT:
            PAIRLOOP(short, int, YAKSA_TYPE__INT16_T, YAKSA_TYPE__INT32_T);
            break;
        case YAKSA_TYPE__LONG_DOUBLE_INT:
            PAIRLOOP(long double, int, YAKSA_TYPE__LONG_DOUBLE, YAKSA_TYPE__INT32_T);
            break;
        default:
            break;
    }
}

/* ------------------------------------------------------------------------- */
/* the range-clipped typemap walk                                            */
/* ------------------------------------------------------------------------- */

typedef struct {
    char *pk;                   /* packed buffer, addressed by packed position - b0 */
    uintptr_t b0, b1;           /* requested packed byte range */
    uintptr_t pos;              /* packed position of the next builtin */
    uintptr_t done;             /* packed position where processing stopped */
    int stop;
    int err;
    int dir;
    yaksa_op_t op;
} walk_s;

static void walk(walk_s * w, const otype * t, char *base, uintptr_t count);

/* count builtins of t at base, base + extent, ... (yaksi_ipack.c step 3/4 at the
 * leaf: only whole builtins are moved) */
static void walk_leaf(walk_s * w, const otype * t, char *base, uintptr_t count)
{
    uintptr_t s = t->size;
    uintptr_t first = 0;
    if (w->pos < w->b0) {
        first = (w->b0 - w->pos) / s;
        w->pos += first * s;
        if (w->pos != w->b0) {
            /* the offset falls inside a builtin: a precondition violation that the
             * reference asserts on (yaksi_ipack_element.c:450-454) */
            w->err = 1;
            w->stop = 1;
            return;
        }
    }
    uintptr_t avail = (w->b1 - w->pos) / s;
    uintptr_t n = OMIN(count - first, avail);
    if (n) {
        char *pk = w->pk + (w->pos - w->b0);
        char *tb = base + (intptr_t) first * t->extent;
        if (w->op == YAKSA_OP__REPLACE && t->is_contig && t->extent == (intptr_t) s) {
            if (w->dir == 0)
                memcpy(pk, tb, n * s);
            else
                memcpy(tb, pk, n * s);
        } else {
            apply_builtin(t->builtin, w->op, w->dir, tb, t->extent, pk, n);
        }
        w->pos += n * s;
    }
    w->done = w->pos;
    if (first + n < count)
        w->stop = 1;    /* the next builtin does not fit in [b0, b1) */
}

static void walk_elem(walk_s * w, const otype * t, char *p)
{
    switch (t->kind) {
        case OK_HVECTOR:
            for (intptr_t j = 0; j < t->count && !w->stop; j++)
                walk(w, t->child, p + j * t->stride, t->blocklength);
            break;
        case OK_BLKHINDX:
            for (intptr_t j = 0; j < t->count && !w->stop; j++)
                walk(w, t->child, p + t->displs[j], t->blocklength);
            break;
        case OK_HINDEXED:
            for (intptr_t j = 0; j < t->count && !w->stop; j++)
                if (t->blens[j])
                    walk(w, t->child, p + t->displs[j], t->blens[j]);
            break;
        case OK_STRUCT:
            for (intptr_t j = 0; j < t->count && !w->stop; j++)
                if (t->blens[j])
                    walk(w, t->types[j], p + t->displs[j], t->blens[j]);
            break;
        case OK_RESIZED:
            walk(w, t->child, p, 1);
            break;
        case OK_CONTIG:
            walk(w, t->child, p, t->count);
            break;
        case OK_SUBARRAY:
            /* the primary type starts at the subarray's first element
             * (yaksi_ipack_backend.c:202-209) */
            walk(w, t->primary, p + t->true_lb - t->primary->true_lb, 1);
            break;
        default:
            assert(0);
    }
}

static void walk(walk_s * w, const otype * t, char *base, uintptr_t count)
{
    if (w->stop || count == 0)
        return;
    uintptr_t total = count * t->size;
    if (w->pos + total <= w->b0) {
        w->pos += total;
        return;
    }
    if (t->kind == OK_BUILTIN) {
        walk_leaf(w, t, base, count);
        return;
    }
    uintptr_t i = 0;
    if (w->pos < w->b0) {
        i = (w->b0 - w->pos) / t->size;
        w->pos += i * t->size;
    }
    /* whole contiguous elements inside the range: one memcpy (seq memcpy path) */
    if (w->op == YAKSA_OP__REPLACE && t->is_contig && w->pos >= w->b0) {
        uintptr_t avail = (w->b1 - w->pos) / t->size;
        uintptr_t n = OMIN(count - i, avail);
        if (n) {
            char *pk = w->pk + (w->pos - w->b0);
            char *tb = base + (intptr_t) i * t->extent + t->true_lb;
            if (w->dir == 0)
                memcpy(pk, tb, n * t->size);
            else
                memcpy(tb, pk, n * t->size);
            w->pos += n * t->size;
            w->done = w->pos;
            i += n;
        }
    }
    for (; i < count && !w->stop; i++) {
        if (w->pos >= w->b1) {
            w->stop = 1;
            break;
        }
        walk_elem(w, t, base + (intptr_t) i * t->extent);
    }
}

static int o_supported_op(yaksa_op_t op)
{
    return op < YAKSA_OP__LAST;
}

static int o_pup(int dir, char *typed, uintptr_t count, otype * t, uintptr_t offset,
                 char *packed, uintptr_t maxbytes, uintptr_t * actual, yaksa_op_t op)
{
    *actual = 0;
    if (count == 0 || t->size == 0)
        return YAKSA_SUCCESS;
    if (!o_supported_op(op))
        return YAKSA_ERR__INTERNAL;
    uintptr_t total = count * t->size;
    if (offset >= total)
        return YAKSA_SUCCESS;
    walk_s w = { 0 };
    w.pk = packed;
    w.b0 = offset;
    w.b1 = offset + OMIN(maxbytes, total - offset);
    w.pos = 0;
    w.done = offset;
    w.dir = dir;
    w.op = op;
    walk(&w, t, typed, count);
    if (w.err)
        return YAKSA_ERR__INTERNAL;
    *actual = w.done - offset;
    return YAKSA_SUCCESS;
}

int yaksa_pack(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
               void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
               yaksa_info_t info, yaksa_op_t op)
{
    (void) info;
    if (incount == 0) {
        *actual_pack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    GET_OR_FAIL(type, t);
    return o_pup(0, (char *) inbuf, incount, t, inoffset, outbuf, max_pack_bytes,
                 actual_pack_bytes, op);
}

int yaksa_ipack(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
                void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
                yaksa_info_t info, yaksa_op_t op, yaksa_request_t * request)
{
    *request = YAKSA_REQUEST__NULL;
    return yaksa_pack(inbuf, incount, type, inoffset, outbuf, max_pack_bytes,
                      actual_pack_bytes, info, op);
}

int yaksa_unpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                 yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                 yaksa_info_t info, yaksa_op_t op)
{
    (void) info;
    if (outcount == 0) {
        *actual_unpack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    GET_OR_FAIL(type, t);
    return o_pup(1, (char *) outbuf, outcount, t, outoffset, (char *) inbuf, insize,
                 actual_unpack_bytes, op);
}

int yaksa_iunpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                  yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                  yaksa_info_t info, yaksa_op_t op, yaksa_request_t * request)
{
    *request = YAKSA_REQUEST__NULL;
    return yaksa_unpack(inbuf, insize, outbuf, outcount, type, outoffset, actual_unpack_bytes,
                        info, op);
}

int yaksa_pack_stream(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
                      void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
                      yaksa_info_t info, yaksa_op_t op, void *stream)
{
    (void) stream;
    return yaksa_pack(inbuf, incount, type, inoffset, outbuf, max_pack_bytes,
                      actual_pack_bytes, info, op);
}

int yaksa_unpack_stream(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                        yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                        yaksa_info_t info, yaksa_op_t op, void *stream)
{
    (void) stream;
    return yaksa_unpack(inbuf, insize, outbuf, outcount, type, outoffset, actual_unpack_bytes,
                        info, op);
}

int yaksa_request_test(yaksa_request_t request, int *completed)
{
    (void) request;
    *completed = 1;
    return YAKSA_SUCCESS;
}

int yaksa_request_wait(yaksa_request_t request)
{
    (void) request;
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* typemap dump: the typed-buffer offset of every packed byte, in pack order  */
/* (tests compare the GPU engine's address computation against it)            */
/* ------------------------------------------------------------------------- */

static void tm_rec(const otype * t, int64_t base, uintptr_t count, int64_t * out, uintptr_t * pos);

static void tm_elem(const otype * t, int64_t p, int64_t * out, uintptr_t * pos)
{
    switch (t->kind) {
        case OK_BUILTIN:{
                /* pair types: two fields (yaksi_ipack_backend.c:13-40) */
                size_t s1 = t->size, off2 = 0, s2 = 0;
                switch (t->builtin) {
                    case YAKSA_TYPE__FLOAT_INT:{
                            struct p_ { float x; int y; };
                            s1 = sizeof(float); off2 = offsetof(struct p_, y); s2 = sizeof(int);
                            break;
                        }
                    case YAKSA_TYPE__DOUBLE_INT:{
                            struct p_ { double x; int y; };
                            s1 = sizeof(double); off2 = offsetof(struct p_, y); s2 = sizeof(int);
                            break;
                        }
                    case YAKSA_TYPE__LONG_INT:{
                            struct p_ { long x; int y; };
                            s1 = sizeof(long); off2 = offsetof(struct p_, y); s2 = sizeof(int);
                            break;
                        }
                    case YAKSA_TYPE__2INT:{
                            struct p_ { int x; int y; };
                            s1 = sizeof(int); off2 = offsetof(struct p_, y); s2 = sizeof(int);
                            break;
                        }
                    case YAKSA_TYPE__SHORT_INT:{
                            struct p_ { short x; int y; };
                            s1 = sizeof(short); off2 = offsetof(struct p_, y); s2 = sizeof(int);
                            break;
                        }
                    case YAKSA_TYPE__LONG_DOUBLE_INT:{
                            struct p_ { long double x; int y; };
                            s1 = sizeof(long double); off2 = offsetof(struct p_, y);
                            s2 = sizeof(int);
                            break;
                        }
                    default:
                        break;
                }
                for (size_t k = 0; k < s1; k++)
                    out[(*pos)++] = p + (int64_t) k;
                for (size_t k = 0; k < s2; k++)
                    out[(*pos)++] = p + (int64_t) (off2 + k);
                break;
            }
        case OK_HVECTOR:
            for (intptr_t j = 0; j < t->count; j++)
                tm_rec(t->child, p + j * t->stride, t->blocklength, out, pos);
            break;
        case OK_BLKHINDX:
            for (intptr_t j = 0; j < t->count; j++)
                tm_rec(t->child, p + t->displs[j], t->blocklength, out, pos);
            break;
        case OK_HINDEXED:
            for (intptr_t j = 0; j < t->count; j++)
                tm_rec(t->child, p + t->displs[j], t->blens[j], out, pos);
            break;
        case OK_STRUCT:
            for (intptr_t j = 0; j < t->count; j++)
                tm_rec(t->types[j], p + t->displs[j], t->blens[j], out, pos);
            break;
        case OK_RESIZED:
            tm_rec(t->child, p, 1, out, pos);
            break;
        case OK_CONTIG:
            tm_rec(t->child, p, t->count, out, pos);
            break;
        case OK_SUBARRAY:
            tm_rec(t->primary, p + t->true_lb - t->primary->true_lb, 1, out, pos);
            break;
    }
}

static void tm_rec(const otype * t, int64_t base, uintptr_t count, int64_t * out, uintptr_t * pos)
{
    for (uintptr_t i = 0; i < count; i++)
        tm_elem(t, base + (int64_t) i * t->extent, out, pos);
}

/* out must hold count * size entries */
int yaksa_oracle_byte_offsets(yaksa_type_t type, uintptr_t count, int64_t * out)
{
    GET_OR_FAIL(type, t);
    uintptr_t pos = 0;
    tm_rec(t, 0, count, out, &pos);
    return pos == count * t->size ? YAKSA_SUCCESS : YAKSA_ERR__INTERNAL;
}

/* ------------------------------------------------------------------------- */
/* segment lists (src/frontend/iov/yaksa_iov.c, yaksa_iov_len.c)              */
/* ------------------------------------------------------------------------- */

int yaksa_iov_len(uintptr_t count, yaksa_type_t type, uintptr_t * iov_len)
{
    GET_OR_FAIL(type, t);
    /* yaksa_iov_len.c:11-19 */
    *iov_len = t->is_contig ? 1 : count * t->num_contig;
    return YAKSA_SUCCESS;
}

/* first field size, second field offset and size of a pair builtin */
static int o_pair_layout(yaksa_type_t h, size_t * s1, size_t * off2, size_t * s2)
{
#define PL(T1, T2) do { struct pl_ { T1 x; T2 y; }; *s1 = sizeof(T1);              \
        *off2 = offsetof(struct pl_, y); *s2 = sizeof(T2); return 1; } while (0)
    switch (h) {
        case YAKSA_TYPE__FLOAT_INT:
            PL(float, int);
        case YAKSA_TYPE__DOUBLE_INT:
            PL(double, int);
        case YAKSA_TYPE__LONG_INT:
            PL(long, int);
        case YAKSA_TYPE__SHORT_INT:
            PL(short, int);
        case YAKSA_TYPE__LONG_DOUBLE_INT:
            PL(long double, int);
        default:
            return 0;
    }
#undef PL
}

/* yaksi_iov (yaksa_iov.c:48-359): returns entries written at iov[0..) */
static int o_iov(const char *buf, uintptr_t count, const otype * t, uintptr_t off,
                 struct iovec *iov, uintptr_t max, uintptr_t * got)
{
    *got = 0;
    if (max == 0)
        return YAKSA_SUCCESS;
    if (t->is_contig) {         /* :64-73, the offset is not applied */
        iov[0].iov_base = (char *) buf + t->true_lb;
        iov[0].iov_len = count * t->size;
        *got = 1;
        return YAKSA_SUCCESS;
    }
    if (off >= count * t->num_contig)
        return YAKSA_SUCCESS;
    if (t->kind == OK_BUILTIN) {        /* BUILTIN_PAIRTYPE_IOV, :12-46 */
        size_t s1, off2, s2;
        if (!o_pair_layout(t->builtin, &s1, &off2, &s2))
            return YAKSA_ERR__INTERNAL;
        if (off2 == s1) {
            const char *z = buf + off * (uintptr_t) t->extent;
            uintptr_t n = OMIN(max, count - off);
            for (uintptr_t x = 0; x < n; x++, z += t->extent) {
                iov[x].iov_base = (char *) z;
                iov[x].iov_len = s1 + s2;
            }
            *got = n;
        } else {
            if (off % 2)
                return YAKSA_ERR__INTERNAL;
            const char *z = buf + off * (uintptr_t) t->extent / 2;
            uintptr_t n = OMIN(max - 1, count * 2 - off);
            for (uintptr_t x = 0; x < n; x += 2, z += t->extent) {
                iov[x].iov_base = (char *) z;
                iov[x].iov_len = s1;
                iov[x + 1].iov_base = (char *) z + off2;
                iov[x + 1].iov_len = s2;
                *got += 2;
            }
        }
        return YAKSA_SUCCESS;
    }
    if (t->kind == OK_CONTIG)
        return o_iov(buf, count * (uintptr_t) t->count, t->child, off, iov, max, got);

    /* every other kind: a sequence of (address, child count, child) blocks per element */
    uintptr_t rem = max, roff = off;
    struct iovec *out = iov;
    const char *sub0 = t->kind == OK_SUBARRAY ? buf + t->true_lb - t->primary->true_lb : buf;
    intptr_t nblk = (t->kind == OK_RESIZED || t->kind == OK_SUBARRAY) ? 1 : t->count;
    for (uintptr_t i = 0; i < count; i++) {
        for (intptr_t j = 0; j < nblk; j++) {
            const otype *ch;
            uintptr_t n;
            const char *p;
            switch (t->kind) {
                case OK_RESIZED:
                    ch = t->child, n = 1, p = buf + (intptr_t) i * t->extent;
                    break;
                case OK_SUBARRAY:
                    ch = t->primary, n = 1, p = sub0 + (intptr_t) i * t->extent;
                    break;
                case OK_HVECTOR:
                    ch = t->child, n = (uintptr_t) t->blocklength;
                    p = buf + (intptr_t) i * t->extent + j * t->stride;
                    break;
                case OK_BLKHINDX:
                    ch = t->child, n = (uintptr_t) t->blocklength;
                    p = buf + (intptr_t) i * t->extent + t->displs[j];
                    break;
                case OK_HINDEXED:
                    ch = t->child, n = (uintptr_t) t->blens[j];
                    p = buf + (intptr_t) i * t->extent + t->displs[j];
                    break;
                default:       /* OK_STRUCT */
                    ch = t->types[j], n = (uintptr_t) t->blens[j];
                    p = buf + (intptr_t) i * t->extent + t->displs[j];
                    break;
            }
            if (n == 0 && (t->kind == OK_HINDEXED || t->kind == OK_STRUCT))
                continue;
            uintptr_t k = ch->is_contig ? 1 : n * ch->num_contig;
            if (roff >= k) {
                roff -= k;
                continue;
            }
            uintptr_t g;
            int rc = o_iov(p, n, ch, roff, out, rem, &g);
            if (rc)
                return rc;
            out += g;
            rem -= g;
            *got += g;
            roff = 0;
            /* the reference stops at a full list for every kind but subarray,
             * whose loop runs on and lists nothing more (:331-354) */
            if (rem == 0)
                return YAKSA_SUCCESS;
        }
    }
    return YAKSA_SUCCESS;
}

int yaksa_iov(const char *buf, uintptr_t count, yaksa_type_t type, uintptr_t iov_offset,
              struct iovec *iov, uintptr_t max_iov_len, uintptr_t * actual_iov_len)
{
    GET_OR_FAIL(type, t);
    return o_iov(buf, count, t, iov_offset, iov, max_iov_len, actual_iov_len);
}

/* yaksi_iov_len_sub (yaksa_iov_len_max.c:20-148): pieces of the first element that
 * does not fit whole, taken while they fit.  Two deliberate differences, both so that
 * the count agrees with the list yaksa_iov returns: the block length of a contiguous
 * child is the type's own (the reference reads the child's union member, :59-69), and
 * zero-length hindexed/struct blocks are skipped as yaksa_iov skips them. */
static void o_len_sub(const otype * t, uintptr_t * rem, uintptr_t * len)
{
    if (t->num_contig == 1 || t->kind == OK_BUILTIN)
        return;         /* whole elements and whole pieces only */
    switch (t->kind) {
        case OK_CONTIG:
        case OK_HVECTOR:
        case OK_BLKHINDX:
        case OK_HINDEXED:{
                const otype *c = t->child;
                if (c->is_contig) {
                    if (t->kind == OK_HINDEXED) {
                        for (intptr_t i = 0; i < t->count; i++) {
                            uintptr_t sub = c->size * (uintptr_t) t->blens[i];
                            if (t->blens[i] == 0)
                                continue;
                            if (*rem < sub)
                                break;
                            *rem -= sub;
                            *len += 1;
                        }
                    } else {
                        uintptr_t sub = c->size * (uintptr_t) t->blocklength;
                        uintptr_t n = *rem / sub;
                        *rem -= n * sub;
                        *len += n;
                    }
                } else {
                    uintptr_t n = *rem / c->size;
                    *rem -= n * c->size;
                    *len += n * c->num_contig;
                    o_len_sub(c, rem, len);
                }
                return;
            }
        case OK_STRUCT:
            for (intptr_t i = 0; i < t->count; i++) {
                const otype *c = t->types[i];
                uintptr_t n = (uintptr_t) t->blens[i];
                if (n == 0)
                    continue;
                if (c->is_contig) {
                    if (*rem < n * c->size)
                        return;
                    *rem -= n * c->size;
                    *len += 1;
                } else if (*rem >= n * c->size) {
                    *rem -= n * c->size;
                    *len += n * c->num_contig;
                } else {
                    n = *rem / c->size;
                    *rem -= n * c->size;
                    *len += n * c->num_contig;
                    o_len_sub(c, rem, len);
                    return;
                }
            }
            return;
        case OK_RESIZED:
            o_len_sub(t->child, rem, len);
            return;
        case OK_SUBARRAY:
            o_len_sub(t->primary, rem, len);
            return;
    }
}

/* yaksi_iov_len_max (yaksa_iov_len_max.c:151-193) */
int yaksa_iov_len_max(uintptr_t count, yaksa_type_t type, uintptr_t max_iov_bytes,
                      uintptr_t * iov_len, uintptr_t * actual_iov_bytes)
{
    GET_OR_FAIL(type, t);
    if (t->is_contig) {
        int fits = max_iov_bytes >= count * t->size;
        *iov_len = fits;
        *actual_iov_bytes = fits ? count * t->size : 0;
        return YAKSA_SUCCESS;
    }
    if (max_iov_bytes >= count * t->size) {
        *iov_len = count * t->num_contig;
        *actual_iov_bytes = count * t->size;
        return YAKSA_SUCCESS;
    }
    uintptr_t rem = max_iov_bytes, len = 0;
    uintptr_t n = t->size ? rem / t->size : 0;
    rem -= n * t->size;
    len += n * t->num_contig;
    o_len_sub(t, &rem, &len);
    *iov_len = len;
    *actual_iov_bytes = max_iov_bytes - rem;
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* flatten / unflatten: a serialisation of the oracle's own type tree (the      */
/* reference copies its in-memory objects, src/frontend/flatten/); the bytes  */
/* only have to round-trip through this library                               */
/* ------------------------------------------------------------------------- */

static uintptr_t o_flat_size(const otype * t)
{
    uintptr_t n = sizeof(otype);
    switch (t->kind) {
        case OK_CONTIG:
        case OK_RESIZED:
        case OK_HVECTOR:
            return n + o_flat_size(t->child);
        case OK_BLKHINDX:
            return n + t->count * sizeof(intptr_t) + o_flat_size(t->child);
        case OK_HINDEXED:
            return n + 2 * t->count * sizeof(intptr_t) + o_flat_size(t->child);
        case OK_STRUCT:
            n += 2 * t->count * sizeof(intptr_t);
            for (intptr_t i = 0; i < t->count; i++)
                n += o_flat_size(t->types[i]);
            return n;
        case OK_SUBARRAY:
            return n + o_flat_size(t->primary);
        default:
            return n;
    }
}

static char *o_flat_put(const otype * t, char *p)
{
    memcpy(p, t, sizeof(otype));
    p += sizeof(otype);
    if (t->kind == OK_HINDEXED || t->kind == OK_STRUCT) {
        memcpy(p, t->blens, t->count * sizeof(intptr_t));
        p += t->count * sizeof(intptr_t);
    }
    if (t->kind == OK_BLKHINDX || t->kind == OK_HINDEXED || t->kind == OK_STRUCT) {
        memcpy(p, t->displs, t->count * sizeof(intptr_t));
        p += t->count * sizeof(intptr_t);
    }
    if (t->kind == OK_STRUCT) {
        for (intptr_t i = 0; i < t->count; i++)
            p = o_flat_put(t->types[i], p);
        return p;
    }
    if (t->kind == OK_SUBARRAY)
        return o_flat_put(t->primary, p);
    if (t->kind != OK_BUILTIN)
        return o_flat_put(t->child, p);
    return p;
}

static otype *o_flat_get(const char **pp)
{
    otype tmp;
    memcpy(&tmp, *pp, sizeof(otype));
    *pp += sizeof(otype);
    if (tmp.kind == OK_BUILTIN) {
        otype *b = o_get(tmp.builtin);
        o_ref(b);
        return b;
    }
    otype *t = o_new(tmp.kind);
    *t = tmp;
    t->refcount = 1;
    size_t arr = (size_t) t->count * sizeof(intptr_t);
    if (t->kind == OK_HINDEXED || t->kind == OK_STRUCT) {
        t->blens = malloc(arr ? arr : 1);
        memcpy(t->blens, *pp, arr);
        *pp += arr;
    }
    if (t->kind == OK_BLKHINDX || t->kind == OK_HINDEXED || t->kind == OK_STRUCT) {
        t->displs = malloc(arr ? arr : 1);
        memcpy(t->displs, *pp, arr);
        *pp += arr;
    }
    if (t->kind == OK_STRUCT) {
        t->types = malloc((t->count ? t->count : 1) * sizeof(otype *));
        for (intptr_t i = 0; i < t->count; i++)
            t->types[i] = o_flat_get(pp);
    } else if (t->kind == OK_SUBARRAY) {
        t->primary = o_flat_get(pp);
    } else {
        t->child = o_flat_get(pp);
    }
    return t;
}

int yaksa_flatten_size(yaksa_type_t type, uintptr_t * flattened_type_size)
{
    GET_OR_FAIL(type, t);
    *flattened_type_size = o_flat_size(t);
    return YAKSA_SUCCESS;
}

int yaksa_flatten(yaksa_type_t type, void *flattened_type)
{
    GET_OR_FAIL(type, t);
    o_flat_put(t, (char *) flattened_type);
    return YAKSA_SUCCESS;
}

int yaksa_unflatten(yaksa_type_t * type, const void *flattened_type)
{
    const char *p = (const char *) flattened_type;
    *type = o_handle_alloc(o_flat_get(&p));
    return YAKSA_SUCCESS;
}
