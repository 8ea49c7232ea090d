/*
 * yk_types.c -- library init/finalize, handle table, info objects, type
 * constructors and bounds queries of the GB300 engine.
 *
 * Constructor results (size, extent, lb/ub, true bounds, alignment, contiguity,
 * num_contig) and the normalising shortcuts are the reference's, because they are
 * observable through the API:
 *   hvector      src/frontend/types/yaksa_vector.c:11-84  (count 1 -> contig)
 *   contig       src/frontend/types/yaksa_contig.c:11-57  (count 1 -> dup)
 *   dup          src/frontend/types/yaksa_dup.c:11-19
 *   resized      src/frontend/types/yaksa_resized.c:11-50 (same lb/extent -> dup)
 *   blkhindx     src/frontend/types/yaksa_blkindx.c:11-110 (progression from 0 -> hvector)
 *   hindexed     src/frontend/types/yaksa_indexed.c:11-125 (equal lengths -> blkhindx)
 *   struct       src/frontend/types/yaksa_struct.c:11-140 (equal types -> hindexed;
 *                ub padded to the largest alignment)
 *   subarray     src/frontend/types/yaksa_subarray.c:11-119 (primary = resized chain)
 *   builtins     src/frontend/init/yaksa_init.c:148-279 (handle == enum value;
 *                unsigned and C-named types alias the fixed-width objects)
 */
#include <stdlib.h>
#include <string.h>
#include <stddef.h>
#include <wchar.h>
#include <assert.h>
#include "yk_internal.h"

pthread_mutex_t yk_global_mutex = PTHREAD_MUTEX_INITIALIZER;
static pthread_mutex_t yk_init_mutex = PTHREAD_MUTEX_INITIALIZER;
static int yk_init_refs = 0;

/* handle table: slot i holds the object of handle i (builtins at their enum values) */
static yk_type **yk_slots = NULL;
static size_t yk_nslots = 0, yk_capslots = 0;
static size_t yk_free_hint = YAKSA_TYPE__LONG_DOUBLE_INT + 1;

int yk_is_initialized(void)
{
    return __atomic_load_n(&yk_init_refs, __ATOMIC_ACQUIRE) > 0;
}

static yaksa_type_t slot_insert(yk_type * t)
{
    pthread_mutex_lock(&yk_global_mutex);
    size_t id = yk_nslots;
    for (size_t i = yk_free_hint; i < yk_nslots; i++)
        if (!yk_slots[i]) {
            id = i;
            break;
        }
    if (id == yk_nslots) {
        if (yk_nslots == yk_capslots) {
            size_t nc = yk_capslots ? 2 * yk_capslots : 1024;
            yk_type **ns = realloc(yk_slots, nc * sizeof(*ns));
            if (!ns) {
                pthread_mutex_unlock(&yk_global_mutex);
                return (yaksa_type_t) - 1;
            }
            yk_slots = ns;
            yk_capslots = nc;
        }
        yk_nslots++;
    }
    yk_slots[id] = t;
    yk_free_hint = id + 1;
    pthread_mutex_unlock(&yk_global_mutex);
    return (yaksa_type_t) id;
}

yk_type *yk_type_get(yaksa_type_t h)
{
    uint64_t id = h & 0xffffffffull;
    pthread_mutex_lock(&yk_global_mutex);
    yk_type *t = id < yk_nslots ? yk_slots[id] : NULL;
    pthread_mutex_unlock(&yk_global_mutex);
    return t;
}

void yk_type_ref(yk_type * t)
{
    __atomic_add_fetch(&t->refcount, 1, __ATOMIC_ACQ_REL);
}

void yk_type_unref(yk_type * t)
{
    if (__atomic_sub_fetch(&t->refcount, 1, __ATOMIC_ACQ_REL))
        return;
    yk_desc_release(t);
    if (t->child)
        yk_type_unref(t->child);
    if (t->primary)
        yk_type_unref(t->primary);
    if (t->types) {
        for (intptr_t i = 0; i < t->count; i++)
            yk_type_unref(t->types[i]);
        free(t->types);
    }
    free(t->blens);
    free(t->displs);
    pthread_mutex_destroy(&t->desc_mutex);
    free(t);
}

static yk_type *type_new(int kind)
{
    yk_type *t = calloc(1, sizeof(yk_type));
    if (!t)
        return NULL;
    t->refcount = 1;
    t->kind = kind;
    pthread_mutex_init(&t->desc_mutex, NULL);
    return t;
}

/* ------------------------------------------------------------------------- */
/* builtins                                                                  */
/* ------------------------------------------------------------------------- */

int yk_base_type_size(int bt)
{
    switch (bt) {
        case YK_BT_BOOL:
            return sizeof(_Bool);
        case YK_BT_CHAR:
        case YK_BT_I8:
            return 1;
        case YK_BT_WCHAR:
            return sizeof(wchar_t);
        case YK_BT_I16:
            return 2;
        case YK_BT_I32:
        case YK_BT_F32:
            return 4;
        case YK_BT_I64:
        case YK_BT_F64:
        case YK_BT_C32:
            return 8;
        case YK_BT_C64:
            return 16;
        case YK_BT_LDOUBLE:
            return sizeof(long double);
        case YK_BT_CLDOUBLE:
            return 2 * sizeof(long double);
        default:
            return 1;
    }
}

/* base type of a non-pair builtin object (by the handle it was created under) */
int yk_builtin_base_type(yaksa_type_t h)
{
    switch (h) {
        case YAKSA_TYPE___BOOL:
            return YK_BT_BOOL;
        case YAKSA_TYPE__CHAR:
            return YK_BT_CHAR;
        case YAKSA_TYPE__WCHAR_T:
            return YK_BT_WCHAR;
        case YAKSA_TYPE__INT8_T:
            return YK_BT_I8;
        case YAKSA_TYPE__INT16_T:
            return YK_BT_I16;
        case YAKSA_TYPE__INT32_T:
            return YK_BT_I32;
        case YAKSA_TYPE__INT64_T:
            return YK_BT_I64;
        case YAKSA_TYPE__FLOAT:
            return YK_BT_F32;
        case YAKSA_TYPE__DOUBLE:
            return YK_BT_F64;
        case YAKSA_TYPE__LONG_DOUBLE:
            return YK_BT_LDOUBLE;
        case YAKSA_TYPE__C_COMPLEX:
            return YK_BT_C32;
        case YAKSA_TYPE__C_DOUBLE_COMPLEX:
            return YK_BT_C64;
        case YAKSA_TYPE__C_LONG_DOUBLE_COMPLEX:
            return YK_BT_CLDOUBLE;
        default:
            return -1;  /* pair types: field by field */
    }
}

static int int_bt(size_t sz)
{
    return sz == 1 ? YK_BT_I8 : sz == 2 ? YK_BT_I16 : sz == 4 ? YK_BT_I32 : YK_BT_I64;
}

static yk_type *mk_scalar(yaksa_type_t h, size_t size, size_t align)
{
    yk_type *t = type_new(YK_K_BUILTIN);
    t->builtin = h;
    t->size = size;
    t->alignment = (int) align;
    t->extent = t->ub = t->true_ub = (intptr_t) size;
    t->is_contig = true;
    t->num_contig = 1;
    t->base_type = yk_builtin_base_type(h);
    t->builtin_size = size;
    t->needs_host_ops = (t->base_type == YK_BT_LDOUBLE || t->base_type == YK_BT_CLDOUBLE);
    return t;
}

/* pair types: size is the sum of the fields, extent the C struct's size
 * (yaksa_init.c:83-122) */
static yk_type *mk_pairtype(yaksa_type_t h, size_t s1, size_t a1, int bt1, size_t s2, size_t a2,
                            int bt2, size_t off2, size_t ssize)
{
    yk_type *t = type_new(YK_K_BUILTIN);
    bool elem_contig = (off2 == s1);
    t->builtin = h;
    t->size = s1 + s2;
    t->alignment = (int) YK_MAX(a1, a2);
    t->extent = t->ub = (intptr_t) ssize;
    t->true_ub = elem_contig ? (intptr_t) t->size : (intptr_t) ssize;
    t->is_contig = (t->size == ssize);
    t->num_contig = 1 + !elem_contig;
    if (bt1 == bt2 && (h == YAKSA_TYPE__C_COMPLEX || h == YAKSA_TYPE__C_DOUBLE_COMPLEX ||
                       h == YAKSA_TYPE__C_LONG_DOUBLE_COMPLEX))
        t->base_type = yk_builtin_base_type(h);
    else
        t->base_type = (bt1 == bt2) ? bt1 : -1;
    t->builtin_size = t->size;
    t->needs_host_ops = (bt1 == YK_BT_LDOUBLE || bt2 == YK_BT_LDOUBLE ||
                         bt1 == YK_BT_CLDOUBLE);
    return t;
}

#define ADD_SCALAR(H, T) \
    do { if (slot_insert(mk_scalar(H, sizeof(T), _Alignof(T))) != (H)) goto fail; } while (0)
#define ADD_PAIR(H, T1, B1, T2, B2) do {                                              \
        struct p_ { T1 x; T2 y; };                                                    \
        if (slot_insert(mk_pairtype(H, sizeof(T1), _Alignof(T1), B1, sizeof(T2),      \
                        _Alignof(T2), B2, offsetof(struct p_, y), sizeof(struct p_))) != (H)) \
            goto fail;                                                                \
    } while (0)

static int add_alias(yaksa_type_t target, yaksa_type_t h)
{
    yk_type *t = yk_type_get(target);
    yk_type_ref(t);
    return slot_insert(t) == h ? 0 : -1;
}

static int add_int_alias(size_t sz, yaksa_type_t h)
{
    static const yaksa_type_t fixed[] = { 0, YAKSA_TYPE__INT8_T, YAKSA_TYPE__INT16_T, 0,
        YAKSA_TYPE__INT32_T, 0, 0, 0, YAKSA_TYPE__INT64_T
    };
    return add_alias(fixed[sz], h);
}

int yaksa_init(yaksa_info_t info)
{
    int rc = YAKSA_SUCCESS;
    pthread_mutex_lock(&yk_init_mutex);
    if (yk_init_refs > 0) {
        __atomic_add_fetch(&yk_init_refs, 1, __ATOMIC_ACQ_REL);
        pthread_mutex_unlock(&yk_init_mutex);
        return YAKSA_SUCCESS;
    }
    yk_nslots = 0;
    yk_free_hint = YAKSA_TYPE__LONG_DOUBLE_INT + 1;

    yk_type *null_t = mk_scalar(YAKSA_TYPE__NULL, 0, 1);
    null_t->num_contig = 0;
    null_t->base_type = YK_BT_NONE;
    if (slot_insert(null_t) != YAKSA_TYPE__NULL)
        goto fail;
    ADD_SCALAR(YAKSA_TYPE___BOOL, _Bool);
    ADD_SCALAR(YAKSA_TYPE__CHAR, char);
    if (add_alias(YAKSA_TYPE__CHAR, YAKSA_TYPE__SIGNED_CHAR) ||
        add_alias(YAKSA_TYPE__CHAR, YAKSA_TYPE__UNSIGNED_CHAR))
        goto fail;
    ADD_SCALAR(YAKSA_TYPE__WCHAR_T, wchar_t);
    ADD_SCALAR(YAKSA_TYPE__INT8_T, int8_t);
    ADD_SCALAR(YAKSA_TYPE__INT16_T, int16_t);
    ADD_SCALAR(YAKSA_TYPE__INT32_T, int32_t);
    ADD_SCALAR(YAKSA_TYPE__INT64_T, int64_t);
    {
        /* the remaining integer handles in enum order, each with its C size */
        static const struct { yaksa_type_t h; size_t sz; } ints[] = {
            {YAKSA_TYPE__UINT8_T, 1}, {YAKSA_TYPE__UINT16_T, 2}, {YAKSA_TYPE__UINT32_T, 4},
            {YAKSA_TYPE__UINT64_T, 8}, {YAKSA_TYPE__INT, sizeof(int)},
            {YAKSA_TYPE__UNSIGNED, sizeof(unsigned)}, {YAKSA_TYPE__SHORT, sizeof(short)},
            {YAKSA_TYPE__UNSIGNED_SHORT, sizeof(unsigned short)},
            {YAKSA_TYPE__LONG, sizeof(long)}, {YAKSA_TYPE__UNSIGNED_LONG, sizeof(unsigned long)},
            {YAKSA_TYPE__LONG_LONG, sizeof(long long)},
            {YAKSA_TYPE__UNSIGNED_LONG_LONG, sizeof(unsigned long long)},
            {YAKSA_TYPE__INT_FAST8_T, sizeof(int_fast8_t)},
            {YAKSA_TYPE__INT_FAST16_T, sizeof(int_fast16_t)},
            {YAKSA_TYPE__INT_FAST32_T, sizeof(int_fast32_t)},
            {YAKSA_TYPE__INT_FAST64_T, sizeof(int_fast64_t)},
            {YAKSA_TYPE__UINT_FAST8_T, sizeof(uint_fast8_t)},
            {YAKSA_TYPE__UINT_FAST16_T, sizeof(uint_fast16_t)},
            {YAKSA_TYPE__UINT_FAST32_T, sizeof(uint_fast32_t)},
            {YAKSA_TYPE__UINT_FAST64_T, sizeof(uint_fast64_t)},
            {YAKSA_TYPE__INT_LEAST8_T, sizeof(int_least8_t)},
            {YAKSA_TYPE__INT_LEAST16_T, sizeof(int_least16_t)},
            {YAKSA_TYPE__INT_LEAST32_T, sizeof(int_least32_t)},
            {YAKSA_TYPE__INT_LEAST64_T, sizeof(int_least64_t)},
            {YAKSA_TYPE__UINT_LEAST8_T, sizeof(uint_least8_t)},
            {YAKSA_TYPE__UINT_LEAST16_T, sizeof(uint_least16_t)},
            {YAKSA_TYPE__UINT_LEAST32_T, sizeof(uint_least32_t)},
            {YAKSA_TYPE__UINT_LEAST64_T, sizeof(uint_least64_t)},
            {YAKSA_TYPE__BYTE, 1}, {YAKSA_TYPE__INTMAX_T, sizeof(intmax_t)},
            {YAKSA_TYPE__UINTMAX_T, sizeof(uintmax_t)}, {YAKSA_TYPE__SIZE_T, sizeof(size_t)},
            {YAKSA_TYPE__INTPTR_T, sizeof(intptr_t)}, {YAKSA_TYPE__UINTPTR_T, sizeof(uintptr_t)},
            {YAKSA_TYPE__PTRDIFF_T, sizeof(ptrdiff_t)},
        };
        for (size_t i = 0; i < sizeof(ints) / sizeof(ints[0]); i++)
            if (add_int_alias(ints[i].sz, ints[i].h))
                goto fail;
    }
    ADD_SCALAR(YAKSA_TYPE__FLOAT, float);
    ADD_SCALAR(YAKSA_TYPE__DOUBLE, double);
    ADD_SCALAR(YAKSA_TYPE__LONG_DOUBLE, long double);
    ADD_PAIR(YAKSA_TYPE__C_COMPLEX, float, YK_BT_F32, float, YK_BT_F32);
    ADD_PAIR(YAKSA_TYPE__C_DOUBLE_COMPLEX, double, YK_BT_F64, double, YK_BT_F64);
    ADD_PAIR(YAKSA_TYPE__C_LONG_DOUBLE_COMPLEX, long double, YK_BT_LDOUBLE, long double,
             YK_BT_LDOUBLE);
    ADD_PAIR(YAKSA_TYPE__FLOAT_INT, float, YK_BT_F32, int, int_bt(sizeof(int)));
    ADD_PAIR(YAKSA_TYPE__DOUBLE_INT, double, YK_BT_F64, int, int_bt(sizeof(int)));
    ADD_PAIR(YAKSA_TYPE__LONG_INT, long, int_bt(sizeof(long)), int, int_bt(sizeof(int)));
    ADD_PAIR(YAKSA_TYPE__2INT, int, int_bt(sizeof(int)), int, int_bt(sizeof(int)));
    ADD_PAIR(YAKSA_TYPE__SHORT_INT, short, int_bt(sizeof(short)), int, int_bt(sizeof(int)));
    ADD_PAIR(YAKSA_TYPE__LONG_DOUBLE_INT, long double, YK_BT_LDOUBLE, int, int_bt(sizeof(int)));

    rc = yk_runtime_init(info ? ((yk_info *) info)->has_wait_kernel : 0);
    if (rc)
        goto fail_unlocked_rc;
    __atomic_store_n(&yk_init_refs, 1, __ATOMIC_RELEASE);
    pthread_mutex_unlock(&yk_init_mutex);
    return YAKSA_SUCCESS;

  fail:
    rc = YAKSA_ERR__INTERNAL;
  fail_unlocked_rc:
    pthread_mutex_unlock(&yk_init_mutex);
    return rc;
}

int yaksa_finalize(void)
{
    pthread_mutex_lock(&yk_init_mutex);
    if (yk_init_refs > 1) {
        __atomic_sub_fetch(&yk_init_refs, 1, __ATOMIC_ACQ_REL);
        pthread_mutex_unlock(&yk_init_mutex);
        return YAKSA_SUCCESS;
    }
    if (yk_init_refs == 0) {
        pthread_mutex_unlock(&yk_init_mutex);
        return YAKSA_SUCCESS;
    }
    yk_runtime_finalize();
    for (size_t i = 0; i <= YAKSA_TYPE__LONG_DOUBLE_INT && i < yk_nslots; i++) {
        yk_type *t = yk_slots[i];
        yk_slots[i] = NULL;
        if (t)
            yk_type_unref(t);
    }
    pthread_mutex_lock(&yk_global_mutex);
    yk_nslots = 0;
    pthread_mutex_unlock(&yk_global_mutex);
    __atomic_store_n(&yk_init_refs, 0, __ATOMIC_RELEASE);
    pthread_mutex_unlock(&yk_init_mutex);
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* info objects (yaksa_info.c:12-64; keys: yaksur_hooks.c:314-341,            */
/* seq/hooks/yaksuri_seq_hooks.c:80-86, cuda/hooks/yaksuri_cudai_info_hooks.c) */
/* ------------------------------------------------------------------------- */

int yaksa_info_create(yaksa_info_t * info)
{
    yk_info *i = calloc(1, sizeof(yk_info));
    if (!i)
        return YAKSA_ERR__OUT_OF_MEM;
    i->refcount = 1;
    i->mapped_device = -1;
    i->iov_pack_threshold = i->iov_unpack_threshold = 16384;
    *info = i;
    return YAKSA_SUCCESS;
}

int yaksa_info_free(yaksa_info_t info)
{
    yk_info *i = info;
    if (i && __atomic_sub_fetch(&i->refcount, 1, __ATOMIC_ACQ_REL) == 0)
        free(i);
    return YAKSA_SUCCESS;
}

int yaksa_info_keyval_append(yaksa_info_t info, const char *key, const void *val,
                             unsigned int vallen)
{
    yk_info *i = info;
    if (!i || !key)
        return YAKSA_ERR__INTERNAL;
    if (!strncmp(key, "yaksa_gpu_driver", YAKSA_INFO_MAX_KEYLEN)) {
        if (!strncmp(val, "nogpu", vallen))
            i->gpu_driver = 2;
        else if (!strncmp(val, "cuda", vallen))
            i->gpu_driver = 1;
        else
            return YAKSA_ERR__NOT_SUPPORTED;    /* ze / hip drivers do not exist here */
    } else if (!strncmp(key, "yaksa_mapped_device", YAKSA_INFO_MAX_KEYLEN)) {
        if (vallen != sizeof(int))
            return YAKSA_ERR__INTERNAL;
        memcpy(&i->mapped_device, val, sizeof(int));
    } else if (!strcmp(key, "yaksa_has_wait_kernel")) {
        const char *v = val;
        i->has_wait_kernel = !strcmp(v, "true") || !strcmp(v, "yes") || !strcmp(v, "1");
    } else if (!strcmp(key, "yaksa_seq_iov_pack_threshold") ||
               !strcmp(key, "yaksa_cuda_iov_pack_threshold")) {
        /* the reference stores the pointer value here (yaksuri_seq_hooks.c:82); this
         * library reads the uintptr_t the pointer refers to */
        if (vallen == sizeof(uintptr_t))
            memcpy(&i->iov_pack_threshold, val, sizeof(uintptr_t));
    } else if (!strcmp(key, "yaksa_seq_iov_unpack_threshold") ||
               !strcmp(key, "yaksa_cuda_iov_unpack_threshold")) {
        if (vallen == sizeof(uintptr_t))
            memcpy(&i->iov_unpack_threshold, val, sizeof(uintptr_t));
    }
    /* other keys (pointer-attribute injection hints) are accepted and ignored */
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* constructors                                                              */
/* ------------------------------------------------------------------------- */

static yk_type *make_contig(intptr_t count, yk_type * in);

static yk_type *make_dup(yk_type * in)
{
    yk_type_ref(in);
    return in;
}

/* GPU-side derived fields shared by every single-child constructor */
static void inherit(yk_type * t, yk_type * in)
{
    t->base_type = in->base_type;
    t->builtin_size = in->builtin_size;
    t->needs_host_ops = in->needs_host_ops;
}

/* lb/ub of `n` consecutive children placed at `disp` (extent may be negative) */
static void child_block_bounds(yk_type * c, intptr_t disp, intptr_t n, intptr_t * lb,
                               intptr_t * ub)
{
    if (c->extent > 0) {
        *lb = disp + c->lb;
        *ub = disp + c->ub + c->extent * (n - 1);
    } else {
        *lb = disp + c->lb + c->extent * (n - 1);
        *ub = disp + c->ub;
    }
}

static yk_type *make_hvector(intptr_t count, intptr_t bl, intptr_t stride, yk_type * in)
{
    if (count == 1)
        return make_contig(bl, in);
    yk_type *t = type_new(YK_K_HVECTOR);
    if (!t)
        return NULL;
    yk_type_ref(in);
    inherit(t, in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size * bl * count;
    t->alignment = in->alignment;
    intptr_t span_lb, span_ub;
    child_block_bounds(in, 0, bl, &span_lb, &span_ub);
    t->lb = span_lb + (stride < 0 ? stride * (count - 1) : 0);
    t->ub = span_ub + (stride > 0 ? stride * (count - 1) : 0);
    t->true_lb = t->lb + in->true_lb - in->lb;
    t->true_ub = t->ub - in->ub + in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = in->is_contig && t->extent == (intptr_t) t->size && stride > 0;
    t->num_contig = t->is_contig ? 1 :
        in->is_contig ? count * in->num_contig : count * bl * in->num_contig;
    t->count = count;
    t->blocklength = bl;
    t->stride = stride;
    t->child = in;
    return t;
}

static yk_type *make_contig(intptr_t count, yk_type * in)
{
    if (count == 1)
        return make_dup(in);
    yk_type *t = type_new(YK_K_CONTIG);
    if (!t)
        return NULL;
    yk_type_ref(in);
    inherit(t, in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size * count;
    t->alignment = in->alignment;
    child_block_bounds(in, 0, count, &t->lb, &t->ub);
    t->true_lb = t->lb + in->true_lb - in->lb;
    t->true_ub = t->ub - in->ub + in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = in->is_contig;
    t->num_contig = t->is_contig ? 1 : count * in->num_contig;
    t->count = count;
    t->child = in;
    return t;
}

static yk_type *make_resized(yk_type * in, intptr_t lb, intptr_t extent)
{
    if (lb == in->lb && extent == in->extent)
        return make_dup(in);
    yk_type *t = type_new(YK_K_RESIZED);
    if (!t)
        return NULL;
    yk_type_ref(in);
    inherit(t, in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size;
    t->alignment = in->alignment;
    t->lb = lb;
    t->ub = lb + extent;
    t->true_lb = in->true_lb;
    t->true_ub = in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = in->is_contig && t->extent == (intptr_t) t->size;
    t->num_contig = in->num_contig;
    t->child = in;
    return t;
}

static yk_type *make_blkhindx(intptr_t count, intptr_t bl, const intptr_t * displs, yk_type * in)
{
    bool progression = (displs[0] == 0);
    for (intptr_t i = 2; i < count && progression; i++)
        progression = (displs[i] - displs[i - 1] == displs[1] - displs[0]);
    if (progression)
        return make_hvector(count, bl, count > 1 ? displs[1] - displs[0] : 0, in);

    yk_type *t = type_new(YK_K_BLKHINDX);
    if (!t)
        return NULL;
    yk_type_ref(in);
    inherit(t, in);
    t->tree_depth = in->tree_depth + 1;
    t->size = in->size * bl * count;
    t->alignment = in->alignment;
    intptr_t dmin = displs[0], dmax = displs[0];
    for (intptr_t i = 1; i < count; i++) {
        dmin = YK_MIN(dmin, displs[i]);
        dmax = YK_MAX(dmax, displs[i]);
    }
    intptr_t lb0, ub0;
    child_block_bounds(in, 0, bl, &lb0, &ub0);
    t->lb = dmin + lb0;
    t->ub = dmax + ub0;
    t->true_lb = t->lb + in->true_lb - in->lb;
    t->true_ub = t->ub - in->ub + in->true_ub;
    t->extent = t->ub - t->lb;
    t->is_contig = in->is_contig && t->extent == (intptr_t) t->size;
    for (intptr_t i = 1; i < count && t->is_contig; i++)
        t->is_contig = (displs[i] == displs[i - 1] + in->extent * bl);
    t->num_contig = t->is_contig ? 1 :
        in->is_contig ? in->num_contig * count : in->num_contig * count * bl;
    t->count = count;
    t->blocklength = bl;
    t->displs = malloc(count * sizeof(intptr_t));
    memcpy(t->displs, displs, count * sizeof(intptr_t));
    t->child = in;
    return t;
}

static yk_type *make_hindexed(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                              yk_type * in)
{
    bool equal = true;
    for (intptr_t i = 1; i < count && equal; i++)
        equal = (blens[i] == blens[i - 1]);
    if (equal)
        return make_blkhindx(count, blens[0], displs, in);

    yk_type *t = type_new(YK_K_HINDEXED);
    if (!t)
        return NULL;
    yk_type_ref(in);
    inherit(t, in);
    t->tree_depth = in->tree_depth + 1;
    t->alignment = in->alignment;
    bool have = false, gap = false;
    intptr_t prev_ub = 0;
    uintptr_t nonempty = 0, total_blocks = 0;
    for (intptr_t i = 0; i < count; i++) {
        t->size += in->size * blens[i];
        total_blocks += blens[i];
        if (!blens[i])
            continue;
        nonempty++;
        intptr_t lb, ub;
        child_block_bounds(in, displs[i], blens[i], &lb, &ub);
        if (i > 0 && lb != prev_ub)
            gap = true;
        prev_ub = ub;
        intptr_t tlb = lb - in->lb + in->true_lb, tub = ub - in->ub + in->true_ub;
        t->lb = have ? YK_MIN(lb, t->lb) : lb;
        t->ub = have ? YK_MAX(ub, t->ub) : ub;
        t->true_lb = have ? YK_MIN(tlb, t->true_lb) : tlb;
        t->true_ub = have ? YK_MAX(tub, t->true_ub) : tub;
        have = true;
    }
    t->extent = t->ub - t->lb;
    t->is_contig = !gap && in->is_contig && t->extent == (intptr_t) t->size;
    t->num_contig = t->is_contig ? 1 :
        in->is_contig ? in->num_contig * nonempty : in->num_contig * total_blocks;
    t->count = count;
    t->blens = malloc(count * sizeof(intptr_t));
    t->displs = malloc(count * sizeof(intptr_t));
    memcpy(t->blens, blens, count * sizeof(intptr_t));
    memcpy(t->displs, displs, count * sizeof(intptr_t));
    t->child = in;
    return t;
}

static yk_type *make_struct(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                            yk_type ** types)
{
    bool same = true;
    for (intptr_t i = 1; i < count && same; i++)
        same = (types[i] == types[i - 1]);
    if (same)
        return make_hindexed(count, blens, displs, types[0]);

    yk_type *t = type_new(YK_K_STRUCT);
    if (!t)
        return NULL;
    bool have = false, gap = false;
    intptr_t prev_true_ub = 0;
    t->base_type = -2;  /* unset */
    t->builtin_size = (uintptr_t) - 1;
    for (intptr_t i = 0; i < count; i++) {
        yk_type *c = types[i];
        yk_type_ref(c);
        t->size += c->size * blens[i];
        t->needs_host_ops |= c->needs_host_ops;
        if (!blens[i])
            continue;
        t->base_type = (t->base_type == -2 || t->base_type == c->base_type) ? c->base_type : -1;
        t->builtin_size = (t->builtin_size == (uintptr_t) - 1 ||
                           t->builtin_size == c->builtin_size) ? c->builtin_size : 0;
        intptr_t lb, ub;
        child_block_bounds(c, displs[i], blens[i], &lb, &ub);
        intptr_t tlb = lb - c->lb + c->true_lb, tub = ub - c->ub + c->true_ub;
        if (i > 0 && tlb != prev_true_ub)
            gap = true;
        prev_true_ub = tub;
        t->alignment = YK_MAX(t->alignment, c->alignment);
        t->lb = have ? YK_MIN(lb, t->lb) : lb;
        t->ub = have ? YK_MAX(ub, t->ub) : ub;
        t->true_lb = have ? YK_MIN(tlb, t->true_lb) : tlb;
        t->true_ub = have ? YK_MAX(tub, t->true_ub) : tub;
        t->tree_depth = have ? YK_MAX(c->tree_depth, t->tree_depth) : c->tree_depth;
        have = true;
    }
    if (t->base_type == -2)
        t->base_type = -1;
    if (t->builtin_size == (uintptr_t) - 1)
        t->builtin_size = 0;
    if (t->alignment > 0) {
        uintptr_t rem = (uintptr_t) (t->ub - t->lb) % (uintptr_t) t->alignment;
        if (rem)
            t->ub += t->alignment - rem;
    }
    t->tree_depth++;
    t->extent = t->ub - t->lb;
    t->is_contig = !gap && t->extent == (intptr_t) t->size;
    for (intptr_t i = 0; i < count && t->is_contig; i++)
        t->is_contig = types[i]->is_contig;
    if (t->is_contig && t->ub == t->extent) {
        t->num_contig = 1;
    } else {
        for (intptr_t i = 0; i < count; i++)
            t->num_contig += (types[i]->is_contig && blens[i]) ? 1 :
                types[i]->num_contig * blens[i];
    }
    t->count = count;
    t->blens = malloc(count * sizeof(intptr_t));
    t->displs = malloc(count * sizeof(intptr_t));
    t->types = malloc(count * sizeof(yk_type *));
    memcpy(t->blens, blens, count * sizeof(intptr_t));
    memcpy(t->displs, displs, count * sizeof(intptr_t));
    memcpy(t->types, types, count * sizeof(yk_type *));
    return t;
}

static yk_type *make_subarray(int ndims, const intptr_t * sizes, const intptr_t * subsizes,
                              const intptr_t * starts, yaksa_subarray_order_e order, yk_type * in)
{
    yk_type *t = type_new(YK_K_SUBARRAY);
    if (!t)
        return NULL;
    inherit(t, in);
    t->tree_depth = in->tree_depth + 1;
    t->alignment = in->alignment;
    t->ndims = ndims;
    /* dimension visiting order: fastest-varying dimension first */
    int fast = (order == YAKSA_SUBARRAY_ORDER__C) ? ndims - 1 : 0;
    int step = (order == YAKSA_SUBARRAY_ORDER__C) ? -1 : 1;
    yk_type *cur = make_contig(subsizes[fast], in);
    intptr_t stride = in->extent;
    for (int k = 1; k < ndims; k++) {
        int dim = fast + step * k;
        stride *= sizes[dim - step];
        yk_type *next = make_hvector(subsizes[dim], 1, stride, cur);
        yk_type_unref(cur);
        cur = next;
    }
    intptr_t extent = in->extent;
    for (int i = 0; i < ndims; i++)
        extent *= sizes[i];
    t->primary = make_resized(cur, 0, extent);
    yk_type_unref(cur);
    t->lb = 0;
    t->ub = t->extent = extent;
    t->size = in->size;
    t->true_lb = in->true_lb;
    t->true_ub = in->true_ub;
    for (int i = 0; i < ndims; i++) {
        t->size *= subsizes[i];
        intptr_t scale = in->extent;
        if (order == YAKSA_SUBARRAY_ORDER__C) {
            for (int j = i + 1; j < ndims; j++)
                scale *= sizes[j];
        } else {
            for (int j = 0; j < i; j++)
                scale *= sizes[j];
        }
        t->true_lb += starts[i] * scale;
        t->true_ub += (starts[i] + subsizes[i] - 1) * scale;
    }
    t->is_contig = in->is_contig && t->extent == (intptr_t) t->size;
    t->num_contig = t->primary->num_contig;
    return t;
}

/* ------------------------------------------------------------------------- */
/* public constructors                                                       */
/* ------------------------------------------------------------------------- */

#define LOOKUP(h, var) yk_type *var = yk_type_get(h); if (!var) return YAKSA_ERR__INTERNAL

static int publish(yk_type * t, yaksa_type_t * newtype)
{
    if (!t)
        return YAKSA_ERR__OUT_OF_MEM;
    yaksa_type_t h = slot_insert(t);
    if (h == (yaksa_type_t) - 1) {
        yk_type_unref(t);
        return YAKSA_ERR__OUT_OF_MEM;
    }
    *newtype = h;
    return YAKSA_SUCCESS;
}

#define EMPTY_RESULT() do { *newtype = YAKSA_TYPE__NULL; return YAKSA_SUCCESS; } while (0)

int yaksa_type_create_hvector(intptr_t count, intptr_t bl, intptr_t stride, yaksa_type_t old,
                              yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (count * (intptr_t) in->size == 0)
        EMPTY_RESULT();
    return publish(make_hvector(count, bl, stride, in), newtype);
}

int yaksa_type_create_vector(intptr_t count, intptr_t bl, intptr_t stride, yaksa_type_t old,
                             yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (count * (intptr_t) in->size == 0)
        EMPTY_RESULT();
    return publish(make_hvector(count, bl, stride * in->extent, in), newtype);
}

int yaksa_type_create_contig(intptr_t count, yaksa_type_t old, yaksa_info_t info,
                             yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (count * (intptr_t) in->size == 0)
        EMPTY_RESULT();
    return publish(make_contig(count, in), newtype);
}

int yaksa_type_create_dup(yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    return publish(make_dup(in), newtype);
}

int yaksa_type_create_hindexed_block(intptr_t count, intptr_t bl, const intptr_t * displs,
                                     yaksa_type_t old, yaksa_info_t info,
                                     yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (count * (intptr_t) in->size == 0)
        EMPTY_RESULT();
    return publish(make_blkhindx(count, bl, displs, in), newtype);
}

int yaksa_type_create_indexed_block(intptr_t count, intptr_t bl, const intptr_t * displs,
                                    yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (count * (intptr_t) in->size == 0)
        EMPTY_RESULT();
    intptr_t *bytes = malloc(count * sizeof(intptr_t));
    if (!bytes)
        return YAKSA_ERR__OUT_OF_MEM;
    for (intptr_t i = 0; i < count; i++)
        bytes[i] = displs[i] * in->extent;
    int rc = publish(make_blkhindx(count, bl, bytes, in), newtype);
    free(bytes);
    return rc;
}

static uintptr_t total_bytes(intptr_t count, const intptr_t * blens, yk_type * in)
{
    uintptr_t s = 0;
    for (intptr_t i = 0; i < count; i++)
        s += in->size * blens[i];
    return s;
}

int yaksa_type_create_hindexed(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                               yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (total_bytes(count, blens, in) == 0)
        EMPTY_RESULT();
    return publish(make_hindexed(count, blens, displs, in), newtype);
}

int yaksa_type_create_indexed(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                              yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (total_bytes(count, blens, in) == 0)
        EMPTY_RESULT();
    intptr_t *bytes = malloc(count * sizeof(intptr_t));
    if (!bytes)
        return YAKSA_ERR__OUT_OF_MEM;
    for (intptr_t i = 0; i < count; i++)
        bytes[i] = displs[i] * in->extent;
    int rc = publish(make_hindexed(count, blens, bytes, in), newtype);
    free(bytes);
    return rc;
}

int yaksa_type_create_resized(yaksa_type_t old, intptr_t lb, intptr_t extent,
                              yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    return publish(make_resized(in, lb, extent), newtype);
}

int yaksa_type_create_struct(intptr_t count, const intptr_t * blens, const intptr_t * displs,
                             const yaksa_type_t * types, yaksa_info_t info,
                             yaksa_type_t * newtype)
{
    (void) info;
    uintptr_t total = 0;
    for (intptr_t i = 0; i < count; i++) {
        LOOKUP(types[i], c);
        total += c->size * blens[i];
    }
    if (total == 0)
        EMPTY_RESULT();
    yk_type **in = malloc(count * sizeof(yk_type *));
    if (!in)
        return YAKSA_ERR__OUT_OF_MEM;
    for (intptr_t i = 0; i < count; i++)
        in[i] = yk_type_get(types[i]);
    int rc = publish(make_struct(count, blens, displs, in), newtype);
    free(in);
    return rc;
}

int yaksa_type_create_subarray(int ndims, const intptr_t * sizes, const intptr_t * subsizes,
                               const intptr_t * starts, yaksa_subarray_order_e order,
                               yaksa_type_t old, yaksa_info_t info, yaksa_type_t * newtype)
{
    (void) info;
    LOOKUP(old, in);
    if (ndims * (intptr_t) in->size == 0)
        EMPTY_RESULT();
    return publish(make_subarray(ndims, sizes, subsizes, starts, order, in), newtype);
}

int yaksa_type_get_size(yaksa_type_t type, uintptr_t * size)
{
    LOOKUP(type, t);
    *size = t->size;
    return YAKSA_SUCCESS;
}

int yaksa_type_get_extent(yaksa_type_t type, intptr_t * lb, intptr_t * extent)
{
    LOOKUP(type, t);
    *lb = t->lb;
    *extent = t->extent;
    return YAKSA_SUCCESS;
}

int yaksa_type_get_true_extent(yaksa_type_t type, intptr_t * lb, intptr_t * extent)
{
    LOOKUP(type, t);
    *lb = t->true_lb;
    *extent = t->true_ub - t->true_lb;
    return YAKSA_SUCCESS;
}

int yaksa_type_free(yaksa_type_t type)
{
    uint64_t id = type & 0xffffffffull;
    if (id <= YAKSA_TYPE__LONG_DOUBLE_INT)
        return YAKSA_SUCCESS;   /* builtin objects live until finalize */
    pthread_mutex_lock(&yk_global_mutex);
    yk_type *t = id < yk_nslots ? yk_slots[id] : NULL;
    if (t) {
        yk_slots[id] = NULL;
        if (id < yk_free_hint)
            yk_free_hint = id;
    }
    pthread_mutex_unlock(&yk_global_mutex);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    yk_type_unref(t);
    return YAKSA_SUCCESS;
}

/* ------------------------------------------------------------------------- */
/* flatten / unflatten (yaksa.h.in:618-634)                                  */
/* ------------------------------------------------------------------------- */

/* A flattened type is one record per node of the type tree, depth first: a fixed
 * header with every derived field, then the node's block-length and displacement
 * arrays, then its children.  Builtin nodes carry only their handle and unflatten to
 * the builtin object itself.  Unlike the reference, which copies its in-memory type
 * objects (pointers included) and so is readable only by the same build
 * (src/frontend/flatten/yaksa_flatten.c:10-95), the records hold no pointers and are
 * position independent; they keep host byte order, like every yaksa message. */
#define YK_FLAT_MAGIC 0x59414b53u       /* "SKAY" */

typedef struct {
    uint32_t magic, kind;
    int64_t builtin, count, blocklength, stride, ndims;
    int64_t tree_depth, alignment;
    uint64_t size, num_contig, builtin_size;
    int64_t extent, lb, ub, true_lb, true_ub;
    int64_t is_contig, base_type, needs_host_ops;
} yk_flat_hdr;

static int flat_has_blens(const yk_type * t)
{
    return t->kind == YK_K_HINDEXED || t->kind == YK_K_STRUCT;
}

static int flat_has_displs(const yk_type * t)
{
    return t->kind == YK_K_BLKHINDX || t->kind == YK_K_HINDEXED || t->kind == YK_K_STRUCT;
}

static uintptr_t flat_size(const yk_type * t)
{
    uintptr_t n = sizeof(yk_flat_hdr);
    if (t->kind == YK_K_BUILTIN)
        return n;
    n += (flat_has_blens(t) + flat_has_displs(t)) * (uintptr_t) t->count * sizeof(int64_t);
    if (t->kind == YK_K_STRUCT) {
        for (intptr_t i = 0; i < t->count; i++)
            n += flat_size(t->types[i]);
    } else {
        n += flat_size(t->kind == YK_K_SUBARRAY ? t->primary : t->child);
    }
    return n;
}

static char *flat_write(const yk_type * t, char *p)
{
    yk_flat_hdr h;
    memset(&h, 0, sizeof(h));
    h.magic = YK_FLAT_MAGIC;
    h.kind = (uint32_t) t->kind;
    h.builtin = (int64_t) t->builtin;
    h.count = t->count;
    h.blocklength = t->blocklength;
    h.stride = t->stride;
    h.ndims = t->ndims;
    h.tree_depth = t->tree_depth;
    h.alignment = t->alignment;
    h.size = t->size;
    h.num_contig = t->num_contig;
    h.builtin_size = t->builtin_size;
    h.extent = t->extent;
    h.lb = t->lb;
    h.ub = t->ub;
    h.true_lb = t->true_lb;
    h.true_ub = t->true_ub;
    h.is_contig = t->is_contig;
    h.base_type = t->base_type;
    h.needs_host_ops = t->needs_host_ops;
    memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    if (t->kind == YK_K_BUILTIN)
        return p;
    for (intptr_t i = 0; flat_has_blens(t) && i < t->count; i++, p += sizeof(int64_t)) {
        int64_t v = t->blens[i];
        memcpy(p, &v, sizeof(v));
    }
    for (intptr_t i = 0; flat_has_displs(t) && i < t->count; i++, p += sizeof(int64_t)) {
        int64_t v = t->displs[i];
        memcpy(p, &v, sizeof(v));
    }
    if (t->kind == YK_K_STRUCT) {
        for (intptr_t i = 0; i < t->count; i++)
            p = flat_write(t->types[i], p);
        return p;
    }
    return flat_write(t->kind == YK_K_SUBARRAY ? t->primary : t->child, p);
}

/* a new reference to the node at *pp; advances *pp past it */
static int flat_read(const char **pp, yk_type ** out)
{
    yk_flat_hdr h;
    memcpy(&h, *pp, sizeof(h));
    *pp += sizeof(h);
    *out = NULL;
    if (h.magic != YK_FLAT_MAGIC || h.kind > YK_K_SUBARRAY)
        return YAKSA_ERR__INTERNAL;
    if (h.kind == YK_K_BUILTIN) {
        yk_type *b = yk_type_get((yaksa_type_t) h.builtin);
        if (!b || b->kind != YK_K_BUILTIN)
            return YAKSA_ERR__INTERNAL;
        yk_type_ref(b);
        *out = b;
        return YAKSA_SUCCESS;
    }
    yk_type *t = type_new((int) h.kind);
    if (!t)
        return YAKSA_ERR__OUT_OF_MEM;
    t->count = h.count;
    t->blocklength = h.blocklength;
    t->stride = h.stride;
    t->ndims = (int) h.ndims;
    t->tree_depth = (int) h.tree_depth;
    t->alignment = (int) h.alignment;
    t->size = h.size;
    t->num_contig = h.num_contig;
    t->builtin_size = h.builtin_size;
    t->extent = h.extent;
    t->lb = h.lb;
    t->ub = h.ub;
    t->true_lb = h.true_lb;
    t->true_ub = h.true_ub;
    t->is_contig = h.is_contig != 0;
    t->base_type = (int) h.base_type;
    t->needs_host_ops = h.needs_host_ops != 0;
    int rc = YAKSA_SUCCESS;
    size_t arr = (size_t) (t->count > 0 ? t->count : 0) * sizeof(intptr_t);
    if (flat_has_blens(t)) {
        t->blens = malloc(arr ? arr : 1);
        if (!t->blens)
            rc = YAKSA_ERR__OUT_OF_MEM;
        for (intptr_t i = 0; !rc && i < t->count; i++, *pp += sizeof(int64_t)) {
            int64_t v;
            memcpy(&v, *pp, sizeof(v));
            t->blens[i] = (intptr_t) v;
        }
    }
    if (!rc && flat_has_displs(t)) {
        t->displs = malloc(arr ? arr : 1);
        if (!t->displs)
            rc = YAKSA_ERR__OUT_OF_MEM;
        for (intptr_t i = 0; !rc && i < t->count; i++, *pp += sizeof(int64_t)) {
            int64_t v;
            memcpy(&v, *pp, sizeof(v));
            t->displs[i] = (intptr_t) v;
        }
    }
    if (!rc && t->kind == YK_K_STRUCT) {
        t->types = calloc(t->count > 0 ? (size_t) t->count : 1, sizeof(yk_type *));
        if (!t->types)
            rc = YAKSA_ERR__OUT_OF_MEM;
        for (intptr_t i = 0; !rc && i < t->count; i++)
            rc = flat_read(pp, &t->types[i]);
        if (rc && t->types) {
            /* children read so far are released with the node below */
            intptr_t got = 0;
            while (got < t->count && t->types[got])
                got++;
            t->count = got;
        }
    } else if (!rc) {
        rc = flat_read(pp, t->kind == YK_K_SUBARRAY ? &t->primary : &t->child);
    }
    if (rc) {
        yk_type_unref(t);
        return rc;
    }
    *out = t;
    return YAKSA_SUCCESS;
}

int yaksa_flatten_size(yaksa_type_t type, uintptr_t * flattened_type_size)
{
    LOOKUP(type, t);
    *flattened_type_size = flat_size(t);
    return YAKSA_SUCCESS;
}

int yaksa_flatten(yaksa_type_t type, void *flattened_type)
{
    LOOKUP(type, t);
    flat_write(t, (char *) flattened_type);
    return YAKSA_SUCCESS;
}

int yaksa_unflatten(yaksa_type_t * type, const void *flattened_type)
{
    *type = YAKSA_TYPE__NULL;
    const char *p = (const char *) flattened_type;
    yk_type *t;
    int rc = flat_read(&p, &t);
    if (rc)
        return rc;
    return publish(t, type);
}
