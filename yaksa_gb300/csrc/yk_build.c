/*
 * yk_build.c -- type tree -> flattened device descriptor (see yk_desc.h).
 *
 * Replaces the reference's two mechanisms for describing a type to a backend: the
 * generated per-(kind, kind, builtin) kernel selection
 * (src/backend/gencomm.py:136-295) and the metadata tree mirrored into managed memory
 * on first use (src/backend/cuda/md/yaksuri_cudai_md.c:21-128).  Here every committed
 * type becomes one chain of levels plus a leaf, built once per type and kept in device
 * memory (not managed memory) until the type is freed.
 *
 * Two flavours per type:
 *   bytes: REPLACE moves bytes, so adjacent pieces merge regardless of base type;
 *   typed: operators need element boundaries, so pair types split into fields and
 *          segments carry their base type (a struct of {int64, float} stays two
 *          segments).
 *
 * The level chain follows the reference's pack order exactly (elements, then blocks,
 * then elements within a block: src/frontend/pup/yaksi_ipack_backend.c:42-220).
 * Structs are expanded into a segment table per struct element, in field order.
 */
#include <stdlib.h>
#include <string.h>
#include <assert.h>
#include <cuda_runtime_api.h>
#include "yk_internal.h"
#include "yk_locate.h"

#define YK_MAX_SEGMENTS (1u << 24)

typedef struct {
    int kind;
    uint64_t count;
    int64_t stride;
    uint64_t cps;
    int64_t *disp;              /* host copies, owned */
    uint64_t *pfx;
} hlev;

typedef struct {
    hlev lv[YK_MAX_LEVELS];
    int nlev;
    int leaf;
    uint64_t run;
    int leaf_type;
    int64_t base;
    /* segment leaf */
    int64_t *soff;
    uint64_t *slen;
    uint8_t *stype;
    size_t nseg, capseg;
    int typed;
    int err;
} hbuild;

static void hb_free(hbuild * b)
{
    for (int i = 0; i < b->nlev; i++) {
        free(b->lv[i].disp);
        free(b->lv[i].pfx);
    }
    free(b->soff);
    free(b->slen);
    free(b->stype);
}

static hlev *push_level(hbuild * b, int kind, uint64_t count, int64_t stride, uint64_t cps)
{
    if (b->nlev >= YK_MAX_LEVELS) {
        b->err = YAKSA_ERR__NOT_SUPPORTED;
        return NULL;
    }
    hlev *l = &b->lv[b->nlev++];
    memset(l, 0, sizeof(*l));
    l->kind = kind;
    l->count = count;
    l->stride = stride;
    l->cps = cps;
    return l;
}

static void add_seg(hbuild * b, int64_t off, uint64_t len, int bt)
{
    if (len == 0 || b->err)
        return;
    if (b->nseg) {
        size_t k = b->nseg - 1;
        if (b->soff[k] + (int64_t) b->slen[k] == off && (!b->typed || b->stype[k] == bt)) {
            b->slen[k] += len;
            return;
        }
    }
    if (b->nseg == b->capseg) {
        if (b->capseg >= YK_MAX_SEGMENTS) {
            b->err = YAKSA_ERR__NOT_SUPPORTED;
            return;
        }
        size_t nc = b->capseg ? 2 * b->capseg : 16;
        int64_t *o = realloc(b->soff, nc * sizeof(int64_t));
        uint64_t *l = realloc(b->slen, nc * sizeof(uint64_t));
        uint8_t *t = realloc(b->stype, nc);
        if (!o || !l || !t) {
            b->soff = o ? o : b->soff;
            b->slen = l ? l : b->slen;
            b->stype = t ? t : b->stype;
            b->err = YAKSA_ERR__OUT_OF_MEM;
            return;
        }
        b->soff = o;
        b->slen = l;
        b->stype = t;
        b->capseg = nc;
    }
    b->soff[b->nseg] = off;
    b->slen[b->nseg] = len;
    b->stype[b->nseg] = (uint8_t) (bt < 0 ? YK_BT_NONE : bt);
    b->nseg++;
}

/* Host-side failure injection for tests: the next `n` device allocations of the
 * library report failure without calling the allocator (no GPU fault is involved). */
static int yk_fail_next = 0;

int yaksa_gb300_debug_fail_alloc(int n)
{
    __atomic_store_n(&yk_fail_next, n > 0 ? n : 0, __ATOMIC_RELEASE);
    return YAKSA_SUCCESS;
}

int yk_fail_injected(void)
{
    int v = __atomic_load_n(&yk_fail_next, __ATOMIC_ACQUIRE);
    while (v > 0) {
        if (__atomic_compare_exchange_n(&yk_fail_next, &v, v - 1, 0, __ATOMIC_ACQ_REL,
                                        __ATOMIC_ACQUIRE))
            return 1;
    }
    return 0;
}

/* field layout of a pair builtin: (offset, size, base type) x 2 */
int yk_pair_fields(yaksa_type_t h, size_t off[2], size_t sz[2], int bt[2])
{
#define PF(T1, B1, T2, B2) do { struct p_ { T1 x; T2 y; };                        \
        off[0] = 0; sz[0] = sizeof(T1); bt[0] = B1;                               \
        off[1] = offsetof(struct p_, y); sz[1] = sizeof(T2); bt[1] = B2; } while (0)
    int bi = sizeof(int) == 4 ? YK_BT_I32 : YK_BT_I64;
    int bl = sizeof(long) == 8 ? YK_BT_I64 : YK_BT_I32;
    int bs = YK_BT_I16;
    switch (h) {
        case YAKSA_TYPE__FLOAT_INT:
            PF(float, YK_BT_F32, int, bi);
            return 1;
        case YAKSA_TYPE__DOUBLE_INT:
            PF(double, YK_BT_F64, int, bi);
            return 1;
        case YAKSA_TYPE__LONG_INT:
            PF(long, bl, int, bi);
            return 1;
        case YAKSA_TYPE__2INT:
            PF(int, bi, int, bi);
            return 1;
        case YAKSA_TYPE__SHORT_INT:
            PF(short, bs, int, bi);
            return 1;
        case YAKSA_TYPE__LONG_DOUBLE_INT:
            PF(long double, YK_BT_LDOUBLE, int, bi);
            return 1;
        default:
            return 0;
    }
#undef PF
}

/* one builtin element at `off` as segments */
static void emit_builtin(hbuild * b, const yk_type * t, int64_t off)
{
    size_t fo[2], fs[2];
    int fb[2];
    if (yk_pair_fields(t->builtin, fo, fs, fb)) {
        add_seg(b, off + (int64_t) fo[0], fs[0], fb[0]);
        add_seg(b, off + (int64_t) fo[1], fs[1], fb[1]);
    } else {
        add_seg(b, off, t->size, t->base_type);
    }
}

/* can `count` consecutive elements of t be one segment? */
static int one_segment(const hbuild * b, const yk_type * t)
{
    if (!t->is_contig)
        return 0;
    if (!b->typed)
        return 1;
    /* typed: a single base type and no pair splitting */
    if (t->base_type < 0)
        return 0;
    if (t->kind == YK_K_BUILTIN) {
        size_t fo[2], fs[2];
        int fb[2];
        return !yk_pair_fields(t->builtin, fo, fs, fb) || fb[0] == fb[1];
    }
    return 1;
}

static void emit(hbuild * b, const yk_type * t, int64_t off, intptr_t count);

static void emit_elem(hbuild * b, const yk_type * t, int64_t off)
{
    switch (t->kind) {
        case YK_K_BUILTIN:
            emit_builtin(b, t, off);
            break;
        case YK_K_CONTIG:
            emit(b, t->child, off, t->count);
            break;
        case YK_K_RESIZED:
            emit(b, t->child, off, 1);
            break;
        case YK_K_HVECTOR:
            for (intptr_t j = 0; j < t->count && !b->err; j++)
                emit(b, t->child, off + j * t->stride, t->blocklength);
            break;
        case YK_K_BLKHINDX:
            for (intptr_t j = 0; j < t->count && !b->err; j++)
                emit(b, t->child, off + t->displs[j], t->blocklength);
            break;
        case YK_K_HINDEXED:
            for (intptr_t j = 0; j < t->count && !b->err; j++)
                if (t->blens[j])
                    emit(b, t->child, off + t->displs[j], t->blens[j]);
            break;
        case YK_K_STRUCT:
            for (intptr_t j = 0; j < t->count && !b->err; j++)
                if (t->blens[j])
                    emit(b, t->types[j], off + t->displs[j], t->blens[j]);
            break;
        case YK_K_SUBARRAY:
            emit(b, t->primary, off + t->true_lb - t->primary->true_lb, 1);
            break;
    }
}

static void emit(hbuild * b, const yk_type * t, int64_t off, intptr_t count)
{
    if (count <= 0 || t->size == 0)
        return;
    if (one_segment(b, t)) {
        add_seg(b, off + t->true_lb, (uint64_t) count * t->size, t->base_type);
        return;
    }
    for (intptr_t i = 0; i < count && !b->err; i++)
        emit_elem(b, t, off + i * t->extent);
}

/* the level chain of one element of t, leaf last */
static void chain(hbuild * b, const yk_type * t)
{
    if (b->err)
        return;
    switch (t->kind) {
        case YK_K_BUILTIN:
            if (one_segment(b, t)) {
                b->leaf = YK_LEAF_RUN;
                b->run = t->size;
                b->leaf_type = t->base_type < 0 ? YK_BT_NONE : t->base_type;
            } else {
                b->leaf = YK_LEAF_SEG;
                emit_builtin(b, t, 0);
            }
            break;
        case YK_K_CONTIG:
            push_level(b, YK_LV_VEC, t->count, t->child->extent, t->child->size);
            chain(b, t->child);
            break;
        case YK_K_RESIZED:
            chain(b, t->child);
            break;
        case YK_K_HVECTOR:
            push_level(b, YK_LV_VEC, t->count, t->stride, t->blocklength * t->child->size);
            push_level(b, YK_LV_VEC, t->blocklength, t->child->extent, t->child->size);
            chain(b, t->child);
            break;
        case YK_K_BLKHINDX:{
                hlev *l = push_level(b, YK_LV_IDX, t->count, 0, t->blocklength * t->child->size);
                if (!l)
                    return;
                l->disp = malloc(t->count * sizeof(int64_t));
                if (!l->disp) {
                    b->err = YAKSA_ERR__OUT_OF_MEM;
                    return;
                }
                for (intptr_t j = 0; j < t->count; j++)
                    l->disp[j] = t->displs[j];
                push_level(b, YK_LV_VEC, t->blocklength, t->child->extent, t->child->size);
                chain(b, t->child);
                break;
            }
        case YK_K_HINDEXED:{
                /* empty blocks hold no bytes: left out, so every block of the level is
                 * at least one child long and block starts strictly increase */
                intptr_t nb = 0;
                for (intptr_t j = 0; j < t->count; j++)
                    nb += t->blens[j] != 0;
                const int keep_all = nb == 0;
                if (keep_all)
                    nb = t->count;
                hlev *l = push_level(b, YK_LV_HIDX, (uint64_t) nb, t->child->extent, t->child->size);
                if (!l)
                    return;
                l->disp = malloc((size_t) nb * sizeof(int64_t));
                l->pfx = malloc(((size_t) nb + 1) * sizeof(uint64_t));
                if (!l->disp || !l->pfx) {
                    b->err = YAKSA_ERR__OUT_OF_MEM;
                    return;
                }
                uint64_t acc = 0;
                intptr_t k = 0;
                for (intptr_t j = 0; j < t->count; j++) {
                    if (!t->blens[j] && !keep_all)
                        continue;
                    l->disp[k] = t->displs[j];
                    l->pfx[k] = acc;
                    acc += (uint64_t) t->blens[j] * t->child->size;
                    k++;
                }
                l->pfx[nb] = acc;
                chain(b, t->child);
                break;
            }
        case YK_K_STRUCT:
            b->leaf = YK_LEAF_SEG;
            emit_elem(b, t, 0);
            break;
        case YK_K_SUBARRAY:
            b->base += t->true_lb - t->primary->true_lb;
            chain(b, t->primary);
            break;
    }
}

/* structural simplifications that keep the decomposition identical */
static void simplify(hbuild * b)
{
    int changed = 1;
    while (changed) {
        changed = 0;
        /* a segment leaf of one segment is a run */
        if (b->leaf == YK_LEAF_SEG && b->nseg == 1) {
            b->base += b->soff[0];
            b->leaf = YK_LEAF_RUN;
            b->run = b->slen[0];
            b->leaf_type = b->stype[0];
            b->nseg = 0;
            changed = 1;
        }
        /* levels of count 1 contribute nothing */
        for (int i = 0; i < b->nlev; i++) {
            hlev *l = &b->lv[i];
            if (l->count == 1 && l->kind == YK_LV_VEC) {
                memmove(&b->lv[i], &b->lv[i + 1], (b->nlev - i - 1) * sizeof(hlev));
                b->nlev--;
                changed = 1;
                break;
            }
            if (l->count == 1 && l->kind == YK_LV_IDX) {
                b->base += l->disp[0];
                free(l->disp);
                memmove(&b->lv[i], &b->lv[i + 1], (b->nlev - i - 1) * sizeof(hlev));
                b->nlev--;
                changed = 1;
                break;
            }
        }
        /* a VEC whose stride equals its child's contiguous run extends the run */
        if (b->nlev && b->leaf == YK_LEAF_RUN) {
            hlev *l = &b->lv[b->nlev - 1];
            if (l->kind == YK_LV_VEC && l->stride == (int64_t) b->run && l->cps == b->run) {
                b->run *= l->count;
                b->nlev--;
                changed = 1;
            }
        }
        /* VEC(c1, c2*s2) over VEC(c2, s2) is VEC(c1*c2, s2) */
        for (int i = 0; i + 1 < b->nlev; i++) {
            hlev *o = &b->lv[i], *n = &b->lv[i + 1];
            if (o->kind == YK_LV_VEC && n->kind == YK_LV_VEC &&
                o->stride == (int64_t) n->count * n->stride && o->cps == n->count * n->cps) {
                o->count *= n->count;
                o->stride = n->stride;
                o->cps = n->cps;
                memmove(&b->lv[i + 1], &b->lv[i + 2], (b->nlev - i - 2) * sizeof(hlev));
                b->nlev--;
                changed = 1;
                break;
            }
        }
    }
}

static uint64_t gcd64(uint64_t a, uint64_t b)
{
    while (b) {
        uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

static uint64_t uabs64(int64_t v)
{
    return v < 0 ? (uint64_t) (-v) : (uint64_t) v;
}

static int pow2_align(uint64_t g, int cap)
{
    int a = 1;
    if (g == 0)
        return cap;
    while (a < cap && (g % (2 * a)) == 0)
        a *= 2;
    return a;
}

static int cmp_i64(const void *x, const void *y)
{
    int64_t a = *(const int64_t *) x, b = *(const int64_t *) y;
    return a < b ? -1 : a > b;
}

/* Conservative test whether two typemap entries of one element can reach the same
 * byte; *span_out receives the byte span one element touches. */
static int check_overlap(hbuild * b, int64_t * span_out)
{
    int64_t span;
    int overlap = 0;
    if (b->leaf == YK_LEAF_RUN) {
        span = (int64_t) b->run;
    } else {
        /* sort (start, end) pairs by start; an entry starting before the previous
         * one's end overlaps it */
        int64_t lo = b->soff[0], hi = b->soff[0] + (int64_t) b->slen[0];
        int64_t *ends = malloc(b->nseg * 2 * sizeof(int64_t));
        if (!ends)
            return 1;
        for (size_t s = 0; s < b->nseg; s++) {
            ends[2 * s] = b->soff[s];
            ends[2 * s + 1] = b->soff[s] + (int64_t) b->slen[s];
            lo = YK_MIN(lo, ends[2 * s]);
            hi = YK_MAX(hi, ends[2 * s + 1]);
        }
        qsort(ends, b->nseg, 2 * sizeof(int64_t), cmp_i64);
        for (size_t s = 1; s < b->nseg; s++)
            if (ends[2 * s] < ends[2 * s - 1])
                overlap = 1;
        free(ends);
        span = hi - lo;
    }
    for (int i = b->nlev - 1; i >= 0; i--) {
        hlev *l = &b->lv[i];
        if (l->kind == YK_LV_VEC) {
            if (l->count > 1 && (int64_t) uabs64(l->stride) < span)
                overlap = 1;
            span = (int64_t) uabs64(l->stride) * (int64_t) (l->count - 1) + span;
        } else if (l->kind == YK_LV_IDX) {
            int64_t *d = malloc(l->count * sizeof(int64_t));
            if (!d)
                return 1;
            memcpy(d, l->disp, l->count * sizeof(int64_t));
            qsort(d, l->count, sizeof(int64_t), cmp_i64);
            for (uint64_t j = 1; j < l->count; j++)
                if (d[j] - d[j - 1] < span)
                    overlap = 1;
            span = d[l->count - 1] - d[0] + span;
            free(d);
        } else {
            /* HIDX: block j covers [disp, disp + (n_j - 1) * |stride| + span) */
            int64_t lo = 0, hi = 0;
            int have = 0;
            int64_t *pairs = malloc(l->count * 2 * sizeof(int64_t));
            uint64_t np = 0;
            if (!pairs)
                return 1;
            for (uint64_t j = 0; j < l->count; j++) {
                uint64_t n = (l->pfx[j + 1] - l->pfx[j]) / (l->cps ? l->cps : 1);
                if (!n)
                    continue;
                if (n > 1 && (int64_t) uabs64(l->stride) < span)
                    overlap = 1;
                int64_t ext = (int64_t) (n - 1) * (int64_t) uabs64(l->stride) + span;
                int64_t s0 = l->disp[j] + (l->stride < 0 ? -(int64_t) (n - 1) * (int64_t) uabs64(l->stride) : 0);
                pairs[2 * np] = s0;
                pairs[2 * np + 1] = s0 + ext;
                np++;
                lo = have ? YK_MIN(lo, s0) : s0;
                hi = have ? YK_MAX(hi, s0 + ext) : s0 + ext;
                have = 1;
            }
            qsort(pairs, np, 2 * sizeof(int64_t), cmp_i64);
            for (uint64_t j = 1; j < np; j++)
                if (pairs[2 * j] < pairs[2 * j - 1])
                    overlap = 1;
            free(pairs);
            span = hi - lo;
        }
    }
    *span_out = span;
    return overlap;
}

/* Granlund-Montgomery magic for unsigned division by d (N = 32 and 64) */
void yk_level_set_magic(yk_level * l)
{
    uint64_t d = l->cps ? l->cps : 1;
    int lg = 0;
    while (lg < 64 && ((uint64_t) 1 << lg) < d)
        lg++;
    l->l = (uint8_t) lg;
    /* m = floor(2^N * (2^l - d) / d) + 1 */
    if (lg < 64) {
        unsigned __int128 num = ((unsigned __int128) (((uint64_t) 1 << lg) - d)) << 64;
        l->m64 = (uint64_t) (num / d) + 1;
    } else {
        l->m64 = 1;
    }
    if (d <= 0xffffffffull) {
        uint64_t num32 = ((((uint64_t) 1 << lg) - d) << 32);
        l->m32 = (uint32_t) (num32 / d + 1);
    } else {
        l->m32 = 0;
    }
}

/* Pack every table into one allocation: device memory, or (to_device == 0) host
 * memory for the CPU address check behind yaksa_gb300_debug_locate. */
/* HIDX tile table: tile size 2^tshift chosen so a tile overlaps about eight blocks on
 * average; tfb[t] = the block holding packed byte t * 2^tshift (clamped to count - 1) */
static uint32_t hidx_tile_shift(const hlev * h)
{
    uint64_t total = h->pfx[h->count];
    uint64_t want = h->count ? (total * 8) / h->count : 64;
    uint32_t s = 6;
    while (s < 40 && ((uint64_t) 1 << s) < want)
        s++;
    while (s < 40 && (total >> s) > (1u << 24))
        s++;    /* at most 16M entries */
    return s;
}

static uint64_t hidx_ntiles(const hlev * h, uint32_t s)
{
    return (h->pfx[h->count] >> s) + 2;
}

static int hidx_has_table(const hlev * h)
{
    return h->kind == YK_LV_HIDX && h->count > 1 && h->count < 0xffffffffull;
}

/* an IDX level whose displacements all fit in 32 bits (it gets an int32 copy) */
static int idx_fits32(const hlev * h)
{
    if (h->kind != YK_LV_IDX || !h->disp || !h->count)
        return 0;
    for (uint64_t j = 0; j < h->count; j++)
        if (h->disp[j] < INT32_MIN || h->disp[j] > INT32_MAX)
            return 0;
    return 1;
}

/* every displacement plus cps - 1 in int32 (idx_fits32 holds) */
static int idx_offsets_fit32(const hlev * h)
{
    if (h->cps == 0 || h->cps > (uint64_t) INT32_MAX)
        return 0;
    for (uint64_t j = 0; j < h->count; j++)
        if (h->disp[j] > (int64_t) INT32_MAX - (int64_t) (h->cps - 1))
            return 0;
    return 1;
}

static int upload(hbuild * b, yk_devdesc * dd, int to_device)
{
    /* table sizes */
    size_t bytes = 0;
    for (int i = 0; i < b->nlev; i++) {
        if (b->lv[i].disp)
            bytes += b->lv[i].count * sizeof(int64_t);
        if (idx_fits32(&b->lv[i]))
            bytes += (b->lv[i].count * sizeof(int32_t) + 7) & ~(size_t) 7;
        if (b->lv[i].pfx)
            bytes += (b->lv[i].count + 1) * sizeof(uint64_t);
        if (hidx_has_table(&b->lv[i]))
            bytes += hidx_ntiles(&b->lv[i], hidx_tile_shift(&b->lv[i])) * sizeof(uint32_t) + 8;
    }
    if (b->leaf == YK_LEAF_SEG)
        bytes += b->nseg * sizeof(int64_t) + (b->nseg + 1) * sizeof(uint64_t) + b->nseg + 16;
    char *host = NULL, *dev = NULL;
    if (bytes) {
        host = malloc(bytes);
        if (!host)
            return YAKSA_ERR__OUT_OF_MEM;
        if (!to_device) {
            dev = host;
        } else if (yk_fail_injected() || cudaMalloc((void **) &dev, bytes) != cudaSuccess) {
            free(host);
            return YAKSA_ERR__OUT_OF_MEM;
        }
    }
    size_t pos = 0;
    yk_desc *d = &dd->d;
    memset(d, 0, sizeof(*d));
    d->nlev = b->nlev;
    for (int i = 0; i < b->nlev; i++) {
        hlev *h = &b->lv[i];
        yk_level *l = &d->lv[i];
        l->kind = h->kind;
        l->count = h->count;
        l->stride = h->stride;
        l->cps = h->cps;
        yk_level_set_magic(l);
        if (h->disp) {
            memcpy(host + pos, h->disp, h->count * sizeof(int64_t));
            l->disp = (const int64_t *) (dev + pos);
            pos += h->count * sizeof(int64_t);
        }
        if (idx_fits32(h)) {
            /* the 32-bit copy right after the table: kernels that read one displacement
             * per element move half the table bytes */
            int32_t *d32 = (int32_t *) (host + pos);
            for (uint64_t j = 0; j < h->count; j++)
                d32[j] = (int32_t) h->disp[j];
            l->has_d32 = YK_D32_TABLE | (idx_offsets_fit32(h) ? YK_D32_OFFSETS : 0);
            pos += (h->count * sizeof(int32_t) + 7) & ~(size_t) 7;
        }
        if (h->pfx) {
            memcpy(host + pos, h->pfx, (h->count + 1) * sizeof(uint64_t));
            l->pfx = (const uint64_t *) (dev + pos);
            pos += (h->count + 1) * sizeof(uint64_t);
        }
        if (hidx_has_table(h)) {
            uint32_t s = hidx_tile_shift(h);
            uint64_t nt = hidx_ntiles(h, s);
            uint32_t *tfb = (uint32_t *) (host + pos);
            uint64_t j = 0;
            for (uint64_t t = 0; t < nt; t++) {
                uint64_t x = t << s;
                /* largest j with pfx[j] <= x, walking forward (pfx is non-decreasing) */
                while (j + 1 <= h->count && h->pfx[j + 1] <= x)
                    j++;
                tfb[t] = (uint32_t) (j < h->count ? j : h->count - 1);
            }
            l->tfb = (const uint32_t *) (dev + pos);
            l->tshift = s;
            pos += nt * sizeof(uint32_t);
            pos = (pos + 7) & ~(size_t) 7;
        }
    }
    d->leaf = b->leaf;
    d->run = b->run;
    d->leaf_type = b->leaf_type;
    d->base = b->base;
    if (b->leaf == YK_LEAF_SEG) {
        d->nseg = b->nseg;
        memcpy(host + pos, b->soff, b->nseg * sizeof(int64_t));
        d->seg_off = (const int64_t *) (dev + pos);
        pos += b->nseg * sizeof(int64_t);
        uint64_t acc = 0;
        uint64_t *pf = (uint64_t *) (host + pos);
        for (size_t s = 0; s < b->nseg; s++) {
            pf[s] = acc;
            acc += b->slen[s];
        }
        pf[b->nseg] = acc;
        d->seg_pfx = (const uint64_t *) (dev + pos);
        pos += (b->nseg + 1) * sizeof(uint64_t);
        memcpy(host + pos, b->stype, b->nseg);
        d->seg_type = (const uint8_t *) (dev + pos);
        pos += b->nseg;
    }
    if (bytes && to_device) {
        /* A synchronous cudaMemcpy from pageable memory may return before the DMA
         * lands; a kernel already resident (the request server) would then read the
         * tables early.  Copy on a private stream and wait for that stream. */
        cudaStream_t us;
        cudaError_t e = cudaStreamCreateWithFlags(&us, cudaStreamNonBlocking);
        if (e == cudaSuccess) {
            e = cudaMemcpyAsync(dev, host, pos, cudaMemcpyHostToDevice, us);
            cudaError_t e2 = cudaStreamSynchronize(us);
            if (e == cudaSuccess)
                e = e2;
            cudaStreamDestroy(us);
        }
        free(host);
        if (e != cudaSuccess) {
            cudaFree(dev);
            return YAKSA_ERR__INTERNAL;
        }
    }
    dd->dev_tables = dev;
    dd->table_bytes = bytes;
    return YAKSA_SUCCESS;
}

static int build(yk_type * t, int typed, yk_devdesc * dd, int to_device)
{
    hbuild b;
    memset(&b, 0, sizeof(b));
    b.typed = typed;
    b.leaf_type = YK_BT_NONE;
    chain(&b, t);
    if (b.err) {
        int e = b.err;
        hb_free(&b);
        return e;
    }
    simplify(&b);

    /* vector alignment: every offset, run length and packed boundary */
    uint64_t g = uabs64(b.base);
    if (b.leaf == YK_LEAF_RUN) {
        g = gcd64(g, b.run);
    } else {
        for (size_t s = 0; s < b.nseg; s++) {
            g = gcd64(g, uabs64(b.soff[s]));
            g = gcd64(g, b.slen[s]);
        }
    }
    uint64_t goff = uabs64(b.base);    /* offsets only: element alignment */
    if (b.leaf == YK_LEAF_SEG)
        for (size_t s = 0; s < b.nseg; s++)
            goff = gcd64(goff, uabs64(b.soff[s]));
    for (int i = 0; i < b.nlev; i++) {
        hlev *l = &b.lv[i];
        if (l->kind == YK_LV_VEC || l->kind == YK_LV_HIDX) {
            g = gcd64(g, uabs64(l->stride));
            goff = gcd64(goff, uabs64(l->stride));
        }
        if (l->disp)
            for (uint64_t j = 0; j < l->count; j++) {
                g = gcd64(g, uabs64(l->disp[j]));
                goff = gcd64(goff, uabs64(l->disp[j]));
            }
        if (l->pfx)
            for (uint64_t j = 0; j <= l->count; j++)
                g = gcd64(g, l->pfx[j]);
        g = gcd64(g, l->cps);
    }
    dd->vec_align = pow2_align(g, 16);
    dd->elem_align = pow2_align(goff, 16);

    /* work-unit granule for operators: gcd of element sizes */
    if (typed) {
        uint64_t u = 0;
        if (b.leaf == YK_LEAF_RUN)
            u = yk_base_type_size(b.leaf_type);
        else
            for (size_t s = 0; s < b.nseg; s++)
                u = gcd64(u, (uint64_t) yk_base_type_size(b.stype[s]));
        dd->unit = (int) (u ? u : 1);
    } else {
        dd->unit = 1;
    }

    int64_t span = 0;
    dd->may_overlap = check_overlap(&b, &span);
    dd->sorted_blocks = 0;
    dd->disp32 = 0;
    if (dd->may_overlap && typed && b.leaf == YK_LEAF_RUN && b.nlev == 1 &&
        b.lv[0].kind == YK_LV_IDX && b.lv[0].cps == b.run) {
        int sorted = 1;
        for (uint64_t j = 1; j < b.lv[0].count && sorted; j++)
            sorted = b.lv[0].disp[j] >= b.lv[0].disp[j - 1];
        dd->sorted_blocks = sorted;
        /* sorted: the first and last displacements bound every target offset */
        const uint64_t n = b.lv[0].count;
        dd->disp32 = sorted && n > 0 && b.run < (1ull << 30) && b.lv[0].disp[0] >= INT32_MIN &&
            b.lv[0].disp[n - 1] <= (int64_t) INT32_MAX - (int64_t) b.run;
    }
    dd->elem_span = span;
    int rc = upload(&b, dd, to_device);
    hb_free(&b);
    return rc;
}

/* Allocation failures are not cached: the next request for the type retries the
 * build, so a transient shortage of device memory does not disable a type for good. */
int yk_desc_get(yk_type * t, int typed, yk_devdesc ** out)
{
    yk_devdesc *dd = typed ? &t->typed_desc : &t->bytes_desc;
    pthread_mutex_lock(&t->desc_mutex);
    if (!dd->built) {
        dd->status = build(t, typed, dd, 1);
        dd->built = dd->status != YAKSA_ERR__OUT_OF_MEM;
    }
    int rc = dd->status;
    pthread_mutex_unlock(&t->desc_mutex);
    *out = dd;
    return rc;
}

/* The descriptor with its tables left on the host heap (built once, kept with the
 * type): the no-allocation entry point copies them into its static device scratch
 * per request instead of keeping a device allocation per type. */
int yk_desc_get_host(yk_type * t, int typed, yk_devdesc ** out)
{
    yk_devdesc *dd = typed ? &t->host_typed_desc : &t->host_bytes_desc;
    pthread_mutex_lock(&t->desc_mutex);
    if (!dd->built) {
        dd->status = build(t, typed, dd, 0);
        dd->built = dd->status != YAKSA_ERR__OUT_OF_MEM;
    }
    int rc = dd->status;
    pthread_mutex_unlock(&t->desc_mutex);
    *out = dd;
    return rc;
}

/* the type's descriptor with the element level VEC(count, extent, size) in front
 * (merged into the first level or the leaf when the layout allows) */
void yk_make_launch_desc(const yk_devdesc * dd, const yk_type * t, uintptr_t count, yk_desc * out)
{
    *out = dd->d;
    if (count <= 1)
        return;
    yk_level e;
    memset(&e, 0, sizeof(e));
    e.kind = YK_LV_VEC;
    e.count = count;
    e.stride = t->extent;
    e.cps = t->size;
    if (out->nlev && out->lv[0].kind == YK_LV_VEC) {
        yk_level *n = &out->lv[0];
        if (e.stride == (int64_t) n->count * n->stride && e.cps == n->count * n->cps) {
            n->count *= count;
            return;
        }
    } else if (!out->nlev && out->leaf == YK_LEAF_RUN && e.stride == (int64_t) out->run &&
               e.cps == out->run) {
        out->run *= count;
        return;
    }
    memmove(&out->lv[1], &out->lv[0], out->nlev * sizeof(yk_level));
    yk_level_set_magic(&e);
    out->lv[0] = e;
    out->nlev++;
}

/* CPU evaluation of the kernels' address computation for the given packed
 * positions; lets tests check every typed-side offset against the oracle. */
int yaksa_gb300_debug_locate(yaksa_type_t type, uintptr_t count, int typed, uintptr_t n,
                             const uint64_t * pos, int64_t * off)
{
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    yk_devdesc dd;
    memset(&dd, 0, sizeof(dd));
    int rc = build(t, typed, &dd, 0);
    if (rc) {
        free(dd.dev_tables);
        return rc;
    }
    yk_desc d;
    yk_make_launch_desc(&dd, t, count, &d);
    int use64 = count * t->size > 0xffffffffull;
    for (uintptr_t i = 0; i < n; i++)
        off[i] = use64 ? yk_locate64(&d, pos[i], NULL, NULL) :
            yk_locate32(&d, (uint32_t) pos[i], NULL, NULL);
    free(dd.dev_tables);
    return YAKSA_SUCCESS;
}

/* the descriptor analysis the launch decisions rest on, for CPU tests */
int yaksa_gb300_debug_desc_info(yaksa_type_t type, int typed, int *vec_align, int *unit,
                                int *may_overlap, int *sorted_blocks, int *nlev)
{
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    yk_devdesc dd;
    memset(&dd, 0, sizeof(dd));
    int rc = build(t, typed, &dd, 0);
    free(dd.dev_tables);
    if (rc)
        return rc;
    *vec_align = dd.vec_align;
    *unit = dd.unit;
    *may_overlap = dd.may_overlap;
    *sorted_blocks = dd.sorted_blocks;
    *nlev = dd.d.nlev;
    return YAKSA_SUCCESS;
}

int yaksa_gb300_debug_d32(yaksa_type_t type, int typed, int *level0_bits, int *disp32)
{
    yk_type *t = yk_type_get(type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    yk_devdesc dd;
    memset(&dd, 0, sizeof(dd));
    int rc = build(t, typed, &dd, 0);
    free(dd.dev_tables);
    if (rc)
        return rc;
    *level0_bits = dd.d.nlev > 0 ? dd.d.lv[0].has_d32 : 0;
    *disp32 = dd.disp32;
    return YAKSA_SUCCESS;
}

void yk_desc_release(yk_type * t)
{
    yk_iov_release(t);
    if (t->bytes_desc.dev_tables)
        cudaFree(t->bytes_desc.dev_tables);
    if (t->typed_desc.dev_tables)
        cudaFree(t->typed_desc.dev_tables);
    t->bytes_desc.dev_tables = t->typed_desc.dev_tables = NULL;
    free(t->host_bytes_desc.dev_tables);
    free(t->host_typed_desc.dev_tables);
    t->host_bytes_desc.dev_tables = t->host_typed_desc.dev_tables = NULL;
}

/* ------------------------------------------------------------------------- */
/* builtin boundaries: the largest builtin start <= pos in the packed stream  */
/* (partial packs move whole builtins only, yaksi_ipack_element.c:442-446)    */
/* ------------------------------------------------------------------------- */

static uintptr_t floor_in(const yk_type * t, uintptr_t r)
{
    if (t->builtin_size)
        return r - r % t->builtin_size;
    switch (t->kind) {
        case YK_K_BUILTIN:
            return 0;
        case YK_K_RESIZED:
            return floor_in(t->child, r);
        case YK_K_SUBARRAY:
            return floor_in(t->primary, r);
        case YK_K_CONTIG:{
                uintptr_t k = r / t->child->size;
                return k * t->child->size + floor_in(t->child, r - k * t->child->size);
            }
        case YK_K_HVECTOR:
        case YK_K_BLKHINDX:{
                uintptr_t cs = t->child->size;
                uintptr_t k = r / cs;
                return k * cs + floor_in(t->child, r - k * cs);
            }
        case YK_K_HINDEXED:{
                uintptr_t acc = 0, cs = t->child->size;
                for (intptr_t j = 0; j < t->count; j++) {
                    uintptr_t bb = (uintptr_t) t->blens[j] * cs;
                    if (r < acc + bb) {
                        uintptr_t rr = r - acc, k = rr / cs;
                        return acc + k * cs + floor_in(t->child, rr - k * cs);
                    }
                    acc += bb;
                }
                return acc;
            }
        case YK_K_STRUCT:{
                uintptr_t acc = 0;
                for (intptr_t j = 0; j < t->count; j++) {
                    uintptr_t cs = t->types[j]->size, bb = (uintptr_t) t->blens[j] * cs;
                    if (r < acc + bb) {
                        uintptr_t rr = r - acc, k = rr / cs;
                        return acc + k * cs + floor_in(t->types[j], rr - k * cs);
                    }
                    acc += bb;
                }
                return acc;
            }
    }
    return r;
}

uintptr_t yk_builtin_floor(yk_type * t, uintptr_t count, uintptr_t pos)
{
    if (pos >= count * t->size)
        return count * t->size;
    uintptr_t e = pos / t->size;
    return e * t->size + floor_in(t, pos - e * t->size);
}

/* Sharding (no counterpart in the reference): rank `rank` of `nranks` takes packed bytes
 * [offset, offset + bytes) of `count` elements of `type`, the n-th part of the packed
 * range with both ends moved down to a builtin boundary.  The parts tile the range
 * exactly, and each is a valid (inoffset, max_pack_bytes) of yaksa_pack / yaksa_unpack,
 * so ranks or GPUs can each move their part with no exchange between them. */
int yaksa_gb300_shard(yaksa_type_t type, uintptr_t count, int rank, int nranks,
                      uintptr_t * offset, uintptr_t * bytes)
{
    *offset = *bytes = 0;
    yk_type *t = yk_type_get(type);
    if (!t || nranks <= 0 || rank < 0 || rank >= nranks)
        return YAKSA_ERR__INTERNAL;
    uintptr_t total = count * t->size;
    if (!total)
        return YAKSA_SUCCESS;
    /* rank * total / nranks without overflow: total < 2^64 and nranks < 2^31 */
    uintptr_t q = total / (uintptr_t) nranks, r = total % (uintptr_t) nranks;
    uintptr_t a = q * (uintptr_t) rank + r * (uintptr_t) rank / (uintptr_t) nranks;
    uintptr_t b = q * (uintptr_t) (rank + 1) + r * (uintptr_t) (rank + 1) / (uintptr_t) nranks;
    a = yk_builtin_floor(t, count, a);
    b = rank + 1 == nranks ? total : yk_builtin_floor(t, count, b);
    *offset = a;
    *bytes = b - a;
    return YAKSA_SUCCESS;
}
