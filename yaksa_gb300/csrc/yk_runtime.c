/*
 * yk_runtime.c -- request routing, progress and completion for the GB300 engine.
 *
 * Replaces the reference's backend router and progress engine
 * (src/backend/src/yaksur_pup.c:12-125, src/backend/src/yaksuri_progress.c:2862-3088)
 * for one GPU:
 *
 *   - every pack/unpack runs on the GPU; there is no CPU pack path.  The CPU only
 *     computes the byte range and the launch parameters;
 *   - buffers the GPU can address directly -- device and managed memory, pinned host
 *     memory, and pageable host memory when the device reports pageable-memory access
 *     (Grace-Blackwell's coherent NVLink-C2C, checked with
 *     cudaDevAttrPageableMemoryAccess) -- are read and written in place by the kernel,
 *     so host data crosses the link once and only the bytes the type touches move;
 *   - buffers it cannot address are staged: the touched span is copied to device
 *     memory from the stream-ordered pool, processed, and copied back;
 *   - a nonblocking request is one pooled CUDA event; test polls it, wait spins on it
 *     (the reference creates and destroys an event per request,
 *     src/backend/cuda/pup/yaksuri_cudai_event.c:13-72).
 *
 * Partial packs follow the reference exactly: the packed range starts at inoffset
 * and ends at the last builtin boundary that fits (src/frontend/pup/yaksi_ipack.c:12-107).
 */
#include <float.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <cuda_runtime_api.h>
#include "yk_internal.h"
#include "yk_tune.h"
#include <nvtx3/nvToolsExt.h>
#include "yaksa_gb300.h"

typedef struct {
    int in_use;
    cudaEvent_t ev;
    yk_type *type;              /* held until completion: a type may be freed in flight */
    void *scratch[2];           /* staged buffers released at completion */
} yk_req;

#define YK_LIB_STREAMS 16     /* at most; YAKSA_GB300_LIB_STREAMS sets how many (4) */

static struct {
    pthread_mutex_t mu;
    int ready;
    int failed;
    int device;
    int pageable_access;        /* the GPU reads/writes pageable host memory (ATS) */
    int host_ptr_ok;            /* registered host memory uses the host address */
    int host_direct;            /* 0: host memory is never addressed in place, always
                                 * staged (YAKSA_GB300_HOST_DIRECT=0) */
    int has_wait_kernel;        /* yaksa_init's yaksa_has_wait_kernel hint: the caller may
                                 * keep a kernel resident that waits on the host, so no
                                 * call may synchronize the device (the reference:
                                 * src/backend/src/yaksuri_progress.c:17-27,
                                 * src/backend/cuda/hooks/yaksuri_cuda_init_hooks.c:14-64) */
    int tma_mode;               /* TMA forms: 0 off, 1 autotuner candidates, 2 forced */
    int red_mode;               /* L2 reductions for order-independent integer operators
                                 * on overlapping blocks: 0 off, 1 where they apply */
    int runs_pack;              /* one-thread-per-element packs of 17..47-byte runs */
    int hidx_forced;           /* contiguous-block hindexed: 1 = hidx_cfg, 0 = autotuner */
    yk_tune_cfg hidx_cfg;
    /* library streams: requests that are not stream-ordered go round robin over
     * these, so independent requests (whose order the API leaves open) overlap on the
     * GPU; streams[0] is also the default stream of graph replays */
    cudaStream_t streams[YK_LIB_STREAMS];
    int nstreams;
    unsigned next_stream;
    yk_req *reqs;
    size_t nreqs;
    size_t *freeidx;            /* stack of free request slots */
    size_t nfree;
    cudaEvent_t *evpool;
    size_t nev, capev;
    /* counters (yaksa_gb300_stats) */
    uint64_t launches, staged_calls, direct_calls, memcpy_calls;
} R = { .mu = PTHREAD_MUTEX_INITIALIZER, .tma_mode = -1, .red_mode = -1 };

/* a library stream for a request that is not stream-ordered (round robin) */
static cudaStream_t lib_stream(void)
{
    unsigned k = __atomic_fetch_add(&R.next_stream, 1, __ATOMIC_RELAXED);
    return R.streams[k % (unsigned) R.nstreams];
}


static int cuda_err(cudaError_t e, const char *what)
{
    if (e == cudaSuccess)
        return YAKSA_SUCCESS;
    fprintf(stderr, "yaksa-gb300: %s failed: %s\n", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? YAKSA_ERR__OUT_OF_MEM : YAKSA_ERR__INTERNAL;
}

int yk_runtime_init(int has_wait_kernel)
{
    /* the GPU is brought up lazily at the first pack/unpack so that type
     * construction works on hosts without a GPU */
    __atomic_store_n(&R.has_wait_kernel, has_wait_kernel ? 1 : 0, __ATOMIC_RELAXED);
    return YAKSA_SUCCESS;
}

static int runtime_ready(void)
{
    if (__atomic_load_n(&R.ready, __ATOMIC_ACQUIRE))
        return YAKSA_SUCCESS;
    pthread_mutex_lock(&R.mu);
    int rc = YAKSA_SUCCESS;
    if (!R.ready && !R.failed) {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) {
            fprintf(stderr, "yaksa-gb300: no CUDA device is available (%s); this library "
                    "runs every pack/unpack on the GPU and has no CPU path\n",
                    e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
            R.failed = 1;
        } else {
            cudaGetDevice(&R.device);
            cudaDeviceGetAttribute(&R.pageable_access, cudaDevAttrPageableMemoryAccess,
                                   R.device);
            cudaDeviceGetAttribute(&R.host_ptr_ok, cudaDevAttrCanUseHostPointerForRegisteredMem,
                                   R.device);
            /* Opt-in: the L2 fetch granularity of this process's context (a hint the
             * driver may clamp; it ends with the process).  Strided types whose runs
             * are shorter than a sector move less DRAM traffic with 32-byte fetches. */
            const char *l2 = getenv("YAKSA_GB300_L2_FETCH_BYTES");
            if (l2 && atoi(l2) > 0)
                cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t) atoi(l2));
            if (R.tma_mode < 0) {
                const char *tm = getenv("YAKSA_GB300_TMA");
                R.tma_mode = tm && tm[0] >= '0' && tm[0] <= '2' ? tm[0] - '0' : 1;
            }
            if (R.red_mode < 0) {
                const char *rm = getenv("YAKSA_GB300_L2_REDUCE");
                R.red_mode = !(rm && rm[0] == '0');
            }
            const char *rp = getenv("YAKSA_GB300_RUNS_PACK");
            R.runs_pack = !(rp && rp[0] == '0');
            const char *hd = getenv("YAKSA_GB300_HOST_DIRECT");
            R.host_direct = !(hd && hd[0] == '0');
            const char *ns = getenv("YAKSA_GB300_LIB_STREAMS");
            R.nstreams = ns ? atoi(ns) : 4;
            if (R.nstreams < 1 || R.nstreams > YK_LIB_STREAMS)
                R.nstreams = 4;
            for (int k = 0; k < R.nstreams && e == cudaSuccess; k++)
                e = cudaStreamCreateWithFlags(&R.streams[k], cudaStreamNonBlocking);
            if (e != cudaSuccess) {
                cuda_err(e, "cudaStreamCreate");
                R.failed = 1;
            } else {
                __atomic_store_n(&R.ready, 1, __ATOMIC_RELEASE);
            }
        }
    }
    if (R.failed)
        rc = YAKSA_ERR__INTERNAL;
    pthread_mutex_unlock(&R.mu);
    return rc;
}

static void stage_finalize(void);

void yk_runtime_finalize(void)
{
    yk_tune_reset();
    stage_finalize();
    pthread_mutex_lock(&R.mu);
    if (R.ready) {
        for (int k = 0; k < R.nstreams; k++)
            cudaStreamSynchronize(R.streams[k]);
        for (size_t i = 0; i < R.nreqs; i++)
            if (R.reqs[i].in_use) {
                cudaEventDestroy(R.reqs[i].ev);
                R.reqs[i].in_use = 0;
            }
        for (size_t i = 0; i < R.nev; i++)
            cudaEventDestroy(R.evpool[i]);
        R.nev = 0;
        for (int k = 0; k < R.nstreams; k++)
            cudaStreamDestroy(R.streams[k]);
        R.ready = 0;
    }
    free(R.reqs);
    R.reqs = NULL;
    R.nreqs = 0;
    free(R.freeidx);
    R.freeidx = NULL;
    R.nfree = 0;
    free(R.evpool);
    R.evpool = NULL;
    R.capev = 0;
    R.failed = 0;
    pthread_mutex_unlock(&R.mu);
}

/* ------------------------------------------------------------------------- */
/* events and requests                                                       */
/* ------------------------------------------------------------------------- */

static int event_get(cudaEvent_t * ev)
{
    pthread_mutex_lock(&R.mu);
    if (R.nev) {
        *ev = R.evpool[--R.nev];
        pthread_mutex_unlock(&R.mu);
        return YAKSA_SUCCESS;
    }
    pthread_mutex_unlock(&R.mu);
    return cuda_err(cudaEventCreateWithFlags(ev, cudaEventDisableTiming), "cudaEventCreate");
}

static void event_put(cudaEvent_t ev)
{
    pthread_mutex_lock(&R.mu);
    if (R.nev == R.capev) {
        size_t nc = R.capev ? 2 * R.capev : 64;
        cudaEvent_t *p = realloc(R.evpool, nc * sizeof(cudaEvent_t));
        if (!p) {
            pthread_mutex_unlock(&R.mu);
            cudaEventDestroy(ev);
            return;
        }
        R.evpool = p;
        R.capev = nc;
    }
    R.evpool[R.nev++] = ev;
    pthread_mutex_unlock(&R.mu);
}

static int request_new(cudaEvent_t ev, yk_type * t, void *s0, void *s1, yaksa_request_t * out)
{
    pthread_mutex_lock(&R.mu);
    if (!R.nfree) {
        size_t nn = R.nreqs ? 2 * R.nreqs : 64;
        yk_req *p = realloc(R.reqs, nn * sizeof(yk_req));
        size_t *f = p ? realloc(R.freeidx, nn * sizeof(size_t)) : NULL;
        if (p)
            R.reqs = p;
        if (!f) {
            pthread_mutex_unlock(&R.mu);
            return YAKSA_ERR__OUT_OF_MEM;
        }
        memset(p + R.nreqs, 0, (nn - R.nreqs) * sizeof(yk_req));
        R.freeidx = f;
        for (size_t k = nn; k > R.nreqs; k--)
            R.freeidx[R.nfree++] = k - 1;       /* lowest index on top */
        R.nreqs = nn;
    }
    size_t i = R.freeidx[--R.nfree];
    R.reqs[i].in_use = 1;
    R.reqs[i].ev = ev;
    R.reqs[i].type = t;
    R.reqs[i].scratch[0] = s0;
    R.reqs[i].scratch[1] = s1;
    pthread_mutex_unlock(&R.mu);
    *out = (yaksa_request_t) (i + 1);   /* 0 is YAKSA_REQUEST__NULL */
    return YAKSA_SUCCESS;
}

static void request_release(size_t i)
{
    pthread_mutex_lock(&R.mu);
    yk_req r = R.reqs[i];
    R.reqs[i].in_use = 0;
    R.freeidx[R.nfree++] = i;
    pthread_mutex_unlock(&R.mu);
    event_put(r.ev);
    if (r.scratch[0])
        cudaFree(r.scratch[0]);
    if (r.scratch[1])
        cudaFree(r.scratch[1]);
    if (r.type)
        yk_type_unref(r.type);
}

static yk_req *request_lookup(yaksa_request_t h, size_t *idx)
{
    uint64_t id = h & 0xffffffffull;
    if (id == 0 || id > R.nreqs || !R.reqs[id - 1].in_use)
        return NULL;
    *idx = id - 1;
    return &R.reqs[id - 1];
}

int yaksa_request_test(yaksa_request_t request, int *completed)
{
    if (request == YAKSA_REQUEST__NULL) {
        *completed = 1;
        return YAKSA_SUCCESS;
    }
    size_t i;
    pthread_mutex_lock(&R.mu);
    yk_req *r = request_lookup(request, &i);
    cudaEvent_t ev = r ? r->ev : NULL;
    pthread_mutex_unlock(&R.mu);
    if (!r)
        return YAKSA_ERR__INTERNAL;
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaErrorNotReady) {
        *completed = 0;
        return YAKSA_SUCCESS;
    }
    *completed = 1;
    request_release(i);
    return cuda_err(e, "kernel completion");
}

int yaksa_request_wait(yaksa_request_t request)
{
    if (request == YAKSA_REQUEST__NULL)
        return YAKSA_SUCCESS;
    size_t i;
    pthread_mutex_lock(&R.mu);
    yk_req *r = request_lookup(request, &i);
    cudaEvent_t ev = r ? r->ev : NULL;
    pthread_mutex_unlock(&R.mu);
    if (!r)
        return YAKSA_ERR__INTERNAL;
    cudaError_t e = cudaEventSynchronize(ev);
    request_release(i);
    return cuda_err(e, "kernel completion");
}

/* ------------------------------------------------------------------------- */
/* pointers                                                                  */
/* ------------------------------------------------------------------------- */

/* device-usable alias of host address p (delta applies to the whole buffer), or
 * 0 with *staged = 1 when the GPU cannot reach it */
static char *device_alias(const char *base, const char *probe, int host_hint, int *staged)
{
    *staged = 0;
    /* Grace-Blackwell: the GPU addresses device memory, pinned and pageable host memory
     * alike through the caller's pointer, so no per-call attribute query is needed
     * (the reference queries both pointers of every request,
     * src/backend/src/yaksur_pup.c:31-58) */
    if (R.host_direct && R.pageable_access && R.host_ptr_ok)
        return (char *) base;
    struct cudaPointerAttributes a;
    memset(&a, 0, sizeof(a));
    cudaError_t e = cudaPointerGetAttributes(&a, probe);
    if (e != cudaSuccess) {
        cudaGetLastError();
        a.type = cudaMemoryTypeUnregistered;
    }
    (void) host_hint;
    switch (a.type) {
        case cudaMemoryTypeDevice:
        case cudaMemoryTypeManaged:
            return (char *) base;
        case cudaMemoryTypeHost:
            if (!R.host_direct && !R.has_wait_kernel) {
                *staged = 1;
                return NULL;
            }
            if (a.devicePointer)
                return (char *) base + ((const char *) a.devicePointer - probe);
            return (char *) base;
        default:
            /* with a wait kernel, pageable memory the GPU can reach is used in place even
             * when staging was asked for: the reference likewise treats unregistered host
             * buffers as registered then */
            if (R.pageable_access && (R.host_direct || R.has_wait_kernel))
                return (char *) base;
            *staged = 1;
            return NULL;
    }
}

/* 1 when p lies in device or managed memory: the reductions of yk_red_kernel are sent
 * only there, never to host memory the GPU reaches over the C2C link */
static int device_memory(const void *p)
{
    struct cudaPointerAttributes a;
    memset(&a, 0, sizeof(a));
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static int pow2_of(uint64_t v)
{
    int a = 16;
    while (a > 1 && (v % (uint64_t) a))
        a >>= 1;
    return a;
}

/* ------------------------------------------------------------------------- */
/* planning: byte range, typed span and pointer routing of one request        */
/* ------------------------------------------------------------------------- */

typedef struct {
    int dir;                    /* 0 pack, 1 unpack */
    yk_type *t;
    uintptr_t count, b0, b1;
    yaksa_op_t op;
    char *typed, *packed;       /* caller's pointers */
    char *dtyped, *dpacked;     /* device-usable aliases */
    int staged;                 /* 1: the GPU cannot address one of the buffers */
    int64_t lo, hi;             /* typed bytes touched, relative to typed */
} yk_plan;

/* The GPU computes long double as IEEE binary128 (yk_quad.h), the long double of
 * aarch64 Linux.  A host whose long double is another format (x87 extended precision
 * on x86_64) has no GPU form of the long double operators. */
#if LDBL_MANT_DIG == 113 && LDBL_MAX_EXP == 16384
#define YK_LDBL_ON_GPU 1
#else
#define YK_LDBL_ON_GPU 0
#endif

/* an arithmetic operator on a type that holds long double */
static int ldbl_arith(yk_type * t, yaksa_op_t op)
{
    return t->needs_host_ops && (op == YAKSA_OP__SUM || op == YAKSA_OP__PROD ||
                                 op == YAKSA_OP__MIN || op == YAKSA_OP__MAX);
}

static int op_needs_host_arith(yk_type * t, yaksa_op_t op)
{
    return !YK_LDBL_ON_GPU && ldbl_arith(t, op);
}

/* Partial packs follow the reference: start at `offset` and stop at the last builtin
 * boundary that fits (src/frontend/pup/yaksi_ipack.c:12-107). */
static int plan(int dir, const void *packed_in, void *packed_out, char *typed, uintptr_t count,
                yk_type * t, uintptr_t offset, uintptr_t maxbytes, yk_info * info, yaksa_op_t op,
                yk_plan * p)
{
    memset(p, 0, sizeof(*p));
    p->dir = dir;
    p->t = t;
    p->count = count;
    p->op = op;
    if (count == 0 || t->size == 0)
        return YAKSA_SUCCESS;
    if (op >= YAKSA_OP__LAST)
        return YAKSA_ERR__INTERNAL;
    uintptr_t total = count * t->size;
    if (offset >= total)
        return YAKSA_SUCCESS;
    uintptr_t b0 = offset;
    if (yk_builtin_floor(t, count, b0) != b0)
        return YAKSA_ERR__INTERNAL;     /* offset inside a builtin: a precondition */
    uintptr_t b1 = yk_builtin_floor(t, count, b0 + YK_MIN(maxbytes, total - b0));
    if (b1 <= b0)
        return YAKSA_SUCCESS;
    if (op != YAKSA_OP__REPLACE && op_needs_host_arith(t, op))
        return YAKSA_ERR__NOT_SUPPORTED;        /* no binary128 long double on this host */
    int rc = runtime_ready();
    if (rc)
        return rc;
    p->b0 = b0;
    p->b1 = b1;
    p->typed = typed;
    p->packed = dir == 0 ? (char *) packed_out : (char *) packed_in;
    uintptr_t e0 = b0 / t->size, e1 = (b1 + t->size - 1) / t->size;
    int64_t ext = t->extent;
    p->lo = (ext >= 0 ? (int64_t) e0 * ext : (int64_t) (e1 - 1) * ext) + t->true_lb;
    p->hi = (ext >= 0 ? (int64_t) (e1 - 1) * ext : (int64_t) e0 * ext) + t->true_ub;
    int host_hint = info && info->gpu_driver == 2;
    int st_t = 0, st_p = 0;
    p->dtyped = device_alias(typed, typed + p->lo, host_hint, &st_t);
    p->dpacked = device_alias(p->packed, p->packed, host_hint, &st_p);
    p->staged = st_t | (st_p << 1);
    return YAKSA_SUCCESS;
}

/* plan() for one yaksa_gb300_pup_t record: kind 0 packs, 1 unpacks, anything else is
 * refused (a corrupt record must not swap the buffer roles) */
static int plan_op(const yaksa_gb300_pup_t * o, yk_type * t, yaksa_info_t info, yk_plan * p)
{
    if (o->kind == 0)
        return plan(0, NULL, o->outbuf, (char *) o->inbuf, o->count, t, o->offset, o->maxbytes,
                    info, o->op, p);
    if (o->kind == 1)
        return plan(1, o->inbuf, NULL, (char *) o->outbuf, o->count, t, o->offset, o->maxbytes,
                    info, o->op, p);
    fprintf(stderr, "yaksa-gb300: request kind %d is neither pack (0) nor unpack (1)\n",
            (int) o->kind);
    return YAKSA_ERR__INTERNAL;
}

/* ------------------------------------------------------------------------- */
/* launch construction                                                       */
/* ------------------------------------------------------------------------- */

enum { YK_X_MEMCPY, YK_X_BYTES, YK_X_TYPED, YK_X_ORDERED };

typedef int (*yk_desc_getter)(yk_type * t, int typed, yk_devdesc ** out);

static int prepare_with(const yk_plan * p, char *typed, char *packed, yk_launch * L, int *kind,
                        int *sorted, yk_desc_getter get)
{
    yk_type *t = p->t;
    uintptr_t count = p->count, b0 = p->b0, n = p->b1 - p->b0;
    yaksa_op_t op = p->op;
    memset(L, 0, sizeof(*L));
    L->typed = typed;
    L->packed = packed;
    L->p0 = b0;
    L->nbytes = n;
    L->op = op;
    L->dir = p->dir;
    L->use64 = (p->b1 > YK_POS32_END);
    L->ldouble = t->needs_host_ops;
    *sorted = 0;
    if (op == YAKSA_OP__REPLACE && t->is_contig) {
        *kind = YK_X_MEMCPY;
        return YAKSA_SUCCESS;
    }
    int typed_op = (op != YAKSA_OP__REPLACE);
    yk_devdesc *dd;
    int rc = get(t, typed_op, &dd);
    if (rc)
        return rc;
    uint64_t ext = (uint64_t) (t->extent < 0 ? -t->extent : t->extent);
    int overlap = p->dir == 1 && (dd->may_overlap || (count > 1 && (int64_t) ext < dd->elem_span));
    yk_devdesc *ddo = dd;
    if (overlap && !typed_op) {
        /* ordered REPLACE uses the typed descriptor's element structure when the
         * sorted-block kernel applies to it */
        yk_devdesc *tdd;
        if (t->base_type > 0 && get(t, 1, &tdd) == YAKSA_SUCCESS && tdd->sorted_blocks)
            ddo = tdd;
    }
    yk_make_launch_desc(ddo, t, count, &L->desc);
    L->regular = -1;
    if (!L->use64 && L->desc.leaf == YK_LEAF_RUN && L->desc.nlev <= YK_REGULAR_MAX) {
        L->regular = L->desc.nlev;
        for (int i = 0; i < L->desc.nlev; i++)
            if (L->desc.lv[i].kind != YK_LV_VEC)
                L->regular = -1;
    }
    L->hidx = L->desc.leaf == YK_LEAF_RUN && L->desc.nlev == 1 &&
        L->desc.lv[0].kind == YK_LV_HIDX && L->desc.lv[0].tfb &&
        L->desc.lv[0].stride == (int64_t) L->desc.lv[0].cps && L->desc.run == L->desc.lv[0].cps;
    if (ddo == dd && !typed_op) {
        /* widest unit that every run, offset, pointer and range bound allows */
        int v = ddo->vec_align;
        v = YK_MIN(v, pow2_of((uint64_t) (uintptr_t) typed));
        v = YK_MIN(v, pow2_of((uint64_t) (uintptr_t) packed));
        v = YK_MIN(v, pow2_of(b0));
        v = YK_MIN(v, pow2_of(n));
        v = YK_MIN(v, pow2_of(t->size));
        if (count > 1)
            v = YK_MIN(v, pow2_of(ext));
        L->vec = v;
        L->typed_op = 0;
    } else {
        /* element granularity; alignment is checked per access in the kernel */
        L->typed_op = 1;
        L->vec = ddo->unit;
        if (!typed_op)
            L->op = YAKSA_OP__REPLACE;
    }
    if (overlap) {
        *kind = YK_X_ORDERED;
        *sorted = ddo->sorted_blocks && L->typed_op && L->desc.nlev == 1 &&
            L->desc.lv[0].kind == YK_LV_IDX &&
            ddo->elem_align >= yk_base_type_size(t->base_type);
        if (*sorted) {
            /* register-typed variant: both sides aligned to the element size */
            uint64_t es = (uint64_t) yk_base_type_size(L->desc.leaf_type);
            uint64_t a = (uint64_t) (uintptr_t) (typed + L->desc.base) | (uint64_t) (uintptr_t) packed |
                b0 | (uint64_t) ddo->elem_align;
            if (es && (a % es) == 0 && (uint64_t) ddo->elem_align >= es) {
                *sorted = 2;
                if (ddo->disp32)
                    *sorted |= YK_ORD_D32;
            }
        }
        /* one level whose every step is one run of the base type: the type's own IDX or
         * VEC level, or (count > 1) the element level over a type that is one run */
        if (__atomic_load_n(&R.red_mode, __ATOMIC_RELAXED) > 0 &&
            L->typed_op && L->desc.nlev == 1 && !L->use64 && L->desc.leaf == YK_LEAF_RUN &&
            L->desc.lv[0].cps == L->desc.run &&
            (L->desc.lv[0].kind == YK_LV_IDX || L->desc.lv[0].kind == YK_LV_VEC) &&
            L->desc.lv[0].cps < (1ull << 32) && yk_red_applies(L->desc.leaf_type, L->op)) {
            /* equal blocks, in any order or at a stride under their length, under an
             * order-independent integer operator: L2 reductions, when both sides sit on
             * the element size and the target is device memory (probed at the lowest
             * byte the request touches: the typed pointer itself may lie outside any
             * allocation, as with absolute displacements) */
            uint64_t es = (uint64_t) yk_base_type_size(L->desc.leaf_type);
            uint64_t a = (uint64_t) (uintptr_t) (typed + L->desc.base) | (uint64_t) (uintptr_t) packed |
                b0 | (uint64_t) ddo->elem_align;
            if (es && (a % es) == 0 && (uint64_t) ddo->elem_align >= es && device_memory(typed + p->lo))
                *sorted |= YK_ORD_RED;
        }
        if (!L->typed_op && !*sorted)
            L->vec = (int) YK_MIN((uint64_t) L->vec, (uint64_t) ddo->vec_align);
    } else {
        *kind = L->typed_op ? YK_X_TYPED : YK_X_BYTES;
    }
    return YAKSA_SUCCESS;
}

/* launch construction over the type's device-resident descriptors */
static int prepare(const yk_plan * p, char *typed, char *packed, yk_launch * L, int *kind,
                   int *sorted)
{
    return prepare_with(p, typed, packed, L, kind, sorted, yk_desc_get);
}

/* A pack of whole elements of one VEC level over a run of 17..47 bytes (not a multiple
 * of 16, so the byte kernels would take 4- or 8-byte units) that starts on 16 bytes in
 * every element: one thread per element, 16-byte loads (yk_cuda_launch_runs_pack).
 * YAKSA_GB300_RUNS_PACK=0 in the environment keeps such packs on the byte kernels. */
static int runs_pack_ok(const yk_launch * L)
{
    const uint64_t r = L->desc.run;
    return R.runs_pack && L->dir == 0 && !L->typed_op && !L->use64 && L->regular == 1 &&
        L->desc.leaf == YK_LEAF_RUN && L->desc.lv[0].kind == YK_LV_VEC && L->desc.lv[0].cps == r &&
        r > 16 && r < 48 && r % 16 && (L->vec == 4 || L->vec == 8) && r % (uint64_t) L->vec == 0 &&
        L->desc.lv[0].stride > 0 && L->desc.lv[0].stride % 16 == 0 &&
        ((uintptr_t) L->typed + (uintptr_t) L->desc.base) % 16 == 0 &&
        L->p0 % r == 0 && L->nbytes % r == 0 && L->nbytes / r > 0;
}

/* tune: pick the launch shape of the REPLACE byte kernels with the autotuner (off for
 * the no-allocation entry point, whose timing events would be a resource allocation) */
static int launch_prepared(const yk_plan * p, const yk_launch * L, int kind, int sorted,
                           cudaStream_t s, int tune)
{
    if (kind == YK_X_MEMCPY) {
        /* contiguous: the packed bytes are the memory bytes from true_lb */
        char *mem = L->typed + p->t->true_lb + L->p0;
        __atomic_add_fetch(&R.memcpy_calls, 1, __ATOMIC_RELAXED);
        return cuda_err(cudaMemcpyAsync(p->dir == 0 ? L->packed : mem,
                                        p->dir == 0 ? mem : L->packed, L->nbytes,
                                        cudaMemcpyDefault, s), "cudaMemcpyAsync");
    }
    __atomic_add_fetch(&R.launches, 1, __ATOMIC_RELAXED);
    const uint64_t units = L->nbytes / (uint64_t) L->vec;
    if (kind == YK_X_ORDERED || kind == YK_X_TYPED || (kind == YK_X_BYTES && L->hidx)) {
        /* the grid cap of the hindexed, typed-operator and sorted-block kernels; the class
         * is keyed by operator and base type as well */
        yk_tune_cfg cfg = { 0, 0, 0 };
        int probe = -1;
        const int fam = kind == YK_X_ORDERED ? YK_TUNE_OWNER : kind == YK_X_TYPED ? YK_TUNE_TYPED :
            L->dir == 1 ? YK_TUNE_HIDX_UNPACK : YK_TUNE_HIDX;
        const int hidx = fam == YK_TUNE_HIDX || fam == YK_TUNE_HIDX_UNPACK;
        if (fam == YK_TUNE_HIDX_UNPACK && R.tma_mode == 2) {
            cfg.variant = YK_VARIANT_BULK;      /* the test hook forces the bulk form */
        } else if (hidx && __atomic_load_n(&R.hidx_forced, __ATOMIC_ACQUIRE)) {
            cfg = R.hidx_cfg;                   /* the test hook forces a shape */
        } else if (tune && (kind != YK_X_ORDERED || sorted))
            probe = yk_tune_begin(yk_tune_key(fam, (int) L->op, L->desc.leaf_type * 17 + L->vec, L->dir,
                                              L->use64, units), fam, units, s, &cfg);
        int e = -1;
        if (cfg.variant == YK_VARIANT_BULK && (R.tma_mode || (hidx && R.hidx_forced)))
            e = yk_cuda_launch_hidx_bulk(L, s, cfg.ctas_per_sm);   /* -1: it does not apply */
        if (e == -1)
            e = kind == YK_X_ORDERED ? yk_cuda_launch_unpack_ordered(L, sorted, s, cfg.ctas_per_sm) :
                yk_cuda_launch_pup_cfg(L, s, cfg.units_per_thread, cfg.ctas_per_sm);
        yk_tune_end(probe, s);
        return cuda_err((cudaError_t) e, "kernel launch");
    }
    const int runs = kind == YK_X_BYTES && runs_pack_ok(L);
    /* a TMA form competes as a candidate of the autotuner (or is forced by the test hook) */
    const int tma = kind == YK_X_BYTES && R.tma_mode &&
        (R.tma_mode == 2 || (tune && units >= yk_tune_min_units())) && yk_cuda_tma_ok(L);
    if (tma && R.tma_mode == 2) {
        int e = yk_cuda_launch_tma(L, s, 0);
        if (e != -1)
            return cuda_err((cudaError_t) e, "kernel launch");
    }
    if (runs && !tma)
        return cuda_err((cudaError_t) yk_cuda_launch_runs_pack(L, (uint32_t) L->desc.run, s),
                        "kernel launch");
    yk_tune_cfg cfg = { 0, 0, runs ? YK_VARIANT_RUNS : YK_VARIANT_BYTES };
    int probe = -1;
    if (tune && kind == YK_X_BYTES) {
        const int fam = runs ? YK_TUNE_RUNS_TMA : tma ? YK_TUNE_SINGLE_TMA : YK_TUNE_SINGLE;
        probe = yk_tune_begin(yk_tune_key(fam, L->regular, L->vec, L->dir, L->use64, units), fam,
                              units, s, &cfg);
    }
    int e = cfg.variant == YK_VARIANT_TMA && tma ? yk_cuda_launch_tma(L, s, cfg.ctas_per_sm) : -1;
    if (e == -1)        /* not the TMA form, or its tensor map could not be encoded */
        e = runs && cfg.variant != YK_VARIANT_BYTES ?
            yk_cuda_launch_runs_pack(L, (uint32_t) L->desc.run, s) :
            yk_cuda_launch_pup_cfg(L, s, cfg.units_per_thread, cfg.ctas_per_sm);
    yk_tune_end(probe, s);
    return cuda_err((cudaError_t) e, "kernel launch");
}

/* L2-reduction form of overlapping unpacks: 0 never, 1 where it applies (default), a
 * negative mode leaves it as it is; *launches receives the form's launches so far */
int yaksa_gb300_debug_l2_reduce(int mode, unsigned long long *launches)
{
    if (mode > 1)
        return YAKSA_ERR__INTERNAL;
    if (mode >= 0)
        __atomic_store_n(&R.red_mode, mode, __ATOMIC_RELAXED);
    if (launches)
        *launches = yk_cuda_red_launches();
    return YAKSA_SUCCESS;
}

/* TMA forms: 0 never, 1 as autotuner candidates (default), 2 always where one exists */
int yaksa_gb300_debug_tma(int mode)
{
    if (mode < 0 || mode > 2)
        return YAKSA_ERR__INTERNAL;
    __atomic_store_n(&R.tma_mode, mode, __ATOMIC_RELAXED);
    return YAKSA_SUCCESS;
}

/* contiguous-block hindexed launches: variant < 0 lets the autotuner choose (the
 * default); otherwise every such launch takes {units, ctas, variant} -- YK_VARIANT_BYTES
 * (0) the shuffle-search kernel in the shape `units` names, YK_VARIANT_BULK (3) the
 * bulk-staged unpack (a pack, or a request outside its rules, takes the shuffle kernel) */
int yaksa_gb300_debug_hidx_shape(int variant, int units, int ctas)
{
    if (variant != YK_VARIANT_BYTES && variant != YK_VARIANT_BULK && variant >= 0)
        return YAKSA_ERR__INTERNAL;
    if (units < 0 || ctas < 0 || ctas > 64)
        return YAKSA_ERR__INTERNAL;
    if (variant < 0) {
        __atomic_store_n(&R.hidx_forced, 0, __ATOMIC_RELEASE);
        return YAKSA_SUCCESS;
    }
    pthread_mutex_lock(&R.mu);
    R.hidx_cfg.units_per_thread = units;
    R.hidx_cfg.ctas_per_sm = ctas;
    R.hidx_cfg.variant = variant;
    __atomic_store_n(&R.hidx_forced, 1, __ATOMIC_RELEASE);
    pthread_mutex_unlock(&R.mu);
    return YAKSA_SUCCESS;
}

static int enqueue(const yk_plan * p, char *typed, char *packed, cudaStream_t s)
{
    yk_launch L;
    int kind, sorted;
    int rc = prepare(p, typed, packed, &L, &kind, &sorted);
    if (rc)
        return rc;
    return launch_prepared(p, &L, kind, sorted, s, 1);
}

/* ------------------------------------------------------------------------- */
/* staging: buffers the GPU cannot address                                    */
/* ------------------------------------------------------------------------- */

/* A ring of fixed slabs (the reference stages through 16 x 1 MiB pinned and device
 * buffers, src/backend/src/yaksuri.h:25-26, src/util/yaksu_buffer_pool.c:77-230).  Each
 * slab is a device half and a pinned-host half, each holding a packed chunk and a typed
 * chunk.  A staged request is cut into chunks; chunk i uses slab i mod nslabs and runs
 * as three event-chained stages on three library streams, so that copies of one chunk
 * overlap the kernel of the next:
 *   in:   wait for the slab to be free; user buffer -> pinned slab (a host function:
 *         plain memcpy on the driver's callback thread), pinned -> device slab;
 *   run:  the chunk's kernel, device slab in place of the unaddressable buffer;
 *   out:  device slab -> pinned slab -> user buffer (host function); the slab is free.
 * Everything is enqueued before the call returns: yaksa_ipack never waits, and the
 * request's event follows the last host copy (the reference's progress engine instead
 * polls its chunks from yaksa_request_test/wait, src/backend/src/yaksuri_progress.c:
 * 2862-3088).  A typed chunk is the span its elements touch, rewritten whole on the way
 * out (bytes of the span outside the typemap get back the values read at the chunk's
 * start).  An element whose span exceeds a slab is staged through one stream-ordered
 * allocation of that span instead. */

#define YK_STAGE_MAX_SLABS 256

typedef struct {
    pthread_mutex_t mu;
    int ready;
    int nslabs;
    size_t slab;                /* bytes of one side (packed or typed) of one slab */
    char *dev, *host;           /* nslabs x 2 x (slab + 16) */
    int host_pageable;          /* host half from malloc (a wait kernel), else pinned */
    cudaEvent_t ev_in[YK_STAGE_MAX_SLABS], ev_run[YK_STAGE_MAX_SLABS],
        ev_free[YK_STAGE_MAX_SLABS], ev_start, ev_end;
    cudaStream_t s_in, s_run, s_out;
    unsigned next;
    uint64_t chunks;
} yk_stage_ring;

static yk_stage_ring ST = { .mu = PTHREAD_MUTEX_INITIALIZER };

/* caller holds ST.mu */
static int stage_ready(void)
{
    if (ST.ready)
        return YAKSA_SUCCESS;
    const char *e = getenv("YAKSA_GB300_STAGE_SLABS");
    ST.nslabs = e ? atoi(e) : 16;
    if (ST.nslabs < 2 || ST.nslabs > YK_STAGE_MAX_SLABS)
        ST.nslabs = 16;
    e = getenv("YAKSA_GB300_STAGE_SLAB_KIB");
    long kib = e ? atol(e) : 1024;
    if (kib < 64 || kib > (1 << 20))
        kib = 1024;
    ST.slab = (size_t) kib << 10;
    size_t bytes = (size_t) ST.nslabs * 2 * (ST.slab + 16);
    if (yk_fail_injected() || cudaMalloc((void **) &ST.dev, bytes) != cudaSuccess) {
        ST.dev = NULL;
        return YAKSA_ERR__OUT_OF_MEM;
    }
    /* with a wait kernel the host half is plain host memory: pinning it
     * (cudaHostAlloc) would synchronize the device against that kernel */
    ST.host_pageable = R.has_wait_kernel;
    if (ST.host_pageable)
        ST.host = yk_fail_injected() ? NULL : malloc(bytes);
    else if (yk_fail_injected() || cudaHostAlloc((void **) &ST.host, bytes, cudaHostAllocPortable) != cudaSuccess)
        ST.host = NULL;
    if (!ST.host) {
        cudaFree(ST.dev);
        ST.dev = ST.host = NULL;
        return YAKSA_ERR__OUT_OF_MEM;
    }
    cudaError_t c = cudaSuccess;
    for (int k = 0; k < ST.nslabs && c == cudaSuccess; k++) {
        c = cudaEventCreateWithFlags(&ST.ev_in[k], cudaEventDisableTiming);
        if (c == cudaSuccess)
            c = cudaEventCreateWithFlags(&ST.ev_run[k], cudaEventDisableTiming);
        if (c == cudaSuccess)
            c = cudaEventCreateWithFlags(&ST.ev_free[k], cudaEventDisableTiming);
    }
    if (c == cudaSuccess)
        c = cudaEventCreateWithFlags(&ST.ev_start, cudaEventDisableTiming);
    if (c == cudaSuccess)
        c = cudaEventCreateWithFlags(&ST.ev_end, cudaEventDisableTiming);
    if (c == cudaSuccess)
        c = cudaStreamCreateWithFlags(&ST.s_in, cudaStreamNonBlocking);
    if (c == cudaSuccess)
        c = cudaStreamCreateWithFlags(&ST.s_run, cudaStreamNonBlocking);
    if (c == cudaSuccess)
        c = cudaStreamCreateWithFlags(&ST.s_out, cudaStreamNonBlocking);
    if (c != cudaSuccess)
        return cuda_err(c, "staging ring setup");
    ST.ready = 1;
    return YAKSA_SUCCESS;
}

static void stage_finalize(void)
{
    pthread_mutex_lock(&ST.mu);
    if (ST.ready) {
        cudaStreamSynchronize(ST.s_in);
        cudaStreamSynchronize(ST.s_run);
        cudaStreamSynchronize(ST.s_out);
        for (int k = 0; k < ST.nslabs; k++) {
            cudaEventDestroy(ST.ev_in[k]);
            cudaEventDestroy(ST.ev_run[k]);
            cudaEventDestroy(ST.ev_free[k]);
        }
        cudaEventDestroy(ST.ev_start);
        cudaEventDestroy(ST.ev_end);
        cudaStreamDestroy(ST.s_in);
        cudaStreamDestroy(ST.s_run);
        cudaStreamDestroy(ST.s_out);
        cudaFree(ST.dev);
        if (ST.host_pageable)
            free(ST.host);
        else
            cudaFreeHost(ST.host);
        ST.dev = ST.host = NULL;
        ST.ready = 0;
    }
    pthread_mutex_unlock(&ST.mu);
}

typedef struct {
    void *dst;
    const void *src;
    size_t n;
} yk_hcopy;

static void CUDART_CB hcopy_fn(void *arg)
{
    yk_hcopy *c = (yk_hcopy *) arg;
    memcpy(c->dst, c->src, c->n);
    free(c);
}

/* a host-side copy in stream order (user memory the GPU cannot address <-> pinned slab) */
static int host_copy(cudaStream_t s, void *dst, const void *src, size_t n)
{
    yk_hcopy *c = malloc(sizeof(*c));
    if (!c)
        return YAKSA_ERR__OUT_OF_MEM;
    c->dst = dst;
    c->src = src;
    c->n = n;
    cudaError_t e = cudaLaunchHostFunc(s, hcopy_fn, c);
    if (e != cudaSuccess) {
        free(c);
        return cuda_err(e, "cudaLaunchHostFunc");
    }
    return YAKSA_SUCCESS;
}

/* typed bytes [lo, hi) touched by the packed range [b0, b1) of (count, t), relative to the
 * typed pointer (the same bounds plan() computes for the whole request) */
static void typed_span(const yk_type * t, uintptr_t b0, uintptr_t b1, int64_t * lo, int64_t * hi)
{
    uintptr_t e0 = b0 / t->size, e1 = (b1 + t->size - 1) / t->size;
    int64_t ext = t->extent;
    *lo = (ext >= 0 ? (int64_t) e0 * ext : (int64_t) (e1 - 1) * ext) + t->true_lb;
    *hi = (ext >= 0 ? (int64_t) (e1 - 1) * ext : (int64_t) e0 * ext) + t->true_ub;
}

/* end of the chunk that starts at packed byte b: at most `slab` packed bytes (when the
 * packed side is staged) and a typed span of at most `slab` bytes (when the typed side
 * is), on builtin boundaries; returns b when not even one element's span fits */
static uintptr_t chunk_end(const yk_plan * p, uintptr_t b, size_t slab)
{
    yk_type *t = p->t;
    uintptr_t e = YK_MIN(p->b1, b + slab);
    if (p->staged & 1) {
        /* whole elements while their span fits */
        uint64_t ext = (uint64_t) (t->extent < 0 ? -t->extent : t->extent);
        uint64_t span1 = (uint64_t) (t->true_ub - t->true_lb);
        if (span1 > slab)
            return b;
        uint64_t m = ext ? 1 + (slab - span1) / ext : p->count;
        uintptr_t eb = b / t->size;
        uintptr_t lim = (eb + m) * t->size;
        e = YK_MIN(e, lim);
        while (e > b) {
            int64_t lo, hi;
            typed_span(t, b, e, &lo, &hi);
            if ((uint64_t) (hi - lo) <= slab)
                break;
            e = b + (e - b) / 2;
        }
    }
    uintptr_t f = yk_builtin_floor(t, p->count, e);
    return f > b ? f : (e == p->b1 ? e : f);
}

/* An element whose typed span exceeds a slab: one stream-ordered allocation of the span
 * (and of the packed range when that side is staged too), released in stream order. */
static int stage_oversize(const yk_plan * p)
{
    cudaStream_t s = ST.s_run;
    uintptr_t n = p->b1 - p->b0;
    size_t span = (size_t) (p->hi - p->lo);
    char *dt = p->dtyped, *dp = p->dpacked;
    void *scr_t = NULL, *scr_p = NULL;
    int rc = YAKSA_SUCCESS;
    if (p->staged & 1) {
        rc = yk_fail_injected() ? YAKSA_ERR__OUT_OF_MEM :
            cuda_err(cudaMallocAsync(&scr_t, span, s), "cudaMallocAsync");
        if (!rc)
            rc = cuda_err(cudaMemcpyAsync(scr_t, p->typed + p->lo, span, cudaMemcpyHostToDevice, s),
                          "stage in");
        dt = (char *) scr_t - p->lo;
    }
    if (!rc && (p->staged & 2)) {
        rc = yk_fail_injected() ? YAKSA_ERR__OUT_OF_MEM :
            cuda_err(cudaMallocAsync(&scr_p, n, s), "cudaMallocAsync");
        if (!rc && (p->dir == 1 || p->op != YAKSA_OP__REPLACE))
            rc = cuda_err(cudaMemcpyAsync(scr_p, p->packed, n, cudaMemcpyHostToDevice, s), "stage in");
        dp = scr_p;
    }
    if (!rc)
        rc = enqueue(p, dt, dp, s);
    if (!rc && p->dir == 0 && (p->staged & 2))
        rc = cuda_err(cudaMemcpyAsync(p->packed, scr_p, n, cudaMemcpyDeviceToHost, s), "stage out");
    if (!rc && p->dir == 1 && (p->staged & 1))
        rc = cuda_err(cudaMemcpyAsync(p->typed + p->lo, scr_t, span, cudaMemcpyDeviceToHost, s),
                      "stage out");
    if (scr_t)
        cudaFreeAsync(scr_t, s);
    if (scr_p)
        cudaFreeAsync(scr_p, s);
    return rc;
}

/* one chunk [cb0, cb1) through slab k (caller holds ST.mu); prev >= 0: the slab of the
 * previous chunk, whose copy out this chunk's copy in must follow (typed spans that a
 * staged unpack writes back may overlap from chunk to chunk) */
static int stage_chunk(const yk_plan * p, uintptr_t cb0, uintptr_t cb1, unsigned k, int prev)
{
    const size_t side = ST.slab + 16;
    char *dslab = ST.dev + (size_t) k * 2 * side, *hslab = ST.host + (size_t) k * 2 * side;
    char *dpk = dslab, *hpk = hslab;            /* packed half */
    yk_plan q = *p;
    q.b0 = cb0;
    q.b1 = cb1;
    uintptr_t n = cb1 - cb0;
    int64_t tlo = 0, thi = 0;
    size_t tmis = 0;
    char *dty = NULL, *hty = NULL;              /* typed half, same alignment mod 16 */
    if (p->staged & 1) {
        typed_span(p->t, cb0, cb1, &tlo, &thi);
        tmis = (size_t) ((uintptr_t) (p->typed + tlo) & 15);
        dty = dslab + side + tmis;
        hty = hslab + side + tmis;
        q.dtyped = dty - tlo;
    } else {
        q.dtyped = p->dtyped;
    }
    q.dpacked = (p->staged & 2) ? dpk : p->dpacked + (cb0 - p->b0);
    char *upk = p->packed + (cb0 - p->b0);       /* the caller's packed bytes of the chunk */
    int rc = cuda_err(cudaStreamWaitEvent(ST.s_in, ST.ev_free[k], 0), "stage wait");
    if (!rc && prev >= 0)
        rc = cuda_err(cudaStreamWaitEvent(ST.s_in, ST.ev_free[prev], 0), "stage wait");
    /* in: what the kernel reads from staged memory */
    if (!rc && (p->staged & 2) && (p->dir == 1 || p->op != YAKSA_OP__REPLACE)) {
        rc = host_copy(ST.s_in, hpk, upk, n);
        if (!rc)
            rc = cuda_err(cudaMemcpyAsync(dpk, hpk, n, cudaMemcpyHostToDevice, ST.s_in), "stage in");
    }
    if (!rc && (p->staged & 1)) {
        rc = host_copy(ST.s_in, hty, p->typed + tlo, (size_t) (thi - tlo));
        if (!rc)
            rc = cuda_err(cudaMemcpyAsync(dty, hty, (size_t) (thi - tlo), cudaMemcpyHostToDevice,
                                          ST.s_in), "stage in");
    }
    if (!rc)
        rc = cuda_err(cudaEventRecord(ST.ev_in[k], ST.s_in), "stage record");
    /* run */
    if (!rc)
        rc = cuda_err(cudaStreamWaitEvent(ST.s_run, ST.ev_in[k], 0), "stage wait");
    if (!rc)
        rc = enqueue(&q, q.dtyped, q.dpacked, ST.s_run);
    if (!rc)
        rc = cuda_err(cudaEventRecord(ST.ev_run[k], ST.s_run), "stage record");
    /* out: what the kernel wrote to staged memory */
    if (!rc)
        rc = cuda_err(cudaStreamWaitEvent(ST.s_out, ST.ev_run[k], 0), "stage wait");
    if (!rc && p->dir == 0 && (p->staged & 2)) {
        rc = cuda_err(cudaMemcpyAsync(hpk, dpk, n, cudaMemcpyDeviceToHost, ST.s_out), "stage out");
        if (!rc)
            rc = host_copy(ST.s_out, upk, hpk, n);
    }
    if (!rc && p->dir == 1 && (p->staged & 1)) {
        rc = cuda_err(cudaMemcpyAsync(hty, dty, (size_t) (thi - tlo), cudaMemcpyDeviceToHost, ST.s_out),
                      "stage out");
        if (!rc)
            rc = host_copy(ST.s_out, p->typed + tlo, hty, (size_t) (thi - tlo));
    }
    if (!rc)
        rc = cuda_err(cudaEventRecord(ST.ev_free[k], ST.s_out), "stage record");
    return rc;
}

/* A request with a buffer the GPU cannot address, ordered after the work already on
 * stream s and before anything enqueued on s later; nothing waits on the host. */
static int run_staged(const yk_plan * p, cudaStream_t s)
{
    __atomic_add_fetch(&R.staged_calls, 1, __ATOMIC_RELAXED);
    pthread_mutex_lock(&ST.mu);
    int rc = stage_ready();
    if (!rc)
        rc = cuda_err(cudaEventRecord(ST.ev_start, s), "stage record");
    if (!rc)
        rc = cuda_err(cudaStreamWaitEvent(ST.s_in, ST.ev_start, 0), "stage wait");
    if (!rc)
        rc = cuda_err(cudaStreamWaitEvent(ST.s_run, ST.ev_start, 0), "stage wait");
    int prev = -1;
    for (uintptr_t b = p->b0; !rc && b < p->b1;) {
        uintptr_t e = chunk_end(p, b, ST.slab);
        if (e <= b) {
            /* one element's typed span is larger than a slab: the whole request at once,
             * after every chunk enqueued so far (stream order on s_run) */
            yk_plan q = *p;
            q.b0 = b;
            typed_span(p->t, q.b0, q.b1, &q.lo, &q.hi);
            if (p->staged & 2)
                q.packed = p->packed + (b - p->b0);
            if (!(p->staged & 2))
                q.dpacked = p->dpacked + (b - p->b0);
            rc = stage_oversize(&q);
            if (!rc)
                rc = cuda_err(cudaEventRecord(ST.ev_end, ST.s_run), "stage record");
            if (!rc)
                rc = cuda_err(cudaStreamWaitEvent(ST.s_out, ST.ev_end, 0), "stage wait");
            break;
        }
        unsigned k = ST.next++ % (unsigned) ST.nslabs;
        rc = stage_chunk(p, b, e, k, (p->dir == 1 && (p->staged & 1)) ? prev : -1);
        prev = (int) k;
        ST.chunks++;
        b = e;
    }
    /* s continues after the last copy out */
    if (!rc)
        rc = cuda_err(cudaEventRecord(ST.ev_end, ST.s_out), "stage record");
    if (!rc)
        rc = cuda_err(cudaStreamWaitEvent(s, ST.ev_end, 0), "stage wait");
    pthread_mutex_unlock(&ST.mu);
    return rc;
}

/* completion for nonblocking / blocking modes: one pooled event */
static int complete(yk_type * t, int mode, cudaStream_t s, yaksa_request_t * request)
{
    if (mode == YK_MODE_STREAM)
        return YAKSA_SUCCESS;
    cudaEvent_t ev;
    int rc = event_get(&ev);
    if (rc)
        return rc;
    rc = cuda_err(cudaEventRecord(ev, s), "cudaEventRecord");
    if (rc) {
        event_put(ev);
        return rc;
    }
    if (mode == YK_MODE_BLOCKING || !request) {
        rc = cuda_err(cudaEventSynchronize(ev), "kernel completion");
        event_put(ev);
        return rc;
    }
    if (t)
        yk_type_ref(t);
    rc = request_new(ev, t, NULL, NULL, request);
    if (rc) {
        cudaEventSynchronize(ev);
        event_put(ev);
        if (t)
            yk_type_unref(t);
    }
    return rc;
}

static int pup(int dir, const void *packed_in, void *packed_out, char *typed, uintptr_t count,
               yk_type * t, uintptr_t offset, uintptr_t maxbytes, uintptr_t * actual,
               yk_info * info, yaksa_op_t op, int mode, void *stream, yaksa_request_t * request);

/* every public pack/unpack call is one NVTX range (a no-op unless a tool is attached) */
int yk_pup(int dir, const void *packed_in, void *packed_out, char *typed, uintptr_t count,
           yk_type * t, uintptr_t offset, uintptr_t maxbytes, uintptr_t * actual,
           yk_info * info, yaksa_op_t op, int mode, void *stream, yaksa_request_t * request)
{
    nvtxRangePushA(dir ? "yaksa unpack" : "yaksa pack");
    int rc = pup(dir, packed_in, packed_out, typed, count, t, offset, maxbytes, actual, info, op,
                 mode, stream, request);
    nvtxRangePop();
    return rc;
}

static int pup(int dir, const void *packed_in, void *packed_out, char *typed, uintptr_t count,
               yk_type * t, uintptr_t offset, uintptr_t maxbytes, uintptr_t * actual,
               yk_info * info, yaksa_op_t op, int mode, void *stream, yaksa_request_t * request)
{
    if (request)
        *request = YAKSA_REQUEST__NULL;
    *actual = 0;
    yk_plan p;
    int rc = plan(dir, packed_in, packed_out, typed, count, t, offset, maxbytes, info, op, &p);
    if (rc || p.b1 == p.b0)
        return rc;
    cudaStream_t s = (mode == YK_MODE_STREAM && stream) ? *(cudaStream_t *) stream : lib_stream();
    if (p.staged) {
        rc = run_staged(&p, s);
    } else {
        __atomic_add_fetch(&R.direct_calls, 1, __ATOMIC_RELAXED);
        rc = enqueue(&p, p.dtyped, p.dpacked, s);
    }
    if (rc)
        return rc;
    *actual = p.b1 - p.b0;
    return complete(t, mode, s, request);
}

/* ------------------------------------------------------------------------- */
/* public pack/unpack (yaksa.h.in:484-575)                                    */
/* ------------------------------------------------------------------------- */

#define TYPE_OR_FAIL(h, t) yk_type *t = yk_type_get(h); if (!t) return YAKSA_ERR__INTERNAL

int yaksa_ipack(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
                void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
                yaksa_info_t info, yaksa_op_t op, yaksa_request_t * request)
{
    *request = YAKSA_REQUEST__NULL;
    *actual_pack_bytes = 0;
    if (incount == 0)
        return YAKSA_SUCCESS;
    TYPE_OR_FAIL(type, t);
    return yk_pup(0, NULL, outbuf, (char *) inbuf, incount, t, inoffset, max_pack_bytes,
                  actual_pack_bytes, info, op, YK_MODE_NONBLOCKING, NULL, request);
}

int yaksa_pack(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
               void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
               yaksa_info_t info, yaksa_op_t op)
{
    *actual_pack_bytes = 0;
    if (incount == 0)
        return YAKSA_SUCCESS;
    TYPE_OR_FAIL(type, t);
    return yk_pup(0, NULL, outbuf, (char *) inbuf, incount, t, inoffset, max_pack_bytes,
                  actual_pack_bytes, info, op, YK_MODE_BLOCKING, NULL, NULL);
}

int yaksa_pack_stream(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
                      void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
                      yaksa_info_t info, yaksa_op_t op, void *stream)
{
    *actual_pack_bytes = 0;
    if (incount == 0)
        return YAKSA_SUCCESS;
    TYPE_OR_FAIL(type, t);
    return yk_pup(0, NULL, outbuf, (char *) inbuf, incount, t, inoffset, max_pack_bytes,
                  actual_pack_bytes, info, op, YK_MODE_STREAM, stream, NULL);
}

int yaksa_iunpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                  yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                  yaksa_info_t info, yaksa_op_t op, yaksa_request_t * request)
{
    *request = YAKSA_REQUEST__NULL;
    *actual_unpack_bytes = 0;
    if (outcount == 0)
        return YAKSA_SUCCESS;
    TYPE_OR_FAIL(type, t);
    return yk_pup(1, inbuf, NULL, (char *) outbuf, outcount, t, outoffset, insize,
                  actual_unpack_bytes, info, op, YK_MODE_NONBLOCKING, NULL, request);
}

int yaksa_unpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                 yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                 yaksa_info_t info, yaksa_op_t op)
{
    *actual_unpack_bytes = 0;
    if (outcount == 0)
        return YAKSA_SUCCESS;
    TYPE_OR_FAIL(type, t);
    return yk_pup(1, inbuf, NULL, (char *) outbuf, outcount, t, outoffset, insize,
                  actual_unpack_bytes, info, op, YK_MODE_BLOCKING, NULL, NULL);
}

int yaksa_unpack_stream(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                        yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                        yaksa_info_t info, yaksa_op_t op, void *stream)
{
    *actual_unpack_bytes = 0;
    if (outcount == 0)
        return YAKSA_SUCCESS;
    TYPE_OR_FAIL(type, t);
    return yk_pup(1, inbuf, NULL, (char *) outbuf, outcount, t, outoffset, insize,
                  actual_unpack_bytes, info, op, YK_MODE_STREAM, stream, NULL);
}

/* ------------------------------------------------------------------------- */
/* batches: many independent requests, one launch for the byte-moving ones    */
/* ------------------------------------------------------------------------- */

static uint64_t gcd_u64(uint64_t a, uint64_t b)
{
    while (b) {
        uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

/* Tile order of a batch launch: multiplying by the integer nearest 0.618 x total that
 * is coprime with the total (Fibonacci hashing) permutes the tiles so that every
 * wave of CTAs holds tiles of every request in proportion to its size. */
static uint32_t tile_multiplier(uint64_t total)
{
    if (total < 3)
        return 1;
    uint64_t m = (uint64_t) ((double) total * 0.6180339887498949);
    if (m < 2)
        m = 2;
    while (gcd_u64(m, total) != 1)
        m++;
    return m < total && m <= 0xffffffffull ? (uint32_t) m : 1;
}

/* One launch per group of at most YK_BATCH_MAX requests of one shape class
 * (regular nests, everything else). */
static int flush_class(yk_launch * ls, int n, int regular, cudaStream_t s)
{
    static __thread yk_batch B;
    for (int i0 = 0; i0 < n; i0 += YK_BATCH_MAX) {
        int m = YK_MIN(YK_BATCH_MAX, n - i0);
        uint64_t units = 0;
        int wide = 0;
        for (int i = 0; i < m; i++) {
            units += ls[i0 + i].nbytes / (uint64_t) ls[i0 + i].vec;
            wide |= ls[i0 + i].use64;
        }
        const int fam = regular ? YK_TUNE_BATCH_REGULAR : YK_TUNE_BATCH;
        yk_tune_cfg cfg;
        int probe = yk_tune_begin(yk_tune_key(fam, regular ? 0 : -1, 0, 0, wide, units), fam, units,
                                  s, &cfg);
        int u = regular ? 1 : cfg.units_per_thread ? cfg.units_per_thread :
            yk_cuda_batch_units_per_thread(units);
        B.n = m;
        B.tile_start[0] = 0;
        for (int i = 0; i < m; i++) {
            B.req[i] = ls[i0 + i];
            B.tile_start[i + 1] = B.tile_start[i] +
                yk_cuda_tiles(ls[i0 + i].nbytes / (uint64_t) ls[i0 + i].vec, u);
        }
        B.tile_mul = m > 1 ? tile_multiplier(B.tile_start[m]) : 1;
        __atomic_add_fetch(&R.launches, 1, __ATOMIC_RELAXED);
        int rc = cuda_err((cudaError_t) yk_cuda_launch_batch(&B, u, regular, cfg.ctas_per_sm, s),
                          "batch launch");
        yk_tune_end(probe, s);
        if (rc)
            return rc;
    }
    return YAKSA_SUCCESS;
}

static int flush_batch(yk_launch * ls, int n, cudaStream_t s)
{
    /* regular requests first (stable partition), then the rest */
    yk_launch *tmp = malloc(sizeof(yk_launch) * (n > 0 ? n : 1));
    if (!tmp)
        return YAKSA_ERR__OUT_OF_MEM;
    int nr = 0, ng = 0;
    for (int i = 0; i < n; i++)
        if (ls[i].regular >= 0)
            tmp[nr++] = ls[i];
    for (int i = 0; i < n; i++)
        if (ls[i].regular < 0)
            tmp[nr + ng++] = ls[i];
    int rc = YAKSA_SUCCESS;
    if (nr)
        rc = flush_class(tmp, nr, 1, s);
    if (!rc && ng)
        rc = flush_class(tmp + nr, ng, 0, s);
    free(tmp);
    return rc;
}

static int batch_run_ranges(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info, cudaStream_t s);

static int batch_run(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info, cudaStream_t s)
{
    nvtxRangePushA("yaksa batch");
    int rc = batch_run_ranges(ops, n, info, s);
    nvtxRangePop();
    return rc;
}

static int batch_run_ranges(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info, cudaStream_t s)
{
    yk_launch *ls = malloc(sizeof(yk_launch) * (n > 0 ? n : 1));
    if (!ls)
        return YAKSA_ERR__OUT_OF_MEM;
    int nb = 0, rc = YAKSA_SUCCESS;
    for (int i = 0; i < n && !rc; i++) {
        yaksa_gb300_pup_t *o = &ops[i];
        o->actual = 0;
        if (o->count == 0)
            continue;
        yk_type *t = yk_type_get(o->type);
        if (!t) {
            rc = YAKSA_ERR__INTERNAL;
            break;
        }
        yk_plan p;
        rc = plan_op(o, t, info, &p);
        if (rc || p.b1 == p.b0)
            continue;
        o->actual = p.b1 - p.b0;
        if (p.staged) {
            rc = run_staged(&p, s);
            continue;
        }
        __atomic_add_fetch(&R.direct_calls, 1, __ATOMIC_RELAXED);
        int kind, sorted;
        rc = prepare(&p, p.dtyped, p.dpacked, &ls[nb], &kind, &sorted);
        if (rc)
            break;
        if (kind == YK_X_BYTES && !ls[nb].use64 && !ls[nb].hidx)
            nb++;
        else
            rc = launch_prepared(&p, &ls[nb], kind, sorted, s, 1);
    }
    if (!rc && nb)
        rc = flush_batch(ls, nb, s);
    free(ls);
    return rc;
}

int yaksa_gb300_pup_batch_stream(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info, void *stream)
{
    int rc = runtime_ready();
    if (rc)
        return rc;
    cudaStream_t s = stream ? *(cudaStream_t *) stream : lib_stream();
    return batch_run(ops, n, info, s);
}

int yaksa_gb300_pup_batch(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info)
{
    int rc = runtime_ready();
    if (rc)
        return rc;
    cudaStream_t s = lib_stream();
    rc = batch_run(ops, n, info, s);
    if (rc)
        return rc;
    return complete(NULL, YK_MODE_BLOCKING, s, NULL);
}

int yaksa_gb300_ipup_batch(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info,
                           yaksa_request_t * request)
{
    *request = YAKSA_REQUEST__NULL;
    int rc = runtime_ready();
    if (rc)
        return rc;
    cudaStream_t s = lib_stream();
    rc = batch_run(ops, n, info, s);
    if (rc)
        return rc;
    return complete(NULL, YK_MODE_NONBLOCKING, s, request);
}

/* ------------------------------------------------------------------------- */
/* one pack/unpack that allocates nothing (no counterpart in the reference)   */
/* ------------------------------------------------------------------------- */

/* For callers that must not allocate device memory: a library sharing the device
 * with an application allocator that owns all of it, or code issuing requests beside
 * a resident persistent kernel, where the cudaFree that eventually releases a type's
 * table allocation would synchronize the device.  The request runs the plain path's
 * kernels; the type's tables (host copy, kept with the type) are written into the
 * static scratch of yk_noalloc.cu on the caller's stream just before the launch. */

#define YK_TABLE_PTRS(d, X)                                                   \
    do {                                                                      \
        for (int i_ = 0; i_ < (d)->nlev; i_++) {                              \
            X((d)->lv[i_].disp);                                              \
            X((d)->lv[i_].pfx);                                               \
            X((d)->lv[i_].tfb);                                               \
        }                                                                     \
        X((d)->seg_off);                                                      \
        X((d)->seg_pfx);                                                      \
        X((d)->seg_type);                                                     \
    } while (0)

static int desc_tables_in(const yk_desc * d, const char *h, uint64_t n)
{
    int in = 0;
#define YK_IN(p) in |= (p) && (const char *) (p) >= h && (const char *) (p) < h + n
    YK_TABLE_PTRS(d, YK_IN);
#undef YK_IN
    return in;
}

static void desc_rebase(yk_desc * d, const char *h, char *scr)
{
#define YK_REBASE(p) if (p) (p) = (void *) (scr + ((const char *) (p) - h))
    YK_TABLE_PTRS(d, YK_REBASE);
#undef YK_REBASE
}

int yaksa_gb300_pup_noalloc(yaksa_gb300_pup_t * o, void *stream)
{
    o->actual = 0;
    yk_type *t = yk_type_get(o->type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    yk_plan p;
    int rc = plan_op(o, t, NULL, &p);
    if (rc || p.b1 == p.b0)
        return rc;
    if (p.staged) {
        fprintf(stderr, "yaksa-gb300: yaksa_gb300_pup_noalloc: a buffer is not addressable "
                "by the GPU and staging it would need device memory\n");
        return YAKSA_ERR__NOT_SUPPORTED;
    }
    void *scr = NULL;
    size_t scr_bytes = 0;
    rc = cuda_err((cudaError_t) yk_noalloc_scratch(&scr, &scr_bytes), "static scratch setup");
    if (rc)
        return rc;
    cudaStream_t s = stream ? *(cudaStream_t *) stream : (cudaStream_t) 0;
    yk_launch L;
    int kind, sorted;
    rc = prepare_with(&p, p.dtyped, p.dpacked, &L, &kind, &sorted, yk_desc_get_host);
    if (rc)
        return rc;
    if (kind != YK_X_MEMCPY) {
        /* the launch reads the tables of exactly one host descriptor (or none) */
        yk_devdesc *src = NULL;
        for (int typed = 0; typed < 2 && !src; typed++) {
            yk_devdesc *dd = typed ? &t->host_typed_desc : &t->host_bytes_desc;
            if (dd->built && dd->dev_tables &&
                desc_tables_in(&L.desc, (const char *) dd->dev_tables, dd->table_bytes))
                src = dd;
        }
        if (src) {
            if (src->table_bytes > scr_bytes) {
                fprintf(stderr, "yaksa-gb300: yaksa_gb300_pup_noalloc: the type's descriptor "
                        "tables take %llu bytes, more than the %zu-byte static scratch\n",
                        (unsigned long long) src->table_bytes, scr_bytes);
                return YAKSA_ERR__NOT_SUPPORTED;
            }
            rc = cuda_err(cudaMemcpyAsync(scr, src->dev_tables, src->table_bytes,
                                          cudaMemcpyHostToDevice, s), "table copy");
            if (rc)
                return rc;
            desc_rebase(&L.desc, (const char *) src->dev_tables, (char *) scr);
        }
    }
    rc = launch_prepared(&p, &L, kind, sorted, s, 0);
    if (!rc)
        o->actual = p.b1 - p.b0;
    return rc;
}

/* ------------------------------------------------------------------------- */
/* persistent request server                                                 */
/* ------------------------------------------------------------------------- */

/* packed bytes per work item; YAKSA_GB300_SERVER_ITEM_KIB in the environment overrides
 * it (a power of two from 16 KiB to 16 MiB).  On the mixed request stream 256 KiB gave
 * the lowest p99 at 97% of the 512 KiB capacity; 128 KiB raised small-request p99. */
#define YK_ITEM_BYTES (256u << 10)

typedef struct {
    uint64_t seq;               /* request sequence number (ticket) */
    uint64_t item0, nitems;
    uint64_t bytes;
    yk_type *t;
    int busy;
    int64_t user;               /* the serving loop's index of the request (-1: none) */
} yk_srv_slot;

/* a request planned for the server: its launch record, work-item kind and granule */
typedef struct {
    yk_type *t;
    yk_plan p;
    yk_launch L;
    uint32_t skind;
    uint64_t gran;
    uint64_t key;               /* its class for the item-cut tuner (0: not tuned) */
} yk_srv_req;

/* requests below this size are cut the same way by every candidate: not tuned */
#define YK_SRV_TUNE_MIN (256u << 10)

struct yaksa_gb300_server_s {
    pthread_mutex_t mu;
    int ctas, running;
    cudaStream_t stream;
    uint32_t qr, qi;
    yk_launch *reqs;            /* pinned, mapped */
    yk_item *items;             /* pinned, mapped */
    unsigned long long *req_done;       /* pinned, mapped: items finished per request slot */
    uint64_t *req_nitems;       /* pinned, mapped: items per request slot */
    unsigned long long *cq;     /* pinned, mapped: completion queue written by the GPU */
    unsigned long long *req_busy;       /* pinned, mapped: summed item busy time (ns) of
                                         * timed requests */
    uint64_t cq_head;           /* next completion queue entry the host reads */
    uint64_t *ctl;              /* pinned, mapped: [0] items published, [1] stop, [2] status */
    unsigned long long *next_item;      /* device: the lanes' claim counters, then the
                                         * completion queue's tail */
    yk_srv_slot *slots;
    int64_t *done_log;          /* serving loop: user indices of requests completed since
                                 * it last looked (NULL: not logged) */
    int ndone;
    uint64_t ctas_launched;     /* resident CTAs launched so far (all launches) */
    uint64_t req_seq, item_seq, oldest_req;
    uint64_t inflight_bytes, budget;
    uint64_t relaunches;
    uint64_t item_bytes;
    uint32_t min_items;         /* split requests into at least this many items (>= 32 KiB) */
    yk_server_args args;
};

static void *pinned(size_t n)
{
    void *p = NULL;
    if (yk_fail_injected() ||
        cudaHostAlloc(&p, n, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess)
        return NULL;
    memset(p, 0, n);
    return p;
}

int yaksa_gb300_server_create(uint32_t ring_requests, uint64_t budget_bytes,
                              yaksa_gb300_server_t * server)
{
    *server = NULL;
    int rc = runtime_ready();
    if (rc)
        return rc;
    struct yaksa_gb300_server_s *S = calloc(1, sizeof(*S));
    if (!S)
        return YAKSA_ERR__OUT_OF_MEM;
    pthread_mutex_init(&S->mu, NULL);
    S->qr = ring_requests ? ring_requests : 4096;
    S->qi = 16 * S->qr;
    S->budget = budget_bytes ? budget_bytes : (64ull << 30);
    S->item_bytes = YK_ITEM_BYTES;
    const char *ik = getenv("YAKSA_GB300_SERVER_ITEM_KIB");
    if (ik) {
        unsigned long v = strtoul(ik, NULL, 10);
        if (v >= 16 && v <= 16384 && !(v & (v - 1)))
            S->item_bytes = (uint64_t) v << 10;
    }
    /* a request is split into at least min_items items (down to 32 KiB each), so that a
     * mid-size request is walked by that many CTAs at once; YAKSA_GB300_SERVER_MIN_ITEMS
     * overrides it (0: items of item_bytes only).  On the mixed request stream 128 cut
     * the p50 of 64 KiB..4 MiB requests from 183 to 53 us and of larger ones from 272 to
     * 189 us, at 98% of the capacity; 256 cost 7% of the capacity. */
    const char *mi = getenv("YAKSA_GB300_SERVER_MIN_ITEMS");
    S->min_items = mi ? (uint32_t) strtoul(mi, NULL, 10) : 128;
    if (S->min_items > 1024)
        S->min_items = 1024;
    S->reqs = pinned(sizeof(yk_launch) * S->qr);
    S->items = pinned(sizeof(yk_item) * S->qi);
    S->req_done = pinned(sizeof(unsigned long long) * S->qr);
    S->req_nitems = pinned(sizeof(uint64_t) * S->qr);
    S->cq = pinned(sizeof(unsigned long long) * S->qr);
    S->req_busy = pinned(sizeof(unsigned long long) * S->qr);
    S->ctl = pinned(64);
    S->slots = calloc(S->qr, sizeof(yk_srv_slot));
    /* device counters: the claim lanes (one 128-byte line each), then the queue's tail */
    const size_t nctr = (size_t) (YK_SRV_LANES + 1) * YK_SRV_LANE_STRIDE;
    if (!S->reqs || !S->items || !S->req_done || !S->req_nitems || !S->cq || !S->ctl ||
        !S->req_busy || !S->slots || yk_fail_injected() ||
        cudaMalloc((void **) &S->next_item, sizeof(unsigned long long) * nctr) != cudaSuccess ||
        cudaMemset(S->next_item, 0, sizeof(unsigned long long) * nctr) != cudaSuccess ||
        cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking) != cudaSuccess) {
        yaksa_gb300_server_destroy(S);
        return YAKSA_ERR__OUT_OF_MEM;
    }
    cudaDeviceSynchronize();
    S->ctas = yk_cuda_server_ctas();
    S->args.reqs = S->reqs;
    S->args.items = S->items;
    S->args.req_done = S->req_done;
    S->args.items_published = &S->ctl[0];
    S->args.stop = (const volatile int *) &S->ctl[1];
    S->args.next_item = S->next_item;
    S->args.status = (volatile uint32_t *) &S->ctl[2];
    S->args.req_nitems = S->req_nitems;
    S->args.cq = S->cq;
    S->args.cq_tail = S->next_item + (size_t) YK_SRV_LANES * YK_SRV_LANE_STRIDE;
    S->args.req_busy = S->req_busy;
    S->args.qi = S->qi;
    S->args.qr = S->qr;
    /* Resident CTAs leave after 2 ms without work, by the GPU's global timer; a device-
     * wide synchronize waits for them, so the window is kept short (a relaunch costs
     * about 30 us).  The poll count bounds the wait as well: an idle poll measured
     * about 12.5 us (the 2 us nap plus the C2C reads of the published count), so 4000
     * polls are about 50 ms. */
    S->args.idle_us = 2000;
    S->args.max_idle_spins = 4000;
    *server = S;
    return YAKSA_SUCCESS;
}

/* a request leaves the server; caller holds S->mu */
static void server_retire(struct yaksa_gb300_server_s *S, yk_srv_slot * sl)
{
    sl->busy = 0;
    S->inflight_bytes -= sl->bytes;
    if (sl->t)
        yk_type_unref(sl->t);
    sl->t = NULL;
    if (S->done_log && sl->user >= 0)
        S->done_log[S->ndone++] = sl->user;
}

/* reclaim finished requests and keep a kernel resident while items are pending; caller
 * holds S->mu.  The GPU appends each finished request's slot to the completion queue, so
 * this costs one read per completion, not one per request in flight. */
static int server_progress_locked(struct yaksa_gb300_server_s *S)
{
    for (;;) {
        unsigned long long *e = &S->cq[S->cq_head % S->qr];
        unsigned long long v = __atomic_load_n(e, __ATOMIC_ACQUIRE);
        if (!v)
            break;              /* empty, or its position taken and the write not seen yet */
        __atomic_store_n(e, 0ull, __ATOMIC_RELAXED);
        S->cq_head++;
        yk_srv_slot *sl = &S->slots[(v - 1) % S->qr];
        if (sl->busy)
            server_retire(S, sl);
    }
    while (S->oldest_req < S->req_seq && !S->slots[S->oldest_req % S->qr].busy)
        S->oldest_req++;
    /* every resident CTA counts its exit: none is resident once the exits reach the CTAs
     * launched (no CUDA call on this path) */
    const volatile uint32_t *st = (const volatile uint32_t *) &S->ctl[2];
    uint64_t exits = (uint64_t) st[0] + (uint64_t) st[1];
    S->running = exits < S->ctas_launched;
    int pending = S->oldest_req < S->req_seq;
    if (pending && !S->running && S->item_seq) {
        int e = yk_cuda_server_launch(&S->args, S->ctas, S->stream);
        if (e)
            return cuda_err((cudaError_t) e, "server launch");
        S->running = 1;
        S->ctas_launched += (uint64_t) S->ctas;
        S->relaunches++;
    }
    return YAKSA_SUCCESS;
}

int yaksa_gb300_server_progress(yaksa_gb300_server_t S)
{
    pthread_mutex_lock(&S->mu);
    int rc = server_progress_locked(S);
    pthread_mutex_unlock(&S->mu);
    return rc;
}

static int server_submit(struct yaksa_gb300_server_s *S, yaksa_gb300_pup_t * o, yaksa_info_t info,
                         uint64_t * ticket, int64_t user);

int yaksa_gb300_server_submit(yaksa_gb300_server_t S, yaksa_gb300_pup_t * o, yaksa_info_t info,
                              uint64_t * ticket)
{
    return server_submit(S, o, info, ticket, -1);
}

/* plan one request for the server: the launch record, its work-item kind and granule,
 * and its class for the item-cut tuner */
static int server_plan(yaksa_gb300_pup_t * o, yaksa_info_t info, yk_srv_req * q)
{
    o->actual = 0;
    memset(q, 0, sizeof(*q));
    yk_type *t = q->t = yk_type_get(o->type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    yk_plan *pp = &q->p;
    int rc = plan_op(o, t, info, pp);
    if (rc)
        return rc;
    const yk_plan p = *pp;
    if (p.staged)
        return YAKSA_ERR__NOT_SUPPORTED;        /* the GPU cannot address a buffer */
    if (ldbl_arith(t, o->op))
        return YAKSA_ERR__NOT_SUPPORTED;        /* the server kernel has no binary128 operators */
    yk_launch L;
    int kind = YK_X_BYTES, sorted = 0;
    if (p.b1 > p.b0) {
        rc = prepare(&p, p.dtyped, p.dpacked, &L, &kind, &sorted);
        if (rc)
            return rc;
    } else {
        memset(&L, 0, sizeof(L));
    }
    uint32_t skind;
    uint64_t gran;
    if (kind == YK_X_MEMCPY) {
        /* contiguous: an empty level chain over one run starting at true_lb */
        memset(&L.desc, 0, sizeof(L.desc));
        L.desc.leaf = YK_LEAF_RUN;
        L.desc.run = ~(uint64_t) 0;
        L.desc.base = t->true_lb;
        L.regular = 0;
        int v = pow2_of((uint64_t) (uintptr_t) p.dtyped + (uint64_t) t->true_lb);
        v = YK_MIN(v, pow2_of((uint64_t) (uintptr_t) p.dpacked));
        v = YK_MIN(v, pow2_of(p.b0));
        v = YK_MIN(v, pow2_of(p.b1 - p.b0));
        L.vec = v;
        L.use64 = p.b1 > YK_POS32_END;
        skind = L.use64 ? YK_SRV_BYTES : YK_SRV_REGULAR;
        gran = (uint64_t) v;
    } else if (kind == YK_X_BYTES && runs_pack_ok(&L) && (uintptr_t) L.packed % 16 == 0 &&
               L.desc.run % 4 == 0 && L.desc.run <= 48) {
        /* struct-like packs: the warp-staged form, items of whole 32-element groups so that
         * each group's packed bytes start on 16 bytes */
        skind = YK_SRV_RUNS;
        gran = 32 * (uint64_t) L.desc.run;
    } else if (kind == YK_X_BYTES) {
        skind = L.hidx ? YK_SRV_HIDX : L.regular >= 0 ? YK_SRV_REGULAR : YK_SRV_BYTES;
        gran = (uint64_t) L.vec;
    } else if (kind == YK_X_TYPED) {
        skind = YK_SRV_TYPED;
        gran = (uint64_t) L.vec;
    } else {
        /* L2 reductions where they apply; the owner items need sorted blocks */
        const int red = (sorted & YK_ORD_RED) != 0, owner = (sorted & 3) != 0;
        skind = red ? YK_SRV_RED : (sorted & 3) == 2 ? YK_SRV_OWNER_T : owner ? YK_SRV_OWNER :
            YK_SRV_ORDERED;
        gran = red || owner ? (uint64_t) yk_base_type_size(L.desc.leaf_type) : (uint64_t) L.vec;
        if (skind == YK_SRV_OWNER_T)
            L.form = yk_cuda_owner_form(&L, sorted);   /* block shift, 32-bit offsets */
    }
    q->L = L;
    q->skind = skind;
    q->gran = gran;
    const uint64_t n = p.b1 - p.b0;
    /* class: item kind, unit, direction, base type for operators, size (power of two) */
    if (skind != YK_SRV_ORDERED && n >= YK_SRV_TUNE_MIN)
        q->key = yk_tune_key(YK_TUNE_SERVER, (int) skind, L.vec, L.dir,
                             L.typed_op ? L.desc.leaf_type & 15 : 0, n);
    return YAKSA_SUCCESS;
}

/* Cut a planned request into work items and publish them.  cfg: the item cut ({0, 0}
 * the server's own); timed: the GPU sums its items' busy time into req_busy of its
 * slot.  user: the serving loop's index of the request, logged at completion (-1:
 * none). */
static int server_enqueue(struct yaksa_gb300_server_s *S, yaksa_gb300_pup_t * o, yk_srv_req * q,
                          const yk_tune_cfg * cfg, int timed, uint64_t * ticket, int64_t user)
{
    int rc;
    yk_type *t = q->t;
    const yk_plan p = q->p;
    const yk_launch L = q->L;
    const uint32_t skind = q->skind;
    const uint64_t gran = q->gran;
    uint64_t n = p.b1 - p.b0;
    uint64_t ib = cfg->units_per_thread ? (uint64_t) cfg->units_per_thread << 10 : S->item_bytes;
    const uint64_t min_items = cfg->units_per_thread ? (uint64_t) cfg->ctas_per_sm : S->min_items;
    while (min_items && ib > (32u << 10) && n < min_items * ib)
        ib >>= 1;       /* mid-size requests: more, smaller items, so more CTAs share them */
    uint64_t chunk = skind == YK_SRV_ORDERED ? (n ? n : 1) : YK_MAX(ib / gran, 1) * gran;
    uint64_t nitems = n ? (n + chunk - 1) / chunk : 0;
    if (nitems > S->qi)
        return YAKSA_ERR__NOT_SUPPORTED;        /* larger than the whole item ring */

    pthread_mutex_lock(&S->mu);
    server_progress_locked(S);
    uint64_t oldest_item = S->oldest_req < S->req_seq ?
        S->slots[S->oldest_req % S->qr].item0 : S->item_seq;
    if (S->req_seq - S->oldest_req >= S->qr || S->item_seq + nitems - oldest_item > S->qi ||
        (S->inflight_bytes && S->inflight_bytes + n > S->budget)) {
        pthread_mutex_unlock(&S->mu);
        return YAKSA_ERR__OUT_OF_MEM;   /* admission refused: retry after progress */
    }
    uint64_t seq = S->req_seq++;
    uint32_t slot = (uint32_t) (seq % S->qr);
    yk_srv_slot *sl = &S->slots[slot];
    sl->seq = seq;
    sl->item0 = S->item_seq;
    sl->nitems = nitems;
    sl->bytes = n;
    sl->busy = nitems > 0;      /* an empty request is complete at once */
    sl->t = NULL;
    sl->user = user;
    if (nitems) {
        sl->t = t;
        yk_type_ref(t);
        S->inflight_bytes += n;
        __atomic_store_n(&S->req_done[slot], 0ull, __ATOMIC_RELAXED);
        S->req_nitems[slot] = nitems;
        S->req_busy[slot] = 0;
        memcpy(&S->reqs[slot], &L, sizeof(L));
        const uint32_t ikind = skind | (timed ? YK_SRV_TIMED : 0u);
        for (uint64_t i = 0; i < nitems; i++) {
            yk_item *it = &S->items[(S->item_seq + i) % S->qi];
            it->seq = S->item_seq + i;
            it->req = slot;
            it->kind = ikind;
            it->pb = p.b0 + i * chunk;
            it->pe = YK_MIN(p.b1, p.b0 + (i + 1) * chunk);
        }
        S->item_seq += nitems;
        /* publish: every record store above happens-before this release store */
        __atomic_store_n(&S->ctl[0], S->item_seq, __ATOMIC_RELEASE);
    }
    o->actual = n;
    rc = server_progress_locked(S);     /* relaunches the resident kernel if it left */
    pthread_mutex_unlock(&S->mu);
    *ticket = seq;
    return rc;
}

/* a request cut the way its class's tuner decided (the server's own cut until then) */
static int server_submit(struct yaksa_gb300_server_s *S, yaksa_gb300_pup_t * o, yaksa_info_t info,
                         uint64_t * ticket, int64_t user)
{
    yk_srv_req q;
    int rc = server_plan(o, info, &q);
    if (rc)
        return rc;
    yk_tune_cfg cfg = { 0, 0, 0 };
    if (q.key)
        yk_tune_server_cfg(q.key, &cfg);
    return server_enqueue(S, o, &q, &cfg, 0, ticket, user);
}

/* One calibration sample: k copies of a request submitted together with item cut cfg,
 * all waited for; *ns = the busy time of all the copies' items summed (each item from
 * its record load to its last byte, on the CTA that ran it).  With the server loaded,
 * resident CTAs always have items, so its throughput is CTAs / (busy time per byte):
 * the sum measures exactly that, unlike the span of one group, which a group too small
 * to fill the GPU would bias towards finer cuts.  The copies run at once, so the items
 * meet the memory contention of a loaded server. */
static int server_tune_group(struct yaksa_gb300_server_s *S, yaksa_gb300_pup_t * o, yk_srv_req * q,
                             const yk_tune_cfg * cfg, int k, double *ns)
{
    uint64_t tk[64];
    int rc = YAKSA_SUCCESS, m = 0;
    *ns = 0;
    struct timespec a, b;
    clock_gettime(CLOCK_MONOTONIC, &a);
    while (m < k && !rc) {
        rc = server_enqueue(S, o, q, cfg, 1, &tk[m], -1);
        if (rc == YAKSA_ERR__OUT_OF_MEM) {
            /* rings or budget full: let the copies in flight finish (bounded) */
            rc = yaksa_gb300_server_progress(S);
            clock_gettime(CLOCK_MONOTONIC, &b);
            if (!rc && b.tv_sec - a.tv_sec > 20)
                rc = YAKSA_ERR__INTERNAL;
            if (!rc && m == 0 && S->oldest_req == S->req_seq)
                return YAKSA_SUCCESS;   /* one copy alone does not fit: no sample */
            continue;
        }
        if (!rc)
            m++;
    }
    for (int i = 0; i < m && !rc; i++)
        rc = yaksa_gb300_server_wait(S, tk[i]);
    if (rc)
        return rc;
    double busy = 0;
    for (int i = 0; i < m; i++)
        busy += (double) __atomic_load_n(&S->req_busy[tk[i] % S->qr], __ATOMIC_ACQUIRE);
    if (m == k)
        *ns = busy;
    return YAKSA_SUCCESS;
}

int yaksa_gb300_server_tune(yaksa_gb300_server_t S, yaksa_gb300_pup_t * ops, int n,
                            yaksa_info_t info, int *classes)
{
    int decided = 0, rc = YAKSA_SUCCESS;
    for (int i = 0; i < n && !rc; i++) {
        /* each undecided class: every candidate cut in turn, a group of copies at a time,
         * until the tuner decides.  The group holds enough copies for 64 MiB (at most 64,
         * and half the request ring) so that the GPU is as full as under load. */
        for (int guard = 0; guard < 64 && !rc; guard++) {
            yk_srv_req q;
            rc = server_plan(&ops[i], info, &q);
            if (rc || !q.key)
                break;
            yk_tune_cfg cfg;
            const int cand = yk_tune_server_next(q.key, &cfg);
            if (cand < 0) {
                decided += guard > 0;
                break;
            }
            const uint64_t bytes = q.p.b1 - q.p.b0;
            uint64_t k = ((64ull << 20) + bytes - 1) / bytes;
            k = YK_MIN(k, 64);
            k = YK_MIN(k, (uint64_t) (S->qr / 2 ? S->qr / 2 : 1));
            double ns = 0;
            rc = server_tune_group(S, &ops[i], &q, &cfg, (int) k, &ns);
            if (!rc && ns > 0)
                yk_tune_server_sample(q.key, cand, ns);
            if (rc || ops[i].actual == 0)
                break;
        }
    }
    if (classes)
        *classes = decided;
    return rc;
}

static int server_done_locked(struct yaksa_gb300_server_s *S, uint64_t ticket)
{
    if (ticket < S->oldest_req)
        return 1;
    yk_srv_slot *sl = &S->slots[ticket % S->qr];
    return ticket < S->req_seq && (sl->seq != ticket || !sl->busy);
}

int yaksa_gb300_server_test(yaksa_gb300_server_t S, uint64_t ticket, int *done)
{
    pthread_mutex_lock(&S->mu);
    int rc = server_progress_locked(S);
    *done = server_done_locked(S, ticket);
    pthread_mutex_unlock(&S->mu);
    return rc;
}

int yaksa_gb300_server_wait(yaksa_gb300_server_t S, uint64_t ticket)
{
    /* bounded: 20 s without completion is reported as an error */
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (;;) {
        int done, rc = yaksa_gb300_server_test(S, ticket, &done);
        if (rc || done)
            return rc;
        clock_gettime(CLOCK_MONOTONIC, &t1);
        if (t1.tv_sec - t0.tv_sec > 20)
            return YAKSA_ERR__INTERNAL;
    }
}

int yaksa_gb300_server_stats(yaksa_gb300_server_t S, uint64_t * requests, uint64_t * items,
                             uint64_t * relaunches, uint32_t * idle_exits)
{
    pthread_mutex_lock(&S->mu);
    *requests = S->req_seq;
    *items = S->item_seq;
    *relaunches = S->relaunches;
    *idle_exits = ((volatile uint32_t *) &S->ctl[2])[0];
    uint32_t rejected = ((volatile uint32_t *) &S->ctl[2])[2];
    if (rejected)
        fprintf(stderr, "yaksa-gb300: server rejected %u work items\n", rejected);
    pthread_mutex_unlock(&S->mu);
    return YAKSA_SUCCESS;
}

int yaksa_gb300_server_destroy(yaksa_gb300_server_t S)
{
    if (!S)
        return YAKSA_SUCCESS;
    int rc = YAKSA_SUCCESS;
    if (S->ctl)
        __atomic_store_n((int *) &S->ctl[1], 1, __ATOMIC_RELEASE);
    if (S->stream) {
        /* resident CTAs leave at their next poll; bounded wait */
        struct timespec t0, t1;
        clock_gettime(CLOCK_MONOTONIC, &t0);
        while (cudaStreamQuery(S->stream) == cudaErrorNotReady) {
            clock_gettime(CLOCK_MONOTONIC, &t1);
            if (t1.tv_sec - t0.tv_sec > 30) {
                rc = YAKSA_ERR__INTERNAL;
                break;
            }
        }
        if (!rc)
            cudaStreamDestroy(S->stream);
    }
    for (uint32_t i = 0; S->slots && i < S->qr; i++)
        if (S->slots[i].t)
            yk_type_unref(S->slots[i].t);
    if (!rc) {
        if (S->next_item)
            cudaFree(S->next_item);
        if (S->reqs)
            cudaFreeHost(S->reqs);
        if (S->items)
            cudaFreeHost(S->items);
        if (S->req_done)
            cudaFreeHost(S->req_done);
        if (S->req_nitems)
            cudaFreeHost(S->req_nitems);
        if (S->cq)
            cudaFreeHost(S->cq);
        if (S->req_busy)
            cudaFreeHost(S->req_busy);
        if (S->ctl)
            cudaFreeHost(S->ctl);
    }
    free(S->slots);
    pthread_mutex_destroy(&S->mu);
    free(S);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* serving loop: replay an arrival schedule through the plain or batched path */
/* ------------------------------------------------------------------------- */

/* The serving loop's graph lane (mode 2).  A request whose record (kind, buffers,
 * count, type, offset, size, operator) repeats runs, from its second sight on, as the
 * replay of a CUDA graph holding the launch captured at that sight: one graph launch
 * and one event instead of the plan, the descriptor lookup, the launch-shape choice and
 * the launch.  The first sight runs the plain path, which builds the type's
 * descriptors, so nothing inside the capture allocates or synchronizes; the captured
 * launch has the shape the autotuner had decided by then (the default while the class
 * is still being timed).  Requests whose buffers need staging keep the plain path. */
typedef struct {
    yaksa_gb300_pup_t rec;
    int used;
    int seen;                   /* sights so far; -1: never captured */
    cudaGraphExec_t exec;
    yk_type *t;                 /* held while the graph exists */
    uintptr_t actual;
} yk_glane_ent;

typedef struct {
    yk_glane_ent *e;
    size_t cap;                 /* a power of two, at least twice the requests */
    cudaStream_t cs;            /* capture stream */
} yk_glane;

static uint64_t graph_captures, graph_replays;

int yaksa_gb300_graph_lane_stats(uint64_t * captures, uint64_t * replays)
{
    *captures = __atomic_load_n(&graph_captures, __ATOMIC_RELAXED);
    *replays = __atomic_load_n(&graph_replays, __ATOMIC_RELAXED);
    return YAKSA_SUCCESS;
}

static int glane_same(const yaksa_gb300_pup_t * a, const yaksa_gb300_pup_t * b)
{
    return a->kind == b->kind && a->inbuf == b->inbuf && a->outbuf == b->outbuf &&
        a->count == b->count && a->type == b->type && a->offset == b->offset &&
        a->maxbytes == b->maxbytes && a->op == b->op;
}

static yk_glane_ent *glane_find(yk_glane * G, const yaksa_gb300_pup_t * o)
{
    const uint64_t w[8] = { (uint64_t) o->kind, (uint64_t) (uintptr_t) o->inbuf,
        (uint64_t) (uintptr_t) o->outbuf, (uint64_t) o->count, (uint64_t) o->type,
        (uint64_t) o->offset, (uint64_t) o->maxbytes, (uint64_t) o->op };
    uint64_t h = 1469598103934665603ull;        /* FNV-1a over the record's words */
    for (int i = 0; i < 8; i++)
        h = (h ^ w[i]) * 1099511628211ull;
    for (size_t i = (size_t) h & (G->cap - 1);; i = (i + 1) & (G->cap - 1)) {
        yk_glane_ent *e = &G->e[i];
        if (!e->used) {
            e->used = 1;
            e->rec = *o;
            return e;
        }
        if (glane_same(&e->rec, o))
            return e;
    }
}

/* capture the request's launch into e->exec; e->seen = -1 when it never will be */
static int glane_capture(yk_glane * G, yk_glane_ent * e, yaksa_gb300_pup_t * o, yaksa_info_t info)
{
    yk_type *t = yk_type_get(o->type);
    if (!t)
        return YAKSA_ERR__INTERNAL;
    yk_plan p;
    int rc = plan_op(o, t, info, &p);
    if (rc)
        return rc;
    if (p.staged || p.b1 == p.b0) {
        e->seen = -1;
        return YAKSA_SUCCESS;
    }
    if (!G->cs && (rc = cuda_err(cudaStreamCreateWithFlags(&G->cs, cudaStreamNonBlocking),
                                 "cudaStreamCreate")))
        return rc;
    rc = cuda_err(cudaStreamBeginCapture(G->cs, cudaStreamCaptureModeThreadLocal),
                  "cudaStreamBeginCapture");
    if (rc)
        return rc;
    const int erc = enqueue(&p, p.dtyped, p.dpacked, G->cs);
    cudaGraph_t g = NULL;
    cudaError_t ce = cudaStreamEndCapture(G->cs, &g);
    if (erc || ce != cudaSuccess || !g) {
        if (g)
            cudaGraphDestroy(g);
        cudaGetLastError();
        e->seen = -1;
        return erc;
    }
    ce = cudaGraphInstantiate(&e->exec, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
        cudaGetLastError();
        e->exec = NULL;
        e->seen = -1;
        return YAKSA_SUCCESS;
    }
    yk_type_ref(t);
    e->t = t;
    e->actual = p.b1 - p.b0;
    __atomic_add_fetch(&graph_captures, 1, __ATOMIC_RELAXED);
    return YAKSA_SUCCESS;
}

/* mode 2's submission: a replay when the record was captured, else the plain path */
static int glane_submit(yk_glane * G, yaksa_gb300_pup_t * o, yaksa_info_t info,
                        yaksa_request_t * req)
{
    yk_glane_ent *e = glane_find(G, o);
    int rc;
    if (!e->exec && e->seen >= 0 && ++e->seen >= 2 && (rc = glane_capture(G, e, o, info)))
        return rc;
    if (e->exec) {
        cudaStream_t s = lib_stream();
        rc = cuda_err(cudaGraphLaunch(e->exec, s), "cudaGraphLaunch");
        if (rc)
            return rc;
        __atomic_add_fetch(&graph_replays, 1, __ATOMIC_RELAXED);
        o->actual = e->actual;
        return complete(e->t, YK_MODE_NONBLOCKING, s, req);
    }
    uintptr_t actual = 0;
    rc = o->kind != 0 && o->kind != 1 ? YAKSA_ERR__INTERNAL : o->kind == 0 ?
        yaksa_ipack(o->inbuf, o->count, o->type, o->offset, o->outbuf, o->maxbytes, &actual, info,
                    o->op, req) :
        yaksa_iunpack(o->inbuf, o->maxbytes, o->outbuf, o->count, o->type, o->offset, &actual, info,
                      o->op, req);
    o->actual = actual;
    return rc;
}

static void glane_free(yk_glane * G, int failed)
{
    if (failed)
        cudaDeviceSynchronize();        /* replays may still run: none is destroyed live */
    for (size_t i = 0; G->e && i < G->cap; i++) {
        if (G->e[i].exec)
            cudaGraphExecDestroy(G->e[i].exec);
        if (G->e[i].t)
            yk_type_unref(G->e[i].t);
    }
    free(G->e);
    if (G->cs)
        cudaStreamDestroy(G->cs);
}

static double now_s(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double) t.tv_sec + 1e-9 * (double) t.tv_nsec;
}

int yaksa_gb300_serve_trace(yaksa_gb300_pup_t * ops, const double *arrival_s, int n, int mode,
                            yaksa_gb300_server_t server, yaksa_info_t info, double *latency_s,
                            double *makespan_s)
{
    int rc = runtime_ready();
    if (rc)
        return rc;
    if ((mode == 1 && !server) || mode < 0 || mode > 2)
        return YAKSA_ERR__INTERNAL;
    uint64_t *handle = calloc(n > 0 ? n : 1, sizeof(uint64_t));
    char *state = calloc(n > 0 ? n : 1, 1);     /* 0 waiting, 1 in flight, 2 done */
    yk_glane G = { NULL, 0, NULL };
    if (mode == 2) {
        G.cap = 16;
        while (G.cap < 2 * (size_t) (n > 0 ? n : 1))
            G.cap *= 2;
        G.e = calloc(G.cap, sizeof(yk_glane_ent));
    }
    if (!handle || !state || (mode == 2 && !G.e)) {
        free(handle);
        free(state);
        free(G.e);
        return YAKSA_ERR__OUT_OF_MEM;
    }
    int next = 0, done = 0, oldest = 0;
    if (mode == 1) {
        /* the server logs the loop's index of each request it completes */
        int64_t *log = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
        if (!log) {
            free(handle);
            free(state);
            return YAKSA_ERR__OUT_OF_MEM;
        }
        pthread_mutex_lock(&server->mu);
        server->done_log = log;
        server->ndone = 0;
        pthread_mutex_unlock(&server->mu);
    }
    double t0 = now_s(), last = t0;
    while (done < n && !rc) {
        double t = now_s() - t0;
        /* admit arrivals in order; a refused request waits at the head (FIFO) */
        while (next < n && arrival_s[next] <= t) {
            yaksa_gb300_pup_t *o = &ops[next];
            if (mode == 1) {
                uint64_t tk;
                int r = server_submit(server, o, info, &tk, next);
                if (r == YAKSA_ERR__OUT_OF_MEM)
                    break;      /* rings or byte budget full: retry after progress */
                if (r) {
                    rc = r;
                    break;
                }
                handle[next] = tk;
                if (!o->actual) {
                    /* an empty request completes at submission, without a queue entry */
                    latency_s[next] = now_s() - t0 - arrival_s[next];
                    state[next++] = 2;
                    done++;
                    continue;
                }
            } else if (mode == 2) {
                yaksa_request_t req = YAKSA_REQUEST__NULL;
                int r = glane_submit(&G, o, info, &req);
                if (r) {
                    rc = r;
                    break;
                }
                handle[next] = req;
            } else {
                yaksa_request_t req;
                uintptr_t actual;
                int r = o->kind != 0 && o->kind != 1 ? YAKSA_ERR__INTERNAL : o->kind == 0 ?
                    yaksa_ipack(o->inbuf, o->count, o->type, o->offset, o->outbuf, o->maxbytes,
                                &actual, info, o->op, &req) :
                    yaksa_iunpack(o->inbuf, o->maxbytes, o->outbuf, o->count, o->type, o->offset,
                                  &actual, info, o->op, &req);
                if (r) {
                    rc = r;
                    break;
                }
                o->actual = actual;
                handle[next] = req;
            }
            state[next] = 1;
            next++;
        }
        /* completions (requests may finish out of order): the server reports the ones it
         * saw, in one progress pass; plain requests are tested one by one */
        if (mode == 1) {
            pthread_mutex_lock(&server->mu);
            rc = server_progress_locked(server);
            double tc = now_s();
            for (int k = 0; k < server->ndone; k++) {
                int64_t i = server->done_log[k];
                if (i >= 0 && i < n && state[i] == 1) {
                    latency_s[i] = tc - t0 - arrival_s[i];
                    state[i] = 2;
                    done++;
                    last = tc;
                }
            }
            server->ndone = 0;
            pthread_mutex_unlock(&server->mu);
        } else {
            double tc = now_s();
            for (int i = oldest; i < next && !rc; i++) {
                if (state[i] != 1)
                    continue;
                int c = 0;
                rc = yaksa_request_test(handle[i], &c);
                if (c) {
                    latency_s[i] = tc - t0 - arrival_s[i];
                    state[i] = 2;
                    done++;
                    last = tc;
                }
            }
        }
        while (oldest < next && state[oldest] == 2)
            oldest++;
    }
    if (mode == 1) {
        pthread_mutex_lock(&server->mu);
        free(server->done_log);
        server->done_log = NULL;
        server->ndone = 0;
        pthread_mutex_unlock(&server->mu);
    }
    *makespan_s = last - t0;
    if (mode == 2)
        glane_free(&G, rc != 0);
    free(handle);
    free(state);
    return rc;
}

/* ------------------------------------------------------------------------- */
/* captured graphs: a fixed sequence of batches replayed with one launch      */
/* ------------------------------------------------------------------------- */

struct yaksa_gb300_graph_s {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    yk_type **types;            /* held while the graph exists */
    int ntypes;
    int nkernels;               /* kernel nodes: launches per replay */
};

int yaksa_gb300_graph_create(yaksa_gb300_pup_t * ops, const int *batch_ends, int nbatches,
                             yaksa_info_t info, yaksa_gb300_graph_t * graph)
{
    *graph = NULL;
    int rc = runtime_ready();
    if (rc)
        return rc;
    int n = nbatches ? batch_ends[nbatches - 1] : 0;
    struct yaksa_gb300_graph_s *g = calloc(1, sizeof(*g));
    if (!g)
        return YAKSA_ERR__OUT_OF_MEM;
    g->types = calloc(n ? n : 1, sizeof(yk_type *));
    if (!g->types) {
        free(g);
        return YAKSA_ERR__OUT_OF_MEM;
    }
    /* build every descriptor and refuse staged requests before capturing: nothing
     * inside the capture may allocate or synchronize */
    for (int i = 0; i < n; i++) {
        yaksa_gb300_pup_t *o = &ops[i];
        if (o->count == 0)
            continue;
        yk_type *t = yk_type_get(o->type);
        if (!t) {
            rc = YAKSA_ERR__INTERNAL;
            break;
        }
        yk_plan p;
        rc = plan_op(o, t, info, &p);
        if (rc)
            break;
        if (p.b1 == p.b0)
            continue;
        if (p.staged) {
            rc = YAKSA_ERR__NOT_SUPPORTED;
            break;
        }
        yk_devdesc *dd;
        if ((rc = yk_desc_get(t, o->op != YAKSA_OP__REPLACE, &dd)) ||
            (o->op == YAKSA_OP__REPLACE && t->base_type > 0 && (rc = yk_desc_get(t, 1, &dd))))
            break;
        yk_type_ref(t);
        g->types[g->ntypes++] = t;
    }
    cudaStream_t cs = NULL;
    if (!rc)
        rc = cuda_err(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!rc)
        rc = cuda_err(cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed), "capture");
    if (!rc) {
        /* captured launches run at replay: counted there, not here */
        uint64_t l0 = __atomic_load_n(&R.launches, __ATOMIC_RELAXED);
        int start = 0;
        for (int b = 0; b < nbatches && !rc; b++) {
            rc = batch_run(ops + start, batch_ends[b] - start, info, cs);
            start = batch_ends[b];
        }
        __atomic_sub_fetch(&R.launches, __atomic_load_n(&R.launches, __ATOMIC_RELAXED) - l0,
                           __ATOMIC_RELAXED);
        cudaError_t e = cudaStreamEndCapture(cs, &g->graph);
        if (!rc)
            rc = cuda_err(e, "capture");
        if (!rc)
            rc = cuda_err(cudaGraphInstantiate(&g->exec, g->graph, 0), "cudaGraphInstantiate");
        size_t nn = 0;
        if (!rc && cudaGraphGetNodes(g->graph, NULL, &nn) == cudaSuccess && nn) {
            cudaGraphNode_t *nodes = malloc(nn * sizeof(cudaGraphNode_t));
            if (nodes && cudaGraphGetNodes(g->graph, nodes, &nn) == cudaSuccess)
                for (size_t i = 0; i < nn; i++) {
                    enum cudaGraphNodeType ty;
                    if (cudaGraphNodeGetType(nodes[i], &ty) == cudaSuccess &&
                        ty == cudaGraphNodeTypeKernel)
                        g->nkernels++;
                }
            free(nodes);
        }
    }
    if (cs)
        cudaStreamDestroy(cs);
    if (rc) {
        yaksa_gb300_graph_free(g);
        return rc;
    }
    *graph = g;
    return YAKSA_SUCCESS;
}

int yaksa_gb300_graph_launch(yaksa_gb300_graph_t g, void *stream)
{
    if (!g)
        return YAKSA_ERR__INTERNAL;
    cudaStream_t s = stream ? *(cudaStream_t *) stream : R.streams[0];
    __atomic_add_fetch(&R.launches, (uint64_t) g->nkernels, __ATOMIC_RELAXED);
    return cuda_err(cudaGraphLaunch(g->exec, s), "cudaGraphLaunch");
}

int yaksa_gb300_graph_free(yaksa_gb300_graph_t g)
{
    if (!g)
        return YAKSA_SUCCESS;
    if (g->exec)
        cudaGraphExecDestroy(g->exec);
    if (g->graph)
        cudaGraphDestroy(g->graph);
    for (int i = 0; i < g->ntypes; i++)
        yk_type_unref(g->types[i]);
    free(g->types);
    free(g);
    return YAKSA_SUCCESS;
}

/* runtime counters for tests and the bench */
int yaksa_gb300_stats(uint64_t * launches, uint64_t * direct_calls, uint64_t * staged_calls,
                      uint64_t * memcpy_calls)
{
    *launches = __atomic_load_n(&R.launches, __ATOMIC_RELAXED);
    *direct_calls = __atomic_load_n(&R.direct_calls, __ATOMIC_RELAXED);
    *staged_calls = __atomic_load_n(&R.staged_calls, __ATOMIC_RELAXED);
    *memcpy_calls = __atomic_load_n(&R.memcpy_calls, __ATOMIC_RELAXED);
    return YAKSA_SUCCESS;
}
