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
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>
#include "yk_internal.h"

typedef struct {
    int in_use;
    cudaEvent_t ev;
    yk_type *type;              /* held until completion: a type may be freed in flight */
    void *scratch[2];           /* staged buffers released at completion */
} yk_req;

static struct {
    pthread_mutex_t mu;
    int ready;
    int failed;
    int device;
    int pageable_access;
    cudaStream_t stream;
    yk_req *reqs;
    size_t nreqs;
    cudaEvent_t *evpool;
    size_t nev, capev;
    /* counters (yaksa_gb300_stats) */
    uint64_t launches, staged_calls, direct_calls, memcpy_calls;
} R = { PTHREAD_MUTEX_INITIALIZER, 0, 0, 0, 0, NULL, NULL, 0, NULL, 0, 0, 0, 0, 0, 0 };

static int cuda_err(cudaError_t e, const char *what)
{
    if (e == cudaSuccess)
        return YAKSA_SUCCESS;
    fprintf(stderr, "yaksa-gb300: %s failed: %s\n", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? YAKSA_ERR__OUT_OF_MEM : YAKSA_ERR__INTERNAL;
}

int yk_runtime_init(void)
{
    /* the GPU is brought up lazily at the first pack/unpack so that type
     * construction works on hosts without a GPU */
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
            e = cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking);
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

void yk_runtime_finalize(void)
{
    pthread_mutex_lock(&R.mu);
    if (R.ready) {
        cudaStreamSynchronize(R.stream);
        for (size_t i = 0; i < R.nreqs; i++)
            if (R.reqs[i].in_use) {
                cudaEventDestroy(R.reqs[i].ev);
                R.reqs[i].in_use = 0;
            }
        for (size_t i = 0; i < R.nev; i++)
            cudaEventDestroy(R.evpool[i]);
        R.nev = 0;
        cudaStreamDestroy(R.stream);
        R.ready = 0;
    }
    free(R.reqs);
    R.reqs = NULL;
    R.nreqs = 0;
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
    size_t i;
    for (i = 0; i < R.nreqs; i++)
        if (!R.reqs[i].in_use)
            break;
    if (i == R.nreqs) {
        size_t nn = R.nreqs ? 2 * R.nreqs : 64;
        yk_req *p = realloc(R.reqs, nn * sizeof(yk_req));
        if (!p) {
            pthread_mutex_unlock(&R.mu);
            return YAKSA_ERR__OUT_OF_MEM;
        }
        memset(p + R.nreqs, 0, (nn - R.nreqs) * sizeof(yk_req));
        R.reqs = p;
        R.nreqs = nn;
    }
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
            if (a.devicePointer)
                return (char *) base + ((const char *) a.devicePointer - probe);
            return (char *) base;
        default:
            if (R.pageable_access)
                return (char *) base;
            *staged = 1;
            return NULL;
    }
}

static int pow2_of(uint64_t v)
{
    int a = 16;
    while (a > 1 && (v % (uint64_t) a))
        a >>= 1;
    return a;
}

/* ------------------------------------------------------------------------- */
/* launch construction                                                       */
/* ------------------------------------------------------------------------- */

static int op_needs_host_arith(yk_type * t, yaksa_op_t op)
{
    return t->needs_host_ops && (op == YAKSA_OP__SUM || op == YAKSA_OP__PROD ||
                                 op == YAKSA_OP__MIN || op == YAKSA_OP__MAX);
}

/* Enqueue the kernel(s) for [b0, b1) on `s`.  typed/packed are device-usable. */
static int enqueue(int dir, char *typed, char *packed, yk_type * t, uintptr_t count,
                   uintptr_t b0, uintptr_t b1, yaksa_op_t op, cudaStream_t s)
{
    uintptr_t n = b1 - b0;
    if (op == YAKSA_OP__REPLACE && t->is_contig) {
        /* contiguous: the packed bytes are the memory bytes from true_lb */
        char *mem = typed + t->true_lb + b0;
        __atomic_add_fetch(&R.memcpy_calls, 1, __ATOMIC_RELAXED);
        return cuda_err(cudaMemcpyAsync(dir == 0 ? packed : mem, dir == 0 ? mem : packed, n,
                                        cudaMemcpyDefault, s), "cudaMemcpyAsync");
    }
    int typed_op = (op != YAKSA_OP__REPLACE);
    yk_devdesc *dd;
    int rc = yk_desc_get(t, typed_op, &dd);
    if (rc)
        return rc;
    int overlap = dir == 1 && (dd->may_overlap ||
                               (count > 1 && (int64_t) (t->extent < 0 ? -t->extent : t->extent)
                                < dd->elem_span));
    yk_devdesc *ddo = dd;
    if (overlap && !typed_op) {
        /* ordered REPLACE reuses the typed descriptor's element structure when the
         * type is homogeneous (owner-computes), else the bytes descriptor */
        yk_devdesc *tdd;
        if (t->base_type > 0 && yk_desc_get(t, 1, &tdd) == YAKSA_SUCCESS && tdd->sorted_blocks)
            ddo = tdd;
    }

    yk_launch L;
    memset(&L, 0, sizeof(L));
    yk_make_launch_desc(ddo, t, count, &L.desc);
    L.typed = typed;
    L.packed = packed;
    L.p0 = b0;
    L.nbytes = n;
    L.op = op;
    L.dir = dir;
    L.use64 = (b1 > 0xffffffffull);
    uint64_t ext = (uint64_t) (t->extent < 0 ? -t->extent : t->extent);
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
        L.vec = v;
        L.typed_op = 0;
    } else {
        /* element granularity; alignment is checked per access in the kernel */
        L.typed_op = 1;
        L.vec = ddo->unit;
        if (!typed_op)
            L.op = YAKSA_OP__REPLACE;
    }
    __atomic_add_fetch(&R.launches, 1, __ATOMIC_RELAXED);
    int e;
    if (overlap) {
        int sorted = ddo->sorted_blocks && L.typed_op && L.desc.nlev == 1 &&
            L.desc.lv[0].kind == YK_LV_IDX && ddo->elem_align >= yk_base_type_size(t->base_type);
        if (!L.typed_op && !sorted)
            L.vec = (int) YK_MIN((uint64_t) L.vec, (uint64_t) ddo->vec_align);
        e = yk_cuda_launch_unpack_ordered(&L, sorted, s);
    } else {
        e = yk_cuda_launch_pup(&L, s);
    }
    return cuda_err((cudaError_t) e, "kernel launch");
}

/* ------------------------------------------------------------------------- */
/* the pack/unpack entry                                                     */
/* ------------------------------------------------------------------------- */

int yk_pup(int dir, const void *packed_in, void *packed_out, char *typed, uintptr_t count,
           yk_type * t, uintptr_t offset, uintptr_t maxbytes, uintptr_t * actual,
           yk_info * info, yaksa_op_t op, int mode, void *stream, yaksa_request_t * request)
{
    if (request)
        *request = YAKSA_REQUEST__NULL;
    *actual = 0;
    if (count == 0 || t->size == 0)
        return YAKSA_SUCCESS;
    if (op >= YAKSA_OP__LAST)
        return YAKSA_ERR__INTERNAL;
    uintptr_t total = count * t->size;
    if (offset >= total)
        return YAKSA_SUCCESS;
    uintptr_t b0 = offset;
    uintptr_t b1 = yk_builtin_floor(t, count, b0 + YK_MIN(maxbytes, total - b0));
    if (yk_builtin_floor(t, count, b0) != b0)
        return YAKSA_ERR__INTERNAL;     /* offset inside a builtin: a precondition */
    if (b1 <= b0)
        return YAKSA_SUCCESS;
    if (op != YAKSA_OP__REPLACE && op_needs_host_arith(t, op))
        return YAKSA_ERR__NOT_SUPPORTED;        /* long double arithmetic has no GPU form */

    int rc = runtime_ready();
    if (rc)
        return rc;

    char *packed = dir == 0 ? (char *) packed_out : (char *) packed_in;
    cudaStream_t s = (mode == YK_MODE_STREAM && stream) ? *(cudaStream_t *) stream : R.stream;
    int host_hint = info && info->gpu_driver == 2;

    /* typed span touched by elements [e0, e1) */
    uintptr_t e0 = b0 / t->size, e1 = (b1 + t->size - 1) / t->size;
    int64_t ext = t->extent;
    int64_t lo = (ext >= 0 ? (int64_t) e0 * ext : (int64_t) (e1 - 1) * ext) + t->true_lb;
    int64_t hi = (ext >= 0 ? (int64_t) (e1 - 1) * ext : (int64_t) e0 * ext) + t->true_ub;

    int st_t = 0, st_p = 0;
    char *dtyped = device_alias(typed, typed + lo, host_hint, &st_t);
    char *dpacked = device_alias(packed, packed, host_hint, &st_p);
    void *scr_t = NULL, *scr_p = NULL;
    uintptr_t n = b1 - b0;

    if (st_t || st_p) {
        /* staged: copy what the kernel reads into device memory, run, copy back */
        __atomic_add_fetch(&R.staged_calls, 1, __ATOMIC_RELAXED);
        if (st_t) {
            rc = cuda_err(cudaMallocAsync(&scr_t, (size_t) (hi - lo), s), "cudaMallocAsync");
            if (rc)
                return rc;
            rc = cuda_err(cudaMemcpyAsync(scr_t, typed + lo, (size_t) (hi - lo),
                                          cudaMemcpyHostToDevice, s), "stage in");
            dtyped = (char *) scr_t - lo;
        }
        if (!rc && st_p) {
            rc = cuda_err(cudaMallocAsync(&scr_p, n, s), "cudaMallocAsync");
            if (!rc && (dir == 1 || op != YAKSA_OP__REPLACE))
                rc = cuda_err(cudaMemcpyAsync(scr_p, packed, n, cudaMemcpyHostToDevice, s),
                              "stage in");
            dpacked = scr_p;
        }
        if (!rc)
            rc = enqueue(dir, dtyped, dpacked, t, count, b0, b1, op, s);
        if (!rc && dir == 0 && st_p)
            rc = cuda_err(cudaMemcpyAsync(packed, scr_p, n, cudaMemcpyDeviceToHost, s),
                          "stage out");
        if (!rc && dir == 1 && st_t)
            rc = cuda_err(cudaMemcpyAsync(typed + lo, scr_t, (size_t) (hi - lo),
                                          cudaMemcpyDeviceToHost, s), "stage out");
        if (scr_t)
            cudaFreeAsync(scr_t, s);
        if (scr_p)
            cudaFreeAsync(scr_p, s);
        if (!rc)
            rc = cuda_err(cudaStreamSynchronize(s), "staged completion");
        if (!rc)
            *actual = n;
        return rc;
    }

    __atomic_add_fetch(&R.direct_calls, 1, __ATOMIC_RELAXED);
    rc = enqueue(dir, dtyped, dpacked, t, count, b0, b1, op, s);
    if (rc)
        return rc;
    *actual = n;
    if (mode == YK_MODE_STREAM)
        return YAKSA_SUCCESS;
    cudaEvent_t ev;
    rc = event_get(&ev);
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
    yk_type_ref(t);
    rc = request_new(ev, t, NULL, NULL, request);
    if (rc) {
        cudaEventSynchronize(ev);
        event_put(ev);
        yk_type_unref(t);
    }
    return rc;
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
    if (incount == 0) {
        *actual_pack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    TYPE_OR_FAIL(type, t);
    return yk_pup(0, NULL, outbuf, (char *) inbuf, incount, t, inoffset, max_pack_bytes,
                  actual_pack_bytes, info, op, YK_MODE_NONBLOCKING, NULL, request);
}

int yaksa_pack(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
               void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
               yaksa_info_t info, yaksa_op_t op)
{
    if (incount == 0) {
        *actual_pack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    TYPE_OR_FAIL(type, t);
    return yk_pup(0, NULL, outbuf, (char *) inbuf, incount, t, inoffset, max_pack_bytes,
                  actual_pack_bytes, info, op, YK_MODE_BLOCKING, NULL, NULL);
}

int yaksa_pack_stream(const void *inbuf, uintptr_t incount, yaksa_type_t type, uintptr_t inoffset,
                      void *outbuf, uintptr_t max_pack_bytes, uintptr_t * actual_pack_bytes,
                      yaksa_info_t info, yaksa_op_t op, void *stream)
{
    if (incount == 0) {
        *actual_pack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    TYPE_OR_FAIL(type, t);
    return yk_pup(0, NULL, outbuf, (char *) inbuf, incount, t, inoffset, max_pack_bytes,
                  actual_pack_bytes, info, op, YK_MODE_STREAM, stream, NULL);
}

int yaksa_iunpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                  yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                  yaksa_info_t info, yaksa_op_t op, yaksa_request_t * request)
{
    *request = YAKSA_REQUEST__NULL;
    if (outcount == 0) {
        *actual_unpack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    TYPE_OR_FAIL(type, t);
    return yk_pup(1, inbuf, NULL, (char *) outbuf, outcount, t, outoffset, insize,
                  actual_unpack_bytes, info, op, YK_MODE_NONBLOCKING, NULL, request);
}

int yaksa_unpack(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                 yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                 yaksa_info_t info, yaksa_op_t op)
{
    if (outcount == 0) {
        *actual_unpack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    TYPE_OR_FAIL(type, t);
    return yk_pup(1, inbuf, NULL, (char *) outbuf, outcount, t, outoffset, insize,
                  actual_unpack_bytes, info, op, YK_MODE_BLOCKING, NULL, NULL);
}

int yaksa_unpack_stream(const void *inbuf, uintptr_t insize, void *outbuf, uintptr_t outcount,
                        yaksa_type_t type, uintptr_t outoffset, uintptr_t * actual_unpack_bytes,
                        yaksa_info_t info, yaksa_op_t op, void *stream)
{
    if (outcount == 0) {
        *actual_unpack_bytes = 0;
        return YAKSA_SUCCESS;
    }
    TYPE_OR_FAIL(type, t);
    return yk_pup(1, inbuf, NULL, (char *) outbuf, outcount, t, outoffset, insize,
                  actual_unpack_bytes, info, op, YK_MODE_STREAM, stream, NULL);
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
