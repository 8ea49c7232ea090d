/*
 * yk_internal.h -- host-side objects of the GB300 engine (types, info, requests).
 *
 * The type object keeps the reference's type model (src/frontend/include/yaksi.h:91-156:
 * kind, size, extent, lb/ub, true bounds, alignment, contiguity, per-kind parameters)
 * so that bounds and constructor results are identical, and adds what the GPU path
 * needs: the homogeneous base type, the uniform builtin size used to round partial
 * packs down to builtin boundaries, and a lazily built device descriptor.
 */
#ifndef YK_INTERNAL_H_INCLUDED
#define YK_INTERNAL_H_INCLUDED

#include <stdint.h>
#include <stdbool.h>
#include <pthread.h>
#include "yaksa.h"
#include "yk_desc.h"

enum { YK_K_BUILTIN, YK_K_CONTIG, YK_K_RESIZED, YK_K_HVECTOR, YK_K_BLKHINDX, YK_K_HINDEXED,
    YK_K_STRUCT, YK_K_SUBARRAY };

typedef struct yk_type yk_type;

/* a device-resident descriptor for one (type, flavour) pair */
typedef struct {
    int built;
    int status;                 /* YAKSA_SUCCESS or the error met while building */
    yk_desc d;                  /* level 0 count is filled per launch */
    void *dev_tables;           /* one device allocation holding every table */
    int vec_align;              /* largest power of two <= 16 dividing all offsets/runs */
    int elem_align;             /* typed: largest power of two dividing all element offsets */
    int unit;                   /* typed: gcd of element sizes (work-unit granule) */
    int may_overlap;            /* some typed-side bytes are reached twice */
    int sorted_blocks;          /* owner-computes ordered unpack applies */
    int disp32;                 /* sorted blocks: every target offset fits in 32 bits */
    int64_t elem_span;          /* bytes one element touches (element-level overlap test) */
    uint64_t table_bytes;
} yk_devdesc;

struct yk_type {
    int refcount;
    int kind;
    int tree_depth;
    int alignment;
    uintptr_t size;
    intptr_t extent, lb, ub, true_lb, true_ub;
    bool is_contig;
    uintptr_t num_contig;
    yaksa_type_t builtin;       /* canonical handle of a builtin object */
    intptr_t count, blocklength, stride;
    intptr_t *blens, *displs;
    yk_type *child;
    yk_type **types;
    int ndims;
    yk_type *primary;

    /* GPU-side derived data */
    int base_type;              /* YK_BT_* if every builtin has the same base type, else -1 */
    uintptr_t builtin_size;     /* size of every builtin (pair = one builtin), 0 if mixed */
    bool needs_host_ops;        /* contains long double data */
    pthread_mutex_t desc_mutex;
    yk_devdesc bytes_desc;      /* REPLACE: byte-exact, merges across base types */
    yk_devdesc typed_desc;      /* operators: segments carry their base type */
    /* the same two descriptors with their tables on the host heap, for requests
     * whose tables travel in the static device scratch (yaksa_gb300_pup_noalloc) */
    yk_devdesc host_bytes_desc;
    yk_devdesc host_typed_desc;
    /* segment list of one element (yaksa_gb300_iov_stream), built at its first use:
     * num_contig (offset, length) pieces on the host and on the device, and which
     * pieces are the first half of a pair builtin listed as two pieces */
    int iov_built, iov_status;
    int64_t *iov_tpl;           /* host: 2 x num_contig words (offset, length) */
    uint8_t *iov_first;
    void *iov_dev;              /* device copy of iov_tpl */
};

typedef struct {
    int refcount;
    int gpu_driver;             /* 0 unset, 1 cuda, 2 nogpu */
    int mapped_device;
    int has_wait_kernel;
    uintptr_t iov_pack_threshold, iov_unpack_threshold;
} yk_info;

/* globals */
extern pthread_mutex_t yk_global_mutex;
int yk_is_initialized(void);

/* type handles */
yk_type *yk_type_get(yaksa_type_t h);
void yk_type_ref(yk_type * t);
void yk_type_unref(yk_type * t);

/* builtin helpers */
int yk_builtin_base_type(yaksa_type_t canonical);
int yk_base_type_size(int bt);

/* descriptors (yk_build.c) */
int yk_desc_get(yk_type * t, int typed, yk_devdesc ** out);
int yk_desc_get_host(yk_type * t, int typed, yk_devdesc ** out);
/* field layout of a pair builtin (float_int, short_int, ...): 1 if h is one */
int yk_pair_fields(yaksa_type_t h, size_t off[2], size_t sz[2], int bt[2]);
/* 1 when a test asked the next device allocation to fail (yaksa_gb300_debug_fail_alloc) */
int yk_fail_injected(void);
/* yk_noalloc.cu: the current device's address of the static descriptor scratch */
int yk_noalloc_scratch(void **ptr, size_t * bytes);
void yk_desc_release(yk_type * t);
void yk_make_launch_desc(const yk_devdesc * dd, const yk_type * t, uintptr_t count, yk_desc * out);
uintptr_t yk_builtin_floor(yk_type * t, uintptr_t count, uintptr_t pos);
/* yk_iov.c: release a type's segment-list template */
void yk_iov_release(yk_type * t);

/* GPU runtime (yk_runtime.c) */
/* has_wait_kernel: the yaksa_has_wait_kernel hint of yaksa_init's info */
int yk_runtime_init(int has_wait_kernel);
void yk_runtime_finalize(void);
int yk_pup(int dir, const void *packed_in, void *packed_out, char *typed, uintptr_t count,
           yk_type * t, uintptr_t offset, uintptr_t maxbytes, uintptr_t * actual,
           yk_info * info, yaksa_op_t op, int mode, void *stream, yaksa_request_t * request);

#define YK_MODE_NONBLOCKING 0
#define YK_MODE_BLOCKING    1
#define YK_MODE_STREAM      2

#define YK_MIN(a, b) ((a) < (b) ? (a) : (b))
#define YK_MAX(a, b) ((a) > (b) ? (a) : (b))

#endif /* YK_INTERNAL_H_INCLUDED */
