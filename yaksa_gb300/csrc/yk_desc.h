/*
 * yk_desc.h -- the flattened, device-resident type descriptor and the launch
 * interface between the C host library and the CUDA kernels.
 *
 * Plain C (no CUDA types), shared by the host code (yk_*.c) and the kernels
 * (yk_kernels.cu, yk_server.cu, yk_device.cuh).
 *
 * A committed type is flattened into a chain of levels, outermost first, ending in a
 * leaf.  A packed byte position p (relative to the start of the packed form of
 * `count` elements) is decomposed level by level, mixed-radix:
 *
 *   VEC  (count, stride, cps):  d = r / cps; r -= d * cps; off += d * stride
 *   IDX  (count, disp[], cps):  d = r / cps; r -= d * cps; off += disp[d]
 *   HIDX (count, disp[], pfx[], stride = child extent, cps = child packed size):
 *                               j = max{ j : pfx[j] <= r }; r -= pfx[j];
 *                               d = r / cps; r -= d * cps; off += disp[j] + d * stride
 *   leaf RUN (run):             off += r                       (r < run)
 *   leaf SEG (nseg, off[], pfx[], type[]):
 *                               s = max{ s : pfx[s] <= r }; off += seg_off[s] + r - pfx[s]
 *
 * Level 0 is always the element level VEC(count, extent, size).  This replaces the
 * reference's per-(kind, kind, type) generated kernels
 * (src/backend/cuda/genpup.py:106-197) and its per-thread linear scan over hindexed
 * blocks (genpup.py:150-163) with one table-driven decomposition.
 *
 * Divisions by cps use the Granlund-Montgomery round-up method for unsigned integer
 * division by invariant integers ("Division by Invariant Integers using
 * Multiplication", PLDI 1994, section 4): m = floor(2^N (2^l - d) / d) + 1 with
 * l = ceil(log2 d); q = (t + ((n - t) >> min(l,1))) >> max(l-1,0), t = mulhi(m, n).
 */
#ifndef YK_DESC_H_INCLUDED
#define YK_DESC_H_INCLUDED

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define YK_MAX_LEVELS 16

enum { YK_LV_VEC = 0, YK_LV_IDX = 1, YK_LV_HIDX = 2 };
enum { YK_LEAF_RUN = 0, YK_LEAF_SEG = 1 };

/* Base element types the kernels compute in.  Operator support per type follows the
 * reference's table (src/backend/gencomm.py:14-27); a combination outside the table
 * leaves the destination untouched. */
enum {
    YK_BT_NONE = 0,     /* raw bytes */
    YK_BT_BOOL,
    YK_BT_CHAR,         /* REPLACE only */
    YK_BT_WCHAR,        /* REPLACE only */
    YK_BT_I8, YK_BT_I16, YK_BT_I32, YK_BT_I64,
    YK_BT_F32, YK_BT_F64,
    YK_BT_C32, YK_BT_C64,       /* float / double complex */
    YK_BT_LDOUBLE, YK_BT_CLDOUBLE,      /* binary128 on the GPU (yk_quad.h) */
    YK_BT_LAST
};

typedef struct {
    int32_t kind;
    int32_t has_d32;            /* IDX, bit YK_D32_TABLE: an int32_t copy of disp[]
                                 * follows it, at (const int32_t *) (disp + count)
                                 * (every displacement fits in 32 bits); bit
                                 * YK_D32_OFFSETS: every displacement plus cps - 1 fits
                                 * too (the offsets inside blocks of cps bytes) */
    uint64_t count;
    int64_t stride;             /* VEC: byte stride; HIDX: child extent */
    uint64_t cps;               /* packed bytes per digit (child packed size) */
    uint64_t m64;               /* division magic (64-bit) */
    uint32_t m32;               /* division magic (32-bit, valid if cps < 2^32) */
    uint8_t l;                  /* ceil(log2 cps) */
    uint8_t pad1[3];
    const int64_t *disp;        /* device: IDX/HIDX displacements */
    const uint64_t *pfx;        /* device: HIDX packed prefix, count + 1 entries */
    const uint32_t *tfb;        /* device: HIDX first block of each 2^tshift-byte packed tile */
    uint32_t tshift;
    uint32_t pad2;
} yk_level;

/* yk_level.has_d32 bits */
#define YK_D32_TABLE 1
#define YK_D32_OFFSETS 2

typedef struct {
    int32_t nlev;
    int32_t leaf;
    uint64_t run;               /* RUN leaf length in bytes */
    uint64_t nseg;              /* SEG leaf */
    const int64_t *seg_off;     /* device */
    const uint64_t *seg_pfx;    /* device, nseg + 1 entries */
    const uint8_t *seg_type;    /* device, base type per segment (typed descriptors) */
    int32_t leaf_type;          /* base type of a RUN leaf (typed descriptors) */
    int32_t pad0;
    int64_t base;               /* constant byte offset added to the typed pointer */
    yk_level lv[YK_MAX_LEVELS];
} yk_desc;

/* One pack/unpack launch over the packed byte range [p0, p0 + nbytes). */
typedef struct {
    yk_desc desc;
    char *typed;                /* device-accessible pointer to the typed (strided) buffer */
    char *packed;               /* device-accessible pointer to packed byte p0 */
    uint64_t p0;
    uint64_t nbytes;
    uint64_t op;                /* yaksa_op_t */
    int32_t dir;                /* 0 = pack, 1 = unpack */
    int32_t vec;                /* bytes per work unit (REPLACE) or unit granule (ops) */
    int32_t typed_op;           /* 1 = elementwise operator on typed descriptor */
    int32_t use64;              /* 1 = positions need 64-bit arithmetic (the packed end
                                 * is above YK_POS32_END) */
    int32_t regular;            /* 0..YK_REGULAR_MAX: that many VEC levels over a RUN leaf
                                 * with 32-bit positions; -1: any other shape */
    int32_t hidx;               /* 1: one HIDX level of contiguous blocks over its run */
    int32_t ldouble;            /* 1: the type holds long double (binary128 operators) */
    int32_t form;               /* server items of sorted blocks (YK_SRV_OWNER_T): the
                                 * launch form the host chose, YK_FORM_* below */
} yk_launch;

#define YK_REGULAR_MAX 3

/* The largest packed end position the 32-bit kernels take.  Their loops step a 32-bit
 * unit index by a grid's stride (at most 64 CTAs per SM of 256 threads, one unit each:
 * under 2^24 units); ending 2^24 below 2^32 keeps index + stride from wrapping, which
 * would restart the loop and never end it. */
#define YK_POS32_END (0xffffffffull - (1ull << 24))

/* Up to YK_BATCH_MAX REPLACE requests with 32-bit positions in one launch; passed by
 * value as the kernel parameter (about 19 KB, under the 32 KB parameter limit). */
#define YK_BATCH_MAX 16
typedef struct {
    int32_t n;
    uint32_t tile_mul;          /* tile g of the launch runs tile (g * tile_mul) mod total,
                                 * a bijection (tile_mul coprime with the total) that
                                 * spreads consecutive CTAs over every request, so the
                                 * bandwidth-bound requests overlap the latency-bound
                                 * ones; 1 = request order */
    uint64_t tile_start[YK_BATCH_MAX + 1];      /* first tile of each request */
    yk_launch req[YK_BATCH_MAX];
} yk_batch;

/* Tiles of one batch request (units per tile depend on the batch's total size). */
int yk_cuda_batch_units_per_thread(uint64_t total_units);
uint64_t yk_cuda_tiles(uint64_t units, int units_per_thread);
int yk_cuda_launch_batch(const yk_batch * b, int units_per_thread, int regular, int ctas_per_sm,
                         void *stream);

/* ---------------------------------------------------------------------------
 * Persistent request server: a device-visible work queue drained by resident CTAs.
 * ------------------------------------------------------------------------- */
enum { YK_SRV_REGULAR = 0, YK_SRV_BYTES, YK_SRV_TYPED, YK_SRV_OWNER, YK_SRV_ORDERED, YK_SRV_HIDX,
    YK_SRV_RED, YK_SRV_OWNER_T, YK_SRV_RUNS, YK_SRV_LAST = YK_SRV_RUNS };
/* flag in yk_item.kind: the item's busy time is added to its request's req_busy */
#define YK_SRV_TIMED 0x100u

typedef struct {
    uint64_t seq;               /* item sequence number (the GPU checks it) */
    uint32_t req;               /* request record slot */
    uint32_t kind;              /* YK_SRV_* */
    uint64_t pb, pe;            /* packed byte range of this item */
} yk_item;

/* Claim lanes of the request server: item t belongs to lane t mod YK_SRV_LANES, and each
 * lane has its own claim counter, so resident CTAs contend on 16 addresses, not one. */
#define YK_SRV_LANES 16
#define YK_SRV_LANE_STRIDE 16

typedef struct {
    yk_launch *reqs;            /* request records (host-mapped, written by the host) */
    yk_item *items;             /* work items (host-mapped, written by the host) */
    unsigned long long *req_done;       /* per request slot: items finished (host-mapped,
                                         * reset by the host, counted by the GPU) */
    const volatile uint64_t *items_published;   /* items visible to the GPU (host) */
    const volatile int *stop;   /* host asks resident CTAs to leave */
    unsigned long long *next_item;      /* device memory: YK_SRV_LANES claim counters, one
                                         * per 128-byte line (YK_SRV_LANE_STRIDE words
                                         * apart); lane k's counter c means its next item
                                         * is c * YK_SRV_LANES + k */
    volatile uint32_t *status;  /* [0] idle exits, [1] stop exits, [2] rejected items */
    const uint64_t *req_nitems; /* per request slot: its item count (host-mapped, written
                                 * by the host before the items are published) */
    unsigned long long *cq;     /* completion queue (host-mapped, qr entries): slot + 1 of
                                 * each finished request, in finishing order; 0 = empty */
    unsigned long long *cq_tail;        /* device memory: next completion queue position */
    unsigned long long *req_busy;       /* per request slot (host-mapped): the summed busy
                                         * time of a timed request's items in ns, each from
                                         * its record load to its last byte (GPU global
                                         * timer; the host zeroes it before publishing) */
    uint32_t qi, qr;            /* ring sizes */
    uint32_t max_idle_spins;    /* iteration bound on the wait for new items */
    uint32_t idle_us;           /* a CTA that finds no item for this long leaves (GPU
                                 * global timer); max_idle_spins bounds it regardless */
} yk_server_args;

int yk_cuda_server_launch(const yk_server_args * a, int ctas, void *stream);

/* REPLACE pack of whole elements of one VEC level over a run of 17..47 bytes (not a
 * multiple of 16) that starts on 16 bytes in every element; units of 4 or 8 bytes */
int yk_cuda_launch_runs_pack(const yk_launch * l, uint32_t run, void *stream);
int yk_cuda_server_ctas(void);

/* Granlund-Montgomery constants for dividing by l->cps (host side). */
void yk_level_set_magic(yk_level * l);

/* Launch on `stream` (a cudaStream_t).  Returns 0 or a cudaError_t value. */
int yk_cuda_launch_pup(const yk_launch * l, void *stream);
/* the same with a launch shape: units per thread for the REPLACE byte kernels, and a
 * grid cap in CTAs per SM for every kernel (0, 0 = the defaults) */
int yk_cuda_launch_pup_cfg(const yk_launch * l, void *stream, int units_per_thread,
                           int ctas_per_sm);

/* Ordered unpack for types whose targets may overlap: sorted-block owner-computes
 * kernel when the descriptor allows it, otherwise a single-warp ordered kernel.
 * sorted_blocks & 3: 0 = any layout; 1 = one IDX level of sorted blocks; 2 = the same
 * with both sides aligned to the element size.  YK_ORD_RED set: one IDX level of equal
 * blocks in any order (or one VEC level), both sides aligned to the element size,
 * under an operator that yk_red_applies() accepts -- the launch folds the elements in
 * with L2 reductions. */
#define YK_ORD_RED 4
/* set with sorted_blocks 2: every target offset (displacement + position in its block)
 * fits in a signed 32-bit integer, so the chunk kernel may compute offsets in 32 bits */
#define YK_ORD_D32 8
int yk_cuda_launch_unpack_ordered(const yk_launch * l, int sorted_blocks, void *stream,
                                  int ctas_per_sm);
/* The sorted-block kernel form of an aligned typed unpack (sorted_blocks 2, 32-bit
 * positions, blocks of a power-of-two byte length): log2 of the block length in bits
 * 0-7, the bytes per lane of the chunk form (8 or 16; 0 for one element per lane) in
 * bits 8-15, YK_FORM_D32 for 32-bit target offsets, and YK_FORM_POW2 set.  0: no such
 * form (the generic kernels apply). */
#define YK_FORM_D32 (1 << 16)
#define YK_FORM_POW2 (1 << 17)
int yk_cuda_owner_form(const yk_launch * l, int sorted_blocks);
/* launches of the L2-reduction form so far */
unsigned long long yk_cuda_red_launches(void);

/* Operators that an overlapping unpack may apply as L2 reductions, in any order: the
 * integer operators whose result does not depend on the order of the contributions
 * (addition modulo 2^n, max, min, and, or, xor), on 4- and 8-byte integers.  The
 * launch also needs element-aligned sides, 32-bit positions and blocks under 2^32
 * bytes. */
static inline int yk_red_applies(int bt, uint64_t op)
{
    return (bt == YK_BT_I32 || bt == YK_BT_I64) &&
        (op == 0 /* MAX */ || op == 1 /* MIN */ || op == 2 /* SUM */ || op == 5 /* BAND */ ||
         op == 7 /* BOR */ || op == 9 /* BXOR */);
}

/* TMA form of a REPLACE launch over a regular nest (yk_tma.cu): 1 when it exists; the
 * launch returns -1 when it does not, else a cudaError_t value. */
int yk_cuda_tma_ok(const yk_launch * l);
int yk_cuda_launch_tma(const yk_launch * l, void *stream, int ctas_per_sm);

/* Segment-list expansion (yk_iov_dev.cu): out[k] = (buf + e * extent + tpl[j].off,
 * tpl[j].len) for piece g = first + k = e * n + j, k < m; with tpl NULL, one piece
 * (buf + off1, len1).  Returns a cudaError_t value. */
int yk_cuda_iov_expand(const char *buf, int64_t extent, const int64_t * tpl, uint64_t n, uint64_t first,
                       uint64_t m, int64_t off1, uint64_t len1, void *out, void *stream);

/* The hindexed unpack with the packed stream staged by bulk copies (yk_kernels.cu): -1
 * when it does not apply, else a cudaError_t value. */
int yk_cuda_launch_hidx_bulk(const yk_launch * l, void *stream, int ctas_per_sm);

/* SM count of the current device (cached). */
int yk_cuda_num_sms(void);

#ifdef __cplusplus
}
#endif
#endif /* YK_DESC_H_INCLUDED */
