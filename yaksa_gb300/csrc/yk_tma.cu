/*
 * yk_tma.cu -- tensor-memory-accelerator (TMA) form of the REPLACE kernels for regular
 * nests: a vector / hvector / subarray nest of up to three strided levels over one
 * contiguous run of at most 256 bytes, whole requests only.  No counterpart in the
 * reference, whose generated kernels move one element per thread
 * (src/backend/cuda/genpup.py:106-197).
 *
 * The typed side is described to the TMA unit as a tensor: dimension 0 is the bytes of
 * one run (from the 16-byte boundary at or below its start), dimensions 1..3 are the
 * nest's levels, innermost first, with the levels' byte strides.  A tile is a box of one
 * row-width (a multiple of 16 bytes) by up to 256 rows of the innermost level:
 *
 *   pack:   cp.async.bulk.tensor loads the box into shared memory (bytes past the run
 *           are zero-filled by the unit, never read from memory); the CTA's threads
 *           copy each row's run to its place in the packed stream with the widest
 *           unit that the run, its offset and the packed pointer allow.  Two stages:
 *           the next tile's load is in flight while this tile is copied out.
 *   unpack: only when every run is a whole number of 16-byte units on a 16-byte
 *           boundary (a box store then writes exactly the runs): cp.async.bulk loads
 *           the tile's packed bytes into shared memory and cp.async.bulk.tensor stores
 *           the box; the unit clips rows past the end.
 *
 * One CTA per tile at a time, tiles grid-stride, one elected thread issues the copies.
 * Every mbarrier wait is bounded: after the limit the CTA records a failure in
 * yk_tma_failures, waits (bounded again) for its copies in flight, and leaves.
 *
 * All addresses are in this GPU's own memory or in host memory it addresses in place;
 * no multicast is used.
 */
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <pthread.h>
#include <stdint.h>
#include <string.h>
#include "yk_desc.h"

#define YK_TMA_THREADS 256
#define YK_TMA_STAGE_BYTES 8192
#define YK_TMA_SPIN_LIMIT (1u << 24)

__device__ unsigned int yk_tma_failures;

struct yk_tma_args {             /* 64-byte aligned: CUtensorMap is */
    CUtensorMap map;            /* typed side, rank 4: {row bytes, n1, n2, n3} */
    char *packed;
    uint32_t run;               /* bytes of one run */
    uint32_t mis;               /* offset of the run within its 16-byte-aligned row */
    uint32_t rowpad;            /* box width in bytes: mis + run rounded up to 16 */
    uint32_t b1;                /* rows per box */
    uint32_t n1, n2, n3;        /* rows of the innermost level, then the outer levels */
    uint32_t tiles1;            /* boxes along n1 */
    uint32_t unit;              /* bytes per packed-side move in the pack copy */
    uint32_t pad;
    uint64_t ntiles;
};

__device__ __forceinline__ uint32_t yk_smem(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

__device__ __forceinline__ void yk_mbar_init(uint64_t *b)
{
    asm volatile ("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(yk_smem(b)) : "memory");
}

__device__ __forceinline__ void yk_mbar_expect(uint64_t *b, uint32_t tx)
{
    asm volatile ("{\n\t.reg .b64 st;\n\t"
                  "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}"
                  :: "r"(yk_smem(b)), "r"(tx) : "memory");
}

__device__ __forceinline__ bool yk_mbar_try(uint64_t *b, uint32_t parity)
{
    uint32_t ok;
    asm volatile ("{\n\t.reg .pred p;\n\t"
                  "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                  "selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(yk_smem(b)), "r"(parity) : "memory");
    return ok != 0;
}

/* bounded wait for a phase; false after the limit (failure recorded once per CTA) */
__device__ __forceinline__ bool yk_mbar_wait(uint64_t *b, uint32_t parity)
{
    for (uint32_t i = 0; i < YK_TMA_SPIN_LIMIT; i++)
        if (yk_mbar_try(b, parity))
            return true;
    return false;
}

__device__ __forceinline__ void yk_tma_load(void *dst, const CUtensorMap * m, int x, int y, int z, int w,
                                            uint64_t *bar)
{
    asm volatile ("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                  " [%0], [%1, {%2, %3, %4, %5}], [%6];"
                  :: "r"(yk_smem(dst)), "l"(m), "r"(x), "r"(y), "r"(z), "r"(w), "r"(yk_smem(bar))
                  : "memory");
}

__device__ __forceinline__ void yk_tma_store(const CUtensorMap * m, int x, int y, int z, int w,
                                             const void *src)
{
    asm volatile ("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group"
                  " [%0, {%1, %2, %3, %4}], [%5];"
                  :: "l"(m), "r"(x), "r"(y), "r"(z), "r"(w), "r"(yk_smem(src)) : "memory");
}

__device__ __forceinline__ void yk_bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile ("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                  :: "r"(yk_smem(dst)), "l"(src), "r"(bytes), "r"(yk_smem(bar)) : "memory");
}

__device__ __forceinline__ void yk_tile_coords(const yk_tma_args & A, uint64_t t, uint32_t *r0, uint32_t *i2,
                                               uint32_t *i3)
{
    const uint32_t t1 = (uint32_t) (t % A.tiles1);
    const uint64_t rest = t / A.tiles1;
    *r0 = t1 * A.b1;
    *i2 = (uint32_t) (rest % A.n2);
    *i3 = (uint32_t) (rest / A.n2);
}

template <typename U>
__device__ __forceinline__ void yk_tma_copy_out(const yk_tma_args & A, const unsigned char *tile,
                                                uint32_t rows, uint64_t q0)
{
    /* the tile's rows are consecutive in the packed stream: rows x run bytes from q0 * run */
    U *dst = (U *) (A.packed + q0 * (uint64_t) A.run);
    const uint32_t per_row = A.run / (uint32_t) sizeof(U);
    const uint32_t total = rows * per_row;
    for (uint32_t k = threadIdx.x; k < total; k += YK_TMA_THREADS) {
        const uint32_t r = k / per_row, c = k - r * per_row;
        dst[k] = *(const U *) (tile + (size_t) r * A.rowpad + A.mis + (size_t) c * sizeof(U));
    }
}

__global__ void __launch_bounds__(YK_TMA_THREADS) yk_tma_pack_kernel(const __grid_constant__ yk_tma_args A)
{
    extern __shared__ __align__(128) unsigned char yk_tma_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int s_ok;
    const uint32_t stage = A.rowpad * A.b1;
    if (threadIdx.x == 0) {
        yk_mbar_init(&bar[0]);
        yk_mbar_init(&bar[1]);
        asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    uint32_t parity = 0;        /* bit k: the phase stage k waits for next */
    uint64_t t = blockIdx.x;
    int s = 0;
    if (threadIdx.x == 0 && t < A.ntiles) {
        uint32_t r0, i2, i3;
        yk_tile_coords(A, t, &r0, &i2, &i3);
        yk_mbar_expect(&bar[0], stage);
        yk_tma_load(yk_tma_smem, &A.map, 0, (int) r0, (int) i2, (int) i3, &bar[0]);
    }
    bool failed = false;
    for (; t < A.ntiles; t += gridDim.x, s ^= 1) {
        /* the next tile's load goes into the other stage (freed at the end of the last
         * iteration by the barrier below) */
        const uint64_t tn = t + gridDim.x;
        if (threadIdx.x == 0) {
            if (tn < A.ntiles) {
                uint32_t r0, i2, i3;
                yk_tile_coords(A, tn, &r0, &i2, &i3);
                /* the generic reads of that stage ended at the last barrier */
                asm volatile ("fence.proxy.async.shared::cta;" ::: "memory");
                yk_mbar_expect(&bar[s ^ 1], stage);
                yk_tma_load(yk_tma_smem + (size_t) (s ^ 1) * stage, &A.map, 0, (int) r0, (int) i2,
                            (int) i3, &bar[s ^ 1]);
            }
            /* one thread decides whether the tile arrived, so the CTA never diverges */
            s_ok = yk_mbar_wait(&bar[s], (parity >> s) & 1);
        }
        __syncthreads();
        if (!s_ok) {
            failed = true;
            break;
        }
        (void) yk_mbar_try(&bar[s], (parity >> s) & 1);     /* observe the completed phase */
        parity ^= 1u << s;
        uint32_t r0, i2, i3;
        yk_tile_coords(A, t, &r0, &i2, &i3);
        const uint32_t rows = min(A.b1, A.n1 - r0);
        const uint64_t q0 = (uint64_t) r0 + (uint64_t) A.n1 * ((uint64_t) i2 + (uint64_t) A.n2 * i3);
        const unsigned char *tile = yk_tma_smem + (size_t) s * stage;
        switch (A.unit) {
            case 16: yk_tma_copy_out<uint4>(A, tile, rows, q0); break;
            case 8: yk_tma_copy_out<uint2>(A, tile, rows, q0); break;
            case 4: yk_tma_copy_out<uint32_t>(A, tile, rows, q0); break;
            case 2: yk_tma_copy_out<uint16_t>(A, tile, rows, q0); break;
            default: yk_tma_copy_out<uint8_t>(A, tile, rows, q0); break;
        }
        /* every thread is done with this stage before a load may overwrite it */
        __syncthreads();
    }
    if (failed && threadIdx.x == 0) {
        atomicAdd(&yk_tma_failures, 1u);
        /* let loads still in flight land before the CTA's shared memory is released */
        (void) yk_mbar_wait(&bar[0], parity & 1);
        (void) yk_mbar_wait(&bar[1], (parity >> 1) & 1);
    }
}

__global__ void __launch_bounds__(YK_TMA_THREADS) yk_tma_unpack_kernel(const __grid_constant__ yk_tma_args A)
{
    extern __shared__ __align__(128) unsigned char yk_tma_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    const uint32_t stage = A.rowpad * A.b1;
    if (threadIdx.x == 0) {
        yk_mbar_init(&bar[0]);
        yk_mbar_init(&bar[1]);
        asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;         /* one thread moves everything: both directions are bulk copies */
    uint32_t parity = 0;
    int s = 0;
    bool failed = false;
    for (uint64_t t = blockIdx.x; t < A.ntiles; t += gridDim.x, s ^= 1) {
        uint32_t r0, i2, i3;
        yk_tile_coords(A, t, &r0, &i2, &i3);
        const uint32_t rows = min(A.b1, A.n1 - r0);
        const uint64_t q0 = (uint64_t) r0 + (uint64_t) A.n1 * ((uint64_t) i2 + (uint64_t) A.n2 * i3);
        unsigned char *buf = yk_tma_smem + (size_t) s * stage;
        /* the store that read this stage two tiles ago is done reading it */
        asm volatile ("cp.async.bulk.wait_group.read 1;" ::: "memory");
        yk_mbar_expect(&bar[s], rows * A.run);
        yk_bulk_load(buf, A.packed + q0 * (uint64_t) A.run, rows * A.run, &bar[s]);
        if (!yk_mbar_wait(&bar[s], (parity >> s) & 1)) {
            failed = true;
            break;
        }
        parity ^= 1u << s;
        asm volatile ("fence.proxy.async.shared::cta;" ::: "memory");
        yk_tma_store(&A.map, 0, (int) r0, (int) i2, (int) i3, buf);
        asm volatile ("cp.async.bulk.commit_group;" ::: "memory");
    }
    if (failed) {
        atomicAdd(&yk_tma_failures, 1u);
        (void) yk_mbar_wait(&bar[0], parity & 1);
        (void) yk_mbar_wait(&bar[1], (parity >> 1) & 1);
    }
    asm volatile ("cp.async.bulk.wait_group 0;" ::: "memory");
}

/* ------------------------------------------------------------------------- */
/* host side                                                                 */
/* ------------------------------------------------------------------------- */

static PFN_cuTensorMapEncodeTiled_v12000 yk_encode;
static pthread_once_t yk_encode_once = PTHREAD_ONCE_INIT;

static void yk_encode_init(void)
{
    cudaDriverEntryPointQueryResult q;
    void *fn = NULL;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
        cudaSuccess && q == cudaDriverEntryPointSuccess)
        yk_encode = (PFN_cuTensorMapEncodeTiled_v12000) fn;
    else
        cudaGetLastError();
}

static int yk_pow2_of(uint64_t v)
{
    int a = 16;
    while (a > 1 && (v % (uint64_t) a))
        a >>= 1;
    return a;
}

/* Whether the launch has a TMA form (see the file comment), and its arguments; the
 * tensor map is encoded only when `encode` is set. */
static bool yk_tma_plan(const yk_launch * L, yk_tma_args * A, bool encode)
{
    const yk_desc & d = L->desc;
    if (L->typed_op || L->use64 || L->regular < 1 || d.leaf != YK_LEAF_RUN || d.nlev < 1 || d.nlev > 3)
        return false;
    const uint64_t run = d.run;
    /* levels outermost first; the packed bytes must be the whole nest, densely */
    uint64_t cps = run;
    for (int i = d.nlev - 1; i >= 0; i--) {
        const yk_level & l = d.lv[i];
        if (l.kind != YK_LV_VEC || l.cps != cps || l.stride <= 0 || (l.stride & 15) ||
            (uint64_t) l.stride >= (1ull << 40) || l.count == 0 || l.count > 0x7fffffffull)
            return false;
        cps *= l.count;
    }
    if (L->p0 != 0 || L->nbytes != cps)
        return false;
    const uintptr_t base = (uintptr_t) (L->typed + d.base);
    const uint32_t mis = (uint32_t) (base & 15);
    const uint64_t rowpad = (mis + run + 15) & ~15ull;
    if (run == 0 || rowpad > 256)
        return false;
    if (L->dir == 1 && (mis != 0 || (run & 15) || ((uintptr_t) L->packed & 15)))
        return false;   /* a box store must write exactly the runs */
    memset(A, 0, sizeof(*A));
    const yk_level *inner = &d.lv[d.nlev - 1];
    A->run = (uint32_t) run;
    A->mis = mis;
    A->rowpad = (uint32_t) rowpad;
    A->n1 = (uint32_t) inner->count;
    A->n2 = d.nlev >= 2 ? (uint32_t) d.lv[d.nlev - 2].count : 1;
    A->n3 = d.nlev >= 3 ? (uint32_t) d.lv[0].count : 1;
    uint32_t b1 = (uint32_t) (YK_TMA_STAGE_BYTES / rowpad);
    if (b1 > 256)
        b1 = 256;
    if (b1 > A->n1)
        b1 = A->n1;
    A->b1 = b1;
    A->tiles1 = (A->n1 + b1 - 1) / b1;
    A->ntiles = (uint64_t) A->tiles1 * A->n2 * A->n3;
    A->packed = L->packed;
    int u = yk_pow2_of(run);
    u = u < yk_pow2_of(mis + 16) ? u : yk_pow2_of(mis + 16);
    int pu = yk_pow2_of((uint64_t) (uintptr_t) L->packed);
    A->unit = (uint32_t) (u < pu ? u : pu);
    /* the tensor: bytes of a row, then the levels innermost first; the strides of absent
     * levels repeat the last one (their extent is 1, so they are never stepped) */
    cuuint64_t dims[4] = { mis + run, A->n1, A->n2, A->n3 };
    cuuint64_t strides[3];
    strides[0] = (cuuint64_t) inner->stride;
    strides[1] = d.nlev >= 2 ? (cuuint64_t) d.lv[d.nlev - 2].stride : strides[0];
    strides[2] = d.nlev >= 3 ? (cuuint64_t) d.lv[0].stride : strides[1];
    cuuint32_t box[4] = { (cuuint32_t) rowpad, b1, 1, 1 }, es[4] = { 1, 1, 1, 1 };
    if (!encode)
        return true;
    pthread_once(&yk_encode_once, yk_encode_init);
    if (!yk_encode)
        return false;
    CUresult r = yk_encode(&A->map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 4, (void *) (base - mis), dims, strides,
                           box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

extern "C" int yk_cuda_tma_ok(const yk_launch * l)
{
    yk_tma_args A;
    return yk_tma_plan(l, &A, false) ? 1 : 0;
}

static unsigned long long yk_tma_launches;

/* launches of the forms that move data with the tensor memory accelerator (tensor maps
 * here, and the bulk-staged hindexed unpack) */
extern "C" void yk_tma_count_launch(void)
{
    __atomic_add_fetch(&yk_tma_launches, 1ull, __ATOMIC_RELAXED);
}

extern "C" int yk_cuda_num_sms(void);

/* Launch the TMA form with ctas_per_sm resident CTAs per SM (0: 4); returns a
 * cudaError_t value, or -1 when the launch has no TMA form. */
extern "C" int yk_cuda_launch_tma(const yk_launch * l, void *stream, int ctas_per_sm)
{
    yk_tma_args A;
    if (!yk_tma_plan(l, &A, true))
        return -1;
    __atomic_add_fetch(&yk_tma_launches, 1ull, __ATOMIC_RELAXED);
    const uint32_t smem = 2 * A.rowpad * A.b1;
    uint64_t cap = (uint64_t) yk_cuda_num_sms() * (uint64_t) (ctas_per_sm > 0 ? ctas_per_sm : 4);
    unsigned g = (unsigned) (A.ntiles < cap ? A.ntiles : cap);
    cudaStream_t s = (cudaStream_t) stream;
    if (l->dir == 0)
        yk_tma_pack_kernel<<<g ? g : 1, YK_TMA_THREADS, smem, s>>>(A);
    else
        yk_tma_unpack_kernel<<<g ? g : 1, YK_TMA_THREADS, smem, s>>>(A);
    return (int) cudaGetLastError();
}

/* launches of the TMA-unit forms so far, and tensor-map waits that ran out (0 in
 * correct operation) */
extern "C" int yaksa_gb300_debug_tma_stats(unsigned long long *launches, unsigned int *failures)
{
    *launches = __atomic_load_n(&yk_tma_launches, __ATOMIC_RELAXED);
    return cudaMemcpyFromSymbol(failures, yk_tma_failures, sizeof(unsigned int)) == cudaSuccess ? 0 : 2;
}
