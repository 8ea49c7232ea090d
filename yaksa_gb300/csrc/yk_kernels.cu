/*
 * yk_kernels.cu -- pack/unpack kernels for sm_103a.
 *
 * One kernel family replaces the reference's 3,720 generated kernels
 * (src/backend/cuda/genpup.py:106-197).  Each thread moves V-byte units of the packed
 * stream; the typed-side address of a unit comes from decomposing its packed position
 * over the descriptor (yk_desc.h).  V is the largest power of two <= 16 that divides
 * every run length, offset and pointer involved, so both the packed side (always
 * contiguous, coalesced) and the typed side move in 16-byte vectors wherever the
 * innermost contiguous run and alignment allow.
 *
 * Operators follow the reference's elementwise definitions exactly
 * (src/backend/seq/genpup.py:302-327, identical on the GPU in
 * src/backend/cuda/genpup.py:336-361): out = op(in, out), integer MAX/MIN as signed
 * compare-selects, float MAX/MIN as the selects x_[in < out] / x_[in > out] (not
 * fmax/fmin), integer SUM/PROD wrapping, LAND/LOR/LXOR producing 0/1.  Float
 * arithmetic uses the _rn intrinsics so no multiply-add is ever contracted into an
 * FMA (the reference compiles with -std=c11, which disables contraction), and complex
 * multiplication recovers infinities with the algorithm of ISO C11 Annex G.5.1 (what
 * libgcc's __mulsc3/__muldc3 implement for the reference's `*=` on _Complex values).
 */
#include "yk_device.cuh"

template <int V, int DIR, int U>
__global__ void __launch_bounds__(YK_THREADS, (U == 1 ? 8 : 4))
yk_regular_kernel(const __grid_constant__ yk_launch L)
{
    const uint32_t nunits = (uint32_t) (L.nbytes / V);
    const uint32_t tile = (uint32_t) YK_THREADS * U;
    for (uint32_t t0 = blockIdx.x * tile; t0 < nunits; t0 += gridDim.x * tile)
        yk_regular_dispatch<V, DIR, U>(L, t0, nunits);
}

/* A batch of regular REPLACE requests: tiles numbered consecutively over requests. */
template <int U>
__global__ void __launch_bounds__(YK_THREADS, (U == 1 ? 8 : 4))
yk_batch_regular_kernel(const __grid_constant__ yk_batch B)
{
    const uint64_t ntiles = B.tile_start[B.n];
    for (uint64_t g0 = blockIdx.x; g0 < ntiles; g0 += gridDim.x) {
        const uint64_t g = B.tile_mul > 1 ? (g0 * B.tile_mul) % ntiles : g0;
        int r = 0;
        while (g >= B.tile_start[r + 1])
            r++;
        const yk_launch & L = B.req[r];
        const uint32_t nunits = (uint32_t) (L.nbytes / (uint64_t) L.vec);
        const uint32_t t0 = (uint32_t) (g - B.tile_start[r]) * (uint32_t) (YK_THREADS * U);
#define YK_RB(V) do { if (L.dir == 0) yk_regular_dispatch<V, 0, U>(L, t0, nunits); \
                      else yk_regular_dispatch<V, 1, U>(L, t0, nunits); } while (0)
        switch (L.vec) {
            case 16: YK_RB(16); break;
            case 8: YK_RB(8); break;
            case 4: YK_RB(4); break;
            case 2: YK_RB(2); break;
            default: YK_RB(1); break;
        }
#undef YK_RB
    }
}

/* Contiguous-block hindexed (one HIDX level whose blocks are contiguous runs): each
 * warp takes groups of 32 consecutive blocks; lane k holds block k's packed start and
 * displacement in registers, the warp walks the group's packed bytes in coalesced
 * strides of 32 units, and each unit finds its block with a 5-step shuffle search over
 * the lanes' starts.  No shared memory, no block barriers, no per-unit index loads. */
#define YK_HW_UNROLL 4

template <int V, int DIR>
__global__ void __launch_bounds__(YK_THREADS)
yk_hidx_kernel(const __grid_constant__ yk_launch L)
{
    typedef typename yk_vec<V>::T VT;
    const yk_level *lv = &L.desc.lv[0];
    const uint64_t p0 = L.p0, p1 = L.p0 + L.nbytes;
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t) blockIdx.x * YK_THREADS + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t) gridDim.x * YK_THREADS) >> 5;
    char *typed = L.typed + L.desc.base;
    VT *packed = (VT *) L.packed;
    /* blocks overlapping [p0, p1) (warp-uniform) */
    const uint64_t jb = yk_hidx_block(lv, p0), je = yk_hidx_block(lv, p1 - 1);
    const uint64_t ngroups = (je - jb + 32) / 32;
    for (uint64_t g = warp; g < ngroups; g += nwarps) {
        const uint64_t j0 = jb + g * 32;
        const uint64_t jl = j0 + (uint64_t) lane;
        const uint64_t my_pfx = jl <= je ? __ldg(lv->pfx + jl) : ~(uint64_t) 0;
        const int64_t my_disp = jl <= je ? __ldg(lv->disp + jl) : 0;
        const uint64_t jend = min(j0 + 32, je + 1);
        uint64_t start = __shfl_sync(0xffffffffu, my_pfx, 0);
        uint64_t end = __ldg(lv->pfx + jend);
        start = max(start, p0);
        end = min(end, p1);
        for (uint64_t base = start; base < end; base += (uint64_t) 32 * V * YK_HW_UNROLL) {
            int64_t off[YK_HW_UNROLL];
            bool act[YK_HW_UNROLL];
#pragma unroll
            for (int k = 0; k < YK_HW_UNROLL; k++) {
                const uint64_t p = base + (uint64_t) (k * 32 + lane) * V;
                act[k] = p < end;
                int idx = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    uint64_t c = __shfl_sync(0xffffffffu, my_pfx, idx + step);
                    if (c <= p)
                        idx += step;
                }
                const uint64_t bp = __shfl_sync(0xffffffffu, my_pfx, idx);
                const int64_t bd = __shfl_sync(0xffffffffu, my_disp, idx);
                off[k] = bd + (int64_t) (p - bp);
            }
            if (DIR == 0) {
                VT v[YK_HW_UNROLL];
#pragma unroll
                for (int k = 0; k < YK_HW_UNROLL; k++)
                    if (act[k])
                        v[k] = yk_ldcg((const VT *) (typed + off[k]));
#pragma unroll
                for (int k = 0; k < YK_HW_UNROLL; k++)
                    if (act[k])
                        packed[(base + (uint64_t) (k * 32 + lane) * V - p0) / V] = v[k];
            } else {
                VT v[YK_HW_UNROLL];
#pragma unroll
                for (int k = 0; k < YK_HW_UNROLL; k++)
                    if (act[k])
                        v[k] = yk_ldcg((const VT *) (packed + (base + (uint64_t) (k * 32 + lane) * V - p0) / V));
#pragma unroll
                for (int k = 0; k < YK_HW_UNROLL; k++)
                    if (act[k])
                        *(VT *) (typed + off[k]) = v[k];
            }
        }
    }
}

/* yk_hidx32_groups over the whole request, MINB CTAs of the block size resident */
template <int V, int DIR, int U, int MINB, bool PF>
__global__ void __launch_bounds__(YK_THREADS, MINB)
yk_hidx32_kernel(const __grid_constant__ yk_launch L)
{
    yk_hidx32_groups<V, DIR, U, PF>(L, L.p0, L.p0 + L.nbytes,
                                    ((uint64_t) blockIdx.x * YK_THREADS + threadIdx.x) >> 5,
                                    ((uint64_t) gridDim.x * YK_THREADS) >> 5);
}


/* ------------------------------------------------------------------------- */
/* hindexed unpack with the packed stream staged by bulk copies               */
/* ------------------------------------------------------------------------- */

/* The unpack of a contiguous-block hindexed request reads the packed stream in order,
 * so that side can move as whole tiles: one elected thread issues cp.async.bulk of the
 * next YK_HB_STAGES tiles (8 KiB each) into shared memory, completion counted by one
 * mbarrier per stage, and the CTA's warps scatter the current tile to the typed side
 * with the shuffle search of yk_hidx32_kernel (lane k holds block k's start relative to
 * the group and its typed offset).  The loads cost no registers, so each SM keeps tens
 * of KiB of packed bytes in flight instead of one vector per lane.  The packed pointer
 * sits on 16 bytes (checked on the host); the last tile's bytes past its last 16-byte
 * boundary are read with plain loads, so nothing beyond the request is read.  Every
 * wait is bounded: a CTA that runs out counts a failure in yk_hb_failures, waits
 * (bounded) for its copies in flight and leaves. */
#define YK_HB_TILE 8192
#define YK_HB_STAGES 3
#define YK_HB_SPINS (1u << 24)

__device__ unsigned int yk_hb_failures;

__device__ __forceinline__ uint32_t yk_hb_smem(const void *p) { return (uint32_t) __cvta_generic_to_shared(p); }

__device__ __forceinline__ bool yk_hb_try(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile ("{\n\t.reg .pred p;\n\t"
                  "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                  "selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(yk_hb_smem(bar)), "r"(parity) : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool yk_hb_wait(uint64_t *bar, uint32_t parity)
{
    for (uint32_t i = 0; i < YK_HB_SPINS; i++)
        if (yk_hb_try(bar, parity))
            return true;
    return false;
}

/* thread 0: tile t (packed bytes [t * TILE, ...) of the request) into stage k */
__device__ __forceinline__ void yk_hb_issue(const yk_launch & L, uint32_t t, unsigned char *stage,
                                            uint64_t *bar)
{
    const uint64_t q0 = (uint64_t) t * YK_HB_TILE;
    const uint32_t bytes = (uint32_t) min((uint64_t) YK_HB_TILE, L.nbytes - q0);
    const uint32_t bulk = bytes & ~15u;
    asm volatile ("{\n\t.reg .b64 st;\n\t"
                  "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n}"
                  :: "r"(yk_hb_smem(bar)), "r"(bulk) : "memory");
    if (bulk)
        asm volatile ("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                      :: "r"(yk_hb_smem(stage)), "l"(L.packed + q0), "r"(bulk), "r"(yk_hb_smem(bar))
                      : "memory");
}

template <int V>
__global__ void __launch_bounds__(YK_THREADS, 4)
yk_hidx_unpack_bulk_kernel(const __grid_constant__ yk_launch L)
{
    typedef typename yk_vec<V>::T VT;
    extern __shared__ __align__(128) unsigned char yk_hb_tiles[];
    __shared__ __align__(8) uint64_t bar[YK_HB_STAGES];
    __shared__ int s_ok;
    const yk_level *lv = &L.desc.lv[0];
    const uint64_t p0 = L.p0, n = L.nbytes;
    const uint32_t ntiles = (uint32_t) ((n + YK_HB_TILE - 1) / YK_HB_TILE);
    char *typed = L.typed + L.desc.base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int k = 0; k < YK_HB_STAGES; k++)
            asm volatile ("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(yk_hb_smem(&bar[k])) : "memory");
        asm volatile ("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int k = 0; k < YK_HB_STAGES; k++) {
            const uint32_t t = blockIdx.x + (uint32_t) k * gridDim.x;
            if (t < ntiles)
                yk_hb_issue(L, t, yk_hb_tiles + (size_t) k * YK_HB_TILE, &bar[k]);
        }
    }
    __syncthreads();
    uint32_t phase = 0;         /* bit k: the parity stage k waits for next */
    bool failed = false;
    int k = 0;
    for (uint32_t t = blockIdx.x; t < ntiles; t += gridDim.x, k = (k + 1 == YK_HB_STAGES) ? 0 : k + 1) {
        unsigned char *tile = yk_hb_tiles + (size_t) k * YK_HB_TILE;
        const uint64_t q0 = (uint64_t) t * YK_HB_TILE;
        const uint32_t bytes = (uint32_t) min((uint64_t) YK_HB_TILE, n - q0);
        if (threadIdx.x == 0) {
            s_ok = yk_hb_wait(&bar[k], (phase >> k) & 1);
            /* the bytes past the last 16-byte boundary (last tile only), plain loads */
            for (uint32_t b = bytes & ~15u; s_ok && b < bytes; b++)
                tile[b] = (unsigned char) L.packed[q0 + b];
        }
        __syncthreads();
        if (!s_ok) {
            failed = true;
            break;
        }
        (void) yk_hb_try(&bar[k], (phase >> k) & 1);      /* observe the completed phase */
        phase ^= 1u << k;
        /* the blocks that intersect the tile, in groups of 32 per warp */
        const uint64_t a = p0 + q0, e = a + bytes;
        const uint64_t jb = yk_hidx_block(lv, a), je = yk_hidx_block(lv, e - 1);
        const uint64_t ngroups = (je - jb + 32) / 32;
        for (uint64_t g = (uint64_t) warp; g < ngroups; g += YK_THREADS / 32) {
            const uint64_t j0 = jb + g * 32, jl = j0 + (uint64_t) lane;
            const uint64_t jend = min(j0 + 32, je + 1);
            const uint64_t gs = max(__ldg(lv->pfx + j0), a);
            const uint32_t ng = (uint32_t) (min(__ldg(lv->pfx + jend), e) - gs);
            uint32_t my_rel = 0xffffffffu;
            int64_t my_adj = 0;
            if (jl < jend) {
                const uint64_t bp = __ldg(lv->pfx + jl);
                my_rel = bp <= gs ? 0u : (uint32_t) (bp - gs);
                my_adj = __ldg(lv->disp + jl) - ((int64_t) bp - (int64_t) gs);
            }
            const unsigned char *src = tile + (gs - a);
            for (uint32_t base = 0; base < ng; base += 32u * V * YK_HW_UNROLL) {
#pragma unroll
                for (int u = 0; u < YK_HW_UNROLL; u++) {
                    const uint32_t r = base + (uint32_t) (u * 32 + lane) * V;
                    int idx = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const uint32_t c = __shfl_sync(0xffffffffu, my_rel, idx + step);
                        if (c <= r)
                            idx += step;
                    }
                    const int64_t off = __shfl_sync(0xffffffffu, my_adj, idx) + (int64_t) r;
                    if (r < ng)
                        *(VT *) (typed + off) = *(const VT *) (src + r);
                }
            }
        }
        /* every warp is done with this stage: refill it with the tile STAGES ahead */
        __syncthreads();
        if (threadIdx.x == 0) {
            const uint32_t tn = t + (uint32_t) YK_HB_STAGES * gridDim.x;
            if (tn < ntiles) {
                asm volatile ("fence.proxy.async.shared::cta;" ::: "memory");
                yk_hb_issue(L, tn, tile, &bar[k]);
            }
        }
    }
    if (failed && threadIdx.x == 0) {
        atomicAdd(&yk_hb_failures, 1u);
        for (int j = 0; j < YK_HB_STAGES; j++)
            (void) yk_hb_wait(&bar[j], (phase >> j) & 1);
    }
}

/* the bulk-staged unpack of a contiguous-block hindexed request: -1 when it does not
 * apply (not an unpack, packed pointer off 16 bytes, above YK_POS32_END bytes), else a
 * cudaError_t */
extern "C" int yk_cuda_launch_hidx_bulk(const yk_launch * l, void *stream, int ctas_per_sm)
{
    if (l->typed_op || !l->hidx || l->dir != 1 || ((uintptr_t) l->packed & 15) ||
        l->nbytes == 0 || l->nbytes > YK_POS32_END)
        return -1;
    yk_tma_count_launch();
    const uint64_t ntiles = (l->nbytes + YK_HB_TILE - 1) / YK_HB_TILE;
    const uint64_t cap = (uint64_t) yk_cuda_num_sms() * (uint64_t) (ctas_per_sm > 0 ? ctas_per_sm : 4);
    const unsigned g = (unsigned) (ntiles < cap ? ntiles : cap);
    const size_t smem = (size_t) YK_HB_STAGES * YK_HB_TILE;
    cudaStream_t s = (cudaStream_t) stream;
    switch (l->vec) {
        case 16: yk_hidx_unpack_bulk_kernel<16><<<g, YK_THREADS, smem, s>>>(*l); break;
        case 8: yk_hidx_unpack_bulk_kernel<8><<<g, YK_THREADS, smem, s>>>(*l); break;
        case 4: yk_hidx_unpack_bulk_kernel<4><<<g, YK_THREADS, smem, s>>>(*l); break;
        case 2: yk_hidx_unpack_bulk_kernel<2><<<g, YK_THREADS, smem, s>>>(*l); break;
        default: yk_hidx_unpack_bulk_kernel<1><<<g, YK_THREADS, smem, s>>>(*l); break;
    }
    return (int) cudaGetLastError();
}

extern "C" int yaksa_gb300_debug_bulk_failures(unsigned int *n)
{
    return cudaMemcpyFromSymbol(n, yk_hb_failures, sizeof(unsigned int)) == cudaSuccess ? 0 : 2;
}


/* Pack of whole elements whose one run (16 < R <= 48 bytes, not a multiple of 16)
 * starts on 16 bytes in every element (extent a multiple of 16): one element per
 * thread, read with ceil(R/16) 16-byte loads and written as R/G pieces of G bytes (the
 * packed side of element i sits at i*R, on G bytes only).  A 16-byte load may cover
 * bytes past the run, but never past the 16-byte block that holds the run's last byte,
 * so it stays inside the caller's page.  Five 4-byte loads per element become two for a
 * 20-byte struct run. */
template <int G>
__global__ void __launch_bounds__(YK_THREADS, 8)
yk_runs_pack_kernel(const __grid_constant__ yk_launch L, uint32_t R)
{
    typedef typename yk_vec<G>::T GT;
    const yk_level & l0 = L.desc.lv[0];
    const int64_t E = l0.stride;
    const uint32_t nel = (uint32_t) (L.nbytes / R), e0 = (uint32_t) (L.p0 / R);
    const char *tb = L.typed + L.desc.base;
    const uint32_t nv = (R + 15) / 16, np = R / G;
    for (uint32_t i = blockIdx.x * YK_THREADS + threadIdx.x; i < nel; i += gridDim.x * YK_THREADS) {
        const char *src = tb + (int64_t) (e0 + i) * E;
        union {
            uint4 w[3];
            GT g[48 / G];
        } v;
#pragma unroll
        for (int k = 0; k < 3; k++)
            if ((uint32_t) k < nv)
                v.w[k] = yk_ldcg((const uint4 *) (src + 16 * k));
        char *dst = L.packed + (uint64_t) i * R;
#pragma unroll
        for (int j = 0; j < 48 / G; j++)
            if ((uint32_t) j < np)
                *(GT *) (dst + j * G) = v.g[j];
    }
}

/* yk_runs_pack_groups over the whole request, each warp with its own stage */
template <int NV>
__global__ void __launch_bounds__(YK_THREADS, 8)
yk_runs_pack_warp_kernel(const __grid_constant__ yk_launch L, uint32_t R)
{
    __shared__ __align__(16) unsigned char stage[YK_THREADS / 32][32 * 48];
    yk_runs_pack_groups<NV>(L, R, stage[threadIdx.x >> 5], ((blockIdx.x * YK_THREADS + threadIdx.x) >> 5) * 32,
                            (uint32_t) (L.nbytes / R), ((gridDim.x * YK_THREADS) >> 5) * 32);
}

extern "C" int yk_cuda_launch_runs_pack(const yk_launch * l, uint32_t run, void *stream);

template <typename IDX, int V, int DIR, int U>
__global__ void __launch_bounds__(YK_THREADS)
yk_bytes_kernel(const __grid_constant__ yk_launch L)
{
    const IDX nunits = (IDX) (L.nbytes / V);
    const IDX tile = (IDX) YK_THREADS * U;
    for (IDX t0 = (IDX) blockIdx.x * tile; t0 < nunits; t0 += (IDX) gridDim.x * tile)
        yk_bytes_tile<IDX, V, DIR, U>(L, t0, nunits);
}

/* Many REPLACE requests in one launch (yaksa_gb300_batch*): the requests' tiles are
 * numbered consecutively and every CTA takes tiles grid-stride, so all requests'
 * memory traffic is in flight together and the launch cost is paid once. */
template <int U>
__global__ void __launch_bounds__(YK_THREADS)
yk_batch_kernel(const __grid_constant__ yk_batch B)
{
    const uint64_t ntiles = B.tile_start[B.n];
    for (uint64_t g0 = blockIdx.x; g0 < ntiles; g0 += gridDim.x) {
        const uint64_t g = B.tile_mul > 1 ? (g0 * B.tile_mul) % ntiles : g0;
        int r = 0;
        while (g >= B.tile_start[r + 1])
            r++;
        const yk_launch & L = B.req[r];
        const uint32_t nunits = (uint32_t) (L.nbytes / (uint64_t) L.vec);
        const uint32_t t0 = (uint32_t) (g - B.tile_start[r]) * (uint32_t) (YK_THREADS * U);
#define YK_BT(V) do { if (L.dir == 0) yk_bytes_tile<uint32_t, V, 0, U>(L, t0, nunits); \
                      else yk_bytes_tile<uint32_t, V, 1, U>(L, t0, nunits); } while (0)
        switch (L.vec) {
            case 16: YK_BT(16); break;
            case 8: YK_BT(8); break;
            case 4: YK_BT(4); break;
            case 2: YK_BT(2); break;
            default: YK_BT(1); break;
        }
#undef YK_BT
    }
}


/* Operators: one work unit = `vec` bytes (the gcd of the element sizes); the unit
 * that starts an element applies op to that whole element. */
template <typename IDX, int DIR, bool LD>
__global__ void __launch_bounds__(YK_THREADS)
yk_typed_kernel(const __grid_constant__ yk_launch L)
{
    const IDX g = (IDX) L.vec;
    const IDX nunits = (IDX) (L.nbytes / L.vec);
    const int op = (int) L.op;
    for (IDX u = (IDX) blockIdx.x * YK_THREADS + threadIdx.x; u < nunits;
         u += (IDX) gridDim.x * YK_THREADS) {
        int bt;
        uint64_t inseg;
        int64_t off = yk_locate<IDX>(L.desc, (IDX) L.p0 + u * g, &bt, &inseg);
        int es = yk_bt_size(bt);
        if (inseg % (uint64_t) es)
            continue;
        char *t = L.typed + off;
        char *p = L.packed + (uint64_t) u * (uint64_t) g;
        if (DIR == 0)
            yk_apply<LD>(bt, op, p, t);
        else
            yk_apply<LD>(bt, op, t, p);
    }
}

/* ------------------------------------------------------------------------- */
/* ordered unpack for overlapping targets                                    */
/* ------------------------------------------------------------------------- */

/* Sorted blocks, typed: the same ownership rule as yk_owner_kernel below, with U
 * elements per thread and every index and data load issued before the ordered
 * combine, so the block-offset and target reads of neighbouring elements overlap
 * instead of forming one dependent chain per element.  Requires elements aligned to
 * their size on both sides (checked on the host). */
template <typename IDX, int BT, int U>
__global__ void __launch_bounds__(YK_THREADS)
yk_owner_typed_kernel(const __grid_constant__ yk_launch L)
{
    typedef typename yk_elem<BT>::T T;
    const yk_level & lv = L.desc.lv[0];
    const IDX es = (IDX) sizeof(T);
    const IDX R = (IDX) lv.cps;
    const IDX p0 = (IDX) L.p0, p1 = (IDX) (L.p0 + L.nbytes);
    const IDX nunits = (IDX) (L.nbytes / sizeof(T));
    const IDX nblk = (IDX) lv.count;
    const int op = (int) L.op;
    const T *packed = (const T *) L.packed;
    char *typed = L.typed + L.desc.base;
    for (IDX t0 = (IDX) blockIdx.x * (YK_THREADS * U); t0 < nunits;
         t0 += (IDX) gridDim.x * (YK_THREADS * U)) {
        int64_t x[U], dnext[U];
        IDX b[U];
        bool own[U];
        T in[U], out[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            own[k] = u < nunits;
            if (!own[k])
                continue;
            IDX p = p0 + u * es;
            b[k] = yk_div(p, lv);
            IDX j = p - b[k] * R;
            int64_t db = __ldg(lv.disp + b[k]);
            int64_t dprev = b[k] > 0 ? __ldg(lv.disp + b[k] - 1) : 0;
            dnext[k] = b[k] + 1 < nblk ? __ldg(lv.disp + b[k] + 1) : INT64_MAX;
            x[k] = db + (int64_t) j;
            if (b[k] > 0 && x[k] < dprev + (int64_t) R && (b[k] - 1) * R + (IDX) (x[k] - dprev) >= p0)
                own[k] = false;         /* an earlier in-range block owns this element */
        }
#pragma unroll
        for (int k = 0; k < U; k++)
            if (own[k]) {
                out[k] = *(const T *) (typed + x[k]);
                in[k] = packed[t0 + (IDX) (k * YK_THREADS + threadIdx.x)];
            }
#pragma unroll
        for (int k = 0; k < U; k++) {
            if (!own[k])
                continue;
            yk_elem<BT>::op(op, in[k], out[k]);
            IDX bb = b[k] + 1;
            int64_t d = dnext[k];
            while (bb < nblk && d <= x[k]) {
                IDX pp = bb * R + (IDX) (x[k] - d);
                if (pp >= p1)
                    break;
                yk_elem<BT>::op(op, packed[(pp - p0) / es], out[k]);
                bb++;
                d = bb < nblk ? __ldg(lv.disp + bb) : INT64_MAX;
            }
            *(T *) (typed + x[k]) = out[k];
        }
    }
}

/* yk_owner_lane_units over the whole request, grid-stride */
template <int BT, int OP, bool D32>
__global__ void __launch_bounds__(YK_THREADS)
yk_owner_lane_kernel(const __grid_constant__ yk_launch L, int rshift)
{
    yk_owner_lane_units<BT, OP, D32>(L, rshift, blockIdx.x * YK_THREADS + threadIdx.x,
                                     (uint32_t) (L.nbytes / sizeof(typename yk_elem<BT>::T)),
                                     gridDim.x * YK_THREADS);
}

/* yk_owner_chunk_units over the whole request, grid-stride.  Complex float is
 * bounded to the 32 registers of full occupancy, with a 32-byte spill in the D32 form:
 * at 40 registers (6 CTAs per SM) the complex PROD config took 180.2 us, at 32 (8 per
 * SM) 170.0 us. */
template <int BT, int OP, int CW, bool D32>
__global__ void __launch_bounds__(YK_THREADS, (BT == YK_BT_C32 ? 7 : 1))
yk_owner_chunk_kernel(const __grid_constant__ yk_launch L, int rshift)
{
    yk_owner_chunk_units<BT, OP, CW, D32>(L, rshift, blockIdx.x * YK_THREADS + threadIdx.x,
                                          (uint32_t) (L.nbytes / CW), gridDim.x * YK_THREADS);
}


/* yk_red_units over the whole request, grid-stride */
template <int BT, int OP, int K, bool D32, bool P2X>
__global__ void __launch_bounds__(YK_THREADS)
yk_red_kernel(const __grid_constant__ yk_launch L)
{
    yk_red_units<BT, OP, K, D32, 4, P2X>(L, blockIdx.x * YK_THREADS + threadIdx.x,
                                 (uint32_t) (L.nbytes / sizeof(typename yk_elem<BT>::T)),
                                 gridDim.x * YK_THREADS);
}

/* Sorted blocks: descriptor = IDX(nblk, disp sorted ascending, cps = R) over a run of
 * R bytes of one base type.  Every target element that receives data gets exactly one
 * owner: the thread of its first in-range contributor, which applies the
 * contributions of all later blocks in block order (the reference's seq order,
 * src/backend/seq/genpup.py:119-211). */
template <typename IDX, bool LD>
__global__ void __launch_bounds__(YK_THREADS)
yk_owner_kernel(const __grid_constant__ yk_launch L)
{
    const yk_level & lv = L.desc.lv[0];
    const int bt = L.desc.leaf_type;
    const IDX es = (IDX) yk_bt_size(bt);
    const IDX R = (IDX) lv.cps;
    const IDX p0 = (IDX) L.p0, p1 = (IDX) (L.p0 + L.nbytes);
    const IDX nunits = (IDX) (L.nbytes / es);
    const int op = (int) L.op;
    for (IDX u = (IDX) blockIdx.x * YK_THREADS + threadIdx.x; u < nunits;
         u += (IDX) gridDim.x * YK_THREADS) {
        IDX p = p0 + u * es;
        IDX b = yk_div(p, lv);
        IDX j = p - b * R;
        int64_t x = __ldg(lv.disp + b) + (int64_t) j;
        if (b > 0) {
            int64_t dprev = __ldg(lv.disp + b - 1);
            if (x < dprev + (int64_t) R && (b - 1) * R + (IDX) (x - dprev) >= p0)
                continue;       /* an earlier in-range block owns this element */
        }
        char *t = L.typed + L.desc.base + x;
        for (IDX bb = b; bb < (IDX) lv.count; bb++) {
            int64_t db = __ldg(lv.disp + bb);
            if (db > x)
                break;
            IDX pp = bb * R + (IDX) (x - db);
            if (pp >= p1)
                break;
            yk_apply<LD>(bt, op, t, L.packed + (pp - p0));
        }
    }
}

/* General ordered fallback: one warp walks the packed range in order, 32 units at a
 * time; a chunk whose target ranges intersect runs lane by lane. */
template <typename IDX, bool LD>
__global__ void yk_ordered_warp_kernel(const __grid_constant__ yk_launch L)
{
    const int lane = threadIdx.x;
    const IDX g = (IDX) L.vec;
    const IDX nunits = (IDX) (L.nbytes / L.vec);
    for (IDX c0 = 0; c0 < nunits; c0 += 32) {
        IDX u = c0 + (IDX) lane;
        bool active = u < nunits;
        int bt = YK_BT_NONE;
        uint64_t inseg = 0;
        int64_t off = 0;
        int len = 0;
        if (active) {
            off = yk_locate<IDX>(L.desc, (IDX) L.p0 + u * g, &bt, &inseg);
            if (L.typed_op) {
                int es = yk_bt_size(bt);
                if (inseg % (uint64_t) es)
                    active = false;
                else
                    len = es;
            } else {
                len = (int) g;
            }
        }
        bool conflict = false;
        for (int k = 0; k < 31; k++) {
            int64_t ooff = __shfl_sync(0xffffffffu, off, k);
            int olen = __shfl_sync(0xffffffffu, active ? len : 0, k);
            if (k < lane && active && olen && off < ooff + olen && ooff < off + len)
                conflict = true;
        }
        bool serial = __any_sync(0xffffffffu, conflict);
        for (int k = 0; k < 32; k++) {
            if ((!serial || k == lane) && active) {
                char *t = L.typed + off;
                char *p = L.packed + (uint64_t) u * (uint64_t) g;
                if (L.typed_op) {
                    yk_apply<LD>(bt, (int) L.op, t, p);
                } else {
                    for (int i = 0; i < len; i++)
                        t[i] = p[i];
                }
            }
            __syncwarp();
            if (!serial)
                break;
        }
    }
}


/* ------------------------------------------------------------------------- */
/* host-side launchers                                                       */
/* ------------------------------------------------------------------------- */

static int yk_sms = 0;

extern "C" int yk_cuda_num_sms(void)
{
    if (!yk_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&yk_sms, cudaDevAttrMultiProcessorCount, dev);
        if (yk_sms <= 0)
            yk_sms = 1;
    }
    return yk_sms;
}

static unsigned yk_grid(uint64_t units, uint64_t per_block, int blocks_per_sm)
{
    uint64_t need = (units + per_block - 1) / per_block;
    uint64_t cap = (uint64_t) yk_cuda_num_sms() * (uint64_t) blocks_per_sm;
    if (need > cap)
        need = cap;
    return (unsigned) (need ? need : 1);
}

/* Units per thread: a launch that fits in the GPU's resident threads a few times over
 * keeps one unit per thread (most requests in flight at once); larger launches take
 * four per thread in a grid-stride loop. */
extern "C" int yk_cuda_batch_units_per_thread(uint64_t total_units)
{
    return total_units <= (uint64_t) yk_cuda_num_sms() * 2048u * 4u ? 1 : YK_UNROLL;
}

extern "C" uint64_t yk_cuda_tiles(uint64_t units, int units_per_thread)
{
    uint64_t per = (uint64_t) YK_THREADS * (uint64_t) units_per_thread;
    return (units + per - 1) / per;
}

template <typename IDX, int U>
static void launch_bytes_u(const yk_launch * l, cudaStream_t s, uint64_t units, int cap)
{
    unsigned g = yk_grid(units, (uint64_t) YK_THREADS * U, cap ? cap : (U == 1 ? 64 : 8));
#define YK_B(V) do { if (l->dir == 0) yk_bytes_kernel<IDX, V, 0, U><<<g, YK_THREADS, 0, s>>>(*l); \
                     else yk_bytes_kernel<IDX, V, 1, U><<<g, YK_THREADS, 0, s>>>(*l); } while (0)
    switch (l->vec) {
        case 16: YK_B(16); break;
        case 8: YK_B(8); break;
        case 4: YK_B(4); break;
        case 2: YK_B(2); break;
        default: YK_B(1); break;
    }
#undef YK_B
}

template <int U>
static void launch_regular_u(const yk_launch * l, cudaStream_t s, uint64_t units, int cap)
{
    unsigned g = yk_grid(units, (uint64_t) YK_THREADS * U, cap ? cap : (U == 1 ? 64 : 8));
#define YK_R(V) do { if (l->dir == 0) yk_regular_kernel<V, 0, U><<<g, YK_THREADS, 0, s>>>(*l); \
                     else yk_regular_kernel<V, 1, U><<<g, YK_THREADS, 0, s>>>(*l); } while (0)
    switch (l->vec) {
        case 16: YK_R(16); break;
        case 8: YK_R(8); break;
        case 4: YK_R(4); break;
        case 2: YK_R(2); break;
        default: YK_R(1); break;
    }
#undef YK_R
}

/* u: units per thread (1 or YK_UNROLL; 0 = by size); cap: CTAs per SM (0 = by u) */
template <typename IDX>
static void launch_bytes(const yk_launch * l, cudaStream_t s, int u, int cap)
{
    uint64_t units = l->nbytes / (uint64_t) l->vec;
    if (u != 1 && u != YK_UNROLL)
        u = yk_cuda_batch_units_per_thread(units);
    if (l->regular >= 0 && sizeof(IDX) == 4) {
        if (u == 1)
            launch_regular_u<1>(l, s, units, cap);
        else
            launch_regular_u<YK_UNROLL>(l, s, units, cap);
    } else if (u == 1) {
        launch_bytes_u<IDX, 1>(l, s, units, cap);
    } else {
        launch_bytes_u<IDX, YK_UNROLL>(l, s, units, cap);
    }
}

extern "C" int yk_cuda_launch_batch(const yk_batch * b, int units_per_thread, int regular,
                                    int ctas_per_sm, void *stream)
{
    cudaStream_t s = (cudaStream_t) stream;
    uint64_t tiles = b->tile_start[b->n];
    if (!tiles)
        return 0;
    uint64_t cap = (uint64_t) yk_cuda_num_sms() *
        (ctas_per_sm > 0 ? (unsigned) ctas_per_sm : (units_per_thread == 1 ? 64u : 8u));
    unsigned g = (unsigned) (tiles < cap ? tiles : cap);
    if (regular) {
        /* one unit per thread: the 40 inlined (vector width, direction, depth) variants
         * fit in 32 registers only at this size, and full occupancy keeps enough loads
         * in flight; large batches loop grid-stride */
        yk_batch_regular_kernel<1><<<g, YK_THREADS, 0, s>>>(*b);
    } else if (units_per_thread == 1) {
        yk_batch_kernel<1><<<g, YK_THREADS, 0, s>>>(*b);
    } else {
        yk_batch_kernel<YK_UNROLL><<<g, YK_THREADS, 0, s>>>(*b);
    }
    return (int) cudaGetLastError();
}

/* the grid of a contiguous-block hindexed launch: one warp per group of 32 blocks, at
 * most `cap` CTAs per SM (the grid loops over the groups) */
static unsigned yk_hidx_grid(const yk_launch * l, int cap)
{
    const uint64_t groups = (l->desc.lv[0].count + 31) / 32;
    const uint64_t ctas = (groups + (YK_THREADS / 32) - 1) / (YK_THREADS / 32);
    const uint64_t most = (uint64_t) yk_cuda_num_sms() * (uint64_t) cap;
    return (unsigned) (ctas < most ? (ctas ? ctas : 1) : most);
}

/* ctas_per_sm 0: as many CTAs as stay resident (MINB per SM), one wave */
template <int V, int DIR, int U, int MINB, bool PF>
static void yk_launch_hidx32(const yk_launch * l, cudaStream_t s, int ctas_per_sm)
{
    const unsigned g = yk_hidx_grid(l, ctas_per_sm > 0 ? ctas_per_sm : MINB);
    yk_hidx32_kernel<V, DIR, U, MINB, PF><<<g, YK_THREADS, 0, s>>>(*l);
}

/* The 32-bit kernel's shapes for 4- and 8-byte units, by `units`: 0 (the default)
 * eight units per lane at 4 resident CTAs per SM, 4 four at 6, 2 two at 8, 16 (unpacks)
 * sixteen at 3.  Measured on the hindexed config (1 GiB, 2^20 int32 blocks, cold L2):
 * pack 72-74 us with eight units, 80 with four, 103 with two; unpack 107, 109-117 and
 * 126 us -- the kernel is bound by the DRAM accesses of the blocks' random typed lines
 * (and for unpacks the read-modify-write of the partial sectors at every block's two
 * ends), not by its loads in flight.  Other unit sizes take four at 6. */
template <int V, int DIR>
static void yk_launch_hidx32_shape(const yk_launch * l, cudaStream_t s, int units, int ctas_per_sm)
{
    if constexpr (V == 4 || V == 8) {
        switch (units) {
            case 2: return yk_launch_hidx32<V, DIR, 2, 8, true>(l, s, ctas_per_sm);
            case 4: return yk_launch_hidx32<V, DIR, 4, 6, true>(l, s, ctas_per_sm);
            case 16:
                if constexpr (DIR == 1)
                    return yk_launch_hidx32<V, DIR, 16, 3, true>(l, s, ctas_per_sm);
                break;
        }
        yk_launch_hidx32<V, DIR, 8, 4, true>(l, s, ctas_per_sm);
    } else {
        yk_launch_hidx32<V, DIR, YK_HW_UNROLL, 6, false>(l, s, ctas_per_sm);
    }
}

/* Contiguous-block hindexed: the 64-bit kernel past 4 GiB of packed bytes, else the
 * 32-bit one in the shape `units` names. */
template <int V>
static void yk_launch_hidx(const yk_launch * l, cudaStream_t s, int units, int ctas_per_sm)
{
    if (l->nbytes > YK_POS32_END) {
        const unsigned g = yk_hidx_grid(l, ctas_per_sm > 0 ? ctas_per_sm : 8);
        if (l->dir == 0)
            yk_hidx_kernel<V, 0><<<g, YK_THREADS, 0, s>>>(*l);
        else
            yk_hidx_kernel<V, 1><<<g, YK_THREADS, 0, s>>>(*l);
        return;
    }
    if (l->dir == 0)
        yk_launch_hidx32_shape<V, 0>(l, s, units, ctas_per_sm);
    else
        yk_launch_hidx32_shape<V, 1>(l, s, units, ctas_per_sm);
}

/* a long double operator other than REPLACE: the binary128 kernel instances */
static bool yk_ld_ops(const yk_launch & c)
{
    return c.ldouble && c.typed_op && c.op != OP_REPLACE;
}

extern "C" int yk_cuda_launch_pup(const yk_launch * l, void *stream)
{
    return yk_cuda_launch_pup_cfg(l, stream, 0, 0);
}

extern "C" int yk_cuda_launch_pup_cfg(const yk_launch * l, void *stream, int units_per_thread,
                                      int ctas_per_sm)
{
    cudaStream_t s = (cudaStream_t) stream;
    if (l->nbytes == 0)
        return 0;
    if (!l->typed_op && l->hidx) {
        switch (l->vec) {
            case 16: yk_launch_hidx<16>(l, s, units_per_thread, ctas_per_sm); break;
            case 8: yk_launch_hidx<8>(l, s, units_per_thread, ctas_per_sm); break;
            case 4: yk_launch_hidx<4>(l, s, units_per_thread, ctas_per_sm); break;
            case 2: yk_launch_hidx<2>(l, s, units_per_thread, ctas_per_sm); break;
            default: yk_launch_hidx<1>(l, s, units_per_thread, ctas_per_sm); break;
        }
    } else if (!l->typed_op) {
        if (l->use64)
            launch_bytes<uint64_t>(l, s, units_per_thread, ctas_per_sm);
        else
            launch_bytes<uint32_t>(l, s, units_per_thread, ctas_per_sm);
    } else {
        const yk_launch & c = *l;
        uint64_t units = c.nbytes / (uint64_t) c.vec;
        unsigned g = yk_grid(units, YK_THREADS, ctas_per_sm > 0 ? ctas_per_sm : 16);
#define YK_TK(IDX, LD) do { if (c.dir == 0) yk_typed_kernel<IDX, 0, LD><<<g, YK_THREADS, 0, s>>>(c); \
                            else yk_typed_kernel<IDX, 1, LD><<<g, YK_THREADS, 0, s>>>(c); } while (0)
        if (yk_ld_ops(c)) {
            if (c.use64)
                YK_TK(uint64_t, true);
            else
                YK_TK(uint32_t, true);
        } else if (c.use64) {
            YK_TK(uint64_t, false);
        } else {
            YK_TK(uint32_t, false);
        }
#undef YK_TK
    }
    return (int) cudaGetLastError();
}

/* the 8-byte chunk form exists for elements under 8 bytes, the 16-byte form for 4- and
 * 8-byte elements other than double; chunk = bytes per lane (0: the per-lane kernel) */
template <int BT, int O>
static bool yk_owner_chunk_launch(const yk_launch & c, int rshift, cudaStream_t s, unsigned g,
                                  int chunk, bool d32)
{
    if constexpr (sizeof(typename yk_elem<BT>::T) == 4 ||
                  (sizeof(typename yk_elem<BT>::T) == 8 && BT != YK_BT_F64)) {
        if (chunk == 16) {
            if (d32)
                yk_owner_chunk_kernel<BT, O, 16, true><<<g, YK_THREADS, 0, s>>>(c, rshift);
            else
                yk_owner_chunk_kernel<BT, O, 16, false><<<g, YK_THREADS, 0, s>>>(c, rshift);
            return true;
        }
    }
    if constexpr (sizeof(typename yk_elem<BT>::T) < 8) {
        if (chunk == 8) {
            yk_owner_chunk_kernel<BT, O, 8, false><<<g, YK_THREADS, 0, s>>>(c, rshift);
            return true;
        }
    }
    return false;
}


/* yk_owner_lane_kernel for (base type, operator) pairs in the operator table; false
 * when the pair has no instance (the caller falls back to the runtime-op kernels) */
template <int BT>
static bool yk_owner_lane_int(const yk_launch & c, int rshift, cudaStream_t s, unsigned g, int chunk,
                              bool d32)
{
    switch ((int) c.op) {
#define YK_OL(O) case O: if (!yk_owner_chunk_launch<BT, O>(c, rshift, s, g, chunk, d32)) {    \
                             if (d32)                                                          \
                                 yk_owner_lane_kernel<BT, O, true><<<g, YK_THREADS, 0, s>>>(c, rshift); \
                             else                                                              \
                                 yk_owner_lane_kernel<BT, O, false><<<g, YK_THREADS, 0, s>>>(c, rshift); \
                         }                                                                     \
                         return true
        YK_OL(OP_MAX); YK_OL(OP_MIN); YK_OL(OP_SUM); YK_OL(OP_PROD); YK_OL(OP_LAND); YK_OL(OP_BAND);
        YK_OL(OP_LOR); YK_OL(OP_BOR); YK_OL(OP_LXOR); YK_OL(OP_BXOR); YK_OL(OP_REPLACE);
    }
    return false;
}

template <int BT>
static bool yk_owner_lane_flt(const yk_launch & c, int rshift, cudaStream_t s, unsigned g, int chunk,
                              bool d32)
{
    switch ((int) c.op) {
        YK_OL(OP_MAX); YK_OL(OP_MIN); YK_OL(OP_SUM); YK_OL(OP_PROD); YK_OL(OP_REPLACE);
    }
    return false;
}

template <int BT>
static bool yk_owner_lane_cplx(const yk_launch & c, int rshift, cudaStream_t s, unsigned g, int chunk,
                              bool d32)
{
    switch ((int) c.op) {
        YK_OL(OP_SUM); YK_OL(OP_PROD); YK_OL(OP_REPLACE);
#undef YK_OL
    }
    return false;
}

/* which of yk_owner_lane_kernel / yk_owner_chunk_kernel serves a launch, and how (the
 * YK_FORM_* fields of yk_desc.h); the server plans its sorted-block items with it too */
extern "C" int yk_cuda_owner_form(const yk_launch * l, int sorted_blocks)
{
    const yk_launch & c = *l;
    const int bt = c.desc.leaf_type;
    if ((sorted_blocks & 3) != 2 || c.use64 ||
        !(bt == YK_BT_I8 || bt == YK_BT_I16 || bt == YK_BT_I32 || bt == YK_BT_I64 ||
          bt == YK_BT_F32 || bt == YK_BT_F64 || bt == YK_BT_C32 || bt == YK_BT_C64))
        return 0;
    const uint64_t R = c.desc.lv[0].cps;
    int rshift = 0;
    while (rshift < 31 && (1ull << rshift) < R)
        rshift++;
    if ((1ull << rshift) != R)
        return 0;
    const uint64_t es = (uint64_t) yk_bt_size(bt);
    /* chunks of CW bytes: blocks a multiple of CW bytes, range and packed pointer on CW
     * bytes.  16-byte chunks for 4- and 8-byte elements (within the register budget of
     * full occupancy), else 8-byte chunks for elements under 8 bytes.  double keeps one
     * element per lane: its arithmetic runs on the FP64 pipe, a small share of the SM's
     * issue rate on GB300, and measured slower with its two operations per lane
     * back to back (double SUM, 2^25 elements: 213 us per lane, 234 us chunked) */
    int chunk = 0;
    if (es <= 8 && bt != YK_BT_F64) {
        const int first = es >= 4 ? 16 : 8, last = es < 8 ? 8 : 16;
        for (int cw = first; cw >= last && !chunk; cw /= 2)
            if (rshift >= (cw == 16 ? 4 : 3) && c.p0 % cw == 0 && c.nbytes % cw == 0 &&
                (uintptr_t) c.packed % cw == 0)
                chunk = cw;
    }
    const bool d32 = (sorted_blocks & YK_ORD_D32) != 0 && (c.desc.lv[0].has_d32 & YK_D32_TABLE);
    return rshift | (chunk << 8) | (d32 ? YK_FORM_D32 : 0) | YK_FORM_POW2;
}

/* the kernel of a form from yk_cuda_owner_form; false when the (type, operator) pair has
 * no instance */
static bool yk_owner_lane_launch(const yk_launch & c, int bt, int form, cudaStream_t s, int cap)
{
    const uint64_t es = (uint64_t) yk_bt_size(bt);
    const int rshift = form & 255, chunk = (form >> 8) & 255;
    const bool d32 = (form & YK_FORM_D32) != 0;
    const uint64_t units = c.nbytes / (chunk ? (uint64_t) chunk : es);
    const unsigned g = yk_grid(units, YK_THREADS, cap > 0 ? cap : 16);
    switch (bt) {
        case YK_BT_I8: return yk_owner_lane_int<YK_BT_I8>(c, rshift, s, g, chunk, d32);
        case YK_BT_I16: return yk_owner_lane_int<YK_BT_I16>(c, rshift, s, g, chunk, d32);
        case YK_BT_I32: return yk_owner_lane_int<YK_BT_I32>(c, rshift, s, g, chunk, d32);
        case YK_BT_I64: return yk_owner_lane_int<YK_BT_I64>(c, rshift, s, g, chunk, d32);
        case YK_BT_F32: return yk_owner_lane_flt<YK_BT_F32>(c, rshift, s, g, chunk, d32);
        case YK_BT_F64: return yk_owner_lane_flt<YK_BT_F64>(c, rshift, s, g, chunk, d32);
        case YK_BT_C32: return yk_owner_lane_cplx<YK_BT_C32>(c, rshift, s, g, chunk, d32);
        case YK_BT_C64: return yk_owner_lane_cplx<YK_BT_C64>(c, rshift, s, g, 0, d32);
    }
    return false;
}

extern "C" int yk_cuda_launch_runs_pack(const yk_launch * l, uint32_t run, void *stream)
{
    const uint64_t nel = l->nbytes / run;
    const unsigned g = yk_grid(nel, YK_THREADS, 8);
    cudaStream_t s = (cudaStream_t) stream;
    /* read once; the initialisation of a function-local static is thread-safe */
    static const bool warp_form = [] {
        const char *e = getenv("YAKSA_GB300_RUNS_WARP");
        return !(e && e[0] == '0');
    }();
    if (warp_form && (uintptr_t) l->packed % 16 == 0 && run % 4 == 0 && run <= 32)
        yk_runs_pack_warp_kernel<2><<<g, YK_THREADS, 0, s>>>(*l, run);
    else if (warp_form && (uintptr_t) l->packed % 16 == 0 && run % 4 == 0 && run <= 48)
        yk_runs_pack_warp_kernel<3><<<g, YK_THREADS, 0, s>>>(*l, run);
    else if (l->vec == 8)
        yk_runs_pack_kernel<8><<<g, YK_THREADS, 0, s>>>(*l, run);
    else
        yk_runs_pack_kernel<4><<<g, YK_THREADS, 0, s>>>(*l, run);
    return (int) cudaGetLastError();
}

/* yk_red_kernel for a 4- or 8-byte integer type and an operator that yk_red_applies()
 * accepts; false when the launch does not fit it */
template <int BT, int K, bool D32, bool P2X = false>
static bool yk_red_launch_bt(const yk_launch & c, cudaStream_t s, unsigned g)
{
    switch ((int) c.op) {
#define YK_RD(O) case O: yk_red_kernel<BT, O, K, D32, P2X><<<g, YK_THREADS, 0, s>>>(c); return true
        YK_RD(OP_MAX); YK_RD(OP_MIN); YK_RD(OP_SUM); YK_RD(OP_BAND); YK_RD(OP_BOR); YK_RD(OP_BXOR);
#undef YK_RD
    }
    return false;
}

static std::atomic<unsigned long long> yk_red_count(0);

extern "C" unsigned long long yk_cuda_red_launches(void)
{
    return yk_red_count.load(std::memory_order_relaxed);
}

static bool yk_red_launch(const yk_launch & c, int bt, cudaStream_t s, int cap)
{
    const int k = c.desc.lv[0].kind;
    if (c.use64 || c.desc.nlev != 1 || (k != YK_LV_IDX && k != YK_LV_VEC) ||
        c.desc.lv[0].cps >= (1ull << 32) || !yk_red_applies(bt, c.op))
        return false;
    const uint64_t units = c.nbytes / (uint64_t) yk_bt_size(bt);
    const unsigned g = yk_grid(units, (uint64_t) YK_THREADS * 4, cap > 0 ? cap : 8);
    /* IDX: the 32-bit copy of the displacements when the level has one; for 4-byte
     * integers also a shift and 32-bit offsets where yk_red_p2x() holds (for 8-byte ones
     * that form measured slower: int64 MAX 120.8 against 110.6 us) */
    const bool d32 = k == YK_LV_IDX && (c.desc.lv[0].has_d32 & YK_D32_TABLE);
    if (bt == YK_BT_I32)
        return k != YK_LV_IDX ? yk_red_launch_bt<YK_BT_I32, YK_LV_VEC, false>(c, s, g) :
            yk_red_p2x(c.desc.lv[0]) ? yk_red_launch_bt<YK_BT_I32, YK_LV_IDX, true, true>(c, s, g) :
            d32 ? yk_red_launch_bt<YK_BT_I32, YK_LV_IDX, true>(c, s, g) :
            yk_red_launch_bt<YK_BT_I32, YK_LV_IDX, false>(c, s, g);
    return k != YK_LV_IDX ? yk_red_launch_bt<YK_BT_I64, YK_LV_VEC, false>(c, s, g) :
        d32 ? yk_red_launch_bt<YK_BT_I64, YK_LV_IDX, true>(c, s, g) :
        yk_red_launch_bt<YK_BT_I64, YK_LV_IDX, false>(c, s, g);
}

extern "C" int yk_cuda_launch_unpack_ordered(const yk_launch * l, int sorted_blocks, void *stream,
                                             int ctas_per_sm)
{
    cudaStream_t s = (cudaStream_t) stream;
    if (l->nbytes == 0)
        return 0;
    const yk_launch & c = *l;
    int bt = c.desc.leaf_type;
    /* order-independent integer operators on aligned equal blocks: L2 reductions */
    if ((sorted_blocks & YK_ORD_RED) && yk_red_launch(c, bt, s, ctas_per_sm)) {
        yk_red_count.fetch_add(1, std::memory_order_relaxed);
        return (int) cudaGetLastError();
    }
    const int form = yk_cuda_owner_form(l, sorted_blocks);
    sorted_blocks &= 3;
    bool typed_ok = sorted_blocks == 2 && (bt == YK_BT_I8 || bt == YK_BT_I16 || bt == YK_BT_I32 ||
                                           bt == YK_BT_I64 || bt == YK_BT_F32 || bt == YK_BT_F64 ||
                                           bt == YK_BT_C32 || bt == YK_BT_C64);
    if (form && yk_owner_lane_launch(c, bt, form, s, ctas_per_sm)) {
        /* launched: power-of-two blocks, operator in the type's table */
    } else if (typed_ok) {
        uint64_t units = c.nbytes / (uint64_t) yk_bt_size(bt);
        unsigned g = yk_grid(units, YK_THREADS * 4, ctas_per_sm > 0 ? ctas_per_sm : 8);
#define YK_OT(IDX) do { switch (bt) {                                                          \
            case YK_BT_I8: yk_owner_typed_kernel<IDX, YK_BT_I8, 4><<<g, YK_THREADS, 0, s>>>(c); break;   \
            case YK_BT_I16: yk_owner_typed_kernel<IDX, YK_BT_I16, 4><<<g, YK_THREADS, 0, s>>>(c); break; \
            case YK_BT_I32: yk_owner_typed_kernel<IDX, YK_BT_I32, 4><<<g, YK_THREADS, 0, s>>>(c); break; \
            case YK_BT_I64: yk_owner_typed_kernel<IDX, YK_BT_I64, 4><<<g, YK_THREADS, 0, s>>>(c); break; \
            case YK_BT_F32: yk_owner_typed_kernel<IDX, YK_BT_F32, 4><<<g, YK_THREADS, 0, s>>>(c); break; \
            case YK_BT_F64: yk_owner_typed_kernel<IDX, YK_BT_F64, 4><<<g, YK_THREADS, 0, s>>>(c); break; \
            case YK_BT_C32: yk_owner_typed_kernel<IDX, YK_BT_C32, 4><<<g, YK_THREADS, 0, s>>>(c); break; \
            default: yk_owner_typed_kernel<IDX, YK_BT_C64, 4><<<g, YK_THREADS, 0, s>>>(c); break;       \
        } } while (0)
        if (c.use64)
            YK_OT(uint64_t);
        else
            YK_OT(uint32_t);
#undef YK_OT
    } else if (sorted_blocks) {
        uint64_t units = c.nbytes / (uint64_t) c.vec;
        unsigned g = yk_grid(units, YK_THREADS, ctas_per_sm > 0 ? ctas_per_sm : 16);
        if (yk_ld_ops(c)) {
            if (c.use64)
                yk_owner_kernel<uint64_t, true><<<g, YK_THREADS, 0, s>>>(c);
            else
                yk_owner_kernel<uint32_t, true><<<g, YK_THREADS, 0, s>>>(c);
        } else if (c.use64) {
            yk_owner_kernel<uint64_t, false><<<g, YK_THREADS, 0, s>>>(c);
        } else {
            yk_owner_kernel<uint32_t, false><<<g, YK_THREADS, 0, s>>>(c);
        }
    } else {
        if (yk_ld_ops(c)) {
            if (c.use64)
                yk_ordered_warp_kernel<uint64_t, true><<<1, 32, 0, s>>>(c);
            else
                yk_ordered_warp_kernel<uint32_t, true><<<1, 32, 0, s>>>(c);
        } else if (c.use64) {
            yk_ordered_warp_kernel<uint64_t, false><<<1, 32, 0, s>>>(c);
        } else {
            yk_ordered_warp_kernel<uint32_t, false><<<1, 32, 0, s>>>(c);
        }
    }
    return (int) cudaGetLastError();
}
