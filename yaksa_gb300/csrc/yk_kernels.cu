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
#include <atomic>
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>
#include "yk_desc.h"
#include "yk_locate.h"
#include "yk_quad.h"

#define YK_THREADS 256
#define YK_UNROLL 4

extern "C" int yk_cuda_num_sms(void);
extern "C" void yk_tma_count_launch(void);

/* address decomposition shared with the host (yk_locate.h) */
/* ------------------------------------------------------------------------- */

__device__ __forceinline__ uint32_t yk_div(uint32_t n, const yk_level & l) { return yk_div32(n, &l); }
__device__ __forceinline__ uint64_t yk_div(uint64_t n, const yk_level & l) { return yk_div64(n, &l); }

template <typename IDX>
__device__ __forceinline__ int64_t yk_locate(const yk_desc & d, IDX p, int *bt, uint64_t * inseg);
template <>
__device__ __forceinline__ int64_t yk_locate<uint32_t>(const yk_desc & d, uint32_t p, int *bt,
                                                       uint64_t * inseg)
{
    return yk_locate32(&d, p, bt, inseg);
}
template <>
__device__ __forceinline__ int64_t yk_locate<uint64_t>(const yk_desc & d, uint64_t p, int *bt,
                                                       uint64_t * inseg)
{
    return yk_locate64(&d, p, bt, inseg);
}

/* ------------------------------------------------------------------------- */
/* REPLACE: byte movement in V-byte units                                    */
/* ------------------------------------------------------------------------- */

template <int V> struct yk_vec;
template <> struct yk_vec<1> { typedef uint8_t T; };
template <> struct yk_vec<2> { typedef uint16_t T; };
template <> struct yk_vec<4> { typedef uint32_t T; };
template <> struct yk_vec<8> { typedef uint2 T; };
template <> struct yk_vec<16> { typedef uint4 T; };

/* Loads cached in L2 only: the strided side is read once, so it does not displace L1.
 * (An isolated 8-byte run still costs a whole 128-byte line from L2 on GB300, whatever
 * the cache operator or prefetch-size qualifier; measured for every documented form.) */
__device__ __forceinline__ uint8_t yk_ldcg(const uint8_t * p)
{
    uint16_t v;
    asm volatile ("ld.global.cg.u8 %0, [%1];" : "=h"(v) : "l"(p));
    return (uint8_t) v;
}

__device__ __forceinline__ uint16_t yk_ldcg(const uint16_t * p)
{
    uint16_t v;
    asm volatile ("ld.global.cg.u16 %0, [%1];" : "=h"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t yk_ldcg(const uint32_t * p)
{
    uint32_t v;
    asm volatile ("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint2 yk_ldcg(const uint2 * p)
{
    uint2 v;
    asm volatile ("ld.global.cg.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ uint4 yk_ldcg(const uint4 * p)
{
    uint4 v;
    asm volatile ("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                  : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}

/* One tile: units t0 + k * YK_THREADS + threadIdx.x, k < U, of a request with
 * `nunits` V-byte units.  All U addresses are computed first and all U loads issued
 * before any store, so every thread keeps U independent memory requests in flight.
 * Loads use ld.global.cg (cache in L2 only): an L1-allocating load of an isolated
 * 8-byte run fills a 128-byte line, which is 16x the useful DRAM traffic for runs
 * at a large stride. */
template <typename IDX, int V, int DIR, int U>
__device__ __forceinline__ void yk_bytes_tile(const yk_launch & L, IDX t0, IDX nunits)
{
    typedef typename yk_vec<V>::T VT;
    const IDX p0 = (IDX) L.p0;
    VT *packed = (VT *) L.packed;
    char *typed = L.typed;
    int64_t off[U];
    VT v[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
        IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
        if (u < nunits)
            off[k] = yk_locate<IDX>(L.desc, p0 + u * (IDX) V, nullptr, nullptr);
    }
    if (DIR == 0) {
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                v[k] = yk_ldcg((const VT *) (typed + off[k]));
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                packed[u] = v[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                v[k] = yk_ldcg((const VT *) (packed + u));
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            IDX u = t0 + (IDX) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                *(VT *) (typed + off[k]) = v[k];
        }
    }
}

/* Regular nests (NL strided levels over one contiguous run, 32-bit positions): the
 * decomposition unrolls at compile time into NL multiply-high/shift/multiply-add steps
 * with no table loads, which keeps the kernel near 32 registers and lets eight
 * 256-thread CTAs share an SM (full occupancy, the most loads in flight). */
/* the few fields of a regular request a tile needs, held in registers */
struct yk_rt {
    char *typed;                /* typed pointer + descriptor base */
    char *packed;
    uint32_t p0;
    uint32_t m[YK_REGULAR_MAX];
    uint32_t cps[YK_REGULAR_MAX];
    uint32_t sh1[YK_REGULAR_MAX], sh2[YK_REGULAR_MAX];
    int64_t stride[YK_REGULAR_MAX];
};

template <int NL>
__device__ __forceinline__ void yk_rt_load(yk_rt & t, const yk_launch & L)
{
    t.typed = L.typed + L.desc.base;
    t.packed = L.packed;
    t.p0 = (uint32_t) L.p0;
#pragma unroll
    for (int i = 0; i < NL; i++) {
        t.m[i] = L.desc.lv[i].m32;
        t.cps[i] = (uint32_t) L.desc.lv[i].cps;
        t.sh1[i] = L.desc.lv[i].l ? 1u : 0u;
        t.sh2[i] = L.desc.lv[i].l ? (uint32_t) L.desc.lv[i].l - 1u : 0u;
        t.stride[i] = L.desc.lv[i].stride;
    }
}

template <int V, int DIR, int U, int NL>
__device__ __forceinline__ void yk_regular_tile(const yk_launch & L, uint32_t t0, uint32_t nunits)
{
    typedef typename yk_vec<V>::T VT;
    yk_rt rt;
    yk_rt_load<NL>(rt, L);
    VT *packed = (VT *) rt.packed;
    char *typed = rt.typed;
    int64_t off[U];
    VT v[U];
#pragma unroll
    for (int k = 0; k < U; k++) {
        uint32_t u = t0 + (uint32_t) (k * YK_THREADS + threadIdx.x);
        uint32_t r = rt.p0 + u * (uint32_t) V;
        int64_t o = 0;
#pragma unroll
        for (int i = 0; i < NL; i++) {
            uint32_t t = __umulhi(rt.m[i], r);
            uint32_t q = (t + ((r - t) >> rt.sh1[i])) >> rt.sh2[i];
            r -= q * rt.cps[i];
            o += (int64_t) q * rt.stride[i];
        }
        off[k] = o + (int64_t) r;
    }
    if (DIR == 0) {
#pragma unroll
        for (int k = 0; k < U; k++)
            if (t0 + (uint32_t) (k * YK_THREADS + threadIdx.x) < nunits)
                v[k] = yk_ldcg((const VT *) (typed + off[k]));
#pragma unroll
        for (int k = 0; k < U; k++) {
            uint32_t u = t0 + (uint32_t) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                packed[u] = v[k];
        }
    } else {
#pragma unroll
        for (int k = 0; k < U; k++) {
            uint32_t u = t0 + (uint32_t) (k * YK_THREADS + threadIdx.x);
            if (u < nunits)
                v[k] = yk_ldcg((const VT *) (packed + u));
        }
#pragma unroll
        for (int k = 0; k < U; k++)
            if (t0 + (uint32_t) (k * YK_THREADS + threadIdx.x) < nunits)
                *(VT *) (typed + off[k]) = v[k];
    }
}

template <int V, int DIR, int U>
__device__ __forceinline__ void yk_regular_dispatch(const yk_launch & L, uint32_t t0,
                                                    uint32_t nunits)
{
    switch (L.regular) {
        case 0: yk_regular_tile<V, DIR, U, 0>(L, t0, nunits); break;
        case 1: yk_regular_tile<V, DIR, U, 1>(L, t0, nunits); break;
        case 2: yk_regular_tile<V, DIR, U, 2>(L, t0, nunits); break;
        default: yk_regular_tile<V, DIR, U, 3>(L, t0, nunits); break;
    }
}

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

/* The same walk for requests under 4 GiB, in packed positions relative to each group's
 * first byte: 32-bit search keys (one shuffle per step instead of two) and per-lane
 * state small enough for every warp slot of the SM to stay resident.  Lane k keeps its
 * block's start relative to the group (0 for a block that starts before the range) and
 * the typed offset of relative position 0 in that block, so a unit's typed offset is one
 * shuffle and one add.
 *
 * The kernel is latency-bound (random block starts, a few KiB per group), so each warp
 * keeps as much in flight as its registers allow: the four index words of its next
 * group are loaded while the current group is walked, and U units per lane move per
 * step.  A pack finds the units' typed offsets first and then loads them; an unpack
 * loads its contiguous packed units first (no offsets needed) and locates each unit
 * only to store it, so no offsets are live across the load.  MINB CTAs of the block
 * size are meant to stay resident; the autotuner chooses among the shapes. */
template <int V, int DIR, int U, int MINB, bool PF>
__global__ void __launch_bounds__(YK_THREADS, MINB)
yk_hidx32_kernel(const __grid_constant__ yk_launch L)
{
    typedef typename yk_vec<V>::T VT;
    const yk_level *lv = &L.desc.lv[0];
    const uint64_t p0 = L.p0, p1 = L.p0 + L.nbytes;
    const int lane = threadIdx.x & 31;
    const uint64_t warp = ((uint64_t) blockIdx.x * YK_THREADS + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t) gridDim.x * YK_THREADS) >> 5;
    char *typed = L.typed + L.desc.base;
    const uint64_t jb = yk_hidx_block(lv, p0), je = yk_hidx_block(lv, p1 - 1);
    const uint64_t ngroups = (je - jb + 32) / 32;
    /* the index words of the group a warp takes next: its first block's packed start,
     * the end of its last block, and this lane's block start and displacement */
    uint64_t f_first = 0, f_end = 0, f_bp = 0;
    int64_t f_disp = 0;
    auto fetch = [&](uint64_t gg) {
        const uint64_t j0 = jb + gg * 32, jl = j0 + (uint64_t) lane;
        const uint64_t jend = min(j0 + 32, je + 1);
        f_first = __ldg(lv->pfx + j0);
        f_end = __ldg(lv->pfx + jend);
        if (jl < jend) {
            f_bp = __ldg(lv->pfx + jl);
            f_disp = __ldg(lv->disp + jl);
        }
    };
    if (PF && warp < ngroups)
        fetch(warp);
    for (uint64_t g = warp; g < ngroups; g += nwarps) {
        const uint64_t j0 = jb + g * 32;
        const uint64_t jl = j0 + (uint64_t) lane;
        const uint64_t jend = min(j0 + 32, je + 1);
        if (!PF)
            fetch(g);
        const uint64_t gs = max(f_first, p0);
        const uint32_t n = (uint32_t) (min(f_end, p1) - gs);
        uint32_t my_rel = 0xffffffffu;
        int64_t my_adj = 0;
        if (jl < jend) {
            my_rel = f_bp <= gs ? 0u : (uint32_t) (f_bp - gs);
            my_adj = f_disp - ((int64_t) f_bp - (int64_t) gs);
        }
        if (PF && g + nwarps < ngroups)
            fetch(g + nwarps);
        VT *pk = (VT *) (L.packed + (gs - p0));
        for (uint32_t base = 0; base < n; base += 32u * V * U) {
            if (DIR == 0) {
                int64_t off[U];
#pragma unroll
                for (int k = 0; k < U; k++) {
                    const uint32_t r = base + (uint32_t) (k * 32 + lane) * V;
                    int idx = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const uint32_t c = __shfl_sync(0xffffffffu, my_rel, idx + step);
                        if (c <= r)
                            idx += step;
                    }
                    off[k] = __shfl_sync(0xffffffffu, my_adj, idx) + (int64_t) r;
                }
                VT v[U];
#pragma unroll
                for (int k = 0; k < U; k++)
                    if (base + (uint32_t) (k * 32 + lane) * V < n)
                        v[k] = yk_ldcg((const VT *) (typed + off[k]));
#pragma unroll
                for (int k = 0; k < U; k++)
                    if (base + (uint32_t) (k * 32 + lane) * V < n)
                        pk[base / V + (uint32_t) (k * 32 + lane)] = v[k];
            } else {
                VT v[U];
#pragma unroll
                for (int k = 0; k < U; k++)
                    if (base + (uint32_t) (k * 32 + lane) * V < n)
                        v[k] = yk_ldcg(pk + base / V + (uint32_t) (k * 32 + lane));
#pragma unroll
                for (int k = 0; k < U; k++) {
                    const uint32_t r = base + (uint32_t) (k * 32 + lane) * V;
                    int idx = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const uint32_t c = __shfl_sync(0xffffffffu, my_rel, idx + step);
                        if (c <= r)
                            idx += step;
                    }
                    const int64_t off = __shfl_sync(0xffffffffu, my_adj, idx) + (int64_t) r;
                    if (r < n)
                        *(VT *) (typed + off) = v[k];
                }
            }
        }
    }
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
 * apply (not an unpack, packed pointer off 16 bytes, 4 GiB or more), else a cudaError_t */
extern "C" int yk_cuda_launch_hidx_bulk(const yk_launch * l, void *stream, int ctas_per_sm)
{
    if (l->typed_op || !l->hidx || l->dir != 1 || ((uintptr_t) l->packed & 15) ||
        l->nbytes == 0 || l->nbytes > 0xffffffffull)
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

/* The same pack with the packed side staged per warp: each lane still reads its run
 * with 16-byte loads and puts its R bytes at lane * R in the warp's shared-memory tile;
 * after __syncwarp the warp writes the tile's 32 * R packed bytes as 16-byte chunks at
 * consecutive addresses.  The per-lane form writes R/4 pieces of 4 bytes at an R-byte
 * stride, so each of its store instructions touches about R sectors for 128 bytes;
 * here a store instruction fills whole sectors.  Only a warp, not the CTA, waits on the
 * tile.  Needs the packed pointer on 16 bytes (checked by the launcher) and R a
 * multiple of 4; a group of fewer than 32 elements writes its last bytes as 4-byte
 * words. */
template <int NV>
__global__ void __launch_bounds__(YK_THREADS, 8)
yk_runs_pack_warp_kernel(const __grid_constant__ yk_launch L, uint32_t R)
{
    __shared__ __align__(16) unsigned char stage[YK_THREADS / 32][32 * 48];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t E = L.desc.lv[0].stride;
    const uint32_t nel = (uint32_t) (L.nbytes / R), e0 = (uint32_t) (L.p0 / R);
    const char *tb = L.typed + L.desc.base;
    const uint32_t nw4 = R / 4;      /* R <= 16 * NV */
    unsigned char *st = stage[w];
    const uint32_t gw = (blockIdx.x * YK_THREADS + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * YK_THREADS) >> 5;
    for (uint32_t i0 = gw * 32; i0 < nel; i0 += nwarps * 32) {
        const uint32_t i = i0 + (uint32_t) lane;
        const uint32_t n = min(32u, nel - i0);
        if (i < nel) {
            const char *src = tb + (int64_t) (e0 + i) * E;
            union {
                uint4 w[NV];
                uint32_t u[4 * NV];
            } v;
#pragma unroll
            for (int k = 0; k < NV; k++)
                v.w[k] = yk_ldcg((const uint4 *) (src + 16 * k));
            uint32_t *sw = (uint32_t *) (st + (uint32_t) lane * R);
#pragma unroll
            for (int j = 0; j < 4 * NV; j++)
                if ((uint32_t) j < nw4)
                    sw[j] = v.u[j];
        }
        __syncwarp();
        char *dst = L.packed + (uint64_t) i0 * R;
        const uint32_t nbytes = n * R, nch = nbytes / 16;
        for (uint32_t c = (uint32_t) lane; c < nch; c += 32)
            *(uint4 *) (dst + 16 * c) = *(const uint4 *) (st + 16 * c);
        for (uint32_t q = nch * 16 + (uint32_t) lane * 4; q < nbytes; q += 128)
            *(uint32_t *) (dst + q) = *(const uint32_t *) (st + q);
        __syncwarp();
    }
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

/* ------------------------------------------------------------------------- */
/* elementwise operators                                                     */
/* ------------------------------------------------------------------------- */

enum { OP_MAX = 0, OP_MIN = 1, OP_SUM = 2, OP_PROD = 3, OP_LAND = 4, OP_BAND = 5, OP_LOR = 6,
    OP_BOR = 7, OP_LXOR = 8, OP_BXOR = 9, OP_REPLACE = 10 };

template <typename T> __device__ __forceinline__ T yk_ld(const char *p)
{
    if (((uintptr_t) p & (sizeof(T) - 1)) == 0)
        return *(const T *) p;
    T v;
    char *q = (char *) &v;
#pragma unroll
    for (int i = 0; i < (int) sizeof(T); i++)
        q[i] = p[i];
    return v;
}

template <typename T> __device__ __forceinline__ void yk_st(char *p, T v)
{
    if (((uintptr_t) p & (sizeof(T) - 1)) == 0) {
        *(T *) p = v;
        return;
    }
    const char *q = (const char *) &v;
#pragma unroll
    for (int i = 0; i < (int) sizeof(T); i++)
        p[i] = q[i];
}

/* integer operators; returns false when op is outside the type's table */
template <typename S, typename U>
__device__ __forceinline__ bool yk_int_op(int op, S in, S & out)
{
    switch (op) {
        case OP_REPLACE:
            out = in;
            return true;
        case OP_MAX:
            out = (in < out) ? out : in;
            return true;
        case OP_MIN:
            out = (in < out) ? in : out;
            return true;
        case OP_SUM:
            out = (S) (U) ((U) out + (U) in);
            return true;
        case OP_PROD:
            out = (S) (U) ((U) out * (U) in);
            return true;
        case OP_LAND:
            out = (S) (out && in);
            return true;
        case OP_LOR:
            out = (S) (out || in);
            return true;
        case OP_LXOR:
            out = (S) (!out != !in);
            return true;
        case OP_BAND:
            out = (S) (out & in);
            return true;
        case OP_BOR:
            out = (S) (out | in);
            return true;
        case OP_BXOR:
            out = (S) (out ^ in);
            return true;
    }
    return false;
}

__device__ __forceinline__ float yk_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double yk_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float yk_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double yk_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float yk_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double yk_mul(double a, double b) { return __dmul_rn(a, b); }

template <typename F>
__device__ __forceinline__ bool yk_flt_op(int op, F in, F & out)
{
    switch (op) {
        case OP_REPLACE:
            out = in;
            return true;
        case OP_MAX:
            out = (in < out) ? out : in;
            return true;
        case OP_MIN:
            out = (in > out) ? out : in;
            return true;
        case OP_SUM:
            out = yk_add(out, in);
            return true;
        case OP_PROD:
            out = yk_mul(out, in);
            return true;
    }
    return false;
}

/* (a + ib) * (c + id) with the infinity recovery of ISO C11 Annex G.5.1 */
template <typename F>
__device__ __forceinline__ void yk_cmul(F a, F b, F c, F d, F & x, F & y)
{
    F ac = yk_mul(a, c), bd = yk_mul(b, d), ad = yk_mul(a, d), bc = yk_mul(b, c);
    x = yk_sub(ac, bd);
    y = yk_add(ad, bc);
    if (isnan(x) && isnan(y)) {
        bool recalc = false;
        const F one = (F) 1, zero = (F) 0;
        if (isinf(a) || isinf(b)) {
            a = copysign(isinf(a) ? one : zero, a);
            b = copysign(isinf(b) ? one : zero, b);
            if (isnan(c))
                c = copysign(zero, c);
            if (isnan(d))
                d = copysign(zero, d);
            recalc = true;
        }
        if (isinf(c) || isinf(d)) {
            c = copysign(isinf(c) ? one : zero, c);
            d = copysign(isinf(d) ? one : zero, d);
            if (isnan(a))
                a = copysign(zero, a);
            if (isnan(b))
                b = copysign(zero, b);
            recalc = true;
        }
        if (!recalc && (isinf(ac) || isinf(bd) || isinf(ad) || isinf(bc))) {
            if (isnan(a))
                a = copysign(zero, a);
            if (isnan(b))
                b = copysign(zero, b);
            if (isnan(c))
                c = copysign(zero, c);
            if (isnan(d))
                d = copysign(zero, d);
            recalc = true;
        }
        if (recalc) {
            const F inf = (F) INFINITY;
            x = yk_mul(inf, yk_sub(yk_mul(a, c), yk_mul(b, d)));
            y = yk_mul(inf, yk_add(yk_mul(a, d), yk_mul(b, c)));
        }
    }
}

template <typename F>
__device__ __forceinline__ bool yk_cplx_op(int op, const F in[2], F out[2])
{
    switch (op) {
        case OP_REPLACE:
            out[0] = in[0];
            out[1] = in[1];
            return true;
        case OP_SUM:
            out[0] = yk_add(out[0], in[0]);
            out[1] = yk_add(out[1], in[1]);
            return true;
        case OP_PROD:{
                F x, y;
                yk_cmul(out[0], out[1], in[0], in[1], x, y);
                out[0] = x;
                out[1] = y;
                return true;
            }
    }
    return false;
}

__device__ __forceinline__ yk_u128 yk_ldq(const char *p)
{
    return ((yk_u128) yk_ld<uint64_t>(p + 8) << 64) | (yk_u128) yk_ld<uint64_t>(p);
}

__device__ __forceinline__ void yk_stq(char *p, yk_u128 v)
{
    yk_st<uint64_t>(p, (uint64_t) v);
    yk_st<uint64_t>(p + 8, (uint64_t) (v >> 64));
}

/* long double and long double complex in binary128: `out = out op in` as the
 * reference's seq loops compute it (MAX and MIN are the selects of the float types) */
__device__ __forceinline__ void yk_q_apply(int bt, int op, char *dst, const char *src)
{
    if (bt == YK_BT_LDOUBLE) {
        const yk_u128 in = yk_ldq(src), out = yk_ldq(dst);
        yk_u128 r;
        switch (op) {
            case OP_REPLACE: r = in; break;
            case OP_MAX: r = yk_q_lt(in, out) ? out : in; break;
            case OP_MIN: r = yk_q_lt(out, in) ? out : in; break;
            case OP_SUM: r = yk_q_add(out, in); break;
            case OP_PROD: r = yk_q_mul(out, in); break;
            default: return;
        }
        yk_stq(dst, r);
        return;
    }
    const yk_u128 ir = yk_ldq(src), ii = yk_ldq(src + 16);
    yk_u128 orr = yk_ldq(dst), oi = yk_ldq(dst + 16);
    switch (op) {
        case OP_REPLACE:
            orr = ir;
            oi = ii;
            break;
        case OP_SUM:
            orr = yk_q_add(orr, ir);
            oi = yk_q_add(oi, ii);
            break;
        case OP_PROD:
            yk_q_cmul(orr, oi, ir, ii, &orr, &oi);
            break;
        default:
            return;
    }
    yk_stq(dst, orr);
    yk_stq(dst + 16, oi);
}

/* apply op to one element of base type bt; `dst` is updated in place from `src`.
 * LD: the instance for types that hold long double, with the binary128 operators;
 * the other instance moves long double bytes for REPLACE only (the host sends every
 * long double operator to the LD instances), which keeps the 128-bit arithmetic out
 * of the register budget of the common kernels. */
template <bool LD>
__device__ __forceinline__ void yk_apply(int bt, int op, char *dst, const char *src)
{
    switch (bt) {
        case YK_BT_BOOL:{
                if (op != OP_REPLACE && op != OP_LAND && op != OP_LOR && op != OP_LXOR)
                    return;
                uint8_t i = yk_ld<uint8_t>(src), o = yk_ld<uint8_t>(dst);
                uint8_t r = op == OP_REPLACE ? i : op == OP_LAND ? (uint8_t) (o && i) :
                    op == OP_LOR ? (uint8_t) (o || i) : (uint8_t) (!o != !i);
                yk_st<uint8_t>(dst, r);
                return;
            }
        case YK_BT_I8:{
                int8_t i = yk_ld<int8_t>(src), o = yk_ld<int8_t>(dst);
                if (yk_int_op<int8_t, uint8_t>(op, i, o))
                    yk_st<int8_t>(dst, o);
                return;
            }
        case YK_BT_I16:{
                int16_t i = yk_ld<int16_t>(src), o = yk_ld<int16_t>(dst);
                if (yk_int_op<int16_t, uint16_t>(op, i, o))
                    yk_st<int16_t>(dst, o);
                return;
            }
        case YK_BT_I32:{
                int32_t i = yk_ld<int32_t>(src), o = yk_ld<int32_t>(dst);
                if (yk_int_op<int32_t, uint32_t>(op, i, o))
                    yk_st<int32_t>(dst, o);
                return;
            }
        case YK_BT_I64:{
                int64_t i = yk_ld<int64_t>(src), o = yk_ld<int64_t>(dst);
                if (yk_int_op<int64_t, uint64_t>(op, i, o))
                    yk_st<int64_t>(dst, o);
                return;
            }
        case YK_BT_F32:{
                float i = yk_ld<float>(src), o = yk_ld<float>(dst);
                if (yk_flt_op<float>(op, i, o))
                    yk_st<float>(dst, o);
                return;
            }
        case YK_BT_F64:{
                double i = yk_ld<double>(src), o = yk_ld<double>(dst);
                if (yk_flt_op<double>(op, i, o))
                    yk_st<double>(dst, o);
                return;
            }
        case YK_BT_C32:{
                float i[2] = { yk_ld<float>(src), yk_ld<float>(src + 4) };
                float o[2] = { yk_ld<float>(dst), yk_ld<float>(dst + 4) };
                if (yk_cplx_op<float>(op, i, o)) {
                    yk_st<float>(dst, o[0]);
                    yk_st<float>(dst + 4, o[1]);
                }
                return;
            }
        case YK_BT_C64:{
                double i[2] = { yk_ld<double>(src), yk_ld<double>(src + 8) };
                double o[2] = { yk_ld<double>(dst), yk_ld<double>(dst + 8) };
                if (yk_cplx_op<double>(op, i, o)) {
                    yk_st<double>(dst, o[0]);
                    yk_st<double>(dst + 8, o[1]);
                }
                return;
            }
        case YK_BT_LDOUBLE: case YK_BT_CLDOUBLE:
            if (LD) {
                yk_q_apply(bt, op, dst, src);
            } else if (op == OP_REPLACE) {
                yk_stq(dst, yk_ldq(src));
                if (bt == YK_BT_CLDOUBLE)
                    yk_stq(dst + 16, yk_ldq(src + 16));
            }
            return;
        default:
            /* CHAR/WCHAR only have REPLACE, which never reaches the typed kernel */
            return;
    }
}

__host__ __device__ __forceinline__ int yk_bt_size(int bt)
{
    switch (bt) {
        case YK_BT_BOOL: case YK_BT_CHAR: case YK_BT_I8: return 1;
        case YK_BT_I16: return 2;
        case YK_BT_WCHAR: case YK_BT_I32: case YK_BT_F32: return 4;
        case YK_BT_I64: case YK_BT_F64: case YK_BT_C32: return 8;
        case YK_BT_C64: case YK_BT_LDOUBLE: return 16;
        case YK_BT_CLDOUBLE: return 32;
        default: return 1;
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

/* element types in registers, for the typed ordered-unpack kernel */
template <int BT> struct yk_elem;
template <> struct yk_elem<YK_BT_I8> {
    typedef int8_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int8_t, uint8_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_I16> {
    typedef int16_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int16_t, uint16_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_I32> {
    typedef int32_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int32_t, uint32_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_I64> {
    typedef int64_t T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_int_op<int64_t, uint64_t>(o, in, out); }
};
template <> struct yk_elem<YK_BT_F32> {
    typedef float T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_flt_op<float>(o, in, out); }
};
template <> struct yk_elem<YK_BT_F64> {
    typedef double T;
    static __device__ __forceinline__ bool op(int o, T in, T & out) { return yk_flt_op<double>(o, in, out); }
};
template <> struct yk_elem<YK_BT_C32> {
    typedef float2 T;
    static __device__ __forceinline__ bool op(int o, T in, T & out)
    {
        float a[2] = { in.x, in.y }, b[2] = { out.x, out.y };
        bool r = yk_cplx_op<float>(o, a, b);
        out = make_float2(b[0], b[1]);
        return r;
    }
};
template <> struct yk_elem<YK_BT_C64> {
    typedef double2 T;
    static __device__ __forceinline__ bool op(int o, T in, T & out)
    {
        double a[2] = { in.x, in.y }, b[2] = { out.x, out.y };
        bool r = yk_cplx_op<double>(o, a, b);
        out = make_double2(b[0], b[1]);
        return r;
    }
};

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

/* Sorted blocks of a power-of-two byte length R, one packed element per lane (32-bit
 * positions), operator fixed at compile time.  The ownership rule of yk_owner_kernel
 * below: element x = disp[b] + j of block b belongs to b unless block b-1 covers x from
 * a position inside the range; no earlier block can cover x when b-1 does not, because
 * the displacements ascend.  The owner folds in the blocks b+1, b+2, ... that start at
 * or before x, in block order.  Lanes of one block read the same displacement words
 * (one broadcast per warp), packed elements are read contiguously across the warp and
 * each block's target run is read and written by consecutive lanes. */
template <int BT, int OP, bool D32>
__global__ void __launch_bounds__(YK_THREADS)
yk_owner_lane_kernel(const __grid_constant__ yk_launch L, int rshift)
{
    typedef typename yk_elem<BT>::T T;
    /* D32: offsets in 32 bits on the level's 32-bit copy of the displacements, where the
     * host found that every target offset fits (as in yk_owner_chunk_kernel) */
    typedef typename std::conditional<D32, int32_t, int64_t>::type OFF;
    constexpr OFF OFF_MAX = D32 ? (OFF) INT32_MAX : (OFF) INT64_MAX;
    constexpr uint32_t es = (uint32_t) sizeof(T);
    /* elements per lane, loads issued together (complex pairs keep one, within the
     * register budget of full occupancy) */
    constexpr int U = (BT == YK_BT_C32 || BT == YK_BT_C64) ? 1 : 2;
    const uint32_t R = 1u << rshift;
    const yk_level & lv = L.desc.lv[0];
    const uint32_t p0 = (uint32_t) L.p0, p1 = (uint32_t) (L.p0 + L.nbytes);
    const uint32_t nblk = (uint32_t) lv.count;
    const uint32_t nunits = (uint32_t) (L.nbytes / es);
    const T *packed = (const T *) L.packed;     /* element 0 is packed byte p0 */
    char *typed = L.typed + L.desc.base;
    const uint32_t nthr = gridDim.x * YK_THREADS;
    auto disp = [&](uint32_t i) -> OFF {
        if constexpr (D32)
            return __ldg((const int32_t *) (lv.disp + lv.count) + i);   /* the 32-bit copy */
        else
            return __ldg(lv.disp + i);
    };
    for (uint32_t u0 = blockIdx.x * YK_THREADS + threadIdx.x; u0 < nunits; u0 += U * nthr) {
        /* every load that does not depend on another first: the block's displacement,
         * its predecessor's and successor's, and the packed element */
        OFF x[U], dn[U];
        uint32_t b[U];
        bool own[U];
        T in[U], out[U], in1[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            const uint32_t u = u0 + k * nthr;
            own[k] = u < nunits;
            if (!own[k])
                continue;
            const uint32_t p = p0 + u * es;
            b[k] = p >> rshift;
            const OFF d = disp(b[k]);
            const OFF dp = b[k] > 0 ? disp(b[k] - 1) : 0;
            dn[k] = b[k] + 1 < nblk ? disp(b[k] + 1) : OFF_MAX;
            in[k] = __ldg(packed + u);
            x[k] = d + (OFF) (p & (R - 1));
            /* an earlier in-range block owns this element */
            if (b[k] > 0 && x[k] < dp + (OFF) R && (b[k] - 1) * R + (uint32_t) (x[k] - dp) >= p0)
                own[k] = false;
        }
        /* then the target element and the next block's contribution, if any */
#pragma unroll
        for (int k = 0; k < U; k++) {
            if (!own[k])
                continue;
            out[k] = *(const T *) (typed + x[k]);
            if (dn[k] <= x[k]) {
                const uint64_t pp = ((uint64_t) (b[k] + 1) << rshift) + (uint64_t) (x[k] - dn[k]);
                if (pp < p1)
                    in1[k] = __ldg(packed + ((uint32_t) pp - p0) / es);
                else
                    dn[k] = OFF_MAX;
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            if (!own[k])
                continue;
            yk_elem<BT>::op(OP, in[k], out[k]);
            if (dn[k] <= x[k]) {
                yk_elem<BT>::op(OP, in1[k], out[k]);
                /* rarer: the blocks after that, in block order */
                for (uint32_t bb = b[k] + 2; bb < nblk; bb++) {
                    const OFF d2 = disp(bb);
                    if (d2 > x[k])
                        break;
                    const uint64_t pp = ((uint64_t) bb << rshift) + (uint64_t) (x[k] - d2);
                    if (pp >= p1)
                        break;  /* later blocks place x later still */
                    yk_elem<BT>::op(OP, __ldg(packed + ((uint32_t) pp - p0) / es), out[k]);
                }
            }
            *(T *) (typed + x[k]) = out[k];
        }
    }
}

/* The same with one CW-byte packed chunk per lane (CW 8 or 16; elements of 1, 2 or 4
 * bytes, or 8-byte elements other than double): the chunk's elements share one block
 * (blocks are a multiple of CW bytes long and the range and the packed pointer sit on
 * CW bytes, checked on the host), so its displacement words and the packed load serve
 * CW/es elements.
 *
 * With at most four elements per chunk the fold has no loop for the common cases: the
 * displacements of the next two blocks are loaded with the chunk's own, their
 * contributions are loaded by predicated loads, and each is folded in by a select.  A
 * warp then executes one instruction stream with all its lanes, instead of a branch
 * per owner and a loop of dependent loads run by a few lanes (which left 12.8 of 32
 * lanes active per instruction).  Only a third later block, rare at these shapes,
 * takes the loop.  double keeps yk_owner_lane_kernel: there every fold is a DADD on
 * GB300's narrow FP64 pipe, which the selects would spend on every lane.
 *
 * D32: offsets and ownership tests in 32 bits on the level's 32-bit copy of the
 * displacements, where the host found that every target offset fits.  Complex float is
 * bounded to the 32 registers of full occupancy, with a 32-byte spill in the D32 form:
 * at 40 registers (6 CTAs per SM) the complex PROD config took 180.2 us, at 32 (8 per
 * SM) 170.0 us. */
template <int BT, int OP, int CW, bool D32>
__global__ void __launch_bounds__(YK_THREADS, (BT == YK_BT_C32 ? 7 : 1))
yk_owner_chunk_kernel(const __grid_constant__ yk_launch L, int rshift)
{
    typedef typename yk_elem<BT>::T T;
    typedef typename yk_vec<CW>::T CT;
    /* target offsets in 32 bits when the host found that every one fits (the level's
     * 32-bit copy of the displacements is read), else in 64 bits */
    typedef typename std::conditional<D32, int32_t, int64_t>::type OFF;
    constexpr OFF OFF_MAX = D32 ? (OFF) INT32_MAX : (OFF) INT64_MAX;
    constexpr uint32_t es = (uint32_t) sizeof(T);
    constexpr int E = CW / (int) es;
    const uint32_t R = 1u << rshift;
    const yk_level & lv = L.desc.lv[0];
    const uint32_t p0 = (uint32_t) L.p0, p1 = (uint32_t) (L.p0 + L.nbytes);
    const uint32_t nblk = (uint32_t) lv.count;
    const uint32_t nchunks = (uint32_t) (L.nbytes / CW);
    const CT *packedc = (const CT *) L.packed;  /* chunk 0 is byte p0 */
    const T *packed = (const T *) L.packed;
    char *typed = L.typed + L.desc.base;
    auto disp = [&](uint32_t i) -> OFF {
        if constexpr (D32)
            return __ldg((const int32_t *) (lv.disp + lv.count) + i);   /* the 32-bit copy */
        else
            return __ldg(lv.disp + i);
    };
    for (uint32_t u = blockIdx.x * YK_THREADS + threadIdx.x; u < nchunks; u += gridDim.x * YK_THREADS) {
        const uint32_t p = p0 + u * CW;
        const uint32_t b = p >> rshift;
        const OFF d = disp(b);
        const OFF dp = b > 0 ? disp(b - 1) : 0;
        const OFF dn = b + 1 < nblk ? disp(b + 1) : OFF_MAX;
        union {
            CT w;
            T e[E];
        } in;
        in.w = __ldg(packedc + u);
        const OFF x0 = d + (OFF) (p & (R - 1));
        bool own[E];
        T out[E];
        if constexpr (E <= 4) {
            const OFF dn2 = b + 2 < nblk ? disp(b + 2) : OFF_MAX;
            bool h1[E], h2[E];
            T c1[E], c2[E];
#pragma unroll
            for (int k = 0; k < E; k++) {
                const OFF x = x0 + (OFF) (k * (int) es);
                /* an earlier in-range block owns this element */
                own[k] = !(b > 0 && x < dp + (OFF) R && (b - 1) * R + (uint32_t) (x - dp) >= p0);
                if (own[k])
                    out[k] = *(const T *) (typed + x);
                /* the next two blocks' elements at x, when they exist and are in range (a
                 * later block places x later in the packed stream still) */
                h1[k] = false;
                h2[k] = false;
                c1[k] = c2[k] = T();
                if (own[k] && dn <= x) {
                    const uint64_t q1 = ((uint64_t) (b + 1) << rshift) + (uint64_t) (x - dn);
                    if (q1 < p1) {
                        h1[k] = true;
                        c1[k] = __ldg(packed + ((uint32_t) q1 - p0) / es);
                        if (dn2 <= x) {
                            const uint64_t q2 = ((uint64_t) (b + 2) << rshift) + (uint64_t) (x - dn2);
                            if (q2 < p1) {
                                h2[k] = true;
                                c2[k] = __ldg(packed + ((uint32_t) q2 - p0) / es);
                            }
                        }
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < E; k++) {
                const OFF x = x0 + (OFF) (k * (int) es);
                T v = out[k];
                yk_elem<BT>::op(OP, in.e[k], v);
                T t = v;
                yk_elem<BT>::op(OP, c1[k], t);
                v = h1[k] ? t : v;
                t = v;
                yk_elem<BT>::op(OP, c2[k], t);
                v = h2[k] ? t : v;
                if (h2[k]) {
                    /* rare: the blocks after those, in block order */
                    for (uint32_t bb = b + 3; bb < nblk; bb++) {
                        const OFF d3 = disp(bb);
                        if (d3 > x)
                            break;
                        const uint64_t pp = ((uint64_t) bb << rshift) + (uint64_t) (x - d3);
                        if (pp >= p1)
                            break;
                        yk_elem<BT>::op(OP, __ldg(packed + ((uint32_t) pp - p0) / es), v);
                    }
                }
                if (own[k])
                    *(T *) (typed + x) = v;
            }
        } else {
#pragma unroll
            for (int k = 0; k < E; k++) {
                const OFF x = x0 + (OFF) (k * (int) es);
                /* an earlier in-range block owns this element */
                own[k] = !(b > 0 && x < dp + (OFF) R && (b - 1) * R + (uint32_t) (x - dp) >= p0);
                if (own[k])
                    out[k] = *(const T *) (typed + x);
            }
#pragma unroll
            for (int k = 0; k < E; k++) {
                if (!own[k])
                    continue;
                const OFF x = x0 + (OFF) (k * (int) es);
                yk_elem<BT>::op(OP, in.e[k], out[k]);
                /* the blocks after this one that start at or before x, in block order */
                OFF dd = dn;
                for (uint32_t bb = b + 1; bb < nblk && dd <= x;) {
                    const uint64_t pp = ((uint64_t) bb << rshift) + (uint64_t) (x - dd);
                    if (pp >= p1)
                        break;
                    yk_elem<BT>::op(OP, __ldg(packed + ((uint32_t) pp - p0) / es), out[k]);
                    bb++;
                    dd = bb < nblk ? disp(bb) : OFF_MAX;
                }
                *(T *) (typed + x) = out[k];
            }
        }
    }
}

/* Reductions at L2 for the integer operators whose result does not depend on the order
 * in which contributions arrive: SUM (addition modulo 2^n), MAX, MIN (signed, as the
 * reference's unsigned handles alias the signed types), BAND, BOR and BXOR, on 4- and
 * 8-byte integers.  The value is sent to the L2 with a reduction (red.global.*, the
 * form an atomic whose result is unused compiles to), which reads, combines and writes
 * the target element there. */
template <int OP, typename T> __device__ __forceinline__ void yk_red(T *p, T v);
template <int OP> __device__ __forceinline__ void yk_red(int32_t *p, int32_t v)
{
    unsigned int *q = (unsigned int *) p;
    if constexpr (OP == OP_SUM) atomicAdd(q, (unsigned int) v);
    else if constexpr (OP == OP_MAX) atomicMax((int *) p, (int) v);
    else if constexpr (OP == OP_MIN) atomicMin((int *) p, (int) v);
    else if constexpr (OP == OP_BAND) atomicAnd(q, (unsigned int) v);
    else if constexpr (OP == OP_BOR) atomicOr(q, (unsigned int) v);
    else atomicXor(q, (unsigned int) v);
}
template <int OP> __device__ __forceinline__ void yk_red(int64_t *p, int64_t v)
{
    unsigned long long *q = (unsigned long long *) p;
    if constexpr (OP == OP_SUM) atomicAdd(q, (unsigned long long) v);
    else if constexpr (OP == OP_MAX) atomicMax((long long *) p, (long long) v);
    else if constexpr (OP == OP_MIN) atomicMin((long long *) p, (long long) v);
    else if constexpr (OP == OP_BAND) atomicAnd(q, (unsigned long long) v);
    else if constexpr (OP == OP_BOR) atomicOr(q, (unsigned long long) v);
    else atomicXor(q, (unsigned long long) v);
}

/* Overlapping blocks of R bytes (one IDX level in any block order, or one VEC level
 * whose stride is under its block) under one of those operators:
 * every packed element in the range is folded into its target element by one L2
 * reduction.  The operators are commutative and associative on integers, so the
 * target ends equal to the reference's in-order application (src/backend/seq/
 * genpup.py:119-211 with the operators of :302-327) whatever order the L2 applies the
 * contributions in, and no lane reads the target or resolves which block comes first.
 * Lane k of a warp takes packed element u0 + k, so the lanes of one block reduce into
 * consecutive target elements (one L2 sector request per 32 bytes).  Both sides are
 * aligned to the element size (checked on the host). */
template <int BT, int OP, int K, bool D32>
__global__ void __launch_bounds__(YK_THREADS)
yk_red_kernel(const __grid_constant__ yk_launch L)
{
    typedef typename yk_elem<BT>::T T;
    constexpr uint32_t es = (uint32_t) sizeof(T);
    constexpr int U = 4;        /* elements per lane, their loads issued together */
    const yk_level & lv = L.desc.lv[0];
    const uint32_t p0 = (uint32_t) L.p0;
    const uint32_t nunits = (uint32_t) (L.nbytes / es);
    const T *packed = (const T *) L.packed;     /* element 0 is packed byte p0 */
    char *typed = L.typed + L.desc.base;
    const uint32_t nthr = gridDim.x * YK_THREADS;
    for (uint32_t u0 = blockIdx.x * YK_THREADS + threadIdx.x; u0 < nunits; u0 += U * nthr) {
        int64_t x[U];
        T in[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            const uint32_t u = u0 + k * nthr;
            if (u < nunits) {
                const uint32_t p = p0 + u * es;
                const uint32_t b = yk_div(p, lv);
                int64_t at;
                if constexpr (K != YK_LV_IDX)
                    at = (int64_t) b * lv.stride;
                else if constexpr (D32)
                    at = __ldg((const int32_t *) (lv.disp + lv.count) + b);
                else
                    at = __ldg(lv.disp + b);
                x[k] = at + (int64_t) (p - b * (uint32_t) lv.cps);
                in[k] = __ldg(packed + u);
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++)
            if (u0 + k * nthr < nunits)
                yk_red<OP>((T *) (typed + x[k]), in[k]);
    }
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
/* persistent request server                                                 */
/* ------------------------------------------------------------------------- */

/* Each function processes the units [ub, ue) of one request with the CTA's threads. */
template <int V, int DIR>
__device__ __noinline__ void yk_srv_regular(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    /* four units per thread, their loads issued together (the launch form's shape) */
    for (uint32_t t0 = (uint32_t) ub; t0 < (uint32_t) ue; t0 += YK_THREADS)
        yk_regular_dispatch<V, DIR, 1>(L, t0, (uint32_t) ue);
}

template <int V, int DIR>
__device__ __noinline__ void yk_srv_bytes(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    for (uint64_t t0 = ub; t0 < ue; t0 += YK_THREADS)
        yk_bytes_tile<uint64_t, V, DIR, 1>(L, t0, ue);
}

__device__ __noinline__ void yk_srv_typed(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    const uint64_t g = (uint64_t) L.vec;
    const int op = (int) L.op;
    for (uint64_t u = ub + threadIdx.x; u < ue; u += YK_THREADS) {
        int bt;
        uint64_t inseg;
        int64_t off = yk_locate<uint64_t>(L.desc, L.p0 + u * g, &bt, &inseg);
        if (inseg % (uint64_t) yk_bt_size(bt))
            continue;
        char *t = L.typed + off;
        char *p = L.packed + u * g;
        if (L.dir == 0)
            yk_apply<false>(bt, op, p, t);
        else
            yk_apply<false>(bt, op, t, p);
    }
}

__device__ __noinline__ void yk_srv_owner(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    const yk_level & lv = L.desc.lv[0];
    const int bt = L.desc.leaf_type;
    const uint64_t es = (uint64_t) yk_bt_size(bt), R = lv.cps;
    const uint64_t p0 = L.p0, p1 = L.p0 + L.nbytes;
    const int op = (int) L.op;
    for (uint64_t u = ub + threadIdx.x; u < ue; u += YK_THREADS) {
        uint64_t p = p0 + u * es;
        uint64_t b = yk_div(p, lv);
        uint64_t j = p - b * R;
        int64_t x = __ldg(lv.disp + b) + (int64_t) j;
        if (b > 0) {
            int64_t dprev = __ldg(lv.disp + b - 1);
            if (x < dprev + (int64_t) R && (b - 1) * R + (uint64_t) (x - dprev) >= p0)
                continue;
        }
        char *t = L.typed + L.desc.base + x;
        for (uint64_t bb = b; bb < lv.count; bb++) {
            int64_t db = __ldg(lv.disp + bb);
            if (db > x)
                break;
            uint64_t pp = bb * R + (uint64_t) (x - db);
            if (pp >= p1)
                break;
            yk_apply<false>(bt, op, t, L.packed + (pp - p0));
        }
    }
}

/* sorted blocks with both sides aligned to the element size (the launch form is
 * yk_owner_lane_kernel): elements [ub, ue) of the request, two per thread, every load
 * that does not depend on another issued first; the owner of a target element (its
 * first in-range contributor) folds in the later blocks in block order. */
template <int BT, int OP>
__device__ __noinline__ void yk_srv_owner_t(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    typedef typename yk_elem<BT>::T T;
    constexpr uint64_t es = sizeof(T);
    constexpr int U = 2;
    constexpr int op = OP;
    const yk_level & lv = L.desc.lv[0];
    const uint64_t R = lv.cps, p0 = L.p0, p1 = L.p0 + L.nbytes, nblk = lv.count;
    const T *packed = (const T *) L.packed;     /* element 0 is packed byte p0 */
    char *typed = L.typed + L.desc.base;
    for (uint64_t u0 = ub + threadIdx.x; u0 < ue; u0 += U * YK_THREADS) {
        int64_t x[U], dn[U];
        uint64_t b[U];
        bool own[U], h1[U];
        T in[U], out[U], in1[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            const uint64_t u = u0 + (uint64_t) k * YK_THREADS;
            own[k] = u < ue;
            h1[k] = false;
            if (!own[k])
                continue;
            const uint64_t p = p0 + u * es;
            b[k] = yk_div(p, lv);
            const int64_t d = __ldg(lv.disp + b[k]);
            const int64_t dp = b[k] > 0 ? __ldg(lv.disp + b[k] - 1) : 0;
            dn[k] = b[k] + 1 < nblk ? __ldg(lv.disp + b[k] + 1) : INT64_MAX;
            in[k] = __ldg(packed + u);
            x[k] = d + (int64_t) (p - b[k] * R);
            /* an earlier in-range block owns this element */
            if (b[k] > 0 && x[k] < dp + (int64_t) R && (b[k] - 1) * R + (uint64_t) (x[k] - dp) >= p0)
                own[k] = false;
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            if (!own[k])
                continue;
            out[k] = *(const T *) (typed + x[k]);
            if (dn[k] <= x[k]) {
                const uint64_t pp = (b[k] + 1) * R + (uint64_t) (x[k] - dn[k]);
                if (pp < p1) {
                    h1[k] = true;
                    in1[k] = __ldg(packed + (pp - p0) / es);
                }
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++) {
            if (!own[k])
                continue;
            yk_elem<BT>::op(op, in[k], out[k]);
            if (h1[k]) {
                yk_elem<BT>::op(op, in1[k], out[k]);
                /* rarer: the blocks after that, in block order */
                for (uint64_t bb = b[k] + 2; bb < nblk; bb++) {
                    const int64_t d2 = __ldg(lv.disp + bb);
                    if (d2 > x[k])
                        break;
                    const uint64_t pp = bb * R + (uint64_t) (x[k] - d2);
                    if (pp >= p1)
                        break;  /* later blocks place x later still */
                    yk_elem<BT>::op(op, __ldg(packed + (pp - p0) / es), out[k]);
                }
            }
            *(T *) (typed + x[k]) = out[k];
        }
    }
}

/* a compile-time instance for complex-float PROD (600 against 510 GB/s on bursts of
 * 16 MiB requests); every other aligned sorted-block request takes the generic item,
 * double SUM included (its instance measured 579 against 624 GB/s at this kernel's
 * register bound) */
__device__ __noinline__ void yk_srv_owner_typed(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    if (L.desc.leaf_type == YK_BT_C32 && (int) L.op == OP_PROD)
        yk_srv_owner_t<YK_BT_C32, OP_PROD>(L, ub, ue);
    else
        yk_srv_owner(L, ub, ue);
}

/* struct-like packs (the launch form is yk_runs_pack_warp_kernel): elements [ib, ie) of
 * the request, ib a multiple of 32 (the host cuts these items in whole 32-element
 * groups), each warp staging a group's runs in shared memory and writing its packed
 * bytes as 16-byte chunks */
static __shared__ __align__(16) unsigned char yk_srv_stage[YK_THREADS / 32][32 * 48];

template <int NV>
__device__ __noinline__ void yk_srv_runs(const yk_launch & L, uint64_t ib, uint64_t ie)
{
    const uint32_t R = (uint32_t) L.desc.run;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t E = L.desc.lv[0].stride;
    const uint32_t e0 = (uint32_t) (L.p0 / R), nw4 = R / 4;
    const char *tb = L.typed + L.desc.base;
    unsigned char *st = yk_srv_stage[w];
    for (uint64_t i0 = ib + (uint64_t) w * 32; i0 < ie; i0 += (YK_THREADS / 32) * 32) {
        const uint64_t i = i0 + (uint64_t) lane;
        const uint32_t n = (uint32_t) min((uint64_t) 32, ie - i0);
        if (i < ie) {
            const char *src = tb + (int64_t) (e0 + i) * E;
            union {
                uint4 w[NV];
                uint32_t u[4 * NV];
            } v;
#pragma unroll
            for (int k = 0; k < NV; k++)
                v.w[k] = yk_ldcg((const uint4 *) (src + 16 * k));
            uint32_t *sw = (uint32_t *) (st + (uint32_t) lane * R);
#pragma unroll
            for (int j = 0; j < 4 * NV; j++)
                if ((uint32_t) j < nw4)
                    sw[j] = v.u[j];
        }
        __syncwarp();
        char *dst = L.packed + i0 * R;
        const uint32_t nbytes = n * R, nch = nbytes / 16;
        for (uint32_t c = (uint32_t) lane; c < nch; c += 32)
            *(uint4 *) (dst + 16 * c) = *(const uint4 *) (st + 16 * c);
        for (uint32_t q = nch * 16 + (uint32_t) lane * 4; q < nbytes; q += 128)
            *(uint32_t *) (dst + q) = *(const uint32_t *) (st + q);
        __syncwarp();
    }
}

/* overlapping equal blocks under an order-independent integer operator (the launch
 * form is yk_red_kernel): elements [ub, ue) of the request, each folded into its target
 * by one L2 reduction */
template <int BT, int OP>
__device__ __noinline__ void yk_srv_red_t(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    typedef typename yk_elem<BT>::T T;
    const yk_level & lv = L.desc.lv[0];
    const uint64_t es = sizeof(T), p0 = L.p0;
    char *typed = L.typed + L.desc.base;
    constexpr int U = 4;        /* elements per thread, their loads issued together */
    for (uint64_t u0 = ub + threadIdx.x; u0 < ue; u0 += U * YK_THREADS) {
        int64_t x[U];
        T v[U];
#pragma unroll
        for (int k = 0; k < U; k++) {
            const uint64_t u = u0 + (uint64_t) k * YK_THREADS;
            if (u < ue) {
                const uint64_t p = p0 + u * es;
                const uint64_t b = yk_div(p, lv);
                const int64_t at = lv.kind == YK_LV_IDX ? __ldg(lv.disp + b) : (int64_t) b * lv.stride;
                x[k] = at + (int64_t) (p - b * lv.cps);
                v[k] = *(const T *) (L.packed + (p - p0));
            }
        }
#pragma unroll
        for (int k = 0; k < U; k++)
            if (u0 + (uint64_t) k * YK_THREADS < ue)
                yk_red<OP>((T *) (typed + x[k]), v[k]);
    }
}

template <int BT>
__device__ __forceinline__ void yk_srv_red_bt(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    switch ((int) L.op) {
        case OP_MAX: yk_srv_red_t<BT, OP_MAX>(L, ub, ue); break;
        case OP_MIN: yk_srv_red_t<BT, OP_MIN>(L, ub, ue); break;
        case OP_SUM: yk_srv_red_t<BT, OP_SUM>(L, ub, ue); break;
        case OP_BAND: yk_srv_red_t<BT, OP_BAND>(L, ub, ue); break;
        case OP_BOR: yk_srv_red_t<BT, OP_BOR>(L, ub, ue); break;
        case OP_BXOR: yk_srv_red_t<BT, OP_BXOR>(L, ub, ue); break;
    }
}

__device__ __noinline__ void yk_srv_red(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    if (L.desc.leaf_type == YK_BT_I32)
        yk_srv_red_bt<YK_BT_I32>(L, ub, ue);
    else if (L.desc.leaf_type == YK_BT_I64)
        yk_srv_red_bt<YK_BT_I64>(L, ub, ue);
}

/* the whole request, in order, by warp 0 (targets that overlap arbitrarily) */
__device__ __noinline__ void yk_srv_ordered(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    if (threadIdx.x >= 32)
        return;
    const int lane = threadIdx.x;
    const uint64_t g = (uint64_t) L.vec;
    for (uint64_t c0 = ub; c0 < ue; c0 += 32) {
        uint64_t u = c0 + (uint64_t) lane;
        bool active = u < ue;
        int bt = YK_BT_NONE;
        uint64_t inseg = 0;
        int64_t off = 0;
        int len = 0;
        if (active) {
            off = yk_locate<uint64_t>(L.desc, L.p0 + u * g, &bt, &inseg);
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
                char *p = L.packed + u * g;
                if (L.typed_op)
                    yk_apply<false>(bt, (int) L.op, t, p);
                else
                    for (int i = 0; i < len; i++)
                        t[i] = p[i];
            }
            __syncwarp();
            if (!serial)
                break;
        }
    }
}

/* contiguous-block hindexed over the packed range [pb, pe): the CTA's warps split the
 * overlapping block groups (see yk_hidx_kernel) */
template <int V, int DIR>
__device__ __noinline__ void yk_srv_hidx(const yk_launch & L, uint64_t pb, uint64_t pe)
{
    typedef typename yk_vec<V>::T VT;
    const yk_level *lv = &L.desc.lv[0];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    char *typed = L.typed + L.desc.base;
    VT *packed = (VT *) L.packed;
    const uint64_t jb = yk_hidx_block(lv, pb), je = yk_hidx_block(lv, pe - 1);
    const uint64_t ngroups = (je - jb + 32) / 32;
    for (uint64_t gi = (uint64_t) w; gi < ngroups; gi += YK_THREADS / 32) {
        const uint64_t j0 = jb + gi * 32, jl = j0 + (uint64_t) lane;
        const uint64_t my_pfx = jl <= je ? __ldg(lv->pfx + jl) : ~(uint64_t) 0;
        const int64_t my_disp = jl <= je ? __ldg(lv->disp + jl) : 0;
        uint64_t start = max(__shfl_sync(0xffffffffu, my_pfx, 0), pb);
        uint64_t end = min(__ldg(lv->pfx + min(j0 + 32, je + 1)), pe);
        for (uint64_t base = start; base < end; base += (uint64_t) 32 * V) {
            const uint64_t p = base + (uint64_t) lane * V;
            int idx = 0;
#pragma unroll
            for (int step = 16; step > 0; step >>= 1) {
                uint64_t c = __shfl_sync(0xffffffffu, my_pfx, idx + step);
                if (c <= p)
                    idx += step;
            }
            const uint64_t bp = __shfl_sync(0xffffffffu, my_pfx, idx);
            const int64_t bd = __shfl_sync(0xffffffffu, my_disp, idx);
            if (p < end) {
                char *t = typed + bd + (int64_t) (p - bp);
                VT *q = packed + (p - L.p0) / V;
                if (DIR == 0)
                    *q = yk_ldcg((const VT *) t);
                else
                    *(VT *) t = yk_ldcg((const VT *) q);
            }
        }
    }
}

__device__ __forceinline__ uint64_t yk_ld_acquire_sys(const volatile uint64_t * p)
{
    uint64_t v;
    asm volatile ("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

/* host-written queue data is read at system scope: never from a stale cached copy */
__device__ __forceinline__ uint64_t yk_ld_sys(const void *p)
{
    uint64_t v;
    asm volatile ("ld.relaxed.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

/* An item of request slot `slot` is finished: count it into the request's completion
 * word; the CTA that finishes the request's last item appends slot + 1 to the completion
 * queue, so the host learns of completions without scanning every request in flight.
 * The item's bytes are made visible to the host first. */
__device__ __forceinline__ unsigned long long yk_globaltimer(void)
{
    unsigned long long t;
    asm volatile ("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void yk_srv_item_done(const yk_server_args & A, uint32_t slot)
{
    __threadfence_system();
    const unsigned long long old = atomicAdd_system(&A.req_done[slot], 1ull);
    if (old + 1 == yk_ld_sys(A.req_nitems + slot)) {
        const unsigned long long pos = atomicAdd(A.cq_tail, 1ull);
        asm volatile ("st.release.sys.global.u64 [%0], %1;"
                      :: "l"(A.cq + pos % A.qr), "l"((unsigned long long) slot + 1ull) : "memory");
    }
}

/* a record the GPU can act on: a known kind, a sane unit and an ordered range */
__device__ __forceinline__ bool yk_item_ok(const yk_item & it, const yk_launch & L)
{
    if ((it.kind & ~YK_SRV_TIMED) > YK_SRV_LAST || it.pe <= it.pb || it.pb < L.p0 ||
        it.pe > L.p0 + L.nbytes)
        return false;
    if (L.vec != 1 && L.vec != 2 && L.vec != 4 && L.vec != 8 && L.vec != 16)
        return false;
    return L.dir == 0 || L.dir == 1;
}

/* Resident CTAs claim work items one at a time (a compare-and-swap on a lane's counter
 * that never runs past the published count), stage the item's request record in shared
 * memory, process the item, and publish its completion.  A CTA tries its home lane
 * first, then the others in turn.  Every wait is bounded: a CTA that finds no new item
 * for idle_us microseconds of the GPU's global timer (or max_idle_spins polls), or sees
 * the stop flag, leaves; the host relaunches the kernel when items are pending and no
 * CTA is resident. */
/* The item functions above are out of line (__noinline__): each gets the kernel's
 * register budget to itself, so the loops of one item kind do not spill for the
 * registers another kind needs (inlined, the kernel spilled up to 3 KB).  That lets the
 * kernel run at 32 registers, eight resident CTAs per SM like the launch kernels: on the
 * mixed request stream 817 GB/s of capacity against 702-769 at six. */
__global__ void __launch_bounds__(YK_THREADS, 8)
yk_server_kernel(const __grid_constant__ yk_server_args A)
{
    __shared__ yk_launch sL;
    __shared__ uint64_t s_item;
    __shared__ int s_cmd;
    __shared__ yk_item s_it;
    uint64_t pub = 0;           /* thread 0: last published count read from the host */
    for (;;) {
        if (threadIdx.x == 0) {
            int cmd = 0;
            /* idle polls of the host-mapped counter back off from 64 ns to 2 us: many
             * resident CTAs polling at full rate would load the C2C link the host's own
             * submissions cross */
            unsigned nap = 64;
            const unsigned long long idle_t0 = yk_globaltimer();
            for (uint32_t spins = 0;; spins++) {
                if (*A.stop) {
                    cmd = 2;
                    break;
                }
                /* the published count only grows: re-read it from host memory only when
                 * every lane has caught up with the copy held here */
                bool pending = false;
                for (int pass = 0; pass < 2 && !pending; pass++) {
                    if (pass == 1)
                        pub = yk_ld_acquire_sys(A.items_published);
                    for (uint32_t i = 0; i < YK_SRV_LANES && cmd == 0; i++) {
                        const uint32_t lane = (blockIdx.x + i) % YK_SRV_LANES;
                        unsigned long long *ctr = A.next_item + lane * YK_SRV_LANE_STRIDE;
                        const unsigned long long c = *(volatile unsigned long long *) ctr;
                        const unsigned long long t = c * YK_SRV_LANES + lane;
                        if (t >= pub)
                            continue;
                        pending = true;
                        if (atomicCAS(ctr, c, c + 1) == c) {
                            s_item = t;
                            cmd = 1;
                        }
                    }
                }
                if (cmd == 1)
                    break;
                if (pending) {
                    if (spins >= 64u * A.max_idle_spins) {
                        cmd = 3;        /* hard bound: leave; the host relaunches */
                        break;
                    }
                    continue;
                }
                if (spins >= A.max_idle_spins ||
                    yk_globaltimer() - idle_t0 >= 1000ull * A.idle_us) {
                    cmd = 3;
                    break;
                }
                __nanosleep(nap);
                nap = nap < 2048 ? 2 * nap : 2048;
            }
            if (cmd == 1) {
                /* the item carries its own sequence number: re-read (bounded) until the
                 * host's write is the one seen */
                const yk_item *src = &A.items[s_item % A.qi];
                uint64_t w[4];
                uint32_t tries = 0;
                do {
                    for (int i = 0; i < 4; i++)
                        w[i] = yk_ld_sys((const uint64_t *) src + i);
                } while (w[0] != s_item && ++tries < 1000);
                if (w[0] != s_item)
                    cmd = 4;
                uint64_t *dst = (uint64_t *) &s_it;
                for (int i = 0; i < 4; i++)
                    dst[i] = w[i];
            }
            s_cmd = cmd;
        }
        __syncthreads();
        int cmd = s_cmd;
        if (cmd == 2 || cmd == 3) {
            if (threadIdx.x == 0)
                atomicAdd((unsigned int *) &A.status[cmd == 2 ? 1 : 0], 1u);
            return;
        }
        if (cmd == 1) {
            /* request record -> shared memory (8-byte words, system-scope loads) */
            const uint64_t *src = (const uint64_t *) (A.reqs + (s_it.req % A.qr));
            uint64_t *dst = (uint64_t *) &sL;
            for (uint32_t i = threadIdx.x; i < sizeof(yk_launch) / 8; i += YK_THREADS)
                dst[i] = yk_ld_sys(src + i);
        }
        __syncthreads();
        if (threadIdx.x == 0 && cmd == 1 && !yk_item_ok(s_it, sL))
            s_cmd = 4;
        __syncthreads();
        cmd = s_cmd;
        if (cmd == 4) {
            /* unusable item: count it, mark it done, move on (never loop on it) */
            if (threadIdx.x == 0) {
                atomicAdd((unsigned int *) &A.status[2], 1u);
                /* counted for its request only when the item record itself was current;
                 * otherwise the request stays incomplete and the host's bounded wait
                 * reports the error */
                if (s_it.seq == s_item)
                    yk_srv_item_done(A, s_it.req % A.qr);
            }
            __syncthreads();
            continue;
        }
        const yk_item it = s_it;
        const bool timed = (it.kind & YK_SRV_TIMED) != 0;
        const unsigned long long tb = timed && threadIdx.x == 0 ? yk_globaltimer() : 0ull;
        const uint64_t g = (uint64_t) sL.vec;
        const uint64_t ub = (it.pb - sL.p0) / g, ue = (it.pe - sL.p0) / g;
        switch (it.kind & ~YK_SRV_TIMED) {
            case YK_SRV_REGULAR:
#define YK_SV(V) do { if (sL.dir == 0) yk_srv_regular<V, 0>(sL, ub, ue); \
                      else yk_srv_regular<V, 1>(sL, ub, ue); } while (0)
                switch (sL.vec) {
                    case 16: YK_SV(16); break;
                    case 8: YK_SV(8); break;
                    case 4: YK_SV(4); break;
                    case 2: YK_SV(2); break;
                    default: YK_SV(1); break;
                }
#undef YK_SV
                break;
            case YK_SRV_BYTES:
#define YK_SB(V) do { if (sL.dir == 0) yk_srv_bytes<V, 0>(sL, ub, ue); \
                      else yk_srv_bytes<V, 1>(sL, ub, ue); } while (0)
                switch (sL.vec) {
                    case 16: YK_SB(16); break;
                    case 8: YK_SB(8); break;
                    case 4: YK_SB(4); break;
                    case 2: YK_SB(2); break;
                    default: YK_SB(1); break;
                }
#undef YK_SB
                break;
            case YK_SRV_TYPED:
                yk_srv_typed(sL, ub, ue);
                break;
            case YK_SRV_OWNER:
                yk_srv_owner(sL, (it.pb - sL.p0) / (uint64_t) yk_bt_size(sL.desc.leaf_type),
                             (it.pe - sL.p0) / (uint64_t) yk_bt_size(sL.desc.leaf_type));
                break;
            case YK_SRV_ORDERED:
                yk_srv_ordered(sL, ub, ue);
                break;
            case YK_SRV_RED:
                yk_srv_red(sL, (it.pb - sL.p0) / (uint64_t) yk_bt_size(sL.desc.leaf_type),
                           (it.pe - sL.p0) / (uint64_t) yk_bt_size(sL.desc.leaf_type));
                break;
            case YK_SRV_RUNS:
                if (sL.desc.run <= 32)
                    yk_srv_runs<2>(sL, (it.pb - sL.p0) / sL.desc.run, (it.pe - sL.p0) / sL.desc.run);
                else
                    yk_srv_runs<3>(sL, (it.pb - sL.p0) / sL.desc.run, (it.pe - sL.p0) / sL.desc.run);
                break;
            case YK_SRV_OWNER_T:
                yk_srv_owner_typed(sL, (it.pb - sL.p0) / (uint64_t) yk_bt_size(sL.desc.leaf_type),
                                   (it.pe - sL.p0) / (uint64_t) yk_bt_size(sL.desc.leaf_type));
                break;
            default:
#define YK_SH(V) do { if (sL.dir == 0) yk_srv_hidx<V, 0>(sL, it.pb, it.pe); \
                      else yk_srv_hidx<V, 1>(sL, it.pb, it.pe); } while (0)
                switch (sL.vec) {
                    case 16: YK_SH(16); break;
                    case 8: YK_SH(8); break;
                    case 4: YK_SH(4); break;
                    case 2: YK_SH(2); break;
                    default: YK_SH(1); break;
                }
#undef YK_SH
                break;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            if (timed)
                atomicAdd_system(A.req_busy + it.req % A.qr, yk_globaltimer() - tb);
            yk_srv_item_done(A, it.req % A.qr);   /* the item's bytes first, then its count */
        }
    }
}

extern "C" int yk_cuda_server_ctas(void)
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, yk_server_kernel, YK_THREADS, 0);
    if (per_sm < 1)
        per_sm = 1;
    return per_sm * yk_cuda_num_sms();
}

extern "C" int yk_cuda_server_launch(const yk_server_args * a, int ctas, void *stream)
{
    yk_server_kernel<<<ctas, YK_THREADS, 0, (cudaStream_t) stream>>>(*a);
    return (int) cudaGetLastError();
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
    if (l->nbytes > 0xffffffffull) {
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

static bool yk_owner_lane_launch(const yk_launch & c, int bt, int rshift, cudaStream_t s, int cap,
                                 bool d32)
{
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
template <int BT, int K, bool D32>
static bool yk_red_launch_bt(const yk_launch & c, cudaStream_t s, unsigned g)
{
    switch ((int) c.op) {
#define YK_RD(O) case O: yk_red_kernel<BT, O, K, D32><<<g, YK_THREADS, 0, s>>>(c); return true
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
    /* IDX: the 32-bit copy of the displacements when the level has one */
    const bool d32 = k == YK_LV_IDX && c.desc.lv[0].has_d32;
    if (bt == YK_BT_I32)
        return k != YK_LV_IDX ? yk_red_launch_bt<YK_BT_I32, YK_LV_VEC, false>(c, s, g) :
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
    const bool d32 = (sorted_blocks & YK_ORD_D32) != 0 && l->desc.lv[0].has_d32;
    sorted_blocks &= 3;
    bool typed_ok = sorted_blocks == 2 && (bt == YK_BT_I8 || bt == YK_BT_I16 || bt == YK_BT_I32 ||
                                           bt == YK_BT_I64 || bt == YK_BT_F32 || bt == YK_BT_F64 ||
                                           bt == YK_BT_C32 || bt == YK_BT_C64);
    const uint64_t R = c.desc.lv[0].cps;
    int rshift = 0;
    while (rshift < 31 && (1ull << rshift) < R)
        rshift++;
    if (typed_ok && !c.use64 && (1ull << rshift) == R &&
        yk_owner_lane_launch(c, bt, rshift, s, ctas_per_sm, d32)) {
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
