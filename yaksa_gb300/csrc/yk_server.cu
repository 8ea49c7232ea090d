/*
 * yk_server.cu -- the persistent request server for sm_103a: resident CTAs claim
 * work items that the host publishes in host-mapped rings, run each with the item
 * function of its kind (the launch kernels' bodies where one exists, yk_device.cuh)
 * and publish completions.
 */
#include "yk_device.cuh"

/* ------------------------------------------------------------------------- */
/* persistent request server                                                 */
/* ------------------------------------------------------------------------- */

/* Each function processes the units [ub, ue) of one request with the CTA's threads. */
template <int V, int DIR>
__device__ __noinline__ void yk_srv_regular(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    /* two units per thread, their loads issued together (one of 16 bytes) */
    constexpr int U = V == 16 ? 1 : 2;
    for (uint32_t t0 = (uint32_t) ub; t0 < (uint32_t) ue; t0 += U * YK_THREADS)
        yk_regular_dispatch<V, DIR, U>(L, t0, (uint32_t) ue);
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

/* Sorted blocks with both sides aligned to the element size, with the block shift and
 * 32-bit offsets of the form the host chose with yk_cuda_owner_form (yk_launch.form):
 * the body of yk_owner_lane_kernel over elements [ub, ue) of the request, one element
 * per lane.  In the server every invariant of an item takes a thread register (the
 * record is in shared memory, not the constant bank), and there fewer live values win:
 * bursts of 16 requests of 16 MiB, GB/s with the launch kernels' forms (16-byte chunks,
 * or two elements per lane) -> this form: double SUM 652 -> 812-841, complex PROD
 * 600 -> 890-906, float SUM 464 -> 646-661, int32 PROD 456 -> 650-662, int16 SUM
 * 272 -> 428, int64 PROD 794-797 (chunks) -> 858-866. */
template <int BT, int OP>
__device__ __noinline__ void yk_srv_owner_t(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    yk_owner_lane_units<BT, OP, true, 1>(L, L.form & 255, (uint32_t) ub + threadIdx.x, (uint32_t) ue,
                                         YK_THREADS);
}

/* the compile-time instances of a base type: SUM, PROD, MAX, MIN (not complex) and
 * REPLACE; false for the other operators */
template <int BT>
__device__ __forceinline__ bool yk_srv_owner_bt(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    constexpr bool cplx = BT == YK_BT_C32 || BT == YK_BT_C64;
    switch ((int) L.op) {
        case OP_SUM: yk_srv_owner_t<BT, OP_SUM>(L, ub, ue); return true;
        case OP_PROD: yk_srv_owner_t<BT, OP_PROD>(L, ub, ue); return true;
        case OP_REPLACE: yk_srv_owner_t<BT, OP_REPLACE>(L, ub, ue); return true;
        case OP_MAX:
            if constexpr (!cplx) {
                yk_srv_owner_t<BT, OP_MAX>(L, ub, ue);
                return true;
            }
            break;
        case OP_MIN:
            if constexpr (!cplx) {
                yk_srv_owner_t<BT, OP_MIN>(L, ub, ue);
                return true;
            }
            break;
    }
    return false;
}

/* aligned sorted blocks: the per-lane body where the blocks are a power of two long,
 * the offsets fit in 32 bits and the operator has an instance, else the generic item */
__device__ __noinline__ void yk_srv_owner_typed(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    bool done = false;
    if ((L.form & YK_FORM_POW2) && (L.form & YK_FORM_D32)) {
        switch (L.desc.leaf_type) {
            case YK_BT_I8: done = yk_srv_owner_bt<YK_BT_I8>(L, ub, ue); break;
            case YK_BT_I16: done = yk_srv_owner_bt<YK_BT_I16>(L, ub, ue); break;
            case YK_BT_I32: done = yk_srv_owner_bt<YK_BT_I32>(L, ub, ue); break;
            case YK_BT_I64: done = yk_srv_owner_bt<YK_BT_I64>(L, ub, ue); break;
            case YK_BT_F32: done = yk_srv_owner_bt<YK_BT_F32>(L, ub, ue); break;
            case YK_BT_F64: done = yk_srv_owner_bt<YK_BT_F64>(L, ub, ue); break;
            case YK_BT_C32: done = yk_srv_owner_bt<YK_BT_C32>(L, ub, ue); break;
            case YK_BT_C64: done = yk_srv_owner_bt<YK_BT_C64>(L, ub, ue); break;
        }
    }
    if (!done)
        yk_srv_owner(L, ub, ue);
}

/* struct-like packs (the launch form is yk_runs_pack_warp_kernel): elements [ib, ie) of
 * the request, ib a multiple of 32 (the host cuts these items in whole 32-element
 * groups), each warp taking every eighth group with its own stage */
static __shared__ __align__(16) unsigned char yk_srv_stage[YK_THREADS / 32][32 * 48];

template <int NV>
__device__ __noinline__ void yk_srv_runs(const yk_launch & L, uint64_t ib, uint64_t ie)
{
    const uint32_t w = threadIdx.x >> 5;
    yk_runs_pack_groups<NV>(L, (uint32_t) L.desc.run, yk_srv_stage[w], (uint32_t) ib + w * 32,
                            (uint32_t) ie, YK_THREADS);
}

/* overlapping equal blocks under an order-independent integer operator (the launch
 * form is yk_red_kernel, with 32-bit positions): elements [ub, ue) of the request, one
 * out-of-line function per level form */
/* two elements per lane, not the launch kernel's four: fewer live registers (bursts of
 * 16 requests of 16 MiB: int64 MAX 785-819 -> 873-898 GB/s, uint32 BXOR 679 -> 722) */
template <int BT, int OP, int K, bool D32, bool P2X = false>
__device__ __noinline__ void yk_srv_red_k(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    yk_red_units<BT, OP, K, D32, 2, P2X>(L, (uint32_t) ub + threadIdx.x, (uint32_t) ue, YK_THREADS);
}

template <int BT, int OP>
__device__ __forceinline__ void yk_srv_red_t(const yk_launch & L, uint64_t ub, uint64_t ue)
{
    const yk_level & lv = L.desc.lv[0];
    if (lv.kind != YK_LV_IDX) {
        yk_srv_red_k<BT, OP, YK_LV_VEC, false>(L, ub, ue);
        return;
    }
    /* the launch's choice of form: the shift and 32-bit offsets for 4-byte integers
     * (server bursts of 16 uint32 BXOR requests of 16 MiB: 572-595 -> 666 GB/s) */
    if constexpr (BT == YK_BT_I32) {
        if (yk_red_p2x(lv)) {
            yk_srv_red_k<BT, OP, YK_LV_IDX, true, true>(L, ub, ue);
            return;
        }
    }
    if (lv.has_d32 & YK_D32_TABLE)
        yk_srv_red_k<BT, OP, YK_LV_IDX, true>(L, ub, ue);
    else
        yk_srv_red_k<BT, OP, YK_LV_IDX, false>(L, ub, ue);
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

/* contiguous-block hindexed over the packed range [pb, pe) of an item (under 4 GiB by
 * construction): the body of yk_hidx32_kernel in its full-occupancy shape, two units
 * per lane and the next group's index words loaded ahead, the CTA's warps taking
 * every eighth group */
template <int V, int DIR>
__device__ __noinline__ void yk_srv_hidx(const yk_launch & L, uint64_t pb, uint64_t pe)
{
    yk_hidx32_groups<V, DIR, 2, true>(L, pb, pe, threadIdx.x >> 5, YK_THREADS / 32);
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
