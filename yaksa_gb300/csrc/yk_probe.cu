/*
 * yk_probe.cu -- a measurement instrument (no counterpart in the reference): the time
 * the GPU needs just to touch the typed-side bytes of a strided layout, with plain
 * loads or plain stores and nothing else.  The bench runs it over the exact addresses
 * of a pack or unpack (the halo x-faces: 8-byte runs, one per 2 KiB grid row) to give
 * the floor that DRAM row accesses set under any kernel that moves those bytes.
 *
 * A pattern is n1 x n0 runs of `run` bytes at base + i1 * s1 + i0 * s0.  Each thread
 * touches one run with the widest power-of-two unit (16 bytes at most) that divides
 * the run, the strides and the base.  Loads are folded into a value stored only when
 * it equals an impossible marker, so they cannot be removed; stores write zeros.
 * All patterns of a call run in one launch, like the batched pack kernel.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include "yaksa_gb300.h"

#define YK_PROBE_MAX 16

struct yk_probe_args {
    yaksa_gb300_rows_t p[YK_PROBE_MAX];
    uint64_t start[YK_PROBE_MAX + 1];   /* first run of each pattern */
    uint32_t unit[YK_PROBE_MAX];
    int n;
    int write;
    uint32_t *sink;
};

/* the loads of the pack kernels: cached in L2 only */
__device__ __forceinline__ uint4 yk_probe_ld(const uint4 *p)
{
    uint4 v;
    asm volatile ("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                  : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
    return v;
}

__device__ __forceinline__ uint2 yk_probe_ld(const uint2 *p)
{
    uint2 v;
    asm volatile ("ld.global.cg.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t yk_probe_ld(const uint32_t *p)
{
    uint32_t v;
    asm volatile ("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ uint32_t yk_fold(uint4 v) { return v.x ^ v.y ^ v.z ^ v.w; }
__device__ __forceinline__ uint32_t yk_fold(uint2 v) { return v.x ^ v.y; }
__device__ __forceinline__ uint32_t yk_fold(uint32_t v) { return v; }

template <typename T>
__device__ __forceinline__ uint32_t yk_probe_run(char *p, uint32_t run, int write)
{
    uint32_t acc = 0;
    for (uint32_t o = 0; o < run; o += sizeof(T)) {
        if (write)
            *(T *) (p + o) = T();
        else
            acc ^= yk_fold(yk_probe_ld((const T *) (p + o)));
    }
    return acc;
}

__global__ void __launch_bounds__(256) yk_probe_kernel(const __grid_constant__ yk_probe_args A)
{
    const uint64_t total = A.start[A.n];
    uint32_t acc = 0;
    for (uint64_t r = blockIdx.x * 256ull + threadIdx.x; r < total; r += (uint64_t) gridDim.x * 256) {
        int k = 0;
        while (r >= A.start[k + 1])
            k++;
        const yaksa_gb300_rows_t &q = A.p[k];
        const uint64_t i = r - A.start[k];
        char *p = (char *) q.base + (int64_t) (i / q.n0) * q.s1 + (int64_t) (i % q.n0) * q.s0;
        switch (A.unit[k]) {
            case 16: acc ^= yk_probe_run<uint4>(p, q.run, A.write); break;
            case 8: acc ^= yk_probe_run<uint2>(p, q.run, A.write); break;
            default: acc ^= yk_probe_run<uint32_t>(p, q.run, A.write); break;
        }
    }
    if (acc == 0x8badf00du && A.sink)
        *A.sink = acc;
}

static uint32_t yk_probe_unit(const yaksa_gb300_rows_t &q)
{
    uint64_t g = q.run | (uint64_t) (uintptr_t) q.base | (uint64_t) (q.s0 < 0 ? -q.s0 : q.s0) |
        (uint64_t) (q.s1 < 0 ? -q.s1 : q.s1);
    return (g & 15) == 0 ? 16 : (g & 7) == 0 ? 8 : 4;
}

extern "C" int yaksa_gb300_probe_rows(const yaksa_gb300_rows_t * pats, int npats, int write,
                                      void *stream)
{
    if (npats < 1 || npats > YK_PROBE_MAX)
        return YAKSA_ERR__NOT_SUPPORTED;
    yk_probe_args A = {};
    A.n = npats;
    A.write = write;
    for (int k = 0; k < npats; k++) {
        const yaksa_gb300_rows_t &q = pats[k];
        if (!q.base || q.n0 == 0 || q.n1 == 0 || q.run == 0 || q.run % 4)
            return YAKSA_ERR__NOT_SUPPORTED;
        A.p[k] = q;
        A.unit[k] = yk_probe_unit(q);
        A.start[k + 1] = A.start[k] + q.n0 * q.n1;
    }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    uint64_t need = (A.start[npats] + 255) / 256, cap = (uint64_t) sms * 8;
    unsigned g = (unsigned) (need < cap ? need : cap);
    cudaStream_t s = stream ? *(cudaStream_t *) stream : (cudaStream_t) 0;
    yk_probe_kernel<<<g ? g : 1, 256, 0, s>>>(A);
    return cudaGetLastError() == cudaSuccess ? YAKSA_SUCCESS : YAKSA_ERR__INTERNAL;
}
