/*
 * yk_iov_dev.cu -- segment lists written by the GPU (no counterpart in the reference,
 * whose yaksa_iov fills a host array, src/frontend/iov/yaksa_iov.c:49-388).  A type's
 * list is `count` copies of one element's pieces, each shifted by the type's extent;
 * one thread writes one struct iovec (address, length) of the requested range.  The list
 * lands in device memory, where a NIC doing a gather (GPUDirect RDMA) or a GPU-initiated
 * transfer reads it without a host round trip.
 */
#include <cuda_runtime.h>
#include <stdint.h>
#include "yk_desc.h"

struct yk_iovec {
    void *base;
    uint64_t len;
};

__global__ void __launch_bounds__(256) yk_iov_expand_kernel(const char *buf, int64_t extent,
                                                            const int64_t *tpl, uint64_t n, uint64_t first,
                                                            uint64_t m, int64_t off1, uint64_t len1,
                                                            yk_iovec *out)
{
    for (uint64_t k = blockIdx.x * 256ull + threadIdx.x; k < m; k += (uint64_t) gridDim.x * 256) {
        yk_iovec v;
        if (tpl) {
            const uint64_t g = first + k, e = g / n, j = g - e * n;
            v.base = (void *) (buf + (int64_t) e * extent + tpl[2 * j]);
            v.len = (uint64_t) tpl[2 * j + 1];
        } else {
            v.base = (void *) (buf + off1);
            v.len = len1;
        }
        out[k] = v;
    }
}

extern "C" int yk_cuda_num_sms(void);

extern "C" int yk_cuda_iov_expand(const char *buf, int64_t extent, const int64_t *tpl, uint64_t n,
                                  uint64_t first, uint64_t m, int64_t off1, uint64_t len1, void *out,
                                  void *stream)
{
    if (!m)
        return 0;
    uint64_t need = (m + 255) / 256, cap = (uint64_t) yk_cuda_num_sms() * 8;
    unsigned g = (unsigned) (need < cap ? need : cap);
    yk_iov_expand_kernel<<<g, 256, 0, (cudaStream_t) stream>>>(buf, extent, tpl, n, first, m, off1, len1,
                                                                (yk_iovec *) out);
    return (int) cudaGetLastError();
}
