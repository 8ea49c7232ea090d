/*
 * Static descriptor scratch for yaksa_gb300_pup_noalloc (no counterpart in the
 * reference).
 *
 * The plain path keeps each type's flattened tables (block displacements, prefix
 * sums, hindexed tile tables, segment lists) in one device allocation made at the
 * type's first pack/unpack.  Two kinds of caller cannot make that allocation:
 *   - a communication library running inside an application whose device memory is
 *     owned by a caching allocator that has reserved it all, so cudaMalloc fails or
 *     fragments the application's pool in the middle of a step;
 *   - code that issues packs while a persistent kernel (this library's request
 *     server, or a peer library's proxy kernel) stays resident: releasing a table
 *     allocation later calls cudaFree, which synchronizes the device and so waits
 *     for that kernel.
 * For them the tables travel with each request into this fixed array, written on the
 * caller's stream just before the kernel that reads them.
 *
 * Setup: the first call on a device resolves the array's address with that device
 * current (cudaGetSymbolAddress, which also loads this module if lazy loading has not
 * yet done so); later calls reuse the address.  Make that first call before any
 * stream capture begins.  Nothing in the array needs to start at zero: each call
 * writes every table byte its kernel reads before the launch.
 */
#include <cuda_runtime.h>
#include <pthread.h>
#include <stddef.h>

#define YK_NOALLOC_SCRATCH_BYTES (8u << 20)     /* the largest table set accepted */
#define YK_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char yk_noalloc_tables[YK_NOALLOC_SCRATCH_BYTES];

static pthread_mutex_t yk_noalloc_mu = PTHREAD_MUTEX_INITIALIZER;
static void *yk_noalloc_addr[YK_NOALLOC_MAX_DEVICES];

/* address of the scratch on the current device (resolved once per device) and its
 * size; returns a cudaError_t value */
extern "C" int yk_noalloc_scratch(void **ptr, size_t *bytes)
{
    *ptr = NULL;
    *bytes = YK_NOALLOC_SCRATCH_BYTES;
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return (int) e;
    if (dev < 0 || dev >= YK_NOALLOC_MAX_DEVICES)
        return (int) cudaErrorInvalidDevice;
    pthread_mutex_lock(&yk_noalloc_mu);
    if (!yk_noalloc_addr[dev]) {
        void *p = NULL;
        e = cudaGetSymbolAddress(&p, yk_noalloc_tables);
        if (e == cudaSuccess)
            yk_noalloc_addr[dev] = p;
    }
    *ptr = yk_noalloc_addr[dev];
    pthread_mutex_unlock(&yk_noalloc_mu);
    return (int) e;
}
