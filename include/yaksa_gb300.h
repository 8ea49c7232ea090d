/*
 * yaksa_gb300.h -- entry points of libyaksa.so beyond the reference's public API.
 *
 * These have no counterpart in the reference's yaksa.h; they expose what this GPU
 * engine adds (runtime counters, the batched request path).  Plain C types only.
 */
#ifndef YAKSA_GB300_H_INCLUDED
#define YAKSA_GB300_H_INCLUDED

#include <stdint.h>
#include "yaksa.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Runtime counters since load: kernel launches, calls served in place (device or
 * GPU-addressable host memory), calls that staged host data through device memory,
 * and contiguous calls served by one copy. */
int yaksa_gb300_stats(uint64_t * launches, uint64_t * direct_calls, uint64_t * staged_calls,
                      uint64_t * memcpy_calls);

/* CPU evaluation of the address computation the kernels perform: for each packed
 * byte position pos[i] of (count, type), off[i] receives the typed-buffer byte offset
 * (relative to the buffer pointer).  typed = 1 selects the operator descriptor,
 * 0 the byte-copy descriptor.  Used to validate descriptors without a GPU. */
int yaksa_gb300_debug_locate(yaksa_type_t type, uintptr_t count, int typed, uintptr_t n,
                             const uint64_t * pos, int64_t * off);

/* The descriptor analysis behind launch decisions: widest byte unit every run and
 * offset allows (vec_align), operator work-unit granule, whether two typemap entries
 * may reach the same byte, whether the sorted-block ordered unpack applies, and the
 * number of levels after simplification. */
int yaksa_gb300_debug_desc_info(yaksa_type_t type, int typed, int *vec_align, int *unit,
                                int *may_overlap, int *sorted_blocks, int *nlev);

#ifdef __cplusplus
}
#endif

#endif /* YAKSA_GB300_H_INCLUDED */
