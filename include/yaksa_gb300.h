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

/* One pack (kind 0) or unpack (kind 1) request, with the arguments of yaksa_pack /
 * yaksa_unpack: pack reads the typed buffer inbuf (count, type) and writes packed bytes
 * [offset, offset + actual) to outbuf; unpack reads maxbytes packed bytes from inbuf
 * into the typed buffer outbuf.  `actual` receives the bytes moved. */
typedef struct {
    int32_t kind;
    int32_t pad;
    const void *inbuf;
    void *outbuf;
    uintptr_t count;
    yaksa_type_t type;
    uintptr_t offset;
    uintptr_t maxbytes;
    yaksa_op_t op;
    uintptr_t actual;
} yaksa_gb300_pup_t;

/* Batched requests (no counterpart in the reference, whose callers issue one
 * yaksa_ipack/yaksa_iunpack per buffer).  The n requests must be independent (no
 * request writes bytes another reads or writes); they may run concurrently.  All
 * device-addressable REPLACE requests share a single kernel launch.
 *   _stream: enqueued on *(cudaStream_t *) stream (NULL: the library stream);
 *   blocking form: returns when every request completed;
 *   i-form: returns a request for yaksa_request_test / yaksa_request_wait. */
int yaksa_gb300_pup_batch_stream(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info, void *stream);
int yaksa_gb300_pup_batch(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info);
int yaksa_gb300_ipup_batch(yaksa_gb300_pup_t * ops, int n, yaksa_info_t info,
                           yaksa_request_t * request);

/* Captured sequences (no counterpart in the reference).  A halo exchange repeats the
 * same packs and unpacks on the same buffers every step; capturing them once into a
 * CUDA graph removes all per-step host work.  ops[0 .. batch_ends[0]) is the first
 * batch, ops[batch_ends[0] .. batch_ends[1]) the second, and so on; batches run in
 * order, the requests of one batch concurrently.  Buffers and types are bound at
 * creation (types stay referenced until yaksa_gb300_graph_free).  Requests whose
 * buffers the GPU cannot address are refused with YAKSA_ERR__NOT_SUPPORTED. */
typedef struct yaksa_gb300_graph_s *yaksa_gb300_graph_t;
int yaksa_gb300_graph_create(yaksa_gb300_pup_t * ops, const int *batch_ends, int nbatches,
                             yaksa_info_t info, yaksa_gb300_graph_t * graph);
int yaksa_gb300_graph_launch(yaksa_gb300_graph_t graph, void *stream);
int yaksa_gb300_graph_free(yaksa_gb300_graph_t graph);

/* Request server (no counterpart in the reference, whose progress engine launches
 * one kernel per request chunk, src/backend/src/yaksuri_progress.c:2862-3088).  A
 * persistent kernel keeps eight CTAs resident per SM and drains a work queue in
 * pinned, device-mapped host memory; requests are split into work items of up to
 * 256 KiB of packed bytes (YAKSA_GB300_SERVER_ITEM_KIB overrides it), and into at least
 * 128 items down to 32 KiB each (YAKSA_GB300_SERVER_MIN_ITEMS), so requests of any size
 * and type share the GPU as they arrive (continuous batching).
 *   create: ring_requests request slots (0: 4096), budget_bytes of packed bytes in
 *           flight (0: 64 GiB);
 *   submit: admits one request or returns YAKSA_ERR__OUT_OF_MEM when the rings or the
 *           byte budget are full (call progress/test and retry); requests whose buffers
 *           the GPU cannot address return YAKSA_ERR__NOT_SUPPORTED;
 *   test/wait: completion of a ticket (wait gives up with YAKSA_ERR__INTERNAL after
 *           20 s); progress: reclaims finished requests and keeps a kernel resident.
 * Resident CTAs that find no work for 2 ms leave; the next submit or progress call
 * relaunches them (about 30 us).  A device-wide synchronize (cudaDeviceSynchronize, or
 * work on the legacy default stream) waits for resident CTAs, so it returns up to 2 ms
 * after the server's last work.  Requests in flight together must be independent. */
typedef struct yaksa_gb300_server_s *yaksa_gb300_server_t;
int yaksa_gb300_server_create(uint32_t ring_requests, uint64_t budget_bytes,
                              yaksa_gb300_server_t * server);
int yaksa_gb300_server_submit(yaksa_gb300_server_t server, yaksa_gb300_pup_t * op,
                              yaksa_info_t info, uint64_t * ticket);
int yaksa_gb300_server_test(yaksa_gb300_server_t server, uint64_t ticket, int *done);
int yaksa_gb300_server_wait(yaksa_gb300_server_t server, uint64_t ticket);
int yaksa_gb300_server_progress(yaksa_gb300_server_t server);
int yaksa_gb300_server_stats(yaksa_gb300_server_t server, uint64_t * requests, uint64_t * items,
                             uint64_t * relaunches, uint32_t * idle_exits);
int yaksa_gb300_server_destroy(yaksa_gb300_server_t server);

/* Calibration of the server's work-item cut (no counterpart in the reference).  A
 * request of 256 KiB or more belongs to a class: work-item kind, unit, direction, base
 * type of an operator, and size to a power of two.  For each request of `ops` whose
 * class has no decision yet, the server runs the request under each candidate cut
 * (largest item 64 KiB to 1 MiB, least number of items 32 to 512), several times.
 * Each run submits enough concurrent copies for 64 MiB (at most 64, and half the
 * request ring), so that the items meet the memory contention of a loaded server. The
 * GPU times every item on the CTA that runs it, and the run's sample is the copies'
 * summed item time: the time per byte that bounds a loaded server's throughput. The
 * cut with the least time becomes the class's decision for every later submission
 * (the server's own cut unless another one is clearly faster).
 * Decisions persist in YAKSA_GB300_TUNE_FILE like the launch shapes.  The requests run
 * several times: for REPLACE their targets hold the result of one run; for other
 * operators they are left unspecified.  *classes (if not NULL) receives the number of
 * classes this call decided.  Call it with no other request of the server in flight. */
int yaksa_gb300_server_tune(yaksa_gb300_server_t server, yaksa_gb300_pup_t * ops, int n,
                            yaksa_info_t info, int *classes);

/* One pack (kind 0) or unpack (kind 1) that allocates nothing (no counterpart in the
 * reference).  For callers that must not allocate device memory: a library whose
 * device memory is all owned by the application's allocator, or code issuing requests
 * beside a resident persistent kernel, where the cudaFree that releases a type's
 * table allocation would synchronize the device.  Same kernels and bytes as
 * yaksa_pack_stream/yaksa_unpack_stream; the type's descriptor tables are copied into
 * a static 8 MiB device array on *stream (NULL: the legacy default stream) just before
 * the kernel; the call returns once both are enqueued and sets op->actual.
 *   - Stream: the legacy default stream (NULL) waits for all work on blocking streams
 *     and blocking streams wait for it.  Beside a resident kernel that runs on a
 *     blocking stream, pass a stream created with cudaStreamNonBlocking, or the table
 *     copy and the kernel wait for the resident kernel to end.
 *   - First calls: the first pack/unpack of the process (through any entry point)
 *     creates the library's own non-blocking streams; the first call on a device
 *     resolves the array's address (and may load the library's module); make these
 *     calls before any stream capture begins.  The first call for a type builds the
 *     type's host-side tables on the host heap, kept with the type until
 *     yaksa_type_free.  None of these allocates device memory.
 *   - kind other than 0 or 1 is refused with YAKSA_ERR__INTERNAL.
 *   - Types whose tables exceed 8 MiB (about 500,000 hindexed blocks) are refused
 *     with YAKSA_ERR__NOT_SUPPORTED and a message on stderr; so are buffers the GPU
 *     cannot address (staging would need device memory).
 *   - Nothing in the array needs to start at zero.  The array is shared: calls whose
 *     work overlaps in time (different streams, no ordering between them) race on it,
 *     so order them on one stream or by events. */
int yaksa_gb300_pup_noalloc(yaksa_gb300_pup_t * op, void *stream);

/* Serving loop (no counterpart in the reference, whose callers issue one
 * yaksa_ipack/yaksa_iunpack per message, src/frontend/include/yaksa.h.in:484,520):
 * replays n requests that arrive at arrival_s[i] seconds after the call starts.
 * mode 0 issues each as yaksa_ipack/yaksa_iunpack on arrival (one launch per
 * request); mode 1 submits them to `server`, admitting in arrival order and holding
 * a refused request (rings or byte budget full) at the head until progress frees
 * room; mode 2 is mode 0 with a graph lane: a request whose record (kind, buffers,
 * count, type, offset, size, operator) was seen before runs as the replay of a CUDA
 * graph of its launch, captured at its second sight (requests that need staging keep
 * the plain path; the graphs live for the call). latency_s[i] = completion time seen
 * by the loop - arrival_s[i]; *makespan_s = time of the last completion. ops[i].actual
 * is set. */
int yaksa_gb300_serve_trace(yaksa_gb300_pup_t * ops, const double *arrival_s, int n, int mode,
                            yaksa_gb300_server_t server, yaksa_info_t info, double *latency_s,
                            double *makespan_s);
/* the graph lane's launches captured and graphs replayed so far (all calls) */
int yaksa_gb300_graph_lane_stats(uint64_t * captures, uint64_t * replays);

/* Launch-shape autotuner (no counterpart in the reference): shape classes seen, classes
 * whose shape is decided, and launches timed so far.  YAKSA_GB300_AUTOTUNE=0 in the
 * environment keeps the default shapes. */
int yaksa_gb300_autotune_stats(uint32_t * classes, uint32_t * decided, uint64_t * probes);

/* Sharding (no counterpart in the reference): the part of the packed range of `count`
 * elements of `type` that rank `rank` of `nranks` moves, as (inoffset, max bytes) of
 * yaksa_pack / yaksa_unpack.  Both ends sit on builtin boundaries and the parts tile the
 * range, so N GPUs or processes each move their part with no exchange.  Host only. */
int yaksa_gb300_shard(yaksa_type_t type, uintptr_t count, int rank, int nranks,
                      uintptr_t * offset, uintptr_t * bytes);

/* Test hook (no counterpart in the reference): the library's next `n` device or pinned
 * allocations fail as if memory were exhausted, without calling the allocator, so that
 * error paths are exercised with no GPU fault.  0 clears it. */
int yaksa_gb300_debug_fail_alloc(int n);

/* Measurement instrument (no counterpart in the reference): touch the typed-side bytes
 * of up to 16 strided layouts in one launch, with plain loads (write = 0) or plain
 * stores of zeros (write = 1) and nothing else.  Pattern k is n1 x n0 runs of `run`
 * bytes (a multiple of 4) at base + i1 * s1 + i0 * s0.  The bench times it over the
 * addresses of a pack or unpack to measure the floor that DRAM row accesses set for
 * any kernel moving those bytes.  Stores overwrite the runs: use scratch buffers. */
typedef struct {
    void *base;
    uint64_t n1;
    int64_t s1;
    uint64_t n0;
    int64_t s0;
    uint32_t run;
    uint32_t pad;
} yaksa_gb300_rows_t;
int yaksa_gb300_probe_rows(const yaksa_gb300_rows_t * pats, int npats, int write, void *stream);

/* Test hook (no counterpart in the reference): the forms of the kernels that move data
 * with the tensor memory accelerator -- the TMA tensor-map kernels for regular nests
 * (cp.async.bulk.tensor over the typed side) and the hindexed unpack that stages the
 * packed stream with cp.async.bulk.  mode 0 never uses them, 1 lets the launch-shape
 * autotuner choose them per shape class where they are faster (the default;
 * YAKSA_GB300_TMA=0/1/2 in the environment sets the initial mode), 2 uses them wherever
 * one exists.  Results are identical in every mode.  yaksa_gb300_debug_tma_stats reports
 * the launches of these forms so far and the tensor-map waits that ran out;
 * yaksa_gb300_debug_bulk_failures the bulk-staged unpack's waits that ran out (both
 * always 0 in correct operation). */
int yaksa_gb300_debug_tma(int mode);
int yaksa_gb300_debug_tma_stats(unsigned long long *launches, unsigned int *failures);
int yaksa_gb300_debug_bulk_failures(unsigned int *n);

/* Test hook (no counterpart in the reference): the L2-reduction form of unpacks whose
 * targets overlap.  When the type is one level of equal blocks (indexed_block,
 * hindexed_block, or indexed/hindexed with equal lengths) in any order, or a vector
 * whose stride is under its block length, or count > 1 elements of one contiguous run
 * whose extent is shorter than the run, the operator
 * is SUM, MAX, MIN, BAND, BOR or BXOR on a 4- or 8-byte integer type, and both buffers
 * sit on the element size, each packed element is folded into its target by one
 * reduction at L2 (red.global) instead of an ordered read-combine-write.  These
 * operators are commutative and associative on integers, so the bytes equal the
 * in-order result.  mode 0 never uses the form, 1 uses it wherever it applies (the
 * default; YAKSA_GB300_L2_REDUCE=0 in the environment sets mode 0), -1 leaves the mode
 * as it is.  *launches (if not NULL) receives the form's launches so far. */
int yaksa_gb300_debug_l2_reduce(int mode, unsigned long long *launches);

/* Test hook (no counterpart in the reference): the launch shape of contiguous-block
 * hindexed packs and unpacks.  variant < 0 lets the launch-shape autotuner choose (the
 * default).  variant 0 forces the shuffle-search kernel with `units` naming its shape
 * for 4- and 8-byte units (0: 8 units per lane at 4 resident CTAs per SM, 4: 4 at 6,
 * 2: 2 at 8; unpacks also 16: 16 at 3) and `ctas` CTAs per SM in the grid (0: the
 * shape's residency, one wave); variant 3
 * forces the bulk-staged unpack with `ctas` CTAs per SM (packs, and unpacks outside its
 * rules, take the shuffle kernel).  Results are identical in every shape. */
int yaksa_gb300_debug_hidx_shape(int variant, int units, int ctas);

/* Segment list on the GPU (no counterpart in the reference, whose yaksa_iov fills a
 * host array, src/frontend/include/yaksa.h.in:609): the same entries as yaksa_iov --
 * count, type, iov_offset and max_iov_len mean the same, and *actual_iov_len is set on
 * return -- written by a kernel into `iov`, an array of struct iovec in memory the GPU
 * can address, enqueued on *(cudaStream_t *) stream (NULL: the legacy default stream).
 * For a NIC gathering from a list in GPU memory (GPUDirect RDMA) or GPU-initiated
 * transfers, with no host round trip per message.  The first call for a type keeps one
 * element's pieces in device memory until yaksa_type_free. */
int yaksa_gb300_iov_stream(const char *buf, uintptr_t count, yaksa_type_t type,
                           uintptr_t iov_offset, struct iovec *iov, uintptr_t max_iov_len,
                           uintptr_t * actual_iov_len, void *stream);

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

/* The 32-bit forms of a descriptor (typed = 1: the operator descriptor), computed on the
 * host: level0_bits receives its first level's bits (1: the displacements fit in 32 bits
 * and a 32-bit copy of them follows the table; 2: every displacement plus the block
 * length fits as well), disp32 whether the sorted-block kernels may take every target
 * offset in 32 bits. */
int yaksa_gb300_debug_d32(yaksa_type_t type, int typed, int *level0_bits, int *disp32);

#ifdef __cplusplus
}
#endif

#endif /* YAKSA_GB300_H_INCLUDED */
