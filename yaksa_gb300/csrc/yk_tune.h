/* yk_tune.h -- launch-shape autotuner of the byte-moving kernels (yk_tune.c) */
#ifndef YK_TUNE_H
#define YK_TUNE_H

#include <stdint.h>

/* SINGLE_TMA: a single launch that also has a TMA form; RUNS_TMA: a struct-like pack
 * (one element per thread) that also has a TMA form */
enum { YK_TUNE_SINGLE = 1, YK_TUNE_BATCH_REGULAR = 2, YK_TUNE_BATCH = 3, YK_TUNE_SINGLE_TMA = 4,
    YK_TUNE_RUNS_TMA = 5, YK_TUNE_HIDX = 6, YK_TUNE_TYPED = 7, YK_TUNE_OWNER = 8,
    YK_TUNE_HIDX_UNPACK = 9, YK_TUNE_SERVER = 10 };

/* BULK: the hindexed unpack with the packed stream staged by cp.async.bulk */
enum { YK_VARIANT_BYTES = 0, YK_VARIANT_TMA = 1, YK_VARIANT_RUNS = 2, YK_VARIANT_BULK = 3 };

typedef struct {
    int units_per_thread;       /* 1 or 4; 0 = chosen by size (hindexed: 2 or 8 name that
                                 * kernel's other two shapes) */
    int ctas_per_sm;            /* grid cap; 0 = by units per thread */
    int variant;                /* YK_VARIANT_*: which kernel runs the launch */
} yk_tune_cfg;

/* shape class of a launch */
uint64_t yk_tune_key(int family, int depth, int vec, int dir, int wide, uint64_t units);
/* the shape to launch with; returns a probe id (>= 0) when this launch is timed, in
 * which case the caller launches and then calls yk_tune_end on the same stream */
int yk_tune_begin(uint64_t key, int family, uint64_t units, void *stream, yk_tune_cfg * cfg);
void yk_tune_end(int probe, void *stream);
void yk_tune_reset(void);

/* Request classes of the persistent server (family YK_TUNE_SERVER): a candidate is the
 * largest work item in KiB (units_per_thread) and the least number of items a request
 * is cut into (ctas_per_sm); {0, 0} is the server's own setting.  Samples are GPU
 * durations of requests that ran alone, reported by the caller, not event timings.
 * yk_tune_server_cfg: 1 and the decision when the class is decided, else 0 and the
 * default; yk_tune_server_next: the candidate to time next (its index), or -1 when the
 * class is decided or cannot be tuned; yk_tune_server_sample records one sample. */
int yk_tune_server_cfg(uint64_t key, yk_tune_cfg * cfg);
int yk_tune_server_next(uint64_t key, yk_tune_cfg * cfg);
void yk_tune_server_sample(uint64_t key, int cand, double ns);
/* launches smaller than this are never timed */
uint64_t yk_tune_min_units(void);

#endif
