/*
 * oracle_pool.c -- a persistent pool of host threads that runs the oracle's
 * yaksa_pack / yaksa_unpack over parts of a packed range.  TEST INFRASTRUCTURE ONLY:
 * the CPU baseline of the bench times the oracle with it on every host core.
 *
 * The reference's seq backend is sequential per call and its library is thread-safe
 * (src/frontend/init/yaksa_init.c:144, src/util/yaksu_atomics.h), so a caller that
 * wants every core splits the packed range with the API's own offset and size
 * arguments (inoffset/max_pack_bytes, src/frontend/pup/yaksi_ipack.c:40-101) and
 * issues one call per part.  The pool does exactly that.  Its threads are created
 * once and wait on a barrier between jobs, so starting a job costs two barrier
 * crossings and no thread creation.
 *
 * Parts end on multiples of `granule` (a builtin boundary of the type), so each part
 * is a whole-builtin request and the parts tile the range.
 */
#define _POSIX_C_SOURCE 200809L      /* barriers and clock_gettime under -std=c11 */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "yaksa.h"

typedef struct {
    int dir;                    /* 0 pack, 1 unpack */
    const void *typed_in;       /* pack: typed source */
    void *typed_out;            /* unpack: typed target */
    uintptr_t count;
    yaksa_type_t type;
    void *packed;
    uintptr_t total;            /* packed bytes of the whole request */
    uintptr_t granule;
    yaksa_op_t op;
} oracle_job;

static struct {
    int n;                      /* threads, the caller included */
    pthread_t *tid;
    pthread_barrier_t start, done;
    const oracle_job *jobs;
    int njobs;
    int stop;
    int err;
} P;

static void run_part(int rank)
{
    for (int j = 0; j < P.njobs; j++) {
        const oracle_job *b = &P.jobs[j];
        uintptr_t g = b->granule ? b->granule : 1;
        uintptr_t units = b->total / g;
        uintptr_t u0 = units * (uintptr_t) rank / (uintptr_t) P.n;
        uintptr_t u1 = units * (uintptr_t) (rank + 1) / (uintptr_t) P.n;
        uintptr_t off = u0 * g, len = (u1 - u0) * g;
        if (rank == P.n - 1)
            len = b->total - off;       /* the tail below one granule goes to the last part */
        if (!len)
            continue;
        uintptr_t actual = 0;
        int rc = b->dir == 0 ?
            yaksa_pack(b->typed_in, b->count, b->type, off, (char *) b->packed + off, len, &actual,
                       NULL, b->op) :
            yaksa_unpack((const char *) b->packed + off, len, b->typed_out, b->count, b->type, off,
                         &actual, NULL, b->op);
        if (rc || actual != len)
            __atomic_store_n(&P.err, 1, __ATOMIC_RELAXED);
    }
}

static void *worker(void *arg)
{
    int rank = (int) (intptr_t) arg;
    for (;;) {
        pthread_barrier_wait(&P.start);
        if (P.stop)
            return NULL;
        run_part(rank);
        pthread_barrier_wait(&P.done);
    }
}

/* nthreads >= 1 host threads (the caller is one of them) */
int oracle_pool_start(int nthreads)
{
    if (P.n)
        return 1;
    P.n = nthreads < 1 ? 1 : nthreads;
    P.stop = 0;
    pthread_barrier_init(&P.start, NULL, (unsigned) P.n);
    pthread_barrier_init(&P.done, NULL, (unsigned) P.n);
    P.tid = calloc((size_t) P.n, sizeof(pthread_t));
    if (!P.tid)
        return 1;
    for (int i = 1; i < P.n; i++)
        if (pthread_create(&P.tid[i], NULL, worker, (void *) (intptr_t) i))
            return 1;
    return 0;
}

/* run every job on all threads, `reps` times; returns seconds per repetition (wall
 * clock of the caller), or a negative value when a part failed */
double oracle_pool_run(const oracle_job *jobs, int njobs, int reps)
{
    struct timespec t0, t1;
    P.jobs = jobs;
    P.njobs = njobs;
    P.err = 0;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int r = 0; r < reps; r++) {
        pthread_barrier_wait(&P.start);
        run_part(0);
        pthread_barrier_wait(&P.done);
    }
    clock_gettime(CLOCK_MONOTONIC, &t1);
    double s = (double) (t1.tv_sec - t0.tv_sec) + 1e-9 * (double) (t1.tv_nsec - t0.tv_nsec);
    return P.err ? -1.0 : s / (reps > 0 ? reps : 1);
}

void oracle_pool_stop(void)
{
    if (!P.n)
        return;
    P.stop = 1;
    pthread_barrier_wait(&P.start);
    for (int i = 1; i < P.n; i++)
        pthread_join(P.tid[i], NULL);
    pthread_barrier_destroy(&P.start);
    pthread_barrier_destroy(&P.done);
    free(P.tid);
    memset(&P, 0, sizeof(P));
}
