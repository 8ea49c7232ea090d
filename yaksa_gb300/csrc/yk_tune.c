/*
 * yk_tune.c -- online autotuner for the launch shape of the byte-moving kernels.
 *
 * The REPLACE kernels (regular nests, generic descriptors, batches) can run with one
 * work unit per thread over many CTAs, or four units per thread in a grid-stride loop
 * over fewer, and the best grid size depends on the descriptor's shape and the request
 * size.  Rather than fixing one rule, each shape class (kernel family, nesting depth,
 * vector width, direction, log2 of the units) times a few candidate shapes on its first
 * real launches: CUDA events around the launch, read back later without waiting
 * (cudaEventQuery at the next tuning decision).  After every candidate has a few
 * samples the class keeps the fastest.  All candidates run the same kernel over the
 * same units, so results do not depend on which one runs.  Launches inside a stream
 * capture, small launches and YAKSA_GB300_AUTOTUNE=0 use the decided (or default)
 * shape without timing.  No reference counterpart: the reference fixes its launch
 * shape (src/backend/cuda/pup/yaksuri_cudai_pup.c:20-48).
 *
 * Families: the REPLACE byte/regular kernels (units per thread x CTAs per SM, and the
 * TMA or one-element-per-thread forms where they exist), batches, and the grid cap of
 * the hindexed, typed-operator and sorted-block kernels.
 *
 * Decisions persist when YAKSA_GB300_TUNE_FILE names a file: each decided class is
 * appended as one line "<device> <class key> <units per thread> <CTAs per SM> <variant>",
 * the device being the GPU's name and SM count, and a later process on the same kind of
 * GPU starts with those classes decided (no timed launches for them).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <cuda_runtime.h>
#include "yk_internal.h"
#include "yk_tune.h"

#define YK_TUNE_SLOTS 512
#define YK_TUNE_PROBES 64
#define YK_TUNE_REPS 4
#define YK_TUNE_MARGIN 0.95f    /* a candidate replaces the default only if 5% faster */
#define YK_TUNE_MIN_UNITS (1u << 15)

/* candidate shapes per family: units per thread, CTAs per SM (0 = default) */
/* candidate shapes per family: units per thread, CTAs per SM; the first is the default
 * rule (units per thread by size, 64 or 8 CTAs per SM) */
static const yk_tune_cfg cand_single[] = { {0, 0, 0}, {1, 64, 0}, {4, 8, 0}, {4, 16, 0}, {1, 16, 0} };
static const yk_tune_cfg cand_batch_regular[] = { {1, 0, 0}, {1, 8, 0}, {1, 4, 0} };
static const yk_tune_cfg cand_batch[] = { {0, 0, 0}, {1, 64, 0}, {4, 8, 0}, {4, 16, 0} };
/* the same launches when a TMA form exists (yk_tma.cu): two residencies of it compete */
static const yk_tune_cfg cand_single_tma[] = { {0, 0, 0}, {1, 64, 0}, {4, 8, 0}, {4, 16, 0},
    {1, 16, 0}, {0, 4, YK_VARIANT_TMA}, {0, 8, YK_VARIANT_TMA} };
static const yk_tune_cfg cand_runs_tma[] = { {0, 0, YK_VARIANT_RUNS}, {0, 4, YK_VARIANT_TMA},
    {0, 8, YK_VARIANT_TMA} };
/* the hindexed shuffle-search kernel: its shapes (units per lane and residency, see
 * yk_launch_hidx32_shape) at one wave, and the default shape at two */
static const yk_tune_cfg cand_hidx[] = { {0, 0, 0}, {0, 8, 0}, {4, 0, 0}, {2, 0, 0} };
/* hindexed unpacks: also sixteen units per lane, and the bulk-staged form */
static const yk_tune_cfg cand_hidx_unpack[] = { {0, 0, 0}, {0, 8, 0}, {4, 0, 0}, {16, 0, 0},
    {0, 4, YK_VARIANT_BULK} };
/* the typed operator kernel and the sorted-block kernels (default 16 CTAs per SM) */
static const yk_tune_cfg cand_grid16[] = { {0, 0, 0}, {0, 8, 0}, {0, 32, 0} };
/* the persistent server's cut of a request into work items: {largest item in KiB, least
 * number of items} ({0, 0}: the server's own setting, 256 KiB and 128 by default) */
static const yk_tune_cfg cand_server[] = { {0, 0, 0}, {1024, 128, 0}, {64, 128, 0}, {256, 32, 0},
    {256, 512, 0} };

#define YK_TUNE_PRELOAD 1024

typedef struct {
    uint64_t key;               /* 0: empty */
    const yk_tune_cfg *cand;
    int ncand;
    float fastest[8];           /* best sample per candidate (ms) */
    int done[8], issued[8];     /* at most 8 candidates per family */
    int best;                   /* -1 while timing */
} slot_t;

typedef struct {
    cudaEvent_t e0, e1;
    int slot, cand;
    int busy;                   /* taken by a launch */
    int armed;                  /* e1 recorded after that launch: may be read */
} probe_t;

typedef struct {
    uint64_t key;
    yk_tune_cfg cfg;
} preload_t;

static struct {
    pthread_mutex_t mu;
    int init, enabled;
    slot_t slots[YK_TUNE_SLOTS];
    probe_t probes[YK_TUNE_PROBES];
    uint64_t nprobes;
    char file[512];             /* decisions file (empty: not persisted) */
    char device[288];           /* "<name>/<SMs>" with spaces as '_' */
    preload_t pre[YK_TUNE_PRELOAD];
    int npre;
    uint32_t loaded;            /* classes decided from the file */
} T = { .mu = PTHREAD_MUTEX_INITIALIZER };

static const yk_tune_cfg *family_cands(int family, int *n)
{
#define YK_C(a) (*n = (int) (sizeof(a) / sizeof(a[0])), a)
    switch (family) {
        case YK_TUNE_SINGLE: return YK_C(cand_single);
        case YK_TUNE_SINGLE_TMA: return YK_C(cand_single_tma);
        case YK_TUNE_RUNS_TMA: return YK_C(cand_runs_tma);
        case YK_TUNE_BATCH_REGULAR: return YK_C(cand_batch_regular);
        case YK_TUNE_HIDX: return YK_C(cand_hidx);
        case YK_TUNE_HIDX_UNPACK: return YK_C(cand_hidx_unpack);
        case YK_TUNE_TYPED: case YK_TUNE_OWNER: return YK_C(cand_grid16);
        case YK_TUNE_SERVER: return YK_C(cand_server);
        default: return YK_C(cand_batch);
    }
#undef YK_C
}

static void persist_locked(const slot_t * s)
{
    if (!T.file[0])
        return;
    FILE *f = fopen(T.file, "a");
    if (!f)
        return;
    const yk_tune_cfg *c = &s->cand[s->best];
    fprintf(f, "%s %llx %d %d %d\n", T.device, (unsigned long long) s->key, c->units_per_thread,
            c->ctas_per_sm, c->variant);
    fclose(f);
}

static void load_locked(void)
{
    const char *fn = getenv("YAKSA_GB300_TUNE_FILE");
    if (!fn || !fn[0] || strlen(fn) >= sizeof(T.file))
        return;
    strcpy(T.file, fn);
    int dev = 0;
    struct cudaDeviceProp pr;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&pr, dev) != cudaSuccess) {
        cudaGetLastError();
        T.file[0] = 0;
        return;
    }
    snprintf(T.device, sizeof(T.device), "%s/%d", pr.name, pr.multiProcessorCount);
    for (char *c = T.device; *c; c++)
        if (*c == ' ')
            *c = '_';
    FILE *f = fopen(T.file, "r");
    if (!f)
        return;
    char line[640], devname[288];
    unsigned long long key;
    int u, c, v;
    while (fgets(line, sizeof(line), f) && T.npre < YK_TUNE_PRELOAD)
        if (sscanf(line, "%287s %llx %d %d %d", devname, &key, &u, &c, &v) == 5 &&
            !strcmp(devname, T.device) && key) {
            T.pre[T.npre].key = key;
            T.pre[T.npre].cfg.units_per_thread = u;
            T.pre[T.npre].cfg.ctas_per_sm = c;
            T.pre[T.npre].cfg.variant = v;
            T.npre++;
        }
    fclose(f);
}

static int log2u(uint64_t v)
{
    int l = 0;
    while (v >>= 1)
        l++;
    return l;
}

uint64_t yk_tune_key(int family, int depth, int vec, int dir, int wide, uint64_t units)
{
    /* nonzero by construction: family is 1..10 */
    return ((uint64_t) family << 32) | ((uint64_t) (depth + 1) << 24) |
        ((uint64_t) vec << 16) | ((uint64_t) dir << 12) | ((uint64_t) wide << 8) |
        (uint64_t) log2u(units);
}

/* one timing sample of candidate c of slot s (ms); decides the class once every
 * candidate has YK_TUNE_REPS samples */
static void record_locked(slot_t * s, int c, float ms)
{
    if (s->done[c] == 0 || ms < s->fastest[c])
        s->fastest[c] = ms;
    s->done[c]++;
    int all = 1;
    for (int k = 0; k < s->ncand; k++)
        all &= s->done[k] >= YK_TUNE_REPS;
    if (all && s->best < 0) {
        /* candidate 0 is the default shape: keep it unless another one's fastest sample
         * beats it clearly (samples are noisy and taken with warm caches) */
        int b = 0;
        for (int k = 1; k < s->ncand; k++)
            if (s->fastest[k] < YK_TUNE_MARGIN * s->fastest[0] && s->fastest[k] < s->fastest[b])
                b = k;
        s->best = b;
        persist_locked(s);
    }
}

static void drain_locked(void)
{
    for (int i = 0; i < YK_TUNE_PROBES; i++) {
        probe_t *p = &T.probes[i];
        if (!p->busy || !p->armed)
            continue;
        cudaError_t e = cudaEventQuery(p->e1);
        if (e == cudaErrorNotReady)
            continue;
        float ms = 0;
        if (e == cudaSuccess && cudaEventElapsedTime(&ms, p->e0, p->e1) == cudaSuccess) {
            record_locked(&T.slots[p->slot], p->cand, ms);
        } else {
            cudaGetLastError();
        }
        p->busy = p->armed = 0;
    }
}

static void init_locked(void)
{
    if (T.init)
        return;
    const char *e = getenv("YAKSA_GB300_AUTOTUNE");
    T.enabled = !(e && e[0] == '0');
    T.init = 1;
    if (T.enabled)
        load_locked();
}

static slot_t *slot_locked(uint64_t key, int family)
{
    uint64_t h = key * 0x9e3779b97f4a7c15ull;
    for (int k = 0; k < YK_TUNE_SLOTS; k++) {
        slot_t *s = &T.slots[(h + (uint64_t) k) % YK_TUNE_SLOTS];
        if (s->key == key)
            return s;
        if (s->key == 0) {
            memset(s, 0, sizeof(*s));
            s->key = key;
            s->best = -1;
            s->cand = family_cands(family, &s->ncand);
            /* a decision from the file, if it names one of this family's candidates */
            for (int i = T.npre - 1; i >= 0 && s->best < 0; i--)
                if (T.pre[i].key == key)
                    for (int c = 0; c < s->ncand; c++)
                        if (!memcmp(&s->cand[c], &T.pre[i].cfg, sizeof(yk_tune_cfg))) {
                            s->best = c;
                            T.loaded++;
                            break;
                        }
            return s;
        }
    }
    return NULL;        /* table full: default shapes */
}

int yk_tune_begin(uint64_t key, int family, uint64_t units, void *stream, yk_tune_cfg * cfg)
{
    cudaStream_t st = (cudaStream_t) stream;
    int nc;
    *cfg = family_cands(family, &nc)[0];        /* the default shape */
    pthread_mutex_lock(&T.mu);
    init_locked();
    if (!T.enabled || units < YK_TUNE_MIN_UNITS) {
        pthread_mutex_unlock(&T.mu);
        return -1;
    }
    /* inside a stream capture: the decided shape (or the default), with no event work */
    enum cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    const int capturing = cudaStreamIsCapturing(st, &cs) != cudaSuccess ||
        cs != cudaStreamCaptureStatusNone;
    if (capturing)
        cudaGetLastError();
    else
        drain_locked();
    slot_t *s = slot_locked(key, family);
    if (!s) {
        pthread_mutex_unlock(&T.mu);
        return -1;
    }
    if (s->best >= 0) {
        *cfg = s->cand[s->best];
        pthread_mutex_unlock(&T.mu);
        return -1;
    }
    if (capturing) {
        pthread_mutex_unlock(&T.mu);
        return -1;      /* no timing inside a capture: default shape */
    }
    /* the candidate with the fewest samples issued */
    int c = 0;
    for (int k = 1; k < s->ncand; k++)
        if (s->issued[k] < s->issued[c])
            c = k;
    int pi = -1;
    for (int i = 0; i < YK_TUNE_PROBES && pi < 0; i++)
        if (!T.probes[i].busy)
            pi = i;
    if (pi < 0) {
        pthread_mutex_unlock(&T.mu);
        return -1;      /* every probe in flight: launch untimed */
    }
    probe_t *p = &T.probes[pi];
    if (!p->e0 && (cudaEventCreate(&p->e0) != cudaSuccess ||
                   cudaEventCreate(&p->e1) != cudaSuccess)) {
        cudaGetLastError();
        pthread_mutex_unlock(&T.mu);
        return -1;
    }
    if (cudaEventRecord(p->e0, st) != cudaSuccess) {
        cudaGetLastError();
        pthread_mutex_unlock(&T.mu);
        return -1;
    }
    p->busy = 1;
    p->armed = 0;
    p->slot = (int) (s - T.slots);
    p->cand = c;
    s->issued[c]++;
    T.nprobes++;
    *cfg = s->cand[c];
    pthread_mutex_unlock(&T.mu);
    return pi;
}

void yk_tune_end(int probe, void *stream)
{
    if (probe < 0)
        return;
    pthread_mutex_lock(&T.mu);
    if (cudaEventRecord(T.probes[probe].e1, (cudaStream_t) stream) != cudaSuccess) {
        cudaGetLastError();
        T.probes[probe].busy = 0;
    } else {
        T.probes[probe].armed = 1;
    }
    pthread_mutex_unlock(&T.mu);
}

int yk_tune_server_cfg(uint64_t key, yk_tune_cfg * cfg)
{
    int n, decided = 0;
    *cfg = family_cands(YK_TUNE_SERVER, &n)[0];
    pthread_mutex_lock(&T.mu);
    init_locked();
    if (T.enabled) {
        slot_t *s = slot_locked(key, YK_TUNE_SERVER);
        if (s && s->best >= 0) {
            *cfg = s->cand[s->best];
            decided = 1;
        }
    }
    pthread_mutex_unlock(&T.mu);
    return decided;
}

int yk_tune_server_next(uint64_t key, yk_tune_cfg * cfg)
{
    int n, c = -1;
    *cfg = family_cands(YK_TUNE_SERVER, &n)[0];
    pthread_mutex_lock(&T.mu);
    init_locked();
    slot_t *s = T.enabled ? slot_locked(key, YK_TUNE_SERVER) : NULL;
    if (s && s->best < 0) {
        c = 0;
        for (int k = 1; k < s->ncand; k++)
            if (s->issued[k] < s->issued[c])
                c = k;
        s->issued[c]++;
        *cfg = s->cand[c];
    } else if (s) {
        *cfg = s->cand[s->best];
    }
    pthread_mutex_unlock(&T.mu);
    return c;
}

void yk_tune_server_sample(uint64_t key, int cand, double ns)
{
    pthread_mutex_lock(&T.mu);
    init_locked();
    slot_t *s = T.enabled ? slot_locked(key, YK_TUNE_SERVER) : NULL;
    if (s && cand >= 0 && cand < s->ncand && ns > 0)
        record_locked(s, cand, (float) (ns * 1e-6));
    pthread_mutex_unlock(&T.mu);
}

uint64_t yk_tune_min_units(void)
{
    return YK_TUNE_MIN_UNITS;
}

void yk_tune_reset(void)
{
    pthread_mutex_lock(&T.mu);
    for (int i = 0; i < YK_TUNE_PROBES; i++) {
        if (T.probes[i].e0) {
            cudaEventDestroy(T.probes[i].e0);
            cudaEventDestroy(T.probes[i].e1);
        }
    }
    memset(T.probes, 0, sizeof(T.probes));
    memset(T.slots, 0, sizeof(T.slots));
    T.nprobes = 0;
    T.init = 0;
    T.npre = 0;
    T.loaded = 0;
    T.file[0] = 0;
    pthread_mutex_unlock(&T.mu);
}

int yaksa_gb300_autotune_stats(uint32_t * classes, uint32_t * decided, uint64_t * probes)
{
    pthread_mutex_lock(&T.mu);
    drain_locked();
    uint32_t n = 0, d = 0;
    for (int i = 0; i < YK_TUNE_SLOTS; i++)
        if (T.slots[i].key) {
            n++;
            d += T.slots[i].best >= 0;
        }
    *classes = n;
    *decided = d;
    *probes = T.nprobes;
    pthread_mutex_unlock(&T.mu);
    return YAKSA_SUCCESS;
}
