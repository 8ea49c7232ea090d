#!/usr/bin/env python3
"""Benchmark of the GB300 pack/unpack engine: every configuration of the metric, on one GPU.

Headline ("halo3d", the 3-level nested halo faces): a 512^3 float32 grid (uniform
[-1, 1) from a seed) and its six depth-2 halo faces described as subarray types (x-faces
{512,512,2}: 8-byte runs at a 2 KiB row stride; y-faces {512,2,512}: 4 KiB runs per
plane; z-faces {2,512,512}: one 2 MiB run).  One step = pack every face into its own
contiguous device buffer, then unpack every face with REPLACE into a second grid, on the
plain path: one yaksa_pack_stream / yaksa_unpack_stream call per face, each face on its
own stream (as a halo exchange posts one message per neighbour), the twelve calls
captured once into a CUDA graph and replayed per step.  Reported per face as well.

The same run measures, each as its own record with a full-size byte comparison against
the oracle and the oracle's own time on the host cores:
  hvector     4-column block of a 1024x16 double matrix (hvector 1024 x 4 doubles, stride 128 B)
  hindexed    int32, 2^20 lognormal blocks at shuffled non-overlapping places in 1 GiB
  struct      {int64, float x3} resized to 32 B, count 8M
  reduce_*    indexed_block 2^22 x 8 at sorted random offsets over 256 MiB targets, unpacked
              with SUM (double), MAX (int64), BXOR (uint32), PROD (complex float)
and the mixed request stream (10,000 requests, Poisson 50k/s) through the plain
per-request path and the persistent-kernel server, p50/p99 latency and capacity.

Metric: packed GB/s (bytes packed + bytes unpacked per second), next to the HBM
roofline: REPLACE moves 2 bytes per packed byte (read strided + write contiguous, or the
mirror), an operator 3 (read packed, read target, write target).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--no-cpu] [--no-stream] [--no-suite] [--cpu-seconds S]
    python bench.py --suite out.jsonl [--suite-only hindexed,struct,...] [--suite-scale K]
    python bench.py --stream out.json [--stream-requests R] [--stream-families halo,struct,...]
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = int(os.environ.get("YK_BENCH_N", "512"))   # grid edge; smaller only for ncu captures
ORACLE_LIB = os.path.join(ROOT, "oracle", "_ref", "liboracle_yaksa.so")
PROFILES = os.path.join(ROOT, "profiles")


def face_specs(n):
    """(name, subsizes, starts) of the six depth-2 faces, C order over sizes {n, n, n}."""
    return [("x-", [n, n, 2], [0, 0, 0]), ("x+", [n, n, 2], [0, 0, n - 2]),
            ("y-", [n, 2, n], [0, 0, 0]), ("y+", [n, 2, n], [0, n - 2, 0]),
            ("z-", [2, n, n], [0, 0, 0]), ("z+", [2, n, n], [n - 2, 0, 0])]


FACES = face_specs(N)
L2_FLUSH_BYTES = 512 << 20
TUNE_CALLS = 28     # calls per shape class before the autotuner has chosen (5 shapes x 4 + slack)
METRIC = "pack+unpack GB/s vs HBM peak (bit-exact); batched p50/p99 us vs plain path"
WORKLOAD = (f"halo3d: {N}^3 float32 grid, 6 depth-2 subarray faces ({2 * N * N * 4 >> 20} MiB "
            "packed each), pack + unpack REPLACE per step, plain path (one call per face)")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def ensure_oracle():
    if not os.path.exists(ORACLE_LIB):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    return ORACLE_LIB


def ncu_traffic(name):
    """dram__bytes_read.sum + dram__bytes_write.sum per launch, from the committed ncu
    summary of a kernel and workload (the `traffic:` lines of profiles/<name>.md), or
    None when no capture exists."""
    p = os.path.join(PROFILES, name + ".md")
    out = {}
    if os.path.exists(p):
        for line in open(p):
            if line.startswith("traffic:"):
                k, v = line[len("traffic:"):].split("=")
                out[k.strip()] = float(v)
    return out


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path):
        self.path = path
        self.proc = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9 or not parts[1].isdigit():
                continue
            sm.append(int(parts[1]))
            smax = int(parts[2])
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


class ColdL2:
    """Between timed launches: write a buffer larger than L2 (the flush), then read a
    second one, so that the timed launch starts with a cold L2 that holds no dirty lines
    (otherwise the flush's own write-backs land inside the timed kernel)."""

    def __init__(self, torch):
        self.w = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        self.r = torch.zeros(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.w.zero_()
        self.sink = self.r.sum()


def event_time(torch, fn, reps, flush, stat=statistics.median):
    """CUDA-event time of fn() on torch's current stream, a cold L2 before each rep."""
    ts = []
    for _ in range(reps):
        flush()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    return stat(ts)


def cpu_model():
    """The host CPU's model name (lscpu), for the baseline records."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


# ---------------------------------------------------------------------------
# the oracle on the host cores: one thread, or every core through its thread pool
# ---------------------------------------------------------------------------

class OracleJob(ctypes.Structure):
    """oracle_job (oracle/oracle_pool.c)"""
    _fields_ = [("dir", ctypes.c_int), ("typed_in", ctypes.c_void_p), ("typed_out", ctypes.c_void_p),
                ("count", ctypes.c_size_t), ("type", ctypes.c_uint64), ("packed", ctypes.c_void_p),
                ("total", ctypes.c_size_t), ("granule", ctypes.c_size_t), ("op", ctypes.c_uint64)]


class OraclePool:
    """The oracle's persistent thread pool: each job's packed range split on builtin
    boundaries over `threads` host threads created once (oracle/oracle_pool.c)."""

    def __init__(self, oracle, threads):
        self.lib = oracle.lib
        self.lib.oracle_pool_start.argtypes = [ctypes.c_int]
        self.lib.oracle_pool_run.argtypes = [ctypes.POINTER(OracleJob), ctypes.c_int, ctypes.c_int]
        self.lib.oracle_pool_run.restype = ctypes.c_double
        self.threads = threads
        assert self.lib.oracle_pool_start(threads) == 0, "oracle pool start failed"

    def run(self, jobs, reps=1):
        arr = (OracleJob * len(jobs))(*jobs)
        s = self.lib.oracle_pool_run(arr, len(jobs), reps)
        assert s >= 0, "an oracle call of the pool failed"
        return s

    def stop(self):
        self.lib.oracle_pool_stop()


def halo_jobs(faces, src, dst, bufs, P):
    """pack every face (granule 4: float), then unpack every face; a thread's unpack part
    reads the packed bytes its own pack part wrote"""
    jobs = [OracleJob(0, src.ctypes.data, None, 1, t, b.ctypes.data, P, 4, 10)
            for (_, t), b in zip(faces, bufs)]
    jobs += [OracleJob(1, None, dst.ctypes.data, 1, t, b.ctypes.data, P, 4, 10)
             for (_, t), b in zip(faces, bufs)]
    return jobs


def make_faces(y, yk, n=N):
    return [(name, y.type_create_subarray([n, n, n], sub, st, yk.SUBARRAY_ORDER_C, yk.TYPE_FLOAT))
            for name, sub, st in face_specs(n)]


def faces_equal_np(np, src, dst, n=N):
    s3, d3 = src.reshape(n, n, n), dst.reshape(n, n, n)
    return all(np.array_equal(s3[sl], d3[sl]) for sl in
               ((slice(None), slice(None), slice(0, 2)), (slice(None), slice(None), slice(n - 2, n)),
                (slice(None), slice(0, 2)), (slice(None), slice(n - 2, n)), (slice(0, 2),),
                (slice(n - 2, n),)))


def cpu_halo(seconds, threads):
    """The oracle (CPU restatement of the reference's seq path) over the halo step on the
    host cores; threads > 1 runs through the oracle's persistent pool."""
    import numpy as np
    import yaksa_gb300 as yk
    o = yk.Yaksa(ensure_oracle())
    o.init()
    faces = make_faces(o, yk)
    rng = np.random.default_rng(1)
    src = rng.uniform(-1, 1, N * N * N).astype(np.float32)
    dst = np.zeros_like(src)
    P = 2 * N * N * 4
    bufs = [np.zeros(P // 4, dtype=np.float32) for _ in faces]
    pool = OraclePool(o, threads)
    jobs = halo_jobs(faces, src, dst, bufs, P)
    one = pool.run(jobs, 1)     # warm
    reps = max(1, int(seconds / max(one, 1e-4)))
    t = pool.run(jobs, reps)
    pool.stop()
    ok = faces_equal_np(np, src, dst)
    for _, tt in faces:
        o.type_free(tt)
    o.finalize()
    moved = 2 * P * len(faces)
    return {"value": moved / t / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "cpu": cpu_model(),
            "sample": f"{reps} steps of the 6-face pack+unpack on the host (host buffers, "
                      f"{threads} thread{'s' if threads > 1 else ''}), {reps * t:.2f} s",
            "ok": ok, "s_per_step": t}


def run_reference(args):
    """--impl reference: the CPU implementation of the path (the oracle, restated from the
    reference's seq backend) on every host core, through its persistent thread pool."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    seconds = max(2.0, min(30.0, 1.0 * args.steps))
    b = cpu_halo(seconds, threads)
    step_bytes = 2 * (2 * N * N * 4) * 6      # six 2 MiB faces, packed and unpacked
    line = {"impl": "reference", "metric": METRIC, "value": b["value"], "unit": "GB/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_bytes / (b["value"] * 1e9) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "bit_exact": bool(b["ok"]),
            "config": {"workload": WORKLOAD, "parallelism": f"host threads x{threads}",
                       "l2": "host caches"},
            "cpu_baseline": {"value": b["value"], "unit": "GB/s", "cores": threads, "kind": "port",
                             "cpu": b["cpu"], "sample": b["sample"], "faces_equal": bool(b["ok"])},
            "e2e": {"value": b["value"], "unit": "GB/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# the other configurations: one record per (config, direction) with a full-size
# byte comparison against the oracle and the oracle's own time on the host
# ---------------------------------------------------------------------------

def suite_types(y, yk, np, rng_seed=7, scale=1):
    """Seeded synthetic inputs with the shapes and distributions of each config (scale > 1
    divides the block and element counts, for profiler captures of the same kernels)."""
    rng = np.random.default_rng(rng_seed)
    out = {}
    # hvector of double: 4-column block of a 1024x16 row-major matrix
    out["hvector"] = dict(mk=lambda L: L.type_create_hvector(1024, 4, 128, yk.TYPE_DOUBLE),
                          base="double", count=1, extent=1024 * 16 * 8, gran=8)
    # single halo faces of the 512^3 float grid, one per orientation: the default run
    # reports every face in its halo section, so these run only when named (profiling)
    for name, sub, st in face_specs(512)[0::2]:
        out["halo_" + name[0]] = dict(
            mk=lambda L, sub=sub, st=st: L.type_create_subarray([512, 512, 512], sub, st,
                                                                yk.SUBARRAY_ORDER_C, yk.TYPE_FLOAT),
            base="float", count=1, extent=512 ** 3 * 4, gran=4, named_only=True)
    # hindexed int32: 2^20 blocks, lognormal lengths (median 16, sigma 1, clipped 1..4096),
    # non-overlapping blocks in shuffled order with random gaps inside 1 GiB
    nb = (1 << 20) // scale
    blens = np.clip(np.round(np.exp(np.log(16) + rng.standard_normal(nb))), 1, 4096).astype(np.int64)
    slots_total = (1 << 30) // 4 // scale
    free = slots_total - int(blens.sum())
    gaps = rng.integers(0, 2 * (free // nb), nb)
    order = rng.permutation(nb)
    starts = np.cumsum(blens[order] + gaps) - blens[order]
    displs = np.empty(nb, dtype=np.int64)
    displs[order] = starts * 4
    assert int(starts[-1] + blens[order][-1]) <= slots_total

    def mk_hindexed(L):
        h = L.type_create_hindexed_arrays(nb, blens.ctypes.data, displs.ctypes.data, yk.TYPE_INT32_T)
        r = L.type_create_resized(h, 0, (1 << 30) // scale)
        L.type_free(h)
        return r
    out["hindexed"] = dict(mk=mk_hindexed, base="int32", count=1, extent=(1 << 30) // scale,
                           keep=(blens, displs), gran=4)

    def mk_struct(L):
        s = L.type_create_struct([1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT])
        r = L.type_create_resized(s, 0, 32)
        L.type_free(s)
        return r
    out["struct"] = dict(mk=mk_struct, base="float", count=(8 << 20) // scale,
                         extent=32 * (8 << 20) // scale, gran=20)
    # indexed_block: 2^22 blocks of 8 elements at sorted random element offsets
    for base, h, es, op in (("double", yk.TYPE_DOUBLE, 8, yk.OP_SUM),
                            ("int64", yk.TYPE_INT64_T, 8, yk.OP_MAX),
                            ("uint32", yk.TYPE_UINT32_T, 4, yk.OP_BXOR),
                            ("c_complex", yk.TYPE_C_COMPLEX, 8, yk.OP_PROD)):
        nel = (256 << 20) // es // scale
        nbk = (1 << 22) // scale
        offs = np.sort(rng.integers(0, nel - 8, nbk)).astype(np.int64)
        out[f"reduce_{base}"] = dict(
            mk=lambda L, offs=offs, h=h, nbk=nbk: L.type_create_indexed_block_array(nbk, 8, offs.ctypes.data, h),
            base=base, count=1, extent=(256 << 20) // scale, op=op, keep=(offs,), gran=0)
    # operators on strided targets that do not overlap (the runtime-operator typed
    # kernel): 4-element blocks at a stride of 6 elements, 64 MiB packed; double SUM, and
    # long double SUM and PROD in binary128 (hosts whose long double is binary128 only).
    # Named only, for profiling: they are not configs of the baseline.
    for name, h, es, base, op in (("strided_sum", yk.TYPE_DOUBLE, 8, "double", yk.OP_SUM),
                                  ("ldouble_sum", yk.TYPE_LONG_DOUBLE, 16, "ldouble", yk.OP_SUM),
                                  ("ldouble_prod", yk.TYPE_LONG_DOUBLE, 16, "ldouble", yk.OP_PROD)):
        nblk = (64 << 20) // (4 * es) // scale
        out[name] = dict(mk=lambda L, nblk=nblk, es=es, h=h: L.type_create_hvector(nblk, 4, 6 * es, h),
                         base=base, count=1, extent=nblk * 6 * es, op=op, gran=es, named_only=True)
    return out


def suite_fill(np, rng, base, nbytes):
    if base == "double":
        return rng.standard_normal(nbytes // 8).view(np.uint8)
    if base == "ldouble":
        # the host's long double (binary128 where these workloads run)
        return rng.standard_normal(nbytes // 16).astype(np.longdouble).view(np.uint8)
    if base == "int64":
        return rng.integers(-(1 << 63), (1 << 63) - 1, nbytes // 8, dtype=np.int64).view(np.uint8)
    if base == "uint32" or base == "int32":
        return rng.integers(0, 1 << 32, nbytes // 4, dtype=np.uint64).astype(np.uint32).view(np.uint8)
    if base == "c_complex":
        n = nbytes // 8
        r = np.exp(rng.uniform(np.log(0.9), np.log(1.1), n))
        a = rng.uniform(0, 2 * np.pi, n)
        return (r * np.exp(1j * a)).astype(np.complex64).view(np.uint8)
    return rng.uniform(-1, 1, nbytes // 4).astype(np.float32).view(np.uint8)


# the committed ncu summary (profiles/<name>.md) whose `traffic: <key> = bytes` line gives
# the DRAM bytes of a config's launch, and the full config's size over the captured case's
SUITE_PROFILE = {("hindexed", "pack"): ("yk_hidx32_kernel_hindexed", "pack", 2),
                 ("hindexed", "unpack"): ("yk_hidx32_kernel_hindexed_unpack", "unpack", 2),
                 ("struct", "pack"): ("yk_runs_pack_warp_kernel_struct", "pack", 1),
                 ("struct", "unpack"): ("yk_regular_kernel_struct", "unpack", 2),
                 ("reduce_double", "unpack"): ("yk_owner_lane_kernel_reduce", "double_sum_full", 1),
                 ("reduce_c_complex", "unpack"): ("yk_owner_chunk_kernel_reduce_complex", "complex_prod", 1),
                 ("reduce_uint32", "unpack"): ("yk_red_kernel_reduce", "uint32_bxor", 1),
                 ("reduce_int64", "unpack"): ("yk_red_kernel_reduce", "int64_max", 1)}


def run_suite(steps, only=None, scale=1, threads=None, log=None):
    """One record per (config, direction): CUDA-event kernel time (median, cold L2), the
    HBM roofline of algorithmic bytes, the full-size byte comparison with the oracle,
    and the oracle's time on 1 thread and on every host core."""
    import numpy as np
    import torch
    import yaksa_gb300 as yk
    y, o = yk.Yaksa(), yk.Yaksa(ensure_oracle())
    y.init()
    o.init()
    hbm, peak_kind = peaks()
    flush = ColdL2(torch)
    stream = torch.cuda.current_stream()
    sh = ctypes.c_void_p(stream.cuda_stream)
    shp = ctypes.addressof(sh)
    rng = np.random.default_rng(11)
    threads = threads or os.cpu_count() or 1
    pool = OraclePool(o, threads)
    lines = []
    for name, w in suite_types(y, yk, np, scale=scale).items():
        if (only and name not in only) or (not only and w.get("named_only")):
            continue
        tp, to = w["mk"](y), w["mk"](o)
        size = y.size(tp)
        count = w["count"]
        P = size * count
        typed_h = suite_fill(np, rng, w["base"], w["extent"])
        packed0 = suite_fill(np, rng, w["base"], P)
        typed_d = torch.from_numpy(typed_h).cuda()
        packed_d = torch.from_numpy(packed0).cuda()
        op = w.get("op", yk.OP_REPLACE)
        dirs = ["unpack"] if op != yk.OP_REPLACE else ["pack", "unpack"]
        for d in dirs:
            prof = SUITE_PROFILE.get((name, d))
            tr = ncu_traffic(prof[0]).get(prof[1]) if prof else None
            tr = tr * prof[2] / scale if tr else None
            def call():
                if d == "pack":
                    y.pack_stream(typed_d.data_ptr(), count, tp, 0, packed_d.data_ptr(), P, shp, op=op)
                else:
                    y.unpack_stream(packed_d.data_ptr(), P, typed_d.data_ptr(), count, tp, 0, shp, op=op)
            # correctness first, from fresh inputs, against the oracle on the host
            typed_d.copy_(torch.from_numpy(typed_h))
            packed_d.copy_(torch.from_numpy(packed0))
            call()
            torch.cuda.synchronize()
            th, ph = typed_h.copy(), packed0.copy()
            t0 = time.perf_counter()
            if d == "pack":
                o.pack(th.ctypes.data, count, to, 0, ph.ctypes.data, P, op=op)
            else:
                o.unpack(ph.ctypes.data, P, th.ctypes.data, count, to, 0, op=op)
            cpu_t = time.perf_counter() - t0
            exact = bool(np.array_equal(typed_d.cpu().numpy(), th) and
                         np.array_equal(packed_d.cpu().numpy(), ph))
            # every host core: the packed range split at multiples of the granule
            # (builtin boundaries) through the API's offset/max-bytes arguments, on the
            # oracle's persistent pool; not for overlapping targets, whose order only
            # one thread keeps
            cpu_nt, nt_exact = None, None
            if w["gran"]:
                th2, ph2 = typed_h.copy(), packed0.copy()
                job = (OracleJob(0, th2.ctypes.data, None, count, to, ph2.ctypes.data, P, w["gran"], op)
                       if d == "pack" else
                       OracleJob(1, None, th2.ctypes.data, count, to, ph2.ctypes.data, P, w["gran"], op))
                cpu_nt = pool.run([job], 1)
                nt_exact = bool(np.array_equal(th2, th) and np.array_equal(ph2, ph))
                del th2, ph2
            del th, ph
            # untimed calls while the launch-shape autotuner settles, then timing: fresh L2
            # each launch, CUDA events on the launching stream
            for _ in range(TUNE_CALLS):
                call()
            t = event_time(torch, call, max(3, steps), flush)
            alg = (2 if op == yk.OP_REPLACE else 3) * P
            line = {"workload": name, "direction": d, "op": int(op), "packed_bytes": P,
                    "time_us": t * 1e6, "packed_GBps": P / t / 1e9,
                    "roofline": {"bound": "hbm", "achieved": alg / t / 1e9, "peak": hbm, "unit": "GB/s",
                                 "frac": alg / t / 1e9 / hbm, "peak_source": peak_kind,
                                 "algorithmic_bytes": alg,
                                 "traffic": tr, "traffic_frac": tr / t / 1e9 / hbm if tr else None},
                    "bit_exact": exact,
                    "cpu_oracle": {"threads": 1, "s": cpu_t, "packed_GBps": P / cpu_t / 1e9},
                    "cpu_oracle_all_cores": ({"threads": threads, "s": cpu_nt, "packed_GBps": P / cpu_nt / 1e9,
                                              "same_bytes": nt_exact} if cpu_nt else
                                             {"note": "overlapping targets: one thread keeps the order"}),
                    "gpu_over_cpu_1thr": cpu_t / t}
            lines.append(line)
            if log:
                print(json.dumps(line), file=log, flush=True)
        y.type_free(tp)
        o.type_free(to)
        del typed_d, packed_d, typed_h, packed0
        torch.cuda.empty_cache()
    pool.stop()
    o.finalize()
    del flush
    torch.cuda.empty_cache()
    return lines


# ---------------------------------------------------------------------------
# the mixed request stream: plain one-launch-per-request path vs the persistent server
# ---------------------------------------------------------------------------

STREAM_CLASSES = [256 << k for k in range(19)]          # packed sizes 256 B .. 64 MiB
STREAM_REDUCE = (("double", "TYPE_DOUBLE", 8, "OP_SUM"), ("int64", "TYPE_INT64_T", 8, "OP_MAX"),
                 ("uint32", "TYPE_UINT32_T", 4, "OP_BXOR"), ("c_complex", "TYPE_C_COMPLEX", 8, "OP_PROD"))


def stream_family_types(yk, np, seed):
    """(family, class) -> dict(mk, base, count, extent, op, dirs): one type per packed-size
    class for each type family of the plain configurations, packed size == class size
    (struct: the largest multiple of its 20-byte element)."""
    rng = np.random.default_rng(seed)
    out = {}
    for S in STREAM_CLASSES:
        # 4-column blocks of an (S/32) x 16 row-major double matrix
        out[("hvector", S)] = dict(mk=lambda L, S=S: L.type_create_hvector(S // 32, 4, 128, yk.TYPE_DOUBLE),
                                   base="double", count=1, extent=(S // 32) * 128, op=yk.OP_REPLACE)
        # x-face of a {Z, Y, 512} float grid, depth 2: 8-byte runs at a 2 KiB row stride
        Y = min(512, S // 8)
        Z = S // 8 // Y
        x0 = int(rng.choice([0, 510]))
        out[("halo", S)] = dict(mk=lambda L, Z=Z, Y=Y, x0=x0: L.type_create_subarray(
            [Z, Y, 512], [Z, Y, 2], [0, 0, x0], yk.SUBARRAY_ORDER_C, yk.TYPE_FLOAT),
            base="float", count=1, extent=Z * Y * 2048, op=yk.OP_REPLACE, xface=(Z, Y, x0))
        # hindexed int32: lognormal block lengths (median 16, sigma 1, clipped 1..4096),
        # non-overlapping blocks in shuffled order inside a resized extent of 4 S
        nel = S // 4
        draw = np.clip(np.round(np.exp(np.log(16) + rng.standard_normal(nel // 8 + 64))), 1, 4096)
        cum = np.cumsum(draw.astype(np.int64))
        nb = int(np.searchsorted(cum, nel)) + 1
        assert nb <= len(draw)
        blens = draw[:nb].astype(np.int64)
        blens[-1] -= int(cum[nb - 1]) - nel
        free = 4 * nel - nel
        gaps = rng.integers(0, 2 * (free // nb) + 1, nb)
        if int(gaps.sum()) > free:
            gaps = gaps * free // int(gaps.sum())
        order = rng.permutation(nb)
        starts = np.cumsum(blens[order] + gaps) - blens[order]
        assert int(starts[-1] + blens[order][-1]) <= 4 * nel
        displs = np.empty(nb, dtype=np.int64)
        displs[order] = starts * 4

        def mk_hind(L, nb=nb, blens=blens, displs=displs, S=S):
            h = L.type_create_hindexed_arrays(nb, blens.ctypes.data, displs.ctypes.data, yk.TYPE_INT32_T)
            r = L.type_create_resized(h, 0, 4 * S)
            L.type_free(h)
            return r
        out[("hindexed", S)] = dict(mk=mk_hind, base="int32", count=1, extent=4 * S, op=yk.OP_REPLACE,
                                    keep=(blens, displs))

        # {int64 x1, float x3} resized to 32 bytes
        def mk_struct(L):
            s = L.type_create_struct([1, 3], [0, 8], [yk.TYPE_INT64_T, yk.TYPE_FLOAT])
            r = L.type_create_resized(s, 0, 32)
            L.type_free(s)
            return r
        out[("struct", S)] = dict(mk=mk_struct, base="float", count=max(1, S // 20), extent=32 * max(1, S // 20),
                                  op=yk.OP_REPLACE)
        # indexed_block of 8-element blocks at sorted random offsets over a 4 S target,
        # unpacked with the config's reduction op
        for base, tname, es, opname in STREAM_REDUCE:
            nbk = max(1, S // (8 * es))
            tel = 4 * S // es
            offs = np.sort(rng.integers(0, tel - 8, nbk)).astype(np.int64)
            out[("reduce_" + base, S)] = dict(
                mk=lambda L, nbk=nbk, offs=offs, tname=tname: L.type_create_indexed_block_array(
                    nbk, 8, offs.ctypes.data, getattr(yk, tname)),
                base=base, count=1, extent=4 * S, op=getattr(yk, opname), keep=(offs,), unpack_only=True)
    return out


def dev_fill(torch, base, nbytes, gen):
    """Valid seeded values of `base` filling a new device buffer of nbytes."""
    n = (nbytes + 15) // 16 * 16
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    if base == "double":
        out.view(torch.float64).normal_(generator=gen)
    elif base == "float":
        out.view(torch.float32).uniform_(-1, 1, generator=gen)
    elif base == "c_complex":
        z = out.view(torch.float32).view(-1, 2)
        r = torch.exp(torch.empty(z.shape[0], device="cuda").uniform_(-0.10536, 0.09531, generator=gen))
        a = torch.empty(z.shape[0], device="cuda").uniform_(0, 6.283185307179586, generator=gen)
        z[:, 0] = r * torch.cos(a)
        z[:, 1] = r * torch.sin(a)
    else:
        out.random_(0, 256, generator=gen)
    return out


def run_stream(nreq=10000, rate=50e3, seed=5, check=True, log=None, floor=True, server_tune=True,
               families=None):
    """10,000 pack/unpack requests with Poisson arrivals at `rate` req/s: families drawn
    uniformly from hvector/halo/hindexed/struct/reduce, packed sizes log-uniform over
    19 power-of-two classes 256 B .. 64 MiB, 20% with the packed buffer in pinned host
    memory.  Each request uses its (family, class) arena: one typed buffer per family
    and one packed buffer per (family, class, host).  Checked requests own private
    buffers and are compared with the oracle after each path: 120 small ones and, for
    every size class, at least one whose typed footprint is at most 256 MiB (the halo
    family's footprint is 256 times its packed size, so its largest classes are checked
    through the other families).  `families` draws from a subset instead (the x-face
    floor is measured only with halo among them).  Returns a dict."""
    import numpy as np
    import torch
    import yaksa_gb300 as yk
    if check:
        ensure_oracle()
    y = yk.Yaksa()
    y.init()
    specs = stream_family_types(yk, np, seed)
    fams = list(families) if families else ["hvector", "halo", "hindexed", "struct", "reduce"]
    rng = np.random.default_rng(seed + 1)
    gen = torch.Generator(device="cuda").manual_seed(seed)
    fam_of = rng.integers(0, len(fams), nreq)
    cls_of = rng.integers(0, len(STREAM_CLASSES), nreq)
    red_of = rng.integers(0, len(STREAM_REDUCE), nreq)
    dir_of = rng.integers(0, 2, nreq)
    host_of = rng.random(nreq) < 0.2
    arrivals = np.cumsum(rng.exponential(1.0 / rate, nreq))
    arrivals -= arrivals[0]
    keys = []
    for i in range(nreq):
        f = fams[fam_of[i]]
        if f == "reduce":
            f = "reduce_" + STREAM_REDUCE[red_of[i]][0]
        keys.append((f, STREAM_CLASSES[cls_of[i]]))
    used = sorted(set(keys), key=lambda k: (k[0], k[1]))
    types = {k: specs[k]["mk"](y) for k in used}
    sizes = {k: y.size(types[k]) * specs[k]["count"] for k in used}
    # arenas: one typed buffer per family (largest extent), packed buffers per key
    arena = {}
    for k in used:
        arena[k[0]] = max(arena.get(k[0], 0), specs[k]["extent"])
    typed = {f: dev_fill(torch, specs[next(k for k in used if k[0] == f)]["base"], n + 256, gen)
             for f, n in arena.items()}
    packed_d = {k: dev_fill(torch, specs[k]["base"], sizes[k] + 256, gen) for k in used}
    packed_h = {}
    for i in range(nreq):
        if host_of[i] and keys[i] not in packed_h:
            packed_h[keys[i]] = packed_d[keys[i]].cpu().pin_memory()
    # checked requests: 120 small ones, and every size class
    chk = set()
    if check:
        small = [i for i in range(nreq) if keys[i][1] <= (256 << 10)]
        chk = set(rng.choice(small, size=min(len(small), 120), replace=False).tolist())
        for S in STREAM_CLASSES:
            cand = [i for i in range(nreq) if keys[i][1] == S and specs[keys[i]]["extent"] <= (256 << 20)]
            if cand:
                chk.update(rng.choice(cand, size=min(2, len(cand)), replace=False).tolist())
    priv = {}
    for i in sorted(chk):
        k = keys[i]
        t0 = typed[k[0]][:specs[k]["extent"] + 256].clone()
        p0 = packed_d[k][:sizes[k] + 256].clone()
        priv[i] = dict(t_init=t0.cpu().numpy(), p_init=p0.cpu().numpy(), t=t0,
                       p=(p0.cpu().pin_memory() if host_of[i] else p0))
    torch.cuda.synchronize()

    def make_ops():
        ops = (yk.PupOp * nreq)()
        for i in range(nreq):
            k = keys[i]
            sp = specs[k]
            if i in priv:
                tptr, pptr = priv[i]["t"].data_ptr(), priv[i]["p"].data_ptr()
            else:
                tptr = typed[k[0]].data_ptr()
                pptr = (packed_h[k] if host_of[i] else packed_d[k]).data_ptr()
            unpack = sp.get("unpack_only") or dir_of[i] == 1
            if unpack:
                ops[i] = yk.unpack_op(pptr, sizes[k], tptr, sp["count"], types[k], 0, op=sp["op"])
            else:
                ops[i] = yk.pack_op(tptr, sp["count"], types[k], 0, pptr, sizes[k], op=sp["op"])
        return ops

    def reset_private():
        for i, pv in priv.items():
            pv["t"].copy_(torch.from_numpy(pv["t_init"]))
            pv["p"].copy_(torch.from_numpy(pv["p_init"]))
        torch.cuda.synchronize()

    o = None
    expect = {}
    if check:
        o = yk.Yaksa(ORACLE_LIB)
        o.init()
        for i in sorted(priv):
            k = keys[i]
            sp = specs[k]
            to = sp["mk"](o)
            th, ph = priv[i]["t_init"].copy(), priv[i]["p_init"].copy()
            if sp.get("unpack_only") or dir_of[i] == 1:
                o.unpack(ph.ctypes.data, sizes[k], th.ctypes.data, sp["count"], to, 0, op=sp["op"])
            else:
                o.pack(th.ctypes.data, sp["count"], to, 0, ph.ctypes.data, sizes[k], op=sp["op"])
            o.type_free(to)
            expect[i] = (th, ph)

    def verify():
        bad = []
        for i, (th, ph) in expect.items():
            gt = priv[i]["t"].cpu().numpy()
            gp = priv[i]["p"].cpu().numpy()
            if not (np.array_equal(gt, th) and np.array_equal(gp, ph)):
                bad.append(i)
        return bad

    total = float(sum(sizes[k] for k in keys))
    checked_classes = sorted(set(keys[i][1] for i in chk))
    res = {"requests": nreq, "rate_per_s": rate, "packed_bytes": total,
           "checked_requests": len(chk), "checked_size_classes": len(checked_classes),
           "largest_checked_bytes": max(checked_classes) if checked_classes else 0,
           "families": fams, "size_classes": [STREAM_CLASSES[0], STREAM_CLASSES[-1]],
           "host_fraction": float(host_of.mean()),
           "arena_bytes": int(sum(arena.values()))}
    zero = np.zeros(nreq)
    srv = yk.Server(y, ring_requests=4096, budget_bytes=8 << 30)
    for mode in ("plain", "graphs", "server"):
        s = srv if mode == "server" else None
        graphs = mode == "graphs"
        if s is not None and server_tune:
            # calibration of the server's item cut per request class (untimed; each
            # class's requests run alone, once per candidate cut and repetition)
            t_tune = time.perf_counter()
            res["server_tuned_classes"] = srv.tune(make_ops())
            res["server_tune_s"] = time.perf_counter() - t_tune
        # warm: every descriptor built and uploaded once, outside the timed runs
        ops = make_ops()
        yk.serve_trace(y, ops, zero, server=s, graphs=graphs)
        torch.cuda.synchronize()
        reset_private()
        ops = make_ops()
        launches0 = y.stats()["launches"]
        g0 = y.graph_lane_stats()
        lat, mk = yk.serve_trace(y, ops, arrivals.tolist(), server=s, graphs=graphs)
        torch.cuda.synchronize()
        launches = y.stats()["launches"] - launches0
        g1 = y.graph_lane_stats()
        bad = verify() if check else []
        lat_us = np.array(lat) * 1e6
        # closed loop: everything arrives at once -> capacity
        ops2 = make_ops()
        _, mk2 = yk.serve_trace(y, ops2, zero, server=s, graphs=graphs)
        torch.cuda.synchronize()
        # latency by packed size: small (<= 64 KiB), medium (<= 4 MiB), large
        sizes_req = np.array([k[1] for k in keys])
        by_size = {}
        for name, lo_, hi_ in (("small", 0, 64 << 10), ("medium", (64 << 10) + 1, 4 << 20),
                               ("large", (4 << 20) + 1, 1 << 40)):
            sel = lat_us[(sizes_req >= lo_) & (sizes_req <= hi_)]
            if len(sel):
                by_size[name] = {"n": int(len(sel)), "p50_us": float(np.percentile(sel, 50)),
                                 "p99_us": float(np.percentile(sel, 99))}
        res[mode] = {"open_loop": {"GBps": total / mk / 1e9, "makespan_s": mk,
                                   "p50_us": float(np.percentile(lat_us, 50)),
                                   "p99_us": float(np.percentile(lat_us, 99)),
                                   "mean_us": float(lat_us.mean()), "kernel_launches": launches,
                                   "graph_captures": g1["captures"] - g0["captures"],
                                   "graph_replays": g1["replays"] - g0["replays"],
                                   "by_size": by_size},
                     "closed_loop": {"GBps": total / mk2 / 1e9, "req_per_s": nreq / mk2, "makespan_s": mk2},
                     "bit_exact": not bad, "mismatched": bad[:10]}
        if log:
            print(json.dumps({mode: res[mode]}), file=log, flush=True)
    res["server_stats"] = srv.stats()
    srv.destroy()
    res["server_over_plain"] = {
        "closed_loop_throughput": res["server"]["closed_loop"]["GBps"] / res["plain"]["closed_loop"]["GBps"],
        "open_loop_p99": res["server"]["open_loop"]["p99_us"] / res["plain"]["open_loop"]["p99_us"]}
    if floor and "halo" in fams:
        res["xface_floor"] = stream_xface_floor(torch, np, y, yk, keys, dir_of, specs, typed, total,
                                                res["plain"]["closed_loop"]["GBps"])
    for k in used:
        y.type_free(types[k])
    if o:
        o.finalize()
    del typed, packed_d, packed_h, priv
    torch.cuda.empty_cache()
    return res


def stream_xface_floor(torch, np, y, yk, keys, dir_of, specs, typed, total, plain_gbps):
    """The halo x-face fifth of the stream alone, as plain 8-byte loads (packs) and
    stores (unpacks) of its rows with the row-touch instrument, 16 requests per launch,
    all launches back to back: a lower bound on the time of any path that serves the
    stream, and so an upper bound on any path's capacity."""
    reads, writes = [], []
    arena = typed["halo"].data_ptr()     # the stream has finished with it: stores may land there
    for i, k in enumerate(keys):
        if k[0] != "halo":
            continue
        Z, Y, x0 = specs[k]["xface"]
        (writes if dir_of[i] == 1 else reads).append(yk.Rows(arena + 4 * x0, Z, Y * 2048, Y, 2048, 8, 0))
    torch.cuda.synchronize()
    flush = ColdL2(torch)
    stream = torch.cuda.current_stream()
    sh = ctypes.c_void_p(stream.cuda_stream)
    shp = ctypes.addressof(sh)

    def run():
        for pats, w in ((reads, 0), (writes, 1)):
            for j in range(0, len(pats), 16):
                y.probe_rows(pats[j:j + 16], w, shp)
    run()
    t = event_time(torch, run, 3, flush, stat=min)
    xbytes = float(sum(k[1] for k in keys if k[0] == "halo"))
    del flush
    cap = total / t / 1e9
    return {"requests": len(reads) + len(writes), "packed_bytes": xbytes, "rows": int(xbytes // 8),
            "touch_s": t, "capacity_bound_GBps": cap, "capacity_ratio_bound": cap / plain_gbps,
            "note": "plain 8-byte loads/stores of the x-face fifth's rows alone (row-touch instrument, "
                    "16 requests per launch); no path can serve the stream faster than this fifth's "
                    "rows can be touched"}


# ---------------------------------------------------------------------------
# the headline: halo faces, plain path per face, batched graph as a second form
# ---------------------------------------------------------------------------

def face_rows(yk, base, name, n=N):
    """Row-touch patterns covering exactly one face's typed bytes (16-byte runs for the
    contiguous faces)."""
    plane, row = n * n * 4, n * 4
    if name[0] == "x":
        return yk.Rows(base + (0 if name == "x-" else (n - 2) * 4), n, plane, n, row, 8, 0)
    if name[0] == "y":
        return yk.Rows(base + (0 if name == "y-" else (n - 2) * row), n, plane, 2 * row // 16, 16, 16, 0)
    return yk.Rows(base + (0 if name == "z-" else (n - 2) * plane), 1, 0, 2 * plane // 16, 16, 16, 0)


def capture(torch, fn):
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        fn()
    return g


def run_halo(args, y, yk, torch, np, world, rank, dist):
    faces = make_faces(y, yk)
    P = 2 * N * N * 4                      # packed bytes per face
    g = torch.Generator(device="cuda").manual_seed(1234 + rank)
    src = torch.rand(N * N * N, device="cuda", generator=g, dtype=torch.float32) * 2 - 1
    dst = torch.zeros_like(src)
    packed = [torch.empty(P, dtype=torch.uint8, device="cuda") for _ in faces]
    flush = ColdL2(torch)
    hbm, peak_kind = peaks()

    def cur():
        return torch.cuda.current_stream()

    def pack_face(i, s):
        h = ctypes.c_void_p(s.cuda_stream)      # alive for the call: the API reads *stream
        y.pack_stream(src.data_ptr(), 1, faces[i][1], 0, packed[i].data_ptr(), P, ctypes.addressof(h))

    def unpack_face(i, s):
        h = ctypes.c_void_p(s.cuda_stream)
        y.unpack_stream(packed[i].data_ptr(), P, dst.data_ptr(), 1, faces[i][1], 0, ctypes.addressof(h))

    def on_stream(fn, s):
        h = ctypes.c_void_p(s.cuda_stream)
        return fn(ctypes.addressof(h))

    # the launch-shape autotuner settles over the first calls of each shape class (a few
    # timed candidates each): make those calls before capturing and timing anything
    pack_batch = y.batch_array([yk.pack_op(src.data_ptr(), 1, t, 0, pk.data_ptr(), P)
                                for (name, t), pk in zip(faces, packed)])
    unpack_batch = y.batch_array([yk.unpack_op(pk.data_ptr(), P, dst.data_ptr(), 1, t, 0)
                                  for (name, t), pk in zip(faces, packed)])
    for _ in range(TUNE_CALLS):
        on_stream(lambda p: y.pup_batch_stream(pack_batch, p), cur())
        on_stream(lambda p: y.pup_batch_stream(unpack_batch, p), cur())
        for i in range(len(faces)):
            pack_face(i, cur())
        for i in range(len(faces)):
            unpack_face(i, cur())
    torch.cuda.synchronize()

    # the plain step: one stream per face (the message to one neighbour), pack then
    # unpack on it; the twelve calls captured once into a CUDA graph
    face_streams = [torch.cuda.Stream() for _ in faces]

    def plain_step_streams():
        main = torch.cuda.current_stream()
        for i, s in enumerate(face_streams):
            s.wait_stream(main)
            with torch.cuda.stream(s):
                pack_face(i, s)
                unpack_face(i, s)
        for s in face_streams:
            main.wait_stream(s)

    def plain_step_one_stream():
        for i in range(len(faces)):
            pack_face(i, cur())
        for i in range(len(faces)):
            unpack_face(i, cur())

    st0 = y.stats()
    g_plain = capture(torch, plain_step_streams)
    st1 = y.stats()
    kernels_per_step = st1["launches"] - st0["launches"]          # counted when captured
    copies_per_step = st1["memcpy_calls"] - st0["memcpy_calls"]   # contiguous faces
    # per face and direction: one plain call captured alone
    g_face, face_kind = {}, {}
    for i, (name, _) in enumerate(faces):
        for d, fn in (("pack", pack_face), ("unpack", unpack_face)):
            l0 = y.stats()["launches"]
            g_face[(name, d)] = capture(torch, lambda i=i, fn=fn: fn(i, cur()))
            face_kind[(name, d)] = ("yk_regular_kernel" if y.stats()["launches"] > l0 else
                                    "cudaMemcpyAsync (contiguous face)")
    # the batched form: one launch per direction for all six faces, a library-captured graph
    graph, _ = y.graph_create([[yk.pack_op(src.data_ptr(), 1, t, 0, pk.data_ptr(), P)
                                for (name, t), pk in zip(faces, packed)],
                               [yk.unpack_op(pk.data_ptr(), P, dst.data_ptr(), 1, t, 0)
                                for (name, t), pk in zip(faces, packed)]])
    g_pack_b, _ = y.graph_create([[yk.pack_op(src.data_ptr(), 1, t, 0, pk.data_ptr(), P)
                                   for (name, t), pk in zip(faces, packed)]])
    g_unpack_b, _ = y.graph_create([[yk.unpack_op(pk.data_ptr(), P, dst.data_ptr(), 1, t, 0)
                                     for (name, t), pk in zip(faces, packed)]])

    def step_batched():
        on_stream(lambda p: y.graph_launch(graph, p), cur())

    for _ in range(args.warmup):
        flush()
        g_plain.replay()
        flush()
        step_batched()
    torch.cuda.synchronize()

    def timed(fn, steps):
        tot = 0.0
        for _ in range(steps):
            flush()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            e1.synchronize()
            tot += e0.elapsed_time(e1) * 1e-3
        return tot

    # the timed region: the plain step, graph replay
    clocks = Clocks(os.path.join(tempfile.gettempdir(), f"yk_clocks_{os.getpid()}.csv"))
    clocks.start()
    time.sleep(0.3)
    launches0 = y.stats()["launches"]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    tot = timed(g_plain.replay, args.steps)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    # the library counts launches when the calls are made (here: at capture), so the
    # timed region's launches are the graph's kernel nodes times the steps
    launches = kernels_per_step * args.steps
    assert y.stats()["launches"] == launches0
    if dist:
        tt = torch.tensor([tot], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tot = tt.item()
    step_bytes = 2 * P * len(faces)       # packed bytes moved per step (pack + unpack)
    ms = tot / args.steps * 1e3
    value = step_bytes * world / (tot / args.steps) / 1e9

    # the other forms of the same step
    tot_one = timed(lambda: plain_step_one_stream(), args.steps)
    tot_b = timed(step_batched, args.steps)
    tot_unc = timed(lambda: (on_stream(lambda p: y.pup_batch_stream(pack_batch, p), cur()),
                             on_stream(lambda p: y.pup_batch_stream(unpack_batch, p), cur())), args.steps)

    # per face: each plain call alone (graph replay, cold L2)
    reps = max(5, args.steps)
    per_face = []
    for (name, d), gg in g_face.items():
        t = event_time(torch, gg.replay, reps, flush)
        per_face.append({"face": name, "direction": d, "time_us": t * 1e6, "packed_GBps": P / t / 1e9,
                         "hbm_frac": 2 * P / t / 1e9 / hbm, "launch": face_kind[(name, d)]})
    # the batched launches alone (graph replay): the dominant kernel of the batched form
    t_bp = event_time(torch, lambda: on_stream(lambda p: y.graph_launch(g_pack_b, p), cur()), reps, flush)
    t_bu = event_time(torch, lambda: on_stream(lambda p: y.graph_launch(g_unpack_b, p), cur()), reps, flush)

    # the floor: plain loads of every face's typed bytes in src (what a pack must read)
    # and plain stores into every face of dst (what an unpack must write), one launch
    # each, cold L2; the x-faces alone as well
    def probe(base, which, write):
        pats = [face_rows(yk, base, name) for name, _ in faces if name in which]
        on_stream(lambda p: y.probe_rows(pats, write, p), cur())
    fl = {}
    for key, which in (("all", ("x-", "x+", "y-", "y+", "z-", "z+")), ("x", ("x-", "x+")), ("x1", ("x-",))):
        fl[key] = (event_time(torch, lambda: probe(src.data_ptr(), which, 0), reps, flush),
                   event_time(torch, lambda: probe(dst.data_ptr(), which, 1), reps, flush))
    floor_us = (fl["all"][0] + fl["all"][1]) * 1e6

    # the measured step ran last in dst order: refresh dst with one plain step, then check
    dst.zero_()
    torch.cuda.synchronize()
    g_plain.replay()
    torch.cuda.synchronize()

    def faces_equal(a, b):
        s3, d3 = a.view(N, N, N), b.view(N, N, N)
        return (torch.equal(s3[:, :, :2], d3[:, :, :2]) and torch.equal(s3[:, :, -2:], d3[:, :, -2:])
                and torch.equal(s3[:, :2, :], d3[:, :2, :]) and torch.equal(s3[:, -2:, :], d3[:, -2:, :])
                and torch.equal(s3[:2], d3[:2]) and torch.equal(s3[-2:], d3[-2:]))
    ok = faces_equal(src, dst)
    # and the packed faces byte for byte against the oracle on the host
    o = yk.Yaksa(ensure_oracle())
    o.init()
    ofaces = make_faces(o, yk)
    src_h = src.cpu().numpy()
    for (name, t), pk in zip(ofaces, packed):
        ob = np.zeros(P, dtype=np.uint8)
        o.pack(src_h.ctypes.data, 1, t, 0, ob.ctypes.data, P)
        ok = ok and np.array_equal(pk.cpu().numpy(), ob)
    for _, t in ofaces:
        o.type_free(t)
    o.finalize()

    # roofline of the dominant kernel of the timed step.  The plain step is twelve launches
    # of yk_regular_kernel; the x-face launches (8-byte units, one 8-byte run per 2 KiB
    # grid row) take the longest.  Each launch's duration is that call alone (one-node
    # graph, CUDA events, cold L2): timing events captured inside the step's graph slow
    # the step itself, so they are not used.  Each launch moves 2 bytes per packed byte.
    alg = 2 * P
    dur = {(f["face"], f["direction"]): f["time_us"] * 1e-6 for f in per_face}
    xkeys = [k for k in dur if k[0][0] == "x"]
    xmean = statistics.mean(dur[k] for k in xkeys)
    share = sum(dur[k] for k in xkeys) / sum(dur.values())
    traffic = ncu_traffic("yk_regular_kernel_halo_xface")
    tr_launch = statistics.mean(traffic.values()) if traffic else None
    xfloor = (fl["x1"][0] + fl["x1"][1]) / 2        # one x-face alone, mean of the directions
    roof = {"bound": "hbm", "achieved": alg / xmean / 1e9, "peak": hbm, "unit": "GB/s",
            "frac": alg / xmean / 1e9 / hbm, "peak_source": peak_kind,
            "traffic": tr_launch, "traffic_frac": (tr_launch / xmean / 1e9 / hbm) if tr_launch else None,
            "traffic_note": "dram__bytes_read.sum + dram__bytes_write.sum per x-face launch from one ncu "
                            "capture (mean of pack and unpack): each 8-byte row costs a 128-byte DRAM fetch",
            "kernel": "yk_regular_kernel<8,*,1> (the x-face launches of the plain step: 4 of its "
                      f"{kernels_per_step} kernel launches, {100 * share:.0f}% of their summed duration "
                      "alone)",
            "duration_source": "each launch alone (one-node graph replay, CUDA events, cold L2)",
            "algorithmic_bytes_per_launch": alg,
            "launch_us": {d + f: dur[(f, d)] * 1e6 for (f, d) in sorted(dur)},
            "launch_us_mean": xmean * 1e6,
            "floor_us": xfloor * 1e6, "frac_vs_floor": xfloor / xmean,
            "floor_note": "row-touch instrument: plain 8-byte loads (pack) and stores (unpack) over one "
                          "x-face's 262,144 rows alone, cold L2, mean of the two directions; what any "
                          "kernel moving that face must at least spend",
            "floor_both_xfaces_us": {"loads": fl["x"][0] * 1e6, "stores": fl["x"][1] * 1e6},
            "step": {"achieved": step_bytes / (ms * 1e-3) / 1e9, "frac": step_bytes / (ms * 1e-3) / 1e9 / hbm,
                     "floor_us": floor_us, "step_us": ms * 1e3, "frac_vs_floor": floor_us / (ms * 1e3),
                     "note": "the whole step: all six faces' bytes over its time; floor = plain loads of "
                             "every face's typed bytes plus plain stores of them, one launch each"}}
    btraffic = {k: v * (N / 384) ** 2 for k, v in ncu_traffic("yk_batch_regular_kernel_halo3d").items()}
    batched = {"value": step_bytes * world / (tot_b / args.steps) / 1e9, "unit": "GB/s",
               "ms_per_step": tot_b / args.steps * 1e3,
               "note": "yaksa_gb300_graph_create of two batches (one launch per direction for all six "
                       "faces), graph replay",
               "roofline": {"bound": "hbm", "kernel": "yk_batch_regular_kernel (6 faces per launch)",
                            "launch_us": {"pack": t_bp * 1e6, "unpack": t_bu * 1e6},
                            "achieved": 2 * P * len(faces) / ((t_bp + t_bu) / 2) / 1e9,
                            "frac": 2 * P * len(faces) / ((t_bp + t_bu) / 2) / 1e9 / hbm,
                            "peak": hbm, "unit": "GB/s",
                            "traffic": (statistics.mean(btraffic.values()) if btraffic else None),
                            "floor_us": floor_us,
                            "frac_vs_floor": floor_us / ((t_bp + t_bu) * 1e6),
                            "note": "launch_us: each batched launch alone from a library-captured graph "
                                    "of that launch, CUDA events, cold L2"}}
    res = dict(value=value, ms=ms, wall=wall, clk=clk, launches=launches, ok=ok, roofline=roof,
               per_face=per_face, batched=batched,
               plain_one_stream={"value": step_bytes * world / (tot_one / args.steps) / 1e9, "unit": "GB/s",
                                 "ms_per_step": tot_one / args.steps * 1e3,
                                 "note": "the twelve calls on one stream, uncaptured (host work per call "
                                         "inside the timed span)"},
               batched_uncaptured={"value": step_bytes * world / (tot_unc / args.steps) / 1e9, "unit": "GB/s",
                                   "ms_per_step": tot_unc / args.steps * 1e3,
                                   "note": "yaksa_gb300_pup_batch_stream per direction, host planning "
                                           "inside the timed span"})

    # e2e through the reference's C-ABI (yaksa_ipack / yaksa_iunpack + yaksa_request_wait):
    # the exchange through host memory, as a halo exchange over host buffers runs it.
    # Every step packs the six faces of the device-resident grid into pinned host send
    # buffers (the step's result, read back to the host: d2h) and unpacks six pinned host
    # receive buffers into the second grid (the step's input from the host: h2d).  The
    # kernels write and read the host buffers in place over NVLink-C2C inside the timed
    # region.  In an exchange the received faces come from the neighbours and do not
    # depend on the faces sent in the same step; here the receive buffers hold the same
    # faces, packed once before timing, so the result is checkable.  All twelve requests
    # are issued before the first wait, and the two directions of the link overlap.
    y.graph_free(graph)
    y.graph_free(g_pack_b)
    y.graph_free(g_unpack_b)
    send = [torch.empty(P, dtype=torch.uint8).pin_memory() for _ in faces]
    recv = [torch.empty(P, dtype=torch.uint8).pin_memory() for _ in faces]

    res["kernels_per_step"] = kernels_per_step
    res["copies_per_step"] = copies_per_step

    def e2e_run(gsrc, gdst, steps, overlap):
        for (name, t), pk in zip(faces, recv):
            y.pack(gsrc.data_ptr(), 1, t, 0, pk.data_ptr(), P)

        def one():
            reqs = [y.ipack(gsrc.data_ptr(), 1, t, 0, pk.data_ptr(), P)[1] for (name, t), pk in zip(faces, send)]
            if not overlap:
                for r in reqs:
                    y.wait(r)
                reqs = []
            reqs += [y.iunpack(pk.data_ptr(), P, gdst.data_ptr(), 1, t, 0)[1]
                     for (name, t), pk in zip(faces, recv if overlap else send)]
            for r in reqs:
                y.wait(r)
        for _ in range(2):
            one()
        t0 = time.perf_counter()
        for _ in range(steps):
            one()
        return (time.perf_counter() - t0) / steps

    e_steps = max(3, args.steps // 2)
    results = {}
    for overlap in (True, False):
        dst.zero_()
        torch.cuda.synchronize()
        results[overlap] = e2e_run(src, dst, e_steps, overlap)
        res["ok"] = res["ok"] and faces_equal(src, dst)
    res["e2e"] = {"value": step_bytes * world / results[True] / 1e9, "unit": "GB/s",
                  "h2d_bytes_per_step": P * len(faces), "d2h_bytes_per_step": P * len(faces),
                  "mode": "per face yaksa_ipack (device grid -> pinned host send buffer) and yaksa_iunpack "
                          "(pinned host receive buffer -> device grid), all twelve issued, then "
                          "yaksa_request_wait on each; kernels access the host buffers in place over "
                          "NVLink-C2C"}
    res["e2e_serial"] = {"value": step_bytes * world / results[False] / 1e9, "unit": "GB/s",
                         "note": "the six packs completed before the six unpacks, which read the send buffers"}
    # the host link's own rate for the step's transfers: the row-touch instrument reads the
    # six receive buffers and writes the six send buffers (12 MiB each way), both launches
    # at once on two streams, GPU-timed; the e2e step moves the same bytes over the link
    s_rd, s_wr = torch.cuda.Stream(), torch.cuda.Stream()
    rd_rows = [yk.Rows(pk.data_ptr(), 1, 0, P // 16, 16, 16, 0) for pk in recv]
    wr_rows = [yk.Rows(pk.data_ptr(), 1, 0, P // 16, 16, 16, 0) for pk in send]

    def link_once():
        e0 = torch.cuda.Event(enable_timing=True)
        e0.record()
        ends = []
        for st, rows, w in ((s_rd, rd_rows, 0), (s_wr, wr_rows, 1)):
            st.wait_event(e0)
            h = ctypes.c_void_p(st.cuda_stream)
            y.probe_rows(rows, w, ctypes.addressof(h))
            e = torch.cuda.Event(enable_timing=True)
            e.record(st)
            ends.append(e)
        torch.cuda.synchronize()
        return max(e0.elapsed_time(e) for e in ends) * 1e-3
    for _ in range(3):
        link_once()
    link_t = statistics.median(link_once() for _ in range(15))
    link_gbps = step_bytes / link_t / 1e9
    res["e2e"]["link_floor"] = {"GBps": link_gbps, "us": link_t * 1e6, "frac": res["e2e"]["value"] / link_gbps,
                                "note": "plain 16-byte loads of the six pinned receive buffers and stores "
                                        "into the six send buffers, at once (row-touch instrument, GPU-timed): "
                                        "the host link's rate for the step's 12 MiB each way"}
    hsrc = src.cpu().pin_memory()
    hdst = torch.zeros_like(hsrc).pin_memory()
    e2e_h = e2e_run(hsrc, hdst, e_steps, True)
    res["ok"] = res["ok"] and faces_equal(hsrc, hdst)
    res["e2e_host_grid"] = {"value": step_bytes * world / e2e_h / 1e9, "unit": "GB/s",
                            "note": "grids and packed buffers all in pinned host memory"}
    for _, t in faces:
        y.type_free(t)
    del src, dst, packed, flush, hsrc, hdst, send, recv, g_plain, g_face
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-suite", action="store_true", help="skip the per-config records")
    ap.add_argument("--suite", default=None,
                    help="run only the per-config records and write their JSON lines to this file")
    ap.add_argument("--suite-only", default=None, help="comma-separated suite workloads")
    ap.add_argument("--suite-scale", type=int, default=1,
                    help="divide the suite's block/element counts (profiler captures)")
    ap.add_argument("--stream", default=None,
                    help="run only the mixed request stream (plain vs server) and write its JSON")
    ap.add_argument("--stream-requests", type=int, default=10000)
    ap.add_argument("--stream-families", default=None,
                    help="comma-separated subset of hvector,halo,hindexed,struct,reduce for --stream")
    ap.add_argument("--no-stream", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.suite:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        lines = run_suite(args.steps, only=args.suite_only.split(",") if args.suite_only else None,
                          scale=args.suite_scale, log=sys.stderr)
        with open(args.suite, "w") as f:
            for l in lines:
                f.write(json.dumps(l) + "\n")
        return
    if args.stream:
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        r = run_stream(nreq=args.stream_requests, log=sys.stderr,
                       families=args.stream_families.split(",") if args.stream_families else None)
        with open(args.stream, "w") as f:
            f.write(json.dumps(r) + "\n")
        print(json.dumps(r))
        return

    import numpy as np
    import torch
    import yaksa_gb300 as yk

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    if not os.path.exists(yk.LIB_PATH):
        from yaksa_gb300 import build
        build.build()
    y = yk.Yaksa()
    y.init()
    h = run_halo(args, y, yk, torch, np, world, rank, dist)
    line = {"metric": METRIC, "value": h["value"], "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": h["ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded uniform [-1,1))",
            "config": {"workload": WORKLOAD,
                       "path": "plain: yaksa_pack_stream + yaksa_unpack_stream per face, each face on its own "
                               "stream, the twelve calls captured once into a CUDA graph and replayed per step",
                       "parallelism": f"replicas x{world}",
                       "l2": "flushed between steps outside the event-timed span: 512 MiB written, then "
                             "512 MiB read so that no dirty flush lines remain"},
            "bit_exact": bool(h["ok"]),
            "roofline": h["roofline"],
            "per_face": h["per_face"],
            "batched_graph": h["batched"],
            "plain_one_stream": h["plain_one_stream"],
            "batched_uncaptured": h["batched_uncaptured"],
            "gpu_launches": h["launches"],
            "clocks": h["clk"],
            "e2e": h["e2e"],
            "e2e_serial": h["e2e_serial"],
            "e2e_host_grid": h["e2e_host_grid"],
            "wall_s": h["wall"]}
    if rank == 0 and not args.no_suite:
        lines = run_suite(args.steps)
        line["suite"] = lines
        line["suite_bit_exact"] = all(l["bit_exact"] for l in lines)
    if rank == 0 and not args.no_stream:
        # the metric's second half: batched (persistent server) vs plain p50/p99 on the
        # mixed request stream (rank 0 reports it; the other replicas have finished)
        r = run_stream(nreq=args.stream_requests, check=True)
        line["stream"] = {
            "workload": f"{r['requests']} pack/unpack requests, Poisson {r['rate_per_s']:.0f}/s, "
                        "families hvector/halo x-face/hindexed/struct/indexed_block-reduce, "
                        "packed sizes log-uniform over 19 power-of-two classes 256 B..64 MiB, "
                        f"{100 * r['host_fraction']:.0f}% packed side in pinned host memory",
            "packed_bytes": r["packed_bytes"],
            "plain": {"p50_us": r["plain"]["open_loop"]["p50_us"], "p99_us": r["plain"]["open_loop"]["p99_us"],
                      "GBps": r["plain"]["open_loop"]["GBps"],
                      "capacity_GBps": r["plain"]["closed_loop"]["GBps"],
                      "capacity_req_per_s": r["plain"]["closed_loop"]["req_per_s"]},
            "plain_graphs": {"p50_us": r["graphs"]["open_loop"]["p50_us"],
                             "p99_us": r["graphs"]["open_loop"]["p99_us"],
                             "GBps": r["graphs"]["open_loop"]["GBps"],
                             "capacity_GBps": r["graphs"]["closed_loop"]["GBps"],
                             "capacity_req_per_s": r["graphs"]["closed_loop"]["req_per_s"],
                             "graph_captures": r["graphs"]["open_loop"]["graph_captures"],
                             "graph_replays": r["graphs"]["open_loop"]["graph_replays"],
                             "bit_exact": r["graphs"]["bit_exact"]},
            "batched": {"p50_us": r["server"]["open_loop"]["p50_us"], "p99_us": r["server"]["open_loop"]["p99_us"],
                        "GBps": r["server"]["open_loop"]["GBps"],
                        "capacity_GBps": r["server"]["closed_loop"]["GBps"],
                        "capacity_req_per_s": r["server"]["closed_loop"]["req_per_s"],
                        "item_cut_tuning": {"classes_decided": r.get("server_tuned_classes"),
                                            "calibration_s": r.get("server_tune_s")}},
            "by_size": {"plain": r["plain"]["open_loop"]["by_size"],
                        "plain_graphs": r["graphs"]["open_loop"]["by_size"],
                        "batched": r["server"]["open_loop"]["by_size"],
                        "classes": "small <= 64 KiB < medium <= 4 MiB < large"},
            "capacity_ratio": r["server_over_plain"]["closed_loop_throughput"],
            "p99_ratio": r["server_over_plain"]["open_loop_p99"],
            "xface_floor": r.get("xface_floor"),
            "bit_exact": r["plain"]["bit_exact"] and r["server"]["bit_exact"] and r["graphs"]["bit_exact"],
            "checked_requests": r["checked_requests"],
            "checked_size_classes": r["checked_size_classes"],
            "largest_checked_bytes": r["largest_checked_bytes"],
            "note": "p50/p99 from arrival to completion seen by the serving loop; capacity = all "
                    "requests arriving at once; plain_graphs = one launch per request with "
                    "repeated request records replayed as captured CUDA graphs; batched = "
                    "persistent-kernel server, its item cut calibrated per request class "
                    "before the timed runs"}
    if rank == 0 and not args.no_cpu:
        b = cpu_halo(args.cpu_seconds, 1)
        line["cpu_baseline"] = {k: b[k] for k in ("value", "unit", "cores", "kind", "cpu", "sample")}
        line["cpu_baseline"]["faces_equal"] = bool(b["ok"])
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
