#!/usr/bin/env python3
"""SA+BWT throughput of libsais_gb300 on one GB300 (or N independent replicas).

A step = suffix array + BWT (with primary index) of one text.  Default
workload: the repetitive genome-like uint8 text of n = 2^28 (order-2 Markov
DNA, GC 0.41, 5% segmental duplications of 1 KiB-1 MiB with 0.1%
substitutions, tandem repeats of period 2-64 x 10-500 copies), seeded
synthetic data standing in for the genome corpora of libsais's benchmarks.

  value    device-resident: text already in HBM, SA (int32) and BWT written to
           HBM by one sort (gsais_sa_bwt_device); CUDA events on the launching
           stream.
  e2e      the same metric through the drop-in libsais API from pinned host
           buffers: libsais() for SA, then libsais_bwt() for the BWT (two
           sorts, exactly the two calls a libsais user makes); the text goes
           up in each call and SA and BWT come back inside the timed region.
           The one-sort host call gsais_sa_bwt is reported beside it.
  roofline the radix-sort digit pass kernel k_radix_pass (the dominant
           kernel): its algorithmic bytes (every key/value pair read and
           written once) over its CUDA-event time inside the timed region,
           against the measured HBM copy bandwidth; traffic = the DRAM bytes
           per algorithmic byte of an ncu capture of the same kernel
           (profiles/radix_pass_traffic.json) times the launch's bytes.
  cpu_baseline  the reference libsais built with OpenMP (oracle/_ref), run by
           this script's reference arm in a child process on the whole
           workload text with every host thread: libsais_omp + libsais_bwt_omp.

--impl reference times that reference step (libsais_omp then libsais_bwt_omp
on the whole text, all host threads; the oracle port on a prefix only when the
reference library could not be built).  Its input comes from the oracle's
build of the text generators, so that arm loads no library of this package.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (generator, n, description)
    "genome_like_2^28": ("genome_like", 1 << 28, "repetitive genome-like uint8 text, n=2^28"),
    "dna_iid_2^24": ("iid", 1 << 24, "i.i.d. uniform ACGT uint8 text, n=2^24"),
    "all_A_2^26": ("constant", 1 << 26, "all-'A' uint8 text, n=2^26"),
    "period7_2^26": ("periodic", 1 << 26, "period-7 'ACGTACG' uint8 text, n=2^26"),
}
METRIC = "SA+BWT input MB/s"
UNIT = "MB/s"
REF_SAMPLE = 1 << 24


def make_text(name: str, n: int) -> np.ndarray:
    from libsais_gb300 import textgen
    gen = WORKLOADS[name][0]
    if gen == "genome_like":
        return textgen.genome_like(n, seed=2)
    if gen == "iid":
        return textgen.iid(n, seed=1)
    if gen == "constant":
        return textgen.constant(n)
    return textgen.periodic(n)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def host_threads() -> int:
    """All host CPUs: this process's CPU affinity is widened to every CPU first
    (a parent that ran CUDA work may have left a narrower mask to its children)."""
    n = os.cpu_count() or 1
    try:
        os.sched_setaffinity(0, set(range(n)))
        return len(os.sched_getaffinity(0))
    except (AttributeError, OSError):
        return n


def bench_config(name: str, n: int) -> dict:
    """The workload description shared by both arms (identical dicts)."""
    return {"workload": name, "n": n, "description": WORKLOADS[name][2], "sa": "int32",
            "outputs": "SA + BWT + primary index", "l2": "inputs larger than L2 (text and SA > 129 MB)"}


def reference_text(name: str, n: int) -> np.ndarray:
    """The workload text from the oracle library's build of the generators
    (the same C source, so the same bytes as make_text)."""
    from libsais_gb300 import textgen
    from oracle.oracle import ORACLE_SO, build
    if not os.path.exists(ORACLE_SO):
        build(with_reference=False)
    textgen.set_library(ORACLE_SO)
    try:
        return make_text(name, n)
    finally:
        textgen.set_library(None)


class ReferenceStep:
    """One SA+BWT step of the reference libsais: libsais_omp for the suffix array,
    then libsais_bwt_omp for the BWT and primary index (include/libsais.h:144,
    :238), on `threads` OpenMP threads.  Output and temporary buffers are
    allocated and touched once, outside the timed calls."""

    def __init__(self, T: np.ndarray, threads: int):
        from oracle.oracle import Reference
        self.lib = Reference().lib
        self.T = np.ascontiguousarray(T)
        n = self.T.size
        self.n, self.threads = n, threads
        self.SA = np.zeros(n, dtype=np.int32)
        self.A = np.zeros(n, dtype=np.int32)
        self.U = np.zeros(n, dtype=np.uint8)
        self.freq = np.zeros(256, dtype=np.int32)

    def __call__(self):
        p = lambda a: a.ctypes.data
        t0 = time.perf_counter()
        rc = self.lib.libsais_omp(p(self.T), p(self.SA), self.n, 0, p(self.freq), self.threads)
        t1 = time.perf_counter()
        prim = self.lib.libsais_bwt_omp(p(self.T), p(self.U), p(self.A), self.n, 0, p(self.freq), self.threads)
        t2 = time.perf_counter()
        if rc != 0 or prim < 0:
            raise SystemExit(f"reference libsais failed: {rc} {prim}")
        return t2 - t0, t1 - t0, t2 - t1, int(prim)


def port_step(T: np.ndarray):
    """SA-IS + BWT by the oracle port (1 thread), when the reference is absent."""
    from oracle.oracle import Oracle
    O = Oracle()
    t0 = time.perf_counter()
    _, SA = O.sa(T)
    O.bwt_from_sa(T, SA)
    return time.perf_counter() - t0


def serving_cpu_reference(sample_jobs: int, jobs_per_rate: int, seed: int = 6):
    """The serving stream's host aggregate: the reference libsais (OpenMP, all
    host threads) on a seeded sample of the stream's jobs, one after another:
    SA + BWT per job (libsais_omp + libsais_bwt_omp, the 16-bit jobs through
    libsais16_omp + libsais16_bwt_omp)."""
    import ctypes
    from libsais_gb300 import textgen
    from oracle.oracle import ORACLE_SO, Reference, build
    if not os.path.exists(ORACLE_SO):
        build(with_reference=False)
    textgen.set_library(ORACLE_SO)
    try:
        jobs = make_serving_jobs(jobs_per_rate, seed)
    finally:
        textgen.set_library(None)
    lib = Reference().lib
    p_, i32 = ctypes.c_void_p, ctypes.c_int32
    for name in ("libsais16_omp",):
        getattr(lib, name).argtypes = [p_, p_, i32, i32, p_, i32]
        getattr(lib, name).restype = i32
    lib.libsais16_bwt_omp.argtypes = [p_, p_, p_, i32, i32, p_, i32]
    lib.libsais16_bwt_omp.restype = i32
    threads = host_threads()
    sample = serving_sample(jobs_per_rate, sample_jobs, seed + 1)
    total, secs = 0, 0.0
    for k in sample:
        t = np.ascontiguousarray(jobs[k])
        n = t.size
        SA = np.zeros(n, dtype=np.int32)
        A = np.zeros(n, dtype=np.int32)
        U = np.zeros(n, dtype=t.dtype)
        freq = np.zeros(65536, dtype=np.int32)
        t0 = time.perf_counter()
        if t.dtype == np.uint16:
            rc = lib.libsais16_omp(t.ctypes.data, SA.ctypes.data, n, 0, freq.ctypes.data, threads)
            prim = lib.libsais16_bwt_omp(t.ctypes.data, U.ctypes.data, A.ctypes.data, n, 0, freq.ctypes.data, threads)
        else:
            rc = lib.libsais_omp(t.ctypes.data, SA.ctypes.data, n, 0, freq.ctypes.data, threads)
            prim = lib.libsais_bwt_omp(t.ctypes.data, U.ctypes.data, A.ctypes.data, n, 0, freq.ctypes.data, threads)
        secs += time.perf_counter() - t0
        if rc != 0 or prim < 0:
            raise SystemExit(f"reference failed on serving job {k}")
        total += n
    return {"mb_s": round(total / 1e6 / secs, 2), "jobs": int(sample.size), "input_mb": round(total / 1e6, 1),
            "threads": threads, "kind": "reference",
            "sample": "seeded sample of the stream's jobs (seed + 101), one after another"}


def run_reference(args, rank):
    """The reference arm: libsais built with OpenMP, on the host cores."""
    if rank != 0:
        return
    if args.serving_cpu:
        os.environ.setdefault("OMP_PROC_BIND", "close")
        os.environ.setdefault("OMP_DYNAMIC", "false")
        print(json.dumps({"serving_cpu": serving_cpu_reference(args.serving_cpu, args.serving_jobs)}), flush=True)
        return
    name = args.workload
    n = args.n or WORKLOADS[name][1]
    os.environ.setdefault("OMP_PROC_BIND", "close")   # read when the OpenMP runtime loads
    os.environ.setdefault("OMP_DYNAMIC", "false")
    from oracle.oracle import REF_SO
    T = reference_text(name, n)
    threads = host_threads()
    detail = {}
    if os.path.exists(REF_SO):
        step = ReferenceStep(T, threads)
        for _ in range(args.warmup):
            step()
        times, sa_t, bwt_t = [], [], []
        for _ in range(args.steps):
            dt, ds, db, _ = step()
            times.append(dt)
            sa_t.append(ds)
            bwt_t.append(db)
        kind, cores, sample_n = "reference", threads, n
        sample = (f"whole workload text (n={n}): libsais_omp + libsais_bwt_omp, {threads} OpenMP threads, "
                  f"reference libsais {_ref_version()} built with gcc -O3 -fopenmp")
        detail = {"sa_ms": round(1e3 * statistics.median(sa_t), 1), "bwt_ms": round(1e3 * statistics.median(bwt_t), 1),
                  "threads": threads, "omp_proc_bind": os.environ.get("OMP_PROC_BIND"),
                  "step_ms_min_max": [round(1e3 * min(times), 1), round(1e3 * max(times), 1)]}
    else:
        sample_n = min(n, args.ref_sample)
        Ts = T[:sample_n].copy()
        for _ in range(args.warmup):
            port_step(Ts)
        times = [port_step(Ts) for _ in range(args.steps)]
        kind, cores = "port", 1
        sample = f"first {sample_n} symbols of the {WORKLOADS[name][2]} (reference library not built here)"
    mean = sum(times) / len(times)
    value = sample_n / 1e6 / mean
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(mean * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": bench_config(name, n), "placement": f"host CPU, {cores} threads",
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    if detail:
        line["reference_detail"] = detail
    print(json.dumps(line), flush=True)


def _ref_version() -> str:
    from oracle.oracle import reference_dir
    try:
        with open(os.path.join(reference_dir(), "VERSION")) as f:
            return f.read().strip()
    except OSError:
        return "?"


def serving_cpu_child(sample_jobs: int, jobs_per_rate: int):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--serving-cpu", str(sample_jobs),
           "--serving-jobs", str(jobs_per_rate)]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    for ln in reversed(r.stdout.splitlines()):
        if ln.startswith("{"):
            return json.loads(ln)["serving_cpu"]
    return {"mb_s": None, "note": "child failed: " + (r.stderr.strip().splitlines() or ["?"])[-1][:160]}


def cpu_baseline_child(name: str, n: int):
    """Runs this script's reference arm (1 warm-up + 1 timed step) in a child
    process and returns its cpu_baseline block: the OpenMP runtime and the
    reference library stay out of this (CUDA) process."""
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--baseline-child", "--workload", name,
           "--n", str(n)]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    for ln in reversed(r.stdout.splitlines()):
        if ln.startswith("{"):
            line = json.loads(ln)
            out = dict(line["cpu_baseline"])
            if "reference_detail" in line:
                out["detail"] = line["reference_detail"]
            return out
    return {"value": None, "unit": UNIT, "cores": 0, "kind": "reference",
            "sample": "child failed: " + (r.stderr.strip().splitlines() or ["?"])[-1][:160]}


def oracle_check_sa_bwt(O, T: np.ndarray, SA: np.ndarray, U: np.ndarray, primary: int) -> bool:
    """SA passes the oracle's linear-time suffix-array check and the BWT and
    primary index equal the ones the oracle derives from it."""
    SA = np.ascontiguousarray(SA, dtype=np.int64)
    if not O.check_sa(T, SA):
        return False
    p, oU, _ = O.bwt_from_sa(T, SA)
    return p == int(primary) and np.array_equal(oU, U)


def run_batched(G, torch, count: int = 4096, steps: int = 3, warmup: int = 1, cpu_strings: int = 32,
                checked: int = 256):
    """The batched workload: `count` uint8 strings, lengths log-uniform over
    256 B - 4 MiB, i.i.d. ACGT with 1% 'N' (seeded).  Times the batched sort
    (all strings in the same launches) against one GPU call per string on the
    same device buffers.  A seeded sample of `checked` strings is checked
    against the oracle (SA check, BWT and primary index); the batched and
    per-string outputs are also compared in full."""
    from libsais_gb300 import textgen
    from oracle.oracle import Oracle
    T, offs = textgen.batch_strings(count, seed=3)
    n = int(offs[-1])
    dT = torch.from_numpy(T).cuda()
    dO = torch.from_numpy(offs).cuda()
    dSA = torch.empty(n, dtype=torch.int32, device="cuda")
    dU = torch.empty(n, dtype=torch.uint8, device="cuda")
    dP = torch.empty(count, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        if G.batch_sa_bwt_device(dT, dO, dSA, dU, dP, stream=stream) != 0:
            raise SystemExit("batched sort failed")
    launches0 = G.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        G.batch_sa_bwt_device(dT, dO, dSA, dU, dP, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / steps
    batched_launches = (G.launch_count() - launches0) / steps
    split = _kernel_split(G, torch, lambda: G.batch_sa_bwt_device(dT, dO, dSA, dU, dP, stream=stream), steps=1)
    bst = G.last_stats()
    # one call per string, same buffers
    pSA = torch.empty_like(dSA)
    pU = torch.empty_like(dU)
    prim = np.zeros(count, dtype=np.int32)
    torch.cuda.synchronize()
    launches0 = G.launch_count()
    t0 = time.perf_counter()
    for s in range(count):
        a, b = int(offs[s]), int(offs[s + 1])
        if b > a:
            prim[s] = G.sa_bwt_device(dT[a:b], pSA[a:b], pU[a:b], stream=stream)
    torch.cuda.synchronize()
    per_string_s = time.perf_counter() - t0
    per_string_launches = G.launch_count() - launches0
    hSA, hU, hP = dSA.cpu().numpy(), dU.cpu().numpy(), dP.cpu().numpy()
    identical = bool(torch.equal(pSA, dSA) and torch.equal(pU, dU) and np.array_equal(prim, hP))
    O = Oracle()
    rng = np.random.default_rng(7)
    sample = np.unique(np.concatenate([[0, count - 1], rng.choice(count, size=min(checked, count), replace=False)]))
    ok = True
    for s in sample:
        a, b = int(offs[s]), int(offs[s + 1])
        ok &= oracle_check_sa_bwt(O, T[a:b], hSA[a:b], hU[a:b], int(hP[s]))
    cpu_n = int(offs[cpu_strings])
    t0 = time.perf_counter()
    for s in range(cpu_strings):
        t = T[int(offs[s]):int(offs[s + 1])]
        _, sa = O.sa(t)
        O.bwt_from_sa(t, sa)
    cpu_s = time.perf_counter() - t0
    return {"strings": count, "total_symbols": n, "batched_mb_s": round(n / 1e6 / (batched_ms / 1e3), 1),
            "batched_ms": round(batched_ms, 2), "batched_launches": batched_launches,
            "rounds": bst["rounds"], "seed_symbols": bst["seed_symbols"], "active_total": bst["active_total"],
            "large_total": bst["large_total"], "kernels_ms": split,
            "per_string_mb_s": round(n / 1e6 / per_string_s, 1), "per_string_ms": round(per_string_s * 1e3, 1),
            "per_string_launches": per_string_launches,
            "speedup_vs_per_string": round(per_string_s * 1e3 / batched_ms, 2),
            "batched_equals_per_string": identical, "oracle_checked_strings": int(sample.size),
            "oracle_sample": "strings 0, count-1 and a seeded (seed 7) sample: SA check + BWT + primary",
            "oracle_ok": bool(ok),
            "cpu_port_mb_s": round(cpu_n / 1e6 / cpu_s, 2), "cpu_sample": f"first {cpu_strings} strings, 1 thread"}


SERVING_RATES = (100, 300, 1000, 3000, 5000)


def make_serving_jobs(count: int, seed: int = 6, pools=None):
    """The serving stream's jobs: lengths log-uniform over 4 KiB - 64 MiB; 70% order-2
    Markov ACGT uint8, 20% uniform 0-255 uint8, 10% uint16 Zipf(1.1) over 1..65535.
    Texts are seeded slices of three seeded pools (so generation stays fast);
    `pools` = (dna, bytes, zipf) arrays to slice (e.g. pinned copies)."""
    from libsais_gb300 import textgen
    u = textgen.uniform(3 * count, seed)
    lens = textgen.loguniform_lengths(count, 4096, 64 << 20, seed + 1)
    if pools is None:
        pools = serving_pools(seed)
    dna, byt, zipf = pools
    jobs = []
    for k in range(count):
        n = int(lens[k])
        pool = dna if u[3 * k] < 0.7 else (byt if u[3 * k] < 0.9 else zipf)
        n = min(n, pool.size)
        a = int(u[3 * k + 1] * (pool.size - n))
        jobs.append(pool[a:a + n])
    return jobs


def serving_pools(seed: int = 6):
    from libsais_gb300 import textgen
    dna = textgen.markov2_dna(1 << 29, seed=seed + 2)
    byt = np.frombuffer(np.random.default_rng(seed + 3).bytes(1 << 27), dtype=np.uint8)
    zipf = textgen.zipf_u16(1 << 26, seed=seed + 4)
    return dna, byt, zipf


def serving_sample(count: int, size: int, seed: int = 6):
    """A seeded sample of job indexes of the stream (for the one-job-at-a-time
    GPU path and the host reference, which cannot run the whole stream)."""
    rng = np.random.default_rng(seed + 100)
    return np.sort(rng.choice(count, size=min(size, count), replace=False))


class OutputRing:
    """Pinned host memory for job outputs, taken and given back in submission
    order; take() blocks while the ring is full (the client's backpressure)."""

    def __init__(self, torch, nbytes: int):
        self.buf = torch.empty(nbytes, dtype=torch.uint8).pin_memory().numpy()
        self.n = nbytes
        self.head = 0       # next free byte (monotone)
        self.tail = 0       # oldest byte still in use (monotone)
        self.cv = threading.Condition()

    def take(self, nbytes: int):
        nbytes = (nbytes + 255) & ~255
        if nbytes > self.n:
            raise ValueError("job larger than the output ring")
        with self.cv:
            while True:
                start = self.head
                off = start % self.n
                if off + nbytes > self.n:   # wrap: skip the ring's tail end
                    start += self.n - off
                    off = 0
                if start + nbytes - self.tail <= self.n:
                    self.head = start + nbytes
                    return start, off, nbytes
                self.cv.wait()

    def give(self, start: int, nbytes: int):
        with self.cv:
            self.tail = start + nbytes
            self.cv.notify_all()

    def views(self, off: int, n: int, dtype):
        SA = self.buf[off:off + 4 * n].view(np.int32)
        isz = np.dtype(dtype).itemsize
        o2 = off + ((4 * n + 255) & ~255)
        U = self.buf[o2:o2 + isz * n].view(dtype)
        return SA, U

    @staticmethod
    def bytes_for(n: int, itemsize: int) -> int:
        return ((4 * n + 255) & ~255) + itemsize * n


def run_serving(G, torch, rates=SERVING_RATES, jobs_per_rate: int = 20000, seed: int = 6, budget: int = 120 << 30,
                workers: int = 3, oracle_jobs: int = 8, plain_sample: int = 300, ring_bytes: int = 8 << 30):
    """The serving stream: `jobs_per_rate` SA+BWT jobs with Poisson arrivals at
    each rate, open loop (latency is measured from each job's scheduled arrival,
    so time spent waiting for output space or for the server counts), under
    an HBM budget, with small jobs coalesced.  Job texts are slices of pinned
    pools and outputs land in a pinned ring.  Checked: the first `oracle_jobs`
    jobs of at most 4 Mi symbols of each rate against the oracle.  Beside it:
    the plain one-job-at-a-time GPU path on a seeded sample of the stream."""
    from libsais_gb300 import textgen
    from oracle.oracle import Oracle
    O = Oracle()
    pools = tuple(torch.from_numpy(np.ascontiguousarray(p)).pin_memory().numpy() if p.dtype != np.uint16 else
                  torch.from_numpy(p.view(np.int16)).pin_memory().numpy().view(np.uint16) for p in serving_pools(seed))
    jobs = make_serving_jobs(jobs_per_rate, seed, pools)
    sym = int(sum(t.size for t in jobs))
    ring = OutputRing(torch, ring_bytes)
    out = {"jobs_per_rate": jobs_per_rate, "input_mb_per_rate": round(sym / 1e6, 1), "budget_bytes": budget,
           "workers": workers, "footprint_bytes_per_symbol": 80.0, "rates": []}
    for rate in rates:
        arrivals = textgen.poisson_arrivals(jobs_per_rate, float(rate), seed + 10 + rate)
        srv = G.Server(hbm_budget_bytes=budget, workers=workers, small_job_symbols=1 << 20, max_batch=256)
        lat = np.zeros(jobs_per_rate)
        check = [k for k in range(jobs_per_rate) if jobs[k].size <= (4 << 20)][:oracle_jobs]
        checked = {}
        ids = [0] * jobs_per_rate
        slots = [None] * jobs_per_rate
        delay = np.zeros(jobs_per_rate)
        submitted = threading.Semaphore(0)
        fails = []

        def waiter():
            for k in range(jobs_per_rate):
                submitted.acquire()
                res, SA, U, q, total, b = srv.wait(ids[k])
                lat[k] = delay[k] + total
                if res < 0:
                    fails.append((k, res))
                if k in check:
                    checked[k] = (res, SA.copy(), U.copy())
                ring.give(slots[k][0], slots[k][2])

        th = threading.Thread(target=waiter, daemon=True)
        th.start()
        t0 = time.perf_counter()
        for k, t in enumerate(jobs):
            wait_s = arrivals[k] - (time.perf_counter() - t0)
            if wait_s > 0:
                time.sleep(wait_s)
            slots[k] = ring.take(OutputRing.bytes_for(t.size, t.itemsize))
            SA, U = ring.views(slots[k][1], t.size, t.dtype)
            delay[k] = (time.perf_counter() - t0) - arrivals[k]
            ids[k] = srv.submit_into(t, SA, U)
            submitted.release()
        th.join()
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        ok = not fails and all(oracle_check_sa_bwt(O, jobs[k], SA, U, res) for k, (res, SA, U) in checked.items())
        lat_ms = lat * 1e3
        out["rates"].append({
            "rate_per_s": rate, "jobs": jobs_per_rate, "wall_s": round(wall, 2),
            "p50_ms": round(float(np.percentile(lat_ms, 50)), 2), "p95_ms": round(float(np.percentile(lat_ms, 95)), 2),
            "p99_ms": round(float(np.percentile(lat_ms, 99)), 2),
            "served_mb_s": round(sym / 1e6 / st["busy_seconds"], 1) if st["busy_seconds"] else None,
            "coalesced_batches": st["batches"], "coalesced_jobs": st["batched_jobs"],
            "hbm_high_water_gb": round(st["hbm_high_water_bytes"] / 1e9, 2), "rejected": st["rejected"],
            "failed": len(fails), "oracle_checked_jobs": len(checked), "oracle_ok": bool(ok)})
    # the plain path: one job at a time through the host C-ABI, pinned buffers, on a sample
    lib = G.load()
    sample = serving_sample(jobs_per_rate, plain_sample, seed)
    s_sym = int(sum(jobs[k].size for k in sample))
    t1 = time.perf_counter()
    for k in sample:
        t = jobs[k]
        start, off, nb = ring.take(OutputRing.bytes_for(t.size, t.itemsize))
        SA, U = ring.views(off, t.size, t.dtype)
        res = lib.gsais_sa_bwt(None, t.ctypes.data, t.itemsize, t.size, SA.ctypes.data, 4, U.ctypes.data, None, 4)
        ring.give(start, nb)
        if res < 0:
            raise SystemExit(f"plain path failed on job {k}: {res}")
    plain_s = time.perf_counter() - t1
    out["plain_one_job_at_a_time"] = {"mb_s": round(s_sym / 1e6 / plain_s, 1), "jobs": int(sample.size),
                                      "input_mb": round(s_sym / 1e6, 1),
                                      "sample": "seeded sample of the stream's jobs (seed + 100)"}
    return out


def _kernel_split(G, torch, fn, steps: int = 2):
    """Per-kernel device time (CUDA events on the launching stream) of `steps`
    calls of fn, in ms per call, largest first; with the rounds run."""
    torch.cuda.synchronize()
    G.profile_reset()
    G.profile_enable(True)
    for _ in range(steps):
        fn()
    torch.cuda.synchronize()
    G.profile_enable(False)
    prof = G.profile_read()
    split = {k: round(v["total_ms"] / steps, 3) for k, v in prof.items() if v["launches"]}
    return dict(sorted(split.items(), key=lambda kv: -kv[1]))


def _timed(torch, fn, steps: int = 3, warmup: int = 1):
    for _ in range(warmup):
        rc = fn()
        if rc < 0:
            raise SystemExit(f"call failed: {rc}")
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


# Algorithmic bytes per symbol: PLCP = Phi (SA read 4, Phi written 4) + the
# Kasai pass (Phi read 4, PLCP written 4, ~2 text bytes amortised); LCP = SA
# read 4, PLCP gathered 4, LCP written 4.
PLCP_BYTES_PER_SYMBOL = 18
LCP_BYTES_PER_SYMBOL = 12


def run_plcp_lcp(G, torch, dT, dSA, n: int, T=None, O=None, gsa: bool = False):
    """PLCP and LCP of the resident text and SA, with their HBM rooflines
    (algorithmic bytes / time / measured copy bandwidth); checked against the
    oracle when T and O are given."""
    peak, kind = peaks()
    dP = torch.empty_like(dSA)
    dL = torch.empty_like(dSA)
    stream = torch.cuda.current_stream()
    plcp_ms = _timed(torch, lambda: G.plcp_device(dT, dSA, dP, gsa=gsa, stream=stream))
    lcp_ms = _timed(torch, lambda: G.lcp_device(dP, dSA, dL, stream=stream))
    out = {"plcp_mb_s": round(n / 1e6 / (plcp_ms / 1e3), 1), "plcp_ms": round(plcp_ms, 3),
           "lcp_mb_s": round(n / 1e6 / (lcp_ms / 1e3), 1), "lcp_ms": round(lcp_ms, 3),
           "roofline": {"plcp": round(PLCP_BYTES_PER_SYMBOL * n / (plcp_ms / 1e3) / 1e9 / peak, 4),
                        "lcp": round(LCP_BYTES_PER_SYMBOL * n / (lcp_ms / 1e3) / 1e9 / peak, 4),
                        "unit": f"fraction of {peak} GB/s ({kind})",
                        "bytes_per_symbol": {"plcp": PLCP_BYTES_PER_SYMBOL, "lcp": LCP_BYTES_PER_SYMBOL}}}
    if T is not None and O is not None:
        SA = dSA.cpu().numpy().astype(np.int64)
        oP = O.plcp(T, SA, gsa=gsa)
        out["plcp_equals_oracle"] = bool(np.array_equal(dP.cpu().numpy().astype(np.int64), oP))
        out["lcp_equals_oracle"] = bool(np.array_equal(dL.cpu().numpy().astype(np.int64), O.lcp(oP, SA)))
    return out


def run_stress(G, torch, names=("all_A_2^26", "period7_2^26"), steps: int = 3):
    """The degenerate texts at n = 2^26: SA+BWT device-resident, checked against
    the oracle (SA check, BWT and primary index, PLCP and LCP)."""
    from oracle.oracle import Oracle
    O = Oracle()
    out = {}
    for name in names:
        n = WORKLOADS[name][1]
        T = make_text(name, n)
        dT = torch.from_numpy(T).cuda()
        dSA = torch.empty(n, dtype=torch.int32, device="cuda")
        dU = torch.empty(n, dtype=torch.uint8, device="cuda")
        stream = torch.cuda.current_stream()
        prim = G.sa_bwt_device(dT, dSA, dU, stream=stream)
        ms = _timed(torch, lambda: G.sa_bwt_device(dT, dSA, dU, stream=stream), steps=steps)
        st = G.last_stats()
        ok = oracle_check_sa_bwt(O, T, dSA.cpu().numpy(), dU.cpu().numpy(), prim)
        pl = run_plcp_lcp(G, torch, dT, dSA, n, T, O)
        out[name] = {"n": n, "sa_bwt_mb_s": round(n / 1e6 / (ms / 1e3), 1), "sa_bwt_ms": round(ms, 3),
                     "rounds": st["rounds"], "radix_passes": st["radix_passes"], "sa_bwt_equals_oracle": bool(ok),
                     "plcp_ms": pl["plcp_ms"], "lcp_ms": pl["lcp_ms"],
                     "plcp_lcp_equal_oracle": bool(pl["plcp_equals_oracle"] and pl["lcp_equals_oracle"])}
        del dT, dSA, dU
        G.release_workspace()
        torch.cuda.empty_cache()
    return out


def run_unbwt(G, U: np.ndarray, primary: int, T: np.ndarray, steps: int = 3, cpu_sample: int = 1 << 24):
    """Inverse BWT of the workload's BWT through libsais_unbwt (host buffers:
    the BWT goes up and the text comes back inside the timed call), the
    device part from the library's CUDA events, and the oracle's LF walk on a
    prefix-sized sample for scale."""
    import time as _t
    out = np.empty_like(U)
    rc, _ = G.libsais_unbwt(U, primary, out=out)
    if rc != 0 or not np.array_equal(out, T):
        raise SystemExit(f"libsais_unbwt did not give the text back: {rc}")
    G.profile_reset()
    G.profile_enable(True)
    t0 = _t.perf_counter()
    for _ in range(steps):
        G.libsais_unbwt(U, primary, out=out)
    host_s = (_t.perf_counter() - t0) / steps
    G.profile_enable(False)
    dev = G.profile_read().get("unbwt", {"launches": 0, "total_ms": 0.0})
    dev_ms = dev["total_ms"] / max(dev["launches"], 1)
    n = U.size
    res = {"n": n, "e2e_mb_s": round(n / 1e6 / host_s, 1), "e2e_ms": round(host_s * 1e3, 3),
           "device_mb_s": round(n / 1e6 / (dev_ms / 1e3), 1) if dev_ms else None, "device_ms": round(dev_ms, 3),
           "round_trip_identical": True}
    try:
        from oracle.oracle import Oracle
        O = Oracle()
        m = min(cpu_sample, n)
        Ts = T[:m]
        p, Us, _, _ = O.libsais_bwt(Ts)
        t0 = _t.perf_counter()
        O.unbwt(Us, p)
        res["cpu_port_mb_s"] = round(m / 1e6 / (_t.perf_counter() - t0), 1)
        res["cpu_sample"] = f"first {m} symbols, LF walk, 1 thread"
    except Exception as exc:   # the oracle is a reported scale only
        res["cpu_port_mb_s"] = None
        res["cpu_note"] = str(exc)[:80]
    return res


def run_gsa(G, torch, reads: int = 1 << 20):
    """Generalized SA + GSA-PLCP + LCP of the read set: 2^20 reads of length
    N(150, 20) clipped to [50, 300] from a 4 Mbp reference with 1% substitutions,
    each terminated by byte 0.  Checked against the oracle's linear-time SA
    checker and its PLCP."""
    from libsais_gb300 import textgen
    from oracle.oracle import Oracle
    T = textgen.reads_gsa(reads, ref_len=4_000_000, seed=4)
    n = T.size
    dT = torch.from_numpy(T).cuda()
    dSA = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    sa_ms = _timed(torch, lambda: G.sa_device(dT, dSA, gsa=True, stream=stream))
    split = _kernel_split(G, torch, lambda: G.sa_device(dT, dSA, gsa=True, stream=stream))
    st = G.last_stats()
    O = Oracle()
    pl = run_plcp_lcp(G, torch, dT, dSA, n, T, O, gsa=True)
    ok_sa = O.check_sa(T, dSA.cpu().numpy().astype(np.int64), gsa=True)
    return {"reads": reads, "n": n, "gsa_mb_s": round(n / 1e6 / (sa_ms / 1e3), 1), "gsa_ms": round(sa_ms, 3),
            "rounds": st["rounds"], "seed_symbols": st["seed_symbols"], "active_total": st["active_total"],
            "large_total": st["large_total"], "kernels_ms": split,
            "plcp_gsa_mb_s": pl["plcp_mb_s"], "lcp_mb_s": pl["lcp_mb_s"], "sa_valid": bool(ok_sa),
            "plcp_matches_oracle": pl["plcp_equals_oracle"], "lcp_matches_oracle": pl["lcp_equals_oracle"]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="genome_like_2^28", choices=sorted(WORKLOADS))
    ap.add_argument("--n", type=int, default=0, help="override the workload length")
    ap.add_argument("--ref-sample", type=int, default=REF_SAMPLE)
    ap.add_argument("--baseline-child", action="store_true",
                    help="reference arm as the cpu_baseline of the other arm: 1 warm-up, 1 timed step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--seed-key-bits", type=int, default=0)
    ap.add_argument("--no-extras", action="store_true", help="skip the measurements beside the headline")
    ap.add_argument("--extras", default="all",
                    help="comma-separated subset of plcp_lcp,unbwt,stress,gsa,batched,serving (default all)")
    ap.add_argument("--batch-strings", type=int, default=4096)
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (built-in tuning defaults)")
    ap.add_argument("--serving-jobs", type=int, default=20000, help="jobs per arrival rate of the serving stream")
    ap.add_argument("--serving-cpu", type=int, default=0, help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.baseline_child:
        args.steps, args.warmup = 1, 1
    else:
        args.warmup = max(args.warmup, 3)

    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch

    import libsais_gb300 as G

    torch.cuda.set_device(local)
    name = args.workload
    n = args.n or WORKLOADS[name][1]
    T = make_text(name, n)
    if args.seed_key_bits:
        G.set_seed_key_bits(args.seed_key_bits)
    tuning = None
    if not args.no_tune:
        # untimed: the autotuner picks this GPU's tile shape and group cut-overs
        # for the workload's (n bucket, code bits) and caches them; every sort
        # below (device and host paths) then runs with that entry
        from libsais_gb300 import autotune
        bits = 2 if WORKLOADS[name][0] == "genome_like" else None
        if bits is not None:
            tuning = autotune.tune(n, bits=bits, text=T, steps=3)
        G.release_workspace()
        torch.cuda.empty_cache()
    dT = torch.from_numpy(T).cuda()
    dSA = torch.empty(n, dtype=torch.int32, device="cuda")
    dU = torch.empty(n, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream()

    prim = None
    for _ in range(args.warmup):
        prim = G.sa_bwt_device(dT, dSA, dU, stream=stream)
        if prim < 0:
            raise SystemExit(f"gsais_sa_bwt_device failed: {prim}")
    stats = G.last_stats()
    used_tuning = G.last_tuning()

    # ---- device-resident timed region
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    torch.cuda.synchronize()
    launches0 = G.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        p = G.sa_bwt_device(dT, dSA, dU, stream=stream)
        if p != prim:
            raise SystemExit(f"primary index changed between steps: {p} vs {prim}")
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    launches = G.launch_count() - launches0
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    ms = reduce_max(dist, ms)
    value = world * n / 1e6 / (ms / 1e3)

    # ---- per-kernel times: the same K steps again with CUDA events recorded
    # around every launch on the launching stream (kept out of the timed region
    # above, where the events would add ~0.5 ms per step)
    torch.cuda.synchronize()
    G.profile_reset()
    G.profile_enable(True)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    for _ in range(args.steps):
        G.sa_bwt_device(dT, dSA, dU, stream=stream)
    p1.record(stream)
    torch.cuda.synchronize()
    G.profile_enable(False)
    prof = G.profile_read()
    profiled_ms = p0.elapsed_time(p1) / args.steps

    # ---- dominant kernel roofline (radix digit pass), from the same timed region
    peak, peak_kind = peaks()
    ks = prof.get("radix_pass", {"launches": 0, "total_ms": 0.0, "bytes": 0})
    roof = None
    if ks["launches"]:
        per_launch_ms = ks["total_ms"] / ks["launches"]
        per_launch_bytes = ks["bytes"] / ks["launches"]
        achieved = per_launch_bytes / (per_launch_ms / 1e3) / 1e9
        traffic = None
        tfile = os.path.join(ROOT, "profiles", "radix_pass_traffic.json")
        if os.path.exists(tfile):
            with open(tfile) as f:
                tr = json.load(f)
            traffic = round(tr["dram_bytes_per_algorithmic_byte"] * per_launch_bytes, 0)
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic, "peak_source": peak_kind,
                "kernel": "k_radix_pass", "launches_per_step": ks["launches"] / args.steps,
                "algorithmic_bytes_per_launch": int(per_launch_bytes), "ms_per_launch": round(per_launch_ms, 4),
                "timing": f"CUDA events around each launch over {args.steps} steps run right after the timed "
                          f"region ({profiled_ms:.3f} ms per step with the events)"}
    kernels = {}
    step_bytes = 0
    for k, v in prof.items():
        if not v["launches"]:
            continue
        kms = v["total_ms"] / args.steps
        kb = v["bytes"] / args.steps
        step_bytes += kb
        kernels[k] = {"launches_per_step": v["launches"] / args.steps, "ms_per_step": round(kms, 3),
                      "algorithmic_bytes_per_step": int(kb),
                      "hbm_frac": round(kb / (kms / 1e3) / 1e9 / peak, 4) if kms > 0 and kb else None}
    step_roof = {"algorithmic_bytes_per_step": int(step_bytes),
                 "achieved_gbs": round(step_bytes / (ms / 1e3) / 1e9, 1),
                 "frac": round(step_bytes / (ms / 1e3) / 1e9 / peak, 4), "peak": peak, "peak_source": peak_kind,
                 "compulsory_bytes_per_step": 6 * n,
                 "note": "sum of the algorithmic bytes of the timed kernels per step over ms_per_step"}

    # ---- end to end through the drop-in libsais API from pinned host buffers
    e2e, e2e_one_sort = None, None
    if not args.no_e2e:
        hT = torch.from_numpy(T).pin_memory()
        hSA = torch.empty(n, dtype=torch.int32).pin_memory()
        hU = torch.empty(n, dtype=torch.uint8).pin_memory()
        hA = np.empty(n, dtype=np.int32)   # libsais_bwt's temporary array (not written by this library)
        hF = np.zeros(256, dtype=np.int32)
        lib = G.load()

        def dropin():
            rc = lib.libsais(hT.data_ptr(), hSA.data_ptr(), n, 0, hF.ctypes.data)
            p = lib.libsais_bwt(hT.data_ptr(), hU.data_ptr(), hA.ctypes.data, n, 0, hF.ctypes.data)
            return p if rc == 0 else rc

        one_sort = lambda: lib.gsais_sa_bwt(None, hT.data_ptr(), 1, n, hSA.data_ptr(), 4, hU.data_ptr(), None, 4)
        for fn, label in ((dropin, "libsais + libsais_bwt"), (one_sort, "gsais_sa_bwt")):
            hSA.fill_(-1)
            hU.fill_(0)
            if fn() != prim:
                raise SystemExit(f"host path ({label}): primary index differs from the device path")
            if not (torch.equal(hSA, dSA.cpu()) and torch.equal(hU, dU.cpu())):
                raise SystemExit(f"host path ({label}): SA/BWT differ from the device path")
        res = {}
        for fn, key in ((dropin, "dropin"), (one_sort, "one_sort")):
            for _ in range(max(args.warmup - 1, 1)):   # untimed: the first DMAs map the pinned pages
                fn()
            barrier(dist)
            t0 = time.perf_counter()
            step_ms = []
            for _ in range(args.steps):
                t1 = time.perf_counter()
                fn()
                step_ms.append((time.perf_counter() - t1) * 1e3)
            dt = reduce_max(dist, (time.perf_counter() - t0) / args.steps)
            res[key] = (dt, step_ms)
        dt, step_ms = res["dropin"]
        e2e = {"value": round(world * n / 1e6 / dt, 3), "unit": UNIT, "h2d_bytes_per_step": 2 * n,
               "d2h_bytes_per_step": n * 4 + n, "ms_per_step": round(dt * 1e3, 3),
               "step_ms_min_max": [round(min(step_ms), 3), round(max(step_ms), 3)],
               "step_ms_median": round(statistics.median(step_ms), 3),
               "api": "libsais() then libsais_bwt() on pinned host buffers (two sorts; the text goes up twice)",
               "note": "value = mean over the timed steps; host-side steps of the shared box vary more than "
                       "device ones (see the median and the fastest step)"}
        dt, step_ms = res["one_sort"]
        e2e_one_sort = {"value": round(world * n / 1e6 / dt, 3), "unit": UNIT, "h2d_bytes_per_step": n,
                        "d2h_bytes_per_step": n * 4 + n, "ms_per_step": round(dt * 1e3, 3),
                        "step_ms_min_max": [round(min(step_ms), 3), round(max(step_ms), 3)],
                        "step_ms_median": round(statistics.median(step_ms), 3),
                        "api": "gsais_sa_bwt (SA and BWT from one sort) on pinned host buffers"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_child(name, n)

    extras = {}
    want = {"plcp_lcp", "unbwt", "stress", "gsa", "batched", "serving"}
    if args.extras != "all":
        want &= set(args.extras.split(","))
    if rank == 0 and world == 1 and not args.no_extras:
        from oracle.oracle import Oracle
        O = Oracle()
        if "plcp_lcp" in want:
            extras["plcp_lcp"] = run_plcp_lcp(G, torch, dT, dSA, n, T, O)
        if "unbwt" in want:
            extras["unbwt"] = run_unbwt(G, dU.cpu().numpy(), prim, T)
        del dT, dSA, dU
        G.release_workspace()
        torch.cuda.empty_cache()
        if "stress" in want:
            extras["stress"] = run_stress(G, torch)
        if "gsa" in want:
            extras["gsa"] = run_gsa(G, torch)
        G.release_workspace()
        if "batched" in want:
            extras["batched"] = run_batched(G, torch, count=args.batch_strings)
        G.release_workspace()
        torch.cuda.empty_cache()
        if "serving" in want:
            extras["serving"] = run_serving(G, torch, jobs_per_rate=args.serving_jobs)
            extras["serving"]["cpu_reference"] = serving_cpu_child(40, args.serving_jobs)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": bench_config(name, n),
            "placement": "replicas" if world > 1 else "single GPU",
            "sort_stats": {"rounds": stats["rounds"], "seed_symbols": stats["seed_symbols"],
                           "radix_passes": stats["radix_passes"], "active_total": stats["active_total"],
                           "pairs_direct": stats["pairs_direct"], "large_total": stats["large_total"]},
            "tuning": {"used": used_tuning, "autotuned": tuning},
            "roofline": roof, "step_roofline": step_roof, "cpu_baseline": cpu, "e2e": e2e,
            "e2e_one_sort": e2e_one_sort, "gpu_launches": launches, "kernels": kernels, "clocks": clocks,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
