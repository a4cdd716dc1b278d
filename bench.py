"""Benchmark of the satsuma2 cross-correlation path on GB300.

Metric: chunk-pairs/s (4096 bp x 4096 bp, both strands), the batched uniform
workload (4096 seeded pairs, homolog length U[200,3500], identity U[70,95]%, 25%
unrelated, 25% reverse-complemented; FFT length 8192, cutoff 1.8).  One "step" =
one pass over that batch.

JSON line (rank 0):
  value         device-resident batch throughput (inputs already in HBM),
                CUDA events on the launching stream, L2 flushed before each step
  e2e           the same through xc_align_pairs with host buffers (pinned
                staging copy, H2D, kernels, D2H and t_result assembly timed)
  plain / served   one pair per call vs continuous-batching serving, and the
                served p50/p99 request latency
  roofline      correlation stage's FP32 work against the FP32 pipe peak
  roofline_scan DoOne window checks per second of the scan kernel, with its
                integer-pipe use from the ncu capture under profiles/
  cpu_baseline  the reference CPU path on this host's cores (bounded sample)
  other_configs device-resident throughput of the uneven-length batch (20000
                pairs, FFT 1024..8192) and of 16384-bp chunks at FFT 32768

--impl reference runs the reference's CPU implementation on the host cores
(the compiled reference when it loads here, else the oracle restatement) and
prints the same metric.

Multi-GPU: the path has no exchange step, so N GPUs run N independent replicas
of the batch ("replicas only"); value = pairs of all ranks / max rank time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import queue as queue_mod
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "chunk-pairs/s (4096bp, both strands) served vs plain on 1 GB300; p50/p99 ms"
UNIT = "chunk-pairs/s"
N_PAIRS = 4096
SEED = 42
TARGET_TOTAL = 4096.0 * 4096   # sum of the target lengths of the workload
L2_FLUSH_BYTES = 512 << 20


def workload(rank=0):
    """Rank r's shard: its own seeded batch (rank 0 is the single-GPU workload)."""
    from satsuma2_gb300 import workloads as W
    return W.uniform_batch(N_PAIRS, seed=shard_seed(rank))


def shard_seed(rank):
    return SEED + rank


def max_over_ranks(v, world):
    """The largest of each rank's v (the slowest rank's time); v itself at N=1."""
    if world <= 1:
        return float(v)
    import torch
    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def fft_flops_per_pair(L=8192):
    """Algorithmic FP32 work of one pair, both strands: 4 target + 8 query
    forward real FFTs + 2 inverse (channel sum by linearity) at 2.5 L log2 L
    each, plus the 4-channel conjugate product-sum (8 flops per bin)."""
    F = 2.5 * L * np.log2(L)
    return 14 * F + 2 * 4 * (L // 2) * 8


def sampled_window_checks(x, items, n=64):
    """DoOne work per pair, both strands: window checks summed over the
    FindTop offsets (the overlap of each diagonal less the 46-base window),
    from the offsets the GPU keeps for n pairs spread over the batch."""
    samp = items[::max(1, len(items) // n)][:n]
    tot = 0
    for t, q in samp:
        d = x.debug_pair(t=t, q=q, signals=False)
        half = d["L"] // 2
        T, Q = len(t), len(q)
        for s in range(2):
            pos = d["offsets"][s].astype(np.int64) - half
            i0 = np.maximum(0, -pos)
            iend = np.minimum(T - 1, Q - pos)
            tot += int(np.maximum(0, iend - i0 - 46).sum())
    return tot / len(samp)


def _ref_worker(conn, shard, fft_len, target_total, use_port):
    """One single-threaded CPU process: the reference's own cross-correlation
    path (oracle/_ref, compiled from the reference's sources) or, where that
    library is absent, the oracle's C restatement, over its shard of pairs
    each time the parent asks."""
    import oracle
    if use_port:
        O = oracle.Oracle()
        P = O.params(target_total=target_total, fft_len=fft_len)
        pairs = [O.pair(t, q) for t, q in shard]

        def run(k):
            O.align_batch(P, pairs[:k], 1)
            return k
    else:
        ref = oracle.Reference()

        def run(k):
            for t, q in shard[:k]:
                ref.align_pair(t, q, fft_len, target_total=target_total)
            return k
    conn.send("ready")
    while True:
        k = conn.recv()
        if k is None:
            return
        conn.send(run(len(shard) if k < 0 else k))


class RefPool:
    """One single-threaded process per host core, each holding its shard of
    the workload (round robin), started with spawn.  step(k) has every process
    run its first k pairs (all of them for k < 0) and returns (pairs, seconds)
    of wall time."""

    def __init__(self, items, fft_len=8192, target_total=TARGET_TOTAL, procs=None):
        import multiprocessing as mp
        import oracle
        self.use_port = not os.path.exists(oracle.REF_SO)
        self.kind = "port" if self.use_port else "reference"
        self.procs = procs or os.cpu_count() or 1
        ctx = mp.get_context("spawn")
        self.conns, self.ps = [], []
        for k in range(self.procs):
            a, b = ctx.Pipe()
            pr = ctx.Process(target=_ref_worker, args=(b, items[k::self.procs], fft_len, target_total,
                                                       self.use_port), daemon=True)
            pr.start()
            self.conns.append(a)
            self.ps.append(pr)
        for c, pr in zip(self.conns, self.ps):
            if not c.poll(300) or c.recv() != "ready":
                self.close()
                raise RuntimeError("reference worker process %d did not start" % pr.pid)

    def step(self, k=-1):
        t0 = time.perf_counter()
        for c in self.conns:
            c.send(k)
        done = sum(c.recv() for c in self.conns)
        return done, time.perf_counter() - t0

    def close(self):
        for c in self.conns:
            try:
                c.send(None)
            except OSError:
                pass
        for pr in self.ps:
            pr.join(timeout=10)
            if pr.is_alive():
                pr.terminate()


def host_cpu():
    """(cores, CPU model) of this host."""
    model = ""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return os.cpu_count() or 1, model


def cpu_baseline(items, seconds=12.0):
    """The reference CPU path on a bounded sample of the workload: one
    single-threaded process per host core, repeated passes over 24 pairs per
    process until about `seconds` have passed."""
    cores, model = host_cpu()
    per = 24
    pool = RefPool(items[:per * cores])
    try:
        pool.step(1)   # warm: libraries loaded, tables built
        done, dt = 0, 0.0
        while dt < seconds:
            n, t = pool.step(-1)
            done += n
            dt += t
    finally:
        pool.close()
    what = ("the reference's own CPU code (oracle/_ref, compiled from its sources)" if pool.kind == "reference"
            else "the oracle's C restatement of the reference CPU path (the compiled reference is absent)")
    return {"value": done / dt, "unit": UNIT, "cores": cores, "kind": pool.kind,
            "sample": "%d pairs of the uniform 4096x4096 workload (FFT 8192) through %s, one single-threaded "
                      "process per core on %d cores (%s), %.1f s" % (done, what, cores, model, dt)}


def run_reference(args):
    """--impl reference: the reference's CPU implementation of the path over the
    same 4096-pair workload, one single-threaded process per host core; each
    step is one full pass over the batch."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    items = workload()
    cores, model = host_cpu()
    pool = RefPool(items)
    try:
        for _ in range(args.warmup):
            pool.step(-1)
        ts = []
        for _ in range(args.steps):
            n, dt = pool.step(-1)
            assert n == len(items)
            ts.append(dt)
    finally:
        pool.close()
    ms = 1000.0 * float(np.mean(ts))
    v = len(items) / (ms / 1000.0)
    what = ("the reference's own CPU code (oracle/_ref, compiled from its sources)" if pool.kind == "reference"
            else "the oracle's C restatement of the reference CPU path (the compiled reference is absent)")
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
           "data": "synthetic (seeded uniform batch, seed %d)" % SEED,
           "config": bench_config(1),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": pool.kind,
                            "sample": "the full %d-pair batch per step through %s, one single-threaded process "
                                      "per core on %d cores (%s)" % (len(items), what, cores, model)},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def bench_config(world):
    """The workload's config object, the same in both arms."""
    return {"workload": "batched uniform: %d chunk pairs 4096x4096 bp, both strands, FFT 8192, "
                        "cutoff 1.8, min_prob 0.99 (slave-faithful), seed %d" % (N_PAIRS, SEED),
            "pairs_per_step": N_PAIRS, "fft_len": 8192, "target_total": TARGET_TOTAL,
            "l2": "512 MB buffer written before every timed step (inputs 33.6 MB)",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def serve_run(x, items, n_threads=4, req_pairs=64, total=16384, rate=None, eager_wait=False, depth=8):
    """Submits requests from n_threads threads; rate (pairs/s) None = as fast as
    admission allows.  eager_wait: a waiter thread per client collects each
    ticket as soon as it is ready (latency as seen by a blocked caller).
    depth: requests a client keeps outstanding before it waits for its oldest.
    Returns (pairs/s, p50, p99)."""
    import satsuma2_gb300 as sg
    # requests built ahead of the clock: the measured path is submit/wait
    reqs = [sg.make_pairs([items[(i * req_pairs + j) % len(items)] for j in range(req_pairs)])
            for i in range(total // req_pairs)]
    lat = []
    lock = threading.Lock()
    t_start = time.perf_counter()
    per_thread = [reqs[k::n_threads] for k in range(n_threads)]
    arrivals = None
    if rate:
        rng = np.random.default_rng(7)
        gaps = rng.exponential(req_pairs / rate, size=len(reqs))
        arrivals = np.cumsum(gaps)

    def waiter(q):
        # collects tickets in submission order as soon as each is ready
        while True:
            item = q.get()
            if item is None:
                return
            tk, t0 = item
            x.wait(tk, timeout_ms=120000)
            with lock:
                lat.append(time.perf_counter() - t0)

    def worker(k):
        tickets = []
        wq, wt = None, None
        if eager_wait:
            wq = queue_mod.Queue()
            wt = threading.Thread(target=waiter, args=(wq,))
            wt.start()
        for j, r in enumerate(per_thread[k]):
            if arrivals is not None:
                due = arrivals[k + j * n_threads]
                now = time.perf_counter() - t_start
                if due > now:
                    time.sleep(due - now)
            while True:
                try:
                    t0 = time.perf_counter()
                    tk = x.submit(r)
                    break
                except sg.XCError as e:
                    if e.code != -8:
                        raise
                    time.sleep(0.0005)
            if eager_wait:
                wq.put((tk, t0))
                continue
            tickets.append((tk, t0))
            # keep a bounded number in flight per thread
            while len(tickets) >= depth:
                tk, t0 = tickets.pop(0)
                x.wait(tk, timeout_ms=120000)
                with lock:
                    lat.append(time.perf_counter() - t0)
        for tk, t0 in tickets:
            x.wait(tk, timeout_ms=120000)
            with lock:
                lat.append(time.perf_counter() - t0)
        if eager_wait:
            wq.put(None)
            wt.join()

    th = [threading.Thread(target=worker, args=(k,)) for k in range(n_threads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    dt = time.perf_counter() - t_start
    lat_ms = sorted(1000.0 * v for v in lat)
    p50 = lat_ms[len(lat_ms) // 2]
    p99 = lat_ms[min(len(lat_ms) - 1, int(round(0.99 * (len(lat_ms) - 1))))]
    return len(reqs) * req_pairs / dt, p50, p99


_GENOME = {}


def genome_workload(seed=SEED):
    """The genome workload (config 3): target and query as uint8 arrays, their
    chunk tables (4096 bp; target overlap 1024) and the 24x24 blocks in
    grid-search order; built once per process."""
    if seed not in _GENOME:
        from satsuma2_gb300 import workloads as W
        t, q, (src, _) = W.serving_genomes(seed=seed, with_map=True)
        tb, qb = np.frombuffer(t, np.uint8), np.frombuffer(q, np.uint8)
        tc = np.array(W.chunk_starts(len(t), 4096, 1024), np.int64)
        qc = np.array(W.chunk_starts(len(q), 4096, 0), np.int64)
        _GENOME[seed] = (tb, qb, tc, qc, W.grid_search_blocks(src, len(tc), len(qc)))
    return _GENOME[seed]


def genome_serving(local, rates=(5000.0, 50000.0, 200000.0, 1000000.0, 2000000.0), seconds=3.0, seed=SEED):
    """Serving on the genome workload: a 20 Mb target (GC 41%) and a query
    derived from it at 80% identity with 30 inversions, 20 segmental
    duplications and 10% novel insertions, chunked as the slave chunks them
    (4096 bp; target overlap 1024), targetTotal = 20e6.  Requests are whole
    24x24 grid blocks (576 chunk pairs) in grid-search order
    (workloads.grid_search_blocks), arriving as a Poisson process at each
    rate for about `seconds`; a waiter thread collects each ticket as soon as
    it is ready.  Per rate: requests, p50/p99 latency (submit to results in
    hand) and the pairs/s completed."""
    import satsuma2_gb300 as sg
    tb, qb, tc, qc, blocks = genome_workload(seed)
    x = sg.XCorr(target_total=float(len(tb)), max_batch=4096, device=local)
    # warm with several blocks (their shapes differ: tails, spectra, yields)
    warm = [x.submit(sg.block_pairs(tb, tc, qb, qc, *blocks[-1 - i])) for i in range(8)]
    for tk in warm:
        x.wait(tk, timeout_ms=120000)
    out = {"workload": "20 Mb target, 80%% identity query (%d bp) with inversions, duplications, insertions; "
                       "%d target x %d query chunks; requests = 24x24 grid blocks in grid-search order "
                       "(%d blocks, %d pairs), Poisson arrivals" % (len(qb), len(tc), len(qc), len(blocks),
                                                                    sum((b[1] - b[0] + 1) * (b[3] - b[2] + 1)
                                                                        for b in blocks)),
           "target_total": float(len(tb)), "rates": {}}
    k0 = 0
    for rate in rates:
        n_req = max(16, int(rate * seconds / 576))
        reqs = [sg.block_pairs(tb, tc, qb, qc, *blocks[(k0 + i) % len(blocks)]) for i in range(n_req)]
        k0 += n_req
        rng = np.random.default_rng(int(rate))
        due = np.cumsum(rng.exponential(1.0, size=n_req) * np.array([len(r) for r in reqs]) / rate)
        lat, recs = [], [0]
        tq = queue_mod.Queue()
        lock = threading.Lock()

        def waiter():
            while True:
                item = tq.get()
                if item is None:
                    return
                tk, t0 = item
                res = x.wait(tk, timeout_ms=120000)
                with lock:
                    lat.append(time.perf_counter() - t0)
                    recs[0] += len(res)

        th = [threading.Thread(target=waiter) for _ in range(4)]
        for w in th:
            w.start()
        t_start = time.perf_counter()
        for i, r in enumerate(reqs):
            d = due[i] - (time.perf_counter() - t_start)
            if d > 0:
                time.sleep(d)
            while True:
                try:
                    t0 = time.perf_counter()
                    tk = x.submit(r)
                    break
                except sg.XCError as e:
                    if e.code != -8:
                        raise
                    time.sleep(0.0005)
            tq.put((tk, t0))
        for _ in th:
            tq.put(None)
        for w in th:
            w.join()
        dt = time.perf_counter() - t_start
        lm = sorted(1000.0 * v for v in lat)
        pairs = sum(len(r) for r in reqs)
        out["rates"]["%d" % int(rate)] = {
            "requests": n_req, "pairs": pairs, "records": recs[0], "seconds": dt,
            "pairs_per_s": pairs / dt, "p50_ms": lm[len(lm) // 2],
            "p99_ms": lm[min(len(lm) - 1, int(round(0.99 * (len(lm) - 1))))], "max_ms": lm[-1]}
    x.close()
    return out


def run_ours(args):
    import torch
    import satsuma2_gb300 as sg
    from satsuma2_gb300 import build
    rank, world, local = dist_env()
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")
    torch.cuda.set_device(local)
    build.build()
    items = workload(rank)
    x = sg.XCorr(target_total=TARGET_TOTAL, device=local)
    # A dedicated stream: the library captures its launches into a CUDA graph,
    # which the legacy default stream does not allow.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    sptr = ctypes.c_void_p(stream.cuda_stream)
    batch = x.upload(items)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        batch.run(sptr)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- timed region: K device-resident steps, each one replay of the
    #      batch's CUDA graph as xc_batch_run runs it ----
    step_ms, stage = [], []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            batch.run(sptr)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    # stage times from the graph with stage events (about 2% slower than the
    # plain graph), after the timed region, L2 flushed the same way
    for k in range(args.steps):
        flush.zero_()
        stage.append(batch.run_timed(sptr))
    torch.cuda.synchronize()
    ms = max_over_ranks(float(np.mean(step_ms)), world)
    value = N_PAIRS * world / (ms / 1000.0)
    launches = args.steps * batch.launches()
    res_dev = batch.results()
    checks_per_pair = sampled_window_checks(x, items)

    # ---- end to end through the C ABI with host buffers ----
    arr, keep = sg.make_pairs(items)
    cap = max(64, 32 * len(items))
    out = np.zeros(cap, sg.RESULT_DTYPE)
    n_out = ctypes.c_size_t()
    for _ in range(max(args.warmup, 3)):
        sg._check(x.lib.xc_align_pairs(x.ctx, arr, len(arr), out.ctypes.data, cap, ctypes.byref(n_out), None), "e2e")
    e2e_t = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sg._check(x.lib.xc_align_pairs(x.ctx, arr, len(arr), out.ctypes.data, cap, ctypes.byref(n_out), None), "e2e")
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t0)
    h2d, d2h = x.transfer_stats()
    e2e_val = N_PAIRS * world / max_over_ranks(float(np.mean(e2e_t)), world)
    same = n_out.value == len(res_dev)

    # ---- plain: one pair per call ----
    plain_n = 256
    x.align([items[0]])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in items[:plain_n]:
        sg._check(x.lib.xc_align_pairs(x.ctx, sg.make_pairs([it])[0], 1, out.ctypes.data, cap,
                                       ctypes.byref(n_out), None), "plain")
    plain = plain_n / (time.perf_counter() - t0)

    # ---- served: continuous batching, saturating and at a fixed arrival rate ----
    xs = sg.XCorr(target_total=TARGET_TOTAL, device=local, max_batch=4096)
    # warm with the measured request shape: the slots meet their batch sizes
    # (graphs, buffers) here rather than in the first timed run
    serve_run(xs, items, n_threads=8, req_pairs=576, total=576 * 64, depth=3)
    # saturating: 8 client threads, each request one grid block of 24 x 24
    # chunk pairs (the slave's t_pair unit), three requests outstanding per
    # client (24 blocks, 13.8k pairs in flight: enough to keep the device
    # busy -- 2.80 M pairs/s against 2.64 M with eight per client, whose
    # latency is queueing, ~12 ms) (three runs of 147k pairs, ~60 ms each;
    # the median run is reported: single runs vary with host scheduling)
    runs = sorted((serve_run(xs, items, n_threads=8, req_pairs=576, total=576 * 256, depth=3) for _ in range(3)),
                  key=lambda r: r[0])
    served, p50_sat, p99_sat = runs[1]
    xs.close()
    # latency and throughput on the genome workload: 24x24 grid blocks in
    # grid-search order at Poisson arrival rates
    config3 = genome_serving(local)
    p50 = config3["rates"]["200000"]["p50_ms"]
    p99 = config3["rates"]["200000"]["p99_ms"]
    rate = 200000.0

    # ---- the other configurations, for reference (device-resident batches,
    #      L2 flushed, median of 3 runs): uneven lengths over FFT buckets
    #      1024..8192, 16384-bp chunks at FFT 32768, and the benchmark batch
    #      at min_prob 0.99999.  After the timed runs each batch's records are
    #      read back (the call fails on any device error word) and its
    #      near-threshold FindTop lags counted. ----
    other = {}
    try:
        from satsuma2_gb300 import workloads as W

        def device_rate(xc, its, reps=3):
            b = xc.upload(its)
            for _ in range(2):
                b.run(sptr)
            torch.cuda.synchronize()
            first = len(b.results())
            ts = []
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            for _ in range(reps):
                flush.zero_()
                e0.record(stream)
                b.run(sptr)
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            recs = len(b.results())
            near, _ = b.straddles()
            b.free()
            return {"pairs": len(its), "pairs_per_s": len(its) / (float(np.median(ts)) / 1000.0),
                    "records": recs, "records_stable": recs == first, "near_threshold_lags": int(near.sum())}

        u = W.uneven_batch(20000, seed=SEED + rank)
        xu = sg.XCorr(fft_len=-1, target_total=float(sum(len(t) for t, _ in u)), device=local)
        other["uneven_20000_fft_1024_8192"] = device_rate(xu, u)
        # the same batch after the autotuner has picked each length's kernel form
        t0 = time.perf_counter()
        table = xu.tune()
        tune_s = time.perf_counter() - t0
        other["uneven_20000_fft_1024_8192_tuned"] = device_rate(xu, u)
        other["tuning"] = {"seconds": tune_s, "table": table.strip().splitlines()}
        xu.close()
        lg = W.large_batch(2000, seed=SEED + rank)
        xg = sg.XCorr(t_chunk=16384, q_chunk=16384, target_total=16384.0 * 2000, device=local)
        other["large_2000_16384bp_fft_32768"] = device_rate(xg, lg)
        xg.close()
        # 24x24 grid blocks of the genome workload as one device batch (7
        # blocks, 4032 pairs of 336 distinct chunks), correlation stage with
        # the spectra path (each chunk transformed once) and without it
        tb, qb, tc, qc, gblocks = genome_workload()
        gb_items = np.concatenate([sg.block_pairs(tb, tc, qb, qc, *bl) for bl in gblocks[:7]])
        for name, env in (("grid_blocks_4032_spectra_on", "1"), ("grid_blocks_4032_spectra_off", "0")):
            os.environ["SATSUMA2_GB300_SPECTRA"] = env
            xs = sg.XCorr(target_total=float(len(tb)), device=local)
            os.environ.pop("SATSUMA2_GB300_SPECTRA")
            rr = device_rate(xs, gb_items)
            bs = xs.upload(gb_items)
            for _ in range(2):
                bs.run(sptr)
            st_ms = []
            for _ in range(5):
                flush.zero_()
                st_ms.append(bs.run_timed(sptr))
            bs.free()
            rr["stage_ms"] = {"corr_findtop": float(np.median([v[0] for v in st_ms])),
                              "scan_filter": float(np.median([v[1] for v in st_ms]))}
            other[name] = rr
            xs.close()
        x5 = sg.XCorr(min_prob=0.99999, target_total=TARGET_TOTAL, device=local)
        other["uniform_4096_min_prob_0.99999"] = device_rate(x5, items)
        x5.close()
        nb, _ = batch.straddles()
        other["uniform_4096_min_prob_0.99_near_threshold_lags"] = int(nb.sum())
    except Exception as exc:   # informational only: never costs the main line
        other["error"] = str(exc)[:200]
    parity_path = os.path.join(ROOT, "profiles", "parity_bench_configs.json")
    parity = None
    if os.path.exists(parity_path):
        with open(parity_path) as f:
            parity = {"source": "tests/test_gpu_bench_scale.py on a GB300 (profiles/parity_bench_configs.json): "
                                "whole batches against the FP64 oracle", "configs": json.load(f)}

    peaks, peak_kind = measured_peaks()
    corr_ms = float(np.mean([s[0] for s in stage]))
    scan_ms = float(np.mean([s[1] for s in stage]))
    fin_ms = float(np.mean([s[2] for s in stage]))
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = 152 * 128 * 2 * sm_max * 1e6 / 1e12
    flops = fft_flops_per_pair() * N_PAIRS
    achieved = flops / (corr_ms / 1000.0) / 1e12
    traffic, counters = None, {}
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            counters = json.load(f)
        traffic = counters.get("corr_pair2_kernel_dram_bytes_per_launch")
    checks = checks_per_pair * N_PAIRS
    # the same algorithmic work on 24x24 grid blocks, where the spectra path
    # transforms each distinct chunk once
    grid_roof = None
    gon = other.get("grid_blocks_4032_spectra_on")
    if gon:
        gflops = fft_flops_per_pair() * gon["pairs"]
        ga = gflops / (gon["stage_ms"]["corr_findtop"] / 1000.0) / 1e12
        grid_roof = {"bound": "fp32", "kernel": "spec_kernel<13> + corr_spec_kernel<13> + hand-back",
                     "workload": "7 grid blocks of the genome workload, %d pairs" % gon["pairs"],
                     "achieved": ga, "peak": fp32_peak, "unit": "TFLOP/s", "frac": ga / fp32_peak,
                     "algorithmic_flops_per_launch": gflops}
    clocks = clk.summary()

    if rank != 0:
        return 0
    cpu = cpu_baseline(items, seconds=args.ref_seconds) if (world == 1 and not args.no_cpu) else None
    out_line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded uniform batch, seed %d)" % SEED,
        "config": bench_config(world),
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "results_match_device_run": bool(same)},
        "plain_pairs_per_s": plain, "served_pairs_per_s": served, "served_vs_plain": served / plain,
        "served_request_pairs": 576, "served_clients": 8, "served_outstanding_per_client": 3,
        "served_runs": "median of 3", "latency_request_pairs": 576,
        "served_p50_ms_saturated": p50_sat, "served_p99_ms_saturated": p99_sat,
        "p50_ms": p50, "p99_ms": p99, "latency_arrival_rate_pairs_per_s": rate,
        "latency_workload": "genome serving (config3 below): 576-pair grid-block requests at Poisson arrivals",
        "config3": config3,
        "stage_ms": {"corr_findtop": corr_ms, "scan_filter": scan_ms, "finalize": fin_ms},
        "roofline": {"bound": "fp32", "kernel": "corr_pair2_kernel<13> + corr_kernel<13> hand-back",
                     "achieved": achieved, "peak": fp32_peak,
                     "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": traffic,
                     "peak_source": "FP32 FMA pipe: 152 SMs x 128 lanes x 2 x %s sm_max_mhz (%s)"
                                    % (sm_max, peak_kind),
                     "algorithmic_flops_per_launch": flops,
                     "note": "algorithmic work is the reference's 14 real FFTs per pair; the kernel shares "
                             "spectra between strands and runs 8 forward + 2 inverse half-length transforms"},
        "roofline_grid_blocks": grid_roof,
        "roofline_scan": {"bound": "int-alu", "kernel": "scan_kernel<13>",
                          "work": "DoOne window checks over the kept offsets (sampled 64 pairs)",
                          "checks_per_launch": checks, "achieved": checks / (scan_ms / 1000.0) / 1e9,
                          "unit": "G window checks/s",
                          "alu_pipe_pct_ncu": counters.get("scan_kernel_alu_pipe_pct"),
                          "issue_active_pct_ncu": counters.get("scan_kernel_issue_active_pct"),
                          "traffic": counters.get("scan_kernel_dram_bytes_per_launch")},
        "gpu_launches": launches,
        "clocks": clocks,
        "cpu_baseline": cpu,
        "results_per_step": len(res_dev),
        "parity": parity,
        "other_configs": other,
    }
    print(json.dumps(out_line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def profile_case(args):
    """Fixed device-resident workload for profiler captures: uploads --pairs
    seeded uniform 4096x4096 chunk pairs (FFT 8192), with --case blocks
    the pairs of 24x24 grid blocks of the genome workload, with --case uneven
    the uneven-length batch (FFT 1024..8192), and runs the batch
    --runs times without timing, so a profiler's launch list maps one-to-one
    onto runs (each run: the correlation kernels, the scan kernel and the
    two finalize kernels)."""
    import satsuma2_gb300 as sg
    from satsuma2_gb300 import build, workloads
    build.build()
    if args.case == "blocks":   # 24x24 grid blocks of the genome workload (spectra path)
        tb, qb, tc, qc, blocks = genome_workload()
        items, k = [], 0
        while sum(len(a) for a in items) < args.pairs:
            items.append(sg.block_pairs(tb, tc, qb, qc, *blocks[k]))
            k += 1
        items = np.concatenate(items)[:args.pairs]
        x = sg.XCorr(target_total=float(len(tb)))
    elif args.case == "uneven":   # uneven lengths over the FFT buckets 1024..8192
        items = workloads.uneven_batch(args.pairs, seed=SEED)
        x = sg.XCorr(fft_len=-1, target_total=float(sum(len(t) for t, _ in items)))
    else:
        items = workloads.uniform_batch(args.pairs, seed=SEED)
        x = sg.XCorr(target_total=TARGET_TOTAL)
    b = x.upload(items)
    for _ in range(args.runs):
        b.run(ctypes.c_void_p(0))
    res = b.results()
    print("pairs %d runs %d results %d" % (args.pairs, args.runs, len(res)))
    b.free()
    x.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--profile-case", action="store_true",
                    help="profiler workload only: upload --pairs pairs and run them --runs times, untimed")
    ap.add_argument("--pairs", type=int, default=N_PAIRS)
    ap.add_argument("--case", default="uniform", choices=["uniform", "blocks", "uneven"],
                    help="profiler workload: uniform pairs, 24x24 grid blocks of the genome workload, "
                         "or the uneven-length batch")
    ap.add_argument("--runs", type=int, default=3)
    args = ap.parse_args()
    if args.profile_case:
        return profile_case(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
