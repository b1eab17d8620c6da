#!/usr/bin/env python
"""bench.py -- throughput of the batched best-first graph search on GB300.

One step = one batched search of the workload's query set (10,000 queries)
over the resident index.  Default workload: 1,000,000 x 128 float32 vectors
with integer values 0-255 (1,000-centre Gaussian mixture, sigma 20; a
synthetic stand-in for SIFT1M's shape), L2, degree-32 graph (shift 5,
FIXED_DEGREE 31, SEARCH_DEGREE 15) built batch-parallel (batch div 64),
top-10, recall@10 against an FP64 exact kNN (tie-aware, a repeated id counted
once).

The default mode measures three arms, each at the smallest pq of a sweep
whose recall@10 reaches the target (0.95), and reports the fastest:
  plain    the search from vertex 0 (the reference's semantics, FP32 rows);
  entries  the same search from each query's nearest entry vertices
           (two-level choice over sampled entries, song_index_set_entries_2level);
  learned  the learned early exit with BF16 rows and FP32 rerank, from the
           same entries.
Beside them: the pq sweep 50-400 of the entries arm at top-10 and top-100,
the top-100 figure, and learned+BF16 against FP32 from the same starts.

  value  queries/s of the reported arm's kernels, queries and index resident
         in HBM, CUDA events on the launching stream, L2 flushed between steps.
  e2e    queries/s through song_search (host query buffer in pinned memory,
         host->device copy, search, device->host copy of the ids), host clock.
  roofline  the search kernel (the step's dominant kernel), timed alone with
         the library's stage events (song_index_set_timing).

`--impl reference` runs the reference's own algorithms on the same workload:
its CPU best-first search (graph.h:169-216, restated in oracle/) on all host
cores over the same graph (built by the oracle's restatement of the
reference builder), at the result size k whose recall@10 matches the target;
and, where the reference's GPU kernel was rebuilt for sm_100 (oracle/_ref),
that kernel on this GPU at matched recall.  It leaves the latter in the cache
directory, where the default arm picks it up (same box, run before it).
Other modes: precision (storage error and recall per row format), serve
(Poisson request stream against two resident indexes), build (graph
construction, GPU vs CPU).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PQ_SWEEP = list(range(40, 50)) + [50, 55, 60, 65, 70, 75, 80, 90, 100, 125, 150, 175, 200, 225, 250, 300, 350, 400,
                                  500, 600, 800, 1000]
PQ_TABLE = [50, 75, 100, 150, 200, 250, 300, 400]   # the reported sweep (top-10; top-100 from pq 100)
CPU_K_SWEEP = [10, 20, 40, 80, 150, 300, 500, 800, 1200, 1600, 2000]
REF_GPU_PQ = [100, 200, 400, 600, 800, 1000]         # pq values of the rebuilt reference kernel


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", default=None,
                   help="default: scale-1m-128d-l2 (precision-1m-960d-cos for --mode precision)")
    p.add_argument("--pq", type=int, default=0, help="0 = smallest pq reaching --recall")
    p.add_argument("--recall", type=float, default=0.95)
    p.add_argument("--topk", type=int, default=10)
    p.add_argument("--nq", type=int, default=0)
    p.add_argument("--build-div", type=int, default=64)
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-table", action="store_true", help="skip the pq 50-400 top-10/top-100 table")
    p.add_argument("--cache", default=os.environ.get("SONG_CACHE", os.path.join(ROOT, "_cache")))
    p.add_argument("--curve", action="store_true", help="time every pq of the sweep (recall/throughput curve)")
    p.add_argument("--mode", choices=["best", "learned", "plain", "entries", "precision", "serve", "build"],
                   default="best",
                   help="best: measure the plain FP32 search (from vertex 0, the reference's semantics), the "
                        "same search from the nearest of --entries sampled entry vertices, and the learned "
                        "early exit + BF16 (+FP32 rerank), and report the fastest at the recall target; "
                        "plain / entries: that path only; learned: the early-exit study (vs the search "
                        "without it and a fixed hop budget, from vertex 0 and from entry points); "
                        "precision: storage error and recall table; serve: Poisson request stream; "
                        "build: graph construction, GPU searches vs the CPU builder")
    p.add_argument("--entries", type=int, default=524288, help="entry vertices of the entries arm (sampled, seeded)")
    p.add_argument("--starts", type=int, default=4, help="start vertices per query: its nearest entries")
    p.add_argument("--coarse", type=int, default=4096,
                   help="two-level entry choice: this many of the entries are cluster heads (0: flat)")
    p.add_argument("--probes", type=int, default=4, help="clusters searched per query (two-level choice)")
    p.add_argument("--multiprobe", default="2,2:1:1,4:1:1,1:2",
                   help="N_MULTIPROBE[:FINISH_CNT[:DOUBLE_CHECK]] settings measured beside the entries arm, each "
                        "at the smallest pq reaching --recall ('' to skip)")
    p.add_argument("--serve-rate", type=float, default=20000.0, help="mean offered queries/s (serve)")
    p.add_argument("--serve-seconds", type=float, default=6.0, help="length of each request stream (serve)")
    p.add_argument("--rerank", type=int, default=100, help="FP32 re-ranked candidates (BF16 path)")
    p.add_argument("--train-queries", type=int, default=20000)
    p.add_argument("--max-pq", type=int, default=1000, help="largest pq of the sweep (--mode learned)")
    p.add_argument("--recall-slack", type=float, default=0.004,
                   help="validation recall@10 the exit may give up against the same search without it")
    args = p.parse_args()
    if args.workload is None:
        args.workload = {"precision": "precision-1m-960d-cos", "learned": "learned-3m-256d-l2"}.get(
            args.mode, "scale-1m-128d-l2")
    return args


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else platform)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------

def graph_path(args, w):
    return os.path.join(args.cache, "%s.div%d.graph" % (w.name, args.build_div))


def load_workload(args, rank=0, barrier=None, builder="gpu"):
    """Data, queries and the degree-32 graph (cached).  builder: "gpu" (the
    product's GPU builder), "cpu" (its CPU builder) or "oracle" (the oracle's
    restatement of the reference builder); all three write the same graph
    bit for bit (tests/test_graph_build_gpu.py, tests/test_oracle_golden.py)."""
    from song_gb300 import datasets as D
    w = D.WORKLOADS[args.workload]
    nq = args.nq or w.n_queries
    t = time.time()
    data = D.base_vectors(w)
    queries = D.query_vectors(w, nq=nq)
    log("[bench] %s: data %s queries %s in %.1fs" % (w.name, data.shape, queries.shape, time.time() - t))
    os.makedirs(args.cache, exist_ok=True)
    gpath = graph_path(args, w)
    if rank == 0 and not os.path.exists(gpath):
        t = time.time()
        bargs = (data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150)
        if builder == "oracle":
            from oracle import oracle as O
            g = O.graph_build(*bargs, batch_div=args.build_div, nthreads=os.cpu_count())
        else:
            import song_gb300 as S
            fn = S.graph_build_gpu if builder == "gpu" else S.graph_build
            kw = {"device": int(os.environ.get("LOCAL_RANK", "0"))} if builder == "gpu" else {}
            g = fn(*bargs, batch_div=args.build_div, nthreads=os.cpu_count(), **kw)
        tmp = gpath + ".tmp%d" % os.getpid()
        g.tofile(tmp)
        os.replace(tmp, gpath)
        log("[bench] graph built in %.1fs (%s builder, batch_div %d, %d threads)"
            % (time.time() - t, builder, args.build_div, os.cpu_count()))
    if barrier:
        barrier()
    graph = np.fromfile(gpath, dtype=np.uint64)
    return w, data, queries, graph


def ground_truth(args, w, data, queries, k, device=None):
    """Exact k nearest ids and the exact 10th and k-th distances (FP64)."""
    from song_gb300 import groundtruth as GT
    path = os.path.join(args.cache, "%s.nq%d.k%d.gt.npz" % (w.name, queries.shape[0], k))
    if os.path.exists(path):
        z = np.load(path)
        return z["ids"], z["kth"], z["kth10"]
    t = time.time()
    ids, kth = GT.exact_knn_fp64(data, queries, k, w.metric, device=device)
    kth10 = GT.distances_fp64(data, queries, ids[:, min(k, 10) - 1:min(k, 10)], w.metric)[:, 0]
    np.savez(path, ids=ids, kth=kth, kth10=kth10)
    log("[bench] fp64 exact kNN (k=%d) in %.1fs" % (k, time.time() - t))
    return ids, kth, kth10


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

REASON_FIELDS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]


class ClockSampler:
    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap,utilization.gpu")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        return self.summary()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        loaded = [r for r in self.rows if num(r[7]) and num(r[7]) > 0] or self.rows
        sm = [num(r[0]) for r in loaded if num(r[0]) is not None]
        mx = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        reasons = set()
        for r in loaded:
            for name, v in zip(REASON_FIELDS, r[3:7]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows), "samples_under_load": len(loaded)}



# ---------------------------------------------------------------------------
# the reference's algorithms (oracle/): CPU search, and its GPU kernel rebuilt
# for sm_100
# ---------------------------------------------------------------------------

def cpu_calibrate_k(w, data, graph, queries, target, gt_kth10, sample=400):
    from oracle import oracle as O
    from song_gb300 import groundtruth as GT
    ox = O.OracleIndex(data, graph, w.shift, O.METRICS[w.metric])
    qs = queries[:sample]
    sweep = []
    for k in CPU_K_SWEEP:
        if k < 10:
            continue
        ids, _ = ox.cpu_search(qs, k)
        r = GT.recall_tie_aware(ids, data, qs, gt_kth10[:sample], w.metric, 10)
        sweep.append((k, round(r, 4)))
        if r >= target:
            return k, sweep
    return CPU_K_SWEEP[-1], sweep


def cpu_time(w, data, graph, queries, k, seconds, nthreads):
    """Times the CPU search on a sample sized to about `seconds` of work."""
    from oracle import oracle as O
    ox = O.OracleIndex(data, graph, w.shift, O.METRICS[w.metric])
    pilot = queries[:max(64, 8 * nthreads)]
    t = time.perf_counter()
    ox.cpu_search(pilot, k, nthreads=nthreads)
    rate = pilot.shape[0] / max(1e-6, time.perf_counter() - t)
    n = int(min(max(256, rate * seconds), 200_000))
    idx = np.arange(n) % queries.shape[0]
    sample = queries[idx]
    t = time.perf_counter()
    ox.cpu_search(sample, k, nthreads=nthreads)
    dt = time.perf_counter() - t
    return n / dt, n, dt


def reference_kernel_sm100(w, data, graph, queries, gt_kth10, target):
    """The reference's own GPU kernel (warp_astar_accelerator.h:41-341)
    rebuilt for sm_100 (oracle/_ref cubins), on this GPU: queries/s of each
    available pq_size (the faster of __ENABLE_MEASURE as shipped and
    removed) and the smallest pq whose recall@10 reaches the target."""
    from oracle import ref_gpu
    from song_gb300 import groundtruth as GT
    metric = w.metric
    pqs = [pq for pq in REF_GPU_PQ if ref_gpu.available(metric, w.dim, pq)]
    if not pqs:
        return {"unavailable": "reference cubins not built on this host (oracle/build_ref_gpu.sh)"}
    nq = queries.shape[0]
    rows = []
    chosen = None
    for pq in pqs:
        best = None
        for measure in (True, False):
            ids, ms = ref_gpu.run(ref_gpu.cubin_path(metric, w.dim, pq, measure), data, graph, w.shift, queries, pq,
                                  measure, repeats=3, heap_pq=max(pqs))
            qps = nq / (float(np.median(ms)) / 1000.0)
            if best is None or qps > best["qps"]:
                rec = GT.recall_tie_aware(ids[:, :10], data, queries, gt_kth10, metric, 10)
                best = {"pq": pq, "qps": round(qps, 1), "recall_at_10": round(rec, 4),
                        "measure_build": measure, "kernel_ms_median": round(float(np.median(ms)), 3)}
        rows.append(best)
        log("[reference sm_100] %s" % best)
        if chosen is None and best["recall_at_10"] >= target:
            chosen = best
    return {"at_target": chosen, "sweep": rows, "queries": nq,
            "kernel": "warp_astar_accelerator.h:41-341 rebuilt for sm_100 (compute_100), one launch per batch"}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU search on all host cores, over the
    same graph (the oracle's builder), and its GPU kernel rebuilt for sm_100."""
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    w, data, queries, graph = load_workload(args, builder="oracle")
    from song_gb300 import groundtruth as GT
    sample = min(400, queries.shape[0])
    _, _, kth10 = ground_truth(args, w, data, queries[:sample], args.topk, device="cpu")
    k, sweep = cpu_calibrate_k(w, data, graph, queries, args.recall, kth10, sample)
    nthreads = os.cpu_count() or 1
    nq = queries.shape[0]
    ox = O.OracleIndex(data, graph, w.shift, O.METRICS[w.metric])
    # a step searches a bounded slice of the workload's queries, sized so the
    # whole run takes about a minute and a half of CPU time
    rate, _, _ = cpu_time(w, data, graph, queries, k, 2.0, nthreads)
    per_step = int(max(64, min(nq, rate * 90.0 / max(1, args.steps + args.warmup))))
    for i in range(args.warmup):
        ox.cpu_search(queries[:per_step], k, nthreads=nthreads)
    times = []
    for i in range(args.steps):
        a = (i * per_step) % nq
        qs = queries[np.arange(a, a + per_step) % nq]
        t = time.perf_counter()
        ox.cpu_search(qs, k, nthreads=nthreads)
        times.append(time.perf_counter() - t)
    value = per_step * args.steps / sum(times)
    ref_gpu = None
    try:
        import torch
        if torch.cuda.is_available():
            _, _, kth10_all = ground_truth(args, w, data, queries, 100)
            ref_gpu = reference_kernel_sm100(w, data, graph, queries, kth10_all, args.recall)
            with open(os.path.join(args.cache, "%s.reference_sm100.json" % w.name), "w") as f:
                json.dump(ref_gpu, f)
    except Exception as e:  # the CPU baseline is this arm's value; the GPU kernel is context
        ref_gpu = {"error": repr(e)}
    line = {
        "impl": "reference", "metric": "queries/s at recall@10>=%.2f, %s" % (args.recall, w.name),
        "value": round(value, 1), "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * sum(times) / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 data, f64-accumulated distances", "data": "synthetic",
        "config": common_config(args, w, nq),
        "arm": {"name": "reference CPU best-first search (graph.h:169-216, oracle restatement), vertex-0 start",
                "k": k, "recall_sweep_k": sweep, "queries_per_step": per_step,
                "graph": "oracle/song_oracle.c orc_graph_build (the reference builder, batch div %d), equal to the "
                         "product builder's graph" % args.build_div},
        "cpu_baseline": {"value": round(value, 1), "unit": "queries/s", "cores": nthreads, "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": "%d queries per step (slices of the workload's query set), k=%d" % (per_step, k)},
        "reference_kernel_sm100": ref_gpu,
        "e2e": {"value": round(value, 1), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def common_config(args, w, nq):
    """The workload description, the same in both arms' lines."""
    return {"workload": w.name, "n": w.n, "dim": w.dim, "metric": w.metric, "top_k": args.topk,
            "recall_target": args.recall, "queries": nq,
            "graph": "shift %d (FIXED_DEGREE %d, SEARCH_DEGREE %d), budget 150, batch div %d"
                     % (w.shift, w.fixed_degree, w.search_degree, args.build_div)}


# ---------------------------------------------------------------------------
# ours
# ---------------------------------------------------------------------------

class Runner:
    """Device-buffer searches of one index over the resident query set."""

    def __init__(self, ix, dq, k, stream):
        import torch
        self.ix, self.dq, self.k, self.stream = ix, dq, k, stream
        nq = dq.shape[0]
        self.out = torch.empty((nq, k), dtype=torch.int64, device="cuda")
        self.hops = torch.empty(nq, dtype=torch.int32, device="cuda")
        self.evals = torch.empty(nq, dtype=torch.int32, device="cuda")

    def __call__(self, pq, stats=False):
        self.ix.search_device(self.dq.data_ptr(), self.dq.shape[0], pq, self.k, self.out.data_ptr(),
                              self.hops.data_ptr() if stats else None, self.evals.data_ptr() if stats else None,
                              self.stream.cuda_stream)

    def ids(self):
        import torch
        torch.cuda.synchronize()
        return self.out.cpu().numpy().view(np.uint64)


def timed_steps(torch, run, pq, steps, flush, stream, stage=None):
    """Per-step ms of `steps` searches (CUDA events on the launching stream,
    L2 flushed before each); with stage (the index, timing enabled) also the
    entry-choice and search-kernel ms of each step."""
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    st = []
    for i in range(steps):
        flush.zero_()
        ev[i][0].record(stream)
        run(pq)
        ev[i][1].record(stream)
        if stage is not None:
            st.append(stage.timing())
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev], st


def sweep_pq(torch, run, w, data, queries, gt_kth, k, target, curve, log_prefix, sweep=PQ_SWEEP):
    """Smallest pq of the sweep whose tie-aware recall@k reaches target."""
    from song_gb300 import groundtruth as GT
    nq = queries.shape[0]
    out, chosen = [], 0
    for cand in sweep:
        if cand < k:
            continue
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        run(cand)
        t0.record(run.stream)
        reps = 3 if curve else 1
        for _ in range(reps):
            run(cand)
        t1.record(run.stream)
        torch.cuda.synchronize()
        qps = reps * nq / (t0.elapsed_time(t1) / 1000.0)
        r = GT.recall_tie_aware(run.ids(), data, queries, gt_kth, w.metric, k)
        out.append([cand, round(r, 4), round(qps, 1)])
        log("[bench] %s pq %d recall@%d %.4f  %.0f q/s" % (log_prefix, cand, k, r, qps))
        if not chosen and r >= target:
            chosen = cand
            if not curve:
                break
    return (chosen or sweep[-1]), out


# ---------------------------------------------------------------------------
# precision: storage error against FP64 and recall per storage / rerank
# ---------------------------------------------------------------------------

def kernel_formula_fp64(metric, q, x):
    """The search's distance (l2: sum (q-x)^2; ip: -q.x; cos: sign*t*t/|x|^2
    with sign = +1 when t < 0, 0 when |x| = 0) evaluated in FP64."""
    q = q.astype(np.float64)
    x = x.astype(np.float64)
    if metric == "l2":
        return ((x - q[..., None, :]) ** 2).sum(-1)
    t = (x * q[..., None, :]).sum(-1)
    if metric == "ip":
        return -t
    nx = (x * x).sum(-1)
    sgn = np.where(t < 0, 1.0, -1.0)
    return np.where(nx > 0, sgn * t * t / np.where(nx > 0, nx, 1.0), 0.0)


def run_precision(args, torch, local):
    """Storage error of the F32/BF16/FP8 rows against FP64 on every exact
    top-k pair, and recall@k / queries/s per storage, rerank on/off, pq."""
    import song_gb300 as S
    from song_gb300 import datasets as D
    from song_gb300 import groundtruth as GT
    w, data, queries, graph = load_workload(args)
    nq, k = queries.shape[0], args.topk
    gt_ids, gt_kth, _ = ground_truth(args, w, data, queries, k)
    stream = torch.cuda.current_stream()
    dq = torch.from_numpy(queries).cuda()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    exact = kernel_formula_fp64(w.metric, queries, data[gt_ids])  # nq x k, FP64 of the FP32 rows
    # vertex 0 stays far below the target on this workload; the entry-point
    # rows go to pq 1000
    pqs_of = {"vertex 0": [args.pq] if args.pq else [100, 400, 1000]}
    pqs_entries = [args.pq] if args.pq else [50, 75, 100, 200, 400]
    table, errors = [], {}
    recall_f32 = {}
    for storage in ("f32", "bf16", "fp8", "bits"):
        ix = S.Index(graph, data, w.shift, w.metric, storage=storage, device=local)
        if storage == "bits":  # 256-bit sign codes: Hamming distance has no FP64 counterpart to compare
            ix.set_hash_planes(S.hash_planes(w.dim))
        uniq = np.unique(gt_ids) if storage != "bits" else None
        if storage != "bits":
            rows = np.concatenate([ix.rows(int(i), 1) for i in uniq])
            dec = S.dequantize_rows(rows, storage, w.dim)
            pos = np.searchsorted(uniq, gt_ids)
            approx = kernel_formula_fp64(w.metric, queries, dec[pos])
            rel = np.abs(approx - exact) / np.maximum(np.abs(exact), 1e-30)
            errors[storage] = {"rel_err_median": float("%.3g" % np.median(rel)),
                               "rel_err_p99": float("%.3g" % np.percentile(rel, 99)),
                               "rel_err_max": float("%.3g" % rel.max()),
                               "pairs": int(rel.size)}
            log("[precision] %s distance error vs FP64 over exact top-%d pairs: %s" % (storage, k, errors[storage]))
        run = Runner(ix, dq, k, stream)
        starts = [("vertex 0", None)]
        if args.entries > 0:
            # the two-level choice (any row width up to 4840 floats)
            two = args.coarse > 0
            n_ent = args.entries if two else min(args.entries, 4096)
            starts.append(("nearest %d of %d entries%s" % (args.starts, n_ent, " (%d clusters, %d probed)"
                                                           % (args.coarse, args.probes) if two else ""),
                           (S.sample_entries(w.n, n_ent, seed=D.SEED_BASE + 10, shuffle=True), two)))
        for start, ent_cfg in starts:
            ents, two = ent_cfg if ent_cfg is not None else (None, False)
            ix.set_entries(ents, starts=args.starts, coarse=args.coarse if two else 0, probes=args.probes)
            for rerank in ((0,) if storage == "f32" else (0, -1)):
                if storage != "f32":
                    ix.set_rerank(rerank)
                for pq in pqs_of.get(start, pqs_entries):
                    run(pq, stats=True)
                    rec = GT.recall_tie_aware(run.ids(), data, queries, gt_kth, w.metric, k)
                    for _ in range(2):
                        run(pq)
                    ms, _ = timed_steps(torch, run, pq, 3, flush, stream)
                    qps = nq / (statistics.median(ms) / 1000.0)
                    if storage == "f32":
                        recall_f32[(start, pq)] = rec
                    row = {"storage": storage, "rerank": "all pq" if rerank == -1 else "none", "start": start,
                           "pq": pq, "recall_at_%d" % k: round(rec, 4),
                           "recall_loss_vs_f32": round(recall_f32[(start, pq)] - rec, 4),
                           "qps": round(qps, 1), "mean_hops": round(float(run.hops.float().mean().item()), 1),
                           "mean_evals": round(float(run.evals.float().mean().item()), 1)}
                    table.append(row)
                    log("[precision] %s" % row)
        ix.free()
    # headline: the fastest configuration reaching the recall target; beside
    # it the fastest such row of each storage (with and without rerank)
    key = "recall_at_%d" % k
    ok = [r for r in table if r[key] >= args.recall]
    per_storage = {}
    for r in ok:
        name = r["storage"] + ("" if r["storage"] == "f32" else " rerank " + r["rerank"])
        if name not in per_storage or r["qps"] > per_storage[name]["qps"]:
            per_storage[name] = r
    best = max(ok, key=lambda r: r["qps"]) if ok else max(table, key=lambda r: r[key])
    line = {"metric": "queries/s at recall@%d>=%.2f, %s" % (k, args.recall, w.name),
            "value": best["qps"], "unit": "queries/s", "n_gpus": 1, "steps": 3, "warmup": 2,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "%s storage, f32 accumulate" % best["storage"],
            "data": "synthetic (seeded Gaussian mixture, GIST1M shape)",
            "config": {"workload": w.name, "n": w.n, "dim": w.dim, "metric": w.metric, "top_k": k,
                       "queries": nq, "best": best, "best_at_target_per_storage": per_storage,
                       "reached_target": bool(ok), "table": table,
                       "distance_error_vs_fp64": errors,
                       "distance_error_note": "search distance formula evaluated in FP64 on the stored (decoded) "
                                              "row vs on the FP32 row, over every exact top-k pair",
                       "l2": "flushed between steps (256 MB write)"}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# serve: Poisson request stream against two resident indexes
# ---------------------------------------------------------------------------

def run_serve(args, torch, local):
    """Poisson stream (mean args.serve_rate queries/s; 1-256 queries per
    request, log-uniform; k from {1,10,100}; pq from {50,100,200,400})
    against the 1M x 128 L2 and 1M x 960 cos indexes held resident together,
    each behind its own persistent search kernel."""
    import song_gb300 as S
    from song_gb300 import datasets as D
    from song_gb300.serve import Server, poisson_stream
    servers, indexes, qsets, names, starts_desc = [], [], [], [], []
    for name in ("scale-1m-128d-l2", "precision-1m-960d-cos"):
        a = argparse.Namespace(**vars(args))
        a.workload = name
        a.nq = 0
        w, data, queries, graph = load_workload(a)
        ix = S.Index(graph, data, w.shift, w.metric, device=local)
        if w.dim <= 364 and args.entries > 0 and args.coarse > 0:
            # two-level entry points, chosen by the server's warps; the 960-d
            # index keeps vertex 0 (a choice over its rows costs more than it saves)
            ix.set_entries(S.sample_entries(w.n, args.entries, seed=D.SEED_BASE + 10, shuffle=True),
                           starts=args.starts, coarse=args.coarse, probes=args.probes)
            names_start = "%s: nearest %d of %d entries (%d clusters, %d probed)" % (
                name, args.starts, args.entries, args.coarse, args.probes)
        else:
            names_start = "%s: vertex 0" % name
        starts_desc.append(names_start)
        indexes.append(ix)
        qsets.append(D.query_vectors(w, nq=max(w.n_queries, 4096)))
        names.append(name)
        del data, graph
    dev_bytes = sum(ix.device_bytes() for ix in indexes)
    for ix in indexes:
        servers.append(Server(ix, max_pq=400, max_k=100, slots=64, slot_queries=256, sm_fraction=0.5))
    pairs = list(zip(servers, qsets))
    poisson_stream(pairs, rate_qps=args.serve_rate, duration_s=1.0, seed=99)  # warm-up stream
    runs = {}
    for rate in (args.serve_rate, 4 * args.serve_rate, 16 * args.serve_rate):
        records, summary = poisson_stream(pairs, rate_qps=rate, duration_s=args.serve_seconds, seed=D.SEED_SERVE,
                                          warmup_s=0.5)
        per = {}
        for si, nm in enumerate(names):
            lat = np.array([r["latency_ms"] for r in records if r["server"] == si and r["t_submit"] >= 0.5])
            if lat.size:
                per[nm] = {"requests": int(lat.size), "p50_ms": round(float(np.percentile(lat, 50)), 3),
                           "p99_ms": round(float(np.percentile(lat, 99)), 3)}
        summary["per_index"] = per
        runs[str(int(rate))] = summary
        log("[serve] offered %.0f q/s: %s" % (rate, summary))
    for s in servers:
        s.close()
    for ix in indexes:
        ix.set_entries(None)
        ix.free()
    main_run = runs[str(int(args.serve_rate))]
    line = {"metric": "p99 request latency at a %.0f queries/s Poisson stream, 1M x 128 L2 + 1M x 960 cos resident"
                      % args.serve_rate,
            "value": main_run["p99_ms"], "unit": "ms", "n_gpus": 1, "steps": main_run["requests"], "warmup": 1,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian mixtures, SIFT1M and GIST1M shapes)",
            "config": {"workload": "serve-two-indexes", "indexes": names, "resident_device_bytes": dev_bytes,
                       "request": "1-256 queries log-uniform, k in {1,10,100}, pq in {50,100,200,400} (pq>=k)",
                       "admission": "64 slots x 256 queries per index (queue memory bound), "
                                    "persistent kernel per index on half the SMs",
                       "starts": starts_desc,
                       "p50_ms": main_run["p50_ms"], "throughput_qps": main_run["throughput_qps"],
                       "load_sweep": runs},
            "e2e": {"value": main_run["throughput_qps"], "unit": "queries/s",
                    "h2d_bytes_per_step": None, "d2h_bytes_per_step": None}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# build: graph construction with the searches on the GPU vs on host threads
# ---------------------------------------------------------------------------

def run_build(args, torch, local):
    """Builds the workload's degree-32 graph with the CPU batch-parallel
    builder (all host threads) and with the GPU builder (searches on the
    GPU, edge updates on the host threads); the graphs must be identical."""
    import hashlib
    import song_gb300 as S
    from song_gb300 import datasets as D
    w = D.WORKLOADS[args.workload]
    data = D.base_vectors(w)
    nt = os.cpu_count() or 1
    bargs = (data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150)
    S.graph_build_gpu(data[:2000], w.metric, w.shift, w.search_degree, w.fixed_degree, 150,
                      batch_div=args.build_div, device=local)  # context and module load
    t = time.perf_counter()
    g_gpu = S.graph_build_gpu(*bargs, batch_div=args.build_div, device=local, nthreads=nt)
    gpu_s = time.perf_counter() - t
    log("[build] GPU builder %.2fs" % gpu_s)
    t = time.perf_counter()
    g_cpu = S.graph_build(*bargs, batch_div=args.build_div, nthreads=nt)
    cpu_s = time.perf_counter() - t
    log("[build] CPU builder %.2fs on %d threads" % (cpu_s, nt))
    same = bool(np.array_equal(g_gpu, g_cpu))
    assert same, "GPU and CPU builders disagree"
    nb, a = 0, 0
    while a < w.n:
        a += max(1, a // args.build_div)
        nb += 1
    line = {"metric": "seconds to build the graph, %s (shift %d, SEARCH_DEGREE %d, budget 150, batch div %d)"
                      % (w.name, w.shift, w.search_degree, args.build_div),
            "value": round(gpu_s, 3), "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 data, f64 distance sums (the reference builder's arithmetic)",
            "data": "synthetic (seeded Gaussian mixture)",
            "config": {"workload": w.name, "n": w.n, "dim": w.dim, "metric": w.metric,
                       "graphs_identical": same, "graph_md5": hashlib.md5(g_gpu.tobytes()).hexdigest(),
                       "batches": nb, "speedup_vs_cpu_builder": round(cpu_s / gpu_s, 2)},
            "cpu_baseline": {"value": round(cpu_s, 3), "unit": "s", "cores": nt, "kind": "port",
                             "sample": "the whole build (this project's restatement of the reference builder, "
                                       "batch-parallel, row-parallel edge updates)"},
            "e2e": {"value": round(gpu_s, 3), "unit": "s", "h2d_bytes_per_step": int(data.nbytes),
                    "d2h_bytes_per_step": None},
            "gpu_launches": 2 * nb}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# learned: the early exit against the search without it and against a fixed
# hop budget, from vertex 0 and from entry points
# ---------------------------------------------------------------------------

def convergence_hops(ix, queries, pq, k):
    """Mean hop after which each query's top-k no longer changes (the labels of
    the plain search's traces), and the mean hops of that search: the room an
    exit has."""
    from song_gb300 import learned as LE
    X, y = LE.trace_dataset(ix, queries, pq, k, max_samples_per_query=0)
    nq = queries.shape[0]
    return float((1.0 - y).sum().item()) / nq, float(X.shape[0]) / nq


def run_learned(args, torch, local):
    """--mode learned: on the workload (default learned-3m-256d-l2), per start
    (vertex 0, entry points): the plain FP32 search at the smallest pq <=
    --max-pq reaching the recall target, the exit trained on traces of
    --train-queries training queries at that pq, a fixed hop budget of the
    exit's mean hops, and the exit with BF16 rows + FP32 rerank; all on the
    held-out query set."""
    import song_gb300 as S
    from song_gb300 import datasets as D
    from song_gb300 import learned as LE
    S.load_library()
    w, data, queries, graph = load_workload(args)
    nq, k = queries.shape[0], args.topk
    _, _, kth10 = ground_truth(args, w, data, queries, k)
    stream = torch.cuda.current_stream()
    dq = torch.from_numpy(queries).cuda()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    train_q = D.query_vectors(w, nq=args.train_queries, seed=D.SEED_TRAIN)
    sweep = [p for p in PQ_SWEEP if p <= args.max_pq] or [args.max_pq]
    entries = S.sample_entries(w.n, args.entries, seed=D.SEED_BASE + 10, shuffle=True) if args.entries > 0 else None
    studies = {}
    for start in ("vertex 0", "entries"):
        if start == "entries" and entries is None:
            continue
        ix = S.Index(graph, data, w.shift, w.metric, device=local)
        if start == "entries":
            ix.set_entries(entries, starts=args.starts, coarse=args.coarse, probes=args.probes)
        run = Runner(ix, dq, k, stream)
        pq, psweep = (args.pq, []) if args.pq else sweep_pq(torch, run, w, data, queries, kth10, k, args.recall,
                                                            False, "plain " + start, sweep=sweep)
        plain = measure_arm(torch, run, pq, 5, flush, stream, data, queries, kth10, w)
        ix.set_hop_limit(1 << 30)  # the learned kernel without an exit (its exact visited set)
        noexit = measure_arm(torch, run, pq, 5, flush, stream, data, queries, kth10, w)
        ix.set_hop_limit(0)
        conv, traced = convergence_hops(ix, queries, pq, k)
        model = LE.fit(ix, train_q, pq, k, epochs=6, data=data, metric=w.metric, recall_slack=args.recall_slack,
                       log=log)
        ix.set_early_exit(model.params, model.threshold, model.min_hops, model.every)
        learned = measure_arm(torch, run, pq, 5, flush, stream, data, queries, kth10, w)
        ix.set_early_exit(None)
        budget = max(1, int(round(learned["mean_hops"])))
        ix.set_hop_limit(budget)
        fixed = measure_arm(torch, run, pq, 5, flush, stream, data, queries, kth10, w)
        ix.set_hop_limit(0)
        ixb = S.Index(graph, data, w.shift, w.metric, storage="bf16", device=local)
        ixb.set_rerank(args.rerank)
        if start == "entries":
            ixb.set_entries(entries, starts=args.starts, coarse=args.coarse, probes=args.probes)
        ixb.set_early_exit(model.params, model.threshold, model.min_hops, model.every)
        learned_bf16 = measure_arm(torch, Runner(ixb, dq, k, stream), pq, 5, flush, stream, data, queries, kth10, w)
        ixb.free()
        ix.free()
        studies[start] = {
            "pq": pq, "plain_fp32": plain, "exit_free_learned_kernel": noexit, "learned_fp32": learned,
            "fixed_budget": dict(fixed, max_hops=budget), "learned_bf16_rerank": learned_bf16,
            "topk_final_after_hops_mean": round(conv, 2), "traced_hops_mean": round(traced, 2),
            "speedup_learned_fp32_vs_plain": round(learned["qps"] / plain["qps"], 3),
            "speedup_learned_bf16_vs_plain": round(learned_bf16["qps"] / plain["qps"], 3),
            "recall_gain_vs_fixed_budget": round(learned["recall_at_10"] - fixed["recall_at_10"], 4),
            "model": {"threshold": model.threshold, "min_hops": model.min_hops, "every": model.every,
                      "train": {kk: model.info[kk] for kk in ("samples", "positive", "trace_s", "train_s", "losses",
                                                              "chosen", "val_recall_no_exit")}},
            "plain_pq_sweep_recall_qps": psweep}
        log("[learned] %s: %s" % (start, studies[start]))
    ok = [(s, v) for s, v in studies.items() if v["learned_bf16_rerank"]["recall_at_10"] >= args.recall]
    pick = max(ok or studies.items(), key=lambda sv: sv[1]["learned_bf16_rerank"]["qps"])
    line = {"metric": "queries/s at recall@10>=%.2f, %s: learned exit + BF16 vs plain FP32" % (args.recall, w.name),
            "value": pick[1]["learned_bf16_rerank"]["qps"], "unit": "queries/s", "n_gpus": 1, "steps": 5,
            "warmup": 2, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 storage, f32 accumulate, f32 rerank", "data": "synthetic (seeded Gaussian mixture)",
            "config": dict(common_config(args, w, nq), train_queries=args.train_queries, max_pq=args.max_pq,
                           reported_start=pick[0], reached_target=bool(ok), studies=studies,
                           mlp="5 -> 32 -> 32 -> 1, BF16 weights, FP32 accumulate, trained by the library's kernels",
                           l2="flushed between steps (256 MB write)")}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# the default mode: plain / entries / learned arms
# ---------------------------------------------------------------------------

def measure_arm(torch, run, pq, steps, flush, stream, data, queries, kth10, w):
    """recall@10, hops, evaluations and kernel queries/s of one arm at pq."""
    from song_gb300 import groundtruth as GT
    run(pq, stats=True)
    rec = GT.recall_tie_aware(run.ids(), data, queries, kth10, w.metric, 10)
    hops = float(run.hops.float().mean().item())
    evals = float(run.evals.float().mean().item())
    for _ in range(2):
        run(pq)
    ms, _ = timed_steps(torch, run, pq, steps, flush, stream)
    med = statistics.median(ms)
    return {"qps": round(queries.shape[0] / (med / 1000.0), 1), "pq": pq, "recall_at_10": round(rec, 4),
            "kernel_ms_median": round(med, 4), "mean_hops": round(hops, 2), "mean_evals": round(evals, 2)}


def pq_table(torch, ix, dq, stream, flush, data, queries, kth10, kth100, w, target):
    """The pq sweep 50-400 at top-10 and (pq >= 100) top-100: recall and
    kernel queries/s; and the smallest pq whose recall@100 reaches target."""
    from song_gb300 import groundtruth as GT
    nq = queries.shape[0]
    r10, r100 = Runner(ix, dq, 10, stream), Runner(ix, dq, 100, stream)
    rows, top100 = [], None
    for pq in PQ_TABLE:
        row = {"pq": pq}
        for k, run, kth in ((10, r10, kth10), (100, r100, kth100)):
            if pq < k:
                continue
            run(pq)
            rec = GT.recall_tie_aware(run.ids(), data, queries, kth, w.metric, k)
            ms, _ = timed_steps(torch, run, pq, 3, flush, stream)
            row["recall_at_%d" % k] = round(rec, 4)
            row["qps_top%d" % k] = round(nq / (statistics.median(ms) / 1000.0), 1)
        rows.append(row)
        log("[bench] table %s" % row)
        if top100 is None and row.get("recall_at_100", 0.0) >= target:
            top100 = {"pq": pq, "recall_at_100": row["recall_at_100"], "qps": row["qps_top100"]}
    return rows, top100


def entry_launches(args, w, nq):
    """Kernels of one entry choice: flat, one; two-level, the query norms and
    a score + select pair per chunk of queries (tensor-core heads, dims a
    multiple of 4: a chunk's BF16 bounds take at most 96 MB, in 128-query
    tiles) or one head kernel, then scan, scatter, cluster and merge kernels."""
    if args.coarse <= 0:
        return 1
    if w.dim % 4 == 0:
        ld = (args.coarse + 7) // 8 * 8
        chunk = max(128, min((nq + 127) // 128 * 128, (96 << 20) // (2 * ld) // 128 * 128))
        heads = 1 + 2 * ((nq + chunk - 1) // chunk)
    else:
        heads = 1
    return heads + 4


def plain_arm(torch, S, args, w, graph, data, queries, kth10, dq, k, stream, flush, local, msteps):
    t = time.time()
    ix32 = S.Index(graph, data, w.shift, w.metric, device=local)
    log("[bench] FP32 index resident (%.2f GB) in %.1fs" % (ix32.device_bytes() / 1e9, time.time() - t))
    run32 = Runner(ix32, dq, k, stream)
    pq32, sweep32 = (args.pq, []) if args.pq else sweep_pq(torch, run32, w, data, queries, kth10, k, args.recall,
                                                            args.curve, "fp32")
    plain = measure_arm(torch, run32, pq32, msteps, flush, stream, data, queries, kth10, w)
    plain["pq_sweep_recall_qps"] = sweep32
    log("[bench] plain FP32: %s" % plain)
    return plain, ix32, run32


def run_search(args, torch, rank, world, local, dist):
    import ctypes

    import song_gb300 as S
    from song_gb300 import datasets as D
    from song_gb300 import groundtruth as GT
    from song_gb300 import learned as LE
    from song_gb300 import replicas as R

    def barrier():
        if dist:
            dist.barrier()

    S.load_library()
    w, data, queries, graph = load_workload(args, rank, barrier)
    nq, k = queries.shape[0], args.topk
    gt_ids, kth100, kth10 = ground_truth(args, w, data, queries, 100)
    stream = torch.cuda.current_stream()
    dq = torch.from_numpy(queries).cuda()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2
    msteps = max(3, args.steps // 2)
    entries = S.sample_entries(w.n, args.entries, seed=D.SEED_BASE + 10, shuffle=True) if args.entries > 0 else None

    def with_entries(ix):
        if entries is not None:
            ix.set_entries(entries, starts=args.starts, coarse=args.coarse, probes=args.probes)

    # ---- plain FP32 search from vertex 0 (the reference's semantics) --------
    plain, ix32, run32 = None, None, None
    if args.mode in ("best", "plain") or entries is None:
        plain, ix32, run32 = plain_arm(torch, S, args, w, graph, data, queries, kth10, dq, k, stream, flush, local,
                                       msteps)

    # ---- the same search from each query's nearest entry vertices ----------
    ent, ixe, rune, table, top100 = None, None, None, [], None
    if args.mode in ("best", "entries") and entries is not None:
        ixe = S.Index(graph, data, w.shift, w.metric, device=local)
        with_entries(ixe)
        rune = Runner(ixe, dq, k, stream)
        pqe, sweepe = (args.pq, []) if args.pq else sweep_pq(torch, rune, w, data, queries, kth10, k, args.recall,
                                                              args.curve, "fp32+entries")
        ent = measure_arm(torch, rune, pqe, msteps, flush, stream, data, queries, kth10, w)
        ent.update({"entries": args.entries, "starts_per_query": args.starts, "coarse": args.coarse,
                    "probes": args.probes, "pq_sweep_recall_qps": sweepe})
        log("[bench] FP32 from entries: %s" % ent)
    # ---- the reference's N_MULTIPROBE / FINISH_CNT knobs on the entries arm --
    multi = None
    if ent and args.multiprobe:
        multi = []
        for spec in args.multiprobe.split(","):
            parts = [int(x) for x in spec.split(":")]
            mp_p, mp_f, mp_d = parts[0], parts[1] if len(parts) > 1 else 1, parts[2] if len(parts) > 2 else 0
            ixe.set_multiprobe(mp_p, mp_f, mp_d)
            pqm, swm = sweep_pq(torch, rune, w, data, queries, kth10, k, args.recall, False,
                                "fp32+entries probes %d finish %d double-check %d" % (mp_p, mp_f, mp_d))
            r = measure_arm(torch, rune, pqm, msteps, flush, stream, data, queries, kth10, w)
            r.update({"n_multiprobe": mp_p, "finish_cnt": mp_f, "double_check": bool(mp_d), "pq_sweep_recall_qps": swm,
                      "vs_single_probe": round(r["qps"] / ent["qps"], 3)})
            multi.append(r)
            log("[bench] multi-probe: %s" % r)
        ixe.set_multiprobe(1, 1)
    if not args.no_table:
        table, top100 = pq_table(torch, ixe or ix32, dq, stream, flush, data, queries, kth10, kth100, w, args.recall)

    # ---- learned early exit + BF16 storage + FP32 rerank, same starts --------
    lrn, ixl, runl, model = None, None, None, None
    if args.mode == "best":
        ixl = S.Index(graph, data, w.shift, w.metric, storage="bf16", device=local)
        ixl.set_rerank(args.rerank)
        with_entries(ixl)
        runl = Runner(ixl, dq, k, stream)
        train_q = D.query_vectors(w, nq=args.train_queries, seed=D.SEED_TRAIN)
        pq0 = ent["pq"] if ent else plain["pq"]
        tried = []
        for cand in [c for c in PQ_SWEEP + [1023] if c >= pq0][:4]:
            model = LE.fit(ixl, train_q, cand, k, epochs=6, data=data, metric=w.metric,
                           recall_slack=args.recall_slack, log=log)
            ixl.set_early_exit(model.params, model.threshold, model.min_hops, model.every)
            runl(cand, stats=True)
            lrec = GT.recall_tie_aware(runl.ids(), data, queries, kth10, w.metric, k)
            tried.append([cand, round(model.threshold, 2), round(lrec, 4)])
            log("[bench] learned+bf16 pq %d threshold %.2f recall@10 %.4f" % (cand, model.threshold, lrec))
            if lrec >= args.recall:
                break
        lrn = measure_arm(torch, runl, cand, msteps, flush, stream, data, queries, kth10, w)
        lrn.update({"threshold": model.threshold, "min_hops": model.min_hops, "rerank": args.rerank,
                    "train_queries": args.train_queries, "recall_slack": args.recall_slack,
                    "tried_pq_threshold_recall": tried,
                    "train": {kk: model.info[kk] for kk in ("samples", "positive", "trace_s", "train_s", "losses",
                                                            "chosen")}})
        log("[bench] learned+bf16: %s" % lrn)

    # ---- the arm reported: the one asked for, or the fastest at the target ---
    arms = {}
    if plain:
        arms["plain"] = (plain, ix32, run32)
    if ent:
        arms["entries"] = (ent, ixe, rune)
    if lrn:
        arms["learned"] = (lrn, ixl, runl)
    if args.mode in arms:
        mode = args.mode
    else:
        ok = [a for a in arms if arms[a][0]["recall_at_10"] >= args.recall] or list(arms)
        mode = max(ok, key=lambda a: arms[a][0]["qps"])
    rep, ix, run = arms[mode]
    pq = rep["pq"]
    log("[bench] arms (q/s, recall@10): %s -> %s"
        % ({a: (v[0]["qps"], v[0]["recall_at_10"]) for a, v in arms.items()}, mode))
    run(pq, stats=True)
    hops = run.hops.cpu().numpy().astype(np.int64)
    evals = run.evals.cpu().numpy().astype(np.int64)
    ids = run.ids()
    rec = GT.recall_tie_aware(ids, data, queries, kth10, w.metric, k)
    rec_ids = GT.recall(ids, gt_ids, k)

    # ---- timed region ---------------------------------------------------------
    ix.set_timing(True)
    sampler = ClockSampler(local)
    sampler.start()
    for _ in range(args.warmup):
        flush.zero_()
        run(pq)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    kernel_ms, stages = timed_steps(torch, run, pq, args.steps, flush, stream, stage=ix)
    wall = time.perf_counter() - wall0
    barrier()
    ix.set_timing(False)
    total_s = R.max_over_ranks(sum(kernel_ms) / 1000.0, dist, "cuda")
    value = R.whole_job_rate(nq, args.steps, world, total_s)

    # e2e: host buffers through song_search (pinned query and id buffers)
    pinned = torch.empty((nq, w.dim), dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = queries
    hq = pinned.numpy()
    out_host = torch.empty((nq, k), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    L = S.load_library()
    for _ in range(max(1, args.warmup)):
        S._check(L.song_search(ix._h, hq.ctypes.data_as(ctypes.c_void_p), nq, pq, k,
                               out_host.ctypes.data_as(ctypes.c_void_p), None, None))
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t = time.perf_counter()
        S._check(L.song_search(ix._h, hq.ctypes.data_as(ctypes.c_void_p), nq, pq, k,
                               out_host.ctypes.data_as(ctypes.c_void_p), None, None))
        e2e_times.append(time.perf_counter() - t)
    clocks = sampler.stop()
    assert np.array_equal(out_host, ids), "e2e results differ from the device-buffer results"
    e2e_s = R.max_over_ranks(sum(e2e_times), dist, "cuda")
    e2e = R.whole_job_rate(nq, args.steps, world, e2e_s)

    # ---- roofline of the search kernel (the step's dominant kernel) ----------
    if mode == "learned":
        row_bytes = 2 * (((w.dim + 7) // 8) * 8)
        rerank_rows = min(args.rerank if args.rerank > 0 else pq, pq)
    else:
        row_bytes = 4 * (((w.dim + 3) // 4) * 4)
        rerank_rows = 0
    alg_bytes = int((4 * w.dim * nq) + hops.sum() * (1 << w.shift) * 4 + evals.sum() * row_bytes
                    + nq * rerank_rows * 4 * w.dim + nq * k * 8)
    entry_ms = [a for a, _ in stages]
    search_ms = [b for _, b in stages]
    mean_search_s = statistics.fmean(search_ms) / 1000.0
    achieved = alg_bytes / mean_search_s / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    traffic, traffic_src = None, None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        try:
            tj = json.load(open(tp)).get("%s/%s/pq%d" % (w.name, mode, pq), {}).get("search_kernel")
            if tj:
                traffic = int(round(tj["dram_bytes"] * nq / tj["queries"]))
                traffic_src = tj.get("source")
        except Exception:
            traffic = None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            from oracle import oracle as O
            O.build()
            sample = min(400, nq)
            ck, csweep = cpu_calibrate_k(w, data, graph, queries, args.recall, kth10, sample)
            nthreads = os.cpu_count() or 1
            crate, n, dt = cpu_time(w, data, graph, queries, ck, args.cpu_seconds, nthreads)
            cpu = {"value": round(crate, 1), "unit": "queries/s", "cores": nthreads, "kind": "port",
                   "cpu_model": cpu_model(),
                   "sample": "%d queries (workload set repeated), k=%d for recall@10>=%.2f, %.1fs"
                             % (n, ck, args.recall, dt),
                   "recall_sweep_k": csweep}
        except Exception as e:  # the baseline must not hide the GPU number
            cpu = {"value": None, "error": repr(e)}

    ref_sm100 = None
    rp = os.path.join(args.cache, "%s.reference_sm100.json" % w.name)
    if os.path.exists(rp):
        try:
            r = json.load(open(rp))
            if r.get("at_target"):
                ref_sm100 = dict(r["at_target"], source="bench.py --impl reference on this machine")
        except Exception:
            ref_sm100 = None

    if rank == 0:
        desc = {"learned": "learned early exit + BF16 storage + FP32 rerank, from the nearest %d of %d entry "
                           "vertices" % (args.starts, args.entries),
                "entries": "FP32 search from the nearest %d of %d entry vertices (%d clusters, %d probed)"
                           % (args.starts, args.entries, args.coarse, args.probes),
                "plain": "plain FP32 search from vertex 0"}[mode]
        same = None
        if lrn and ent:
            same = {"learned_bf16": {kk: lrn[kk] for kk in ("qps", "pq", "recall_at_10", "mean_hops")},
                    "fp32": {kk: ent[kk] for kk in ("qps", "pq", "recall_at_10", "mean_hops")},
                    "ratio": round(lrn["qps"] / ent["qps"], 3),
                    "both_at_target": lrn["recall_at_10"] >= args.recall and ent["recall_at_10"] >= args.recall}
        config = common_config(args, w, nq)
        config.update({
            "learned_vs_fp32_same_starts": same,
            "reference_sm100_qps": ref_sm100["qps"] if ref_sm100 else None,
            "reference_sm100": ref_sm100,
            "plain_fp32_vs_reference_sm100": round(plain["qps"] / ref_sm100["qps"], 3) if ref_sm100 and plain
            else None,
            "top100": top100,
            "pq_table": table,
            "multi_probe_from_entries": multi,
            "l2": "flushed between steps (256 MB write); index > L2",
            "parallelism": "replicas" if world > 1 else "single GPU"})
        line = {
            "metric": "queries/s at recall@10>=%.2f, %s" % (args.recall, w.name),
            "value": round(value, 1), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1000 * total_s / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "bf16 storage, f32 accumulate, f32 rerank" if mode == "learned" else "f32",
            "data": "synthetic (seeded Gaussian mixture, SIFT1M shape)",
            "config": config,
            "arm": {"name": desc, "mode": mode, "pq": pq, "recall_at_10": round(rec, 4),
                    "recall_at_10_ids": round(rec_ids, 4), "mean_hops": round(float(hops.mean()), 2),
                    "mean_evals": round(float(evals.mean()), 2),
                    "entry_ms_mean": round(statistics.fmean(entry_ms), 4),
                    "search_kernel_ms_mean": round(statistics.fmean(search_ms), 4)},
            "arms": {"plain_fp32": plain, "fp32_from_entries": ent, "learned_bf16": lrn},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "kernel": "search_kernel (per launch = one step's 10,000 queries)",
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "traffic_source": traffic_src,
                         "step_achieved": round(alg_bytes / (statistics.fmean(kernel_ms) / 1000.0) / 1e9, 1),
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks
                         else "fallback"},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e, 1), "unit": "queries/s", "h2d_bytes_per_step": int(nq * w.dim * 4),
                    "d2h_bytes_per_step": int(nq * k * 8)},
            "gpu_launches": args.steps * (1 + (0 if mode == "plain" or entries is None
                                               else entry_launches(args, w, nq))),
            "clocks": clocks,
            "kernel_ms": {"min": round(min(kernel_ms), 4), "median": round(statistics.median(kernel_ms), 4),
                          "max": round(max(kernel_ms), 4)},
            "wall_s_timed": round(wall, 4),
        }
        print(json.dumps(line), flush=True)
    for a in arms.values():
        a[1].free()


def main():
    args = parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if args.mode == "precision":
        run_precision(args, torch, local)
    elif args.mode == "serve":
        run_serve(args, torch, local)
    elif args.mode == "build":
        run_build(args, torch, local)
    elif args.mode == "learned":
        run_learned(args, torch, local)
    else:
        run_search(args, torch, rank, world, local, dist)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
