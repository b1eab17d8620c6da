"""Times the reference's own GPU kernel, rebuilt for sm_100, on the bench
workload (1M x 128 L2, the same graph, 10,000 queries) over its pq_size
values, with __ENABLE_MEASURE as shipped and removed, next to recall@10.

TEST INFRASTRUCTURE ONLY (the reference GPU baseline).  Usage on the GPU host:

    python oracle/ref_gpu_bench.py [--pq 100,200,...] [--repeats 3]

Prints one JSON line per (pq, measure) and a summary line.
"""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--pq", default="100,200,400,600,800,1000")
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--build-div", type=int, default=64)
    ap.add_argument("--cache", default=os.environ.get("SONG_CACHE", os.path.join(ROOT, "_cache")))
    a = ap.parse_args()
    import bench
    from oracle import ref_gpu
    from song_gb300 import groundtruth as GT

    class Args:
        workload = "scale-1m-128d-l2"
        nq = 0
        build_div = a.build_div
        cache = a.cache
    w, data, queries, graph = bench.load_workload(Args)
    gt_ids, gt_kth = bench.ground_truth(Args, w, data, queries, 10)
    nq = queries.shape[0]
    best = {}
    pqs = [int(x) for x in a.pq.split(",")]
    for pq in pqs:
        for measure in (True, False):
            path = ref_gpu.cubin_path("l2", w.dim, pq, measure)
            if not os.path.exists(path):
                continue
            ids, ms = ref_gpu.run(path, data, graph, w.shift, queries, pq, measure, repeats=a.repeats,
                                  heap_pq=max(pqs))
            rec = GT.recall_tie_aware(ids[:, :10], data, queries, gt_kth, w.metric, 10)
            qps = nq / (float(np.median(ms)) / 1000.0)
            row = {"pq": pq, "measure": measure, "kernel_ms": [round(float(x), 3) for x in ms],
                   "qps": round(qps, 1), "recall_at_10": round(rec, 4)}
            print(json.dumps(row), flush=True)
            if pq not in best or qps > best[pq]["qps"]:
                best[pq] = row
    print(json.dumps({"reference_sm100_best_per_pq": best}), flush=True)


if __name__ == "__main__":
    main()
