"""Generates the golden fixtures in tests/golden/ from the REFERENCE's own code.

Run in the development container, where the reference tree is readable:

    bash oracle/build_ref.sh && python tests/golden/make_golden.py [search fixhash fma multiprobe]

Everything stored as an expected output comes from oracle/_ref, i.e. from the
reference's own source files compiled where they lie:
  * graphs      -- FixedDegreeGraph::add_vertex (graph.h:149-167), sequential
                   insertion, dumped by its own dump()
  * kernel ids  -- the search steps of warp_astar_accelerator.h:111-335 driven
                   through the reference's smmh2.h / bin_heap.h / fixhash.h,
                   with its N_MULTIPROBE / FINISH_CNT knobs (:29-30) at their
                   defaults and, in search_multiprobe.npz, away from them
  * CPU ids     -- FixedDegreeGraph::astar_multi_start_search (graph.h:169-216)
  * hash ops    -- FixHash<int, 8*pq> (fixhash.h) add/del/test answers
Inputs are seeded synthetic vectors (song_gb300.datasets.mixture).  The GPU
host never runs this script; it reads the .npz files.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from song_gb300 import datasets as D  # noqa: E402

# name, metric, shift, kind, n, dim, centres
CASES = [
    ("cos_s4_d16", "cos", 4, "unit", 1500, 16, 26),
    ("l2_s5_d32", "l2", 5, "byte", 1500, 32, 26),
    ("ip_s5_d24", "ip", 5, "unit", 1200, 24, 26),
    ("cos_s5_d26", "cos", 5, "unit", 1200, 26, 26),
]
PQS = (10, 50, 100)
CPU_KS = (10, 50)
NQ = 48


def make_search_case(name, metric, shift, kind, n, dim, centres):
    data = D.mixture(kind, n, dim, centres, seed=11, center_seed=111)
    queries = D.mixture(kind, NQ, dim, centres, seed=12, center_seed=111)
    m = O.METRICS[metric]
    graph = O.ref_build_graph(data, shift, m)
    assert graph.max() < 2 ** 32
    out = dict(data=data, queries=queries, graph=graph.astype(np.uint32), shift=np.int32(shift),
               metric=np.int32(m), pqs=np.array(PQS, np.int32), cpu_ks=np.array(CPU_KS, np.int32))
    for pq in PQS:
        ids, hops, evals, popped = O.ref_kernel_search(data, graph, shift, m, queries, pq)
        out["kernel_ids_%d" % pq] = ids
        out["kernel_hops_%d" % pq] = hops
        out["kernel_evals_%d" % pq] = evals
        out["kernel_popped_%d" % pq] = popped
    for k in CPU_KS:
        out["cpu_ids_%d" % k] = O.ref_cpu_search(data, graph, shift, m, queries, k)
    np.savez_compressed(os.path.join(HERE, "search_%s.npz" % name), **out)


def make_fixhash_case():
    rng = np.random.default_rng(5)
    out = {}
    for pq, keyspace, nops in ((8, 1 << 20, 20000), (100, 1 << 22, 20000)):
        live, ops, keys = [], [], []
        for _ in range(nops):
            r = rng.random()
            if r < 0.4 and len(live) < 2 * pq:
                k = int(rng.integers(0, keyspace))
                ops.append(0)
                keys.append(k)
                live.append(k)
            elif r < 0.7 and live:
                k = live.pop(int(rng.integers(0, len(live))))
                ops.append(1)
                keys.append(k)
            else:
                # half of the tests ask for a key known to be present
                k = live[int(rng.integers(0, len(live)))] if (live and rng.random() < 0.5) else int(rng.integers(0, keyspace))
                ops.append(2)
                keys.append(k)
        ops = np.array(ops, np.int32)
        keys = np.array(keys, np.int32)
        out["ops_%d" % pq] = ops
        out["keys_%d" % pq] = keys
        out["results_%d" % pq] = O.ref_fixhash_ops(pq, ops, keys)
    np.savez_compressed(os.path.join(HERE, "fixhash_ops.npz"), **out)


def make_fma_probe():
    """Query / vector pairs whose L2 order differs between fused (nvcc's
    default contraction) and separate multiply-add in the kernel's
    lane-strided sums (only possible for dim > 32, where a lane adds more
    than one term), each embedded in a 128-vertex graph searched at pq 100.
    Expected ids come from the harness (reference containers, FMA); the ids
    the oracle gives without FMA are stored too and must differ."""
    rng = np.random.default_rng(7)
    dim, n, shift, pq = 128, 128, 5, 100
    probes = []
    while len(probes) < 4:
        q = rng.standard_normal(dim).astype(np.float32)
        a = (q + rng.standard_normal(dim).astype(np.float32)).astype(np.float32)
        b = a.copy()
        for i in rng.choice(dim, 3, replace=False):
            b[i] = np.nextafter(b[i], np.float32(np.inf) if rng.random() < .5 else np.float32(-np.inf))
        fa, fb = O.kernel_distance(O.L2, q, a, True), O.kernel_distance(O.L2, q, b, True)
        na, nb = O.kernel_distance(O.L2, q, a, False), O.kernel_distance(O.L2, q, b, False)
        if (fa < fb) != (na < nb) and fa != fb and na != nb:
            probes.append((q, a, b))
    graph = np.zeros((n, 1 << shift), np.uint64)
    for v in range(n):
        graph[v, 0] = 31
        graph[v, 1:32] = [(v + 1 + j) % n for j in range(31)]
    graph = graph.reshape(-1)
    datas, queries, fma_ids, nofma_ids = [], [], [], []
    for q, a, b in probes:
        far = (q + 8.0 * rng.standard_normal((n, dim))).astype(np.float32)
        far[1], far[2] = a, b
        ids, _, _, popped = O.ref_kernel_search(far, graph, shift, O.L2, q[None, :], pq)
        assert popped[0] == pq
        ox = O.OracleIndex(far, graph, shift, O.L2)
        nf, *_ = ox.kernel_search(q[None, :], pq, O.MODE_REF, use_fma=False)
        assert not np.array_equal(nf, ids)
        datas.append(far)
        queries.append(q)
        fma_ids.append(ids[0])
        nofma_ids.append(nf[0])
    np.savez_compressed(os.path.join(HERE, "fma_probe.npz"), data=np.array(datas), queries=np.array(queries),
                        graph=graph.astype(np.uint32), shift=np.int32(shift), pq=np.int32(pq),
                        fma_ids=np.array(fma_ids), nofma_ids=np.array(nofma_ids))


# (probes, finish_cnt, double_check): the N_MULTIPROBE / FINISH_CNT knobs of
# warp_astar_accelerator.h:29-30 and its __ENABLE_MULTIPROBE_DOUBLE_CHECK
# switch (:307-310) away from their defaults (1, 1, off).
MULTI_KNOBS = ((2, 1, 0), (4, 1, 0), (1, 2, 0), (3, 3, 0), (2, 1, 1), (4, 2, 1))
MULTI_CASES = ("cos_s4_d16", "l2_s5_d32")


def make_multiprobe_case():
    """Kernel search results with multi-probe / finish-count knobs, on the
    graphs and queries of two search fixtures (read back from their files)."""
    out = {}
    for name in MULTI_CASES:
        z = np.load(os.path.join(HERE, "search_%s.npz" % name))
        graph = z["graph"].astype(np.uint64)
        for probes, fc, dc in MULTI_KNOBS:
            for pq in PQS:
                ids, hops, evals, popped = O.ref_kernel_search(z["data"], graph, int(z["shift"]), int(z["metric"]),
                                                               z["queries"], pq, probes, fc, dc)
                key = "%s_p%d_f%d_d%d_%d" % (name, probes, fc, dc, pq)
                out["ids_" + key] = ids
                out["hops_" + key] = hops
                out["evals_" + key] = evals
                out["popped_" + key] = popped
    out["knobs"] = np.array(MULTI_KNOBS, np.int32)
    np.savez_compressed(os.path.join(HERE, "search_multiprobe.npz"), **out)


def main():
    if not O.ref_available(4) or not O.ref_available(5):
        raise SystemExit("oracle/_ref not built: run bash oracle/build_ref.sh first")
    only = sys.argv[1:]
    if not only or "search" in only:
        for case in CASES:
            make_search_case(*case)
            print("wrote search_%s.npz" % case[0])
    if not only or "fixhash" in only:
        make_fixhash_case()
        print("wrote fixhash_ops.npz")
    if not only or "fma" in only:
        make_fma_probe()
        print("wrote fma_probe.npz")
    if not only or "multiprobe" in only:
        make_multiprobe_case()
        print("wrote search_multiprobe.npz")


if __name__ == "__main__":
    main()
