"""The CPU oracle against the golden vectors the reference's own code produced
(tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, GOLDEN


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_ref_mode_matches_reference_kernel_steps(oracle, name):
    g = load_golden(name)
    ix = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    for pq in g["pqs"]:
        ids, hops, evals, popped = ix.kernel_search(g["queries"], int(pq), oracle.MODE_REF)
        assert np.array_equal(ids, g["kernel_ids_%d" % pq])
        assert np.array_equal(hops, g["kernel_hops_%d" % pq])
        assert np.array_equal(evals, g["kernel_evals_%d" % pq])
        assert np.array_equal(popped, g["kernel_popped_%d" % pq])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_cpu_search_matches_reference(oracle, name):
    g = load_golden(name)
    ix = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    for k in g["cpu_ks"]:
        ids, _ = ix.cpu_search(g["queries"], int(k))
        assert np.array_equal(ids, g["cpu_ids_%d" % k])


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_lex_mode_differs_only_by_ties(oracle, name):
    """The GB300 kernel's specification (sorted queues, ties by id) against the
    reference's heaps: every query whose ids differ must part at a tie."""
    g = load_golden(name)
    ix = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    for pq in g["pqs"]:
        lex, *_ = ix.kernel_search(g["queries"], int(pq), oracle.MODE_LEX)
        ref = g["kernel_ids_%d" % pq]
        for i in np.nonzero((lex != ref).any(axis=1))[0]:
            _, la = ix.kernel_search_log(g["queries"][i], int(pq), oracle.MODE_REF)
            _, lb = ix.kernel_search_log(g["queries"][i], int(pq), oracle.MODE_LEX)
            cls, at = oracle.classify(la, lb)
            assert cls == 1, "query %d pq %d parts at event %d without a tie" % (i, pq, at)


def test_fixhash_matches_reference(oracle):
    z = np.load(GOLDEN + "/fixhash_ops.npz")
    for pq in (8, 100):
        got = oracle.fixhash_ops(pq, z["ops_%d" % pq], z["keys_%d" % pq])
        assert np.array_equal(got, z["results_%d" % pq])


def test_fixhash_loses_entries_like_the_reference(oracle):
    """The reference's backward-shift delete can drop a live key (fixhash.h:59-93);
    the fixture sequence for the 64-slot table exercises it."""
    z = np.load(GOLDEN + "/fixhash_ops.npz")
    ops, keys, res = z["ops_8"], z["keys_8"], z["results_8"]
    live = {}
    false_neg = 0
    for op, k, r in zip(ops, keys, res):
        if op == 0:
            live[k] = live.get(k, 0) + 1
        elif op == 1:
            if live.get(k, 0):
                live[k] -= 1
        elif live.get(k, 0) and r == 0:
            false_neg += 1
    assert false_neg > 0


def test_kernel_distance_order(oracle):
    """Lane-strided sums + butterfly differ from a plain left-to-right sum in
    float; check the restatement on a hand case against a numpy model."""
    rng = np.random.default_rng(3)
    for dim in (1, 16, 31, 32, 33, 100, 128, 960):
        q = rng.standard_normal(dim).astype(np.float32)
        x = rng.standard_normal(dim).astype(np.float32)
        part = np.zeros(32, np.float32)
        for lane in range(32):
            acc = np.float32(0)
            for j in range(lane, dim, 32):
                d = np.float32(q[j] - x[j])
                acc = np.float32(np.float64(d) * np.float64(d) + np.float64(acc))  # exact fma then round
            part[lane] = acc
        for off in (16, 8, 4, 2, 1):
            part = (part + part[np.arange(32) ^ off]).astype(np.float32)
        assert oracle.kernel_distance(oracle.L2, q, x) == part[0]


def test_cpu_distance_matches_double_accumulation(oracle):
    rng = np.random.default_rng(4)
    x = rng.standard_normal(77).astype(np.float32)
    q = rng.standard_normal(77).astype(np.float32)
    ref = 0.0
    for a, b in zip(x, q):
        d = np.float32(a - b)
        ref += float(np.float32(d * d))
    assert oracle.cpu_distance(oracle.L2, x, q) == ref


def test_fma_probe_separates_contraction(oracle):
    """dim 128 L2 cases whose order depends on fused vs separate multiply-add:
    the oracle with FMA reproduces the reference containers' ids, without FMA
    it does not."""
    z = np.load(GOLDEN + "/fma_probe.npz")
    graph = z["graph"].astype(np.uint64)
    for i in range(z["data"].shape[0]):
        ox = oracle.OracleIndex(z["data"][i], graph, int(z["shift"]), oracle.L2)
        f, *_ = ox.kernel_search(z["queries"][i:i + 1], int(z["pq"]), oracle.MODE_REF, use_fma=True)
        nf, *_ = ox.kernel_search(z["queries"][i:i + 1], int(z["pq"]), oracle.MODE_REF, use_fma=False)
        assert np.array_equal(f[0], z["fma_ids"][i]) and np.array_equal(nf[0], z["nofma_ids"][i])
        assert not np.array_equal(f[0], nf[0])


@pytest.mark.parametrize("name", ["l2_s5_d32", "cos_s4_d16"])
def test_trace_is_consistent_with_the_search(oracle, name):
    """The oracle's per-hop trace runs the same search (ids, hops, evals) and
    its top-k change count only grows, ending at the final count; the hop
    feature counts hops and the stagnation feature restarts at each change."""
    g = load_golden(name)
    ox = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    q = g["queries"][:16]
    ids, hops, evals, _ = ox.kernel_search(q, 100, oracle.MODE_LEX_EXACT)
    for i in range(q.shape[0]):
        tr, fin, out, h, e = ox.kernel_search_trace(q[i], 100, 10, 4096)
        assert np.array_equal(out, ids[i]) and h == hops[i] and e == evals[i]
        assert tr.shape[0] == h and tr[-1, 5] == fin and np.all(np.diff(tr[:, 5]) >= 0)
        assert np.allclose(2.0 ** (tr[:, 0] * 10.0) - 1.0, np.arange(1, h + 1), atol=1e-3)
        stag = np.rint(2.0 ** (tr[:, 2] * 10.0) - 1.0)
        changed = np.concatenate([[True], np.diff(tr[:, 5]) > 0])
        assert np.all(stag[changed] == 0) and np.all(stag[~changed] > 0)


def test_two_level_entry_choice_follows_its_definition(oracle):
    """orc_nearest_entry_2level against a direct restatement: heads are
    ids[:coarse]; every other entry joins its nearest head; a query takes the
    ns nearest entries of its `probes` nearest heads' clusters (ties to the
    smaller id throughout); and the flat choice against brute force."""
    g = load_golden("cos_s5_d26")
    metric = int(g["metric"])
    ox = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), metric)
    rng = np.random.default_rng(3)
    ent = rng.choice(g["data"].shape[0], 120, replace=False).astype(np.uint64)
    coarse, probes, ns = 9, 3, 2
    q = g["queries"][:12]

    def dist(qv, i):
        return oracle.kernel_distance(metric, qv, g["data"][int(i)])

    def nearest(qv, ids, m):
        return sorted(ids, key=lambda i: (dist(qv, i), int(i)))[:m]

    heads = list(ent[:coarse])
    owner = {int(e): int(e) for e in heads}
    for e in ent[coarse:]:
        owner[int(e)] = int(nearest(g["data"][int(e)], heads, 1)[0])
    got = ox.nearest_entry_2level(q, ent, coarse, probes, ns)
    for i in range(q.shape[0]):
        probed = set(int(h) for h in nearest(q[i], heads, probes))
        cand = [e for e in ent if owner[int(e)] in probed]
        assert [int(x) for x in got[i]] == [int(x) for x in nearest(q[i], cand, ns)]
    flat = ox.nearest_entry(q, ent, ns=4)
    for i in range(q.shape[0]):
        assert [int(x) for x in flat[i]] == [int(x) for x in nearest(q[i], list(ent), 4)]


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_builder_reproduces_reference_graph(oracle, name):
    """orc_graph_build one vertex at a time is the reference's own builder:
    the golden graphs were written by it."""
    g = load_golden(name)
    shift = int(g["shift"])
    built = oracle.graph_build(g["data"], int(g["metric"]), shift, 7 if shift == 4 else 15, (1 << shift) - 1, 150,
                               batch_div=0, nthreads=1)
    assert np.array_equal(built, g["graph"])


@pytest.mark.parametrize("name,n,div", [("scale-1m-128d-l2", 20000, 64), ("small-15k-16d-cos", 15000, 64),
                                        ("precision-1m-960d-cos", 2000, 16)])
def test_oracle_builder_batches_equal_the_product_builder(oracle, song, name, n, div):
    """With batch_div > 0 the oracle's builder and the product's batch-parallel
    builder agree bit for bit (the reference arm of the bench builds its graph
    with the oracle, so both arms search the same graph)."""
    from song_gb300 import datasets as D
    w = D.WORKLOADS[name]
    data = D.base_vectors(w, n=n)
    args = (data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150)
    a = oracle.graph_build(*args, batch_div=div, nthreads=4)
    b = song.graph_build(*args, batch_div=div, nthreads=4)
    assert np.array_equal(a, b)


def test_ref_mode_matches_reference_multiprobe_steps(oracle):
    """The N_MULTIPROBE / FINISH_CNT knobs (warp_astar_accelerator.h:29-30,
    184-232) and the double-check switch (:307-310) away from their defaults:
    REF mode against the reference containers' results."""
    z = np.load(GOLDEN + "/search_multiprobe.npz")
    for name in ("cos_s4_d16", "l2_s5_d32"):
        g = load_golden(name)
        ix = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
        for probes, fc, dc in z["knobs"]:
            for pq in g["pqs"]:
                key = "%s_p%d_f%d_d%d_%d" % (name, probes, fc, dc, pq)
                ids, hops, evals, popped = ix.kernel_search(g["queries"], int(pq), oracle.MODE_REF,
                                                            probes=int(probes), finish_cnt=int(fc),
                                                            double_check=bool(dc))
                assert np.array_equal(ids, z["ids_" + key]), key
                assert np.array_equal(hops, z["hops_" + key]), key
                assert np.array_equal(evals, z["evals_" + key]), key
                assert np.array_equal(popped, z["popped_" + key]), key


def test_lex_mode_multiprobe_differs_only_by_ties(oracle):
    z = np.load(GOLDEN + "/search_multiprobe.npz")
    for name in ("cos_s4_d16", "l2_s5_d32"):
        g = load_golden(name)
        ix = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
        for probes, fc, dc in z["knobs"]:
            kw = dict(probes=int(probes), finish_cnt=int(fc), double_check=bool(dc))
            for pq in g["pqs"]:
                lex, *_ = ix.kernel_search(g["queries"], int(pq), oracle.MODE_LEX, **kw)
                ref = z["ids_%s_p%d_f%d_d%d_%d" % (name, probes, fc, dc, pq)]
                for i in np.nonzero((lex != ref).any(axis=1))[0]:
                    _, la = ix.kernel_search_log(g["queries"][i], int(pq), oracle.MODE_REF, **kw)
                    _, lb = ix.kernel_search_log(g["queries"][i], int(pq), oracle.MODE_LEX, **kw)
                    cls, at = oracle.classify(la, lb)
                    assert cls == 1, "%s %s pq %d query %d parts without a tie" % (name, kw, pq, i)
