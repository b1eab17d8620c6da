"""GPU parity of the search kernel, through the C ABI.

The kernel is compared with
  * the oracle's LEX mode (its specification): ids, hops and distance
    evaluations bit-exact on every query;
  * the reference's own search steps (golden fixtures from oracle/_ref): ids
    equal on every query except those whose REF and LEX decision logs part at
    a float tie, which are counted, listed and checked to be ties.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu


def _index(song, g, **kw):
    return song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"]), **kw)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_matches_oracle_bit_exact(song, oracle, name):
    g = load_golden(name)
    ox = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    with _index(song, g) as ix:
        for pq in list(g["pqs"]) + [2, 7, 333]:
            pq = int(pq)
            ids, hops, evals = ix.search(g["queries"], pq, pq, stats=True)
            o_ids, o_hops, o_evals, _ = ox.kernel_search(g["queries"], pq, oracle.MODE_LEX)
            assert np.array_equal(ids, o_ids), "pq %d" % pq
            assert np.array_equal(hops, o_hops)
            assert np.array_equal(evals, o_evals)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_matches_reference_except_listed_ties(song, oracle, name, capsys):
    g = load_golden(name)
    ox = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    ties = []
    with _index(song, g) as ix:
        for pq in g["pqs"]:
            pq = int(pq)
            ids = ix.search(g["queries"], pq, pq)
            ref = g["kernel_ids_%d" % pq]
            for i in np.nonzero((ids != ref).any(axis=1))[0]:
                _, la = ox.kernel_search_log(g["queries"][i], pq, oracle.MODE_REF)
                _, lb = ox.kernel_search_log(g["queries"][i], pq, oracle.MODE_LEX)
                cls, at = oracle.classify(la, lb)
                assert cls == 1, "query %d pq %d differs from the reference without a tie" % (i, pq)
                ties.append((pq, int(i), int(at), oracle.EV_NAMES[int(la[at]["kind"])], float(la[at]["dist"])))
    with capsys.disabled():
        print("\n[%s] %d query results differ from the reference, all at float ties: %s"
              % (name, len(ties), ties[:8]))


def test_k_prefix_and_entry_points(song, oracle):
    g = load_golden("l2_s5_d32")
    with _index(song, g) as ix:
        full = ix.search(g["queries"], 100, 100)
        for k in (1, 10, 99):
            assert np.array_equal(ix.search(g["queries"], 100, k), full[:, :k])
        one = song.astar_search_batch(g["queries"], 100, g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
        assert np.array_equal(one, full)
        import torch
        dq = torch.from_numpy(g["queries"]).cuda()
        dout = torch.empty((dq.shape[0], 100), dtype=torch.int64, device="cuda")
        s = torch.cuda.current_stream()
        ix.search_device(dq.data_ptr(), dq.shape[0], 100, 100, dout.data_ptr(), stream=s.cuda_stream)
        s.synchronize()
        assert np.array_equal(dout.cpu().numpy().view(np.uint64), full)
        assert ix.search(g["queries"][:0], 10, 10).shape == (0, 10)


def _random_case(song, n, dim, metric, shift, seed, kind="unit"):
    from song_gb300 import datasets as D
    data = D.mixture(kind, n, dim, 8, seed=seed, center_seed=seed + 50)
    q = D.mixture(kind, 40, dim, 8, seed=seed + 1, center_seed=seed + 50)
    fixed = (1 << shift) - 1
    graph = song.graph_build(data, metric, shift, max(1, fixed // 2), fixed, 150, batch_div=0, nthreads=1)
    return data, q, graph


@pytest.mark.parametrize("dim,metric,shift", [(1, 0, 5), (3, 2, 4), (33, 1, 5), (130, 0, 5), (960, 2, 5),
                                              (26, 2, 3)])
def test_dims_and_shifts(song, oracle, dim, metric, shift):
    data, q, graph = _random_case(song, 700, dim, metric, shift, seed=dim)
    ox = oracle.OracleIndex(data, graph, shift, metric)
    with song.Index(graph, data, shift, metric) as ix:
        for pq in (16, 64):
            ids, hops, evals = ix.search(q, pq, pq, stats=True)
            o_ids, o_hops, o_evals, _ = ox.kernel_search(q, pq, oracle.MODE_LEX)
            assert np.array_equal(ids, o_ids)
            assert np.array_equal(evals, o_evals)


def test_small_graph_queue_runs_dry(song, oracle):
    """n < pq: the queue empties before pq vertices are popped; unfilled output
    slots are UINT64_MAX (the reference reads past its heap there)."""
    data, q, graph = _random_case(song, 30, 8, 0, 4, seed=3)
    ox = oracle.OracleIndex(data, graph, 4, 0)
    with song.Index(graph, data, 4, 0) as ix:
        ids = ix.search(q, 64, 64)
        o_ids, _, _, popped = ox.kernel_search(q, 64, oracle.MODE_LEX)
        assert np.array_equal(ids, o_ids)
        assert (popped < 64).all()
        assert (ids[:, 63] == song.NO_ID).all()


def test_degenerate_graphs(song, oracle):
    rng = np.random.default_rng(9)
    n, dim, shift = 64, 12, 3
    data = rng.standard_normal((n, dim)).astype(np.float32)
    data[5] = 0.0  # a zero vector: cosine distance 0 by the reference's rule
    graph = np.zeros(n << shift, np.uint64).reshape(n, 8)
    for v in range(n):
        deg = int(rng.integers(0, 8))
        graph[v, 0] = deg
        graph[v, 1:1 + deg] = rng.integers(0, n, deg)  # duplicates allowed
    graph[7, 0] = 0
    graph = graph.reshape(-1)
    q = rng.standard_normal((32, dim)).astype(np.float32)
    for metric in (0, 1, 2):
        ox = oracle.OracleIndex(data, graph, shift, metric)
        with song.Index(graph, data, shift, metric) as ix:
            for pq in (2, 5, 40):
                ids, hops, evals = ix.search(q, pq, pq, stats=True)
                o_ids, o_hops, o_evals, _ = ox.kernel_search(q, pq, oracle.MODE_LEX)
                assert np.array_equal(ids, o_ids)
                assert np.array_equal(hops, o_hops)
                assert np.array_equal(evals, o_evals)
    # vertex 0 without edges: one pop, one result
    g0 = graph.copy().reshape(n, 8)
    g0[0, 0] = 0
    with song.Index(g0.reshape(-1), data, shift, 0) as ix:
        ids = ix.search(q[:3], 10, 10)
        assert (ids[:, 0] == 0).all() and (ids[:, 1:] == song.NO_ID).all()


def test_largest_pq(song, oracle):
    g = load_golden("cos_s4_d16")
    ox = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    with _index(song, g) as ix:
        ids = ix.search(g["queries"][:16], 1023, 1023)
        o_ids, *_ = ox.kernel_search(g["queries"][:16], 1023, oracle.MODE_LEX)
        assert np.array_equal(ids, o_ids)


def test_fixhash_slot_function_on_device(song, oracle):
    rng = np.random.default_rng(1)
    ids = np.concatenate([np.arange(0, 70000, dtype=np.uint32),
                          rng.integers(0, 2 ** 31 - 1, 50000, dtype=np.uint32),
                          np.array([2 ** 31 - 1, 65535, 65536], np.uint32)])
    for pq in (2, 10, 100, 400, 1023):
        got = song.debug_fixhash(ids, pq)
        exp = np.array([oracle.lib().orc_fixhash_hash(8 * pq, int(x)) for x in ids[::97]], np.int32)
        assert np.array_equal(got[::97], exp)


def test_recall_matches_reference_semantics(song, oracle):
    """Small workload (15k x 16, cosine, degree-16 graph, pq 100): recall@10 of
    the kernel equals that of the reference-semantics oracle within 0.002,
    against an FP64 brute-force kNN."""
    from song_gb300 import datasets as D
    from song_gb300 import groundtruth as GT
    w = D.SMALL
    data = D.base_vectors(w)
    q = D.query_vectors(w, nq=2000)
    graph = song.graph_build(data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150, batch_div=0)
    gt, _ = GT.exact_knn_fp64(data, q, 10, w.metric)
    ox = oracle.OracleIndex(data, graph, w.shift, oracle.COS)
    with song.Index(graph, data, w.shift, w.metric) as ix:
        ids = ix.search(q, 100, 10)
    ref, *_ = ox.kernel_search(q, 100, oracle.MODE_REF)
    r_gpu = GT.recall(ids, gt, 10)
    r_ref = GT.recall(ref[:, :10], gt, 10)
    assert abs(r_gpu - r_ref) <= 0.002, (r_gpu, r_ref)
