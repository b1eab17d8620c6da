"""The measurement's own arithmetic, on the CPU: the FP64 exact k-nearest
neighbours behind every recall figure (song_gb300/groundtruth.py) against a
full brute force, the two recall definitions on hand-made cases, and the
seeded synthetic workloads (song_gb300/datasets.py): deterministic, with the
shapes, metrics and value ranges of the configurations they stand in for."""
import numpy as np
import pytest

from song_gb300 import datasets as D
from song_gb300 import groundtruth as GT


def _brute(data, queries, k, metric):
    n = data.shape[0]
    ids = np.tile(np.arange(n, dtype=np.int64), (queries.shape[0], 1))
    d = GT.distances_fp64(data, queries, ids, metric)
    order = np.lexsort((ids, d), axis=1)[:, :k]
    return np.take_along_axis(ids, order, 1), np.take_along_axis(d, order, 1)


@pytest.mark.parametrize("metric", ["l2", "ip", "cos"])
def test_exact_knn_matches_brute_force(metric):
    rng = np.random.default_rng(3)
    data = rng.standard_normal((900, 24)).astype(np.float32)
    data[17] = 0.0  # a zero-norm row: distance 0 under cos, as in the kernel
    queries = rng.standard_normal((50, 24)).astype(np.float32)
    ids, kth = GT.exact_knn_fp64(data, queries, 10, metric, device="cpu")
    b_ids, b_d = _brute(data, queries, 10, metric)
    assert np.array_equal(ids, b_ids)
    assert np.array_equal(kth, b_d[:, 9])


def test_exact_knn_with_ties_keeps_the_kth_distance():
    """Integer-valued L2 data (the 1M x 128 workload's kind) has many equal
    distances: the k-th distance is exact and the returned ids are k of the
    ids at or below it, ties to the smaller id."""
    data = D.mixture("byte", 2000, 8, 4, seed=5, center_seed=6)
    queries = D.mixture("byte", 30, 8, 4, seed=7, center_seed=6)
    ids, kth = GT.exact_knn_fp64(data, queries, 10, "l2", device="cpu")
    b_ids, b_d = _brute(data, queries, 10, "l2")
    assert np.array_equal(kth, b_d[:, 9])
    d = GT.distances_fp64(data, queries, ids, "l2")
    assert np.all(d <= kth[:, None])
    assert np.array_equal(ids, b_ids)


def test_recall_definitions():
    gt = np.array([[1, 2, 3, 4], [5, 6, 7, 8]])
    found = np.array([[4, 1, 9, 3], [6, 0, 0, 0]])
    assert GT.recall(found, gt, 4) == pytest.approx((3 + 1) / 8)
    assert GT.recall(found, gt, 2) == pytest.approx((1 + 1) / 4)  # first two of each row only
    # Tie-aware: on a line, the query at 0 has id 0 at distance 0 and ids 1
    # and 2 both at distance 1, the exact 2nd-nearest distance, so either
    # of them counts as the 2nd.
    data = np.array([[0.0], [1.0], [-1.0], [5.0]], dtype=np.float32)
    q = np.array([[0.0]], dtype=np.float32)
    ids, kth = GT.exact_knn_fp64(data, q, 2, "l2", device="cpu")
    assert list(ids[0]) == [0, 1] and kth[0] == 1.0
    assert GT.recall_tie_aware(np.array([[0, 2]]), data, q, kth, "l2", 2) == 1.0
    assert GT.recall_tie_aware(np.array([[0, 3]]), data, q, kth, "l2", 2) == 0.5
    # an empty slot (UINT64_MAX) is never correct
    empty = np.array([[0, 0xFFFFFFFFFFFFFFFF]], dtype=np.uint64)
    assert GT.recall_tie_aware(empty, data, q, kth, "l2", 2) == 0.5
    # an id returned twice (a vertex the visited hash lost, listed again) counts once
    assert GT.recall_tie_aware(np.array([[0, 0]]), data, q, kth, "l2", 2) == 0.5
    assert GT.recall_tie_aware(np.array([[1, 0, 1]]), data, q, kth, "l2", 3) == pytest.approx(2 / 3)


@pytest.mark.parametrize("kind,lo,hi,integer", [("byte", 0, 255, True), ("unit", -1, 1, False),
                                                ("unit01", 0, 1, False), ("normal", -np.inf, np.inf, False)])
def test_mixtures_are_seeded_and_in_range(kind, lo, hi, integer):
    a = D.mixture(kind, 3000, 16, 10, seed=1, center_seed=9, chunk=1000)
    b = D.mixture(kind, 3000, 16, 10, seed=1, center_seed=9, chunk=1000)
    c = D.mixture(kind, 3000, 16, 10, seed=2, center_seed=9, chunk=1000)
    assert a.dtype == np.float32 and a.shape == (3000, 16)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert a.min() >= lo and a.max() <= hi
    if integer:
        assert np.array_equal(a, np.rint(a))


def test_workload_table():
    w = D.WORKLOADS
    s = w["scale-1m-128d-l2"]
    assert (s.n, s.dim, s.metric, s.shift, s.fixed_degree, s.search_degree, s.n_queries, s.kind) == \
        (1_000_000, 128, "l2", 5, 31, 15, 10_000, "byte")
    m = w["small-15k-16d-cos"]
    assert (m.n, m.dim, m.metric, m.shift, m.fixed_degree, m.centers, m.n_queries) == \
        (15_000, 16, "cos", 4, 15, 26, 5_000)
    p = w["precision-1m-960d-cos"]
    assert (p.n, p.dim, p.metric, p.n_queries, p.centers, p.kind) == (1_000_000, 960, "cos", 1_000, 500, "unit01")
    g = w["learned-3m-256d-l2"]
    assert (g.n, g.dim, g.metric, g.centers, g.n_queries) == (3_000_000, 256, "l2", 2_000, 10_000)
    for x in w.values():
        assert x.fixed_degree == (1 << x.shift) - 1
    # base and query sets share the mixture's centres: queries sit near base points
    q = D.query_vectors(m, nq=20)
    base = D.base_vectors(m, n=4000)
    _, kth = GT.exact_knn_fp64(base, q, 1, "l2", device="cpu")
    assert np.median(kth) < 16 * (2 * 0.15) ** 2
