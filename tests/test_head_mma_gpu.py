"""Head phase of the two-level entry choice on the tensor cores (head_mma.cu).

  * the TF32 tcgen05 scores stay inside the error bound the shortlist relies
    on (|s~ - q.x| <= (2^-9 + 2^-14) |q||x|), with room to spare;
  * the searches from the tensor-core shortlist equal those from the exact
    CUDA-core scan and the oracle (same starts, ids, hops, evaluations) for
    every metric, for dims of one to thirty 32-float slabs (stage reuse), and
    when a query batch spans several score chunks;
  * a copy wait that cannot complete returns SONG_ERR_TIMEOUT and leaves the
    index usable.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(song, n, dim, metric, nq, seed, kind="unit"):
    from song_gb300 import datasets as D
    data = D.mixture(kind, n, dim, 16, seed=seed, center_seed=seed + 50)
    q = D.mixture(kind, nq, dim, 16, seed=seed + 1, center_seed=seed + 50)
    graph = song.graph_build(data, metric, 5, 15, 31, 150, batch_div=0, nthreads=4)
    return data, q, graph


@pytest.mark.parametrize("dim,kind", [(128, "byte"), (96, "unit"), (260, "unit")])
def test_scores_within_the_error_bound(song, dim, kind):
    import torch
    data, q, graph = _case(song, 3000, dim, 0, 700, seed=dim, kind=kind)
    rng = np.random.default_rng(dim)
    ent = rng.choice(len(data), 1500, replace=False).astype(np.uint64)
    coarse = 300
    with song.Index(graph, data, 5, 0) as ix:
        ix.set_entries(ent, starts=2, coarse=coarse, probes=4)
        assert ix.debug_head_path(True)
        heads = data[np.sort(ent[:coarse])].astype(np.float64)  # coarse rows in id order
        ld = (coarse + 3) // 4 * 4
        dq = torch.from_numpy(q).cuda()
        ds = torch.zeros((len(q), ld), dtype=torch.float32, device="cuda")
        ix.debug_head_scores(dq.data_ptr(), len(q), ds.data_ptr(), ld)
        got = ds.cpu().numpy()[:, :coarse].astype(np.float64)
    exact = q.astype(np.float64) @ heads.T
    scale = np.linalg.norm(q.astype(np.float64), axis=1)[:, None] * np.linalg.norm(heads, axis=1)[None, :]
    ratio = float(np.max(np.abs(got - exact) / np.maximum(scale, 1e-30)))
    bound = 2.0 ** -9 + 2.0 ** -14
    print("\n[head scores] dim %d: max |s~ - q.x| / (|q||x|) = %.3g (bound %.3g)" % (dim, ratio, bound))
    assert ratio <= 0.75 * bound


@pytest.mark.parametrize("dim,metric", [(128, 0), (128, 1), (128, 2), (32, 0), (200, 2), (960, 0)])
def test_tensor_shortlist_equals_exact_scan_and_oracle(song, oracle, dim, metric):
    data, q, graph = _case(song, 2500, dim, metric, 300, seed=dim + 7 * metric)
    ox = oracle.OracleIndex(data, graph, 5, metric)
    rng = np.random.default_rng(dim + metric)
    ent = rng.choice(len(data), 900, replace=False).astype(np.uint64)
    coarse, probes, ns = 150, 4, 3
    starts = ox.nearest_entry_2level(q, ent, coarse, probes, ns)
    o_ids, o_hops, o_evals, _ = ox.kernel_search_from(q, starts, 40, oracle.MODE_LEX)
    with song.Index(graph, data, 5, metric) as ix:
        ix.set_entries(ent, starts=ns, coarse=coarse, probes=probes)
        assert ix.debug_head_path(True)
        ix.debug_head_stats(True)
        ids, hops, evals = ix.search(q, 40, 40, stats=True)
        nq_seen, rescored, full = ix.debug_head_stats(False)
        ix.debug_head_path(False)
        ids0, hops0, evals0 = ix.search(q, 40, 40, stats=True)
    assert nq_seen == len(q)
    print("\n[head shortlist] dim %d metric %d: %.1f of %d heads re-scored per query, %d full scans"
          % (dim, metric, rescored / nq_seen, coarse, full))
    assert np.array_equal(ids, ids0) and np.array_equal(hops, hops0) and np.array_equal(evals, evals0)
    assert np.array_equal(ids, o_ids) and np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)


@pytest.mark.parametrize("dim,metric", [(128, 0), (64, 2), (256, 1)])
def test_large_clusters_many_queries(song, oracle, dim, metric):
    """16 clusters of ~250 entries probed by ~500 queries each: many warp
    tasks per cluster, several row buffers per task; the same starts as the
    oracle with either head phase."""
    data, q, graph = _case(song, 6000, dim, metric, 2000, seed=dim + metric + 100)
    ox = oracle.OracleIndex(data, graph, 5, metric)
    rng = np.random.default_rng(dim + 1)
    ent = rng.choice(len(data), 4000, replace=False).astype(np.uint64)
    coarse, probes, ns = 16, 4, 4
    starts = ox.nearest_entry_2level(q, ent, coarse, probes, ns)
    o_ids, o_hops, o_evals, _ = ox.kernel_search_from(q, starts, 30, oracle.MODE_LEX)
    with song.Index(graph, data, 5, metric) as ix:
        ix.set_entries(ent, starts=ns, coarse=coarse, probes=probes)
        assert ix.debug_head_path(True)
        got = ix.search(q, 30, 30, stats=True)
        ix.debug_head_path(False)
        ref = ix.search(q, 30, 30, stats=True)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    assert np.array_equal(got[0], o_ids) and np.array_equal(got[1], o_hops) and np.array_equal(got[2], o_evals)


def test_batch_spanning_several_score_chunks(song, oracle):
    """2048 coarse entries: a chunk holds 4096 queries' scores, so 9000
    queries take three chunks (the last one partial)."""
    data, q, graph = _case(song, 6000, 64, 0, 9000, seed=3)
    rng = np.random.default_rng(3)
    ent = rng.choice(len(data), 4096, replace=False).astype(np.uint64)
    with song.Index(graph, data, 5, 0) as ix:
        ix.set_entries(ent, starts=2, coarse=2048, probes=3)
        assert ix.debug_head_path(True)
        ids, hops, evals = ix.search(q, 30, 10, stats=True)
        ix.debug_head_path(False)
        ids0, hops0, evals0 = ix.search(q, 30, 10, stats=True)
    assert np.array_equal(ids, ids0) and np.array_equal(hops, hops0) and np.array_equal(evals, evals0)


def test_unaligned_dims_fall_back_to_the_exact_scan(song, oracle):
    data, q, graph = _case(song, 800, 26, 2, 50, seed=11)
    ox = oracle.OracleIndex(data, graph, 5, 2)
    ent = np.arange(0, 800, 4, dtype=np.uint64)
    starts = ox.nearest_entry_2level(q, ent, 20, 3, 2)
    with song.Index(graph, data, 5, 2) as ix:
        ix.set_entries(ent, starts=2, coarse=20, probes=3)
        assert not ix.debug_head_path(True)
        ids = ix.search(q, 30, 30)
    assert np.array_equal(ids, ox.kernel_search_from(q, starts, 30, oracle.MODE_LEX)[0])


def test_head_copy_wait_that_cannot_complete_times_out(song):
    import torch
    data, q, graph = _case(song, 1200, 64, 0, 200, seed=5)
    ent = np.arange(0, 1200, 3, dtype=np.uint64)
    with song.Index(graph, data, 5, 0) as ix:
        ix.set_entries(ent, starts=2, coarse=100, probes=2)
        assert ix.debug_head_path(True)
        expected = ix.search(q, 30, 10)
        dq = torch.from_numpy(q).cuda()
        ds = torch.zeros((len(q), 100), dtype=torch.float32, device="cuda")
        ix.debug_set_wait(wait_limit=2000, extra_tx=16)
        t = time.perf_counter()
        with pytest.raises(song.SongError):
            ix.debug_head_scores(dq.data_ptr(), len(q), ds.data_ptr(), 100)
        with pytest.raises(song.SongError) as e:
            ix.search(q, 30, 10)
        assert e.value.status == song.SONG_ERR_TIMEOUT
        assert time.perf_counter() - t < 20.0
        ix.debug_set_wait()
        assert np.array_equal(ix.search(q, 30, 10), expected)
