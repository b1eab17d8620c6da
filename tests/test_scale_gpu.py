"""The 1,000,000 x 128 L2 workload at full size, where the oracle is too slow
to replay every query, checked through properties that hold at any size:

* every row holds distinct valid ids, in ascending exact distance, ties in
  ascending id.  The values are integers 0-255, so every partial sum of a
  distance is an integer below 2^24 and the kernel's FP32 distance is the
  exact one, whatever the summation order;
* the first k ids of a search with k = pq are the k-id search's (one search,
  one top list);
* the same ids again on a second run, and through the device-buffer call;
* from the two-level entry points (262,144 entries, 2048 clusters, 4 probed,
  4 starts) recall@10 against the FP64 exact kNN reaches 0.95 at pq 55, and
  the search needs fewer hops than from vertex 0 at the same pq."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MISSING = np.uint64(0xFFFFFFFFFFFFFFFF)


@pytest.fixture(scope="module")
def scale(song):
    from song_gb300 import datasets as D
    w = D.WORKLOADS["scale-1m-128d-l2"]
    data = D.base_vectors(w)
    queries = D.query_vectors(w)
    graph = song.graph_build_gpu(data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150, batch_div=64,
                                 device=0, nthreads=os.cpu_count())
    ix = song.Index(graph, data, w.shift, w.metric)
    yield w, data, queries, ix
    ix.free()


def _well_formed(ids, data, queries):
    from song_gb300 import groundtruth as GT
    n = data.shape[0]
    valid = ids != MISSING
    # a missing slot is only ever followed by missing slots
    assert np.all(valid[:, :-1] | ~valid[:, 1:])
    assert np.all(ids[valid] < n)
    for row, v in zip(ids, valid):
        assert len(set(row[v].tolist())) == int(v.sum())
    d = GT.distances_fp64(data, queries, ids, "l2")
    step = np.diff(d, axis=1)
    both = valid[:, 1:]
    assert np.all(step[both] >= 0)
    tie = both & (step == 0)
    assert np.all(np.diff(ids.astype(np.int64), axis=1)[tie] > 0)


def test_full_scale_plain_search_properties(song, scale):
    w, data, queries, ix = scale
    ids10, hops, evals = ix.search(queries, 55, 10, stats=True)
    _well_formed(ids10, data, queries)
    full = ix.search(queries, 55, 55)
    _well_formed(full, data, queries)
    assert np.array_equal(full[:, :10], ids10)
    assert np.array_equal(ix.search(queries, 55, 10), ids10)
    assert np.all(hops > 0) and np.all(evals >= hops)


def test_full_scale_entry_points_reach_the_recall_target(song, scale):
    import torch
    from song_gb300 import datasets as D
    from song_gb300 import groundtruth as GT
    w, data, queries, ix = scale
    _, plain_hops, _ = ix.search(queries, 55, 10, stats=True)
    ix.set_entries(song.sample_entries(w.n, 262144, seed=D.SEED_BASE + 10, shuffle=True), starts=4, coarse=2048,
                   probes=4)
    try:
        ids, hops, evals = ix.search(queries, 55, 10, stats=True)
        _well_formed(ids, data, queries)
        # the device-buffer call on a stream gives the same ids
        dq = torch.from_numpy(np.ascontiguousarray(queries)).cuda()
        out = torch.empty((queries.shape[0], 10), dtype=torch.int64, device="cuda")
        stream = torch.cuda.Stream()
        torch.cuda.synchronize()  # the upload above ran on another stream
        ix.search_device(dq.data_ptr(), queries.shape[0], 55, 10, out.data_ptr(), None, None, stream.cuda_stream)
        stream.synchronize()
        assert np.array_equal(out.cpu().numpy().view(np.uint64), ids)
        _, kth = GT.exact_knn_fp64(data, queries, 10, "l2")
        rec = GT.recall_tie_aware(ids, data, queries, kth, "l2", 10)
        assert rec >= 0.95, rec
        assert hops.mean() < plain_hops.mean()
    finally:
        ix.set_entries(None)
