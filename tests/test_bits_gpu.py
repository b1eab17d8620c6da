"""The 256-bit code row format (SONG_STORAGE_BITS), the reference's bit-hash
path (hash_warp_no_heap_astar_accelerator.h:22-41 codes, __popc distances) as
a row format of the same search:

* the base and query codes equal the oracle's orc_hash_codes bit for bit (the
  dot products summed as the kernel sums distances);
* without rerank, ids, hops and evaluations equal the oracle's LEX search over
  the codes with Hamming distances;
* with the FP32 rerank, the ids are the oracle's final list re-sorted by the
  index metric's FP32 distance;
* the rerank brings recall close to the FP32 rows' on a clustered workload."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu


def _bits_index(song, g, planes):
    ix = song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"]), storage="bits")
    ix.set_hash_planes(planes)
    return ix


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_codes_and_hamming_search_match_oracle(song, oracle, name):
    g = load_golden(name)
    planes = song.hash_planes(g["data"].shape[1], seed=5)
    codes = oracle.hash_codes(g["data"], planes)
    qcodes = oracle.hash_codes(g["queries"], planes)
    with _bits_index(song, g, planes) as ix:
        assert np.array_equal(ix.rows().view(np.uint32), codes)
        ix.set_rerank(0)
        ids, hops, evals = ix.search(g["queries"], 50, 50, stats=True)
        ox = oracle.OracleIndex(codes.view(np.float32), g["graph"], int(g["shift"]), oracle.HAMMING)
        o_ids, o_hops, o_evals, _ = ox.kernel_search(qcodes.view(np.float32), 50, oracle.MODE_LEX)
        assert np.array_equal(ids, o_ids)
        assert np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)
        # FP32 rerank of the whole list (the default), then the first 10
        ix.set_rerank(-1)
        rr = ix.search(g["queries"], 50, 10)
    fx = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    for i, row in enumerate(o_ids):
        row = row[row != oracle.NO_ID]
        d = [oracle.kernel_distance(int(g["metric"]), g["queries"][i], g["data"][v]) for v in row]
        order = sorted(range(len(row)), key=lambda j: (d[j], int(row[j])))
        assert list(rr[i][:min(10, len(row))]) == [row[j] for j in order[:10]], (name, i)


def test_rerank_recovers_recall(song):
    from song_gb300 import datasets as D
    from song_gb300 import groundtruth as GT
    w = D.WORKLOADS["small-15k-16d-cos"]
    data = D.base_vectors(w)
    q = D.query_vectors(w, nq=1000)
    graph = song.graph_build(data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150, batch_div=64)
    _, kth = GT.exact_knn_fp64(data, q, 10, w.metric)
    with song.Index(graph, data, w.shift, w.metric) as f32:
        r32 = GT.recall_tie_aware(f32.search(q, 200, 10), data, q, kth, w.metric, 10)
    with song.Index(graph, data, w.shift, w.metric, storage="bits") as ix:
        ix.set_hash_planes(song.hash_planes(w.dim))
        rb = GT.recall_tie_aware(ix.search(q, 200, 10), data, q, kth, w.metric, 10)
        ix.set_rerank(0)
        rn = GT.recall_tie_aware(ix.search(q, 200, 10), data, q, kth, w.metric, 10)
    print("recall@10 pq 200: f32 %.4f, bits + rerank %.4f, bits alone %.4f" % (r32, rb, rn))
    assert rb > rn and rb > r32 - 0.1


def test_bits_index_needs_planes(song):
    g = load_golden("cos_s4_d16")
    with song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"]), storage="bits") as ix:
        with pytest.raises(song.SongError):
            ix.search(g["queries"], 20, 10)
