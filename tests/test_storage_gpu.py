"""BF16 and FP8-E4M3 storage with FP32 re-rank.

The low-precision search is an FP32 search over the dequantised vectors (BF16
widens exactly; FP8 is decoded and multiplied by the row's scale in float), so
with re-rank off its ids, hops and evaluations must equal the oracle's LEX
search over the rows the index stores.  With re-rank on, the first k must be
the best R list entries re-sorted by the exact FP32 kernel distance."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu


def _bf16_rne(x):
    u = x.view(np.uint32).astype(np.uint64)
    r = (u + 0x7FFF + ((u >> 16) & 1)) >> 16
    return r.astype(np.uint16)


@pytest.mark.parametrize("storage", ["bf16", "fp8"])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_low_precision_search_equals_oracle_on_stored_rows(song, oracle, storage, name):
    g = load_golden(name)
    shift, metric = int(g["shift"]), int(g["metric"])
    with song.Index(g["graph"], g["data"], shift, metric, storage=storage) as ix:
        ix.set_rerank(0)
        deq = song.dequantize_rows(ix.rows(), storage, g["data"].shape[1])
        ox = oracle.OracleIndex(deq, g["graph"], shift, metric)
        for pq in (10, 50, 100):
            ids, hops, evals = ix.search(g["queries"], pq, pq, stats=True)
            o_ids, o_hops, o_evals, _ = ox.kernel_search(g["queries"], pq, oracle.MODE_LEX)
            assert np.array_equal(ids, o_ids), (storage, pq)
            assert np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)


@pytest.mark.parametrize("storage", ["bf16", "fp8"])
def test_rerank_orders_by_exact_fp32(song, oracle, storage):
    g = load_golden("l2_s5_d32")
    shift, metric = int(g["shift"]), int(g["metric"])
    data, q = g["data"], g["queries"]
    with song.Index(g["graph"], data, shift, metric, storage=storage) as ix:
        deq = song.dequantize_rows(ix.rows(), storage, data.shape[1])
        ox = oracle.OracleIndex(deq, g["graph"], shift, metric)
        pq, k = 50, 10
        o_ids, *_ = ox.kernel_search(q, pq, oracle.MODE_LEX)
        for R in (10, 25, -1):
            ix.set_rerank(R)
            got = ix.search(q, pq, k)
            RR = pq if R == -1 else max(R, k)
            for i in range(q.shape[0]):
                cand = o_ids[i, :RR]
                d = np.array([oracle.kernel_distance(metric, q[i], data[c]) for c in cand], np.float32)
                order = np.lexsort((cand, d))
                assert np.array_equal(got[i], cand[order][:k]), (storage, R, i)


def test_bf16_rows_are_round_to_nearest_even(song):
    g = load_golden("cos_s5_d26")
    with song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"]), storage="bf16") as ix:
        raw = ix.rows()
    got = raw.view(np.uint16)[:, :g["data"].shape[1]]
    assert np.array_equal(got, _bf16_rne(np.ascontiguousarray(g["data"])))


def test_fp8_rows_match_e4m3_conversion(song):
    ml = pytest.importorskip("ml_dtypes")
    g = load_golden("ip_s5_d24")
    data = g["data"]
    with song.Index(g["graph"], data, int(g["shift"]), int(g["metric"]), storage="fp8") as ix:
        raw = ix.rows()
    dim = data.shape[1]
    dpad = (dim + 15) // 16 * 16
    scale = raw[:, dpad:dpad + 4].copy().view(np.float32)[:, 0]
    amax = np.abs(data).max(axis=1)
    exp_scale = np.where(amax > 0, (amax / np.float32(448.0)).astype(np.float32), np.float32(1.0))
    assert np.array_equal(scale, exp_scale)
    y = (data / scale[:, None]).astype(np.float32)
    ref = np.clip(y, -448, 448).astype(ml.float8_e4m3fn).view(np.uint8)
    assert np.array_equal(raw[:, :dim], ref)


def test_recall_with_rerank_close_to_fp32(song):
    from song_gb300 import datasets as D, groundtruth as GT
    w = D.SMALL
    data = D.base_vectors(w)
    q = D.query_vectors(w, nq=1000)
    graph = song.graph_build(data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150, batch_div=0)
    gt, _ = GT.exact_knn_fp64(data, q, 10, w.metric)
    rec = {}
    for st in ("f32", "bf16", "fp8"):
        with song.Index(graph, data, w.shift, w.metric, storage=st) as ix:
            rec[st] = GT.recall(ix.search(q, 100, 10), gt, 10)
    assert rec["bf16"] >= rec["f32"] - 0.01 and rec["fp8"] >= rec["f32"] - 0.03, rec
