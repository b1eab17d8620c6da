"""Learned early exit (small workload: 15k x 16 cos, degree-16 graph, pq 200).

Trained on traces of the plain search over training queries (seed 3) by the
library's own kernels, evaluated on held-out queries (seed 2): the exit must
cut the mean hop count substantially while keeping recall@10 within 0.01 of
the plain search, and beat a fixed hop budget of the same mean hop count."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small(song):
    from song_gb300 import datasets as D, groundtruth as GT
    w = D.SMALL
    data = D.base_vectors(w)
    graph = song.graph_build(data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150, batch_div=0)
    train_q = D.query_vectors(w, nq=6000, seed=D.SEED_TRAIN)
    test_q = D.query_vectors(w, nq=2000)
    gt, _ = GT.exact_knn_fp64(data, test_q, 10, w.metric)
    return w, data, graph, train_q, test_q, gt


def test_trace_labels_are_monotone(song, small):
    import torch
    from song_gb300 import learned as LE
    w, data, graph, train_q, _, _ = small
    with song.Index(graph, data, w.shift, w.metric) as ix:
        X, y = LE.trace_dataset(ix, train_q[:300], 200, 10)
    X, y = X.cpu().numpy(), y.cpu().numpy()
    # feature 0 is log2(1 + hop) / 10: consecutive within a query
    hop = np.rint(2.0 ** (X[:, 0] * 10.0) - 1.0).astype(np.int64)
    starts = np.nonzero(hop == 1)[0]
    assert len(starts) == 300
    for a, b in zip(starts, list(starts[1:]) + [len(hop)]):
        assert np.array_equal(hop[a:b], np.arange(1, b - a + 1))
        lab = y[a:b]
        assert lab[-1] == 1.0 and np.all(np.diff(lab) >= 0)  # once final, always final


def test_learned_exit_gains_over_plain_and_fixed_budget(song, small, capsys):
    import torch
    from song_gb300 import groundtruth as GT, learned as LE
    w, data, graph, train_q, test_q, gt = small
    pq, k = 200, 10
    with song.Index(graph, data, w.shift, w.metric) as ix:
        model = LE.fit(ix, train_q, pq, k, epochs=6, data=data, metric=w.metric, recall_slack=0.005)
        dq = torch.from_numpy(test_q).cuda()
        p_ids, p_hops, _ = LE.plain_stats(ix, dq, pq, k)
        l_ids, l_hops, _ = LE.evaluate(ix, dq, pq, k, model.params, model.threshold, model.min_hops, model.every)
        budget = int(round(l_hops.mean()))
        f_ids, f_hops, _ = LE.evaluate(ix, dq, pq, k, max_hops=budget)
    r_plain, r_learned, r_fixed = (GT.recall(x, gt, k) for x in (p_ids, l_ids, f_ids))
    with capsys.disabled():
        print("\n[learned exit] plain hops %.1f recall %.4f | learned hops %.1f recall %.4f | "
              "fixed budget %d hops recall %.4f | threshold %.2f, %d samples"
              % (p_hops.mean(), r_plain, l_hops.mean(), r_learned, budget, r_fixed, model.threshold,
                 model.info["samples"]))
    assert l_hops.mean() < 0.85 * p_hops.mean()
    assert r_learned >= r_plain - 0.01
    assert r_learned > r_fixed


@pytest.mark.parametrize("storage", ["f32", "bf16"])
def test_learned_kernel_without_exit_matches_exact_visited_oracle(song, oracle, storage):
    """The learned kernel keeps an exact visited set (no parity claim with the
    reference's FixHash); with the exit disabled it must equal the oracle's
    LEX_EXACT search over the stored rows bit for bit."""
    import torch
    from conftest import load_golden
    from song_gb300 import learned as LE
    for name in ("l2_s5_d32", "cos_s4_d16"):
        g = load_golden(name)
        shift, metric = int(g["shift"]), int(g["metric"])
        with song.Index(g["graph"], g["data"], shift, metric, storage=storage) as ix:
            ix.set_rerank(0)
            deq = song.dequantize_rows(ix.rows(), storage, g["data"].shape[1])
            ox = oracle.OracleIndex(deq, g["graph"], shift, metric)
            dq = torch.from_numpy(g["queries"]).cuda()
            for pq in (10, 100):
                ids, hops, evals = LE.evaluate(ix, dq, pq, pq, max_hops=1 << 30)
                o_ids, o_hops, o_evals, _ = ox.kernel_search(g["queries"], pq, oracle.MODE_LEX_EXACT)
                assert np.array_equal(ids, o_ids), (name, storage, pq)
                assert np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)


def test_trace_features_match_oracle(song, oracle):
    """Per-hop features and top-k change counts traced by the learned kernel
    equal the oracle's restatement (orc_kernel_search_trace): counts and hop
    numbers exactly, features to FP32 rounding (the kernel's log2 is the fast
    hardware approximation)."""
    import torch
    from conftest import load_golden
    for name in ("l2_s5_d32", "cos_s4_d16"):
        g = load_golden(name)
        shift, metric = int(g["shift"]), int(g["metric"])
        ox = oracle.OracleIndex(g["data"], g["graph"], shift, metric)
        q = g["queries"][:48]
        nq, th = q.shape[0], 512
        with song.Index(g["graph"], g["data"], shift, metric) as ix:
            for pq, k in ((100, 10), (40, 1)):
                dq = torch.from_numpy(np.ascontiguousarray(q)).cuda()
                tr = torch.zeros(nq * th * 6, dtype=torch.float32, device="cuda")
                fin = torch.zeros(nq * 2, dtype=torch.int32, device="cuda")
                out = torch.empty((nq, k), dtype=torch.int64, device="cuda")
                s = torch.cuda.current_stream()
                ix.trace_device(dq.data_ptr(), nq, pq, k, th, tr.data_ptr(), fin.data_ptr(), out.data_ptr(),
                                stream=s.cuda_stream)
                s.synchronize()
                tr = tr.view(nq, th, 6).cpu().numpy()
                fin = fin.view(nq, 2).cpu().numpy()
                for i in range(nq):
                    otr, ofin, oids, _, _ = ox.kernel_search_trace(q[i], pq, k, th)
                    n = otr.shape[0]
                    assert fin[i, 0] == ofin and fin[i, 1] == n, (name, pq, i)
                    assert np.array_equal(tr[i, :n, 5], otr[:, 5])
                    np.testing.assert_allclose(tr[i, :n, :5], otr[:, :5], rtol=2e-5, atol=2e-6)
