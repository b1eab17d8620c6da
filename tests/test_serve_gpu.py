"""Continuous-batching server: two resident indexes served at once by
persistent kernels, requests of differing size, pq and k admitted as slots
free up.  Every request's ids must equal what song_search returns for the
same queries alone (the kernel is deterministic per query: tolerance 0)."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _requests(rng, nreq, nq_total, choices_pq, choices_k):
    out = []
    for _ in range(nreq):
        size = int(rng.integers(1, 49))
        start = int(rng.integers(0, nq_total - size + 1))
        k = int(rng.choice(choices_k))
        pq = int(max(k, rng.choice(choices_pq)))
        out.append((start, size, pq, k))
    return out


def test_two_indexes_in_the_mix_equal_alone(song):
    from song_gb300.serve import Server
    rng = np.random.default_rng(0)
    cases = [load_golden("l2_s5_d32"), load_golden("cos_s4_d16")]
    indexes = [song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"])) for g in cases]
    reqs = [_requests(rng, 40, g["queries"].shape[0], (10, 50, 100), (1, 10, 50)) for g in cases]
    # results alone, before any server holds the GPU
    alone = [[ix.search(g["queries"][s:s + n], pq, k) for (s, n, pq, k) in rr]
             for ix, g, rr in zip(indexes, cases, reqs)]
    servers = [Server(ix, max_pq=100, max_k=50, slots=3, slot_queries=64, sm_fraction=0.5) for ix in indexes]
    try:
        pending = {}
        for si in range(2):
            for ri, (s, n, pq, k) in enumerate(reqs[si]):
                t = servers[si].submit(cases[si]["queries"][s:s + n], pq, k)
                pending[(si, t)] = ri
        got = [[None] * len(reqs[0]), [None] * len(reqs[1])]
        import time
        t0 = time.time()
        while pending and time.time() - t0 < 60:
            for si in range(2):
                for t in servers[si].poll():
                    ri = pending.pop((si, t))
                    s, n, pq, k = reqs[si][ri]
                    got[si][ri] = servers[si].result(t, n, k)
        assert not pending, "requests not completed"
        for si in range(2):
            for ri in range(len(reqs[si])):
                assert np.array_equal(got[si][ri], alone[si][ri]), (si, ri)
    finally:
        for s in servers:
            s.close()
        for ix in indexes:
            ix.free()


@pytest.mark.parametrize("two_level", [False, True])
def test_server_with_entry_points_equals_search(song, two_level):
    """With entry points on the index, the server's warps choose each query's
    starts themselves; the ids must equal song_search's (whose starts come
    from the pre-pass kernels) on the same index, and the entries stay fixed
    while the server exists."""
    import time
    from song_gb300.serve import Server
    rng = np.random.default_rng(1)
    g = load_golden("l2_s5_d32" if two_level else "cos_s5_d26")
    ix = song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"]))
    ent = rng.choice(g["data"].shape[0], 256, replace=False).astype(np.uint64)
    if two_level:
        ix.set_entries(ent, starts=3, coarse=16, probes=4)
    else:
        ix.set_entries(ent, starts=3)
    reqs = _requests(rng, 30, g["queries"].shape[0], (10, 50, 100), (1, 10))
    alone = [ix.search(g["queries"][s:s + n], pq, k) for (s, n, pq, k) in reqs]
    srv = Server(ix, max_pq=100, max_k=10, slots=4, slot_queries=64, sm_fraction=0.5)
    try:
        with pytest.raises(song.SongError):  # the server holds the entries
            ix.set_entries(None)
        with pytest.raises(song.SongError):  # pq below the number of starts
            srv.submit(g["queries"][:1], 2, 1)
        pending = {srv.submit(g["queries"][s:s + n], pq, k): ri for ri, (s, n, pq, k) in enumerate(reqs)}
        got = [None] * len(reqs)
        t0 = time.time()
        while pending and time.time() - t0 < 60:
            for t in srv.poll():
                ri = pending.pop(t)
                s, n, pq, k = reqs[ri]
                got[ri] = srv.result(t, n, k)
        assert not pending, "requests not completed"
        for ri in range(len(reqs)):
            assert np.array_equal(got[ri], alone[ri]), ri
    finally:
        srv.close()
    ix.set_entries(None)  # released with the server
    ix.free()


def test_poisson_stream_results_and_latency(song, capsys):
    from song_gb300 import datasets as D
    from song_gb300.serve import Server, poisson_stream
    w = D.SMALL
    data = D.base_vectors(w)
    q = D.query_vectors(w, nq=4000)
    graph = song.graph_build(data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150, batch_div=16)
    with song.Index(graph, data, w.shift, w.metric) as ix:
        with Server(ix, max_pq=400, max_k=100, slots=64, slot_queries=256) as srv:
            records, summary = poisson_stream([(srv, q)], rate_qps=20000, duration_s=1.5, keep_results=True, seed=4)
        for r in records[:40]:
            exp = ix.search(q[r["start"]:r["start"] + r["size"]], r["pq"], r["k"])
            assert np.array_equal(r["ids"], exp)
    with capsys.disabled():
        print("\n[serve] %s" % summary)
    assert summary["requests"] > 10 and summary["p99_ms"] > 0
