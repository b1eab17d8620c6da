"""GPU parity of the search kernel with the reference's N_MULTIPROBE /
FINISH_CNT knobs (warp_astar_accelerator.h:29-30,178-232) and its
__ENABLE_MULTIPROBE_DOUBLE_CHECK switch (:307-310) set away from their
defaults, through the C ABI (song_index_set_multiprobe).

The kernel is compared with the oracle's LEX mode under the same knobs (ids,
hops and distance evaluations bit-exact), and with the reference-container
results of tests/golden/search_multiprobe.npz except at listed float ties."""
import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu

KNOBS = [(2, 1, 0), (4, 1, 0), (1, 2, 0), (3, 3, 0), (4, 2, 0), (2, 1, 1), (4, 1, 1), (1, 1, 1), (3, 2, 1)]


def _kw(probes, fc, dc):
    return dict(probes=int(probes), finish_cnt=int(fc), double_check=bool(dc))


def _index(song, g, **kw):
    return song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"]), **kw)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_multiprobe_matches_oracle_bit_exact(song, oracle, name):
    g = load_golden(name)
    ox = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
    with _index(song, g) as ix:
        for knob in KNOBS:
            ix.set_multiprobe(*knob)
            for pq in list(g["pqs"]) + [2, 7, 333]:
                pq = int(pq)
                ids, hops, evals = ix.search(g["queries"], pq, pq, stats=True)
                o_ids, o_hops, o_evals, _ = ox.kernel_search(g["queries"], pq, oracle.MODE_LEX, **_kw(*knob))
                assert np.array_equal(ids, o_ids), (knob, pq)
                assert np.array_equal(hops, o_hops), (knob, pq)
                assert np.array_equal(evals, o_evals), (knob, pq)
        # back to the reference's default search
        ix.set_multiprobe(1, 1, 0)
        ids = ix.search(g["queries"], 50, 50)
        assert np.array_equal(ids, ox.kernel_search(g["queries"], 50, oracle.MODE_LEX)[0])


def test_multiprobe_matches_reference_except_listed_ties(song, oracle, capsys):
    z = np.load(GOLDEN + "/search_multiprobe.npz")
    ties = []
    for name in ("cos_s4_d16", "l2_s5_d32"):
        g = load_golden(name)
        ox = oracle.OracleIndex(g["data"], g["graph"], int(g["shift"]), int(g["metric"]))
        with _index(song, g) as ix:
            for probes, fc, dc in z["knobs"]:
                kw = _kw(probes, fc, dc)
                ix.set_multiprobe(*kw.values())
                for pq in g["pqs"]:
                    pq = int(pq)
                    ids = ix.search(g["queries"], pq, pq)
                    ref = z["ids_%s_p%d_f%d_d%d_%d" % (name, probes, fc, dc, pq)]
                    for i in np.nonzero((ids != ref).any(axis=1))[0]:
                        _, la = ox.kernel_search_log(g["queries"][i], pq, oracle.MODE_REF, **kw)
                        _, lb = ox.kernel_search_log(g["queries"][i], pq, oracle.MODE_LEX, **kw)
                        cls, at = oracle.classify(la, lb)
                        assert cls == 1, "%s %s pq %d query %d: not a tie" % (name, kw, pq, i)
                        ties.append((name, tuple(kw.values()), pq, int(i)))
    with capsys.disabled():
        print("\n[multiprobe] %d query results differ from the reference, all at float ties" % len(ties))


def _random_case(song, n, dim, metric, shift, seed, nq=40):
    from song_gb300 import datasets as D
    data = D.mixture("unit", n, dim, 8, seed=seed, center_seed=seed + 50)
    q = D.mixture("unit", nq, dim, 8, seed=seed + 1, center_seed=seed + 50)
    fixed = (1 << shift) - 1
    graph = song.graph_build(data, metric, shift, max(1, fixed // 2), fixed, 150, batch_div=0, nthreads=1)
    return data, q, graph


@pytest.mark.parametrize("dim,metric,shift", [(3, 2, 4), (130, 0, 5), (960, 2, 5), (33, 1, 3)])
def test_multiprobe_dims_pq_and_entry_points(song, oracle, dim, metric, shift):
    """Wide rows (two-row staging), queues up to S = 16 and one-row staging at
    pq >= 512, and several start vertices."""
    data, q, graph = _random_case(song, 1500, dim, metric, shift, seed=dim + 7)
    ox = oracle.OracleIndex(data, graph, shift, metric)
    rng = np.random.default_rng(dim)
    entries = rng.choice(len(data), 64, replace=False).astype(np.uint64)
    with song.Index(graph, data, shift, metric) as ix:
        for knob in ((4, 1, 0), (2, 3, 0), (4, 1, 1)):
            ix.set_multiprobe(*knob)
            for pq in (16, 333, 600):
                ids, hops, evals = ix.search(q, pq, pq, stats=True)
                o_ids, o_hops, o_evals, _ = ox.kernel_search(q, pq, oracle.MODE_LEX, **_kw(*knob))
                assert np.array_equal(ids, o_ids), (knob, pq)
                assert np.array_equal(hops, o_hops)
                assert np.array_equal(evals, o_evals)
            ix.set_entries(entries, starts=3)
            starts = ox.nearest_entry(q, entries, ns=3)
            ids, hops, evals = ix.search(q, 64, 64, stats=True)
            o_ids, o_hops, o_evals, _ = ox.kernel_search_from(q, starts, 64, oracle.MODE_LEX, **_kw(*knob))
            assert np.array_equal(ids, o_ids)
            assert np.array_equal(evals, o_evals)
            ix.set_entries(None)


def test_multiprobe_duplicate_listing(song, oracle):
    """Edges repeated across and within rows: with several pops per iteration a
    vertex can be listed, evaluated and queued twice, as in the reference."""
    rng = np.random.default_rng(21)
    n, dim, shift = 80, 10, 3
    data = rng.standard_normal((n, dim)).astype(np.float32)
    graph = np.zeros((n, 8), np.uint64)
    for v in range(n):
        deg = int(rng.integers(0, 8))
        graph[v, 0] = deg
        graph[v, 1:1 + deg] = rng.integers(0, 12, deg)  # a small pool: many shared neighbours
    graph = graph.reshape(-1)
    q = rng.standard_normal((48, dim)).astype(np.float32)
    for metric in (0, 1, 2):
        ox = oracle.OracleIndex(data, graph, shift, metric)
        with song.Index(graph, data, shift, metric) as ix:
            for knob in KNOBS:
                ix.set_multiprobe(*knob)
                for pq in (2, 5, 40):
                    ids, hops, evals = ix.search(q, pq, pq, stats=True)
                    o_ids, o_hops, o_evals, _ = ox.kernel_search(q, pq, oracle.MODE_LEX, **_kw(*knob))
                    assert np.array_equal(ids, o_ids), (metric, knob, pq)
                    assert np.array_equal(hops, o_hops)
                    assert np.array_equal(evals, o_evals)


def test_multiprobe_argument_errors(song):
    g = load_golden("l2_s5_d32")
    with _index(song, g) as ix:
        for probes, fc in ((0, 1), (5, 1), (2, 0)):
            with pytest.raises(song.SongError):
                ix.set_multiprobe(probes, fc)
        ix.set_multiprobe(2, 1)
        with pytest.raises(song.SongError):
            ix.set_hop_limit(10)
        from song_gb300.serve import Server
        with pytest.raises(song.SongError):
            Server(ix, max_pq=64, max_k=10, slots=2, slot_queries=8)
        ix.set_multiprobe(1, 1, True)
        with pytest.raises(song.SongError):
            ix.set_hop_limit(10)
        ix.set_multiprobe(1, 1)
        ix.set_hop_limit(10)
        with pytest.raises(song.SongError):
            ix.set_multiprobe(2, 1)
    with _index(song, g, storage="bf16") as ix:
        with pytest.raises(song.SongError):
            ix.set_multiprobe(2, 1)
