"""Entry points (song_index_set_entries): every query starts from its
nearest entry vertices (one or several) instead of vertex 0.  The entry
choice and the search from it must equal the oracle's (orc_nearest_entry +
orc_kernel_search_from) bit for bit, for F32 and BF16 storage and for the
learned kernel with its exit off; clearing the entries restores the
reference's start at vertex 0."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu


def _entries(n, count, seed):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, count, replace=False)).astype(np.uint64)


@pytest.mark.parametrize("ns", [1, 3, 8])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_search_from_nearest_entries_matches_oracle(song, oracle, name, ns):
    g = load_golden(name)
    shift, metric = int(g["shift"]), int(g["metric"])
    ox = oracle.OracleIndex(g["data"], g["graph"], shift, metric)
    ent = _entries(g["data"].shape[0], 64, 5)
    starts = ox.nearest_entry(g["queries"], ent, ns=ns)
    assert len(set(np.asarray(starts).reshape(len(starts), -1)[:, 0].tolist())) > 1
    with song.Index(g["graph"], g["data"], shift, metric) as ix:
        ix.set_entries(ent, starts=ns)
        for pq in (10, 50, 100):
            ids, hops, evals = ix.search(g["queries"], pq, pq, stats=True)
            o_ids, o_hops, o_evals, _ = ox.kernel_search_from(g["queries"], starts, pq, oracle.MODE_LEX)
            assert np.array_equal(ids, o_ids), (name, pq)
            assert np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)
        ix.set_entries(None)
        ids = ix.search(g["queries"], 50, 50)
        o_ids, _, _, _ = ox.kernel_search(g["queries"], 50, oracle.MODE_LEX)
        assert np.array_equal(ids, o_ids)


@pytest.mark.parametrize("storage", ["bf16"])
def test_entries_with_low_precision_rows(song, oracle, storage):
    g = load_golden("cos_s5_d26")
    shift, metric = int(g["shift"]), int(g["metric"])
    ent = _entries(g["data"].shape[0], 100, 6)
    starts = oracle.OracleIndex(g["data"], g["graph"], shift, metric).nearest_entry(g["queries"], ent, ns=4)
    with song.Index(g["graph"], g["data"], shift, metric, storage=storage) as ix:
        ix.set_rerank(0)
        ix.set_entries(ent, starts=4)
        deq = song.dequantize_rows(ix.rows(), storage, g["data"].shape[1])
        ox = oracle.OracleIndex(deq, g["graph"], shift, metric)
        ids, hops, evals = ix.search(g["queries"], 60, 60, stats=True)
        o_ids, o_hops, o_evals, _ = ox.kernel_search_from(g["queries"], starts, 60, oracle.MODE_LEX)
        assert np.array_equal(ids, o_ids) and np.array_equal(hops, o_hops)


def test_learned_kernel_from_entries_matches_exact_visited_oracle(song, oracle):
    import torch
    from song_gb300 import learned as LE
    g = load_golden("l2_s5_d32")
    shift, metric = int(g["shift"]), int(g["metric"])
    ox = oracle.OracleIndex(g["data"], g["graph"], shift, metric)
    ent = _entries(g["data"].shape[0], 50, 7)
    starts = ox.nearest_entry(g["queries"], ent, ns=2)
    with song.Index(g["graph"], g["data"], shift, metric) as ix:
        ix.set_entries(ent, starts=2)
        dq = torch.from_numpy(g["queries"]).cuda()
        ids, hops, evals = LE.evaluate(ix, dq, 100, 100, max_hops=1 << 30)
    o_ids, o_hops, o_evals, _ = ox.kernel_search_from(g["queries"], starts, 100, oracle.MODE_LEX_EXACT)
    assert np.array_equal(ids, o_ids) and np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)


def test_entry_arguments_are_checked(song):
    g = load_golden("ip_s5_d24")
    n = g["data"].shape[0]
    with song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"])) as ix:
        with pytest.raises(song.SongError):
            ix.set_entries(np.array([0, n], dtype=np.uint64))
        with pytest.raises(song.SongError):
            ix.set_entries(np.zeros(song.SONG_MAX_ENTRIES + 1, dtype=np.uint64))
        with pytest.raises(song.SongError):  # more starts than entries
            ix.set_entries(np.array([1, 2], dtype=np.uint64), starts=3)
        with pytest.raises(song.SongError):
            ix.set_entries(np.arange(20, dtype=np.uint64), starts=song.SONG_MAX_STARTS + 1)
        ix.set_entries(np.arange(20, dtype=np.uint64), starts=8)
        with pytest.raises(song.SongError):  # starts > pq
            ix.search(g["queries"][:3], 5, 5)
        ix.set_entries(np.array([n - 1], dtype=np.uint64))  # a single entry is allowed
        assert ix.search(g["queries"][:3], 20, 5).shape == (3, 5)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_two_level_entries_match_oracle(song, oracle, name):
    """Two-level choice (song_index_set_entries_2level): the first `coarse`
    entries are clusters, the rest join their nearest; each query searches
    its `probes` nearest clusters.  Same starts and same search as the
    oracle's orc_nearest_entry_2level + orc_kernel_search_from."""
    g = load_golden(name)
    shift, metric = int(g["shift"]), int(g["metric"])
    ox = oracle.OracleIndex(g["data"], g["graph"], shift, metric)
    rng = np.random.default_rng(9)
    ent = rng.choice(g["data"].shape[0], 300, replace=False).astype(np.uint64)  # unsorted on purpose
    for coarse, probes, ns in ((20, 4, 3), (7, 2, 2), (1, 1, 1)):
        starts = ox.nearest_entry_2level(g["queries"], ent, coarse, probes, ns)
        with song.Index(g["graph"], g["data"], shift, metric) as ix:
            ix.set_entries(ent, starts=ns, coarse=coarse, probes=probes)
            ids, hops, evals = ix.search(g["queries"], 60, 60, stats=True)
        o_ids, o_hops, o_evals, _ = ox.kernel_search_from(g["queries"], starts, 60, oracle.MODE_LEX)
        assert np.array_equal(ids, o_ids), (name, coarse, probes, ns)
        assert np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)


@pytest.mark.parametrize("dim,metric", [(200, 0), (200, 1), (200, 2), (130, 0), (400, 0), (960, 2)])
def test_two_level_wide_rows_match_oracle(song, oracle, dim, metric):
    """Rows wider than 128 floats: each lane sums several 32-float groups per
    row (one partial group at 130); from 200 floats on the blocks stage one
    row tile at a time, and at 400 and 960 floats they shrink to fewer warps
    and 8-row tiles to fit shared memory.  Clusters of ~75 rows take several
    tiles."""
    from song_gb300 import datasets as D
    shift = 5
    data = D.mixture("unit", 700, dim, 8, seed=dim + metric, center_seed=dim + 50)
    q = D.mixture("unit", 40, dim, 8, seed=dim + metric + 1, center_seed=dim + 50)
    graph = song.graph_build(data, metric, shift, 15, 31, 150, batch_div=0, nthreads=1)
    ox = oracle.OracleIndex(data, graph, shift, metric)
    rng = np.random.default_rng(dim)
    ent = rng.choice(700, 300, replace=False).astype(np.uint64)
    for coarse, probes, ns in ((20, 4, 3), (4, 2, 2)):
        starts = ox.nearest_entry_2level(q, ent, coarse, probes, ns)
        with song.Index(graph, data, shift, metric) as ix:
            ix.set_entries(ent, starts=ns, coarse=coarse, probes=probes)
            ids, hops, evals = ix.search(q, 40, 40, stats=True)
        o_ids, o_hops, o_evals, _ = ox.kernel_search_from(q, starts, 40, oracle.MODE_LEX)
        assert np.array_equal(ids, o_ids), (dim, metric, coarse, probes, ns)
        assert np.array_equal(hops, o_hops) and np.array_equal(evals, o_evals)


def test_two_level_arguments_are_checked(song):
    g = load_golden("l2_s5_d32")
    with song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"])) as ix:
        ent = np.arange(40, dtype=np.uint64)
        rc = song.load_library().song_index_set_entries_2level(ix._h, ent.ctypes.data, 40, 0, 1, 1)
        assert rc == song.SONG_ERR_ARG  # no coarse entries
        for bad in (dict(coarse=41, probes=1), dict(coarse=4, probes=5),
                    dict(coarse=8, probes=2, starts=3)):
            kw = dict(starts=1)
            kw.update(bad)
            with pytest.raises(song.SongError):
                ix.set_entries(ent, **kw)
        with pytest.raises(song.SongError):  # duplicate ids
            ix.set_entries(np.array([3, 4, 3], dtype=np.uint64), starts=1, coarse=2, probes=1)
        with pytest.raises(song.SongError):
            ix.set_entries(np.array([3, 4, 3], dtype=np.uint64), starts=1)
        ix.set_entries(ent, starts=2, coarse=8, probes=2)
        assert ix.search(g["queries"][:4], 20, 5).shape == (4, 5)
        ix.set_entries(None)
