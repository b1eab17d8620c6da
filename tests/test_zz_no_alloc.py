"""song_search_noalloc, the host-buffer search that allocates no device memory.

Some callers cannot let a library call cudaMalloc: a service that has given
its whole GPU to its own memory pool, or a request path that must not pay for
an allocation that may synchronise the device.  This entry point keeps all of
its scratch (device copies of queries and ids, the kernel's work counter and
error flag) in one fixed device array per GPU.  The test checks, through the
C ABI, that two calls in a row return exactly what song_search returns, and
that a batch too large for the array is refused.  It is collected last so a
stop-at-first-failure run has already run every other test.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_noalloc_matches_song_search_twice(song):
    g = load_golden("l2_s5_d32")
    with song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"])) as ix:
        q1 = g["queries"]
        q2 = g["queries"][::-1][:17].copy()  # a second, smaller batch over the same scratch
        for q, pq, k in ((q1, 100, 100), (q2, 50, 10)):
            expected = ix.search(q, pq, k)
            got = ix.search_noalloc(q, pq, k)
            assert np.array_equal(got, expected)


def test_noalloc_rejects_batches_beyond_its_scratch(song):
    g = load_golden("cos_s4_d16")
    with song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"])) as ix:
        nq = 80_000  # 80k x 16 x 4 + 80k x 100 x 8 bytes > 16 MiB
        q = np.resize(g["queries"], (nq, g["queries"].shape[1]))
        with pytest.raises(song.SongError) as e:
            ix.search_noalloc(q, 100, 100)
        assert e.value.status == song.SONG_ERR_ARG and "scratch" in str(e.value)


def test_noalloc_starts_at_vertex_0_whatever_the_entry_points(song):
    """Entry points set on the index are not used: the ids are song_search's
    with the entries cleared."""
    g = load_golden("l2_s5_d32")
    with song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"])) as ix:
        q = g["queries"]
        plain = ix.search(q, 50, 10)
        ix.set_entries(song.sample_entries(ix.n, 64, seed=3), starts=2)
        try:
            assert np.array_equal(ix.search_noalloc(q, 50, 10), plain)
            assert np.array_equal(ix.search_noalloc(q, 50, 10), plain)
        finally:
            ix.set_entries(None)
