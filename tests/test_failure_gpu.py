"""Failure paths, made without faulting the GPU: an allocation failure
injected on the host, a device wait that nothing completes (bounded, so the
kernel gives up and reports it), a request the test keeps from the device
(the host's bounded wait gives up), and the server's idle exit and relaunch.
After each, the library keeps working and returns the same ids as before."""
import time

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _index(song, name="l2_s5_d32"):
    g = load_golden(name)
    return g, song.Index(g["graph"], g["data"], int(g["shift"]), int(g["metric"]))


def test_injected_allocation_failure_returns_oom_and_frees(song):
    g = load_golden("l2_s5_d32")
    args = (g["graph"], g["data"], int(g["shift"]), int(g["metric"]))
    for n in (1, 2, 3):  # the rows, the adjacency, the counters
        song.debug_fail_alloc(n)
        with pytest.raises(song.SongError) as e:
            song.Index(*args)
        assert e.value.status == song.SONG_ERR_OOM
    song.debug_fail_alloc(0)
    with song.Index(*args) as ix:  # nothing left over: a normal index works
        assert np.array_equal(ix.search(g["queries"], 50, 10), ix.search(g["queries"], 50, 10))


def test_search_wait_that_cannot_complete_times_out(song):
    g, ix = _index(song)
    with ix:
        expected = ix.search(g["queries"], 50, 10)
        ix.debug_set_wait(wait_limit=2000, extra_tx=16)
        t = time.perf_counter()
        with pytest.raises(song.SongError) as e:
            ix.search(g["queries"], 50, 10)
        assert e.value.status == song.SONG_ERR_TIMEOUT
        assert time.perf_counter() - t < 10.0
        ix.debug_set_wait()  # defaults
        assert np.array_equal(ix.search(g["queries"], 50, 10), expected)


def test_server_wait_times_out_on_a_held_request_then_completes(song):
    from song_gb300.serve import Server
    g, ix = _index(song)
    with ix:
        q = np.ascontiguousarray(g["queries"][:16])
        expected = ix.search(q, 50, 10)
        with Server(ix, max_pq=100, max_k=10, slots=4, slot_queries=32, sm_fraction=0.25) as srv:
            srv.hold(True)
            t = srv.submit(q, 50, 10)
            with pytest.raises(song.SongError) as e:
                srv.wait(t, 50)
            assert e.value.status == song.SONG_ERR_TIMEOUT
            srv.hold(False)
            srv.wait(t, 10_000)
            assert np.array_equal(srv.result(t, 16, 10), expected)


def test_server_idle_exit_and_relaunch(song):
    from song_gb300.serve import Server
    g, ix = _index(song)
    with ix:
        q = np.ascontiguousarray(g["queries"][:8])
        expected = ix.search(q, 50, 10)
        with Server(ix, max_pq=100, max_k=10, slots=4, slot_queries=32, sm_fraction=0.25) as srv:
            srv.set_idle_polls(2000)  # about a millisecond idle, for the next launch
            t = srv.submit(q, 50, 10)
            srv.wait(t, 10_000)
            assert np.array_equal(srv.result(t, 8, 10), expected)
            # the kernel launched at creation still has the default (~1 s)
            # limit; wait for it and its successors to leave
            deadline = time.time() + 10
            while srv.running() and time.time() < deadline:
                time.sleep(0.01)
            assert not srv.running()
            t = srv.submit(q, 50, 10)  # relaunches
            srv.wait(t, 10_000)
            assert np.array_equal(srv.result(t, 8, 10), expected)
