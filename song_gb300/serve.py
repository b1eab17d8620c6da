"""Python view of the continuous-batching server (song_server_* in
include/song_gb300.h) and a Poisson request-stream driver that reports
latency percentiles and throughput.  No counterpart in the reference."""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import Index, _check, _ptr, load_library


class Server:
    def __init__(self, index: Index, max_pq=400, max_k=100, slots=64, slot_queries=256, sm_fraction=1.0):
        self.index = index
        self.max_k = max_k
        self._h = ctypes.c_void_p()
        _check(load_library().song_server_create(index._h, max_pq, max_k, slots, slot_queries, float(sm_fraction),
                                                 ctypes.byref(self._h)))

    def submit(self, queries, pq, k):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        t = ctypes.c_uint64()
        _check(load_library().song_server_submit(self._h, _ptr(q), q.shape[0], pq, k, ctypes.byref(t)))
        return t.value

    def poll(self, max_n=1024):
        buf = np.empty(max_n, dtype=np.uint64)
        n = ctypes.c_int()
        _check(load_library().song_server_poll(self._h, _ptr(buf), max_n, ctypes.byref(n)))
        return buf[:n.value].tolist()

    def result(self, ticket, nq, k):
        out = np.empty((nq, k), dtype=np.uint64)
        a, b = ctypes.c_int(), ctypes.c_int()
        _check(load_library().song_server_result(self._h, ticket, _ptr(out), ctypes.byref(a), ctypes.byref(b)))
        assert a.value == nq and b.value == k
        return out

    def set_idle_polls(self, polls):
        """Warps leave after `polls` idle polls (~0.5 us each); the next
        submission relaunches them."""
        _check(load_library().song_server_set_idle_polls(self._h, int(polls)))

    def running(self):
        r = ctypes.c_int()
        _check(load_library().song_server_running(self._h, ctypes.byref(r)))
        return bool(r.value)

    def wait(self, ticket, timeout_ms):
        """Waits for a request (SongError with status SONG_ERR_TIMEOUT if it
        has not completed within timeout_ms)."""
        _check(load_library().song_server_wait(self._h, ctypes.c_uint64(ticket), int(timeout_ms)))

    def hold(self, on=True):
        """Test hook: keep admitted requests from the kernel until released."""
        _check(load_library().song_debug_server_hold(self._h, int(bool(on))))

    def close(self):
        if self._h and self._h.value:
            load_library().song_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_stream(servers, rate_qps, duration_s, k_choices=(1, 10, 100), pq_choices=(50, 100, 200, 400),
                   max_request=256, seed=4, keep_results=False, warmup_s=0.0):
    """Drives `servers` (list of (Server, queries array)) with a Poisson stream
    of requests whose mean query rate is rate_qps: each request picks a server
    uniformly, a size log-uniform in [1, max_request], k and pq uniformly from
    the choices (pq >= k).  Returns per-request records and a summary."""
    rng = np.random.default_rng(seed)
    mean_size = (max_request - 1) / np.log(max_request)  # mean of a log-uniform on [1, max]
    req_rate = rate_qps / mean_size
    t0 = time.perf_counter()
    t_next = t0
    outstanding = {}
    records = []
    issued = 0
    while True:
        now = time.perf_counter()
        if now - t0 < duration_s and now >= t_next:
            si = int(rng.integers(len(servers)))
            srv, qset = servers[si]
            size = int(np.clip(np.exp(rng.uniform(0.0, np.log(max_request))), 1, max_request))
            k = int(rng.choice(k_choices))
            pq = int(max(k, rng.choice(pq_choices)))
            start = int(rng.integers(0, qset.shape[0] - size + 1))
            q = qset[start:start + size]
            t_sub = time.perf_counter()
            ticket = srv.submit(q, pq, k)
            outstanding[(si, ticket)] = (t_sub, size, pq, k, start)
            issued += 1
            t_next += rng.exponential(1.0 / req_rate)
        for si, (srv, _) in enumerate(servers):
            for ticket in srv.poll():
                t_sub, size, pq, k, start = outstanding.pop((si, ticket))
                ids = srv.result(ticket, size, k)
                rec = {"server": si, "size": size, "pq": pq, "k": k, "start": start,
                       "latency_ms": (time.perf_counter() - t_sub) * 1000.0, "t_submit": t_sub - t0}
                if keep_results:
                    rec["ids"] = ids
                records.append(rec)
        if time.perf_counter() - t0 >= duration_s and not outstanding:
            break
        if not outstanding and time.perf_counter() < t_next:
            time.sleep(min(50e-6, max(0.0, t_next - time.perf_counter())))
    wall = time.perf_counter() - t0
    lat = np.array([r["latency_ms"] for r in records if r["t_submit"] >= warmup_s]) if records else np.zeros(1)
    nqs = sum(r["size"] for r in records)
    summary = {"requests": len(records), "queries": nqs, "wall_s": round(wall, 3),
               "throughput_qps": round(nqs / wall, 1), "offered_qps": rate_qps,
               "p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
               "mean_ms": round(float(lat.mean()), 3)}
    return records, summary
