"""song_gb300: batched best-first graph search on GB300 (sm_103a).

Python view of the C ABI in include/song_gb300.h (libsong_gb300.so, built
in-tree by song_gb300/build.py).  The search runs only in the CUDA kernels of
that library; there is no CPU path, and importing this package fails if the
library has not been built.

Reference surface mirrored here (sunbelbd/song):
  * Index.search          <- GraphWrapper::search_top_k_batch (kernelgraph.h:269-272)
  * astar_search_batch    <- WarpAStarAccelerator::astar_multi_start_search_batch
                             (warp_astar_accelerator.h:347-423)
  * graph_build           <- FixedDegreeGraph::add_vertex loop (graph.h:149-167, main.cu:15-18)
  * read/write bfsg files <- Data::dump/load, *Graph::dump/load (data.h:164-175, kernelgraph.h:255-267)

Additions without a reference counterpart: graph_build_gpu (the builder's
searches on the GPU, same graph), Index.set_entries (queries start from their
nearest entry vertices instead of vertex 0; flat or two-level choice), BF16 /
FP8 storage with FP32 rerank, the learned early exit (learned.py), the
continuous-batching server (serve.py) and search_noalloc.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB_PATH

SONG_OK, SONG_ERR_ARG, SONG_ERR_OOM, SONG_ERR_TIMEOUT, SONG_ERR_CUDA, SONG_ERR_IO = range(6)
SONG_MAX_ENTRIES = 65536  # include/song_gb300.h
SONG_MAX_STARTS = 8
SONG_MAX_ENTRIES_2LEVEL = 1 << 20
SONG_MAX_COARSE = 16384
METRICS = {"l2": 0, "ip": 1, "cos": 2}
STORAGES = {"f32": 0, "bf16": 1, "fp8": 2, "bits": 3}
HASH_BITS = 256
MAX_PQ = 1023
NO_ID = np.uint64(0xFFFFFFFFFFFFFFFF)

# Every function include/song_gb300.h declares; tests check the library exports them.
EXPORTED = [
    "song_status_string", "song_last_error", "song_index_create", "song_index_load",
    "song_index_free", "song_index_info", "song_search", "song_search_device",
    "song_astar_search_batch", "song_graph_build", "song_graph_build_gpu", "song_index_set_entries", "song_index_set_entries_2level", "song_debug_fixhash", "song_search_noalloc",
    "song_index_set_rerank", "song_index_rows", "song_index_set_early_exit", "song_search_trace_device",
    "song_index_set_hop_limit", "song_index_set_multiprobe", "song_index_set_timing", "song_index_timing", "song_mlp_train_device", "song_mlp_grad", "song_mlp_forward",
    "song_server_create", "song_server_submit", "song_server_poll", "song_server_result", "song_server_destroy",
    "song_index_set_hash_planes",
    "song_server_set_idle_polls", "song_server_running", "song_server_wait", "song_debug_fail_alloc",
    "song_debug_set_wait", "song_debug_server_hold", "song_debug_head_path", "song_debug_head_stats",
    "song_debug_head_scores",
]
MLP_PARAMS = 1281
TRACE_FIELDS = 6


class SongError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s (status %d): %s" % (_STATUS.get(status, "error"), status, message))
        self.status = status


_STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "device wait timed out",
           4: "CUDA error", 5: "I/O error"}

_lib = None


def load_library():
    """Load libsong_gb300.so; raises if it was not built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("libsong_gb300.so not built: run `python -c \"import __graft_entry__ as g; "
                          "g.build()\"` or `python song_gb300/build.py`")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    i32 = ctypes.c_int
    u64 = ctypes.c_uint64
    L.song_status_string.restype = ctypes.c_char_p
    L.song_status_string.argtypes = [i32]
    L.song_last_error.restype = ctypes.c_char_p
    L.song_last_error.argtypes = []
    L.song_index_create.restype = i32
    L.song_index_create.argtypes = [P, P, u64, i32, i32, i32, i32, i32, ctypes.POINTER(P)]
    L.song_index_load.restype = i32
    L.song_index_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, u64, i32, i32, i32, i32, i32,
                                  ctypes.POINTER(P)]
    L.song_index_free.restype = i32
    L.song_index_free.argtypes = [P]
    L.song_index_info.restype = i32
    L.song_index_info.argtypes = [P, P, P, P, P, P, P]
    L.song_search.restype = i32
    L.song_search.argtypes = [P, P, i32, i32, i32, P, P, P]
    L.song_search_device.restype = i32
    L.song_search_device.argtypes = [P, P, i32, i32, i32, P, P, P, P]
    L.song_astar_search_batch.restype = i32
    L.song_astar_search_batch.argtypes = [P, i32, i32, P, P, P, i32, u64, i32, i32]
    L.song_graph_build.restype = i32
    L.song_graph_build.argtypes = [P, u64, i32, i32, i32, i32, i32, i32, i32, i32, P]
    L.song_index_set_entries.restype = i32
    L.song_index_set_entries.argtypes = [P, P, i32, i32]
    L.song_index_set_entries_2level.restype = i32
    L.song_index_set_entries_2level.argtypes = [P, P, i32, i32, i32, i32]
    L.song_graph_build_gpu.restype = i32
    L.song_graph_build_gpu.argtypes = [P, u64, i32, i32, i32, i32, i32, i32, i32, i32, i32, P]
    L.song_index_set_rerank.restype = i32
    L.song_index_set_rerank.argtypes = [P, i32]
    L.song_index_rows.restype = i32
    L.song_index_rows.argtypes = [P, u64, u64, P, ctypes.c_size_t, ctypes.POINTER(i32)]
    L.song_index_set_early_exit.restype = i32
    L.song_index_set_early_exit.argtypes = [P, P, ctypes.c_float, i32, i32]
    L.song_search_trace_device.restype = i32
    L.song_search_trace_device.argtypes = [P, P, i32, i32, i32, i32, P, P, P, P, P, P]
    L.song_index_set_hop_limit.restype = i32
    L.song_index_set_hop_limit.argtypes = [P, i32]
    L.song_debug_head_path.restype = i32
    L.song_debug_head_path.argtypes = [P, i32, ctypes.POINTER(i32)]
    L.song_debug_head_stats.restype = i32
    L.song_debug_head_stats.argtypes = [P, i32, P]
    L.song_debug_head_scores.restype = i32
    L.song_debug_head_scores.argtypes = [P, P, i32, P, i32]
    L.song_index_set_multiprobe.restype = i32
    L.song_index_set_multiprobe.argtypes = [P, i32, i32, i32]
    L.song_index_set_timing.restype = i32
    L.song_index_set_timing.argtypes = [P, i32]
    L.song_index_timing.restype = i32
    L.song_index_timing.argtypes = [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    L.song_mlp_train_device.restype = i32
    L.song_mlp_train_device.argtypes = [P, P, P, ctypes.c_int64, P, i32, i32, ctypes.c_float, P, P, P]
    L.song_mlp_grad.restype = i32
    L.song_mlp_grad.argtypes = [P, P, P, i32, P, P, P]
    L.song_mlp_forward.restype = i32
    L.song_mlp_forward.argtypes = [P, i32, P, P]
    L.song_server_create.restype = i32
    L.song_server_create.argtypes = [P, i32, i32, i32, i32, ctypes.c_float, ctypes.POINTER(P)]
    L.song_server_submit.restype = i32
    L.song_server_submit.argtypes = [P, P, i32, i32, i32, ctypes.POINTER(ctypes.c_uint64)]
    L.song_server_poll.restype = i32
    L.song_server_poll.argtypes = [P, P, i32, ctypes.POINTER(i32)]
    L.song_server_result.restype = i32
    L.song_server_result.argtypes = [P, ctypes.c_uint64, P, ctypes.POINTER(i32), ctypes.POINTER(i32)]
    L.song_server_destroy.restype = i32
    L.song_server_destroy.argtypes = [P]
    L.song_index_set_hash_planes.restype = i32
    L.song_index_set_hash_planes.argtypes = [P, P]
    L.song_server_set_idle_polls.restype = i32
    L.song_server_set_idle_polls.argtypes = [P, ctypes.c_uint32]
    L.song_server_running.restype = i32
    L.song_server_running.argtypes = [P, ctypes.POINTER(i32)]
    L.song_server_wait.restype = i32
    L.song_server_wait.argtypes = [P, ctypes.c_uint64, i32]
    L.song_debug_fail_alloc.restype = i32
    L.song_debug_fail_alloc.argtypes = [i32]
    L.song_debug_set_wait.restype = i32
    L.song_debug_set_wait.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32]
    L.song_debug_server_hold.restype = i32
    L.song_debug_server_hold.argtypes = [P, i32]
    L.song_search_noalloc.restype = i32
    L.song_search_noalloc.argtypes = [P, P, i32, i32, i32, P]
    L.song_debug_fixhash.restype = i32
    L.song_debug_fixhash.argtypes = [P, i32, i32, P]
    _lib = L
    return L


def _check(rc):
    if rc != SONG_OK:
        msg = load_library().song_last_error().decode(errors="replace")
        raise SongError(rc, msg)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _metric(m):
    return METRICS[m] if isinstance(m, str) else int(m)


def _storage(s):
    return STORAGES[s] if isinstance(s, str) else int(s)


class Index:
    """A resident index on one GPU (song_index_create / song_index_load)."""

    def __init__(self, graph, data, shift, metric, storage="f32", device=0, _handle=None):
        L = load_library()
        self._h = ctypes.c_void_p()
        if _handle is not None:
            self._h = _handle
        else:
            data = np.ascontiguousarray(data, dtype=np.float32)
            graph = np.ascontiguousarray(graph, dtype=np.uint64).reshape(-1)
            n, dim = data.shape
            if graph.size != (n << shift):
                raise ValueError("graph has %d slots, expected n << shift = %d" % (graph.size, n << shift))
            _check(L.song_index_create(_ptr(graph), _ptr(data), n, dim, shift, _metric(metric),
                                       _storage(storage), device, ctypes.byref(self._h)))
        n = ctypes.c_uint64()
        dim, sh, me, st = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        nb = ctypes.c_uint64()
        _check(L.song_index_info(self._h, ctypes.byref(n), ctypes.byref(dim), ctypes.byref(sh),
                                 ctypes.byref(me), ctypes.byref(st), ctypes.byref(nb)))
        self.n, self.dim, self.shift, self.metric, self.storage = n.value, dim.value, sh.value, me.value, st.value
        self.device = device

    @classmethod
    def load(cls, graph_path, data_path, n, dim, shift, metric, storage="f32", device=0):
        L = load_library()
        h = ctypes.c_void_p()
        _check(L.song_index_load(graph_path.encode(), data_path.encode(), n, dim, shift,
                                 _metric(metric), _storage(storage), device, ctypes.byref(h)))
        return cls(None, None, shift, metric, storage, device, _handle=h)

    def device_bytes(self):
        nb = ctypes.c_uint64()
        _check(load_library().song_index_info(self._h, None, None, None, None, None, ctypes.byref(nb)))
        return nb.value

    def search(self, queries, pq, k=None, stats=False):
        """Host-buffer search (song_search): returns nq x k uint64 ids, and
        per-query hops and distance evaluations when stats=True."""
        k = pq if k is None else k
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if q.ndim != 2 or q.shape[1] != self.dim:
            raise ValueError("queries must be nq x %d" % self.dim)
        nq = q.shape[0]
        out = np.empty((nq, k), dtype=np.uint64)
        hops = np.empty(nq, dtype=np.int32) if stats else None
        evals = np.empty(nq, dtype=np.int32) if stats else None
        _check(load_library().song_search(self._h, _ptr(q), nq, pq, k, _ptr(out), _ptr(hops), _ptr(evals)))
        return (out, hops, evals) if stats else out

    def set_rerank(self, rerank):
        """BF16/FP8 storage: FP32 re-rank of the best `rerank` final candidates
        (-1 = all pq, 0 = none)."""
        _check(load_library().song_index_set_rerank(self._h, int(rerank)))

    def rows(self, first=0, count=None):
        """Stored rows as raw bytes (count x row_bytes uint8)."""
        L = load_library()
        rb = ctypes.c_int()
        _check(L.song_index_rows(self._h, 0, 0, None, 0, ctypes.byref(rb)))
        count = self.n - first if count is None else count
        out = np.empty((count, rb.value), dtype=np.uint8)
        _check(L.song_index_rows(self._h, first, count, _ptr(out), out.nbytes, ctypes.byref(rb)))
        return out

    def set_early_exit(self, weights, threshold=0.0, min_hops=8, every=1):
        """Attach the early-exit network (MLP_PARAMS FP32 weights) or detach it (None)."""
        w = None if weights is None else np.ascontiguousarray(weights, dtype=np.float32)
        if w is not None and w.size != MLP_PARAMS:
            raise ValueError("expected %d weights" % MLP_PARAMS)
        _check(load_library().song_index_set_early_exit(self._h, _ptr(w), float(threshold), int(min_hops), int(every)))

    def set_entries(self, ids, starts=1, coarse=0, probes=0):
        """Entry points: each query starts from the `starts` nearest of these
        vertices (None or empty: vertex 0, the reference's start).  coarse >
        0: two-level choice, ids[:coarse] are the coarse entries and each
        query searches only its `probes` nearest coarse entries' clusters."""
        e = None if ids is None else np.ascontiguousarray(ids, dtype=np.uint64)
        L = load_library()
        if coarse > 0:
            _check(L.song_index_set_entries_2level(self._h, _ptr(e), int(e.size), int(coarse), int(probes),
                                                   int(starts)))
            return
        _check(L.song_index_set_entries(self._h, _ptr(e) if e is not None and e.size else None,
                                        0 if e is None else int(e.size), int(starts)))

    def set_timing(self, enable=True):
        """Record CUDA events around the entry choice and the search kernel of
        every later search (song_index_set_timing)."""
        _check(load_library().song_index_set_timing(self._h, int(bool(enable))))

    def timing(self):
        """(entry-choice ms, search-kernel ms) of the last search."""
        a, b = ctypes.c_float(), ctypes.c_float()
        _check(load_library().song_index_timing(self._h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def set_hop_limit(self, max_hops):
        """Fixed hop budget (0 = off), the heuristic the learned exit is compared with."""
        _check(load_library().song_index_set_hop_limit(self._h, int(max_hops)))

    def debug_head_path(self, use_tensor_cores=True):
        """Head phase of the two-level entry choice: tensor-core shortlist
        (default) or the exact CUDA-core scan; returns whether the tensor
        path is prepared for this index."""
        prepared = ctypes.c_int(0)
        _check(load_library().song_debug_head_path(self._h, int(bool(use_tensor_cores)), ctypes.byref(prepared)))
        return bool(prepared.value)

    def debug_head_stats(self, enable=True):
        """Counts since the previous call: (queries, coarse entries re-scored
        exactly, shortlist overflows); enable keeps counting."""
        st = np.zeros(3, dtype=np.uint64)
        _check(load_library().song_debug_head_stats(self._h, int(bool(enable)), st.ctypes.data_as(ctypes.c_void_p)))
        return tuple(int(x) for x in st)

    def debug_head_scores(self, q_ptr, nq, scores_ptr, ld):
        """Tensor-core approximate dot products of nq device queries with the
        coarse entries into a device buffer (nq x ld floats)."""
        _check(load_library().song_debug_head_scores(self._h, ctypes.c_void_p(q_ptr), int(nq),
                                                     ctypes.c_void_p(scores_ptr), int(ld)))

    def set_multiprobe(self, probes=1, finish_cnt=1, double_check=False):
        """The reference kernel's N_MULTIPROBE / FINISH_CNT knobs
        (warp_astar_accelerator.h:29-30) and __ENABLE_MULTIPROBE_DOUBLE_CHECK
        switch (:307-310) as run-time values; (1, 1, False) is the
        reference's default search."""
        _check(load_library().song_index_set_multiprobe(self._h, int(probes), int(finish_cnt),
                                                        int(bool(double_check))))

    def trace_device(self, q_ptr, nq, pq, k, trace_hops, trace_ptr, final_ptr, out_ptr,
                     hops_ptr=None, evals_ptr=None, stream=None):
        """Plain search with per-hop feature tracing (device pointers)."""
        _check(load_library().song_search_trace_device(
            self._h, ctypes.c_void_p(q_ptr), nq, pq, k, trace_hops, ctypes.c_void_p(trace_ptr),
            ctypes.c_void_p(final_ptr), ctypes.c_void_p(out_ptr),
            ctypes.c_void_p(hops_ptr) if hops_ptr else None,
            ctypes.c_void_p(evals_ptr) if evals_ptr else None,
            ctypes.c_void_p(stream) if stream else None))

    def search_noalloc(self, queries, pq, k=None):
        """song_search_noalloc: the host-buffer search that allocates no device
        memory (scratch in a fixed 16 MiB device array per GPU)."""
        k = pq if k is None else k
        q = np.ascontiguousarray(queries, dtype=np.float32)
        out = np.empty((q.shape[0], k), dtype=np.uint64)
        _check(load_library().song_search_noalloc(self._h, _ptr(q), q.shape[0], pq, k, _ptr(out)))
        return out

    def search_device(self, q_ptr, nq, pq, k, out_ptr, hops_ptr=None, evals_ptr=None, stream=None):
        """Device-buffer search (song_search_device): raw device pointers
        (e.g. torch.Tensor.data_ptr()), enqueued on `stream` (a raw
        cudaStream_t handle or None)."""
        _check(load_library().song_search_device(self._h, ctypes.c_void_p(q_ptr), nq, pq, k,
                                                 ctypes.c_void_p(out_ptr),
                                                 ctypes.c_void_p(hops_ptr) if hops_ptr else None,
                                                 ctypes.c_void_p(evals_ptr) if evals_ptr else None,
                                                 ctypes.c_void_p(stream) if stream else None))

    def set_hash_planes(self, planes):
        """SONG_STORAGE_BITS: the HASH_BITS x dim hyperplanes of the 256-bit
        sign codes; codes every base vector (song_index_set_hash_planes)."""
        h = np.ascontiguousarray(planes, dtype=np.float32)
        if h.shape != (HASH_BITS, self.dim):
            raise ValueError("planes must be %d x %d" % (HASH_BITS, self.dim))
        _check(load_library().song_index_set_hash_planes(self._h, _ptr(h)))

    def debug_set_wait(self, wait_limit=1 << 24, extra_tx=0):
        """Test hook (song_debug_set_wait): the kernel's bounded waits give up
        after wait_limit polls; extra_tx bytes that no copy delivers make a
        wait that cannot complete."""
        _check(load_library().song_debug_set_wait(self._h, int(wait_limit), int(extra_tx)))

    def free(self):
        if getattr(self, "_h", None) and self._h.value:
            load_library().song_index_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.free()


def astar_search_batch(queries, pq, data, graph, shift, metric):
    """One-shot drop-in for astar_multi_start_search_batch: nq x pq ids."""
    q = np.ascontiguousarray(queries, dtype=np.float32)
    data = np.ascontiguousarray(data, dtype=np.float32)
    graph = np.ascontiguousarray(graph, dtype=np.uint64)
    n, dim = data.shape
    out = np.empty((q.shape[0], pq), dtype=np.uint64)
    _check(load_library().song_astar_search_batch(_ptr(q), q.shape[0], pq, _ptr(out), _ptr(data),
                                                  _ptr(graph), shift, n, dim, _metric(metric)))
    return out


def graph_build(data, metric, shift=5, search_degree=15, fixed_degree=31, budget=150,
                batch_div=0, nthreads=None):
    """Proximity graph in the bfsg.graph layout (n << shift uint64)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, dim = data.shape
    out = np.empty(n << shift, dtype=np.uint64)
    _check(load_library().song_graph_build(_ptr(data), n, dim, _metric(metric), shift, search_degree,
                                           fixed_degree, budget, batch_div,
                                           nthreads or os.cpu_count() or 1, _ptr(out)))
    return out


def sample_entries(n, count=4096, seed=11, shuffle=False):
    """count distinct vertex ids drawn uniformly from 0..n-1 (seeded), sorted,
    or in draw order with shuffle=True (then any prefix is itself a uniform
    sample, e.g. the coarse entries of a two-level choice)."""
    rng = np.random.default_rng(seed)
    ids = rng.choice(n, min(count, n), replace=False).astype(np.uint64)
    return ids if shuffle else np.sort(ids)


def graph_build_gpu(data, metric, shift=5, search_degree=15, fixed_degree=31, budget=150,
                    batch_div=64, device=0, nthreads=None):
    """graph_build with the searches of every batch on the GPU; the same graph
    bit for bit."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, dim = data.shape
    out = np.empty(n << shift, dtype=np.uint64)
    _check(load_library().song_graph_build_gpu(_ptr(data), n, dim, _metric(metric), shift, search_degree,
                                               fixed_degree, budget, batch_div, device,
                                               nthreads or os.cpu_count() or 1, _ptr(out)))
    return out


def hash_planes(dim, seed=123):
    """HASH_BITS x dim standard-normal hyperplanes (seeded), for SONG_STORAGE_BITS."""
    return np.random.default_rng(seed).standard_normal((HASH_BITS, dim)).astype(np.float32)


def debug_fail_alloc(n):
    """Test hook: the n-th next device allocation of the library fails (0: none)."""
    _check(load_library().song_debug_fail_alloc(int(n)))


def debug_fixhash(ids, pq):
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    out = np.empty(ids.size, dtype=np.int32)
    _check(load_library().song_debug_fixhash(_ptr(ids), ids.size, pq, _ptr(out)))
    return out


def write_bfsg(graph_path, data_path, graph, data):
    """bfsg.graph (uint64) and bfsg.data (float32) as the reference dumps them."""
    np.ascontiguousarray(graph, dtype=np.uint64).tofile(graph_path)
    np.ascontiguousarray(data, dtype=np.float32).tofile(data_path)


def read_bfsg(graph_path, data_path, n, dim, shift):
    graph = np.fromfile(graph_path, dtype=np.uint64, count=n << shift)
    data = np.fromfile(data_path, dtype=np.float32, count=n * dim).reshape(n, dim)
    return graph, data


# ---------------------------------------------------------------------------
# Decoding of stored low-precision rows (for inspection and tests)
# ---------------------------------------------------------------------------

def _e4m3_table():
    t = np.zeros(256, dtype=np.float32)
    for b in range(256):
        sgn = -1.0 if b & 0x80 else 1.0
        e = (b >> 3) & 0xF
        m = b & 0x7
        if e == 0xF and m == 0x7:
            t[b] = np.nan
        elif e == 0:
            t[b] = sgn * (m / 8.0) * 2.0 ** -6
        else:
            t[b] = sgn * (1.0 + m / 8.0) * 2.0 ** (e - 7)
    return t


E4M3 = _e4m3_table()


def dequantize_rows(raw, storage, dim):
    """FP32 values the kernel computes with, from Index.rows() bytes."""
    st = _storage(storage)
    if st == 0:
        return raw.view(np.float32)[:, :dim].copy()
    if st == 1:
        u16 = raw.view(np.uint16)[:, :dim].astype(np.uint32)
        return (u16 << 16).view(np.float32)
    dpad = (dim + 15) // 16 * 16
    scale = raw[:, dpad:dpad + 4].copy().view(np.float32)[:, 0]
    vals = E4M3[raw[:, :dim]]
    return (vals * scale[:, None]).astype(np.float32)


# ---------------------------------------------------------------------------
# Early-exit network: training kernels (device) and checks (host)
# ---------------------------------------------------------------------------

def mlp_init(seed=0):
    """He-style initial FP32 parameters in the SONG_MLP_PARAMS layout."""
    rng = np.random.default_rng(seed)
    p = np.zeros(MLP_PARAMS, dtype=np.float32)
    p[0:160] = rng.standard_normal(160) * np.sqrt(2.0 / 5)
    p[192:1216] = rng.standard_normal(1024) * np.sqrt(2.0 / 32)
    p[1248:1280] = rng.standard_normal(32) * np.sqrt(1.0 / 32)
    return p


def mlp_grad(x, y, params, w=None):
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    w = None if w is None else np.ascontiguousarray(w, np.float32)
    params = np.ascontiguousarray(params, np.float32)
    g = np.empty(MLP_PARAMS, np.float32)
    loss = np.zeros(1, np.float32)
    _check(load_library().song_mlp_grad(_ptr(x), _ptr(y), _ptr(w), x.shape[0], _ptr(params), _ptr(g), _ptr(loss)))
    return g, float(loss[0])


def mlp_forward(x, params):
    x = np.ascontiguousarray(x, np.float32)
    params = np.ascontiguousarray(params, np.float32)
    out = np.empty(x.shape[0], np.float32)
    _check(load_library().song_mlp_forward(_ptr(x), x.shape[0], _ptr(params), _ptr(out)))
    return out


def mlp_train_device(x_ptr, y_ptr, w_ptr, n, perm_ptr, epochs, batch, lr, params_ptr, loss_ptr=None, stream=None):
    """song_mlp_train_device on raw device pointers."""
    v = lambda a: ctypes.c_void_p(a) if a else None
    _check(load_library().song_mlp_train_device(v(x_ptr), v(y_ptr), v(w_ptr), int(n), v(perm_ptr), int(epochs),
                                                int(batch), float(lr), v(params_ptr), v(loss_ptr), v(stream)))
