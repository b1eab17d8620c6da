"""Python view of the CPU oracle (oracle/song_oracle.c) and of the reference
harness (oracle/ref_harness.cpp -> oracle/_ref/).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
the cpu_baseline / reference legs of bench.py, always as the correctness reference or the
timed CPU baseline, never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libsong_oracle.so")
REF_DIR = os.path.join(HERE, "_ref")

L2, IP, COS, HAMMING = 0, 1, 2, 3
METRICS = {"l2": L2, "ip": IP, "cos": COS}
MODE_REF, MODE_LEX, MODE_LEX_EXACT = 0, 1, 2
TRACE_FIELDS = 6  # 5 early-exit features + number of changes of the top-k set
NO_ID = np.uint64(0xFFFFFFFFFFFFFFFF)

EV_NAMES = {1: "POP", 2: "FINISH", 3: "TEVICT", 4: "SKIP", 5: "INSERT", 6: "QEVICT", 7: "TEST",
            8: "OUT"}


class _Index(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("graph", ctypes.c_void_p), ("n", ctypes.c_uint64),
                ("dim", ctypes.c_int32), ("shift", ctypes.c_int32), ("metric", ctypes.c_int32),
                ("pad", ctypes.c_int32)]


EVENT_DTYPE = np.dtype([("kind", np.int32), ("pad", np.uint32), ("id", np.uint64),
                        ("dist", np.float32), ("pad2", np.uint32)])


def build(force: bool = False) -> str:
    """Compile song_oracle.c with gcc (contraction off, portable flags)."""
    src = os.path.join(HERE, "song_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(os.path.join(HERE, "song_oracle.h"))):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math",
                           "-fPIC", "-shared", "-pthread", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def build_ref() -> bool:
    """Build oracle/_ref from the reference tree when it is present."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.check_call(["bash", script])
    return ref_available()


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        i32 = ctypes.c_int
        L.orc_kernel_distance.restype = ctypes.c_float
        L.orc_kernel_distance.argtypes = [i32, i32, P, P, i32]
        L.orc_cpu_distance.restype = ctypes.c_double
        L.orc_cpu_distance.argtypes = [i32, i32, P, P]
        L.orc_kernel_search.restype = i32
        L.orc_kernel_search.argtypes = [P, P, i32, i32, i32, i32, P, P, P, P, i32]
        L.orc_kernel_search_log.restype = i32
        L.orc_kernel_search_log.argtypes = [P, P, i32, i32, i32, P, P, i32, P]
        L.orc_kernel_search_log_multi.restype = i32
        L.orc_kernel_search_log_multi.argtypes = [P, P, i32, i32, i32, i32, i32, i32, P, P, i32, P]
        L.orc_classify.restype = i32
        L.orc_classify.argtypes = [P, i32, P, i32, P]
        L.orc_kernel_search_from.restype = i32
        L.orc_kernel_search_from.argtypes = [P, P, i32, P, i32, i32, i32, i32, P, P, P, P, i32]
        L.orc_kernel_search_multi.restype = i32
        L.orc_kernel_search_multi.argtypes = [P, P, i32, P, i32, i32, i32, i32, i32, i32, i32, P, P, P, P, i32]
        L.orc_nearest_entry_2level.restype = i32
        L.orc_nearest_entry_2level.argtypes = [P, P, i32, P, i32, i32, i32, i32, i32, P, i32]
        L.orc_nearest_entry.restype = i32
        L.orc_nearest_entry.argtypes = [P, P, i32, P, i32, i32, i32, P]
        L.orc_kernel_search_trace.restype = i32
        L.orc_kernel_search_trace.argtypes = [P, P, i32, i32, i32, i32, i32, P, P, P, P, P, P]
        L.orc_hash_codes.restype = i32
        L.orc_hash_codes.argtypes = [P, ctypes.c_uint64, i32, P, i32, P]
        L.orc_graph_build.restype = i32
        L.orc_graph_build.argtypes = [P, ctypes.c_uint64, i32, i32, i32, i32, i32, i32, i32, i32, P]
        L.orc_cpu_search.restype = i32
        L.orc_cpu_search.argtypes = [P, P, i32, i32, P, P, i32]
        L.orc_fixhash_hash.restype = i32
        L.orc_fixhash_hash.argtypes = [i32, ctypes.c_uint64]
        L.orc_fixhash_init.argtypes = [P, i32]
        L.orc_fixhash_add.argtypes = [P, i32, ctypes.c_int32]
        L.orc_fixhash_test.restype = i32
        L.orc_fixhash_test.argtypes = [P, i32, ctypes.c_int32]
        L.orc_fixhash_del.argtypes = [P, i32, ctypes.c_int32]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


class OracleIndex:
    """Holds host arrays in the reference's file layouts (bfsg.data: n x dim f32;
    bfsg.graph: n << shift uint64, slot 0 = degree)."""

    def __init__(self, data: np.ndarray, graph: np.ndarray, shift: int, metric: int):
        self.data = np.ascontiguousarray(data, dtype=np.float32)
        self.graph = np.ascontiguousarray(graph, dtype=np.uint64).reshape(-1)
        self.n, self.dim = self.data.shape
        self.shift = int(shift)
        self.metric = int(metric)
        assert self.graph.size == self.n << self.shift
        self._s = _Index(self.data.ctypes.data, self.graph.ctypes.data, self.n, self.dim,
                         self.shift, self.metric, 0)

    @property
    def ref(self):
        return ctypes.byref(self._s)

    def kernel_search(self, queries, pq, mode=MODE_LEX, use_fma=True, nthreads=None, probes=1, finish_cnt=1,
                      double_check=False):
        """Batched search from vertex 0.  probes / finish_cnt / double_check
        are the reference's N_MULTIPROBE / FINISH_CNT (warp_astar_accelerator.h:
        29-30) and __ENABLE_MULTIPROBE_DOUBLE_CHECK (:307-310)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        out = np.empty((nq, pq), dtype=np.uint64)
        hops = np.empty(nq, dtype=np.int32)
        evals = np.empty(nq, dtype=np.int32)
        popped = np.empty(nq, dtype=np.int32)
        if probes == 1 and finish_cnt == 1 and not double_check:
            rc = lib().orc_kernel_search(self.ref, _ptr(q), nq, pq, mode, int(use_fma), _ptr(out),
                                         _ptr(hops), _ptr(evals), _ptr(popped),
                                         nthreads or default_threads())
        else:
            rc = lib().orc_kernel_search_multi(self.ref, _ptr(q), nq, None, 1, pq, int(probes), int(finish_cnt),
                                               int(double_check), mode, int(use_fma), _ptr(out), _ptr(hops),
                                               _ptr(evals), _ptr(popped), nthreads or default_threads())
        if rc != 0:
            raise ValueError("orc_kernel_search failed")
        return out, hops, evals, popped

    def kernel_search_from(self, queries, starts, pq, mode=MODE_LEX, use_fma=True, nthreads=None, probes=1,
                           finish_cnt=1, double_check=False):
        """kernel_search with query i starting from the vertices starts[i]
        (an nq-vector: one start each; nq x ns: ns starts each)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        st = np.ascontiguousarray(starts, dtype=np.uint64)
        ns = 1 if st.ndim == 1 else st.shape[1]
        nq = q.shape[0]
        out = np.empty((nq, pq), dtype=np.uint64)
        hops = np.empty(nq, dtype=np.int32)
        evals = np.empty(nq, dtype=np.int32)
        popped = np.empty(nq, dtype=np.int32)
        rc = lib().orc_kernel_search_multi(self.ref, _ptr(q), nq, _ptr(st), ns, pq, int(probes), int(finish_cnt),
                                           int(double_check), mode, int(use_fma), _ptr(out), _ptr(hops),
                                           _ptr(evals), _ptr(popped), nthreads or default_threads())
        if rc != 0:
            raise ValueError("orc_kernel_search_from failed")
        return out, hops, evals, popped

    def nearest_entry(self, queries, entries, ns=1, use_fma=True):
        """Per query, the ns entry vertices nearest by the kernel's distance,
        ascending (an nq-vector when ns == 1, else nq x ns)."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        e = np.ascontiguousarray(entries, dtype=np.uint64)
        out = np.empty((q.shape[0], ns), dtype=np.uint64)
        if lib().orc_nearest_entry(self.ref, _ptr(q), q.shape[0], _ptr(e), e.size, ns, int(use_fma), _ptr(out)) != 0:
            raise ValueError("orc_nearest_entry failed")
        return out[:, 0].copy() if ns == 1 else out

    def nearest_entry_2level(self, queries, entries, coarse, probes, ns, use_fma=True, nthreads=None):
        """Two-level entry choice (orc_nearest_entry_2level): nq x ns."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        e = np.ascontiguousarray(entries, dtype=np.uint64)
        out = np.empty((q.shape[0], ns), dtype=np.uint64)
        if lib().orc_nearest_entry_2level(self.ref, _ptr(q), q.shape[0], _ptr(e), e.size, coarse, probes, ns,
                                          int(use_fma), _ptr(out), nthreads or default_threads()) != 0:
            raise ValueError("orc_nearest_entry_2level failed")
        return out

    def kernel_search_log(self, query, pq, mode, use_fma=True, cap=1 << 18, probes=1, finish_cnt=1,
                          double_check=False):
        q = np.ascontiguousarray(query, dtype=np.float32).reshape(-1)
        out = np.empty(pq, dtype=np.uint64)
        log = np.zeros(cap, dtype=EVENT_DTYPE)
        n = ctypes.c_int(0)
        rc = lib().orc_kernel_search_log_multi(self.ref, _ptr(q), pq, int(probes), int(finish_cnt),
                                               int(double_check), mode,
                                               int(use_fma), _ptr(out), _ptr(log), cap, ctypes.byref(n))
        if rc != 0:
            raise ValueError("orc_kernel_search_log failed")
        if n.value > cap:
            raise ValueError("event log overflow")
        return out, log[:n.value]

    def kernel_search_trace(self, query, pq, k, trace_hops, mode=MODE_LEX_EXACT, use_fma=True):
        """One query with the learned kernel's per-hop trace
        (song_oracle.h: orc_kernel_search_trace).  Returns (trace
        [traced x 6], final top-k version, ids, hops, evals)."""
        q = np.ascontiguousarray(query, dtype=np.float32).reshape(-1)
        tr = np.zeros((trace_hops, TRACE_FIELDS), dtype=np.float32)
        fin, traced, hops, evals = (ctypes.c_int32(0) for _ in range(4))
        out = np.empty(pq, dtype=np.uint64)
        rc = lib().orc_kernel_search_trace(self.ref, _ptr(q), pq, k, mode, int(use_fma), trace_hops, _ptr(tr),
                                           ctypes.byref(fin), ctypes.byref(traced), _ptr(out),
                                           ctypes.byref(hops), ctypes.byref(evals))
        if rc != 0:
            raise ValueError("orc_kernel_search_trace failed")
        return tr[:traced.value], fin.value, out, hops.value, evals.value

    def cpu_search(self, queries, k, nthreads=None):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        out = np.empty((nq, k), dtype=np.uint64)
        ex = np.empty(nq, dtype=np.int32)
        rc = lib().orc_cpu_search(self.ref, _ptr(q), nq, k, _ptr(out), _ptr(ex),
                                  nthreads or default_threads())
        if rc != 0:
            raise ValueError("orc_cpu_search failed")
        return out, ex


def hash_codes(rows, planes, use_fma=True):
    """256-bit sign codes (n x 8 uint32) of rows from 256 hyperplanes, summed as
    the kernel sums (orc_hash_codes)."""
    rows = np.ascontiguousarray(rows, dtype=np.float32)
    planes = np.ascontiguousarray(planes, dtype=np.float32)
    n, dim = rows.shape
    assert planes.shape == (256, dim)
    out = np.empty((n, 8), dtype=np.uint32)
    if lib().orc_hash_codes(_ptr(rows), n, dim, _ptr(planes), int(use_fma), _ptr(out)) != 0:
        raise ValueError("orc_hash_codes failed")
    return out


def graph_build(data, metric, shift=5, search_degree=15, fixed_degree=31, budget=150, batch_div=0, nthreads=None):
    """The reference's CPU builder restated (orc_graph_build): the bfsg.graph
    array (n << shift uint64)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, dim = data.shape
    out = np.empty(n << shift, dtype=np.uint64)
    m = METRICS[metric] if isinstance(metric, str) else int(metric)
    if lib().orc_graph_build(_ptr(data), n, dim, m, shift, search_degree, fixed_degree, budget, batch_div,
                             nthreads or default_threads(), _ptr(out)) != 0:
        raise ValueError("orc_graph_build failed")
    return out


def classify(log_a, log_b):
    """0 identical, 1 first difference is a float tie, 2 anything else; and the
    index of the first difference (-1 if none)."""
    at = ctypes.c_int(-1)
    a = np.ascontiguousarray(log_a)
    b = np.ascontiguousarray(log_b)
    r = lib().orc_classify(_ptr(a), len(a), _ptr(b), len(b), ctypes.byref(at))
    return r, at.value


def kernel_distance(metric, q, x, use_fma=True):
    q = np.ascontiguousarray(q, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    return lib().orc_kernel_distance(metric, q.size, _ptr(q), _ptr(x), int(use_fma))


def cpu_distance(metric, x, q):
    q = np.ascontiguousarray(q, dtype=np.float32)
    x = np.ascontiguousarray(x, dtype=np.float32)
    return lib().orc_cpu_distance(metric, q.size, _ptr(x), _ptr(q))


class FixHash:
    """The visited hash of the reference's default build, on its own."""

    def __init__(self, pq):
        self.cap = 8 * pq
        self.tab = np.empty(self.cap, dtype=np.int32)
        lib().orc_fixhash_init(_ptr(self.tab), self.cap)

    def hash(self, x):
        return lib().orc_fixhash_hash(self.cap, x)

    def add(self, x):
        lib().orc_fixhash_add(_ptr(self.tab), self.cap, int(x))

    def test(self, x):
        return bool(lib().orc_fixhash_test(_ptr(self.tab), self.cap, int(x)))

    def delete(self, x):
        lib().orc_fixhash_del(_ptr(self.tab), self.cap, int(x))


# ---------------------------------------------------------------------------
# Reference harness (oracle/_ref), present only where the reference tree was
# available at build time.
# ---------------------------------------------------------------------------

def ref_available(shift: int = 5) -> bool:
    return os.path.exists(os.path.join(REF_DIR, "libsongref_s%d.so" % shift))


_ref_libs = {}


def ref_lib(shift: int):
    if shift not in _ref_libs:
        path = os.path.join(REF_DIR, "libsongref_s%d.so" % shift)
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i32 = ctypes.c_int
        u64 = ctypes.c_uint64
        L.ref_build_graph.restype = i32
        L.ref_build_graph.argtypes = [P, u64, i32, i32, ctypes.c_char_p, ctypes.c_char_p]
        L.ref_cpu_search.restype = i32
        L.ref_cpu_search.argtypes = [ctypes.c_char_p, ctypes.c_char_p, u64, i32, i32, P, i32, i32, P]
        L.ref_kernel_search.restype = i32
        L.ref_kernel_search.argtypes = [P, P, u64, i32, i32, i32, P, i32, i32, P, P, P, P]
        L.ref_kernel_search_multi.restype = i32
        L.ref_kernel_search_multi.argtypes = [P, P, u64, i32, i32, i32, P, i32, i32, i32, i32, i32, P, P, P, P]
        L.ref_fixhash_ops.restype = i32
        L.ref_fixhash_ops.argtypes = [i32, P, P, i32, P]
        L.ref_graph_shift.restype = i32
        L.ref_graph_fixed_degree.restype = i32
        L.ref_graph_search_degree.restype = i32
        assert L.ref_graph_shift() == shift
        _ref_libs[shift] = L
    return _ref_libs[shift]


def ref_build_graph(data: np.ndarray, shift: int, metric: int) -> np.ndarray:
    """The reference's sequential CPU builder (graph.h:149-167)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, dim = data.shape
    with tempfile.TemporaryDirectory() as td:
        g = os.path.join(td, "bfsg.graph").encode()
        d = os.path.join(td, "bfsg.data").encode()
        rc = ref_lib(shift).ref_build_graph(_ptr(data), n, dim, metric, g, d)
        assert rc == 0
        graph = np.fromfile(g.decode(), dtype=np.uint64)
        back = np.fromfile(d.decode(), dtype=np.float32).reshape(n, dim)
    assert np.array_equal(back, data)
    return graph


def ref_cpu_search(data, graph, shift, metric, queries, k):
    data = np.ascontiguousarray(data, dtype=np.float32)
    n, dim = data.shape
    q = np.ascontiguousarray(queries, dtype=np.float32)
    out = np.empty((q.shape[0], k), dtype=np.uint64)
    with tempfile.TemporaryDirectory() as td:
        gp = os.path.join(td, "bfsg.graph")
        dp = os.path.join(td, "bfsg.data")
        np.ascontiguousarray(graph, dtype=np.uint64).tofile(gp)
        data.tofile(dp)
        rc = ref_lib(shift).ref_cpu_search(gp.encode(), dp.encode(), n, dim, metric, _ptr(q),
                                           q.shape[0], k, _ptr(out))
        assert rc == 0
    return out


def ref_kernel_search(data, graph, shift, metric, queries, pq, probes=1, finish_cnt=1, double_check=False):
    """The kernel's search steps through the reference containers; probes,
    finish_cnt and double_check are N_MULTIPROBE, FINISH_CNT
    (warp_astar_accelerator.h:29-30) and __ENABLE_MULTIPROBE_DOUBLE_CHECK
    (:307-310)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    graph = np.ascontiguousarray(graph, dtype=np.uint64)
    n, dim = data.shape
    q = np.ascontiguousarray(queries, dtype=np.float32)
    nq = q.shape[0]
    out = np.empty((nq, pq), dtype=np.uint64)
    hops = np.empty(nq, dtype=np.int32)
    evals = np.empty(nq, dtype=np.int32)
    popped = np.empty(nq, dtype=np.int32)
    rc = ref_lib(shift).ref_kernel_search_multi(_ptr(data), _ptr(graph), n, dim, shift, metric, _ptr(q),
                                                nq, pq, int(probes), int(finish_cnt), int(double_check),
                                                _ptr(out), _ptr(hops),
                                                _ptr(evals), _ptr(popped))
    if rc != 0:
        raise ValueError("pq %d not instantiated in the reference harness" % pq)
    return out, hops, evals, popped


def ref_fixhash_ops(pq, ops, keys):
    """Run an add(0)/del(1)/test(2) sequence on the reference FixHash."""
    ops = np.ascontiguousarray(ops, dtype=np.int32)
    keys = np.ascontiguousarray(keys, dtype=np.int32)
    res = np.empty(ops.size, dtype=np.int32)
    rc = ref_lib(5).ref_fixhash_ops(pq, _ptr(ops), _ptr(keys), ops.size, _ptr(res))
    if rc != 0:
        raise ValueError("pq %d not instantiated" % pq)
    return res


def fixhash_ops(pq, ops, keys):
    """The same sequence on the oracle's restatement."""
    h = FixHash(pq)
    res = np.full(len(ops), -1, dtype=np.int32)
    for i, (op, k) in enumerate(zip(ops, keys)):
        if op == 0:
            h.add(k)
        elif op == 1:
            h.delete(k)
        else:
            res[i] = int(h.test(k))
    return res
