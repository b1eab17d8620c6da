"""Runs the reference's own GPU search kernel (rebuilt for sm_100 by
oracle/build_ref_gpu.sh into oracle/_ref/*.cubin) through
oracle/ref_gpu_runner.cpp.

TEST INFRASTRUCTURE ONLY: pins the oracle's distance arithmetic (nvcc's
default FMA contraction) against the reference binary, and times the
reference kernel as the GPU baseline.  The cubins are built in the
development container (the reference tree is not on the GPU host) and
travel with the working tree; the runner is compiled where it runs.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libref_gpu_runner.so")


def cubin_path(metric: str, dim: int, pq: int, measure: bool = True) -> str:
    return os.path.join(REF_DIR, "warp_astar_%s_d%d_pq%d_%s.cubin" % (metric, dim, pq, "measure" if measure else "nomeasure"))


def available(metric: str, dim: int, pq: int) -> bool:
    return os.path.exists(cubin_path(metric, dim, pq, True)) and os.path.exists(cubin_path(metric, dim, pq, False))


def build() -> str:
    src = os.path.join(HERE, "ref_gpu_runner.cpp")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-I" + os.path.join(cuda, "include"), src,
                           "-o", tmp, "-L" + os.path.join(cuda, "lib64", "stubs"), "-lcuda"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        P = ctypes.c_void_p
        L.refgpu_run.restype = ctypes.c_int
        L.refgpu_run.argtypes = [ctypes.c_char_p, ctypes.c_int, P, ctypes.c_uint64, ctypes.c_int, P, ctypes.c_int, P,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
        _lib = L
    return _lib


def run(cubin: str, data, graph, shift: int, queries, pq: int, measure: bool, repeats: int = 1,
        heap_pq: int = 1023):
    """Launches the reference kernel; returns (ids nq x pq uint64, kernel ms per
    repeat).  heap_pq: the largest pq_size the process will launch (sizes the
    device heap on the first call)."""
    data = np.ascontiguousarray(data, dtype=np.float32)
    graph = np.ascontiguousarray(graph, dtype=np.uint64)
    q = np.ascontiguousarray(queries, dtype=np.float32)
    n, dim = data.shape
    out = np.empty((q.shape[0], pq), dtype=np.uint64)
    ms = np.zeros(max(1, repeats), dtype=np.float32)
    err = ctypes.create_string_buffer(512)
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = lib().refgpu_run(cubin.encode(), int(measure), p(data), n, dim, p(graph), shift, p(q), q.shape[0], pq,
                          int(heap_pq), p(out), p(ms), max(1, repeats), err, 512)
    if rc != 0:
        raise RuntimeError("reference kernel: %s (%d)" % (err.value.decode(), rc))
    return out, ms
