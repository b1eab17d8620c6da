"""Builds libsong_gb300.so in-tree (song_gb300/_lib/) for sm_103a.

nvcc compiles the CUDA translation units with
`-gencode arch=compute_103a,code=sm_103a`; the host-only graph builder is
compiled by g++ without floating-point contraction (its distances must match
the reference's CPU arithmetic).  Translation units compile in parallel.
No torch, no cmake.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(LIB_DIR, "libsong_gb300.so")
CLI_PATH = os.path.join(LIB_DIR, "song")

CUDA_SOURCES = ["search.cu", "search_f32.cu", "search_bf16.cu", "search_fp8.cu", "search_bits.cu", "search_learned.cu", "search_multi.cu", "head_mma.cu",
                "capi.cu", "noalloc.cu", "mlp.cu", "serve.cu", "graph_build_gpu.cu", "entries.cu"]
CXX_SOURCES = ["graph_build.cpp"]
HEADERS = ["device_common.cuh", "internal.h", "reg_queue.cuh", "search_kernel.cuh", "graph_build.h",
           "entry_choice.cuh", "entry_tiles.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc_path())))


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = nvcc_path()
    common_deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "song_gb300.h"),
                                                              os.path.abspath(__file__)]
    jobs = []
    objs = []
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + common_deps):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC, "-c", src, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for s in CXX_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + common_deps):
            jobs.append(["g++", "-std=c++17", "-O3", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
                         "-pthread", "-I" + INCLUDE, "-I" + CSRC, "-c", src, "-o", obj])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT) for j in jobs]
    failed = []
    for j, p in zip(jobs, procs):
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        if p.returncode != 0:
            failed.append((j, text))
        elif verbose and text.strip():
            sys.stderr.write(text)
    if failed:
        msg = "\n".join("$ %s\n%s" % (" ".join(j), t) for j, t in failed)
        raise RuntimeError("build failed:\n" + msg)
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-lpthread",
                               "-L" + os.path.join(cuda_home(), "lib64")])
        os.replace(tmp, LIB_PATH)
    cli_src = os.path.join(CSRC, "song_cli.cpp")
    if force or _stale(CLI_PATH, [cli_src, LIB_PATH] + common_deps):
        tmp = CLI_PATH + ".tmp%d" % os.getpid()
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + INCLUDE, cli_src, "-o", tmp,
                               "-L" + LIB_DIR, "-lsong_gb300", "-Wl,-rpath,$ORIGIN", "-pthread"])
        os.replace(tmp, CLI_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
