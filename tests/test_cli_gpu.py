"""The drop-in command line on the GPU (reference argv, main.cu:49-100): the
GPU builder writes the reference's graph, and test mode prints, line by
line, exactly the ids of the oracle's search -- from vertex 0 as the
reference starts, and from entry points when SONG_ENTRIES is set."""
import os
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from test_cli_cpu import write_libsvm

pytestmark = pytest.mark.gpu


def _run(args, cwd, **env):
    from song_gb300.build import CLI_PATH
    e = dict(os.environ, **{k: str(v) for k, v in env.items()})
    return subprocess.run([CLI_PATH] + args, cwd=str(cwd), env=e, capture_output=True, text=True, timeout=300)


def _sample_ids(n, count, seed):
    """The CLI's entry sample: partial Fisher-Yates driven by splitmix64."""
    perm = list(range(n))
    x = seed
    m = (1 << 64) - 1
    for i in range(count):
        x = (x + 0x9E3779B97F4A7C15) & m
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        z ^= z >> 31
        j = i + z % (n - i)
        perm[i], perm[j] = perm[j], perm[i]
    return np.array(perm[:count], dtype=np.uint64)


def test_cli_gpu_build_writes_reference_graph(song, tmp_path):
    g = load_golden("cos_s4_d16")
    write_libsvm(str(tmp_path / "base.libsvm"), g["data"])
    r = _run(["build", "base.libsvm", "0", "0", str(g["data"].shape[0]), str(g["data"].shape[1]), "0", "cos"],
             tmp_path, SONG_SHIFT=4, SONG_SEARCH_DEGREE=7, SONG_FIXED_DEGREE=15, SONG_BUILD_GPU=1)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(str(tmp_path / "bfsg.graph"), dtype=np.uint64), g["graph"])


@pytest.mark.parametrize("entries", [0, 64])
def test_cli_test_mode_prints_the_oracle_ids(song, oracle, tmp_path, entries):
    g = load_golden("l2_s5_d32")
    data, queries = g["data"], g["queries"]
    data.astype(np.float32).tofile(str(tmp_path / "bfsg.data"))
    g["graph"].astype(np.uint64).tofile(str(tmp_path / "bfsg.graph"))
    write_libsvm(str(tmp_path / "q.libsvm"), queries)
    pq, show = 50, 10
    env = {"SONG_ENTRIES": entries, "SONG_STARTS": 3} if entries else {}
    r = _run(["test", "0", "q.libsvm", str(pq), str(data.shape[0]), str(data.shape[1]), str(show), "l2"],
             tmp_path, **env)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip("\n").split("\n")
    assert len(lines) == queries.shape[0]
    ox = oracle.OracleIndex(data, g["graph"], int(g["shift"]), int(g["metric"]))
    if entries:
        starts = ox.nearest_entry(queries, _sample_ids(data.shape[0], entries, 11), ns=3)
        o_ids = ox.kernel_search_from(queries, starts, pq, oracle.MODE_LEX)[0]
    else:
        o_ids = ox.kernel_search(queries, pq, oracle.MODE_LEX)[0]
    for i, line in enumerate(lines):
        assert [int(x) for x in line.split()] == [int(x) for x in o_ids[i, :show]], i


def test_cli_binary_queries_and_results(song, oracle, tmp_path):
    """SONG_QUERY_FORMAT=f32 + SONG_RESULTS: float32 query rows in, nq x
    return_top_k uint64 ids out (UINT64_MAX beyond pq), the oracle's ids."""
    g = load_golden("l2_s5_d32")
    data, queries = g["data"], g["queries"]
    data.astype(np.float32).tofile(str(tmp_path / "bfsg.data"))
    g["graph"].astype(np.uint64).tofile(str(tmp_path / "bfsg.graph"))
    queries.astype(np.float32).tofile(str(tmp_path / "q.f32"))
    pq, show = 20, 25
    r = _run(["test", "0", "q.f32", str(pq), str(data.shape[0]), str(data.shape[1]), str(show), "l2"],
             tmp_path, SONG_QUERY_FORMAT="f32", SONG_RESULTS="ids.u64")
    assert r.returncode == 0, r.stderr
    assert r.stdout == ""
    got = np.fromfile(str(tmp_path / "ids.u64"), dtype=np.uint64).reshape(queries.shape[0], show)
    ox = oracle.OracleIndex(data, g["graph"], int(g["shift"]), int(g["metric"]))
    o_ids = np.asarray(ox.kernel_search(queries, pq, oracle.MODE_LEX)[0], dtype=np.uint64)
    assert np.array_equal(got[:, :pq], o_ids[:, :pq])
    assert np.all(got[:, pq:] == np.uint64(0xFFFFFFFFFFFFFFFF))


def test_cli_multiprobe_knobs(song, oracle, tmp_path):
    """SONG_N_MULTIPROBE / SONG_FINISH_CNT / SONG_MULTIPROBE_DOUBLE_CHECK: the
    knobs the reference compiles in, here per run; the oracle's ids under the
    same knobs."""
    g = load_golden("l2_s5_d32")
    data, queries = g["data"], g["queries"]
    data.astype(np.float32).tofile(str(tmp_path / "bfsg.data"))
    g["graph"].astype(np.uint64).tofile(str(tmp_path / "bfsg.graph"))
    write_libsvm(str(tmp_path / "q.libsvm"), queries)
    pq, show = 50, 10
    ox = oracle.OracleIndex(data, g["graph"], int(g["shift"]), int(g["metric"]))
    for probes, fc, dc in ((2, 1, 1), (3, 2, 0)):
        r = _run(["test", "0", "q.libsvm", str(pq), str(data.shape[0]), str(data.shape[1]), str(show), "l2"],
                 tmp_path, SONG_N_MULTIPROBE=probes, SONG_FINISH_CNT=fc, SONG_MULTIPROBE_DOUBLE_CHECK=dc)
        assert r.returncode == 0, r.stderr
        o_ids = ox.kernel_search(queries, pq, oracle.MODE_LEX, probes=probes, finish_cnt=fc,
                                 double_check=bool(dc))[0]
        lines = r.stdout.strip("\n").split("\n")
        for i, line in enumerate(lines):
            assert [int(x) for x in line.split()] == [int(x) for x in o_ids[i, :show]], (probes, fc, dc, i)
    r = _run(["test", "0", "q.libsvm", str(pq), str(data.shape[0]), str(data.shape[1]), str(show), "l2"],
             tmp_path, SONG_N_MULTIPROBE=9)
    assert r.returncode != 0 and "probes" in r.stderr
