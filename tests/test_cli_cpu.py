"""The drop-in command-line driver (reference argv, main.cu:49-100): its build
mode parses one-based LIBSVM text (parser.h) and writes bfsg.graph/bfsg.data
that equal the reference builder's files.  CPU only (build mode needs no GPU)."""
import os
import subprocess

import numpy as np

from conftest import load_golden


def write_libsvm(path, data):
    with open(path, "w") as f:
        for i, row in enumerate(data):
            f.write("%d " % (i % 26) + " ".join("%d:%.9g" % (j + 1, v) for j, v in enumerate(row) if v != 0) + "\n")


def test_cli_build_writes_reference_graph(song, tmp_path):
    from song_gb300.build import CLI_PATH
    g = load_golden("cos_s4_d16")
    data = g["data"]
    src = tmp_path / "base.libsvm"
    write_libsvm(str(src), data)
    env = dict(os.environ, SONG_SHIFT="4", SONG_SEARCH_DEGREE="7", SONG_FIXED_DEGREE="15")
    r = subprocess.run([CLI_PATH, "build", str(src), "0", "0", str(data.shape[0]), str(data.shape[1]), "0", "cos"],
                       cwd=str(tmp_path), env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got_g = np.fromfile(str(tmp_path / "bfsg.graph"), dtype=np.uint64)
    got_d = np.fromfile(str(tmp_path / "bfsg.data"), dtype=np.float32).reshape(data.shape)
    assert np.array_equal(got_d, data)
    assert np.array_equal(got_g, g["graph"])


def test_cli_usage_and_bad_metric(song):
    from song_gb300.build import CLI_PATH
    r = subprocess.run([CLI_PATH], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Usage" in r.stdout
    r = subprocess.run([CLI_PATH, "test", "a", "b", "10", "5", "4", "1", "hamming"], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and "Usage" in r.stdout
