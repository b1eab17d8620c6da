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


def test_cli_convert_writes_float32_rows(song, tmp_path):
    """`song convert` densifies LIBSVM vectors as build and test do."""
    from song_gb300.build import CLI_PATH
    data = load_golden("cos_s4_d16")["data"][:300]
    write_libsvm(str(tmp_path / "q.libsvm"), data)
    r = subprocess.run([CLI_PATH, "convert", "q.libsvm", str(data.shape[1]), "q.f32"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(str(tmp_path / "q.f32"), dtype=np.float32).reshape(data.shape), data)
    r = subprocess.run([CLI_PATH, "convert", "q.libsvm", "0", "q.f32"], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "dim" in r.stderr


def test_cli_build_reads_float32_rows(song, tmp_path):
    """SONG_DATA_FORMAT=f32: the base vectors as raw float32 rows (the
    bfsg.data layout) give the same files as the LIBSVM text."""
    from song_gb300.build import CLI_PATH
    g = load_golden("cos_s4_d16")
    data = g["data"]
    data.astype(np.float32).tofile(str(tmp_path / "base.f32"))
    env = dict(os.environ, SONG_SHIFT="4", SONG_SEARCH_DEGREE="7", SONG_FIXED_DEGREE="15", SONG_DATA_FORMAT="f32")
    r = subprocess.run([CLI_PATH, "build", "base.f32", "0", "0", str(data.shape[0]), str(data.shape[1]), "0", "cos"],
                       cwd=str(tmp_path), env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(str(tmp_path / "bfsg.data"), dtype=np.float32).reshape(data.shape), data)
    assert np.array_equal(np.fromfile(str(tmp_path / "bfsg.graph"), dtype=np.uint64), g["graph"])


def test_cli_binary_input_errors(song, tmp_path):
    from song_gb300.build import CLI_PATH
    np.zeros(10, dtype=np.float32).tofile(str(tmp_path / "odd.f32"))  # 10 floats: not rows of 4
    args = [CLI_PATH, "build", "odd.f32", "0", "0", "2", "4", "0", "l2"]
    r = subprocess.run(args, cwd=str(tmp_path), env=dict(os.environ, SONG_DATA_FORMAT="f32"),
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "whole number of rows" in r.stderr
    r = subprocess.run(args, cwd=str(tmp_path), env=dict(os.environ, SONG_DATA_FORMAT="fvecs"),
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "SONG_DATA_FORMAT" in r.stderr
    r = subprocess.run([CLI_PATH, "build", "missing.f32", "0", "0", "2", "4", "0", "l2"], cwd=str(tmp_path),
                       env=dict(os.environ, SONG_DATA_FORMAT="f32"), capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "not found" in r.stderr
