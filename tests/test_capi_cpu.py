"""The C-ABI library without a GPU: it loads, exports every symbol the header
declares, validates arguments before touching CUDA, and its (host-only)
graph builder reproduces the reference builder's graphs."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN_CASES, ROOT, load_golden


def header_functions():
    text = open(os.path.join(ROOT, "include", "song_gb300.h")).read()
    return sorted(set(re.findall(r"^\w[\w \*]*?\b(song_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(song):
    L = song.load_library()
    declared = header_functions()
    assert declared, "no declarations parsed"
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(song.EXPORTED) == declared


def test_status_strings(song):
    L = song.load_library()
    assert L.song_status_string(0) == b"ok"
    assert L.song_status_string(3) == b"device wait timed out"


def _create(song, graph, data, shift, metric=0, storage=0):
    L = song.load_library()
    h = ctypes.c_void_p()
    data = np.ascontiguousarray(data, np.float32)
    graph = np.ascontiguousarray(graph, np.uint64)
    rc = L.song_index_create(graph.ctypes.data_as(ctypes.c_void_p), data.ctypes.data_as(ctypes.c_void_p),
                             data.shape[0], data.shape[1], shift, metric, storage, 0, ctypes.byref(h))
    return rc, L.song_last_error().decode()


def test_malformed_graphs_rejected_before_upload(song):
    data = np.zeros((4, 8), np.float32)
    g = np.zeros(4 << 2, np.uint64)
    g[0] = 4  # degree 4 > 3 slots
    rc, msg = _create(song, g, data, 2)
    assert rc == song.SONG_ERR_ARG and "degree" in msg
    g[0] = 1
    g[1] = 9  # id >= n
    rc, msg = _create(song, g, data, 2)
    assert rc == song.SONG_ERR_ARG and "neighbour" in msg
    rc, _ = _create(song, np.zeros(4 << 6, np.uint64), data, 6)
    assert rc == song.SONG_ERR_ARG
    rc, _ = _create(song, np.zeros(4 << 2, np.uint64), data, 2, metric=7)
    assert rc == song.SONG_ERR_ARG


def test_search_argument_checks(song):
    L = song.load_library()
    rc = L.song_search(None, None, 1, 10, 10, None, None, None)
    assert rc == song.SONG_ERR_ARG


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_graph_builder_reproduces_reference_graph(song, name):
    g = load_golden(name)
    shift = int(g["shift"])
    fixed = (1 << shift) - 1
    search_degree = 7 if shift == 4 else 15
    metric = int(g["metric"])
    built = song.graph_build(g["data"], metric, shift, search_degree, fixed, 150, batch_div=0, nthreads=1)
    assert np.array_equal(built, g["graph"])


def test_batched_builder_is_deterministic_and_valid(song):
    g = load_golden("l2_s5_d32")
    a = song.graph_build(g["data"], 0, 5, 15, 31, 150, batch_div=20, nthreads=4)
    b = song.graph_build(g["data"], 0, 5, 15, 31, 150, batch_div=20, nthreads=2)
    assert np.array_equal(a, b)
    rows = a.reshape(-1, 32)
    assert (rows[:, 0] <= 31).all()
    n = rows.shape[0]
    for r in rows[:200]:
        ids = r[1:1 + int(r[0])]
        assert (ids < n).all()


def test_header_is_plain_c(song, tmp_path):
    """include/song_gb300.h compiles as strict C99 and links against the
    library: every declared function is addressable from C, and the status
    calls work without a GPU."""
    import shutil
    import subprocess
    from song_gb300.build import LIB_DIR
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = header_functions()
    src = tmp_path / "abi.c"
    src.write_text(
        "#include \"song_gb300.h\"\n#include <string.h>\n"
        "typedef void (*fn)(void);\n"
        "static fn table[] = {\n" + ",\n".join("  (fn)%s" % n for n in names) + "\n};\n"
        "int main(void) {\n"
        "  size_t i;\n"
        "  for (i = 0; i < sizeof table / sizeof table[0]; ++i) if (!table[i]) return 2;\n"
        "  return strcmp(song_status_string(SONG_OK), \"ok\") != 0;\n"
        "}\n")
    exe = tmp_path / "abi"
    r = subprocess.run([cc, "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I" + os.path.join(ROOT, "include"),
                        str(src), "-L" + LIB_DIR, "-lsong_gb300", "-Wl,-rpath," + LIB_DIR, "-o", str(exe)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(exe)], timeout=60).returncode == 0
