"""GPU graph construction (song_graph_build_gpu): the searches of every batch
run on the GPU, the edge updates on the host.  The graph must equal the CPU
builder's bit for bit: with one vertex per batch that is the reference's own
sequential graph (the golden fixtures, written by the reference's builder),
and with batch_div > 0 the CPU batch-parallel builder's graph on the same
data, for each metric."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_gpu_builder_reproduces_reference_graph(song, name):
    g = load_golden(name)
    shift = int(g["shift"])
    search_degree = 7 if shift == 4 else 15
    built = song.graph_build_gpu(g["data"], int(g["metric"]), shift, search_degree, (1 << shift) - 1, 150,
                                 batch_div=0)
    assert np.array_equal(built, g["graph"])


@pytest.mark.parametrize("case", [("small-15k-16d-cos", 15000), ("scale-1m-128d-l2", 40000),
                                  ("learned-3m-256d-l2", 8000), ("precision-1m-960d-cos", 4000)])
def test_gpu_builder_equals_cpu_builder(song, case):
    from song_gb300 import datasets as D
    name, n = case
    w = D.WORKLOADS[name]
    data = D.base_vectors(w, n=n)
    args = (data, w.metric, w.shift, w.search_degree, w.fixed_degree, 150)
    cpu = song.graph_build(*args, batch_div=64)
    gpu = song.graph_build_gpu(*args, batch_div=64)
    assert np.array_equal(gpu, cpu)


def test_gpu_builder_inner_product(song):
    rng = np.random.default_rng(7)
    data = rng.standard_normal((6000, 24)).astype(np.float32)
    cpu = song.graph_build(data, "ip", 5, 15, 31, 150, batch_div=32)
    gpu = song.graph_build_gpu(data, "ip", 5, 15, 31, 150, batch_div=32)
    assert np.array_equal(gpu, cpu)
