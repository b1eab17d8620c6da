"""The reference's own GPU kernel, rebuilt for sm_100 (oracle/build_ref_gpu.sh),
against the golden fixtures and the oracle.

Pins what the host harness could only assume: the reference binary's
distances are the lane-strided sums with FMA contraction.  Its ids equal the
golden ids (the reference containers driven on the host with FMA) on every
query; the oracle's REF mode without FMA is reported for contrast.  Skipped
where the prebuilt cubins are absent."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden

pytestmark = pytest.mark.gpu

NAMES = {0: "l2", 1: "ip", 2: "cos"}


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_reference_kernel_matches_golden(oracle, name, capsys):
    from oracle import ref_gpu
    g = load_golden(name)
    metric, shift = int(g["metric"]), int(g["shift"])
    dim = g["data"].shape[1]
    ox = oracle.OracleIndex(g["data"], g["graph"], shift, metric)
    nofma_differs = []
    for pq in g["pqs"]:
        pq = int(pq)
        if not ref_gpu.available(NAMES[metric], dim, pq):
            pytest.skip("reference cubins not built on this host")
        for measure in (True, False):
            ids, _ = ref_gpu.run(ref_gpu.cubin_path(NAMES[metric], dim, pq, measure), g["data"], g["graph"], shift,
                                 g["queries"], pq, measure)
            assert np.array_equal(ids, g["kernel_ids_%d" % pq]), (name, pq, measure)
        nf, *_ = ox.kernel_search(g["queries"], pq, oracle.MODE_REF, use_fma=False)
        nofma_differs.append(int((nf != g["kernel_ids_%d" % pq]).any(axis=1).sum()))
    with capsys.disabled():
        print("\n[%s] reference sm_100 kernel == golden (FMA) on all queries; without FMA the oracle "
              "differs on %s queries (pq %s)" % (name, nofma_differs, list(g["pqs"])))


def test_reference_kernel_contracts_to_fma():
    """The reference binary orders the FMA-probe pairs as fused multiply-add
    does, not as separate multiply and add (settles nvcc's contraction of
    tmp += a*b in warp_astar_accelerator.h:244-256 by experiment)."""
    import os
    from conftest import GOLDEN
    from oracle import ref_gpu
    z = np.load(os.path.join(GOLDEN, "fma_probe.npz"))
    pq = int(z["pq"])
    if not ref_gpu.available("l2", 128, pq):
        pytest.skip("reference cubins not built on this host")
    graph = z["graph"].astype(np.uint64)
    for i in range(z["data"].shape[0]):
        ids, _ = ref_gpu.run(ref_gpu.cubin_path("l2", 128, pq, False), z["data"][i], graph, int(z["shift"]),
                             z["queries"][i:i + 1], pq, False)
        assert np.array_equal(ids[0], z["fma_ids"][i])
        assert not np.array_equal(ids[0], z["nofma_ids"][i])


def test_gb300_kernel_on_fma_probe(song):
    import os
    from conftest import GOLDEN
    z = np.load(os.path.join(GOLDEN, "fma_probe.npz"))
    graph = z["graph"].astype(np.uint64)
    for i in range(z["data"].shape[0]):
        with song.Index(graph, z["data"][i], int(z["shift"]), 0) as ix:
            ids = ix.search(z["queries"][i:i + 1], int(z["pq"]))
        assert np.array_equal(ids[0], z["fma_ids"][i])
