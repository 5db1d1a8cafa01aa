"""Host-side logic that needs no GPU: the server's admission bound, the
seeded workload generators and the benchmark's reporting helpers."""
import importlib.util
import os

import numpy as np

from resmcm_ari_gb300 import serve, synth, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_predicted_bytes_walks_the_split_tree():
    # chain of 3 matrices (dims 10 x 20 x 30 x 40), split (0,2) at 1: nodes (0,2) and (0,1)
    c = np.zeros((3, 3))
    c[0, 2], c[0, 1], c[1, 2] = 1000.0, 300.0, 7777.0
    split = np.zeros((3, 3), np.int32)
    split[0, 2] = 1
    dims = [10, 20, 30, 40]
    got = serve.predicted_bytes(c, split, dims)
    want = (12 * 1000 + 8 * 11 + 40 * 10) + (12 * 300 + 8 * 11 + 40 * 10)
    assert got == want


def test_generators_are_seeded():
    a = workloads.retail_four_chains(0.002, seed=3)
    b = workloads.retail_four_chains(0.002, seed=3)
    c = workloads.retail_four_chains(0.002, seed=4)
    for ra, rb in zip(a.relations, b.relations):
        assert np.array_equal(ra.src, rb.src) and np.array_equal(ra.dst, rb.dst)
    assert any(not np.array_equal(ra.dst, rc.dst) for ra, rc in zip(a.relations, c.relations))
    assert a.metapaths == ["1-4-3-5-1-2-2", "2-3-1-1-0-0-1-2-2", "3-5-1-2-2-3-1-4-3",
                           "2-3-1-4-3-5-1-1-0-0-1-2-2"]


def test_random_walks_follow_the_schema():
    g = workloads.retail_four_chains(0.002, seed=1)
    kinds = {(r.src_type, r.et_fwd, r.dst_type) for r in g.relations}
    kinds |= {(r.dst_type, r.et_rev, r.src_type) for r in g.relations}
    walks = synth.random_metapaths(5, g, 50, lengths=(2, 6))
    assert walks == synth.random_metapaths(5, g, 50, lengths=(2, 6))
    for mp in walks:
        x = [int(v) for v in mp.split("-")]
        assert 2 <= (len(x) - 1) // 2 <= 6
        for i in range(0, len(x) - 2, 2):
            assert (x[i], x[i + 1], x[i + 2]) in kinds


def test_poisson_stream_is_seeded_and_ordered():
    g = workloads.retail_four_chains(0.002, seed=1)
    graphs = [(g, g.metapaths)]
    s1 = workloads.poisson_queries(9, 500.0, 0.2, graphs, lengths=(3, 6))
    s2 = workloads.poisson_queries(9, 500.0, 0.2, graphs, lengths=(3, 6))
    assert s1 == s2 and len(s1) > 20
    times = [t for t, _, _ in s1]
    assert times == sorted(times) and times[-1] <= 0.2
    for _, gi, mp in s1:
        assert gi == 0 and 3 <= mp.count("-") // 2 <= 6


def test_bench_reporting_helpers():
    b = _bench()
    assert b.replica_value(4, 8, 2.0) == 16.0
    assert b.max_over_ranks(3.5, 1) == 3.5
    hbm, kind = b.peak_hbm()
    tf, tkind = b.peak_tensor()
    assert hbm > 1000 and tf > 100 and kind in ("measured", "fallback") and tkind == kind
    tr = b.traffic_from_profiles()
    assert tr is not None and tr["bytes_per_alg_byte"] > 1.0
