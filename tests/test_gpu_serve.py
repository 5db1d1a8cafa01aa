"""The query server (rmcm_server_*): results in the mix equal results alone,
queries overlap on the device, admission by RES-predicted bytes holds the
budget, and bad queries complete with their error."""
import numpy as np
import pytest

from resmcm_ari_gb300 import serve, synth, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def two_graphs(native):
    eng = native.Engine(device=0)
    g0 = synth.dblp_like(n_a=3000, n_p=6000, n_v=20, seed=7)
    g1 = workloads.retail_four_chains(scale=0.01, seed=1)
    hg0 = native.HeteroGraph.from_synthetic(eng, g0)
    hg1 = native.HeteroGraph.from_synthetic(eng, g1)
    cats = [serve.catalog(eng, hg0, g0, 10, seed=1, lengths=(2, 8), max_bytes=2e8),
            serve.catalog(eng, hg1, g1, 10, seed=2, lengths=(2, 8), max_bytes=2e8)]
    yield eng, [hg0, hg1], cats
    hg0.close()
    hg1.close()
    eng.close()


def test_results_in_the_mix_equal_results_alone(native, two_graphs):
    eng, graphs, cats = two_graphs
    assert all(len(c) >= 5 for c in cats)
    stream = serve.poisson_stream(11, 2000.0, 80, cats)
    alone = serve.run_plain(eng, graphs, stream)
    srv = native.Server(eng, lanes=4)
    for hg in graphs:
        srv.add_graph(hg)
    mixed = serve.run_served(srv, stream)
    st = srv.stats()
    srv.close()
    assert mixed["completed_ok"] == len(stream) == alone["completed_ok"]
    for i in range(len(stream)):
        assert mixed["results"][i] == alone["results"][i], stream[i]
    assert st["completed"] == len(stream) and st["rejected"] == 0
    assert st["max_running"] > 1            # queries overlapped on the device


def test_admission_holds_the_budget_and_rejects_what_never_fits(native, two_graphs):
    eng, graphs, cats = two_graphs
    preds = []
    for gi, cat in enumerate(cats):
        for mp in cat:
            leaves = graphs[gi].leaves(mp)
            c = eng.estimate(leaves)
            split, _, _ = eng.order(c)
            dims = [m.shape[0] for m in leaves] + [leaves[-1].shape[1]]
            preds.append((serve.predicted_bytes(c, split, dims), gi, mp))
    preds.sort()
    budget = int(preds[len(preds) // 2][0] * 1.5)
    srv = native.Server(eng, lanes=4, mem_budget_bytes=budget)
    for hg in graphs:
        srv.add_graph(hg)
    for tag, (p, gi, mp) in enumerate(preds * 2):
        srv.submit(gi, mp, tag)
    srv.drain()
    res = {r["tag"]: r for r in srv.poll(cap=4096)}
    st = srv.stats()
    srv.close()
    assert len(res) == 2 * len(preds)
    for tag, (p, gi, mp) in enumerate(preds * 2):
        r = res[tag]
        assert abs(r["est_bytes"] - p) <= 1e-6 * p
        if p > budget:
            assert r["status"] == native.ENOMEM
        else:
            assert r["status"] == native.OK
    assert 0 < st["peak_reserved"] <= budget


def test_bad_queries_complete_with_their_error(native, two_graphs):
    eng, graphs, cats = two_graphs
    srv = native.Server(eng, lanes=2)
    srv.add_graph(graphs[0])
    srv.submit(0, "0-99-1", 1)          # no such edge type: empty leaf, still a valid chain
    srv.submit(0, "1-2", 2)             # vertex and edge types do not alternate
    srv.submit(5, cats[0][0], 3)        # no such graph
    srv.drain()
    res = {r["tag"]: r for r in srv.poll()}
    srv.close()
    assert res[2]["status"] == native.EINVAL and res[3]["status"] == native.EINVAL
    assert res[1]["status"] in (native.OK, native.EINVAL)
