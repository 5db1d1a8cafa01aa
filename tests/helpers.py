"""Test helpers: fixtures on disk, graph re-creation, structure hashes, DP ties."""
import hashlib
import json
import os

import numpy as np

from resmcm_ari_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["tiny_dblp", "dblp_small", "hin4_small", "config0_full"]


def load_fixture(name: str) -> dict:
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def make_graph(fx: dict):
    kw = dict(fx["kwargs"])
    if "relations" in kw:
        kw["relations"] = [tuple(r) for r in kw["relations"]]
    if "mean_deg" in kw:
        kw["mean_deg"] = tuple(kw["mean_deg"])
    return getattr(synth, fx["generator"])(**kw)


def adjacency_sha(g) -> str:
    ptr, nbr, et = g.adjacency()
    h = hashlib.sha256()
    for a in (g.vertex_types().astype("<i4"), ptr.astype("<i8"), nbr.astype("<i4"), et.astype("<i4")):
        h.update(a.tobytes())
    return h.hexdigest()


def structure_sha(rowptr, col) -> str:
    h = hashlib.sha256()
    h.update(np.asarray(rowptr, "<i8").tobytes())
    h.update(np.asarray(col, "<i4").tobytes())
    return h.hexdigest()


def min_decision_gap(c) -> float:
    """Smallest relative gap between the best and second-best split over the DP.

    Re-runs the reference's DP recurrence (efficient/resmcm.cpp:520-536) in
    Python and reports how close any decision came to a tie; orders may differ
    legitimately only when this is below the estimate tolerance.
    """
    c = np.array(c, dtype=np.float64)
    L = c.shape[0]
    for i in range(L):
        c[i, i] = 0.0
    m = np.zeros((L, L))
    gap = np.inf
    for l in range(1, L):
        for i in range(L - l):
            j = i + l
            costs = []
            for k in range(i, j):
                tmp = c[i, k] + c[k + 1, j] + c[i, j]
                costs.append(m[i, k] + m[k + 1, j] + tmp)
            costs.sort()
            m[i, j] = costs[0]
            if len(costs) > 1:
                gap = min(gap, (costs[1] - costs[0]) / max(abs(costs[1]), 1e-300))
    return gap
