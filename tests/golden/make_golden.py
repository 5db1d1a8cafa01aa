"""Generate the golden fixtures in this directory from the reference itself.

Runs only where a checkout of swordzlim/RESMCM_ARI is present: it builds
``oracle/_ref/libref_resmcm.so`` (the reference's efficient/resmcm.cpp
compiled in place, see oracle/Makefile) and drives the reference's own
classes on seeded synthetic graphs written in the reference text format:

* ``DynamicOptimizer::rows_sparse_optimal_matrix_chain_order`` at one OpenMP
  thread (deterministic FP64 sums) → ``c``, ``m``, ``split``;
* ``get_optimal_chain_order`` → ``pairs``;
* ``SSP_dynamic`` → the result rows, sorted, in per-type local ids, stored as
  nnz + SHA-256 of (rowptr int64 LE || col int32 LE), and in full for the
  small cases.

The graphs themselves are not stored: the generator name, its arguments and
the SHA-256 of the generated adjacency are, so a test re-creates the exact
graph and checks it is the one the fixture was made from.

    python tests/golden/make_golden.py [--ref /path/to/RESMCM_ARI]
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from resmcm_ari_gb300 import synth  # noqa: E402

# (fixture name, generator, kwargs, meta-paths or None for the generator's own,
#  store full structure?)
CASES = [
    ("tiny_dblp", "tiny_dblp", {}, None, True),
    ("dblp_small", "dblp_like", {"n_a": 3000, "n_p": 6000, "n_v": 20, "seed": 7},
     ["1-3-0-1-2-4-0-0-1", "1-3-0-0-1", "0-0-1-3-0", "2-4-0-0-1-3-0-1-2", "0-1-2-4-0",
      "1-3-0-0-1-3-0-0-1", "0-0-1-3-0-1-2-4-0-0-1-3-0"], False),
    ("hin4_small", "random_hin",
     {"seed": 11, "type_sizes": [2000, 1500, 800, 300],
      "relations": [[0, 1], [1, 2], [2, 3], [0, 2], [1, 3]], "mean_deg": [2, 5]},
     ("random", 17, 14, (2, 9)), False),
    ("config0_full", "dblp_like", {}, ["1-3-0-1-2-4-0-0-1"], False),
    # the plain-at-scale workload the benchmark times: U=1M, I=300k, C=2k,
    # T=20k, its four chains
    ("retail_full", "retail_like", {"seed": 1}, None, False),
]


def make_graph(gen: str, kwargs: dict):
    fn = getattr(synth, gen)
    kw = dict(kwargs)
    if "relations" in kw:
        kw["relations"] = [tuple(r) for r in kw["relations"]]
    if "mean_deg" in kw:
        kw["mean_deg"] = tuple(kw["mean_deg"])
    return fn(**kw)


def case_metapaths(g, spec):
    if spec is None:
        return list(g.metapaths)
    if isinstance(spec, tuple) and spec[0] == "random":
        _, seed, count, lengths = spec
        return synth.random_metapaths(seed, g, count, lengths)
    return list(spec)


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=oracle.DEFAULT_REF)
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    oracle.build(args.ref)
    if not oracle.ref_available():
        sys.exit("reference checkout not found: cannot make golden fixtures")
    for name, gen, kwargs, mps, full in CASES:
        if args.only and name != args.only:
            continue
        g = make_graph(gen, kwargs)
        paths = case_metapaths(g, mps)
        with tempfile.TemporaryDirectory() as d:
            files = g.write_text(d, paths)
            rg = oracle.RefGraph(files["graph"], files["vertex"], files["edge"])
            out = {"generator": gen, "kwargs": kwargs, "adjacency_sha256": adjacency_sha(g),
                   "n": g.n, "m": g.m, "made_by": "reference efficient/resmcm.cpp via oracle/ref_harness.cpp",
                   "paths": []}
            for mp in paths:
                L = len(oracle.parse_metapath(mp)[1])
                rec = {"metapath": mp, "len": L}
                if L >= 2:
                    c, m, s, pairs = rg.estimate(mp, threads=1)
                    rec.update({"c": c.tolist(), "m": m.tolist(), "split": s.tolist(), "pairs": pairs.tolist()})
                    # dense-dimension order of efficient/naive.cpp (no estimator)
                    vts = oracle.parse_metapath(mp)[0]
                    dims = [g.type_sizes[t] if t < len(g.type_sizes) else 0 for t in range(max(vts) + 1)]
                    ds, dm, dp = oracle.ref_naive_order(dims, vts)
                    rec.update({"dense_split": ds.tolist(), "dense_m": dm.tolist(), "dense_pairs": dp.tolist()})
                rowptr, col, nnz, _ = rg.chain(mp, threads=8)
                rec["nnz"] = int(nnz)
                rec["rows"] = int(rowptr.size - 1)
                rec["structure_sha256"] = structure_sha(rowptr, col)
                if full:
                    rec["rowptr"] = rowptr.tolist()
                    rec["col"] = col.tolist()
                out["paths"].append(rec)
                print(f"{name}: {mp} nnz={nnz}", flush=True)
            rg.close()
        with open(os.path.join(HERE, f"{name}.json"), "w") as f:
            json.dump(out, f, indent=1)
            f.write("\n")


if __name__ == "__main__":
    main()
