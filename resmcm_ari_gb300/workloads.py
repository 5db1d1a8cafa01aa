"""Seeded workloads of the measured configurations.

* ``dblp_small_chain``   three-type P/A/V graph, chain A-P-V-P-A (plain, CPU-runnable size)
* ``retail_four_chains`` four-type U/I/C/T graph and its four chains (plain at scale)
* ``batch_chains``       five-type schema graph and 512 seeded random-walk
                         meta-paths of 2-10 matrices, filtered by the RES estimate
* ``poisson_queries``    a seeded Poisson arrival stream of meta-path queries
                         over two resident graphs (served)
* ``stress_graph``       X/Y/Z graph with both-side Zipf(1.6) degrees; its
                         12-matrix chain ``STRESS_CHAIN`` runs in uint64
                         (memory bound)

The published datasets of the reference's paper are not redistributable, so
these synthetic graphs stand in for them with the configured sizes, degree
laws and chain shapes.  Every generator is deterministic in its seed.
"""
from __future__ import annotations

import math

import numpy as np

from . import synth

# 5-type schema of the batched workload: a ring with one chord
BATCH_SCHEMA = [(0, 1), (1, 2), (2, 3), (3, 4), (4, 0), (1, 3)]


def batch_graph(seed: int = 2, sizes=(10_000, 500_000), mean_deg=(5, 40), s_range=(1.3, 2.0),
                scale: float = 1.0) -> synth.SyntheticHIN:
    """Five types with log-uniform sizes; per relation a mean degree in
    ``mean_deg`` and Zipf(s) degree laws on both sides, s in ``s_range``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo, hi = math.log(sizes[0]), math.log(sizes[1])
    type_sizes = [max(2, int(round(math.exp(rng.uniform(lo, hi)) * scale))) for _ in range(5)]
    g = synth.SyntheticHIN(f"batch_s{seed}_x{scale:g}", type_sizes)
    for r, (a, b) in enumerate(BATCH_SCHEMA):
        d = float(rng.uniform(*mean_deg))
        s = float(rng.uniform(*s_range))
        na, nb = type_sizes[a], type_sizes[b]
        edges = int(min(na * d, na * nb * 0.5))
        src, dst = synth.chung_lu(rng, na, nb, edges, s, s)
        g.relations.append(synth.Relation(a, b, 2 * r, 2 * r + 1, src, dst))
    return g


def batch_walks(seed: int, g: synth.SyntheticHIN, count: int, lengths=(2, 10)) -> list:
    """Seeded random walks over the schema (lengths uniform in ``lengths``)."""
    return synth.random_metapaths(seed, g, count, lengths)


def batch_chains(engine, graph, g: synth.SyntheticHIN, count: int = 512, seed: int = 3, lengths=(2, 10),
                 max_est_nnz: float = 2e6, max_est_cost: float = 4e7, max_tries: int = 200_000) -> list:
    """``count`` walks whose RES estimates fit: estimated result nnz at most
    ``max_est_nnz`` and estimated chain cost (the DP's m[0][len-1], the sum of
    the estimated intermediate sizes) at most ``max_est_cost``.  Unbounded
    walks over these degrees reach dense results of up to 10^11 entries; the
    filter is the estimator's own admission signal, computed on the GPU."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out, tried = [], 0
    while len(out) < count and tried < max_tries:
        mp = synth.random_metapaths(int(rng.integers(1 << 31)), g, 1, lengths)[0]
        tried += 1
        leaves = graph.leaves(mp)
        c = engine.estimate(leaves)
        L = c.shape[0]
        if c[0, L - 1] > max_est_nnz:
            continue
        _, m, _ = engine.order(c)
        if m[0, L - 1] > max_est_cost:
            continue
        out.append(mp)
    return out


def retail_four_chains(scale: float = 1.0, seed: int = 1) -> synth.SyntheticHIN:
    sc = lambda x: max(2, int(round(x * scale)))  # noqa: E731
    return synth.retail_like(n_u=sc(1_000_000), n_i=sc(300_000), n_c=sc(2_000), n_t=sc(20_000),
                             ui_edges=sc(20_000_000), seed=seed)


def dblp_small_chain(seed: int = 0) -> synth.SyntheticHIN:
    return synth.dblp_like(seed=seed)


def poisson_queries(seed: int, rate_qps: float, duration_s: float, graphs: list, lengths=(2, 8)) -> list:
    """Arrival times (seconds) and (graph index, meta-path) of a Poisson stream;
    each query picks its graph uniformly among ``graphs`` (a list of
    (SyntheticHIN, candidate meta-paths)) and one of that graph's paths of a
    length in ``lengths``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    while True:
        t += float(rng.exponential(1.0 / rate_qps))
        if t > duration_s:
            break
        gi = int(rng.integers(len(graphs)))
        cands = [mp for mp in graphs[gi][1] if lengths[0] <= (mp.count("-") // 2) <= lengths[1]]
        out.append((t, gi, cands[int(rng.integers(len(cands)))]))
    return out


def stress_graph(seed: int = 4, n_x: int = 5_000_000, n_y: int = 5_000_000, n_z: int = 100_000,
                 xy_edges: int = 60_000_000, yz=(1, 4), s: float = 1.6) -> synth.SyntheticHIN:
    """X/Y/Z graph: X-Y with both-side Zipf(s) degrees, each Y linked to 1-4 Z."""
    rng = np.random.Generator(np.random.PCG64(seed))
    src, dst = synth.chung_lu(rng, n_x, n_y, xy_edges, s, s)
    lo, hi = yz
    cnt = rng.integers(lo, hi + 1, size=n_y)
    ysrc = np.repeat(np.arange(n_y, dtype=np.int64), cnt)
    zdst = rng.integers(0, n_z, size=ysrc.size).astype(np.int64)
    ysrc, zdst = synth.dedup_pairs_keep_order(ysrc, zdst, n_z)
    g = synth.SyntheticHIN(f"stress_s{seed}", [n_x, n_y, n_z])
    g.relations = [synth.Relation(0, 1, 0, 1, src, dst), synth.Relation(1, 2, 2, 3, ysrc, zdst)]
    return g


# Z-Y-X-Y-X-Y-Z-Y-X-Y-X-Y-Z over the stress graph (X=0, Y=1, Z=2; edge types
# X->Y 0, Y->X 1, Y->Z 2, Z->Y 3): twelve matrices, a Z x Z result.
STRESS_CHAIN = "2-3-1-1-0-0-1-1-0-0-1-2-2-3-1-1-0-0-1-1-0-0-1-2-2"


def stress_scaled(scale: float, seed: int = 4) -> synth.SyntheticHIN:
    """The stress graph with every vertex and edge count multiplied by ``scale``."""
    return stress_graph(seed=seed, n_x=max(2, int(5_000_000 * scale)), n_y=max(2, int(5_000_000 * scale)),
                        n_z=max(2, int(100_000 * scale)), xy_edges=max(1, int(60_000_000 * scale)))


def relation_csr(g: synth.SyntheticHIN, rel: int, forward: bool = True):
    """CSR (rowptr int64, col int32) of one direction of a relation in local
    ids, rows sorted by column: the leaf matrix of that edge type, built
    without the graph's text-order adjacency (fast at tens of millions of
    edges)."""
    r = g.relations[rel]
    src, dst = (r.src, r.dst) if forward else (r.dst, r.src)
    nrows = g.type_sizes[r.src_type if forward else r.dst_type]
    key = src.astype(np.int64) * np.int64(1 << 32) + dst.astype(np.int64)
    key = np.sort(key)
    rows = (key >> 32).astype(np.int64)
    col = (key & 0xFFFFFFFF).astype(np.int32)
    rowptr = np.zeros(nrows + 1, np.int64)
    np.cumsum(np.bincount(rows, minlength=nrows), out=rowptr[1:])
    return rowptr, col


# leaves of the stress chain Z-Y-X-Y-X-Y-Z-Y-X-Y-X-Y-Z: (relation, forward)
# per position; relation 0 is X-Y, 1 is Y-Z
STRESS_LEAVES = [(1, False), (0, False), (0, True), (0, False), (0, True), (1, True),
                 (1, False), (0, False), (0, True), (0, False), (0, True), (1, True)]


def chain_plan(c: np.ndarray, split: np.ndarray, dims: list, leaf_bytes: list, val_bytes: int = 8) -> dict:
    """Device bytes of a chain's products in a given order, from the RES
    estimates: every product (i, j) of the split tree at (4 + val_bytes)
    bytes per estimated entry plus 8 per row pointer, and the live set of the
    executor's stack machine (free after use, as efficient/resmcm.cpp:702-760)
    while each product runs: resident leaves, the intermediates on the stack
    and the product's output."""
    L = c.shape[0]
    per = 4 + val_bytes

    def nbytes(i, j):
        return per * float(c[i, j]) + 8.0 * (dims[i] + 1)

    nodes, peak = [], [0.0, None]
    resident = float(sum(leaf_bytes))

    def run(i, j, held):
        # returns the bytes of (i, j)'s result; `held` = bytes live outside it
        if i == j:
            return 0.0
        k = int(split[i, j])
        left = run(i, k, held)
        right = run(k + 1, j, held + left)
        out = nbytes(i, j)
        live = resident + held + left + right + out
        nodes.append({"i": i, "j": j, "est_nnz": float(c[i, j]), "bytes": out, "live_bytes": live})
        if live > peak[0]:
            peak[0], peak[1] = live, (i, j)
        return out

    run(0, L - 1, 0.0)
    return {"products": nodes, "peak_live_bytes": peak[0], "peak_at": peak[1],
            "largest_intermediate_nnz": max((n["est_nnz"] for n in nodes if (n["i"], n["j"]) != (0, L - 1)),
                                            default=0.0),
            "result_nnz": float(c[0, L - 1])}
