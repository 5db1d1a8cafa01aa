"""Served meta-path queries: a seeded Poisson arrival stream over resident
graphs, run through the query server (rmcm_server_*) and, for comparison,
through the plain one-query-at-a-time path (rmcm_run_metapath) on the same
arrival times.

Both report, per query, the latency from its arrival to its completion
(queueing included) and its result as (nnz, digest), so the two runs can be
compared query by query; throughput is completed queries over the time from
the first arrival to the last completion.
"""
from __future__ import annotations

import time

import numpy as np

from . import OK, synth


def predicted_bytes(c: np.ndarray, split: np.ndarray, dims: list) -> float:
    """Device bytes the server predicts for a chain (the admission rule of
    rmcm_server: every node of the split tree at 12 bytes per estimated entry,
    8 per row pointer, 40 per row of scratch)."""
    L = c.shape[0]
    total, st = 0.0, [(0, L - 1)]
    while st:
        i, j = st.pop()
        if i == j:
            continue
        rows = float(dims[i])
        total += 12.0 * float(c[i, j]) + 8.0 * (rows + 1) + 40.0 * rows
        k = int(split[i, j])
        st += [(i, k), (k + 1, j)]
    return total


def catalog(engine, hg, g: synth.SyntheticHIN, count: int, seed: int, lengths=(2, 8),
            max_bytes: float = float("inf"), max_tries: int = 20000) -> list:
    """``count`` distinct seeded random-walk meta-paths of ``g`` whose
    predicted bytes stay within ``max_bytes`` (the estimator's own signal;
    no limit by default)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out, seen, tries = [], set(), 0
    while len(out) < count and tries < max_tries:
        tries += 1
        mp = synth.random_metapaths(int(rng.integers(1 << 31)), g, 1, lengths)[0]
        if mp in seen:
            continue
        seen.add(mp)
        leaves = hg.leaves(mp)
        c = engine.estimate(leaves)
        split, _, _ = engine.order(c)
        dims = [m.shape[0] for m in leaves] + [leaves[-1].shape[1]]
        if predicted_bytes(c, split, dims) <= max_bytes:
            out.append(mp)
    return out


def poisson_stream(seed: int, rate_qps: float, count: int, catalogs: list) -> list:
    """[(arrival s, graph index, meta-path)]: exponential gaps at ``rate_qps``,
    the graph drawn uniformly, then a path uniformly from its catalog."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t, out = 0.0, []
    for _ in range(count):
        t += float(rng.exponential(1.0 / rate_qps))
        gi = int(rng.integers(len(catalogs)))
        out.append((t, gi, catalogs[gi][int(rng.integers(len(catalogs[gi])))]))
    return out


def _summary(lat: list, first: float, last: float, n_ok: int, n: int) -> dict:
    lat = np.asarray(lat, np.float64)
    span = max(last - first, 1e-9)
    return {"queries": n, "completed_ok": n_ok, "qps": n_ok / span, "span_s": span,
            "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
            "mean_ms": float(lat.mean() * 1e3) if lat.size else None}


def run_served(server, stream: list, lead_s: float = 0.05) -> dict:
    """Submits ``stream`` at its arrival times and collects every result."""
    results = {}
    base = server.now() + lead_s
    for i, (t, gi, mp) in enumerate(stream):
        arrival = base + t
        while True:
            left = arrival - server.now()
            if left <= 0:
                break
            for r in server.poll(wait_s=min(left, 0.01)):
                results[r["tag"]] = r
        server.submit(gi, mp, i, arrival)
    server.drain()
    for r in server.poll():
        results[r["tag"]] = r
    from . import ENOMEM
    ok = [r for r in results.values() if r["status"] == OK]
    lat = [r["t_done"] - r["t_submit"] for r in ok]
    first = base + stream[0][0]
    last = max(r["t_done"] for r in results.values())
    out = _summary(lat, first, last, len(ok), len(stream))
    out["rejected"] = sum(1 for r in results.values() if r["status"] == ENOMEM)
    out["results"] = {k: (r["status"], r["nnz"], r["digest"]) for k, r in results.items()}
    out["admission_wait_ms_p99"] = float(np.percentile([r["t_admit"] - r["t_submit"] for r in ok], 99) * 1e3) if ok else None
    return out


def admits(engine, hg, mp: str, budget: float) -> bool:
    """The server's admission rule for one query: its predicted bytes (RES
    estimates of its DP order) fit the whole budget."""
    leaves = hg.leaves(mp)
    c = engine.estimate(leaves)
    split, _, _ = engine.order(c)
    dims = [m.shape[0] for m in leaves] + [leaves[-1].shape[1]]
    return predicted_bytes(c, split, dims) <= budget


def run_plain(engine, graphs: list, stream: list, lead_s: float = 0.05, budget: float = float("inf")) -> dict:
    """The same arrivals through rmcm_run_metapath, one query at a time.  A
    query the server's admission rule rejects against ``budget`` is rejected
    here too (estimate and order only, like the server), so both paths run
    the same work and give the same results."""
    from . import ENOMEM
    results, lat = {}, []
    base = time.perf_counter() + lead_s
    last = base
    for i, (t, gi, mp) in enumerate(stream):
        arrival = base + t
        now = time.perf_counter()
        if now < arrival:
            time.sleep(arrival - now)
        try:
            if not admits(engine, graphs[gi], mp, budget):
                results[i] = (ENOMEM, 0, 0)
            else:
                C, _, rc = engine.run_metapath(graphs[gi], mp, keep=True)
                nnz, dig = engine.digest(C)
                C.free()
                results[i] = (rc, nnz, dig)
        except Exception as e:  # an error is that query's result
            results[i] = (getattr(e, "status", -1), 0, 0)
        last = time.perf_counter()
        if results[i][0] == OK:
            lat.append(last - arrival)
    n_ok = sum(1 for r in results.values() if r[0] == OK)
    out = _summary(lat, base + stream[0][0], last, n_ok, len(stream))
    out["results"] = results
    out["rejected"] = sum(1 for r in results.values() if r[0] == ENOMEM)
    return out
