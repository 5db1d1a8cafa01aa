"""Autotuner of the SpGEMM row binning for a set of meta-paths.

The search space is the row-binning tunables of a handle (rmcm_set_tuning):

* ``hash_max_flops``  row-bin threshold between the hash bins and the
  dense / rank bins: {32, 128, 512, 2048, 8192}
* ``hash_load``       hash-table load factor bound: {0.5, 0.7}
* ``threads_per_row`` threads on one short row (<= 32 products): {1, 4, 32, 128}
* ``warp_max_flops``  largest row (products) of an output at most 2048
  columns wide that gets a warp of its own: {0, 512, 2048, 8192}

Each candidate is measured the way the meta-paths are served: recorded as a
batch (rmcm_batch_create) and replayed as one CUDA graph, best of ``reps``
replays.  Every candidate's per-path (nnz, digest) must equal the default
tuning's — tunables move rows between kernels, never change a result — and a
mismatch raises.  ``coordinate`` mode sweeps one tunable at a time from the
current best (5 + 2 + 4 + 4 candidates); ``grid`` mode tries all 160.
"""
from __future__ import annotations

import itertools
import time

SPACE = {
    "hash_max_flops": [32, 128, 512, 2048, 8192],
    "hash_load": [0.5, 0.7],
    "threads_per_row": [1, 4, 32, 128],
    "warp_max_flops": [0, 512, 2048, 8192],
}


class TuningMismatch(RuntimeError):
    pass


def _measure(engine, graph, paths, cfg, lanes, reps, ref, fused=False):
    engine.set_tuning(**cfg)
    t0 = time.perf_counter()
    b = engine.batch(graph, paths, lanes=lanes, fused=fused)
    record_s = time.perf_counter() - t0
    try:
        best = float("inf")
        for _ in range(reps):
            nnz, dig, sec = b.run()
            best = min(best, sec)
            got = list(zip(nnz.tolist(), dig.tolist()))
            if ref is not None and got != ref:
                bad = [paths[i] for i, (x, y) in enumerate(zip(got, ref)) if x != y]
                raise TuningMismatch(f"tuning {cfg} changed the results of {bad[:3]}")
        return best, record_s, got
    finally:
        b.free()


def tune(engine, graph, paths: list, lanes: int = 8, reps: int = 3, mode: str = "coordinate",
         space: dict | None = None, apply: bool = True, fused: bool = False) -> dict:
    """Returns {"best": cfg, "best_s": seconds, "default_s": seconds,
    "table": [(cfg, seconds, record seconds)]} and, with ``apply``, leaves
    the best tuning set on the engine.  ``fused``: measure fused batches
    (rmcm_batch_create_fused) instead of per-chain lanes."""
    space = dict(SPACE if space is None else space)
    default = engine.get_tuning()
    base = {k: default[k] for k in space}
    t_def, rec_def, ref = _measure(engine, graph, paths, base, lanes, reps, None, fused)
    table = [(dict(base), t_def, rec_def)]
    seen = {tuple(sorted(base.items()))}
    best, best_s = dict(base), t_def

    def consider(cfg):
        nonlocal best, best_s
        key = tuple(sorted(cfg.items()))
        if key in seen:
            return
        seen.add(key)
        s, rec, _ = _measure(engine, graph, paths, cfg, lanes, reps, ref, fused)
        table.append((dict(cfg), s, rec))
        if s < best_s:
            best, best_s = dict(cfg), s

    if mode == "grid":
        names = list(space)
        for vals in itertools.product(*(space[n] for n in names)):
            consider(dict(zip(names, vals)))
    elif mode == "coordinate":
        for name in space:
            start = dict(best)
            for v in space[name]:
                cfg = dict(start)
                cfg[name] = v
                consider(cfg)
    else:
        raise ValueError("mode must be 'coordinate' or 'grid'")
    engine.set_tuning(**(best if apply else base))
    return {"best": best, "best_s": best_s, "default": base, "default_s": t_def, "table": table}
