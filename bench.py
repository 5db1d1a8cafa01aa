"""Benchmark: meta-path chains per second on one GB300 (plain drop-in path).

Workload: seeded retail-style heterogeneous graph (U=1,000,000 users,
I=300,000 items, C=2,000 categories, T=20,000 tags; 20M U-I edges with Zipf
degrees on both sides, one category per item, 5-15 tags per item) and its
four meta-path chains I-T-I-C, C-I-U-I-C, T-I-C-I-T, C-I-T-I-U-I-C.  One step
is one pass of the hot path (RES estimator -> warp DP -> binned Gustavson
SpGEMM chain) over all four chains, results computed in full and freed.

* value: chains/s with the leaf CSRs resident in HBM when the timed region
  starts (CUDA events on the engine's stream, barrier + sync on both sides).
* e2e: the same chains through the C ABI from pinned HOST buffers: per step
  every leaf CSR is uploaded (rmcm_mat_upload), the chain runs, and every
  result CSR (rowptr, columns, counts) is copied back to pinned host memory
  (rmcm_mat_download_async: a result's copy overlaps the next chain's work,
  and a loader handle on a helper thread uploads the next chain's leaves
  meanwhile; the step ends when every copy has landed).
* roofline: the dominant numeric SpGEMM pass (largest event time), its
  algorithmic bytes (A + touched B rows + C) over its event-timed duration,
  against the measured HBM copy bandwidth.
* cpu_baseline: the oracle port of the reference's algorithm (Boolean
  Gustavson, OpenMP, all host cores) on the same four chains.
* batched: 512 seeded random-walk meta-paths (2-10 matrices) over a five-type
  schema graph, one at a time through rmcm_run_metapath versus one batch
  recorded once and replayed as a CUDA graph (after the autotuner's sweep of
  the row-binning tunables); chains/s of both and whether every nnz matches.
* served: Poisson query streams over two resident graphs (the A/P/V graph and
  the retail graph) at two offered rates, the plain one-query-at-a-time path
  versus the query server; queries/s, p50 and p99 latency of both and
  whether every result (nnz + digest) matches.
* stress: the twelve-matrix uint64 chain over the X/Y/Z graph at x0.1 vertex
  and edge counts (intermediates of ~1e9 entries); time, multiply-adds per
  second, peak device bytes, and the largest estimated intermediate of the
  RES order versus left to right.

--impl reference times that CPU implementation alone, as the reference arm.
Multi-GPU (torchrun): every rank runs the full workload on its own GPU
(independent replicas, weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from resmcm_ari_gb300 import synth  # noqa: E402

WORKLOAD = ("retail U=1M I=300k C=2k T=20k, U-I 20M edges (Zipf 1.7 users x Zipf 1.3 items), "
            "1 category/item (Zipf 1.1), 5-15 tags/item; chains I-T-I-C, C-I-U-I-C, T-I-C-I-T, C-I-T-I-U-I-C")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the graph (profiling captures)")
    ap.add_argument("--chains", default="all", help="comma list of chain indices to run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-clocks", action="store_true")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--detail", action="store_true", help="per-product stats to stderr")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched (CUDA graph) section")
    ap.add_argument("--no-served", action="store_true", help="skip the served (query server) section")
    ap.add_argument("--no-stress", action="store_true", help="skip the stress (12-matrix uint64 chain) section")
    ap.add_argument("--no-parity", action="store_true", help="skip the parity check against the oracle")
    ap.add_argument("--tune", action="append", default=[], metavar="NAME=VALUE",
                    help="set a row-binning tunable of the engine before the run (rmcm_set_tuning)")
    return ap.parse_args()


def make_graph(scale: float, seed: int):
    """The seeded retail graph (regenerated on every run: about 20 s, and
    nothing stale can be measured)."""
    from resmcm_ari_gb300 import workloads
    return workloads.retail_four_chains(scale=scale, seed=seed)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def peak_tensor():
    """Dense bf16 tensor peak (TFLOP/s, burst) -- FP16 runs at the same rate."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


def traffic_from_profiles():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "dense_numeric_traffic.txt")
    if not os.path.exists(p):
        return None
    out = {}
    for ln in open(p):
        if ":" in ln:
            k, v = ln.split(":", 1)
            out[k.strip()] = v.strip()
    try:
        return {"bytes_per_alg_byte": float(out["dram_bytes_per_algorithmic_byte"]), "source": p}
    except (KeyError, ValueError):
        return None


def sparse_bound_from_profiles():
    """Issue and pipe figures of the dominant product's sparse kernel from the
    committed ncu summary, if any: the bound it reaches (not HBM)."""
    p = os.path.join(ROOT, "profiles", "dense_light_retail_half.md")
    if not os.path.exists(p):
        return None
    out = {"source": os.path.relpath(p, ROOT)}
    keys = {"issue active": "issue_active_pct", "L1 / shared pipe": "l1_shared_pipe_pct",
            "DRAM throughput": "dram_pct"}
    for ln in open(p):
        for k, name in keys.items():
            if ln.startswith("| " + k):
                try:
                    out[name] = float(ln.split("|")[2].strip().split("%")[0])
                except (IndexError, ValueError):
                    pass
    return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int) -> float:
    """The largest value of x over the ranks (every rank gets it); the
    process group's backend decides the tensor's device."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank: int, ws: int, seconds_max: float) -> float:
    """Whole-job throughput of independent replicas: every rank processed
    units_per_rank units; the job took the slowest rank's time."""
    return units_per_rank * ws / seconds_max


def cpu_reference(g, metapaths, steps, warmup, sample_note):
    """Oracle port of the reference's algorithm on all host cores: chains/s over full passes."""
    import oracle
    oracle.build()
    og = oracle.OracleGraph.from_synthetic(g)
    threads = os.cpu_count() or 1
    times = []
    for it in range(warmup + steps):
        t0 = time.perf_counter()
        for mp in metapaths:
            og.chain(mp, oracle.MODE_BOOL, threads=threads, export=False)
        dt = time.perf_counter() - t0
        if it >= warmup:
            times.append(dt)
    per_step = sum(times) / len(times)
    return {"value": len(metapaths) / per_step, "unit": "chains/s", "cores": threads, "kind": "port",
            "sample": sample_note, "s_per_pass": per_step}


def run_reference(args):
    ws, rank, _ = dist_env()
    if ws > 1 and rank != 0:
        return
    g = make_graph(args.scale, args.seed)
    mps = select(g.metapaths, args.chains)
    steps, warmup = max(1, args.steps), max(0, args.warmup)
    cb = cpu_reference(g, mps, steps, warmup, f"{len(mps)} full chains per step ({WORKLOAD})")
    line = {"impl": "reference", "metric": "chains/s", "value": cb["value"], "unit": "chains/s", "n_gpus": 0,
            "steps": steps, "warmup": warmup, "ms_per_step": cb["s_per_pass"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bool", "data": "synthetic",
            "config": {"workload": WORKLOAD, "chains": mps},
            "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": cb["value"], "unit": "chains/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "oracle port of efficient/resmcm.cpp (Boolean bitmap Gustavson, OpenMP dynamic schedule); "
                    "the reference's own binary cannot run here (its source is not on this host and compiled "
                    "x86 objects do not travel to it)"}
    print(json.dumps(line), flush=True)


def batched_section(rg, device, seed=2, count=512, walk_cap=1e9, group_bytes=48e9, reps=3, tune=True):
    """Meta-paths of 2-10 matrices drawn by seeded random walks over the
    five-type schema graph at its configured sizes (types of 10k-500k
    vertices, 5-40 edges per row): a walk whose RES-predicted bytes exceed
    ``walk_cap`` is rejected by the estimator (counted) and walks are drawn
    until ``count`` are admitted.  One chain at a time through
    rmcm_run_metapath versus fused batches (estimator levels, DP and one
    block-diagonal SpGEMM per wave for all chains, one CUDA graph each;
    walks grouped so that a group's predicted bytes stay within
    ``group_bytes``), after the autotuner's sweep of the configured
    row-binning tunables on the first group."""
    from resmcm_ari_gb300 import autotune, serve, synth, workloads
    g = workloads.batch_graph(seed=seed, scale=1.0)
    eng = rg.Engine(device=device)
    hg = rg.HeteroGraph.from_synthetic(eng, g)
    paths, preds, drawn, k = [], [], 0, 0
    while len(paths) < count and drawn < 64 * count:
        for mp in synth.random_metapaths(3 + k, g, 256, (2, 10)):
            drawn += 1
            leaves = hg.leaves(mp)
            c = eng.estimate(leaves)
            split, _, _ = eng.order(c)
            dims = [m.shape[0] for m in leaves] + [leaves[-1].shape[1]]
            pb = serve.predicted_bytes(c, split, dims)
            if pb <= walk_cap:
                paths.append(mp)
                preds.append(pb)
                if len(paths) == count:
                    break
        k += 1
    groups, cur, acc = [], [], 0.0
    for mp, pb in zip(paths, preds):
        if cur and acc + pb > group_bytes:
            groups.append(cur)
            cur, acc = [], 0.0
        cur.append(mp)
        acc += pb
    if cur:
        groups.append(cur)
    for mp in paths:                                   # leaves built untimed
        eng.run_metapath(hg, mp, keep=False)
    t0 = time.perf_counter()
    plain = []
    for mp in paths:
        C, _, _ = eng.run_metapath(hg, mp, keep=True)
        plain.append(eng.digest(C))
        C.free()
    plain_s = time.perf_counter() - t0
    out = {"workload": f"five-type schema graph at its configured sizes {g.type_sizes} "
                       f"({sum(r.src.size for r in g.relations)} edges), seeded random-walk meta-paths of 2-10 "
                       f"matrices, uint32 with uint64 escalation",
           "type_sizes": g.type_sizes, "chains": len(paths), "walks_drawn": drawn,
           "rejected_by_estimate": drawn - len(paths), "walk_cap_bytes": walk_cap,
           "groups": len(groups), "predicted_bytes": float(sum(preds)),
           "plain_chains_per_s": len(paths) / plain_s, "result_nnz": int(sum(n for n, _ in plain))}
    if tune and groups:
        t0 = time.perf_counter()
        space = {k_: v for k_, v in autotune.SPACE.items() if k_ != "warp_max_flops"}
        res = autotune.tune(eng, hg, groups[0], reps=2, mode="coordinate", space=space, fused=True)
        out["autotune"] = {"best": res["best"], "best_ms": res["best_s"] * 1e3, "default_ms": res["default_s"] * 1e3,
                           "candidates": len(res["table"]), "group_chains": len(groups[0]),
                           "seconds": time.perf_counter() - t0}
    dev_s, wall_s, launches, nodes, record_s, same = 0.0, 0.0, 0, 0, 0.0, True
    i0 = 0
    for grp in groups:
        t0 = time.perf_counter()
        bt = eng.batch(hg, grp, fused=True)
        record_s += time.perf_counter() - t0
        info = bt.info()
        launches += info["launches_per_run"]
        nodes += info["graph_nodes"]
        walls, devs = [], []
        for _ in range(reps):
            t1 = time.perf_counter()
            nnz, dig, dev = bt.run()
            walls.append(time.perf_counter() - t1)
            devs.append(dev)
            same = same and [(int(a), int(x)) for a, x in zip(nnz, dig)] == plain[i0:i0 + len(grp)]
        wall_s += sorted(walls)[len(walls) // 2]
        dev_s += sorted(devs)[len(devs) // 2]
        bt.free()
        i0 += len(grp)
    out.update({"batched_chains_per_s": len(paths) / wall_s, "speedup_vs_plain": plain_s / wall_s,
                "ms_per_run": wall_s * 1e3, "device_ms_per_run": dev_s * 1e3, "record_s": record_s,
                "graph_nodes": nodes, "gpu_launches_per_run": launches, "identical_results": same,
                "tuning": eng.get_tuning()})
    hg.close()
    eng.close()
    return out


def served_section(rg, eng, hg_retail, g_retail, rates=(10.0, 100.0, 500.0, 2000.0), queries=60, lanes=8,
                   span_s=6.0):
    """Poisson streams of meta-path queries (2-8 matrices, seeded random
    walks, no size filter) over two resident graphs, the A/P/V graph and the
    retail graph, 50/50: plain one query at a time versus the query server
    (admission of RES-predicted bytes against 64 GB; the plain path applies
    the same rule).  At the low rates the stream is cut to ``span_s`` seconds
    of arrivals."""
    from resmcm_ari_gb300 import serve, synth
    budget = 64 << 30
    g0 = synth.dblp_like()
    hg0 = rg.HeteroGraph.from_synthetic(eng, g0)
    cats = [serve.catalog(eng, hg0, g0, 24, seed=1), serve.catalog(eng, hg_retail, g_retail, 24, seed=2)]
    graphs = [hg0, hg_retail]
    admitted = [[serve.admits(eng, graphs[gi], mp, budget) for mp in cat] for gi, cat in enumerate(cats)]
    srv = rg.Server(eng, lanes=lanes, mem_budget_bytes=budget)
    srv.add_graph(hg0)
    srv.add_graph(hg_retail)
    out = {"workload": "Poisson arrivals, 2-8-matrix seeded random-walk meta-paths (24 per graph, no size "
                       "filter) over the A/P/V graph and the retail graph, 50/50; queries whose RES-predicted "
                       "bytes exceed the 64 GB budget are rejected by both paths",
           "budget_bytes": budget, "lanes": lanes,
           "catalog_admitted": [int(sum(a)) for a in admitted], "catalog_size": [len(c) for c in cats],
           "rates": []}
    for rate in rates:
        n = int(min(queries, max(20, rate * span_s)))
        stream = serve.poisson_stream(7, rate, n, cats)
        p = serve.run_plain(eng, graphs, stream, budget=budget)
        s_ = serve.run_served(srv, stream)
        same = all(s_["results"][i] == p["results"][i] for i in range(len(stream)))
        out["rates"].append({"offered_qps": rate, "queries": n,
                             "plain": {k: p[k] for k in ("qps", "p50_ms", "p99_ms", "rejected")},
                             "served": {k: s_[k] for k in ("qps", "p50_ms", "p99_ms", "rejected")},
                             "qps_ratio": s_["qps"] / p["qps"], "identical_results": same})
    st = srv.stats()
    out["peak_reserved_bytes"] = st["peak_reserved"]
    out["max_running"] = st["max_running"]
    srv.close()
    hg0.close()
    return out


def stress_plan(rg, device, g, mp, capacity):
    """RES estimates, DP order and the memory plan of the stress chain on
    graph g, from leaves built straight from the relations (no run)."""
    from resmcm_ari_gb300 import workloads
    eng = rg.Engine(device=device, valtype=rg.VAL_U64)
    cache, leaves = {}, []
    for rel, fw in workloads.STRESS_LEAVES:
        if (rel, fw) not in cache:
            rp, col = workloads.relation_csr(g, rel, fw)
            r = g.relations[rel]
            cols = g.type_sizes[r.dst_type if fw else r.src_type]
            cache[(rel, fw)] = eng.upload(rp, col, cols=cols, valtype=rg.VAL_U64)
        leaves.append(cache[(rel, fw)])
    c = eng.estimate(leaves)
    split, _, pairs = eng.order(c)
    dims = [m.shape[0] for m in leaves] + [leaves[-1].shape[1]]
    leaf_bytes = [m.nnz * 12 + (m.shape[0] + 1) * 8 for m in cache.values()]
    plan = workloads.chain_plan(c, split, dims, leaf_bytes)
    l2r = [float(c[0, j]) for j in range(1, c.shape[0])]
    for m in cache.values():
        m.free()
    eng.close()
    # the final product can run in blocks of rows (rmcm_run_metapath_blocks):
    # then its output need not be whole, but its operands must be
    fin = plan["products"][-1]
    live_wo_final = max([n["live_bytes"] for n in plan["products"][:-1]] + [fin["live_bytes"] - fin["bytes"]])
    return {"order_pairs": pairs.tolist(),
            "products": [{k: (round(v) if isinstance(v, float) else v) for k, v in n.items()}
                         for n in plan["products"]],
            "largest_intermediate_est_nnz": plan["largest_intermediate_nnz"], "result_est_nnz": plan["result_nnz"],
            "peak_live_bytes": plan["peak_live_bytes"], "peak_at_product": plan["peak_at"],
            "peak_live_bytes_final_in_blocks": live_wo_final, "device_bytes": capacity,
            "fits_whole": plan["peak_live_bytes"] <= capacity, "fits_final_in_blocks": live_wo_final <= capacity,
            "left_to_right_largest_est_nnz": max(l2r)}


def stress_section(rg, device, scale=0.1):
    """The twelve-matrix uint64 chain Z-Y-X-Y-X-Y-Z-Y-X-Y-X-Y-Z over the X/Y/Z
    graph (both-side Zipf(1.6) X-Y degrees): at the configured size (X = Y =
    5M, Z = 100k, 60M X-Y edges) its RES estimates and memory plan decide
    whether it can run on this GPU at all; the chain is run, timed, at vertex
    and edge counts x``scale``."""
    import torch
    from resmcm_ari_gb300 import workloads
    capacity = torch.cuda.mem_get_info(device)[1]
    mp = workloads.STRESS_CHAIN
    t0 = time.perf_counter()
    full = workloads.stress_graph()
    full_plan = stress_plan(rg, device, full, mp, capacity)
    full_plan["seconds"] = time.perf_counter() - t0
    full_plan["workload"] = (f"X=Y={full.type_sizes[0]}, Z={full.type_sizes[2]}, X-Y {full.relations[0].src.size} "
                             f"edges, Y-Z {full.relations[1].src.size} edges")
    del full
    g = workloads.stress_scaled(scale)
    eng = rg.Engine(device=device, valtype=rg.VAL_U64)
    hg = rg.HeteroGraph.from_synthetic(eng, g)
    leaves = hg.leaves(mp, rg.VAL_U64)
    c = eng.estimate(leaves)
    split, _, _ = eng.order(c)
    L = c.shape[0]
    inter = []

    def walk(i, j):
        if i != j:
            k = int(split[i, j])
            walk(i, k)
            walk(k + 1, j)
            inter.append(float(c[i, j]))

    walk(0, L - 1)
    eng.mem_peak(reset=True)
    C, t, rc = eng.run_metapath(hg, mp, keep=True)
    peak = eng.mem_peak()
    out = {"workload": f"X=Y={g.type_sizes[0]}, Z={g.type_sizes[2]}, X-Y {g.relations[0].src.size} edges "
                       f"(both-side Zipf 1.6), Y-Z 1-4 per Y; chain {mp} (12 matrices), uint64 with overflow check",
           "scale": scale, "status": int(rc), "result_nnz": int(C.nnz), "seconds": t["total_s"],
           "spgemm_s": t["spgemm_s"], "multiply_adds": int(t["flops"]),
           "multiply_adds_per_s": t["flops"] / t["total_s"] if t["total_s"] else None,
           "peak_device_bytes": int(peak),
           "est_largest_intermediate_nnz": {"res_order": max(inter), "left_to_right": max(c[0, j] for j in range(1, L))},
           "configured_size_plan": full_plan}
    C.free()
    hg.close()
    eng.close()
    return out


def parity_section(eng, hg, g, mps, rg, threads=None):
    """Results of the timed workload against the CPU oracle, after the timed
    region: per chain the GPU result's nnz and order-free digest (structure
    and exact path counts, rmcm_mat_digest) against the counting oracle's,
    the estimates within 1e-9 relative of the oracle's one-thread sums, and
    the multiplication order against the oracle's.  Where the reference's own
    result sizes for this graph are on disk (the fixture made by the
    reference), the nnz is checked against them too."""
    import oracle
    oracle.build()
    t0 = time.perf_counter()
    og = oracle.OracleGraph.from_synthetic(g)
    threads = threads or os.cpu_count() or 1
    ref_nnz = {}
    fx = os.path.join(ROOT, "tests", "golden", "retail_full.json")
    if os.path.exists(fx) and g.name == "retail_like_u1000000_i300000_c2000_t20000_s1":
        with open(fx) as f:
            ref_nnz = {r["metapath"]: int(r["nnz"]) for r in json.load(f)["paths"]}
    chains, ok = [], True
    for mp in mps:
        C, _, rc = eng.run_metapath(hg, mp, keep=True)
        n_gpu, d_gpu = eng.digest(C)
        C.free()
        r = og.chain(mp, oracle.MODE_COUNT, threads=threads, export=False, digest=True)
        leaves = hg.leaves(mp, rg.VAL_U32)
        c_gpu = eng.estimate(leaves)
        c_orc = og.estimate(mp, threads=1)
        nz = c_orc != 0
        rel = float((np.abs(c_gpu[nz] - c_orc[nz]) / np.abs(c_orc[nz])).max(initial=0.0))
        est_ok = bool(np.array_equal(c_gpu[~nz], c_orc[~nz]) and rel <= 1e-9)
        _, _, pairs_gpu = eng.order(c_gpu)
        _, _, pairs_orc = oracle.dp(c_orc)
        rec = {"metapath": mp, "nnz": int(n_gpu), "nnz_equal": int(n_gpu) == int(r.nnz),
               "digest_equal": int(d_gpu) == int(r.digest) and r.status == oracle.ORC_OK,
               "estimates_max_rel_err": rel, "estimates_ok": est_ok,
               "order_equal": bool(np.array_equal(np.asarray(pairs_gpu).reshape(-1),
                                                  np.asarray(pairs_orc).reshape(-1)))}
        if mp in ref_nnz:
            rec["reference_nnz_equal"] = int(n_gpu) == ref_nnz[mp]
        ok = ok and rec["nnz_equal"] and rec["digest_equal"] and est_ok and rec["order_equal"] and \
            rec.get("reference_nnz_equal", True)
        chains.append(rec)
    og.close()
    return {"ok": bool(ok), "against": "counting oracle (exact uint64 path counts, oracle/oracle.c) on the "
                                      "same graph; nnz also against the reference's own results where its "
                                      "fixture covers the graph",
            "oracle_threads": threads, "seconds": time.perf_counter() - t0, "chains": chains}


def guarded(name, fn, *a, **kw):
    """Run an optional section; a failure becomes an error field in the line
    instead of ending the benchmark."""
    try:
        return fn(*a, **kw)
    except Exception as e:  # noqa: BLE001 -- reported, not swallowed
        import traceback
        traceback.print_exc(file=sys.stderr)
        return {"error": f"{name}: {type(e).__name__}: {e}"}


def select(mps, spec):
    if spec == "all":
        return list(mps)
    return [mps[int(i)] for i in spec.split(",")]


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    import resmcm_ari_gb300 as rg

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    rg.build()
    g = make_graph(args.scale, args.seed)
    mps = select(g.metapaths, args.chains)

    stream = torch.cuda.current_stream()
    eng = rg.Engine(device=local, valtype=rg.VAL_AUTO, stream=stream.cuda_stream)
    if args.tune:
        eng.set_tuning(**{k: float(v) if "." in v else int(v) for k, v in (t.split("=", 1) for t in args.tune)})
    hg = rg.HeteroGraph.from_synthetic(eng, g)
    leaves = {mp: hg.leaves(mp, rg.VAL_U32) for mp in mps}
    # uint64 leaves too (used when a chain escalates on overflow), built untimed
    for mp in mps:
        hg.leaves(mp, rg.VAL_U64)

    def step():
        nnz = 0
        for mp in mps:
            C, t, _ = eng.run_metapath(hg, mp, keep=True)
            nnz += C.nnz
            C.free()
        return nnz

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # warm-up: the first pass collects the algorithmic bytes of every product
    eng.set_profiling(2)
    step_nnz = step()
    bytes_stats = eng.product_stats(reset=True)
    eng.set_profiling(1)
    for _ in range(max(0, args.warmup - 1)):
        step()
    eng.product_stats(reset=True)

    clocks = rg_clock = ClockSampler(local)
    if not args.no_clocks:
        rg_clock.start()
    launches0 = eng.kernel_launches
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    elapsed_ms = ev0.elapsed_time(ev1)
    launches = eng.kernel_launches - launches0
    clk = rg_clock.stop() if not args.no_clocks else None
    timed_stats = eng.product_stats(reset=True)
    eng.set_profiling(0)
    elapsed_ms = max_over_ranks(elapsed_ms, ws)
    ms_per_step = elapsed_ms / args.steps
    value = replica_value(len(mps), ws, ms_per_step / 1e3)

    # roofline of the dominant SpGEMM product: bytes from the first pass, event
    # times of all its passes (analysis, symbolic, numeric) from the timed region
    nprod = len(bytes_stats)
    per_prod_ms = [[] for _ in range(nprod)]
    for i, st in enumerate(timed_stats):
        per_prod_ms[i % nprod].append(st["analyze_ms"] + st["symbolic_ms"] + st["numeric_ms"])
    avg_ms = [sum(x) / len(x) if x else 0.0 for x in per_prod_ms]
    dom = int(np.argmax(avg_ms)) if nprod else 0
    peak, peak_kind = peak_hbm()
    roof = None
    if nprod:
        b = bytes_stats[dom]
        alg = b["bytes_a"] + b["bytes_b_touched"] + b["bytes_c"]
        achieved = alg / (avg_ms[dom] / 1e3) / 1e9
        tr = traffic_from_profiles()
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_kind": f"of {peak_kind}",
                "traffic": (alg * tr["bytes_per_alg_byte"]) if tr else None,
                "kernel": "SpGEMM product with the largest time per step (all its passes)",
                "product": {k: b[k] for k in ("rows", "inner", "cols", "nnz_a", "nnz_c", "flops", "bin_rows",
                                              "gemm_inner", "gemm_limbs")},
                "algorithmic_bytes": alg, "launch_ms": avg_ms[dom],
                "multiply_adds_per_s": b["flops"] / (avg_ms[dom] / 1e3),
                "sparse_kernel_bound": sparse_bound_from_profiles()}
        # the tensor-core part (exact FP16 GEMM of the heavy inner indices):
        # the product with the most dense multiply-adds, and every GEMM
        gemm_ms = [0.0] * nprod
        for i, st in enumerate(timed_stats):
            gemm_ms[i % nprod] += st["gemm_ms"] / max(1, len(per_prod_ms[i % nprod]))
        macs_of = [b_["rows"] * b_["gemm_inner"] * b_["cols"] * b_["gemm_limbs"] for b_ in timed_stats[:nprod]]
        gi = int(np.argmax(macs_of)) if nprod else 0
        if nprod and gemm_ms[gi] > 0:
            gb = timed_stats[gi]
            macs = macs_of[gi]
            tf = 2.0 * macs / (gemm_ms[gi] / 1e3) / 1e12
            tpeak, tkind = peak_tensor()
            roof["tensor_part"] = {"bound": "tensor", "achieved": tf, "peak": tpeak, "unit": "TFLOP/s",
                                   "frac": tf / tpeak, "peak_kind": f"of {tkind} bf16 burst",
                                   "all_gemms": [{"rows": timed_stats[i]["rows"], "cols": timed_stats[i]["cols"],
                                                  "gemm_inner": timed_stats[i]["gemm_inner"],
                                                  "gemm_limbs": timed_stats[i]["gemm_limbs"], "ms": gemm_ms[i],
                                                  "tflops": 2.0 * macs_of[i] / (gemm_ms[i] / 1e3) / 1e12}
                                                 for i in range(nprod) if gemm_ms[i] > 0],
                                   "kernel": "k_tc_seed: tcgen05 FP16 GEMM (FP32 accumulation in TMEM, TMA-fed, "
                                             "limbs combined into integer seeds) of the heavy inner indices",
                                   "product": {k: gb[k] for k in ("rows", "inner", "cols", "gemm_inner",
                                                                   "gemm_limbs")},
                                   "dense_multiply_adds": macs, "gemm_ms": gemm_ms[gi]}
        tot_alg = sum(s_["bytes_a"] + s_["bytes_b_touched"] + s_["bytes_c"] for s_ in bytes_stats)
        tot_ms = sum(avg_ms)
        roof["all_products"] = {"achieved": tot_alg / (tot_ms / 1e3) / 1e9, "ms_per_step": tot_ms,
                                "frac": tot_alg / (tot_ms / 1e3) / 1e9 / peak}

    if args.detail and rank == 0:
        for i, b in enumerate(bytes_stats):
            row = {k: b[k] for k in ("rows", "inner", "cols", "nnz_a", "nnz_b", "nnz_c", "flops", "bin_rows",
                                      "valtype", "touched_rows", "touched_nnz", "gemm_inner", "gemm_limbs")}
            reps = [st for j, st in enumerate(timed_stats) if j % nprod == i]
            for key in ("analyze_ms", "symbolic_ms", "numeric_ms"):
                row[key] = sum(st[key] for st in reps) / max(1, len(reps))
            alg = b["bytes_a"] + b["bytes_b_touched"] + b["bytes_c"]
            row["alg_bytes"] = alg
            row["numeric_gbs"] = alg / (row["numeric_ms"] / 1e3) / 1e9 if row["numeric_ms"] else None
            row["gflops_numeric"] = b["flops"] / (row["numeric_ms"] / 1e3) / 1e9 if row["numeric_ms"] else None
            print("PRODUCT " + json.dumps(row), file=sys.stderr, flush=True)

    # end to end through the C ABI from pinned host buffers
    e2e = None
    if not args.no_e2e:
        host = {}
        h2d = 0
        for mp in mps:
            mats = []
            for L in leaves[mp]:
                rp, col, val = L.download(values=False)
                rows, cols = L.shape
                trp = torch.from_numpy(rp).pin_memory()
                tcol = torch.from_numpy(col).pin_memory()
                mats.append((trp, tcol, cols))
                h2d += rp.nbytes + col.nbytes
            host[mp] = mats
        # result buffers (pinned) sized from the device run
        res_rows = {}
        for mp in mps:
            C, _, _ = eng.run_metapath(hg, mp)
            res_rows[mp] = (C.shape[0], C.nnz, C.valtype)
            C.free()
        d2h = 0
        outbuf = {}
        for mp, (rows, nnz, vt) in res_rows.items():
            outbuf[mp] = (torch.empty(rows + 1, dtype=torch.int64, pin_memory=True),
                          torch.empty(max(nnz, 1), dtype=torch.int32, pin_memory=True),
                          torch.empty(max(nnz, 1), dtype=torch.int64 if vt == rg.VAL_U64 else torch.int32,
                                      pin_memory=True))
            d2h += (rows + 1) * 8 + nnz * 4 + nnz * (8 if vt == rg.VAL_U64 else 4)

        # a loader handle uploads (and validates) the next chain's leaves on a
        # helper thread while this one multiplies the current chain
        loader = rg.Engine(device=local, valtype=rg.VAL_AUTO)
        from concurrent.futures import ThreadPoolExecutor
        pool = ThreadPoolExecutor(max_workers=1)

        def upload(mp):
            mats = [loader.upload_ptr(trp.data_ptr(), tcol.data_ptr(), trp.numel() - 1, cols)
                    for trp, tcol, cols in host[mp]]
            loader.synchronize()
            return mats

        def e2e_step():
            # a chain's result travels to the host on the transfer stream while
            # the next chain's leaves are uploaded and multiplied
            fut = pool.submit(upload, mps[0])
            for i, mp in enumerate(mps):
                mats = fut.result()
                if i + 1 < len(mps):
                    fut = pool.submit(upload, mps[i + 1])
                Cm, _, _ = eng.chain(mats)
                rp_b, col_b, val_b = outbuf[mp]
                eng.download_async(Cm, rp_b.data_ptr(), col_b.data_ptr(), val_b.data_ptr())
                Cm.free()
                done.append(mats)
            eng.transfers_wait()
            for mats in done:
                for m in mats:
                    m.free()
            done.clear()

        done = []

        for _ in range(max(1, min(args.warmup, 2))):
            e2e_step()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        barrier()
        e2e_s = (time.perf_counter() - t0) / args.steps
        e2e_s = max_over_ranks(e2e_s, ws)
        pool.shutdown()
        loader.close()
        e2e = {"value": replica_value(len(mps), ws, e2e_s), "unit": "chains/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "ms_per_step": e2e_s * 1e3}

    parity = batched = served = stress = None
    if rank == 0 and not args.no_parity:
        parity = guarded("parity", parity_section, eng, hg, g, mps, rg)
    if rank == 0 and not args.no_batched:
        batched = guarded("batched", batched_section, rg, local)
    if rank == 0 and not args.no_served:
        served = guarded("served", served_section, rg, eng, hg, g)
    if rank == 0 and not args.no_stress:
        stress = guarded("stress", stress_section, rg, local)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = guarded("cpu_baseline", cpu_reference, g, mps, 2, 1,
                      f"two full passes over the {len(mps)} chains after one warm-up pass ({WORKLOAD})")
        cpu.pop("s_per_pass", None)

    if rank == 0:
        line = {
            "metric": "chains/s", "value": value, "unit": "chains/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": WORKLOAD if args.scale == 1.0 else f"{WORKLOAD} (scaled x{args.scale:g})",
                       "chains": mps, "values": "uint32 path counts, uint64 from the first overflowing product; "
                                                "estimator and DP in FP64",
                       "l2": "inputs larger than L2 (leaf CSRs %.0f MB, results %.0f MB per step)" % (
                           sum(L.nnz * 8 + (L.shape[0] + 1) * 8 for mp in mps for L in leaves[mp]) / 1e6,
                           step_nnz * 8 / 1e6),
                       "parallelism": f"replicas x{ws}"},
            "nnz_per_s": step_nnz * ws / (ms_per_step / 1e3),
            "result_nnz_per_step": step_nnz,
            "e2e": e2e, "roofline": roof, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches,
            "parity": parity, "batched": batched, "served": served, "stress": stress,
        }
        print(json.dumps(line), flush=True)
    hg.close()
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
