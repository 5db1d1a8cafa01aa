"""Seeded synthetic heterogeneous information networks (HINs).

The published RESMCM datasets (DBLP, IMDB, FourSquare) are not redistributable
here, so every workload is a seeded synthetic graph with the shapes, sizes and
degree distributions of the measured configurations.  A graph is produced in
the reference's in-memory form (typed vertices, typed directed adjacency) and
can be written in the reference's three text files:

* ``vertex.txt``: ``vid vt`` per line (``DataReader::readVertexType``,
  efficient/resmcm.cpp:115-135);
* ``edge.txt``: ``eid et`` per line (``DataReader::readEdgeType``,
  efficient/resmcm.cpp:137-176);
* ``graph.txt``: ``vid (nbr eid)*`` per line (``DataReader::readGraph``,
  efficient/resmcm.cpp:86-113).

Every undirected relation becomes two directed edge types (explicit
transposes).  Vertex ids are contiguous per type.  Each directed adjacency
entry has its own edge id, numbered in ``graph.txt`` order.

Determinism: numpy's ``PCG64`` generator is platform independent, so the same
seed yields byte-identical graphs on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np


# --------------------------------------------------------------------------
# sampling helpers
# --------------------------------------------------------------------------

def zipf_cdf(k: int, s: float) -> np.ndarray:
    """Cumulative distribution of a Zipf(s) law truncated to ranks 1..k."""
    w = np.arange(1, k + 1, dtype=np.float64) ** (-s)
    c = np.cumsum(w)
    return c / c[-1]


def zipf_ranks(rng: np.random.Generator, k: int, s: float, size) -> np.ndarray:
    """Draw 0-based ranks from a truncated Zipf(s) law over k items."""
    cdf = zipf_cdf(k, s)
    u = rng.random(size)
    r = np.searchsorted(cdf, u, side="right")
    return np.minimum(r, k - 1).astype(np.int64)


def zipf_truncation_for_mean(s: float, mean: float, kmax: int) -> int:
    """Smallest support size K (≤ kmax) whose truncated Zipf(s) mean reaches ``mean``."""
    lo, hi = 1, kmax
    k = np.arange(1, kmax + 1, dtype=np.float64)
    w = k ** (-s)
    cw = np.cumsum(w)
    ckw = np.cumsum(k * w)
    while lo < hi:
        mid = (lo + hi) // 2
        if ckw[mid - 1] / cw[mid - 1] >= mean:
            hi = mid
        else:
            lo = mid + 1
    return lo


def sorted_unique(key: np.ndarray) -> np.ndarray:
    """Sorted distinct values of an int64 array (sort based; numpy's hash unique is slow)."""
    k = np.sort(key)
    if k.size == 0:
        return k
    keep = np.empty(k.size, bool)
    keep[0] = True
    np.not_equal(k[1:], k[:-1], out=keep[1:])
    return k[keep]


def dedup_pairs_keep_order(src: np.ndarray, dst: np.ndarray, ncols: int):
    """Drop repeated (src, dst) pairs, keeping first occurrences in draw order."""
    key = src.astype(np.int64) * np.int64(ncols) + dst.astype(np.int64)
    order = np.argsort(key, kind="stable")
    k = key[order]
    keep = np.ones(k.size, bool)
    if k.size:
        keep[1:] = k[1:] != k[:-1]
    first = np.sort(order[keep])
    return src[first], dst[first]


# --------------------------------------------------------------------------
# graph container
# --------------------------------------------------------------------------

@dataclass
class Relation:
    """One undirected relation between two vertex types.

    ``src``/``dst`` hold local ids in generation order; ``et_fwd`` labels the
    src→dst direction and ``et_rev`` the dst→src one.
    """
    src_type: int
    dst_type: int
    et_fwd: int
    et_rev: int
    src: np.ndarray
    dst: np.ndarray


@dataclass
class SyntheticHIN:
    name: str
    type_sizes: list
    relations: list = field(default_factory=list)
    metapaths: list = field(default_factory=list)
    _adj: tuple = None

    @property
    def n(self) -> int:
        return int(sum(self.type_sizes))

    @property
    def type_offsets(self) -> np.ndarray:
        return np.concatenate([[0], np.cumsum(self.type_sizes)]).astype(np.int64)

    def vertex_types(self) -> np.ndarray:
        return np.repeat(np.arange(len(self.type_sizes), dtype=np.int32),
                         self.type_sizes)

    def adjacency(self):
        """Global typed adjacency in ``graph.txt`` order.

        Returns ``(ptr int64[n+1], nbr int32[m], et int32[m])``.  A vertex's
        entries follow relation order; within a relation the forward entries
        come in generation order and the reverse entries in the order their
        forward edges were generated.
        """
        if self._adj is not None:
            return self._adj
        off = self.type_offsets
        srcs, dsts, ets = [], [], []
        for r in self.relations:
            gs = r.src.astype(np.int64) + off[r.src_type]
            gd = r.dst.astype(np.int64) + off[r.dst_type]
            srcs += [gs, gd]
            dsts += [gd, gs]
            ets += [np.full(gs.size, r.et_fwd, np.int32),
                    np.full(gd.size, r.et_rev, np.int32)]
        if srcs:
            s = np.concatenate(srcs)
            d = np.concatenate(dsts)
            e = np.concatenate(ets)
        else:
            s = np.zeros(0, np.int64); d = np.zeros(0, np.int64); e = np.zeros(0, np.int32)
        order = np.argsort(s, kind="stable")
        s, d, e = s[order], d[order], e[order]
        ptr = np.zeros(self.n + 1, np.int64)
        np.cumsum(np.bincount(s, minlength=self.n), out=ptr[1:])
        self._adj = (ptr, d.astype(np.int32), e.astype(np.int32))
        return self._adj

    @property
    def m(self) -> int:
        return int(self.adjacency()[0][-1])

    def write_text(self, directory: str, metapaths=None) -> dict:
        """Write vertex.txt, edge.txt, graph.txt (and metapaths.txt) in the reference format."""
        os.makedirs(directory, exist_ok=True)
        ptr, nbr, et = self.adjacency()
        n, m = self.n, int(ptr[-1])
        vt = self.vertex_types()
        paths = {k: os.path.join(directory, k + ".txt")
                 for k in ("vertex", "edge", "graph", "metapaths")}
        with open(paths["vertex"], "w") as f:
            f.write("".join(f"{v} {t}\n" for v, t in zip(range(n), vt.tolist())))
        with open(paths["edge"], "w") as f:
            f.write("".join(f"{e} {t}\n" for e, t in zip(range(m), et.tolist())))
        eid = np.arange(m, dtype=np.int64)
        nb = nbr.tolist()
        ei = eid.tolist()
        p = ptr.tolist()
        with open(paths["graph"], "w") as f:
            lines = []
            for v in range(n):
                a, b = p[v], p[v + 1]
                parts = [str(v)]
                for q in range(a, b):
                    parts.append(f"{nb[q]} {ei[q]}")
                lines.append(" ".join(parts) + "\n")
            f.write("".join(lines))
        mps = self.metapaths if metapaths is None else metapaths
        with open(paths["metapaths"], "w") as f:
            f.write("".join(mp + "\n" for mp in mps))
        return paths


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------

def tiny_dblp() -> SyntheticHIN:
    """Hand-checkable 8-vertex P/A/V graph (types P=0, A=1, V=2).

    Edge types follow the DBLP schema of tool/generate_DBLP.cpp:329-358:
    P→A 0, P→V 1, A→P 3, V→P 4.
    """
    g = SyntheticHIN("tiny_dblp", [4, 3, 1])
    # papers 0..3, authors 0..2, venue 0
    pa_src = np.array([0, 0, 1, 2, 2, 3], np.int64)
    pa_dst = np.array([0, 1, 1, 0, 2, 2], np.int64)
    pv_src = np.array([0, 1, 2, 3], np.int64)
    pv_dst = np.array([0, 0, 0, 0], np.int64)
    g.relations = [Relation(0, 1, 0, 3, pa_src, pa_dst),
                   Relation(0, 2, 1, 4, pv_src, pv_dst)]
    g.metapaths = ["1-3-0-0-1", "1-3-0-1-2-4-0-0-1", "0-0-1-3-0-0-1-3-0",
                   "2-4-0-0-1-3-0-1-2", "0-1-2"]
    return g


def dblp_like(n_a=30_000, n_p=60_000, n_v=50, seed=0, authors=(1, 5),
              s_author=1.1, s_venue=1.2) -> SyntheticHIN:
    """Three-type P/A/V graph of the small plain single-chain workload.

    Each paper draws its author count uniformly from ``authors`` and chooses
    the authors by Zipf(``s_author``) over A (repeats dropped); each paper
    has exactly one venue drawn by Zipf(``s_venue``).  Types: P=0, A=1, V=2.
    Chain A-P-V-P-A is ``1-3-0-1-2-4-0-0-1``.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    perm_a = rng.permutation(n_a)
    perm_v = rng.permutation(n_v)
    lo, hi = authors
    cnt = rng.integers(lo, hi + 1, size=n_p)
    draws = perm_a[zipf_ranks(rng, n_a, s_author, (n_p, hi))]
    keep = np.arange(hi)[None, :] < cnt[:, None]
    for c in range(1, hi):                      # drop repeats within a paper
        dup = (draws[:, :c] == draws[:, c:c + 1]).any(axis=1)
        keep[:, c] &= ~dup
    pa_src = np.repeat(np.arange(n_p, dtype=np.int64), hi).reshape(n_p, hi)[keep]
    pa_dst = draws[keep].astype(np.int64)
    pv_src = np.arange(n_p, dtype=np.int64)
    pv_dst = perm_v[zipf_ranks(rng, n_v, s_venue, n_p)].astype(np.int64)
    g = SyntheticHIN(f"dblp_like_a{n_a}_p{n_p}_v{n_v}_s{seed}", [n_p, n_a, n_v])
    g.relations = [Relation(0, 1, 0, 3, pa_src, pa_dst),
                   Relation(0, 2, 1, 4, pv_src, pv_dst)]
    g.metapaths = ["1-3-0-1-2-4-0-0-1"]
    return g


def chung_lu(rng: np.random.Generator, n_a: int, n_b: int, edges: int, s_a: float, s_b: float):
    """Bipartite edges with Zipf degree laws on both sides (Chung–Lu style).

    Side A gets i.i.d. degrees from Zipf(``s_a``) truncated so that the mean
    is ``edges / n_a``; side B gets weights from Zipf(``s_b``) truncated to
    mean ``edges / n_b``.  Each A stub picks a B endpoint with probability
    proportional to its weight.  Repeated pairs are dropped and topped up
    with fresh draws until exactly ``edges`` distinct pairs remain (or the
    draws stop adding pairs).  Pairs come back sorted by (a, b).
    """
    ka = zipf_truncation_for_mean(s_a, edges / n_a, max(2, n_b))
    kb = zipf_truncation_for_mean(s_b, edges / n_b, max(2, n_a))
    deg_a = zipf_ranks(rng, ka, s_a, n_a) + 1
    w_b = (zipf_ranks(rng, kb, s_b, n_b) + 1).astype(np.float64)
    cdf_b = np.cumsum(w_b)
    cdf_b /= cdf_b[-1]
    cdf_a = np.cumsum(deg_a.astype(np.float64))
    cdf_a /= cdf_a[-1]

    def draw_b(size):
        return np.minimum(np.searchsorted(cdf_b, rng.random(size), side="right"), n_b - 1)

    a = np.repeat(np.arange(n_a, dtype=np.int64), deg_a)
    key = sorted_unique(a * np.int64(n_b) + draw_b(a.size))
    for _ in range(8):
        short = edges - key.size
        if short <= 0:
            break
        extra = int(short * 1.2) + 16
        ea = np.minimum(np.searchsorted(cdf_a, rng.random(extra), side="right"), n_a - 1)
        grown = sorted_unique(np.concatenate([key, ea.astype(np.int64) * np.int64(n_b) + draw_b(extra)]))
        if grown.size == key.size:
            break
        key = grown
    if key.size > edges:
        key = np.sort(rng.choice(key, size=edges, replace=False))
    return key // n_b, key % n_b


def retail_like(n_u=1_000_000, n_i=300_000, n_c=2_000, n_t=20_000, ui_edges=20_000_000,
                seed=1, s_user=1.7, s_item=1.3, s_cat=1.1, tags=(5, 15)) -> SyntheticHIN:
    """Four-type U/I/C/T graph of the plain-at-scale workload.

    Types U=0, I=1, C=2, T=3.  Edge types U→I 0, I→U 1, I→C 2, C→I 3,
    I→T 4, T→I 5.  U–I has ``ui_edges`` distinct edges with user degrees
    Zipf(``s_user``) and item popularity Zipf(``s_item``) (``chung_lu``).
    Each item has one category by Zipf(``s_cat``) and a uniform 5–15
    distinct tags.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    perm_u = rng.permutation(n_u)
    perm_i = rng.permutation(n_i)
    perm_c = rng.permutation(n_c)
    ui_src, ui_dst = chung_lu(rng, n_u, n_i, ui_edges, s_user, s_item)
    ui_src, ui_dst = perm_u[ui_src], perm_i[ui_dst]
    order = np.lexsort((ui_dst, ui_src))
    ui_src, ui_dst = ui_src[order].astype(np.int64), ui_dst[order].astype(np.int64)
    ic_src = np.arange(n_i, dtype=np.int64)
    ic_dst = perm_c[zipf_ranks(rng, n_c, s_cat, n_i)].astype(np.int64)
    lo, hi = tags
    tcnt = rng.integers(lo, hi + 1, size=n_i)
    tsrc = np.repeat(np.arange(n_i, dtype=np.int64), tcnt)
    tdst = rng.integers(0, n_t, size=tsrc.size).astype(np.int64)
    it_src, it_dst = dedup_pairs_keep_order(tsrc, tdst, n_t)
    g = SyntheticHIN(f"retail_like_u{n_u}_i{n_i}_c{n_c}_t{n_t}_s{seed}", [n_u, n_i, n_c, n_t])
    g.relations = [Relation(0, 1, 0, 1, ui_src, ui_dst),
                   Relation(1, 2, 2, 3, ic_src, ic_dst),
                   Relation(1, 3, 4, 5, it_src, it_dst)]
    g.metapaths = ["1-4-3-5-1-2-2",            # I-T-I-C
                   "2-3-1-1-0-0-1-2-2",        # C-I-U-I-C
                   "3-5-1-2-2-3-1-4-3",        # T-I-C-I-T
                   "2-3-1-4-3-5-1-1-0-0-1-2-2"]  # C-I-T-I-U-I-C
    return g


def random_hin(seed: int, type_sizes, relations, mean_deg=(2, 6), s_range=(1.3, 2.0)):
    """Generic seeded HIN: ``relations`` is a list of (src_type, dst_type).

    Each relation gives the src side a Zipf(s) degree (s drawn from
    ``s_range``) and picks dst vertices by Zipf(s) popularity.  Edge types
    are numbered 2r (forward) and 2r+1 (reverse).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    g = SyntheticHIN(f"random_hin_s{seed}", list(type_sizes))
    for r, (a, b) in enumerate(relations):
        na, nb = type_sizes[a], type_sizes[b]
        s = float(rng.uniform(*s_range))
        md = float(rng.uniform(*mean_deg))
        k = zipf_truncation_for_mean(s, md, max(2, nb))
        deg = zipf_ranks(rng, k, s, na) + 1
        src = np.repeat(rng.permutation(na).astype(np.int64), deg)
        dst = rng.permutation(nb)[zipf_ranks(rng, nb, s, src.size)].astype(np.int64)
        src, dst = dedup_pairs_keep_order(src, dst, nb)
        g.relations.append(Relation(a, b, 2 * r, 2 * r + 1, src, dst))
    return g


def random_metapaths(seed: int, g: SyntheticHIN, count: int, lengths=(2, 6)):
    """Seeded random walks over the schema graph of ``g`` → meta-path strings."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nbrs = {}
    for r in g.relations:
        nbrs.setdefault(r.src_type, []).append((r.et_fwd, r.dst_type))
        nbrs.setdefault(r.dst_type, []).append((r.et_rev, r.src_type))
    starts = sorted(nbrs)
    out = []
    for _ in range(count):
        L = int(rng.integers(lengths[0], lengths[1] + 1))
        t = starts[int(rng.integers(len(starts)))]
        parts = [str(t)]
        for _ in range(L):
            et, t2 = nbrs[t][int(rng.integers(len(nbrs[t])))]
            parts += [str(et), str(t2)]
            t = t2
        out.append("-".join(parts))
    return out
