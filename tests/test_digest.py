"""The order-free result digest (rmcm_mat_digest, csr_digest) on the host:
its definition restated with Python integers, and its independence of the
entry order."""
import numpy as np

from resmcm_ari_gb300 import csr_digest

M64 = (1 << 64) - 1


def mix(x: int) -> int:
    x ^= x >> 30
    x = (x * 0xBF58476D1CE4E5B9) & M64
    x ^= x >> 27
    x = (x * 0x94D049BB133111EB) & M64
    return x ^ (x >> 31)


def slow_digest(rowptr, col, val):
    acc = 0
    for r in range(len(rowptr) - 1):
        for e in range(rowptr[r], rowptr[r + 1]):
            acc = (acc + mix((mix((r << 32) | int(col[e])) + int(val[e])) & M64)) & M64
    return acc


def test_digest_matches_its_definition():
    rng = np.random.default_rng(5)
    rowptr = np.concatenate([[0], np.cumsum(rng.integers(0, 6, 40))]).astype(np.int64)
    nnz = int(rowptr[-1])
    col = rng.integers(0, 1 << 31, nnz).astype(np.int32)
    val = rng.integers(1, 1 << 63, nnz, dtype=np.uint64)
    n, d = csr_digest(rowptr, col, val)
    assert n == nnz and d == slow_digest(rowptr, col, val)
    # values omitted count as ones
    assert csr_digest(rowptr, col)[1] == slow_digest(rowptr, col, np.ones(nnz, np.uint64))


def test_digest_ignores_entry_order_but_not_values():
    rowptr = np.array([0, 3, 5], np.int64)
    col = np.array([4, 1, 9, 2, 0], np.int32)
    val = np.array([1, 2, 3, 4, 5], np.uint64)
    perm_col = np.array([9, 4, 1, 0, 2], np.int32)
    perm_val = np.array([3, 1, 2, 5, 4], np.uint64)
    assert csr_digest(rowptr, col, val) == csr_digest(rowptr, perm_col, perm_val)
    val2 = val.copy()
    val2[0] += 1
    assert csr_digest(rowptr, col, val) != csr_digest(rowptr, col, val2)
    assert csr_digest(np.array([0], np.int64), np.zeros(0, np.int32)) == (0, 0)


def test_oracle_digest_equals_the_host_digest_of_its_export(oracle_mod):
    """The oracle's C digest (used at full workload sizes, where exporting
    the result is too large) is the same function as csr_digest."""
    from resmcm_ari_gb300 import synth
    g = synth.dblp_like(n_a=800, n_p=1600, n_v=10, seed=3)
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for mp, mode in (("1-3-0-1-2-4-0-0-1", oracle_mod.MODE_COUNT), ("0-0-1-3-0", oracle_mod.MODE_BOOL)):
        r = og.chain(mp, mode, threads=2, digest=True)
        assert r.digest == csr_digest(r.rowptr, r.col, r.val)[1]
        assert r.nnz == int(r.rowptr[-1])
