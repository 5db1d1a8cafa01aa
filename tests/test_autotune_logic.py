"""Host logic of the autotuner (resmcm_ari_gb300.autotune) against a fake
engine: no GPU.  The fake's replay time depends on the tuning; one setting
can be told to change a result."""
import numpy as np
import pytest

from resmcm_ari_gb300 import autotune


class _FakeBatch:
    def __init__(self, eng):
        self.eng = eng

    def run(self):
        t = self.eng.cost(self.eng.tuning)
        dig = np.arange(4, dtype=np.uint64) + np.uint64(7)
        if self.eng.tuning == self.eng.bad:
            dig[2] += np.uint64(1)
        return np.arange(4, dtype=np.int64) * 10, dig, t

    def free(self):
        self.eng.freed += 1


class _FakeEngine:
    def __init__(self, bad=None):
        self.tuning = {"threads_per_row": 4, "hash_max_flops": 4096, "dense_ratio": 16, "warp_max_flops": 2048,
                       "hash_load": 0.5, "gemm_inv_density": 512, "gemm_min_mflops": 512}
        self.bad = bad
        self.freed = 0
        self.created = 0

    def get_tuning(self):
        return dict(self.tuning)

    def set_tuning(self, **kw):
        self.tuning.update(kw)

    def batch(self, graph, paths, lanes=8, fused=False):
        self.created += 1
        return _FakeBatch(self)

    @staticmethod
    def cost(t):
        # best at hash_max_flops 512, threads_per_row 32, warp_max_flops 8192, hash_load 0.7
        return (1.0 + abs(np.log2(t["hash_max_flops"] / 512)) + (t["threads_per_row"] != 32)
                + (t["warp_max_flops"] != 8192) + (t["hash_load"] != 0.7))


def test_coordinate_search_finds_the_measured_best():
    eng = _FakeEngine()
    res = autotune.tune(eng, None, ["p"] * 4, reps=2, mode="coordinate")
    assert res["best"] == {"hash_max_flops": 512, "hash_load": 0.7, "threads_per_row": 32, "warp_max_flops": 8192}
    assert res["best_s"] == min(t for _, t, _ in res["table"])
    # repeats skipped: at most 1 + 5 + 2 + 4 + 4 candidates, every batch freed
    assert len(res["table"]) <= 16 and eng.freed == eng.created == len(res["table"])
    assert eng.get_tuning()["threads_per_row"] == 32 and eng.get_tuning()["gemm_inv_density"] == 512


def test_grid_search_tries_every_combination():
    eng = _FakeEngine()
    res = autotune.tune(eng, None, ["p"], reps=1, mode="grid", apply=False)
    # the defaults (hash_max_flops 4096 is not a grid point) plus the 160 points
    assert len(res["table"]) == 1 + 5 * 2 * 4 * 4
    assert eng.get_tuning()["hash_max_flops"] == 4096   # apply=False restores the defaults


def test_a_tuning_that_changes_a_result_is_refused():
    bad = {"threads_per_row": 4, "hash_max_flops": 128, "dense_ratio": 16, "warp_max_flops": 2048,
           "hash_load": 0.5, "gemm_inv_density": 512, "gemm_min_mflops": 512}
    eng = _FakeEngine(bad=bad)
    with pytest.raises(autotune.TuningMismatch):
        autotune.tune(eng, None, ["a", "b", "c", "d"], reps=1, mode="coordinate")


def test_unknown_mode_is_rejected():
    with pytest.raises(ValueError):
        autotune.tune(_FakeEngine(), None, ["p"], mode="random")
