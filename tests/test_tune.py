"""
Launch-shape autotuner (fractalshades_gb300/tune.py): candidates, cache keys
and the cache round trip on CPU with a stand-in context whose launches report
a planted kernel time; the tuned shapes on the GPU are in test_gpu_tune.
"""
import json

import pytest

from fractalshades_gb300 import _native as nat
from fractalshades_gb300 import tune


class FakeCtx:
    """Reports a kernel time that depends on the launch shape only."""
    device = 0

    def __init__(self, cost):
        self.cost = cost
        self.calls = []

    def perturb_tiles(self, calc, tiles, where):
        self.calls.append((calc.block, calc.ctas_per_sm))
        self.last = self.cost(calc.block, calc.ctas_per_sm)

    std_tiles = perturb_tiles

    def stats(self):
        return {"kernel_ms": self.last}


def test_candidates_respect_launch_bounds():
    fe = nat.make_calc(max_iter=10, M_divergence=2., mode="fe32")
    assert max(b for b, _ in tune.candidates(fe, True)) == 128
    std = nat.make_calc(max_iter=10, M_divergence=2.)
    assert max(b for b, _ in tune.candidates(std, False)) == 256
    assert all(b % 32 == 0 and k >= 0 for b, k in tune.candidates(std, False))


def test_kernel_kinds_differ():
    a = nat.make_calc(max_iter=10, M_divergence=2., mode="fe32")
    b = nat.make_calc(max_iter=10, M_divergence=2., mode="fe32", interior=True)
    c = nat.make_calc(max_iter=10, M_divergence=2., mode="fe32", flavor=1)
    kinds = {tune.kernel_kind(a, True), tune.kernel_kind(b, True), tune.kernel_kind(c, True),
             tune.kernel_kind(a, False)}
    assert len(kinds) == 4


def test_autotune_picks_fastest_and_caches(tmp_path, monkeypatch):
    monkeypatch.setenv("FSG_TUNE_CACHE", str(tmp_path / "shapes.json"))
    calc = nat.make_calc(max_iter=10, M_divergence=2., mode="fe32", flavor=1)
    ctx = FakeCtx(lambda b, k: 5.0 if (b, k) == (128, 2) else 7.0 + b / 256)
    out = tune.autotune(ctx, calc, [], perturb=True, repeats=2, device="GB300")
    assert (out["block"], out["ctas_per_sm"]) == (128, 2)
    assert len(ctx.calls) == 2 * len(tune.candidates(calc, True))
    data = json.loads((tmp_path / "shapes.json").read_text())
    assert data["GB300|" + tune.kernel_kind(calc, True)]["block"] == 128
    shaped = tune.apply(calc, True, "GB300")
    assert (shaped.block, shaped.ctas_per_sm) == (128, 2)
    assert (calc.block, calc.ctas_per_sm) == (0, 0)          # the input is not modified
    # another device or kernel kind has no entry
    assert tune.apply(calc, True, "other").block == 0
    assert tune.lookup(nat.make_calc(max_iter=10, M_divergence=2.), False, "GB300") is None


def test_cache_entries_out_of_bounds_are_ignored(tmp_path, monkeypatch):
    path = tmp_path / "shapes.json"
    monkeypatch.setenv("FSG_TUNE_CACHE", str(path))
    calc = nat.make_calc(max_iter=10, M_divergence=2., mode="fe32")
    path.write_text(json.dumps({"X|" + tune.kernel_kind(calc, True):
                                {"block": 256, "ctas_per_sm": 0, "kernel_ms": 1.0}}))
    assert tune.lookup(calc, True, "X") is None      # above the FE32 kernel's 128
