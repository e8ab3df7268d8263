"""The launch-configuration tuner of batched evaluations (dpgb.autotune) on
the CPU, with a fake batch and a fake timer (no kernel runs): the sweep
finds each bucket's best work-item size, skips empty buckets and keeps the
incumbent within the minimum gain; the cache serves a second call without
timing, is keyed by the bucket populations and the model shape, and is
re-swept on request; a failing tuner leaves the defaults (the registry
semantics of deepmd/kernels/autotune.py:45-87)."""
import json

import pytest


class FakeBatch:
    def __init__(self, frames, atoms, shape="se_e2_a test"):
        self._fa = (list(frames), list(atoms))
        self.dp = type("DP", (), {"shape_key": shape})()
        self.set_calls = []

    def buckets(self):
        return self._fa

    def set_tiles(self, t):
        self.set_calls.append(list(t))


def bowl(best):
    """ms of a tile setting: a bowl around best[k] in every bucket."""
    import math

    def f(tiles):
        return 10.0 + sum(0.0 if b == 0 else abs(math.log2(max(t, 16)) - math.log2(b)) for t, b in zip(tiles, best))

    return f


def test_sweep_finds_each_bucket_best():
    from dpgb.autotune import sweep_tiles

    calls = []
    f = bowl([64, 256, 0, 512])

    def timer(t):
        calls.append(list(t))
        return f(t)

    res = sweep_tiles([10, 20, 0, 5], [500, 6000, 0, 15000], timer)
    assert res["tiles"] == [64, 256, 0, 512]
    assert res["ms"] == pytest.approx(10.0)
    assert res["default_ms"] > res["ms"]
    # bucket 2 is empty: never swept; the largest bucket (3) goes first
    assert all(t[2] == 0 for t in calls)
    assert calls[1][3] != 0 and calls[1][:3] == [0, 0, 0]
    assert len(calls) == 1 + 3 * 6


def test_sweep_keeps_incumbent_within_min_gain():
    from dpgb.autotune import sweep_tiles

    res = sweep_tiles([1, 1, 1, 1], [1, 1, 1, 1], lambda t: 10.0 - 0.001 * sum(x > 0 for x in t), min_gain=0.01)
    assert res["tiles"] == [0, 0, 0, 0]


def test_tune_batch_cache(tmp_path):
    from dpgb.autotune import tune_batch

    path = str(tmp_path / "tune.json")
    b = FakeBatch([3, 4, 5, 6], [300, 1200, 6000, 18000])
    n = []

    def timer(t):
        n.append(1)
        return bowl([32, 128, 512, 1024])(t)

    r1 = tune_batch(b, time_tiles=timer, device_name="GPU-X", cache=path)
    assert not r1["cached"] and r1["tiles"] == [32, 128, 512, 1024]
    assert b.set_calls[-1] == r1["tiles"]
    swept = len(n)
    r2 = tune_batch(b, time_tiles=timer, device_name="GPU-X", cache=path)
    assert r2["cached"] and r2["tiles"] == r1["tiles"] and len(n) == swept
    # another population, another GPU or another model shape: a new sweep
    tune_batch(FakeBatch([3, 4, 5, 7], [300, 1200, 6000, 21000]), time_tiles=timer, device_name="GPU-X", cache=path)
    tune_batch(b, time_tiles=timer, device_name="GPU-Y", cache=path)
    tune_batch(FakeBatch([3, 4, 5, 6], [300, 1200, 6000, 18000], shape="other"), time_tiles=timer,
               device_name="GPU-X", cache=path)
    assert len(json.load(open(path))) == 4
    r3 = tune_batch(b, time_tiles=timer, device_name="GPU-X", cache=path, force=True)
    assert not r3["cached"] and len(n) > 4 * swept


def test_corrupt_cache_is_ignored(tmp_path):
    from dpgb.autotune import tune_batch

    path = tmp_path / "tune.json"
    path.write_text("{not json")
    r = tune_batch(FakeBatch([1, 0, 0, 0], [50, 0, 0, 0]), time_tiles=bowl([64, 0, 0, 0]), device_name="G",
                   cache=str(path))
    assert r["tiles"] == [64, 0, 0, 0] and not r["cached"]
    assert json.load(open(path))


def test_failing_tuner_keeps_defaults():
    from dpgb import autotune as A

    saved = dict(A._TUNERS)
    try:
        A.register_autotuner("broken", lambda target: 1 / 0)
        A.register_autotuner("ok", lambda target: {"tiles": [1, 2, 3, 4]})
        A.register_autotuner("ok", lambda target: {"tiles": [5, 6, 7, 8]})  # replaces
        A._TUNERS.pop("batch_tiles", None)
        out = A.run_autotune(object())
        assert out == {"broken": None, "ok": {"tiles": [5, 6, 7, 8]}}
    finally:
        A._TUNERS.clear()
        A._TUNERS.update(saved)
