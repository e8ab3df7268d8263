"""Per-bucket work items of batched evaluations (dpgb_batch_set_tiles) and
their tuner (dpgb.autotune) on the GPU: with tiles set, the persistent
embedding / table kernels draw their items from a device queue; every
result — energies, forces, virials — must equal the default split's bit for
bit (the items only regroup rows), for the tensor-core embedding (alloy
model) and the fused table kernels (compressed water), through plain
evaluations and graph replays; the tuner's sweep leaves the results
unchanged and its cache serves the second call."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZES = (32, 108, 256, 500, 864, 2048, 2916, 4000)  # every bucket at least once


def _frames(seed=11):
    from dpgb import synth

    rng = np.random.default_rng(seed)
    return [synth.fcc_alloy_frame(n, rng) for n in SIZES]


def _eval(b, coord, graph):
    e, f, v = b.eval(coord, use_graph=graph)
    return e, np.concatenate(f), v


def _same(r1, r2):
    for a, b in zip(r1, r2):
        np.testing.assert_array_equal(a, b)


def test_buckets_reported(cuda):
    from dpgb import params as P
    from dpgb.deeppot import DeepPot

    frames = _frames()
    b = DeepPot(P.init_params(P.alloy_config(), seed=5), "mixed").batch(frames)
    fr, at = b.buckets()
    n = [len(t) for _, t, _ in frames]
    want = [[x for x in n if x <= 128], [x for x in n if 128 < x <= 512], [x for x in n if 512 < x <= 2048],
            [x for x in n if x > 2048]]
    assert fr == [len(w) for w in want] and at == [sum(w) for w in want]
    assert b.tiles() == [0, 0, 0, 0]
    with pytest.raises(Exception):
        b.set_tiles([-1, 0, 0, 0])


@pytest.mark.parametrize("tiles", [[32, 64, 128, 256], [0, 16, 0, 1024], [7, 7, 7, 7]])
def test_tiles_do_not_change_results_tc(cuda, tiles):
    from dpgb import params as P
    from dpgb.deeppot import DeepPot

    frames = _frames()
    coord = np.concatenate([c for c, _, _ in frames])
    b = DeepPot(P.init_params(P.alloy_config(), seed=5), "mixed").batch(frames)
    ref = _eval(b, coord, False)
    b.set_tiles(tiles)
    assert b.tiles() == tiles
    _same(_eval(b, coord, False), ref)
    _eval(b, coord, True)  # capture
    _same(_eval(b, coord, True), ref)  # replay
    b.set_tiles([0, 0, 0, 0])
    _same(_eval(b, coord, True), ref)


def test_tiles_do_not_change_results_tables(cuda):
    """The compressed water model's fused table kernels on a batch of water
    boxes of three sizes."""
    from conftest import water_params
    from dpgb import synth
    from dpgb.deeppot import DeepPot

    frames = [synth.water_box(n, seed=20 + n) for n in (3, 4, 6, 8)]  # 81, 192, 648, 1536 atoms
    frames = [(c, t, b.reshape(9)) for c, t, b in frames]
    coord = np.concatenate([c for c, _, _ in frames])
    b = DeepPot(water_params(compressed=True), "mixed").batch(frames)
    ref = _eval(b, coord, False)
    for tiles in ([16, 32, 64, 0], [100, 100, 100, 100]):
        b.set_tiles(tiles)
        _same(_eval(b, coord, False), ref)
        _eval(b, coord, True)
        _same(_eval(b, coord, True), ref)


def test_tuner_sweep_and_cache(cuda, tmp_path):
    import torch

    from dpgb import autotune as A, params as P
    from dpgb.deeppot import DeepPot

    frames = _frames(seed=12)
    coord = np.concatenate([c for c, _, _ in frames])
    b = DeepPot(P.init_params(P.alloy_config(), seed=5), "mixed").batch(frames)
    ref = _eval(b, coord, False)
    cdev = torch.tensor(coord, dtype=torch.float64, device="cuda")
    path = str(tmp_path / "tune.json")
    r = A.tune_batch(b, cdev, cache=path, candidates=(0, 64, 256))
    assert not r["cached"] and b.tiles() == r["tiles"]
    assert r["ms"] <= r["default_ms"] and len(r["trials"]) == 1 + 4 * 2
    _same(_eval(b, coord, False), ref)
    b.set_tiles([0, 0, 0, 0])
    r2 = A.tune_batch(b, cdev, cache=path)
    assert r2["cached"] and b.tiles() == r["tiles"]
