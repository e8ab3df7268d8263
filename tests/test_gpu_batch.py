"""Batches of periodic frames of different sizes (dpgb_batch_*): one set of
launches for all frames, optionally replayed from a CUDA graph, against the
frame-by-frame evaluation (FP64: to rounding; mixed: within the stated
tolerance of FP64)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _frames(n=7, seed=3, hi=700):
    """Random frames plus two one-cell-thick rods (a prime number of fcc
    cells: 1 x 1 x 37 and 1 x 1 x 401 cells, so reach 2 across two faces and
    an elongated cell grid)."""
    from dpgb import synth

    rng = np.random.default_rng(seed + 100)
    return synth.fcc_alloy_batch(nframes=n, seed=seed, lo=32, hi=hi) + [
        synth.fcc_alloy_frame(4 * 37, rng), synth.fcc_alloy_frame(4 * 401, rng)]


@pytest.fixture(scope="module")
def alloy_params():
    from dpgb import params as P

    return P.init_params(P.alloy_config(), seed=5)


def test_batch_fp64_matches_frame_by_frame(cuda, alloy_params):
    from dpgb.deeppot import DeepPot

    frames = _frames()
    dp = DeepPot(alloy_params, "fp64")
    b = dp.batch(frames)
    e, f, v = b.eval([c for c, _, _ in frames])
    for k, (c, t, box) in enumerate(frames):
        e1, f1, v1 = dp.eval(c.reshape(1, -1), box.reshape(1, 9), t)
        assert rel(e[k], e1[0]) < 1e-12
        assert rel(f[k], f1[0]) < 1e-10
        assert rel(v[k], v1[0]) < 1e-10


def test_batch_graph_replay(cuda, alloy_params):
    """A captured evaluation replayed on new coordinates equals a plain one."""
    from dpgb.deeppot import DeepPot

    frames = _frames(seed=4)
    dp = DeepPot(alloy_params, "mixed")
    b = dp.batch(frames)
    rng = np.random.default_rng(2)
    c0 = np.concatenate([c for c, _, _ in frames])
    b.eval(c0, use_graph=True)  # plain evaluation, then capture
    c1 = c0 + rng.normal(0, 0.02, size=c0.shape)
    e_g, f_g, v_g = b.eval(c1, use_graph=True)  # replay
    e_p, f_p, v_p = b.eval(c1, use_graph=False)
    np.testing.assert_array_equal(e_g, e_p)
    for a, c in zip(f_g, f_p):
        np.testing.assert_array_equal(a, c)
    np.testing.assert_array_equal(v_g, v_p)
    # another system on the same handle in between: the batch re-captures
    c2, t2, box2 = frames[0]
    dp.eval(c2.reshape(1, -1), box2.reshape(1, 9), t2)
    e_r, f_r, _ = b.eval(c1, use_graph=True)
    np.testing.assert_array_equal(e_r, e_p)


def test_batch_mixed_vs_fp64(cuda, alloy_params):
    from dpgb.deeppot import DeepPot

    frames = _frames(seed=6)
    coords = [c for c, _, _ in frames]
    e64, f64, _ = DeepPot(alloy_params, "fp64").batch(frames).eval(coords)
    e32, f32, _ = DeepPot(alloy_params, "mixed").batch(frames).eval(coords)
    fa, fb = np.concatenate(f32), np.concatenate(f64)
    n = fa.shape[0]
    assert float(np.sqrt(np.mean((fa - fb) ** 2))) <= 1e-3
    assert float(np.sqrt(np.mean((fa - fb) ** 2))) <= 2e-2 * float(np.sqrt(np.mean(fb ** 2)))
    nat = np.array([len(t) for _, t, _ in frames])
    assert np.max(np.abs(e32 - e64) / nat) < 2e-4
    assert n == nat.sum()
