"""CUDA-graph replay of the single-system evaluation (dpgb_deeppot_set_graph):
replays give bitwise the plain evaluation's results; skin lists keep
evolving on the device under replay; a new box or another system computed
on the handle makes the next call re-capture; open boundaries run without
a graph."""
import numpy as np
import pytest

from conftest import water_params

pytestmark = pytest.mark.gpu


def _water(seed, n=8):
    from dpgb import synth

    return synth.water_box(n, seed=seed)


def _eval(dp, c, box, t):
    import torch

    out = dp.eval_device(torch.from_numpy(c.reshape(1, -1)).cuda(), box.reshape(1, 9), t)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_graph_replay_matches_plain(cuda, precision):
    import torch
    from dpgb.deeppot import DeepPot

    c, t, box = _water(21)
    plain = DeepPot(water_params(), precision)
    graph = DeepPot(water_params(), precision)
    graph.set_graph(True)
    rng = np.random.default_rng(3)
    x = torch.from_numpy(c.reshape(1, -1)).cuda()
    outs = None
    for k in range(5):
        x.add_(torch.from_numpy(rng.normal(0, 0.02, size=x.shape)).cuda())
        o0 = plain.eval_device(x, box.reshape(1, 9), t)
        outs = graph.eval_device(x, box.reshape(1, 9), t, out=outs)  # same buffers: replayed from k = 1 on
        torch.cuda.synchronize()
        for key in ("energy", "force", "virial"):
            np.testing.assert_array_equal(outs[key].cpu().numpy(), o0[key].cpu().numpy())
    graph.check_status()


def test_graph_with_skin_lists(cuda):
    import torch
    from dpgb.deeppot import DeepPot

    c, t, box = _water(22)
    fresh = DeepPot(water_params(), "fp64")
    graph = DeepPot(water_params(), "fp64")
    graph.set_skin(2.0, 4)
    graph.set_graph(True)
    rng = np.random.default_rng(4)
    x = torch.from_numpy(c.reshape(1, -1)).cuda()
    outs = None
    for k in range(9):
        x.add_(torch.from_numpy(rng.normal(0, 0.02, size=x.shape)).cuda())
        o0 = fresh.eval_device(x, box.reshape(1, 9), t)
        outs = graph.eval_device(x, box.reshape(1, 9), t, out=outs)
        torch.cuda.synchronize()
        f0, f1 = o0["force"].cpu().numpy(), outs["force"].cpu().numpy()
        assert np.abs(f1 - f0).max() <= 1e-11 * np.abs(f0).max()
        if k % 4 == 0:  # a build call: bitwise the fresh list's results
            np.testing.assert_array_equal(f1, f0)
    graph.check_status()


def test_graph_recaptures(cuda):
    """A new box, and another system evaluated on the handle in between,
    both make the next call re-capture (the results stay those of a plain
    evaluation)."""
    import torch
    from dpgb.deeppot import DeepPot

    c, t, box = _water(23)
    c2, t2, box2 = _water(24, n=6)
    plain = DeepPot(water_params(), "mixed")
    graph = DeepPot(water_params(), "mixed")
    graph.set_graph(True)
    x = torch.from_numpy(c.reshape(1, -1)).cuda()
    outs = graph.eval_device(x, box.reshape(1, 9), t)
    outs = graph.eval_device(x, box.reshape(1, 9), t, out=outs)
    box_b = box * 1.01
    o_b = graph.eval_device(x, box_b.reshape(1, 9), t, out=outs)  # new box
    torch.cuda.synchronize()
    ref = plain.eval_device(x, box_b.reshape(1, 9), t)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(o_b["force"].cpu().numpy(), ref["force"].cpu().numpy())
    other = _eval(graph, c2, box2, t2)  # another system on the handle
    np.testing.assert_array_equal(other["force"], _eval(plain, c2, box2, t2)["force"])
    o_c = graph.eval_device(x, box_b.reshape(1, 9), t, out=outs)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(o_c["force"].cpu().numpy(), ref["force"].cpu().numpy())


def test_graph_host_api_and_open_boundary(cuda):
    from dpgb.deeppot import DeepPot

    c, t, box = _water(25)
    plain = DeepPot(water_params(), "mixed")
    graph = DeepPot(water_params(), "mixed")
    graph.set_graph(True)
    for _ in range(3):  # host buffers: the library's own device copies, replayed
        e1, f1, v1 = graph.eval(c.reshape(1, -1), box.reshape(1, 9), t)
    e0, f0, v0 = plain.eval(c.reshape(1, -1), box.reshape(1, 9), t)
    np.testing.assert_array_equal(f1, f0)
    np.testing.assert_array_equal(e1, e0)
    # open boundary: no graph, plain results
    sub = c[:300] - c[:300].min(0)
    e1, f1, _ = graph.eval(sub.reshape(1, -1), None, t[:300])
    e0, f0, _ = plain.eval(sub.reshape(1, -1), None, t[:300])
    np.testing.assert_array_equal(f1, f0)
